/*
 * cpvs_oracle.cpp -- CPU restatement of the reference's shadow build and
 * visibility lookup (TobiasRp/cpvs).
 *
 * TEST INFRASTRUCTURE ONLY.  This is the oracle the CUDA path is compared
 * against: only tests/, __graft_entry__.smoke() and bench.py's CPU baseline
 * leg load it.  The product never links or calls it.
 *
 * Parity pin: this restatement is checked against (1) the reference's own
 * sources compiled in place (oracle/_ref/libcpvs_ref.so, see Makefile) on
 * seeded random and scene depth maps, byte for byte on the DAG words, and
 * (2) the golden fixtures under tests/golden/, which were written from that
 * reference build and from the reference's own test images.
 *
 * Each function names the reference lines it restates.  Where the reference
 * is undefined (see `ref_defined` below) this restatement produces the DAG
 * the reference's algorithm intends and reports the condition.
 *
 * Parity unpinned: the shader restatements (oracle_grid_evaluate's float
 * transform and oracle_shade) follow the GLSL of shader/traverse.cs and
 * shader/shade.frag, which need a GL context that no machine here provides;
 * GLSL leaves their float32 operation order open, so the order is defined
 * here, and the GPU path is checked against it bit for bit.  The lookup part of evaluate is pinned
 * like the other lookups.
 */
#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <functional>
#include <thread>
#include <unordered_map>
#include <vector>

namespace {

constexpr uint32_t kInnerWords = 9;  /* mask + 8 child slots   (src/CompressedShadowUtil.h:9)  */
constexpr uint32_t kLeafWords = 17;  /* mask + 8 x 64-bit masks (src/CompressedShadowUtil.h:10) */

/* std::min<float> / std::max<float> as the pyramid uses them
 * (src/MinMaxHierarchy.cpp:29-49): the second argument wins only on a strict
 * compare, which fixes the result for signed zeros and NaN. */
inline float fmin_ref(float a, float b) { return (b < a) ? b : a; }
inline float fmax_ref(float a, float b) { return (a < b) ? b : a; }

/* Min-max pyramid (src/MinMaxHierarchy.cpp:9-27, 51-97).  Level 0 is the
 * depth image itself; level L>=1 holds (n>>L)^2 (min,max) pairs. */
struct Pyramid {
    uint32_t n = 0;
    int num_levels = 0;
    const float* root = nullptr;
    std::vector<std::vector<float>> lv;  // lv[L-1]: interleaved (min,max)

    float mn(int L, uint32_t x, uint32_t y) const {
        if (L == 0) return root[(size_t)y * n + x];
        return lv[L - 1][((size_t)y * (n >> L) + x) * 2];
    }
    float mx(int L, uint32_t x, uint32_t y) const {
        if (L == 0) return root[(size_t)y * n + x];
        return lv[L - 1][((size_t)y * (n >> L) + x) * 2 + 1];
    }
};

void reduce_rows(const Pyramid& P, int L, std::vector<float>& out, uint32_t y0, uint32_t y1) {
    const uint32_t so = P.n >> L;
    for (uint32_t y = y0; y < y1; ++y)
        for (uint32_t x = 0; x < so; ++x) {
            const uint32_t ix = 2 * x, iy = 2 * y;
            /* pred(pred(a,b), pred(c,d)) with a=(2x,2y) b=(2x+1,2y) c=(2x,2y+1) d=(2x+1,2y+1) */
            float lo = fmin_ref(fmin_ref(P.mn(L - 1, ix, iy), P.mn(L - 1, ix + 1, iy)),
                                fmin_ref(P.mn(L - 1, ix, iy + 1), P.mn(L - 1, ix + 1, iy + 1)));
            float hi = fmax_ref(fmax_ref(P.mx(L - 1, ix, iy), P.mx(L - 1, ix + 1, iy)),
                                fmax_ref(P.mx(L - 1, ix, iy + 1), P.mx(L - 1, ix + 1, iy + 1)));
            out[((size_t)y * so + x) * 2] = lo;
            out[((size_t)y * so + x) * 2 + 1] = hi;
        }
}

int log2_exact(uint32_t n) {
    int l = 0;
    while ((1u << l) < n) ++l;
    return l;
}

void build_pyramid(Pyramid& P, const float* depth, uint32_t n, int threads) {
    P.n = n;
    P.root = depth;
    const int levels = log2_exact(n);  // levels without the root
    P.num_levels = levels + 1;
    P.lv.assign(levels, {});
    for (int L = 1; L <= levels; ++L) {
        const uint32_t so = n >> L;
        P.lv[L - 1].assign((size_t)so * so * 2, 0.f);
        /* The reference splits the rows of a level over 4 threads once the
         * input is >= 256 wide (src/MinMaxHierarchy.cpp:56-67). */
        int t = (threads > 1 && (n >> (L - 1)) >= 256) ? threads : 1;
        if (t == 1) {
            reduce_rows(P, L, P.lv[L - 1], 0, so);
        } else {
            std::vector<std::thread> pool;
            for (int i = 0; i < t; ++i) {
                uint32_t y0 = (uint32_t)((uint64_t)so * i / t), y1 = (uint32_t)((uint64_t)so * (i + 1) / t);
                pool.emplace_back(reduce_rows, std::cref(P), L, std::ref(P.lv[L - 1]), y0, y1);
            }
            for (auto& th : pool) th.join();
        }
    }
}

/* Visibility classes (src/CompressedShadow.h:22-26). */
enum : uint32_t { SHADOW = 0, VISIBLE = 1, PARTIAL = 2 };

/* cs::visible (src/CompressedShadowUtil.h:35-43). */
inline uint32_t classify(float zlo, float zhi, float dmin, float dmax) {
    if (zhi <= dmin) return VISIBLE;
    if (zlo >= dmax) return SHADOW;
    return PARTIAL;
}
/* cs::absoluteVisible (src/CompressedShadowUtil.h:51-57). */
inline uint32_t classify_voxel(float zlo, float zhi, float d) {
    const float mid = (zlo + zhi) * 0.5f;
    return (mid <= d) ? VISIBLE : SHADOW;
}

/* cs::createChildmask (src/CompressedShadowUtil.cpp:20-54).  `H` is the
 * depth scale of the level, (n >> level) * zTileNum (:16-18). */
uint32_t child_mask(const Pyramid& P, int L, int ox, int oy, int oz, uint32_t H) {
    const float h = (float)H;
    uint32_t m = 0;
    for (uint32_t c = 0; c < 8; ++c) {
        const uint32_t x = c & 1, y = (c >> 1) & 1, z = c >> 2;
        const uint32_t zc = (uint32_t)oz + z;
        const float lo = P.mn(L, ox + x, oy + y), hi = P.mx(L, ox + x, oy + y);
        uint32_t v = (L > 0) ? classify((float)zc, (float)(zc + 1), lo * h, hi * h)
                             : classify_voxel((float)zc, (float)(zc + 1), lo * h);
        m |= v << (2 * c);
    }
    return m;
}

/* createLeafmask + cs::createChildmask1x1x8 (src/CompressedShadowUtil.cpp:59-99):
 * the leaf at level-2 coordinate (cx,cy,cz) covers the 8x8x8 voxels at
 * 4*(cx,cy,cz); slice s gets a 64-bit mask with bit x+8y set where the voxel
 * centre lies at or above the depth (lit). */
void leaf_slices(const Pyramid& P, int cx, int cy, int cz, uint32_t H0, uint64_t out[8]) {
    const float h = (float)H0;
    const int bx = cx * 4, by = cy * 4, bz = cz * 4;
    for (int s = 0; s < 8; ++s) {
        const int z = bz + s;
        uint64_t m = 0;
        for (int y = 0; y < 8; ++y)
            for (int x = 0; x < 8; ++x) {
                const float d = P.mn(0, bx + x, by + y);
                const uint64_t bit = classify_voxel((float)z, (float)(z + 1), d * h);
                m |= bit << (x + 8 * y);
            }
        out[s] = m;
    }
}

inline uint32_t slice_class(uint64_t m) {
    if (m == ~0ull) return VISIBLE;
    if (m == 0) return SHADOW;
    return PARTIAL;
}

inline uint32_t partial_count(uint32_t mask) { return (uint32_t)__builtin_popcount(mask & 0xAAAAu); }

struct Level {
    std::vector<uint32_t> mask;       // 16-bit child mask per node
    std::vector<int32_t> cx, cy, cz;  // node coordinate (level-L texel units)
    std::vector<uint32_t> first;      // index of the first child in level L-1
    std::vector<uint64_t> slices;     // leaf level only: 8 masks per node
    std::vector<uint32_t> uid;        // unique id after the merge
    std::vector<uint32_t> uniq;       // uid -> index of its first occurrence
    size_t size() const { return mask.size(); }
};

struct Result {
    std::vector<uint32_t> dag;
    uint32_t num_levels = 0;
    int ref_defined = 1;
    std::vector<uint64_t> tree_nodes;    // per level (index = level)
    std::vector<uint64_t> unique_nodes;  // per level
};

/* Hash of a node's signature for the merge index. */
struct VecHash {
    size_t operator()(const std::vector<uint64_t>& v) const {
        uint64_t h = 0x9E3779B97F4A7C15ull ^ v.size();
        for (uint64_t x : v) {
            h ^= x + 0x9E3779B97F4A7C15ull + (h << 6) + (h >> 2);
        }
        return (size_t)h;
    }
};

/* Whole build: CompressedShadow::create (src/CompressedShadow.cpp:49-59) =
 * constructSvo (:87-169, :171-190), mergeCommonSubtrees (:215-241 with
 * cs::mergeLevel, src/CompressedShadowUtil.h:154-182), removeUnusedNodes
 * (:271-304) and compress (:326-392).
 *
 * The SVO is built level by level in breadth-first order (parent order, then
 * child index).  The merge keeps, per level, the first occurrence of every
 * distinct node (mask plus merged child identities, or mask plus leafmasks);
 * `linear_merge` selects the reference's own linear scan over the kept nodes
 * instead of a hash index (same result, the reference's cost).  The final
 * layout is levels top-down, unique nodes in first-occurrence order, inner
 * nodes as 1+k words and leaves as 1+2k words, child slots holding absolute
 * word offsets. */
void build(const Pyramid& P, uint32_t zIdx, uint32_t zNum, bool leafmasks_opt, bool linear_merge, Result& R) {
    const int NL = P.num_levels;
    R.num_levels = (uint32_t)NL;
    /* useLeafmasks: numLevels-3 >= 2 (src/CompressedShadow.cpp:20-27) */
    const bool leafmasks = leafmasks_opt && (NL - 3) >= 2;
    const int bottom = leafmasks ? 2 : 0;
    const int root = NL - 2;
    std::vector<Level> lv(NL);

    auto H = [&](int L) -> uint32_t { return (P.n >> L) * zNum; };

    /* top-down: root at (0,0,2*zTileIndex) (src/CompressedShadow.cpp:54) */
    lv[root].cx.push_back(0);
    lv[root].cy.push_back(0);
    lv[root].cz.push_back((int32_t)(2 * zIdx));
    for (int L = root; L >= bottom; --L) {
        Level& cur = lv[L];
        const size_t n = cur.cx.size();
        if (L == 2 && leafmasks) {
            cur.slices.resize(n * 8);
            cur.mask.resize(n);
            for (size_t i = 0; i < n; ++i) {
                uint64_t* s = &cur.slices[i * 8];
                leaf_slices(P, cur.cx[i], cur.cy[i], cur.cz[i], H(0), s);
                uint32_t m = 0;
                for (int k = 0; k < 8; ++k) m |= slice_class(s[k]) << (2 * k);
                cur.mask[i] = m;
            }
            break;
        }
        cur.mask.resize(n);
        cur.first.resize(n);
        Level* nxt = (L > bottom) ? &lv[L - 1] : nullptr;
        for (size_t i = 0; i < n; ++i) {
            uint32_t m = child_mask(P, L, cur.cx[i], cur.cy[i], cur.cz[i], H(L));
            cur.mask[i] = m;
            if (!nxt) continue;
            cur.first[i] = (uint32_t)nxt->cx.size();
            /* cs::getChildCoordinates (src/CompressedShadowUtil.cpp:101-117) */
            for (uint32_t c = 0; c < 8; ++c)
                if (m & (2u << (2 * c))) {
                    nxt->cx.push_back((cur.cx[i] + (int32_t)(c & 1)) * 2);
                    nxt->cy.push_back((cur.cy[i] + (int32_t)((c >> 1) & 1)) * 2);
                    nxt->cz.push_back((cur.cz[i] + (int32_t)(c >> 2)) * 2);
                }
        }
        if (!nxt || nxt->cx.empty()) break;
    }

    /* Where the reference's levelExists() mis-reads an SVO that stops above
     * its last level (src/CompressedShadow.cpp:208-213, 285-288) the
     * reference reads past its array; flag that case. */
    int deepest = root;
    for (int L = root; L >= bottom; --L)
        if (!lv[L].cx.empty()) deepest = L;
    if (leafmasks)
        R.ref_defined = !(deepest >= 4 && deepest <= root - 1);
    else
        R.ref_defined = !(deepest >= 1 && deepest <= root - 1);

    /* bottom-up merge, root excluded */
    for (int L = bottom; L < root; ++L) {
        Level& cur = lv[L];
        const size_t n = cur.cx.size();
        cur.uid.assign(n, 0);
        cur.uniq.clear();
        const bool is_leaf = leafmasks && L == 2;
        auto sig = [&](size_t i, std::vector<uint64_t>& s) {
            s.clear();
            s.push_back(cur.mask[i]);
            if (is_leaf) {
                for (int k = 0; k < 8; ++k) s.push_back(cur.slices[i * 8 + k]);
            } else {
                const uint32_t k = partial_count(cur.mask[i]);
                for (uint32_t r = 0; r < k; ++r) s.push_back(lv[L - 1].uid[cur.first[i] + r]);
            }
        };
        std::vector<uint64_t> s, t;
        if (linear_merge) {
            for (size_t i = 0; i < n; ++i) {
                sig(i, s);
                size_t u = 0;
                for (; u < cur.uniq.size(); ++u) {
                    sig(cur.uniq[u], t);
                    if (s == t) break;
                }
                if (u == cur.uniq.size()) cur.uniq.push_back((uint32_t)i);
                cur.uid[i] = (uint32_t)u;
            }
        } else {
            std::unordered_map<std::vector<uint64_t>, uint32_t, VecHash> index;
            index.reserve(n * 2 + 16);
            for (size_t i = 0; i < n; ++i) {
                sig(i, s);
                auto it = index.find(s);
                if (it == index.end()) {
                    const uint32_t u = (uint32_t)cur.uniq.size();
                    index.emplace(s, u);
                    cur.uniq.push_back((uint32_t)i);
                    cur.uid[i] = u;
                } else {
                    cur.uid[i] = it->second;
                }
            }
        }
    }
    lv[root].uid.assign(1, 0);
    lv[root].uniq.assign(1, 0);

    /* layout: level base offsets, then each unique node's word offset */
    R.tree_nodes.assign(NL, 0);
    R.unique_nodes.assign(NL, 0);
    std::vector<std::vector<uint32_t>> off(NL);
    uint64_t total = 0;
    for (int L = root; L >= bottom; --L) {
        Level& cur = lv[L];
        R.tree_nodes[L] = cur.cx.size();
        R.unique_nodes[L] = cur.uniq.size();
        const bool is_leaf = leafmasks && L == 2;
        off[L].resize(cur.uniq.size());
        for (size_t u = 0; u < cur.uniq.size(); ++u) {
            off[L][u] = (uint32_t)total;
            const uint32_t k = partial_count(cur.mask[cur.uniq[u]]);
            total += 1 + (is_leaf ? 2 * k : k);
        }
    }
    R.dag.assign(total, 0);
    for (int L = root; L >= bottom; --L) {
        Level& cur = lv[L];
        const bool is_leaf = leafmasks && L == 2;
        for (size_t u = 0; u < cur.uniq.size(); ++u) {
            const uint32_t i = cur.uniq[u];
            uint32_t* w = &R.dag[off[L][u]];
            w[0] = cur.mask[i];
            const uint32_t k = partial_count(cur.mask[i]);
            if (is_leaf) {
                uint32_t r = 0;
                for (int s2 = 0; s2 < 8; ++s2)
                    if (slice_class(cur.slices[i * 8 + s2]) == PARTIAL) {
                        w[1 + 2 * r] = (uint32_t)cur.slices[i * 8 + s2];
                        w[2 + 2 * r] = (uint32_t)(cur.slices[i * 8 + s2] >> 32);
                        ++r;
                    }
            } else {
                for (uint32_t r = 0; r < k; ++r) w[1 + r] = off[L - 1][lv[L - 1].uid[cur.first[i] + r]];
            }
        }
    }
}

/* getChildOffset (src/CompressedShadow.cpp:394-402): rank of `child` among
 * the node's partial children. */
inline uint32_t child_rank(uint32_t mask, uint32_t child) {
    return (uint32_t)__builtin_popcount(mask & (0xAAAAu >> (16 - 2 * child)));
}

/* CompressedShadow::traverse after the NDC quantisation
 * (src/CompressedShadow.cpp:404-463).  `base` is added to every pointer
 * read, which turns it into the shader's relative descent
 * (shader/traverse.cs:90-129) over a concatenated DAG buffer. */
uint32_t descend(const uint32_t* dag, uint32_t base, int num_levels, bool leafmasks, int32_t px, int32_t py,
                 int32_t pz) {
    uint32_t off = base;
    int level = num_levels - 2;
    const int min_level = leafmasks ? 3 : 0;
    for (; level >= min_level; --level) {
        const int32_t bit = 1 << level;
        const uint32_t c = ((px & bit) ? 1u : 0u) + ((py & bit) ? 2u : 0u) + ((pz & bit) ? 4u : 0u);
        const uint32_t m = dag[off];
        const uint32_t v = (m >> (2 * c)) & 3u;
        if (v & 1u) return VISIBLE;
        if (!(v & 2u)) return SHADOW;
        off = base + dag[off + 1 + child_rank(m, c)];
    }
    if (!leafmasks) return PARTIAL;
    const uint32_t c = (uint32_t)(pz & 7);
    const uint32_t m = dag[off];
    const uint32_t v = (m >> (2 * c)) & 3u;
    if (v & 1u) return VISIBLE;
    if (!(v & 2u)) return SHADOW;
    const uint32_t idx = off + child_rank(m, c) * 2 + 1;
    const uint32_t bit = (uint32_t)((px & 7) + 8 * (py & 7));
    const uint32_t word = (bit < 32) ? dag[idx] : dag[idx + 1];
    return (word & (1u << (bit & 31))) ? VISIBLE : SHADOW;
}

/* cs::getPathFromNDC (src/CompressedShadowUtil.h:62-75): float32, in this
 * order: +1, *0.5, *(R-1), truncate. */
inline int32_t quantise(float v, float scale) {
    float t = v + 1.0f;
    t = t * 0.5f;
    return (int32_t)(t * scale);
}

}  // namespace

extern "C" {

/* All pyramid levels 1..numLevels-1 back to back, (min,max) interleaved.
 * Returns numLevels. */
int oracle_pyramid(const float* depth, uint32_t n, float* out, int threads) {
    Pyramid P;
    build_pyramid(P, depth, n, threads);
    size_t o = 0;
    for (auto& l : P.lv) {
        std::memcpy(out + o, l.data(), l.size() * sizeof(float));
        o += l.size();
    }
    return P.num_levels;
}

uint32_t oracle_child_mask(const float* depth, uint32_t n, int level, int x, int y, int z, uint32_t zNum) {
    Pyramid P;
    build_pyramid(P, depth, n, 1);
    return child_mask(P, level, x, y, z, (n >> level) * zNum);
}

struct OracleShadow {
    Result r;
    int leafmasks;
};

/* Build one DAG.  flags bit 0: leafmasks; bit 1: linear (reference-cost) merge.
 * `threads` is used by the pyramid only, as in the reference. */
void* oracle_build(const float* depth, uint32_t n, uint32_t zIdx, uint32_t zNum, uint32_t flags, int threads) {
    Pyramid P;
    build_pyramid(P, depth, n, threads);
    auto* h = new OracleShadow;
    build(P, zIdx, zNum, (flags & 1) != 0, (flags & 2) != 0, h->r);
    h->leafmasks = ((flags & 1) != 0) && ((int)h->r.num_levels - 3) >= 2;
    return h;
}

void oracle_free(void* h) { delete static_cast<OracleShadow*>(h); }
size_t oracle_dag_size(void* h) { return static_cast<OracleShadow*>(h)->r.dag.size(); }
const uint32_t* oracle_dag_words(void* h) { return static_cast<OracleShadow*>(h)->r.dag.data(); }
uint32_t oracle_num_levels(void* h) { return static_cast<OracleShadow*>(h)->r.num_levels; }
int oracle_uses_leafmasks(void* h) { return static_cast<OracleShadow*>(h)->leafmasks; }
int oracle_ref_defined(void* h) { return static_cast<OracleShadow*>(h)->r.ref_defined; }
/* tree (pre-merge) and unique (post-merge) node counts of `level` */
uint64_t oracle_tree_nodes(void* h, int level) {
    auto& v = static_cast<OracleShadow*>(h)->r.tree_nodes;
    return (level >= 0 && (size_t)level < v.size()) ? v[level] : 0;
}
uint64_t oracle_unique_nodes(void* h, int level) {
    auto& v = static_cast<OracleShadow*>(h)->r.unique_nodes;
    return (level >= 0 && (size_t)level < v.size()) ? v[level] : 0;
}

/* cs::mergeLevel (src/CompressedShadowUtil.h:154-182) over `words` holding
 * equal-size nodes: keeps the first occurrence of every distinct node, writes
 * the kept nodes to `out` (zero padded to numWords), the level-relative word
 * offset each node maps to into `mapping` (one entry per node), and returns
 * the kept count. */
uint32_t oracle_merge_level(const uint32_t* words, uint32_t numWords, uint32_t nodeSize, uint32_t* out,
                            uint32_t* mapping) {
    const uint32_t nodes = numWords / nodeSize;
    std::memset(out, 0, numWords * sizeof(uint32_t));
    uint32_t kept = 0;
    for (uint32_t i = 0; i < nodes; ++i) {
        uint32_t u = 0;
        for (; u < kept; ++u)
            if (std::memcmp(words + (size_t)i * nodeSize, out + (size_t)u * nodeSize, nodeSize * 4) == 0) break;
        if (u == kept) {
            std::memcpy(out + (size_t)kept * nodeSize, words + (size_t)i * nodeSize, nodeSize * 4);
            ++kept;
        }
        mapping[i] = u * nodeSize;
    }
    return kept;
}

/* getTotalVisibility (src/CompressedShadow.cpp:66-72) of a DAG's root mask. */
int oracle_total_visibility(const uint32_t* dag) {
    if (dag[0] == 0x5555u) return VISIBLE;
    if (dag[0] == 0u) return SHADOW;
    return PARTIAL;
}

static void run_parallel(uint64_t n, int threads, const std::function<void(uint64_t, uint64_t)>& f);

/* Lookup by integer voxel coordinate (the path the reference derives from
 * NDC), xyz interleaved int32.  Output one class byte per query. */
void oracle_lookup_voxel(const uint32_t* dag, uint32_t num_levels, int leafmasks, const int32_t* xyz, uint64_t n,
                         uint8_t* out, int threads) {
    run_parallel(n, threads, [&](uint64_t a, uint64_t b) {
        for (uint64_t i = a; i < b; ++i)
            out[i] = (uint8_t)descend(dag, 0, (int)num_levels, leafmasks != 0, xyz[3 * i], xyz[3 * i + 1],
                                      xyz[3 * i + 2]);
    });
}

/* CompressedShadow::traverse(ndc) over n points (xyz interleaved float32). */
void oracle_lookup_ndc(const uint32_t* dag, uint32_t num_levels, int leafmasks, const float* xyz, uint64_t n,
                       uint8_t* out, int threads) {
    const float scale = (float)(int32_t)((1u << (num_levels - 1)) - 1);
    run_parallel(n, threads, [&](uint64_t a, uint64_t b) {
        for (uint64_t i = a; i < b; ++i)
            out[i] = (uint8_t)descend(dag, 0, (int)num_levels, leafmasks != 0, quantise(xyz[3 * i], scale),
                                      quantise(xyz[3 * i + 1], scale), quantise(xyz[3 * i + 2], scale));
    });
}

/* The shader's grid routing and descent (shader/traverse.cs:41-133) over a
 * concatenated DAG buffer and a cubic grid of `length`^3 cells, each cell
 * holding its DAG's start offset.  A cell whose DAG is uniformly lit or
 * shadowed answers that class (the intent of the sentinels in
 * src/CompressedShadowContainer.cpp:8-9,71-91).  Points whose grid cell lies
 * outside the grid answer VISIBLE. */
void oracle_grid_lookup_ndc(const uint32_t* dag, const uint32_t* cell_offset, uint32_t length, uint32_t dag_levels,
                            int leafmasks, const float* xyz, uint64_t n, uint8_t* out, int threads) {
    int grid_levels = log2_exact(length);
    const uint32_t res = 1u << (dag_levels + grid_levels - 1);
    const float scale = (float)(res - 1);
    run_parallel(n, threads, [&](uint64_t a, uint64_t b) {
        for (uint64_t i = a; i < b; ++i) {
            const int32_t px = quantise(xyz[3 * i], scale), py = quantise(xyz[3 * i + 1], scale),
                          pz = quantise(xyz[3 * i + 2], scale);
            const int32_t gx = px >> (dag_levels - 1), gy = py >> (dag_levels - 1), gz = pz >> (dag_levels - 1);
            if (gx < 0 || gy < 0 || gz < 0 || gx >= (int32_t)length || gy >= (int32_t)length ||
                gz >= (int32_t)length) {
                out[i] = VISIBLE;
                continue;
            }
            const uint32_t base = cell_offset[((size_t)gz * length + gy) * length + gx];
            out[i] = (uint8_t)descend(dag, base, (int)dag_levels, leafmasks != 0, px, py, pz);
        }
    });
}

/* CompressedShadowContainer::evaluate (src/CompressedShadowContainer.cpp:93-124)
 * with the shader's per-pixel body (shader/traverse.cs:134-148): pixel i's
 * position (the first three of its `fpp` floats) times the column-major
 * light view-projection m as c_r = ((m[r]*x + m[4+r]*y) + m[8+r]*z) + m[12+r]
 * (the shader's lightViewProj * vec4(pos, 1); float32, no contraction), the
 * perspective divide ndc = c.xyz / c.w, the path of getPathFromNDC at the
 * grid's resolution, then the grid lookup of oracle_grid_lookup_ndc.  Output
 * one byte per pixel: 255 lit / 0 shadowed, or with filter f > 1 the
 * percentage-closer fraction round(255 * lit / f^2) over the paths
 * (px+dx, py+dy, pz), dx, dy in -(f-1)/2 .. f/2 (the reference declares the
 * filter size, src/CompressedShadowContainer.h:70-73, but its shader never
 * uses it; this is the definition the GPU path implements). */
void oracle_grid_evaluate(const uint32_t* dag, const uint32_t* cell_offset, uint32_t length, uint32_t dag_levels,
                          int leafmasks, const float* pos, uint64_t n, uint32_t fpp, const float* m, uint32_t filter,
                          uint8_t* out, int threads) {
    const int grid_levels = log2_exact(length);
    const float scale = (float)((1u << (dag_levels + grid_levels - 1)) - 1u);
    const int64_t lim = (int64_t)length << (dag_levels - 1);
    const int f = filter < 1 ? 1 : (int)filter;
    const int lo = -((f - 1) / 2), hi = f / 2;
    auto sample = [&](int64_t px, int64_t py, int64_t pz) -> bool {
        if (px < 0 || py < 0 || pz < 0 || px >= lim || py >= lim || pz >= lim) return true;
        const int s = (int)dag_levels - 1;
        const uint32_t base = cell_offset[((size_t)(pz >> s) * length + (size_t)(py >> s)) * length + (size_t)(px >> s)];
        return descend(dag, base, (int)dag_levels, leafmasks != 0, (int32_t)px, (int32_t)py, (int32_t)pz) == VISIBLE;
    };
    run_parallel(n, threads, [&](uint64_t a, uint64_t b) {
        for (uint64_t i = a; i < b; ++i) {
            const float x = pos[fpp * i], y = pos[fpp * i + 1], z = pos[fpp * i + 2];
            float c[4];
            for (int r = 0; r < 4; ++r) {
                float t = m[r] * x;
                t = t + m[4 + r] * y;
                t = t + m[8 + r] * z;
                c[r] = t + m[12 + r];
            }
            const int64_t px = quantise(c[0] / c[3], scale), py = quantise(c[1] / c[3], scale),
                          pz = quantise(c[2] / c[3], scale);
            uint32_t cnt = 0;
            for (int dy = lo; dy <= hi; ++dy)
                for (int dx = lo; dx <= hi; ++dx) cnt += sample(px + dx, py + dy, pz) ? 1u : 0u;
            const uint32_t f2 = (uint32_t)(f * f);
            out[i] = (f == 1) ? (uint8_t)(cnt ? 255u : 0u) : (uint8_t)((255u * cnt + f2 / 2u) / f2);
        }
    });
}

/* The deferred shading fragment shader (shader/shade.frag:34-56) per pixel,
 * with the texture reads as buffer reads.  Float32, no contraction, each
 * operation in the order written:
 *   L = l / sqrt((lx*lx + ly*ly) + lz*lz)                    normalize(light.direction)
 *   diffuse = max(0, (Nx*Lx + Ny*Ly) + Nz*Lz)                max(0.0, dot(N, L))
 *   vis = max(byte / 255, 0)                                 renderShadow != 0: the r8 image
 *   or evaluateShadowMap (:23-32): c = M * (pos, 1) as in oracle_grid_evaluate,
 *      s = c.xyz / c.w * 0.5 + 0.5, depth texel (floor(s.x*side), floor(s.y*side))
 *      of the nearest-filtered map, 1.0 (the border colour set by
 *      clampShadowMap, src/ShadowMap.cpp:3-9) outside it; vis = d < s.z ? 0 : 1
 *   colour = ((0.15 + diffuse*vis) * albedo.rgb, albedo.a)   ambient 0.15 (:21)
 * `vis` null selects the shadow-map branch. */
void oracle_shade(uint64_t n, const float* nrm, uint32_t fpn, const float* alb, const uint8_t* vis, const float* pos,
                  uint32_t fpp, const float* sm, uint32_t side, const float* m, const float* light, float* out) {
    const float len = std::sqrt(light[0] * light[0] + light[1] * light[1] + light[2] * light[2]);
    const float lx = light[0] / len, ly = light[1] / len, lz = light[2] / len;
    const float fside = (float)side;
    for (uint64_t i = 0; i < n; ++i) {
        float v;
        if (vis) {
            v = (float)vis[i] / 255.0f;
            v = v > 0.0f ? v : 0.0f;
        } else {
            const float x = pos[fpp * i], y = pos[fpp * i + 1], z = pos[fpp * i + 2];
            float c[4];
            for (int r = 0; r < 4; ++r) {
                float t = m[r] * x;
                t = t + m[4 + r] * y;
                t = t + m[8 + r] * z;
                c[r] = t + m[12 + r];
            }
            float s[3];
            for (int k = 0; k < 3; ++k) {
                s[k] = c[k] / c[3];
                s[k] = s[k] * 0.5f;
                s[k] = s[k] + 0.5f;
            }
            const float fx = std::floor(s[0] * fside), fy = std::floor(s[1] * fside);
            float d = 1.0f;
            if (fx >= 0.0f && fx < fside && fy >= 0.0f && fy < fside) d = sm[(uint64_t)fy * side + (uint64_t)fx];
            v = (d < s[2]) ? 0.0f : 1.0f;
        }
        const float nx = nrm[fpn * i], ny = nrm[fpn * i + 1], nz = nrm[fpn * i + 2];
        float dot = nx * lx;
        dot = dot + ny * ly;
        dot = dot + nz * lz;
        const float diffuse = dot > 0.0f ? dot : 0.0f;
        const float scattered = 0.15f + diffuse * v;
        out[4 * i] = scattered * alb[4 * i];
        out[4 * i + 1] = scattered * alb[4 * i + 1];
        out[4 * i + 2] = scattered * alb[4 * i + 2];
        out[4 * i + 3] = alb[4 * i + 3];
    }
}

}  // extern "C"

static void run_parallel(uint64_t n, int threads, const std::function<void(uint64_t, uint64_t)>& f) {
    if (threads <= 1 || n < 4096) {
        f(0, n);
        return;
    }
    std::vector<std::thread> pool;
    for (int t = 0; t < threads; ++t) {
        uint64_t a = n * t / threads, b = n * (t + 1) / threads;
        pool.emplace_back(f, a, b);
    }
    for (auto& th : pool) th.join();
}
