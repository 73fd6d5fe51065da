// Batched visibility lookups against resident DAGs.
//
// Replaces CompressedShadow::traverse (src/CompressedShadow.cpp:394-463) and
// the per-pixel descent of shader/traverse.cs:41-133.  One thread per query:
// quantise the NDC point with the reference's float32 order
// (src/CompressedShadowUtil.h:70-75: +1, *0.5, *(R-1), truncate), descend
// from the root choosing child x|y<<1|z<<2 from bit `level` of the path,
// stop at a lit or shadowed child, and finish in the 64-bit leafmask.  The
// answer of 32 consecutive queries is packed by one ballot into one word.
//
// The descent is a chain of dependent L1/L2 hits (an 8192^2 map's DAG is
// 9.4 MB), so every hop is kept short -- 32-bit offsets, one bounds check
// per node (DAG buffers carry a zeroed tail of kDagPad words, so both reads
// of a node stay inside the buffer once its offset is), and the child's
// 2-bit class and rank from one shift and one popcount.  The first `depth`
// levels below the root are replaced by a dense 3-D "top grid" of
// (2^depth)^3 words, indexed by the top `depth` bits of the quantised x, y,
// z: the node offset the descent reaches after those levels, or a lit /
// shadow sentinel.  It lives in global memory (L2-resident; up to 8 levels,
// at most 8x the DAG's size), so one load replaces up to 8 dependent hops --
// and each thread carries Q independent queries (Q picked per DAG depth and
// input kind, device or host memory, by timing Q = 1, 2, 4 on the first
// batch).  A leafmask DAG with a top grid and few levels below it takes
// k_lookup_fixed (the levels unrolled, 32-bit indices); any other DAG
// k_lookup.  Query points and answer words are touched once, so they go
// through the caches evict-first (ld/st .cs): a batch streams hundreds of MB
// past L2 and would otherwise push the DAG and its top grid out of it.  The
// grid lookups and evaluate (k_grid_lookup, k_grid_evaluate) route through
// the grid's cells and a grid index the same way.
#include <algorithm>
#include <type_traits>

#include "common.cuh"

namespace cpvs {
namespace {

constexpr int kThreads = 256;
constexpr uint32_t kCellShadow = 0xFFFFFFFFu, kCellLit = 0xFFFFFFFEu;

__device__ __forceinline__ int32_t quantise(float v, float scale) {
    const float t = __fmul_rn(__fadd_rn(v, 1.0f), 0.5f);
    return __float2int_rz(__fmul_rn(t, scale));
}

// 2 * child index at `level`: bit `level` of x, y, z at weights 2, 4, 8.
__device__ __forceinline__ uint32_t child2(int32_t px, int32_t py, int32_t pz, int level) {
    return (((uint32_t)px >> level) & 1u) * 2u + (((uint32_t)py >> level) & 1u) * 4u +
           (((uint32_t)pz >> level) & 1u) * 8u;
}

// Descent from node `off` at `level` down to the leafmask, pointers relative
// to `base` (the DAG's first word).  Returns true when the voxel is lit.  A
// node offset outside the DAG (a malformed buffer) answers "shadow".
__device__ __forceinline__ bool descend(const uint32_t* __restrict__ dag, uint32_t words, uint32_t base,
                                        uint32_t off, int level, int min_level, bool leafmasks, int32_t px,
                                        int32_t py, int32_t pz) {
    for (; level >= min_level; --level) {
        if (off >= words) return false;
        const uint32_t c2 = child2(px, py, pz, level);
        const uint32_t m = __ldg(dag + off);
        const uint32_t v = (m >> c2) & 3u;
        if (v != kPartial) return v == kVisible;
        // rank among partial children = popcount of the partial bits below c2
        const uint32_t rank = __popc(m & 0xAAAAu & ((1u << c2) - 1u));
        off = base + __ldg(dag + off + 1u + rank);
    }
    if (!leafmasks) return true;  // unreachable: level 0 has no partial children
    if (off >= words) return false;
    const uint32_t c2 = ((uint32_t)pz & 7u) * 2u;
    const uint32_t m = __ldg(dag + off);
    const uint32_t v = (m >> c2) & 3u;
    if (v != kPartial) return v == kVisible;
    const uint32_t rank = __popc(m & 0xAAAAu & ((1u << c2) - 1u));
    const uint32_t b = ((uint32_t)px & 7u) + 8u * ((uint32_t)py & 7u);
    const uint32_t w = __ldg(dag + off + 1u + 2u * rank + (b >> 5));
    return (w >> (b & 31u)) & 1u;
}

// descend() for a leafmask DAG whose NL inner levels above the leaves are
// known at compile time (the levels below a grid index): the same reads and
// checks, unrolled, with constant shifts.
template <int NL>
__device__ __forceinline__ bool descend_fixed(const uint32_t* __restrict__ dag, uint32_t words, uint32_t base,
                                              uint32_t off, int32_t px, int32_t py, int32_t pz) {
#pragma unroll
    for (int s = 0; s < NL; ++s) {
        const int level = 3 + NL - 1 - s;
        if (off >= words) return false;
        const uint32_t c2 = child2(px, py, pz, level);
        const uint32_t m = __ldg(dag + off);
        const uint32_t v = (m >> c2) & 3u;
        if (v != kPartial) return v == kVisible;
        off = base + __ldg(dag + off + 1u + __popc(m & 0xAAAAu & ((1u << c2) - 1u)));
    }
    if (off >= words) return false;
    const uint32_t c2 = ((uint32_t)pz & 7u) * 2u;
    const uint32_t m = __ldg(dag + off);
    const uint32_t v = (m >> c2) & 3u;
    if (v != kPartial) return v == kVisible;
    const uint32_t rank = __popc(m & 0xAAAAu & ((1u << c2) - 1u));
    const uint32_t b = ((uint32_t)px & 7u) + 8u * ((uint32_t)py & 7u);
    const uint32_t w = __ldg(dag + off + 1u + 2u * rank + (b >> 5));
    return (w >> (b & 31u)) & 1u;
}

// Top grid: cell (cx, cy, cz) at index (cz << 2 depth) | (cy << depth) | cx
// holds the node offset the descent reaches after the `depth` levels below
// the root whose child bits are those of cx, cy, cz (most significant
// first), or a sentinel when it ended in a lit or shadowed child on the way.
__device__ __forceinline__ uint32_t top_cell(int32_t px, int32_t py, int32_t pz, int shift, int depth) {
    const uint32_t m = (1u << depth) - 1u;
    return ((((uint32_t)pz >> shift) & m) << (2 * depth)) | ((((uint32_t)py >> shift) & m) << depth) |
           (((uint32_t)px >> shift) & m);
}

// One thread per cell of depth `depth` - 1: its descent, then the eight
// cells below it from one mask load and up to eight independent pointer
// loads (neighbouring cells share all but their last level, so walking
// each cell alone would repeat the same chain eight times).
__global__ void k_top_index(const uint32_t* __restrict__ dag, uint32_t words, int depth, uint32_t* __restrict__ out) {
    const int dp = depth - 1;
    const uint32_t pcells = 1u << (3 * dp);
    const uint32_t pm = (1u << dp) - 1u;
    for (uint32_t pc = blockIdx.x * blockDim.x + threadIdx.x; pc < pcells; pc += gridDim.x * blockDim.x) {
        const uint32_t px = pc & pm, py = (pc >> dp) & pm, pz = pc >> (2 * dp);
        uint32_t off = 0, entry = 0;
        bool done = false;
        for (int d = 0; d < dp; ++d) {
            const int b = dp - 1 - d;
            const uint32_t c = ((px >> b) & 1u) | (((py >> b) & 1u) << 1) | (((pz >> b) & 1u) << 2);
            if (off >= words) {
                entry = kCellShadow;
                done = true;
                break;
            }
            const uint32_t m = dag[off];
            const uint32_t v = (m >> (2u * c)) & 3u;
            if (v != kPartial) {
                entry = (v == kVisible) ? kCellLit : kCellShadow;
                done = true;
                break;
            }
            off = dag[off + 1u + __popc(m & 0xAAAAu & ((1u << (2u * c)) - 1u))];
        }
        uint32_t m = 0;
        if (!done) {
            if (off >= words) {
                entry = kCellShadow;
                done = true;
            } else {
                m = dag[off];
            }
        }
#pragma unroll
        for (uint32_t c = 0; c < 8; ++c) {
            uint32_t e = entry;
            if (!done) {
                const uint32_t v = (m >> (2u * c)) & 3u;
                e = v == kPartial ? dag[off + 1u + __popc(m & 0xAAAAu & ((1u << (2u * c)) - 1u))]
                                  : (v == kVisible ? kCellLit : kCellShadow);
            }
            const uint32_t cx = 2u * px + (c & 1u), cy = 2u * py + ((c >> 1) & 1u), cz = 2u * pz + (c >> 2);
            out[(cz << (2 * depth)) | (cy << depth) | cx] = e;
        }
    }
}

// Q queries per thread, carried through the levels in lockstep so that each
// level issues Q independent loads (the descent is a chain of dependent
// L1/L2 hits, so memory-level parallelism per thread sets the rate).  Query
// q of a thread is i = (w*Q + q)*32 + lane: each of the Q ballots packs 32
// consecutive queries into one output word.
template <bool NDC, int Q>
__global__ void __launch_bounds__(kThreads)
    k_lookup(const uint32_t* __restrict__ dag, uint32_t words, int num_levels, bool leafmasks,
             const uint32_t* __restrict__ top, int depth, const void* __restrict__ q, uint64_t n,
             uint32_t* __restrict__ bits) {
    const int lane = threadIdx.x & 31;
    const int root = num_levels - 2, min_level = leafmasks ? 3 : 0;
    const int shift = root - depth + 1;  // the top grid takes bits root .. shift of each coordinate
    const uint64_t nwords = (n + 31) / 32;
    const uint64_t ngroups = (nwords + Q - 1) / Q;
    const uint64_t nw = ((uint64_t)gridDim.x * blockDim.x) >> 5;
    const float scale = (float)((1u << (num_levels - 1)) - 1u);
    if (Q == 1) {
        // one query per thread, each descending on its own; the point of the
        // thread's next query is requested before the current one descends
        uint64_t w = ((uint64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
        uint32_t nx = 0, ny = 0, nz = 0;
        auto fetch = [&](uint64_t wq) {
            const uint64_t iq = wq * 32 + (uint64_t)lane;
            if (wq < nwords && iq < n) {
                const uint32_t* p = static_cast<const uint32_t*>(q) + 3 * iq;
                nx = __ldcs(p);
                ny = __ldcs(p + 1);
                nz = __ldcs(p + 2);
            }
        };
        fetch(w);
        for (; w < nwords; w += nw) {
            const uint64_t i = w * 32 + (uint64_t)lane;
            const uint32_t rx = nx, ry = ny, rz = nz;
            fetch(w + nw);
            bool lit = false;
            if (i < n) {
                int32_t px, py, pz;
                if (NDC) {
                    px = quantise(__uint_as_float(rx), scale);
                    py = quantise(__uint_as_float(ry), scale);
                    pz = quantise(__uint_as_float(rz), scale);
                } else {
                    px = (int32_t)rx;
                    py = (int32_t)ry;
                    pz = (int32_t)rz;
                }
                uint32_t off = 0;
                int level = root;
                bool done = false;
                if (depth > 0) {
                    const uint32_t e = __ldg(top + top_cell(px, py, pz, shift, depth));
                    if (e >= kCellLit) {
                        lit = (e == kCellLit);
                        done = true;
                    } else {
                        off = e;
                        level = root - depth;
                    }
                }
                if (!done) lit = descend(dag, words, 0u, off, level, min_level, leafmasks, px, py, pz);
            }
            const uint32_t word = __ballot_sync(0xffffffffu, lit);
            if (lane == 0) __stcs(bits + w, word);
        }
        return;
    }
    for (uint64_t gidx = ((uint64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5; gidx < ngroups; gidx += nw) {
        int32_t px[Q], py[Q], pz[Q];
        uint32_t off[Q];
        bool done[Q], lit[Q];
#pragma unroll
        for (int k = 0; k < Q; ++k) {
            const uint64_t i = (gidx * Q + k) * 32 + (uint64_t)lane;
            done[k] = true;
            lit[k] = false;
            off[k] = 0;
            px[k] = py[k] = pz[k] = 0;
            if (i < n) {
                if (NDC) {
                    const float* p = static_cast<const float*>(q) + 3 * i;
                    px[k] = quantise(__ldcs(p), scale);
                    py[k] = quantise(__ldcs(p + 1), scale);
                    pz[k] = quantise(__ldcs(p + 2), scale);
                } else {
                    const int32_t* p = static_cast<const int32_t*>(q) + 3 * i;
                    px[k] = __ldcs(p);
                    py[k] = __ldcs(p + 1);
                    pz[k] = __ldcs(p + 2);
                }
                done[k] = false;
            }
        }
        int level = root;
        if (depth > 0) {
#pragma unroll
            for (int k = 0; k < Q; ++k) {
                if (done[k]) continue;
                const uint32_t e = __ldg(top + top_cell(px[k], py[k], pz[k], shift, depth));
                if (e >= kCellLit) {
                    lit[k] = (e == kCellLit);
                    done[k] = true;
                } else {
                    off[k] = e;
                }
            }
            level = root - depth;
        }
        for (; level >= min_level; --level) {
            uint32_t m[Q];
#pragma unroll
            for (int k = 0; k < Q; ++k) {
                if (!done[k] && off[k] >= words) {
                    done[k] = true;  // malformed DAG: shadow
                    lit[k] = false;
                }
                m[k] = done[k] ? 0u : __ldg(dag + off[k]);
            }
            uint32_t slot[Q];
#pragma unroll
            for (int k = 0; k < Q; ++k) {
                slot[k] = 0;
                if (done[k]) continue;
                const uint32_t c2 = child2(px[k], py[k], pz[k], level);
                const uint32_t v = (m[k] >> c2) & 3u;
                if (v != kPartial) {
                    lit[k] = (v == kVisible);
                    done[k] = true;
                } else {
                    slot[k] = off[k] + 1u + __popc(m[k] & 0xAAAAu & ((1u << c2) - 1u));
                }
            }
            bool any = false;
#pragma unroll
            for (int k = 0; k < Q; ++k) {
                if (!done[k]) off[k] = __ldg(dag + slot[k]);
                any |= !done[k];
            }
            if (!__any_sync(0xffffffffu, any)) break;
        }
        if (leafmasks) {
            uint32_t m[Q];
#pragma unroll
            for (int k = 0; k < Q; ++k) {
                if (!done[k] && off[k] >= words) {
                    done[k] = true;
                    lit[k] = false;
                }
                m[k] = done[k] ? 0u : __ldg(dag + off[k]);
            }
#pragma unroll
            for (int k = 0; k < Q; ++k) {
                if (done[k]) continue;
                const uint32_t c2 = ((uint32_t)pz[k] & 7u) * 2u;
                const uint32_t v = (m[k] >> c2) & 3u;
                if (v != kPartial) {
                    lit[k] = (v == kVisible);
                } else {
                    const uint32_t rank = __popc(m[k] & 0xAAAAu & ((1u << c2) - 1u));
                    const uint32_t b = ((uint32_t)px[k] & 7u) + 8u * ((uint32_t)py[k] & 7u);
                    const uint32_t w = __ldg(dag + off[k] + 1u + 2u * rank + (b >> 5));
                    lit[k] = (w >> (b & 31u)) & 1u;
                }
            }
        }
#pragma unroll
        for (int k = 0; k < Q; ++k) {
            const uint32_t word = __ballot_sync(0xffffffffu, lit[k]);
            const uint64_t wi = gidx * Q + k;
            if (lane == 0 && wi < nwords) __stcs(bits + wi, word);
        }
    }
}

// The common case in straight-line code: a leafmask DAG with a top grid
// and NL inner levels below it (the c1 workload: levels 4 and 3), fewer
// than 2^31 queries.  The levels are unrolled, each query carries an
// `alive` flag instead of leaving a loop, and indices are 32-bit, so a
// query costs fewer instructions than in k_lookup; Q queries per thread are
// interleaved level by level, so each level issues Q independent loads with
// no lockstep loop around them.  The next group's points are requested
// before the current group descends.  Same answers as k_lookup: every node
// offset is checked against `words` before its mask is read, and the zeroed
// tail keeps a node's pointer and leaf words inside the buffer.
template <bool NDC, int Q, int NL>
__global__ void __launch_bounds__(kThreads)
    k_lookup_fixed(const uint32_t* __restrict__ dag, uint32_t words, int num_levels, const uint32_t* __restrict__ top,
                   int depth, const void* __restrict__ q, uint32_t n, uint32_t* __restrict__ bits) {
    const uint32_t lane = threadIdx.x & 31u;
    const int root = num_levels - 2;
    const int shift = root - depth + 1;  // the top grid takes bits root .. shift of each coordinate
    const int low = shift - NL;          // bit of the last inner level (3)
    const uint32_t nwords = (n + 31u) / 32u;
    const uint32_t ngroups = (nwords + Q - 1u) / Q;
    const uint32_t nw = (gridDim.x * blockDim.x) >> 5;
    const float scale = (float)((1u << (num_levels - 1)) - 1u);
    uint32_t nx[Q] = {}, ny[Q] = {}, nz[Q] = {};
    auto fetch = [&](uint32_t g) {
#pragma unroll
        for (int k = 0; k < Q; ++k) {
            const uint32_t i = (g * Q + k) * 32u + lane;
            if (g < ngroups && i < n) {
                const uint32_t* p = static_cast<const uint32_t*>(q) + 3u * (size_t)i;
                nx[k] = __ldcs(p);
                ny[k] = __ldcs(p + 1);
                nz[k] = __ldcs(p + 2);
            }
        }
    };
    uint32_t g = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    fetch(g);
    for (; g < ngroups; g += nw) {
        // this group's points, then the next group's requested before these
        // are used (two groups' reads in flight while a point arrives)
        uint32_t rx[Q], ry[Q], rz[Q];
#pragma unroll
        for (int k = 0; k < Q; ++k) {
            rx[k] = nx[k];
            ry[k] = ny[k];
            rz[k] = nz[k];
        }
        fetch(g + nw);
        int32_t px[Q], py[Q], pz[Q];
        uint32_t off[Q];
        bool alive[Q], lit[Q];
#pragma unroll
        for (int k = 0; k < Q; ++k) {
            const uint32_t i = (g * Q + k) * 32u + lane;
            if (NDC) {
                px[k] = quantise(__uint_as_float(rx[k]), scale);
                py[k] = quantise(__uint_as_float(ry[k]), scale);
                pz[k] = quantise(__uint_as_float(rz[k]), scale);
            } else {
                px[k] = (int32_t)rx[k];
                py[k] = (int32_t)ry[k];
                pz[k] = (int32_t)rz[k];
            }
            alive[k] = i < n;
            lit[k] = false;
            off[k] = 0;
        }
#pragma unroll
        for (int k = 0; k < Q; ++k) {
            const uint32_t e = alive[k] ? __ldg(top + top_cell(px[k], py[k], pz[k], shift, depth)) : kCellShadow;
            if (e >= kCellLit) {
                lit[k] = alive[k] && e == kCellLit;
                alive[k] = false;
            } else {
                off[k] = e;
            }
        }
#pragma unroll
        for (int s = 0; s < NL; ++s) {
            const int b = NL - 1 - s;  // this level's bit above `low`
            uint32_t m[Q];
#pragma unroll
            for (int k = 0; k < Q; ++k) {
                if (alive[k] && off[k] >= words) alive[k] = false;  // malformed DAG: shadow
                m[k] = alive[k] ? __ldg(dag + off[k]) : 0u;
            }
#pragma unroll
            for (int k = 0; k < Q; ++k) {
                if (!alive[k]) continue;
                const uint32_t c2 = child2(px[k] >> low, py[k] >> low, pz[k] >> low, b);
                const uint32_t v = (m[k] >> c2) & 3u;
                if (v != kPartial) {
                    lit[k] = v == kVisible;
                    alive[k] = false;
                } else {
                    off[k] = __ldg(dag + off[k] + 1u + __popc(m[k] & 0xAAAAu & ((1u << c2) - 1u)));
                }
            }
        }
        // the leaf: slice z & 7, bit (x & 7) + 8 (y & 7) of its mask pair
        uint32_t m[Q];
#pragma unroll
        for (int k = 0; k < Q; ++k) {
            if (alive[k] && off[k] >= words) alive[k] = false;
            m[k] = alive[k] ? __ldg(dag + off[k]) : 0u;
        }
#pragma unroll
        for (int k = 0; k < Q; ++k) {
            if (alive[k]) {
                const uint32_t c2 = ((uint32_t)pz[k] & 7u) * 2u;
                const uint32_t v = (m[k] >> c2) & 3u;
                if (v != kPartial) {
                    lit[k] = v == kVisible;
                } else {
                    const uint32_t rank = __popc(m[k] & 0xAAAAu & ((1u << c2) - 1u));
                    const uint32_t bb = ((uint32_t)px[k] & 7u) + 8u * ((uint32_t)py[k] & 7u);
                    lit[k] = (__ldg(dag + off[k] + 1u + 2u * rank + (bb >> 5)) >> (bb & 31u)) & 1u;
                }
            }
        }
#pragma unroll
        for (int k = 0; k < Q; ++k) {
            const uint32_t word = __ballot_sync(0xffffffffu, lit[k]);
            const uint32_t wi = g * Q + k;
            if (lane == 0 && wi < nwords) __stcs(bits + wi, word);
        }
    }
}

// One grid sample at an integer path (shader/traverse.cs:75-88 routing):
// outside the grid answers lit, a uniform cell its class, else the descent
// of the cell's DAG with pointers relative to its first word.
// With a grid top index (`gtop`, depth `gdepth` levels of every cell DAG;
// see k_grid_top_index) the first levels are one load.
struct GridTop {
    const uint32_t* top;  // null: none
    int depth;            // levels of each cell DAG it resolves
    int bits;             // log2(length) + depth: index bits per axis
};

// NL >= 0: a leafmask grid with an index, NL inner levels below it
// (descend_fixed); -1: any grid.
template <int NL = -1>
__device__ __forceinline__ bool grid_sample(const uint32_t* __restrict__ dag, uint32_t words,
                                            const uint32_t* __restrict__ cells, uint32_t length, int dag_levels,
                                            bool leafmasks, GridTop gt, int64_t px, int64_t py, int64_t pz) {
    const int sh = dag_levels - 1;
    const int64_t lim = (int64_t)length << sh;
    if (px < 0 || py < 0 || pz < 0 || px >= lim || py >= lim || pz >= lim) return true;
    const uint32_t cell = __ldg(cells + ((size_t)(pz >> sh) * length + (size_t)(py >> sh)) * length + (size_t)(px >> sh));
    int level = dag_levels - 2;
    uint32_t off = cell;
    if (gt.top) {
        const int s = sh - gt.depth;
        const uint32_t e = __ldg(gt.top + ((((uint64_t)pz >> s) << (2 * gt.bits)) | (((uint64_t)py >> s) << gt.bits) |
                                           ((uint64_t)px >> s)));
        if (e >= kCellLit) return e == kCellLit;  // uniform cell, or the descent ended in the top levels
        if constexpr (NL >= 0) return descend_fixed<NL>(dag, words, cell, e, (int32_t)px, (int32_t)py, (int32_t)pz);
        off = e;
        level -= gt.depth;
    } else {
        if (cell == kCellShadow) return false;
        if (cell == kCellLit) return true;
    }
    return descend(dag, words, cell, off, level, leafmasks ? 3 : 0, leafmasks, (int32_t)px, (int32_t)py, (int32_t)pz);
}

// Grid top index: entry (gx, gy, gz) at index (gz << 2 bits) | (gy << bits) | gx,
// bits = log2(length) + depth, is the absolute DAG offset of the node that
// the cell's descent reaches after `depth` levels, or a lit / shadow sentinel
// (a uniform cell, or a lit / shadowed child on the way).
__global__ void k_grid_top_index(const uint32_t* __restrict__ dag, uint32_t words,
                                 const uint32_t* __restrict__ cells, uint32_t length, int dag_levels, int depth,
                                 int bits, uint32_t* __restrict__ out) {
    const uint64_t total = 1ull << (3 * bits);
    const uint32_t m = (1u << bits) - 1u;
    for (uint64_t t = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; t < total; t += (uint64_t)gridDim.x * blockDim.x) {
        const uint32_t gx = (uint32_t)t & m, gy = (uint32_t)(t >> bits) & m, gz = (uint32_t)(t >> (2 * bits));
        const uint32_t cell = cells[((size_t)(gz >> depth) * length + (gy >> depth)) * length + (gx >> depth)];
        uint32_t entry;
        if (cell >= kCellLit) {
            entry = cell;
        } else {
            uint32_t off = cell;
            entry = 0;
            bool done = false;
            for (int d = 0; d < depth; ++d) {
                const int b = depth - 1 - d;
                const uint32_t c = ((gx >> b) & 1u) | (((gy >> b) & 1u) << 1) | (((gz >> b) & 1u) << 2);
                if (off >= words) {
                    entry = kCellShadow;
                    done = true;
                    break;
                }
                const uint32_t mk = dag[off];
                const uint32_t v = (mk >> (2u * c)) & 3u;
                if (v != kPartial) {
                    entry = (v == kVisible) ? kCellLit : kCellShadow;
                    done = true;
                    break;
                }
                off = cell + dag[off + 1u + __popc(mk & 0xAAAAu & ((1u << (2u * c)) - 1u))];
            }
            if (!done) entry = off;
        }
        out[t] = entry;
    }
}

// The same index from one thread per entry of resolution bits - 1 (depth
// >= 1): the descent to its node, then its eight entries from one mask load
// and up to eight independent pointer loads.
__global__ void k_grid_top_index_parents(const uint32_t* __restrict__ dag, uint32_t words,
                                         const uint32_t* __restrict__ cells, uint32_t length, int depth, int bits,
                                         uint32_t* __restrict__ out) {
    const int pb = bits - 1, dp = depth - 1;
    const uint64_t total = 1ull << (3 * pb);
    const uint32_t m = (1u << pb) - 1u;
    for (uint64_t t = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; t < total; t += (uint64_t)gridDim.x * blockDim.x) {
        const uint32_t px = (uint32_t)t & m, py = (uint32_t)(t >> pb) & m, pz = (uint32_t)(t >> (2 * pb));
        const uint32_t cell = cells[((size_t)(pz >> dp) * length + (py >> dp)) * length + (px >> dp)];
        uint32_t entry = cell, off = cell, mk = 0;
        bool done = cell >= kCellLit;  // a uniform cell: every entry is its sentinel
        for (int d = 0; d < dp && !done; ++d) {
            const int b = dp - 1 - d;
            const uint32_t c = ((px >> b) & 1u) | (((py >> b) & 1u) << 1) | (((pz >> b) & 1u) << 2);
            if (off >= words) {
                entry = kCellShadow;
                done = true;
                break;
            }
            const uint32_t w = dag[off];
            const uint32_t v = (w >> (2u * c)) & 3u;
            if (v != kPartial) {
                entry = (v == kVisible) ? kCellLit : kCellShadow;
                done = true;
                break;
            }
            off = cell + dag[off + 1u + __popc(w & 0xAAAAu & ((1u << (2u * c)) - 1u))];
        }
        if (!done) {
            if (off >= words) {
                entry = kCellShadow;
                done = true;
            } else {
                mk = dag[off];
            }
        }
#pragma unroll
        for (uint32_t c = 0; c < 8; ++c) {
            uint32_t e = entry;
            if (!done) {
                const uint32_t v = (mk >> (2u * c)) & 3u;
                e = v == kPartial ? cell + dag[off + 1u + __popc(mk & 0xAAAAu & ((1u << (2u * c)) - 1u))]
                                  : (v == kVisible ? kCellLit : kCellShadow);
            }
            const uint64_t gx = 2ull * px + (c & 1u), gy = 2ull * py + ((c >> 1) & 1u), gz = 2ull * pz + (c >> 2);
            out[(gz << (2 * bits)) | (gy << bits) | gx] = e;
        }
    }
}

// Grid routing (shader/traverse.cs:75-88): the path at resolution
// 2^(dag_levels+grid_levels-1), its top bits select the cell, the cell word
// holds the DAG offset or a uniform-cell sentinel; then the cell's descent
// (grid_sample, with the grid top index when there is one).
template <int NL>
__global__ void __launch_bounds__(kThreads)
    k_grid_lookup(const uint32_t* __restrict__ dag, uint32_t words, const uint32_t* __restrict__ cells,
                  uint32_t length, int dag_levels, int grid_levels, bool leafmasks, GridTop gt,
                  const float* __restrict__ q, uint64_t n, uint32_t* __restrict__ bits) {
    const int lane = threadIdx.x & 31;
    const uint64_t nwords = (n + 31) / 32;
    const uint64_t nw = ((uint64_t)gridDim.x * blockDim.x) >> 5;
    const float scale = (float)((1u << (dag_levels + grid_levels - 1)) - 1u);
    for (uint64_t w = ((uint64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5; w < nwords; w += nw) {
        const uint64_t i = w * 32 + (uint64_t)lane;
        bool lit = false;
        if (i < n) {
            const float* p = q + 3 * i;
            const int32_t px = quantise(__ldcs(p), scale), py = quantise(__ldcs(p + 1), scale), pz = quantise(__ldcs(p + 2), scale);
            lit = grid_sample<NL>(dag, words, cells, length, dag_levels, leafmasks, gt, px, py, pz);
        }
        const uint32_t word = __ballot_sync(0xffffffffu, lit);
        if (lane == 0) __stcs(bits + w, word);
    }
}

// World-space evaluation (src/CompressedShadowContainer.cpp:93-124,
// shader/traverse.cs:134-148): pixel i's position p (the first three of its
// `fpp` floats) goes through the column-major light view-projection m as
// c_r = ((m[r]*x + m[4+r]*y) + m[8+r]*z) + m[12+r] (the shader's
// lightViewProj * vec4(p, 1), no contraction), ndc = c.xyz / c.w, then the
// grid lookup.  With filter f > 1, the f x f texel footprint around the
// path (offsets -(f-1)/2 .. f/2 in x and y, same depth voxel) is sampled and
// the lit fraction written as round(255 * lit / f^2) -- percentage-closer
// filtering, which the reference declares (setFilterSize) but never
// implements.  U8: one byte per pixel (0 / 255 when f <= 1, as an r8 image
// stores 0.0 / 1.0); else one bit per pixel, 32 per word.
struct EvalMatrix {
    float m[16];
};

template <bool U8, int NL>
__global__ void __launch_bounds__(kThreads)
    k_grid_evaluate(const uint32_t* __restrict__ dag, uint32_t words, const uint32_t* __restrict__ cells,
                    uint32_t length, int dag_levels, int grid_levels, bool leafmasks, GridTop gt,
                    const float* __restrict__ pos, uint32_t fpp, uint64_t n, EvalMatrix M, int filter,
                    void* __restrict__ out) {
    const int lane = threadIdx.x & 31;
    const uint64_t nwords = (n + 31) / 32;
    const uint64_t nw = ((uint64_t)gridDim.x * blockDim.x) >> 5;
    const float scale = (float)((1u << (dag_levels + grid_levels - 1)) - 1u);
    const int lo = -((filter - 1) / 2), hi = filter / 2;
    const uint32_t f2 = (uint32_t)(filter * filter);
    // four floats per pixel on a 16-byte boundary: one load per position
    const bool vec4 = fpp == 4 && (reinterpret_cast<uintptr_t>(pos) & 15u) == 0;
    float nx = 0.f, ny = 0.f, nz = 0.f;
    auto fetch = [&](uint64_t wq) {
        const uint64_t iq = wq * 32 + (uint64_t)lane;
        if (wq < nwords && iq < n) {
            const float* p = pos + (size_t)fpp * iq;
            if (vec4) {
                const float4 v = __ldcs(reinterpret_cast<const float4*>(p));
                nx = v.x;
                ny = v.y;
                nz = v.z;
            } else {
                nx = __ldcs(p);
                ny = __ldcs(p + 1);
                nz = __ldcs(p + 2);
            }
        }
    };
    uint64_t w = ((uint64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    fetch(w);
    for (; w < nwords; w += nw) {
        const uint64_t i = w * 32 + (uint64_t)lane;
        // this pixel's position, then the next one's requested before this
        // one descends
        const float x = nx, y = ny, z = nz;
        fetch(w + nw);
        bool lit = false;
        uint32_t cnt = 0;
        if (i < n) {
            float c[4];
#pragma unroll
            for (int r = 0; r < 4; ++r)
                c[r] = __fadd_rn(__fadd_rn(__fadd_rn(__fmul_rn(M.m[r], x), __fmul_rn(M.m[4 + r], y)),
                                           __fmul_rn(M.m[8 + r], z)),
                                 M.m[12 + r]);
            const int64_t px = quantise(__fdiv_rn(c[0], c[3]), scale);
            const int64_t py = quantise(__fdiv_rn(c[1], c[3]), scale);
            const int64_t pz = quantise(__fdiv_rn(c[2], c[3]), scale);
            if (filter <= 1) {
                lit = grid_sample<NL>(dag, words, cells, length, dag_levels, leafmasks, gt, px, py, pz);
                cnt = lit ? 1u : 0u;
            } else {
                for (int dy = lo; dy <= hi; ++dy)
                    for (int dx = lo; dx <= hi; ++dx)
                        cnt += grid_sample<NL>(dag, words, cells, length, dag_levels, leafmasks, gt, px + dx,
                                               py + dy, pz)
                                   ? 1u
                                   : 0u;
            }
        }
        if (U8) {
            if (i < n)
                __stcs(static_cast<uint8_t*>(out) + i,
                       filter <= 1 ? (uint8_t)(cnt ? 255u : 0u) : (uint8_t)((255u * cnt + f2 / 2u) / f2));
        } else {
            const uint32_t word = __ballot_sync(0xffffffffu, lit);
            if (lane == 0) __stcs(static_cast<uint32_t*>(out) + w, word);
        }
    }
}

// One query against a table entry: its top grid first when it has one.
__device__ __forceinline__ bool multi_descend(const MultiDag& D, int32_t px, int32_t py, int32_t pz) {
    const int root = (int)D.num_levels - 2, min_level = D.leafmasks ? 3 : 0;
    int level = root;
    uint32_t off = 0;
    if (D.top) {
        const int depth = (int)D.top_depth;
        const uint32_t e = __ldg(D.top + top_cell(px, py, pz, root - depth + 1, depth));
        if (e >= kCellLit) return e == kCellLit;
        off = e;
        level = root - depth;
    }
    return descend(D.dag, D.words, 0u, off, level, min_level, D.leafmasks != 0, px, py, pz);
}

// Many resident DAGs at once: query i descends DAG dags[ids[i]] (its own
// depth and leafmask mode); ids outside the table answer "shadow".
__global__ void __launch_bounds__(kThreads)
    k_multi_lookup(const MultiDag* __restrict__ dags, uint32_t ndags, const uint32_t* __restrict__ ids,
                   const float* __restrict__ q, uint64_t n, uint32_t* __restrict__ bits) {
    const int lane = threadIdx.x & 31;
    const uint64_t nwords = (n + 31) / 32;
    const uint64_t nw = ((uint64_t)gridDim.x * blockDim.x) >> 5;
    for (uint64_t w = ((uint64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5; w < nwords; w += nw) {
        const uint64_t i = w * 32 + (uint64_t)lane;
        bool lit = false;
        if (i < n) {
            const uint32_t id = __ldcs(ids + i);
            if (id < ndags) {
                const MultiDag D = dags[id];
                const float scale = (float)((1u << (D.num_levels - 1)) - 1u);
                const float* p = q + 3 * i;
                const int32_t px = quantise(__ldcs(p), scale), py = quantise(__ldcs(p + 1), scale), pz = quantise(__ldcs(p + 2), scale);
                lit = multi_descend(D, px, py, pz);
            }
        }
        const uint32_t word = __ballot_sync(0xffffffffu, lit);
        if (lane == 0) __stcs(bits + w, word);
    }
}

// Segmented multi-DAG lookup: many independent requests in one launch.
// Segment s owns output words [word_start, word_start + ceil(n/32)); warp w
// finds its segment by binary search and answers 32 of its queries, reading
// the request's points and writing its bits where they lie (device memory,
// or host memory the GPU reads in place).
__global__ void __launch_bounds__(kThreads)
    k_segment_lookup(const MultiDag* __restrict__ dags, uint32_t ndags, const LookupSegment* __restrict__ segs,
                     uint32_t nsegs, uint64_t total_words) {
    const int lane = threadIdx.x & 31;
    const uint64_t nw = ((uint64_t)gridDim.x * blockDim.x) >> 5;
    for (uint64_t w = ((uint64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5; w < total_words; w += nw) {
        uint32_t lo = 0, hi = nsegs;
        while (hi - lo > 1) {
            const uint32_t mid = (lo + hi) / 2;
            if (segs[mid].word_start <= w) lo = mid; else hi = mid;
        }
        const LookupSegment sg = segs[lo];
        const uint64_t lw = w - sg.word_start;
        const uint64_t i = lw * 32 + (uint64_t)lane;
        bool lit = false;
        if (i < sg.n && sg.dag < ndags) {
            const MultiDag D = dags[sg.dag];
            const float scale = (float)((1u << (D.num_levels - 1)) - 1u);
            const float* p = sg.xyz + 3 * i;
            const int32_t px = quantise(__ldcs(p), scale), py = quantise(__ldcs(p + 1), scale), pz = quantise(__ldcs(p + 2), scale);
            lit = multi_descend(D, px, py, pz);
        }
        const uint32_t word = __ballot_sync(0xffffffffu, lit);
        if (lane == 0) __stcs(sg.bits + lw, word);
    }
}

uint32_t lookup_grid(int num_sms, uint64_t n) {
    const uint64_t warps = (n + 31) / 32;
    const uint64_t blocks = (warps * 32 + kThreads - 1) / kThreads;
    const uint64_t cap = (uint64_t)(num_sms > 0 ? num_sms : 152) * 8;
    return (uint32_t)(blocks < 1 ? 1 : (blocks < cap ? blocks : cap));
}

int device_sms() {
    int dev = 0, sms = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    return sms;
}

}  // namespace

int top_index_depth(uint32_t num_levels, bool leafmasks, uint64_t words, uint32_t max_factor) {
    const int root = (int)num_levels - 2, min_level = leafmasks ? 3 : 0;
    int d = root - min_level + 1;
    if (d > kTopIndexDepth) d = kTopIndexDepth;
    // no larger than max_factor times the DAG (at least 64 KiB)
    const uint64_t limit = words * 4 * max_factor > 65536 ? words * 4 * max_factor : 65536;
    while (d > 0 && (uint64_t(4) << (3 * d)) > limit) --d;
    return d < 0 ? 0 : d;
}

cpvs_status launch_top_index(const uint32_t* dag, uint64_t words, int depth, uint32_t* out, cudaStream_t st) {
    if (depth <= 0) return CPVS_OK;
    const uint32_t parents = 1u << (3 * (depth - 1));  // one thread per cell of depth - 1
    k_top_index<<<(parents + 255) / 256, 256, 0, st>>>(dag, (uint32_t)words, depth, out);
    CPVS_CUDA(cudaGetLastError());
    return CPVS_OK;
}

// Inner levels below the top grid that k_lookup_fixed unrolls (0 ..
// kFixedLevels); other DAGs take k_lookup.
constexpr int kFixedLevels = 6;

template <bool NDC, int Q, int NL>
bool launch_fixed_nl(int nl, uint32_t g, cudaStream_t st, const uint32_t* dag, uint64_t words, uint32_t num_levels,
                     const uint32_t* top, int depth, const void* xyz, uint64_t n, uint32_t* bits) {
    if (nl == NL) {
        k_lookup_fixed<NDC, Q, NL><<<g, kThreads, 0, st>>>(dag, (uint32_t)words, (int)num_levels, top, depth, xyz,
                                                           (uint32_t)n, bits);
        return true;
    }
    if constexpr (NL < kFixedLevels) {
        return launch_fixed_nl<NDC, Q, NL + 1>(nl, g, st, dag, words, num_levels, top, depth, xyz, n, bits);
    } else {
        return false;
    }
}

template <bool NDC, int Q>
void launch_lookup_q(uint32_t g, cudaStream_t st, const uint32_t* dag, uint64_t words, uint32_t num_levels,
                     bool leafmasks, const uint32_t* top, int depth, const void* xyz, uint64_t n, uint32_t* bits) {
    // the straight-line kernel where it applies: leafmasks, a top grid, at
    // most kFixedLevels inner levels below it, fewer than 2^31 queries
    const int nl = (int)num_levels - 2 - depth - 3 + 1;
    if (Q <= 2 && leafmasks && top && depth > 0 && nl >= 0 && n < (1ull << 31) &&
        launch_fixed_nl<NDC, (Q <= 2 ? Q : 2), 0>(nl, g, st, dag, words, num_levels, top, depth, xyz, n, bits))
        return;
    k_lookup<NDC, Q><<<g, kThreads, 0, st>>>(dag, (uint32_t)words, (int)num_levels, leafmasks, top, depth, xyz, n,
                                             bits);
}

cpvs_status launch_lookup(const uint32_t* dag, uint64_t words, uint32_t num_levels, bool leafmasks,
                          const uint32_t* top, int top_depth, const void* xyz, bool ndc, uint64_t n, uint32_t* bits,
                          cudaStream_t st, Timing* timing, int queries_per_thread) {
    if (n == 0) return CPVS_OK;
    KernelTimer kt(timing, K_LOOKUP, st);
    const int Q = (queries_per_thread == 1 || queries_per_thread == 2) ? queries_per_thread : 4;
    const uint32_t g = lookup_grid(device_sms(), (n + Q - 1) / Q);
    const int depth = top ? top_depth : 0;
    if (ndc) {
        if (Q == 1) launch_lookup_q<true, 1>(g, st, dag, words, num_levels, leafmasks, top, depth, xyz, n, bits);
        else if (Q == 2) launch_lookup_q<true, 2>(g, st, dag, words, num_levels, leafmasks, top, depth, xyz, n, bits);
        else launch_lookup_q<true, 4>(g, st, dag, words, num_levels, leafmasks, top, depth, xyz, n, bits);
    } else {
        if (Q == 1) launch_lookup_q<false, 1>(g, st, dag, words, num_levels, leafmasks, top, depth, xyz, n, bits);
        else if (Q == 2) launch_lookup_q<false, 2>(g, st, dag, words, num_levels, leafmasks, top, depth, xyz, n, bits);
        else launch_lookup_q<false, 4>(g, st, dag, words, num_levels, leafmasks, top, depth, xyz, n, bits);
    }
    CPVS_CUDA(cudaGetLastError());
    return CPVS_OK;
}

int tune_lookup(const uint32_t* dag, uint64_t words, uint32_t num_levels, bool leafmasks, const uint32_t* top,
                int top_depth, const void* xyz, bool ndc, uint64_t n, uint32_t* bits, cudaStream_t st) {
    // up to 2^24 queries (~0.1 ms per launch), best of three timed runs
    // after a warm-up, so that launch-to-launch noise does not pick the
    // variant.  The sample's 201 MB of points exceed L2 as a large batch's do:
    // a sample that stays in L2 after the warm-up favours the variants that
    // hide latency over the one that streams best.  A batch may be ordered
    // (surface points first, say), so a large one is sampled in four chunks
    // spread over it: chunk c starts at c*n/4 rounded down to a whole answer
    // word; chunks of sample/4 (a multiple of 32, at most n/4) end inside the
    // batch and its answer words.
    const uint64_t sample = n < (1ull << 24) ? n : (1ull << 24);
    const int chunks = n > sample ? 4 : 1;
    const uint64_t per = chunks == 1 ? sample : (sample / chunks) & ~31ull;
    const size_t qbytes = 12;  // three floats or three int32 per query
    cudaEvent_t a = nullptr, b = nullptr;
    if (cudaEventCreate(&a) != cudaSuccess || cudaEventCreate(&b) != cudaSuccess) {
        cudaGetLastError();
        return 4;
    }
    int best = 4;
    float best_ms = 1e30f;
    for (int q : {1, 2, 4}) {
        float ms = 1e30f;
        for (int rep = 0; rep < 4; ++rep) {  // the first run warms the caches
            float t = 0.f;
            cudaEventRecord(a, st);
            for (int c = 0; c < chunks; ++c) {
                const uint64_t off = (n / chunks * c) & ~31ull;
                launch_lookup(dag, words, num_levels, leafmasks, top, top_depth,
                              static_cast<const char*>(xyz) + off * qbytes, ndc, per, bits + off / 32, st, nullptr, q);
            }
            cudaEventRecord(b, st);
            cudaEventSynchronize(b);
            cudaEventElapsedTime(&t, a, b);
            if (rep > 0 && t < ms) ms = t;
        }
        if (ms < best_ms) {
            best_ms = ms;
            best = q;
        }
    }
    cudaEventDestroy(a);
    cudaEventDestroy(b);
    cudaGetLastError();
    return best;
}

cpvs_status launch_multi_lookup(const MultiDag* dags, uint32_t ndags, const uint32_t* ids, const float* xyz, uint64_t n,
                                uint32_t* bits, cudaStream_t st, Timing* timing) {
    if (n == 0) return CPVS_OK;
    KernelTimer kt(timing, K_MULTI_LOOKUP, st);
    k_multi_lookup<<<lookup_grid(device_sms(), n), kThreads, 0, st>>>(dags, ndags, ids, xyz, n, bits);
    CPVS_CUDA(cudaGetLastError());
    return CPVS_OK;
}

cpvs_status launch_segment_lookup(const MultiDag* dags, uint32_t ndags, const LookupSegment* segs, uint32_t nsegs,
                                  uint64_t total_words, cudaStream_t st, Timing* timing) {
    if (total_words == 0 || nsegs == 0) return CPVS_OK;
    KernelTimer kt(timing, K_MULTI_LOOKUP, st);
    k_segment_lookup<<<lookup_grid(device_sms(), total_words * 32), kThreads, 0, st>>>(dags, ndags, segs, nsegs,
                                                                                     total_words);
    CPVS_CUDA(cudaGetLastError());
    return CPVS_OK;
}

int grid_top_depth(uint32_t length, uint32_t dag_levels, bool leafmasks, uint64_t words) {
    const int root = (int)dag_levels - 2, min_level = leafmasks ? 3 : 0;
    const int gl = log2_u32(length);
    int d = root - min_level + 1;
    if (d > kTopIndexDepth) d = kTopIndexDepth;
    // no larger than 8x the combined DAG (at least 64 KiB, at most 64 MiB),
    // as a shadow's own top grid: one more level in the index (8 instead of
    // 7 for an 8192^2 map's 9.4 MB DAG) took a 4K frame's evaluate from
    // 0.147 to 0.126 ms
    uint64_t limit = words * 32 > 65536 ? words * 32 : 65536;
    if (limit > (64ull << 20)) limit = 64ull << 20;
    while (d > 0 && (uint64_t(4) << (3 * (gl + d))) > limit) --d;
    return d < 0 ? 0 : d;
}

// Inner levels below a grid index that the grid kernels unroll (0 ..
// kFixedLevels), or -1: leafmask cell DAGs with an index only.
int grid_fixed_levels(uint32_t dag_levels, bool leafmasks, const GridTop& gt) {
    if (!leafmasks || !gt.top || gt.depth <= 0) return -1;
    const int nl = (int)dag_levels - 2 - gt.depth - 3 + 1;
    return nl >= 0 && nl <= kFixedLevels ? nl : -1;
}

// Calls f(std::integral_constant<int, nl>) for nl in [NL, kFixedLevels];
// false when nl is outside.
template <int NL, typename F>
bool dispatch_levels(int nl, F&& f) {
    if (nl == NL) {
        f(std::integral_constant<int, NL>());
        return true;
    }
    if constexpr (NL < kFixedLevels) {
        return dispatch_levels<NL + 1>(nl, f);
    } else {
        return false;
    }
}

cpvs_status launch_grid_top_index(const uint32_t* dag, uint64_t words, const uint32_t* cells, uint32_t length,
                                  uint32_t dag_levels, int depth, uint32_t* out, cudaStream_t st) {
    const int bits = log2_u32(length) + depth;
    if (depth >= 1) {
        const uint64_t parents = 1ull << (3 * (bits - 1));
        const uint32_t g = (uint32_t)std::min<uint64_t>((parents + 255) / 256, 152ull * 32);
        k_grid_top_index_parents<<<g, 256, 0, st>>>(dag, (uint32_t)words, cells, length, depth, bits, out);
    } else {
        const uint64_t total = 1ull << (3 * bits);
        const uint32_t g = (uint32_t)std::min<uint64_t>((total + 255) / 256, 152ull * 32);
        k_grid_top_index<<<g, 256, 0, st>>>(dag, (uint32_t)words, cells, length, (int)dag_levels, depth, bits, out);
    }
    CPVS_CUDA(cudaGetLastError());
    return CPVS_OK;
}

cpvs_status launch_grid_evaluate(const uint32_t* dag, uint64_t words, const uint32_t* cells, uint32_t length,
                                 uint32_t dag_levels, bool leafmasks, const uint32_t* gtop, int gdepth,
                                 const float* positions, uint32_t fpp, uint64_t n, const float* light_view_proj,
                                 uint32_t filter, bool u8, void* out, cudaStream_t st, Timing* timing) {
    const GridTop gt{gtop, gtop ? gdepth : 0, (int)log2_u32(length) + (gtop ? gdepth : 0)};
    if (n == 0) return CPVS_OK;
    KernelTimer kt(timing, K_EVALUATE, st);
    EvalMatrix M;
    for (int k = 0; k < 16; ++k) M.m[k] = light_view_proj[k];
    const uint32_t g = lookup_grid(device_sms(), n);
    const int gl = log2_u32(length);
    auto launch = [&](auto nlc) {
        constexpr int NLv = decltype(nlc)::value;
        if (u8)
            k_grid_evaluate<true, NLv><<<g, kThreads, 0, st>>>(dag, (uint32_t)words, cells, length, (int)dag_levels,
                                                               gl, leafmasks, gt, positions, fpp, n, M, (int)filter,
                                                               out);
        else
            k_grid_evaluate<false, NLv><<<g, kThreads, 0, st>>>(dag, (uint32_t)words, cells, length,
                                                                (int)dag_levels, gl, leafmasks, gt, positions, fpp, n,
                                                                M, (int)filter, out);
    };
    if (!dispatch_levels<0>(grid_fixed_levels(dag_levels, leafmasks, gt), launch))
        launch(std::integral_constant<int, -1>());
    CPVS_CUDA(cudaGetLastError());
    return CPVS_OK;
}

cpvs_status launch_grid_lookup(const uint32_t* dag, uint64_t words, const uint32_t* cells, uint32_t length,
                               uint32_t dag_levels, bool leafmasks, const uint32_t* gtop, int gdepth, const float* xyz,
                               uint64_t n, uint32_t* bits, cudaStream_t st, Timing* timing) {
    if (n == 0) return CPVS_OK;
    KernelTimer kt(timing, K_GRID_LOOKUP, st);
    const GridTop gt{gtop, gtop ? gdepth : 0, (int)log2_u32(length) + (gtop ? gdepth : 0)};
    const uint32_t g = lookup_grid(device_sms(), n);
    auto launch = [&](auto nlc) {
        k_grid_lookup<decltype(nlc)::value><<<g, kThreads, 0, st>>>(dag, (uint32_t)words, cells, length,
                                                                    (int)dag_levels, log2_u32(length), leafmasks, gt,
                                                                    xyz, n, bits);
    };
    if (!dispatch_levels<0>(grid_fixed_levels(dag_levels, leafmasks, gt), launch))
        launch(std::integral_constant<int, -1>());
    CPVS_CUDA(cudaGetLastError());
    return CPVS_OK;
}

}  // namespace cpvs
