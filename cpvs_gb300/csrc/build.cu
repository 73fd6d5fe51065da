// Sparse-voxel-DAG build of one or many shadow z-tiles on the device.
//
// Replaces CompressedShadow::create (src/CompressedShadow.cpp:49-59):
// constructSvo + constructLastLevels (:87-190), mergeCommonSubtrees with
// cs::mergeLevel (:215-259, src/CompressedShadowUtil.h:137-182),
// removeUnusedNodes (:261-304) and compress (:306-392).  The DAG words equal
// the reference's whenever its own build is defined.
//
// The reference's output is fully determined by three facts, which the
// kernels below reproduce level-synchronously instead of with pointer
// rewriting:
//   1. the SVO lists every level's nodes in breadth-first order (parents in
//      order, children in child-index order x | y<<1 | z<<2);
//   2. the merge keeps, per level, the FIRST occurrence of each distinct
//      node, where a node is its 16-bit mask plus the merged identities of
//      its children (inner levels) or its mask plus 64-bit leafmasks
//      (leaf level), and
//   3. the final array holds the levels top-down, each level's kept nodes in
//      first-occurrence order, an inner node as 1+k words (mask, absolute
//      child offsets) and a leaf as 1+2k words (mask, lo/hi of each partial
//      slice's leafmask).
//
// Pipeline per build (all DAGs of a batch at once; each node carries its
// job id and never merges across jobs), captured once per plan as a CUDA
// graph of chained (programmatic dependent) launches:
//   k_clear                 per-build counters, look-back flags and tickets
//   top-down expansion:     k_expand_cluster for the levels of at most the
//                           plan's cluster cap of nodes (one thread-block
//                           cluster), then k_expand_lb per level (classify,
//                           block scan + decoupled look-back, write
//                           children)                  -- breadth-first order
//   leaf level (beside the expansion, from the map and pyramid level 3):
//                           k_leaf_columns + k_leaf_columns_heavy (runs of
//                           equal leaves per texel column), k_leaf_classes
//                           (hash insert of the non-uniform runs' classes);
//                           then k_leaf_resolve (each listed leaf's class)
//   bottom-up merge:        k_dedup_insert per inner level (open-addressing
//                           hash; a class's slot is its merged identity,
//                           atomicMin keeps its first occurrence), with
//                           k_merge_scan_lb per level on a forked stream
//                           (ranks and word offsets of the kept nodes), and
//                           k_merge_cluster for the cluster levels
//   layout:                 k_layout (per-job level bases, root masks)
// then one host synchronisation (the DAG's size) and k_emit_all.  Every
// look-back wait is bounded in time and reports an error bit instead of
// hanging.  The allocation-free build at the end of this file uses separate
// multi-pass kernels (k_expand_count/k_expand_write, k_leaf_masks,
// k_dedup_insert/resolve/scan/remap, k_emit) that need no plan.
#include <algorithm>
#include <cstring>
#include <string>

#include <cooperative_groups.h>

#include "common.cuh"

namespace cpvs {
namespace {

namespace cg = cooperative_groups;

constexpr int kThreads = 256;

// Zeroes up to four byte ranges (each starting 16-byte aligned) in one launch.
struct ClearRanges {
    char* p[4];
    uint64_t n[4];
};
__global__ void __launch_bounds__(kThreads) k_clear(ClearRanges r) {
    chain_enter();
    const uint64_t t = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x, stride = (uint64_t)gridDim.x * blockDim.x;
#pragma unroll
    for (int k = 0; k < 4; ++k) {
        uint4* q = reinterpret_cast<uint4*>(r.p[k]);
        const uint64_t nv = r.n[k] / 16;
        for (uint64_t i = t; i < nv; i += stride) q[i] = make_uint4(0u, 0u, 0u, 0u);
        for (uint64_t i = nv * 16 + t; i < r.n[k]; i += stride) r.p[k][i] = 0;
    }
}

struct JobDev {
    const float2* pyr;  // pyramid levels 1..log2(n)
    const float* depth;  // level 0
    uint32_t n, num_levels, z_idx, z_num;
    uint32_t group;      // leaf column group of its source (build plans with leafmasks)
    uint32_t pad;
    uint64_t col_base;   // that group's first column record
};

// Per-level node arrays (capacity `cap`).
struct LevelDev {
    uint64_t* coord;   // packed node coordinate at this level
    uint32_t* job;
    uint32_t* mask;
    uint32_t* first;   // index of the first child in the level below
    uint32_t* uid;     // single-call builds: representative, then rank among the level's kept nodes
    uint32_t* slot;    // hash slot of the node's class: its merged identity for the level above
    uint32_t* uniq;    // rank -> node index of the first occurrence
    uint32_t* woff;    // rank -> word offset (running over the level)
    uint64_t* slices;  // leaf level: 8 leafmasks per node
    uint64_t* hash;    // leaf level: signature hash per node
    unsigned long long* table;  // this level's hash slots (build plans): after
                                // the merge, (rank << 32 | representative)
    uint64_t table_mask;        // slots - 1
};

// Per-job, per-level bookkeeping of segment boundaries (jobs are contiguous
// in every level).
struct SegDev {
    uint32_t* nstart;  // [job * L_MAX + level]
    uint32_t* nend;
    uint32_t* ustart;
    uint32_t* uend;
    uint32_t* wstart;
    uint32_t* wend;
};

struct Injected {  // a job's root, entering at its root level
    uint64_t coord;
    uint32_t job;
    uint32_t pad;
};

__device__ __forceinline__ uint32_t seg_index(uint32_t job, int L) { return job * CPVS_MAX_LEVELS + (uint32_t)L; }

// cs::createChildmask (src/CompressedShadowUtil.cpp:20-54) for the node at
// `c` (level-L texel units): children x|y<<1|z<<2 over the 2x2 texels of
// level L and z-cells z, z+1; 2 bits each (01 lit, 00 shadow, 10 partial).
// Level 0 uses cs::absoluteVisible and never yields partial children.
// A node whose 2x2 texels would fall outside its level (only possible after
// an internal check already failed) reads nothing and yields mask 0.
__device__ __forceinline__ uint32_t node_mask(const JobDev& J, int L, uint64_t c, uint32_t* err) {
    const uint32_t x = unpack_x(c), y = unpack_y(c), z = unpack_z(c);
    const uint32_t W = J.n >> L;
    if (x + 1u >= W || y + 1u >= W) {
        atomicOr(err, 4u);
        return 0u;
    }
    const float H = __uint2float_rn((J.n >> L) * J.z_num);
    float mn[4], mx[4];
    if (L == 0) {
        const float2 r0 = *reinterpret_cast<const float2*>(J.depth + (size_t)y * J.n + x);
        const float2 r1 = *reinterpret_cast<const float2*>(J.depth + (size_t)(y + 1) * J.n + x);
        mn[0] = mx[0] = r0.x;
        mn[1] = mx[1] = r0.y;
        mn[2] = mx[2] = r1.x;
        mn[3] = mx[3] = r1.y;
    } else {
        const float2* P = J.pyr + pyramid_level_offset_dev(J.n, L);
        const float4 r0 = *reinterpret_cast<const float4*>(P + (size_t)y * W + x);
        const float4 r1 = *reinterpret_cast<const float4*>(P + (size_t)(y + 1) * W + x);
        mn[0] = r0.x; mx[0] = r0.y;
        mn[1] = r0.z; mx[1] = r0.w;
        mn[2] = r1.x; mx[2] = r1.y;
        mn[3] = r1.z; mx[3] = r1.w;
    }
    uint32_t m = 0;
#pragma unroll
    for (uint32_t ch = 0; ch < 8; ++ch) {
        const uint32_t t = ch & 3u, zc = z + (ch >> 2);
        uint32_t v;
        if (L > 0)
            v = classify_cell(zc, __fmul_rn(mn[t], H), __fmul_rn(mx[t], H));
        else
            v = voxel_lit(zc, __fmul_rn(mn[t], H)) ? kVisible : kShadow;
        m |= v << (2u * ch);
    }
    return m;
}

// node_mask without side effects: a node whose 2x2 texels fall outside its
// level sets `bad` (the caller reports error bit 4) and yields mask 0.
__device__ __forceinline__ uint32_t node_mask_nf(const JobDev& J, int L, uint64_t c, bool& bad) {
    const uint32_t x = unpack_x(c), y = unpack_y(c), z = unpack_z(c);
    const uint32_t W = J.n >> L;
    if (x + 1u >= W || y + 1u >= W) {
        bad = true;
        return 0u;
    }
    const float H = __uint2float_rn((J.n >> L) * J.z_num);
    float mn[4], mx[4];
    if (L == 0) {
        const float2 r0 = *reinterpret_cast<const float2*>(J.depth + (size_t)y * J.n + x);
        const float2 r1 = *reinterpret_cast<const float2*>(J.depth + (size_t)(y + 1) * J.n + x);
        mn[0] = mx[0] = r0.x;
        mn[1] = mx[1] = r0.y;
        mn[2] = mx[2] = r1.x;
        mn[3] = mx[3] = r1.y;
    } else {
        const float2* P = J.pyr + pyramid_level_offset_dev(J.n, L);
        const float4 r0 = __ldg(reinterpret_cast<const float4*>(P + (size_t)y * W + x));
        const float4 r1 = __ldg(reinterpret_cast<const float4*>(P + (size_t)(y + 1) * W + x));
        mn[0] = r0.x; mx[0] = r0.y;
        mn[1] = r0.z; mx[1] = r0.w;
        mn[2] = r1.x; mx[2] = r1.y;
        mn[3] = r1.z; mx[3] = r1.w;
    }
    uint32_t m = 0;
#pragma unroll
    for (uint32_t ch = 0; ch < 8; ++ch) {
        const uint32_t t = ch & 3u, zc = z + (ch >> 2);
        uint32_t v;
        if (L > 0)
            v = classify_cell(zc, __fmul_rn(mn[t], H), __fmul_rn(mx[t], H));
        else
            v = voxel_lit(zc, __fmul_rn(mn[t], H)) ? kVisible : kShadow;
        m |= v << (2u * ch);
    }
    return m;
}

// node_mask_nf for L > 0 with the level's texels at P (W x W, global or
// shared memory).
__device__ __forceinline__ uint32_t node_mask_at(const float2* P, uint32_t W, float H, uint64_t c, bool& bad) {
    const uint32_t x = unpack_x(c), y = unpack_y(c), z = unpack_z(c);
    if (x + 1u >= W || y + 1u >= W) {
        bad = true;
        return 0u;
    }
    const float4 r0 = *reinterpret_cast<const float4*>(P + (size_t)y * W + x);
    const float4 r1 = *reinterpret_cast<const float4*>(P + (size_t)(y + 1) * W + x);
    const float mn[4] = {r0.x, r0.z, r1.x, r1.z}, mx[4] = {r0.y, r0.w, r1.y, r1.w};
    uint32_t m = 0;
#pragma unroll
    for (uint32_t ch = 0; ch < 8; ++ch) {
        const uint32_t t = ch & 3u, zc = z + (ch >> 2);
        m |= classify_cell(zc, __fmul_rn(mn[t], H), __fmul_rn(mx[t], H)) << (2u * ch);
    }
    return m;
}

// Asynchronous block-wide copy of `bytes` (rounded up to 16) from global to
// shared memory, both 16-byte aligned; the source array must extend to the
// rounded size (arena arrays are padded to 256 bytes).  The copies bypass L1
// (data written by other blocks of the launch is read from L2); fetch_wait
// completes every copy the block issued.
__device__ __forceinline__ void fetch_async(void* dst, const void* src, uint32_t bytes) {
    const uint32_t n16 = (bytes + 15u) / 16u;
    const uint32_t d = (uint32_t)__cvta_generic_to_shared(dst);
    const char* g = static_cast<const char*>(src);
    for (uint32_t k = threadIdx.x; k < n16; k += blockDim.x)
        asm volatile("cp.async.cg.shared.global [%0], [%1], 16;" ::"r"(d + 16u * k), "l"(g + 16u * k) : "memory");
}
__device__ __forceinline__ void fetch_wait() {
    asm volatile("cp.async.wait_all;" ::: "memory");
    __syncthreads();
}

// ---------------------------------------------------------------- top-down
// The multi-pass kernels (k_expand_count, k_expand_write, k_classify_bottom,
// k_leaf_masks, k_dedup_insert<true>, k_dedup_resolve, k_dedup_scan,
// k_dedup_remap, k_emit) serve only the allocation-free build
// (cpvs_shadow_build_noalloc, at the end of this file): it has no plan, so
// no look-back flags or tickets.  Changes to the node layout or the error
// bits of the main path must be mirrored in them.
//
// Pass 1: per-CTA sum of partial children over its chunk of level L.
__global__ void __launch_bounds__(kThreads)
    k_expand_count(LevelDev cur, const uint32_t* __restrict__ counts, const JobDev* __restrict__ jobs, uint32_t njobs,
                   int L, uint2* partials, uint32_t* err) {
    __shared__ uint64_t red[32];
    uint32_t b, e;
    block_chunk(counts[L], b, e);
    uint64_t s = 0;
    for (uint32_t i = b + threadIdx.x; i < e; i += blockDim.x) {
        const uint32_t j = cur.job[i];
        uint32_t m = 0;
        if (j < njobs) {
            m = node_mask(jobs[j], L, cur.coord[i], err);
        } else {
            atomicOr(err, 8u);
            cur.job[i] = 0;  // keep later passes' job lookups in range
        }
        cur.mask[i] = m;
        s += partial_children(m);
    }
    s = block_sum_u64(s, red);
    if (threadIdx.x == 0) partials[blockIdx.x] = make_uint2((uint32_t)s, 0u);
}

// Pass 2: scan the partials, then write first[], the children's coordinates
// and jobs (children after the `ninj` roots that enter level L-1), and the
// level L-1 count.  Also records each job's node range at level L.
__global__ void __launch_bounds__(kThreads)
    k_expand_write(LevelDev cur, LevelDev nxt, uint32_t* counts, int L, const uint2* __restrict__ partials,
                   const Injected* __restrict__ inj, uint32_t ninj, SegDev seg, uint32_t cap_next, uint32_t* err) {
    __shared__ uint32_t sm[64];
    const uint32_t n = counts[L];
    uint32_t b, e;
    block_chunk(n, b, e);
    uint32_t run = ninj + block_prefix_of_partials(partials, blockIdx.x, sm).x;
    if (blockIdx.x == gridDim.x - 1 && threadIdx.x == 0) {
        // total children = prefix of the last block + its own partial; a
        // level never counts more nodes than it can hold
        const uint32_t total = run + partials[blockIdx.x].x;
        if (total > cap_next) atomicOr(err, 1u);
        counts[L - 1] = total < cap_next ? total : cap_next;
    }
    if (blockIdx.x == 0)
        for (uint32_t r = threadIdx.x; r < ninj; r += blockDim.x) {
            nxt.coord[r] = inj[r].coord;
            nxt.job[r] = inj[r].job;
        }
    for (uint32_t t0 = b; t0 < e; t0 += blockDim.x) {
        const uint32_t i = t0 + threadIdx.x;
        const bool valid = i < e;
        const uint32_t m = valid ? cur.mask[i] : 0u;
        const uint32_t k = partial_children(m);
        uint2 tot;
        const uint2 p = block_exclusive_scan2(make_uint2(k, 0u), tot, sm);
        if (valid && run + p.x + k > cap_next) {
            // more children than the level bound: drop them (the count
            // already includes them; their slots keep stale coordinates,
            // which node_mask rejects) and report
            atomicOr(err, 1u);
            cur.mask[i] = m & 0x5555u;
            cur.first[i] = 0;
        } else if (valid) {
            const uint32_t f = run + p.x;
            cur.first[i] = f;
            const uint64_t c = cur.coord[i];
            const uint32_t x = unpack_x(c), y = unpack_y(c), z = unpack_z(c), j = cur.job[i];
            uint32_t r = 0;
#pragma unroll
            for (uint32_t ch = 0; ch < 8; ++ch)
                if (m & (2u << (2u * ch))) {
                    // cs::getChildCoordinates (src/CompressedShadowUtil.cpp:101-117)
                    nxt.coord[f + r] = pack_xyz((x + (ch & 1u)) * 2u, (y + ((ch >> 1) & 1u)) * 2u, (z + (ch >> 2)) * 2u);
                    nxt.job[f + r] = j;
                    ++r;
                }
            if (i == 0 || cur.job[i - 1] != j) seg.nstart[seg_index(j, L)] = i;
            if (i == n - 1 || cur.job[i + 1] != j) seg.nend[seg_index(j, L)] = i + 1;
        }
        run += tot.x;
    }
}

// Bottom level without leafmasks (level 0): masks only, no children.
__global__ void __launch_bounds__(kThreads)
    k_classify_bottom(LevelDev cur, const uint32_t* __restrict__ counts, const JobDev* __restrict__ jobs,
                      uint32_t njobs, int L, SegDev seg, uint32_t* err) {
    chain_enter();
    const uint32_t n = counts[L];
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        const uint32_t j = cur.job[i];
        if (j >= njobs) {
            atomicOr(err, 8u);
            cur.mask[i] = 0;
            cur.job[i] = 0;
            continue;
        }
        cur.mask[i] = node_mask(jobs[j], L, cur.coord[i], err);
        if (i == 0 || cur.job[i - 1] != j) seg.nstart[seg_index(j, L)] = i;
        if (i == n - 1 || cur.job[i + 1] != j) seg.nend[seg_index(j, L)] = i + 1;
    }
}

// Leaf level (level 2 with leafmasks): createChildmask1x1x8 + createLeafmask
// (src/CompressedShadowUtil.cpp:59-99).  The leaf at level-2 coordinate c
// covers voxels x in [4c.x, 4c.x+8), y likewise, z in [bz, bz+8) with
// bz = 4c.z; slice s gets bit x+8y when the voxel centre lies at or above the
// depth: mid(bz+s) <= d*H0, with mid(z) = (z + (z+1)) * 0.5 in float32
// (cs::absoluteVisible).  For z < 2^23 that midpoint is exactly z + 0.5, so
// a texel is lit in the slices s < k, k = clamp(Z - bz + 1, 0, 8), where
// Z = floor(d*H0 - 0.5) is the highest lit voxel of that texel column: the
// same comparisons the reference makes, taken eight at a time.
//
// One thread per leaf: 16 independent 16-byte loads cover the 8x8 depth
// footprint; the four bits of each texel's k are packed into four 64-bit
// planes, from which the eight slice masks follow by bit logic
// (slice s = {t : k_t > s}).
// Lit voxels among z = bz .. bz+7 of a texel with v = fl(d * H0): voxel z is
// lit iff z + 0.5 <= v (src/CompressedShadowUtil.h:35-57), so the count is
// clamp(floor(x), 0, 8) with x = v - (bz + 0.5) + 1, exactly.  Two roundings
// toward minus infinity give it without a float-to-int conversion:
//   w = sat(fl_down(x / 8))  -- one fused multiply-add, v * 0.125 plus the
//       exact constant (0.5 - bz) * 0.125; scaling by 1/8 is exact, so
//       floor(8 w) = floor(fl_down(x)) = floor(x) for x in [0, 8], the
//       saturation clamps to [0, 1] and sends NaN to 0 (as z + 0.5 <= NaN is
//       false);
//   fl_down(8 w + 1.5 * 2^23): the unit in the last place there is 1, so
//       the sum is 1.5 * 2^23 + floor(8 w) and its bit pattern is
//       0x4B400000 + count (count in the low four bits).
// `s` is 0.125 for v = fl(d * H0).  When H0 is a power of two, d * H0 is
// exact (a power-of-two scaling neither rounds nor, for H0 >= 1,
// underflows; an overflow to infinity saturates alike), so the raw depth d
// with s = H0 / 8 gives the same fused result without the product.
__device__ __forceinline__ uint32_t lit_count_bits(float v, float s, float c8) {
    float w;
    asm("fma.rm.sat.f32 %0, %1, %2, %3;" : "=f"(w) : "f"(v), "f"(s), "f"(c8));
    return __float_as_uint(__fmaf_rd(w, 8.0f, 12582912.0f));
}
constexpr uint32_t kCountBias = 0x4B400000u;

// Eight counts as nibbles (texel x at bits 4x..4x+3) -> four bytes, byte b
// holding bit b of every texel's count (texel x at bit x): the bit-index
// rotation (x2 x1 x0 b1 b0) -> (b1 b0 x2 x1 x0) as four delta swaps.
__device__ __forceinline__ uint32_t delta_swap(uint32_t x, uint32_t m, int d) {
    const uint32_t t = ((x >> d) ^ x) & m;
    return x ^ t ^ (t << d);
}
__device__ __forceinline__ uint32_t nibbles_to_planes(uint32_t w) {
    w = delta_swap(w, 0x22222222u, 1);
    w = delta_swap(w, 0x0a0a0a0au, 3);
    w = delta_swap(w, 0x00cc00ccu, 6);
    return delta_swap(w, 0x0000f0f0u, 12);
}

// Per texel row of a leaf: the eight lit counts as nibbles (texel x at bits
// 4x..4x+3).
template <bool POW2>
__device__ __forceinline__ void leaf_rows(const float* row0, uint32_t nmap, float H, float c8, uint32_t W[8]) {
    const float s = POW2 ? __fmul_rn(H, 0.125f) : 0.125f;
#pragma unroll
    for (int y = 0; y < 8; ++y) {
        const float4 a = __ldg(reinterpret_cast<const float4*>(row0 + (size_t)y * nmap));
        const float4 b = __ldg(reinterpret_cast<const float4*>(row0 + (size_t)y * nmap + 4));
        const float v[8] = {a.x, a.y, a.z, a.w, b.x, b.y, b.z, b.w};
        uint32_t w = 0;
#pragma unroll
        for (int x = 0; x < 8; ++x) w += lit_count_bits(POW2 ? v[x] : __fmul_rn(v[x], H), s, c8) << (4 * x);
        // every term carried kCountBias above its nibble: remove them all
        constexpr uint32_t bias = kCountBias + (kCountBias << 4) + (kCountBias << 8) + (kCountBias << 12) +
                                  (kCountBias << 16) + (kCountBias << 20) + (kCountBias << 24) + (kCountBias << 28);
        W[y] = w - bias;
    }
}

// The eight 64-bit slice masks of a leaf and its 16-bit class mask (01 lit /
// 00 shadow / 10 partial per slice, src/CompressedShadowUtil.cpp:59-99) from
// the lit counts of its 8x8 texels (W[y]: row y, texel x at nibble x).  Per
// texel row the eight counts, packed as nibbles, are transposed into count
// bit-planes; slice s is then {texels with count > s}.  Two common kinds of
// leaf skip the transposes: all 64 counts equal to k (a flat patch of
// surface: slices 0..k-1 full, the rest empty) and all counts 0 or 8 (a wall
// crossing the leaf: every slice the set of count-8 texels).  Every path
// gives the same masks for the same counts.
// A leaf whose 64 counts all equal k (k0 receives it): its slices 0..k-1
// are full, the rest empty.  These are the only leaves with such masks.
__device__ __forceinline__ bool leaf_uniform(const uint32_t W[8], uint32_t& k0) {
    k0 = W[0] & 0xFu;
    const uint32_t rep = k0 * 0x11111111u;
    bool uniform = true;
#pragma unroll
    for (int y = 0; y < 8; ++y) uniform = uniform && W[y] == rep;
    return uniform;
}
__device__ __forceinline__ uint32_t uniform_class_mask(uint32_t k) { return 0x5555u & ((1u << (2u * k)) - 1u); }

__device__ __forceinline__ void leaf_masks_from_counts(const uint32_t W[8], uint64_t M[8], uint32_t& mask) {
    uint32_t k0;
    const bool uniform = leaf_uniform(W, k0);
    bool binary = true;
#pragma unroll
    for (int y = 0; y < 8; ++y) binary = binary && (W[y] & 0x77777777u) == 0u;
    if (uniform) {
#pragma unroll
        for (uint32_t q = 0; q < 8; ++q) M[q] = q < k0 ? ~0ull : 0ull;
        mask = uniform_class_mask(k0);
    } else if (binary) {
        // every count is 0 or 8 (a wall of the shadow volume crossing the
        // leaf): all eight slices are the set of count-8 texels, and every
        // slice is partial.  Bit 3 of each row's nibbles, gathered to a byte.
        uint64_t p3 = 0;
#pragma unroll
        for (int y = 0; y < 8; ++y) {
            uint32_t x = (W[y] >> 3) & 0x11111111u;
            x = (x | (x >> 3)) & 0x03030303u;
            x = (x | (x >> 6)) & 0x000F000Fu;
            x = (x | (x >> 12)) & 0xFFu;
            p3 |= (uint64_t)x << (8 * y);
        }
#pragma unroll
        for (int q = 0; q < 8; ++q) M[q] = p3;
        mask = 0xAAAAu;
    } else {
        // per row: byte b = count bit b of the row's 8 texels; then byte b of
        // rows 0..7 into plane b (row y at byte y): 4x4 byte transposes of
        // rows 0..3 and 4..7
        uint32_t R[8];
#pragma unroll
        for (int y = 0; y < 8; ++y) R[y] = nibbles_to_planes(W[y]);
        uint32_t plo[4], phi[4];
#pragma unroll
        for (int half = 0; half < 2; ++half) {
            const uint32_t r0 = R[4 * half], r1 = R[4 * half + 1], r2 = R[4 * half + 2], r3 = R[4 * half + 3];
            const uint32_t A = __byte_perm(r0, r1, 0x5140), B = __byte_perm(r0, r1, 0x7362);
            const uint32_t C = __byte_perm(r2, r3, 0x5140), D = __byte_perm(r2, r3, 0x7362);
            uint32_t* dst = half ? phi : plo;
            dst[0] = __byte_perm(A, C, 0x5410);
            dst[1] = __byte_perm(A, C, 0x7632);
            dst[2] = __byte_perm(B, D, 0x5410);
            dst[3] = __byte_perm(B, D, 0x7632);
        }
        const uint64_t P0 = plo[0] | ((uint64_t)phi[0] << 32), P1 = plo[1] | ((uint64_t)phi[1] << 32);
        const uint64_t P2 = plo[2] | ((uint64_t)phi[2] << 32), P3 = plo[3] | ((uint64_t)phi[3] << 32);
        // slice s = {t : k_t >= s+1}, k_t in [0, 8]
        M[0] = P0 | P1 | P2 | P3;
        M[1] = P1 | P2 | P3;
        M[2] = P3 | P2 | (P1 & P0);
        M[3] = P3 | P2;
        M[4] = P3 | (P2 & (P1 | P0));
        M[5] = P3 | (P2 & P1);
        M[6] = P3 | (P2 & P1 & P0);
        M[7] = P3;
        mask = 0;
#pragma unroll
        for (int q = 0; q < 8; ++q) {
            const uint32_t cls = (M[q] == ~0ull) ? kVisible : (M[q] == 0ull ? kShadow : kPartial);
            mask |= cls << (2 * q);
        }
    }
}

// Signature hash of a leaf: its job and its eight slice masks.
__device__ __forceinline__ uint64_t leaf_hash(uint32_t j, const uint64_t M[8]) {
    uint64_t h = (uint64_t)(j + 1) * kGolden;
#pragma unroll
    for (int q = 0; q < 8; ++q) {
        h = (h ^ M[q]) * 0xD6E8FEB86659FD93ull;
        h ^= h >> 32;
    }
    return fmix64(h);
}

// The slice masks, class mask and signature hash of the leaf at level-2
// coordinate `c` of job `j` (the 8x8x8 voxels at 4c), read from the depth
// map.  Returns false for a stale slot (an internal check already failed):
// the caller then treats it as an empty leaf of job 0 (j becomes 0).
template <bool POW2>
__device__ __forceinline__ bool leaf_compute(const JobDev* __restrict__ jobs, uint32_t njobs, uint64_t c,
                                             uint64_t M[8], uint32_t& mask, uint64_t& hash, uint32_t& j) {
    const uint32_t bx = unpack_x(c) * 4u, by = unpack_y(c) * 4u, bz = unpack_z(c) * 4u;
    if (j >= njobs || bx + 8u > __ldg(&jobs[j].n) || by + 8u > __ldg(&jobs[j].n)) {
#pragma unroll
        for (int q = 0; q < 8; ++q) M[q] = 0ull;
        mask = 0;
        j = 0;
        hash = 0;
        return false;
    }
    const uint32_t nmap = __ldg(&jobs[j].n);
    const uint32_t Hu = nmap * __ldg(&jobs[j].z_num);
    const float c8 = __fmul_rn(__fsub_rn(0.5f, __uint2float_rn(bz)), 0.125f);  // exact: bz < 2^23
    const float* row0 = jobs[j].depth + (size_t)by * nmap + bx;
    uint32_t W[8];
    leaf_rows<POW2>(row0, nmap, __uint2float_rn(Hu), c8, W);
    leaf_masks_from_counts(W, M, mask);
    hash = leaf_hash(j, M);
    return true;
}

__device__ __forceinline__ void leaf_segments(const LevelDev& lv, SegDev& seg, uint32_t i, uint32_t n, uint32_t j,
                                              int L, uint32_t njobs, uint32_t* err) {
    if (j >= njobs) {
        atomicOr(err, 128u);  // a node's job out of range: reported, not followed
        return;
    }
    if (i == 0 || lv.job[i - 1] != j) seg.nstart[seg_index(j, L)] = i;
    if (i == n - 1 || lv.job[i + 1] != j) seg.nend[seg_index(j, L)] = i + 1;
}

__device__ __forceinline__ void store_slices(const LevelDev& lv, uint32_t i, const uint64_t M[8]) {
    ulonglong2* o = reinterpret_cast<ulonglong2*>(lv.slices + (size_t)i * 8);
#pragma unroll
    for (int q = 0; q < 4; ++q) o[q] = make_ulonglong2(M[2 * q], M[2 * q + 1]);
}

// Leaf masks into per-leaf arrays (masks, class mask, hash) for a separate
// dedup_insert pass.
__global__ void __launch_bounds__(kThreads)
    k_leaf_masks(LevelDev lv, const uint32_t* __restrict__ counts, const JobDev* __restrict__ jobs, uint32_t njobs,
                 int L, SegDev seg, uint32_t* err) {
    const uint32_t n = counts[L];
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        uint64_t M[8], h;
        uint32_t mask, j;
        j = lv.job[i];
        const bool ok = leaf_compute<false>(jobs, njobs, lv.coord[i], M, mask, h, j);
        store_slices(lv, i, M);
        lv.mask[i] = mask;
        lv.hash[i] = h;
        if (!ok) {
            atomicOr(err, 4u);
            lv.job[i] = 0;
            continue;
        }
        leaf_segments(lv, seg, i, n, j, L, njobs, err);
    }
}

__device__ __forceinline__ unsigned long long ld_acquire(const unsigned long long* p) {
    unsigned long long v;
    asm volatile("ld.acquire.gpu.global.u64 %0, [%1];" : "=l"(v) : "l"(p) : "memory");
    return v;
}

// ------------------------------------------------------------ leaf columns
// The leaf level (level 2 with leafmasks) of a build plan is computed per
// texel column instead of per leaf.  A leaf at level-2 coordinate c covers
// the 8x8 texels of level-3 texel (c.x/2, c.y/2) -- its column -- and the
// voxels of level-3 z-cell zc = c.z/2.  Its parent classified exactly that
// (column, z-cell) as partial against the column's level-3 min/max, so
// every leaf lies in its column's partial z-cells [zlo, zhi]; along them
// the eight slice masks change only where some texel's highest lit voxel
// Z_t (lit iff z + 0.5 <= fl(d * H0)) enters or leaves the z-cell: a texel
// counts 8 lit voxels while 8 zc + 7 <= Z_t, then between 1 and 7 for at
// most one z-cell, then 0.  The partial z-cells of a column therefore fall
// into runs of equal leaves (the c1 workload: 7.3 M leaves, 1.24 M runs).
//
// k_leaf_columns (one thread per column, beside the expansion) walks the
// runs of every column of the batch's maps over the z-tiles of the jobs that
// use it: a run whose leaves are uniform (every texel's count equal) takes
// a fixed class per (job, count) from the column's min/max alone; the other
// runs' masks are computed once from the map (k_leaf_columns_heavy, for
// the columns that reach one), and k_leaf_classes inserts each such run's
// class (job, masks) into a hash table; a class's identity is the index of
// the run entry that first claimed it.  k_leaf_resolve (after the expansion
// has listed the leaves in breadth-first order) looks each leaf's run up
// and lowers its class's first-occurrence index -- the class record keeps
// (rank << 32 | smallest leaf index), as the inner levels' table slots do.
// Leaves of a column whose ancestors are not all partial get runs too
// (never referenced, never kept); a run covers at least one leaf cell, so
// the runs fit in the level's planned capacity.

struct LeafGroupDev {      // one source map and z_num; its jobs' z-tiles are distinct
    const float2* lvl3;    // pyramid level 3 of the map: (n/8)^2 (min, max) pairs
    const float* depth;    // the map, n x n
    const uint32_t* nan_flag;  // nonzero if the map holds a NaN (null: unknown)
    uint32_t n, z_num;
    uint32_t job_lo, job_cnt;  // its jobs in the z-tile table, ordered by z_idx
    uint64_t col_base;         // its first column record
};

struct LeafColumns {
    const LeafGroupDev* groups;
    const uint2* ztiles;        // (z_idx, job) per job, by group, ordered by z_idx
    const uint32_t* meta;       // [0] groups, [1] column records in use
    uint4* colrec;              // per column q: [2q] (first run entry, run count), [2q+1] a copy of its first run
    uint4* runs;                // per run: last z-cell, class id, class mask, job
    uint32_t run_cap;
    unsigned int* run_ctr;      // run entries reserved (zeroed per build)
    uint64_t* cls_slices;       // per class id: the 8 slice masks
    uint32_t* cls_job;          // per class id: its job
    unsigned long long* crec;   // per class id: rank << 32 | first occurrence
    unsigned long long* table;  // class hash table: tag << 32 | class id
    uint64_t table_mask;
    uint32_t njobs;             // uniform classes: id run_cap + 9 * job + k (all counts k)
    uint2* pending;             // non-uniform runs for k_leaf_classes: (run entry, index of the
                                // column record's copy of it, or 0)
    unsigned int* pending_ctr;  // their count (zeroed per build)
    uint4* heavy;               // columns whose walk needs their texels: (column, job index, z-cell, entry)
    unsigned int* heavy_ctr;    // their count (zeroed per build)
};

// The last z-cell (at most zmax) through which a texel with value v (the
// count functions' v: the raw depth for power-of-two heights, else
// fl(d * H)) stays fully lit: floor(v / 8 - 0.9375), see column_counts.
__device__ __forceinline__ uint32_t full_run_end(float v, float s, uint32_t zmax) {
    float t;
    asm("fma.rm.f32 %0, %1, %2, %3;" : "=f"(t) : "f"(v), "f"(s), "f"(-0.9375f));
    t = floorf(t);
    return t >= __uint2float_rn(zmax) ? zmax : (uint32_t)t;  // t >= zc here (the texel is full at zc)
}

// Lit counts of the column at (row0, row stride nmap) for the leaf of
// z-cell zc (W as leaf_rows gives them), and the last z-cell through which
// the leaf stays the same: zc itself when a texel is partly lit there, else
// the first z-cell after which a fully lit texel stops being full (or zmax).
// A texel with count 8 has Z_t >= 8 zc + 7 and stays full through
// floor((Z_t - 7) / 8) = floor(v / 8 - 0.9375) with v = fl(d * H0): one
// fused multiply-add rounded down gives that floor exactly (the exact value
// is rounded toward the integer below it, which is representable).  NaN
// depths count 0 everywhere; +inf counts 8 everywhere (its run never ends).
template <bool POW2>
__device__ __forceinline__ uint32_t column_counts(const float* row0, uint32_t nmap, float H, uint32_t zc,
                                                  uint32_t zmax, uint32_t W[8]) {
    const float s = POW2 ? __fmul_rn(H, 0.125f) : 0.125f;
    const float c8 = __fmul_rn(__fsub_rn(0.5f, __uint2float_rn(8u * zc)), 0.125f);  // exact: 8 zc < 2^23
    constexpr uint32_t bias = kCountBias + (kCountBias << 4) + (kCountBias << 8) + (kCountBias << 12) +
                              (kCountBias << 16) + (kCountBias << 20) + (kCountBias << 24) + (kCountBias << 28);
    float vfull = __int_as_float(0x7f800000);  // smallest v among the fully lit texels
    uint32_t part = 0;
    // all sixteen 16-byte loads of the 8x8 footprint in flight at once
    float4 r[16];
#pragma unroll
    for (int y = 0; y < 8; ++y) {
        r[2 * y] = __ldg(reinterpret_cast<const float4*>(row0 + (size_t)y * nmap));
        r[2 * y + 1] = __ldg(reinterpret_cast<const float4*>(row0 + (size_t)y * nmap + 4));
    }
#pragma unroll
    for (int y = 0; y < 8; ++y) {
        const float4 a = r[2 * y], b = r[2 * y + 1];
        const float d[8] = {a.x, a.y, a.z, a.w, b.x, b.y, b.z, b.w};
        uint32_t w = 0;
#pragma unroll
        for (int x = 0; x < 8; ++x) {
            const float v = POW2 ? d[x] : __fmul_rn(d[x], H);
            const uint32_t cb = lit_count_bits(v, s, c8);
            w += cb << (4 * x);
            vfull = cb == kCountBias + 8u ? fminf(vfull, v) : vfull;
        }
        W[y] = w - bias;
        part |= W[y] & 0x77777777u;  // some count in 1..7
    }
    if (part) return zc;
    return full_run_end(vfull, s, zmax);
}

// Inserts the class of run entry `cid` (job j, masks M, hash h) into the
// class hash table and returns the class id: the entry index of the run that
// claimed the class's slot.  Every run's masks and job were stored at its own
// entry index by the column pass, an earlier kernel, so a slot's claimant is
// compared straight from memory (no publication order to keep).
__device__ __forceinline__ uint32_t leaf_class_insert(const LeafColumns& lc, uint64_t h, uint32_t j,
                                                      const uint64_t M[8], uint32_t cid, uint32_t* err) {
    const unsigned long long key = (h & 0xFFFFFFFF00000000ull) | cid;
    uint64_t s = h & lc.table_mask;
    for (uint64_t probe = 0; probe <= lc.table_mask; ++probe) {
        unsigned long long e = __ldcg(&lc.table[s]);
        if (e == kEmptySlot) {
            e = atomicCAS(&lc.table[s], kEmptySlot, key);
            if (e == kEmptySlot) return cid;
        }
        if ((e >> 32) == (key >> 32)) {
            const uint32_t r = (uint32_t)e;
            if (r < lc.run_cap) {
                const ulonglong2* o = reinterpret_cast<const ulonglong2*>(lc.cls_slices + (size_t)r * 8);
                const uint32_t jr = __ldg(lc.cls_job + r);
                ulonglong2 x[4];
#pragma unroll
                for (int q = 0; q < 4; ++q) x[q] = __ldg(o + q);
                bool same = jr == j;
#pragma unroll
                for (int q = 0; q < 4; ++q) same = same && x[q].x == M[2 * q] && x[q].y == M[2 * q + 1];
                if (same) return r;
            }
        }
        s = (s + 1) & lc.table_mask;
    }
    atomicOr(err, 16u);  // table full: the result is void, reported (the plan grows)
    return cid;
}

// One thread per non-uniform run: its class id into the run entry.
__global__ void __launch_bounds__(kThreads) k_leaf_classes(LeafColumns lc, uint32_t* err) {
    const uint32_t np = *lc.pending_ctr;
    for (uint32_t p = blockIdx.x * blockDim.x + threadIdx.x; p < np; p += gridDim.x * blockDim.x) {
        const uint2 pe = lc.pending[p];
        const uint32_t cid = pe.x;
        if (cid >= lc.run_cap) {
            atomicOr(err, 512u);
            continue;
        }
        const ulonglong2* o = reinterpret_cast<const ulonglong2*>(lc.cls_slices + (size_t)cid * 8);
        uint64_t M[8];
#pragma unroll
        for (int q = 0; q < 4; ++q) {
            const ulonglong2 t = o[q];
            M[2 * q] = t.x;
            M[2 * q + 1] = t.y;
        }
        const uint32_t j = lc.cls_job[cid];
        const uint32_t id = leaf_class_insert(lc, leaf_hash(j, M), j, M, cid, err);
        lc.runs[cid].y = id;
        if (pe.y) lc.colrec[pe.y].y = id;  // the column record's copy of its first run
    }
}

// Partial z-cells [zlo, zhi] of a column against its level-3 bounds b
// (min, max) and level-3 height H3: !((zc+1) <= lo) && !(zc >= hi)
// (cs::visible, src/CompressedShadowUtil.h:35-43) with lo/hi the bounds
// times H3, a contiguous range; NaN bounds are partial.  Empty: zlo > zhi.
__device__ __forceinline__ void column_partial_range(float2 b, uint32_t H3, uint32_t& zlo, uint32_t& zhi) {
    const float Hf = __uint2float_rn(H3);
    const float lo_s = __fmul_rn(b.x, Hf), hi_s = __fmul_rn(b.y, Hf);
    zlo = lo_s != lo_s ? 0u : (uint32_t)fminf(fmaxf(floorf(lo_s), 0.f), Hf);
    const float top = hi_s != hi_s ? Hf : fminf(fmaxf(ceilf(hi_s), 0.f), Hf);  // zhi + 1
    if (top == 0.f) {
        zlo = 1u;
        zhi = 0u;
    } else {
        zhi = (uint32_t)top - 1u;
    }
}

// Column q of the batch: its group, its coordinates and its partial range.
struct ColumnAt {
    uint32_t g, C, cx, cy, zlo, zhi;
    float2 b;  // the column's level-3 (min, max)
};
__device__ __forceinline__ ColumnAt column_at(const LeafColumns& lc, uint32_t ngroups, uint64_t q) {
    uint32_t lo = 0, hi = ngroups;  // the last group whose first column is <= q
    while (hi - lo > 1) {
        const uint32_t mid = (lo + hi) >> 1;
        if (__ldg(&lc.groups[mid].col_base) <= q) lo = mid; else hi = mid;
    }
    ColumnAt c;
    c.g = lo;
    const LeafGroupDev& G = lc.groups[lo];
    c.C = __ldg(&G.n) >> 3;
    const uint32_t local = (uint32_t)(q - __ldg(&G.col_base)), lg = 31u - (uint32_t)__clz((int)c.C);
    c.cx = local & (c.C - 1u);
    c.cy = local >> lg;
    c.b = __ldg(G.lvl3 + local);
    column_partial_range(c.b, c.C * __ldg(&G.z_num), c.zlo, c.zhi);
    return c;
}

// Partial leaf cells of a column over its group's z-tiles.
__device__ __forceinline__ uint32_t column_cells(const LeafColumns& lc, const ColumnAt& c) {
    const LeafGroupDev& G = lc.groups[c.g];
    const uint32_t jl = __ldg(&G.job_lo), jc = __ldg(&G.job_cnt);
    uint32_t cells = 0;
    for (uint32_t k = 0; k < jc && c.zlo <= c.zhi; ++k) {
        const uint32_t z0 = __ldg(&lc.ztiles[jl + k].x) * c.C;
        const uint32_t a = max(c.zlo, z0), e = min(c.zhi, z0 + c.C - 1u);
        if (a <= e) cells += e - a + 1u;
    }
    return cells;
}

// One run of column c at z-cell zc (range end e, job `job`), written to run
// entry cid: its last z-cell is returned.  A lit count is monotone in the
// depth, so when the column's lowest and highest depth have the same count
// at zc every texel has it (a uniform leaf) and the texels need not be read
// (`minmax`: the map holds no NaN, which the min/max reduction may hide).
// LIGHT: a run that needs the texels is not taken (returns false); else the
// texels are read, and a non-uniform run stores its masks, job and an empty
// record at its own entry and joins the pending list of k_leaf_classes.
// `first` (non-null for a column's first run): where the column record keeps
// a copy of the entry.
template <bool POW2, bool LIGHT>
__device__ __forceinline__ bool column_run(const LeafColumns& lc, const ColumnAt& c, const float* row0, uint32_t nmap,
                                           float H0, bool minmax, uint32_t zc, uint32_t e, uint32_t job, uint32_t cid,
                                           uint32_t& last, uint4* first) {
    uint32_t k0 = 0;
    bool uni = false;
    if (minmax) {
        const float s = POW2 ? __fmul_rn(H0, 0.125f) : 0.125f;
        const float c8 = __fmul_rn(__fsub_rn(0.5f, __uint2float_rn(8u * zc)), 0.125f);
        const float vlo = POW2 ? c.b.x : __fmul_rn(c.b.x, H0), vhi = POW2 ? c.b.y : __fmul_rn(c.b.y, H0);
        const uint32_t clo = lit_count_bits(vlo, s, c8), chi = lit_count_bits(vhi, s, c8);
        if (clo == chi) {
            uni = true;
            k0 = clo - kCountBias;
            last = k0 == 8u ? full_run_end(vlo, s, e) : (k0 == 0u ? e : zc);
        }
    }
    if (LIGHT && !uni) return false;
    uint32_t W[8];
    if (!uni) {
        last = column_counts<POW2>(row0, nmap, H0, zc, e, W);
        uni = leaf_uniform(W, k0);
    }
    uint32_t id, mask;
    if (uni) {
        id = lc.run_cap + 9u * job + k0;
        mask = uniform_class_mask(k0);
    } else {
        uint64_t M[8];
        leaf_masks_from_counts(W, M, mask);
        ulonglong2* o = reinterpret_cast<ulonglong2*>(lc.cls_slices + (size_t)cid * 8);
#pragma unroll
        for (int q = 0; q < 4; ++q) o[q] = make_ulonglong2(M[2 * q], M[2 * q + 1]);
        lc.cls_job[cid] = job;
        lc.crec[cid] = kEmptySlot;
        id = cid;
    }
    if (!LIGHT) {
        // the non-uniform runs of the warp's active lanes join the pending
        // list with one atomic add
        const unsigned act = __activemask();
        const unsigned want = __ballot_sync(act, !uni);
        if (want) {
            const int lead = __ffs((int)want) - 1;
            const uint32_t lane = threadIdx.x & 31u;
            uint32_t at = 0;
            if ((int)lane == lead) at = atomicAdd(lc.pending_ctr, (unsigned)__popc(want));
            at = __shfl_sync(act, at, lead);
            if (!uni)
                lc.pending[at + __popc(want & ((1u << lane) - 1u))] =
                    make_uint2(id, first ? (uint32_t)(first - lc.colrec) : 0u);
        }
    }
    const uint4 entry = make_uint4(last, id, mask, job);
    lc.runs[cid] = entry;
    if (first) *first = entry;
    return true;
}

// Walks the runs of column c from job index k and z-cell zc on, writing run
// entries from off + nrun; LIGHT stops at the first run that needs the
// texels and returns false with (k, zc) at that run.
template <bool POW2, bool LIGHT>
__device__ __forceinline__ bool column_walk(const LeafColumns& lc, const ColumnAt& c, uint64_t q, uint32_t off,
                                            uint32_t& nrun, uint32_t& k, uint32_t& zc) {
    const LeafGroupDev& G = lc.groups[c.g];
    const uint32_t jl = __ldg(&G.job_lo), jc = __ldg(&G.job_cnt), nmap = __ldg(&G.n);
    const float* row0 = G.depth + (size_t)(c.cy * 8u) * nmap + c.cx * 8u;
    const float H0 = __uint2float_rn(nmap * __ldg(&G.z_num));
    const uint32_t* nf = G.nan_flag;
    const bool minmax = nf && __ldg(nf) == 0u;
    for (; k < jc; ++k) {
        const uint2 zt = __ldg(&lc.ztiles[jl + k]);
        const uint32_t z0 = zt.x * c.C;
        const uint32_t e = min(c.zhi, z0 + c.C - 1u);
        zc = max(zc, max(c.zlo, z0));
        while (zc <= e) {
            uint32_t last;
            if (!column_run<POW2, LIGHT>(lc, c, row0, nmap, H0, minmax, zc, e, zt.y, off + nrun, last,
                                         nrun ? nullptr : lc.colrec + 2 * q + 1))
                return false;
            ++nrun;
            zc = last + 1u;
        }
        zc = 0;
    }
    return true;
}

// The runs of every column of the batch's maps, first pass.  A block takes
// a chunk of kColChunk columns, kColItems per thread: it counts their
// partial leaf cells, reserves that many run entries with one atomic add,
// and walks each column's runs as far as the min/max shortcut carries
// them.  Uniform leaves (all 64 counts equal to k: flat surface, 77% of the
// 8192^2 workload's runs) take the fixed class id run_cap + 9 * job + k;
// the first block writes those classes' masks and empty records.  A column
// that reaches a run needing its texels is queued, with the state to
// resume from, for k_leaf_columns_heavy, so the texel work runs on full
// warps instead of on the few lanes of each warp that have it.
constexpr int kColItems = 2;
constexpr uint32_t kColChunk = kThreads * kColItems;

template <bool POW2>
__global__ void __launch_bounds__(kThreads) k_leaf_columns(LeafColumns lc, uint32_t* err) {
    __shared__ uint32_t sm[64];
    __shared__ uint32_t s_base;
    const uint32_t ngroups = lc.meta[0];
    const uint64_t ncols = lc.meta[1];
    if (blockIdx.x == 0)
        for (uint32_t u = threadIdx.x; u < 9u * lc.njobs; u += blockDim.x) {
            const uint32_t id = lc.run_cap + u, k = u % 9u;
            ulonglong2* o = reinterpret_cast<ulonglong2*>(lc.cls_slices + (size_t)id * 8);
#pragma unroll
            for (uint32_t q = 0; q < 4; ++q)
                o[q] = make_ulonglong2(2 * q < k ? ~0ull : 0ull, 2 * q + 1 < k ? ~0ull : 0ull);
            lc.cls_job[id] = u / 9u;
            lc.crec[id] = kEmptySlot;
        }
    for (uint64_t chunk = blockIdx.x; chunk * kColChunk < ncols; chunk += gridDim.x) {
        const uint64_t q0 = chunk * kColChunk + threadIdx.x;
        uint32_t sum = 0;
#pragma unroll
        for (int it = 0; it < kColItems; ++it) {
            const uint64_t q = q0 + (uint64_t)it * kThreads;
            if (q < ncols) sum += column_cells(lc, column_at(lc, ngroups, q));
        }
        uint2 tot;
        const uint32_t pre = block_exclusive_scan2(make_uint2(sum, 0u), tot, sm).x;
        if (threadIdx.x == 0) s_base = tot.x ? atomicAdd(lc.run_ctr, tot.x) : 0u;
        __syncthreads();
        const uint32_t base = s_base;
        __syncthreads();
        const bool fits = (uint64_t)base + tot.x <= lc.run_cap;
        if (!fits && threadIdx.x == 0) atomicOr(err, 1u);  // more runs than the plan holds: reported, the plan grows
        uint32_t off = base + pre;
#pragma unroll 1
        for (int it = 0; it < kColItems; ++it) {
            const uint64_t q = q0 + (uint64_t)it * kThreads;
            bool queue = false;
            uint32_t k = 0, zc = 0, nrun = 0, cells = 0;
            if (q < ncols) {
                const ColumnAt c = column_at(lc, ngroups, q);
                cells = column_cells(lc, c);
                if (cells && fits) queue = !column_walk<POW2, true>(lc, c, q, off, nrun, k, zc);
                lc.colrec[2 * q] = make_uint4(off, nrun, 0u, 0u);
            }
            // queue the columns that need their texels, one atomic per warp
            const unsigned want = __ballot_sync(0xffffffffu, queue);
            if (want) {
                const int lead = __ffs((int)want) - 1;
                const uint32_t lane = threadIdx.x & 31u;
                uint32_t at = 0;
                if ((int)lane == lead) at = atomicAdd(lc.heavy_ctr, (unsigned)__popc(want));
                at = __shfl_sync(0xffffffffu, at, lead);
                if (queue) lc.heavy[at + __popc(want & ((1u << lane) - 1u))] = make_uint4((uint32_t)q, k, zc, off + nrun);
            }
            off += cells;
        }
    }
}

// Second pass: one thread per queued column resumes its walk where the
// first pass stopped, reading the texels where a run needs them.
template <bool POW2>
__global__ void __launch_bounds__(kThreads, 2) k_leaf_columns_heavy(LeafColumns lc) {
    const uint32_t ngroups = lc.meta[0];
    const uint32_t nh = *lc.heavy_ctr;
    for (uint32_t h = blockIdx.x * blockDim.x + threadIdx.x; h < nh; h += gridDim.x * blockDim.x) {
        const uint4 w = lc.heavy[h];
        const ColumnAt c = column_at(lc, ngroups, w.x);
        const uint32_t off = lc.colrec[2 * (uint64_t)w.x].x;
        uint32_t nrun = w.w - off, k = w.y, zc = w.z;
        column_walk<POW2, false>(lc, c, w.x, off, nrun, k, zc);
        lc.colrec[2 * (uint64_t)w.x].y = nrun;
    }
}

// Every leaf (breadth-first order) takes its class from its column's runs:
// class id (its merged identity for level 3) and class mask; then the
// class's first-occurrence index is lowered to the leaf's if smaller.
// Leaves of one class in one warp: only the first (lowest index) updates.
// The column record's two halves (run count, first run) arrive together, so
// a leaf whose z-cell the first run covers (most) costs one round trip.
struct LeafRec {  // a leaf's column record, fetched ahead of its use
    uint4 h, e0;     // (first run entry, run count), the first run
    uint32_t zc;     // the leaf's level-3 z-cell
    bool in;         // the job and column exist
};

__device__ __forceinline__ LeafRec leaf_rec_fetch(const LeafColumns& lc, const JobDev* __restrict__ jobs,
                                                  uint32_t njobs, uint64_t c, uint32_t j) {
    LeafRec r;
    r.in = false;
    r.zc = 0;
    r.h = r.e0 = make_uint4(0u, 0u, 0u, 0u);
    if (j >= njobs) return r;
    const uint32_t C = __ldg(&jobs[j].n) >> 3;
    const uint32_t cx = unpack_x(c) >> 1, cy = unpack_y(c) >> 1;
    if (cx >= C || cy >= C) return r;
    const uint4* rp = lc.colrec + 2 * (__ldg(&jobs[j].col_base) + (uint64_t)cy * C + cx);
    r.h = rp[0];
    r.e0 = rp[1];
    r.zc = unpack_z(c) >> 1;
    r.in = true;
    return r;
}

__device__ __forceinline__ uint32_t leaf_class_of(const LeafColumns& lc, const LeafRec& r, uint32_t j, uint32_t& mask,
                                                  bool& ok) {
    ok = false;
    mask = 0;
    if (!r.in || r.h.y == 0) return 0;
    uint4 e = r.e0;
    for (uint32_t k = 1; r.zc > e.x && k < r.h.y; ++k) e = lc.runs[r.h.x + k];
    if (r.zc > e.x) return 0;
    ok = e.w == j && e.y < lc.run_cap + 9u * lc.njobs;
    mask = e.z;
    return e.y;
}

// The uniform classes (9 per job, the most frequent) keep their smallest
// leaf index per block in shared memory and lower the class record once per
// block; other classes lower it per warp (the warp's lowest lane of each).
constexpr uint32_t kResUniform = 9 * 64;

struct LeafFirst {  // a block's running minima of the uniform classes
    uint32_t* umin;  // shared, kResUniform entries
    bool on;         // 9 * njobs <= kResUniform
};

__device__ __forceinline__ LeafFirst leaf_first_begin(uint32_t* umin, uint32_t njobs) {
    LeafFirst f{umin, 9u * njobs <= kResUniform};
    if (f.on)
        for (uint32_t t = threadIdx.x; t < 9u * njobs; t += blockDim.x) umin[t] = ~0u;
    return f;  // the caller synchronises the block before the first update
}

// Leaf i of class `id`: lowers the class's first occurrence.
__device__ __forceinline__ void leaf_first_update(const LeafColumns& lc, const LeafFirst& f, uint32_t id, uint32_t i) {
    if (f.on && id >= lc.run_cap) {
        atomicMin(&f.umin[id - lc.run_cap], i);
    } else {
        const unsigned same = __match_any_sync(__activemask(), id);
        if ((threadIdx.x & 31u) == (uint32_t)(__ffs((int)same) - 1)) {
            const uint32_t r = __ldcg(reinterpret_cast<const uint32_t*>(lc.crec + id));
            if (r > i) atomicMin(lc.crec + id, 0xFFFFFFFF00000000ull | i);
        }
    }
}

// After the block's last update (the caller synchronises the block first).
__device__ __forceinline__ void leaf_first_flush(const LeafColumns& lc, const LeafFirst& f) {
    if (!f.on) return;
    for (uint32_t t = threadIdx.x; t < 9u * lc.njobs; t += blockDim.x) {
        const uint32_t v = f.umin[t];
        if (v == ~0u) continue;
        unsigned long long* rec = lc.crec + lc.run_cap + t;
        if (__ldcg(reinterpret_cast<const uint32_t*>(rec)) > v) atomicMin(rec, 0xFFFFFFFF00000000ull | v);
    }
}

// Leaf i (job j, column record r) of the level: its class id into slot,
// its class mask, its first occurrence; returns its job (0 when out of
// range).
__device__ __forceinline__ uint32_t leaf_resolve_one(const LevelDev& lv, uint32_t njobs, const LeafColumns& lc,
                                                     const LeafFirst& f, uint32_t i, const LeafRec& r, uint32_t j,
                                                     uint32_t* err) {
    uint32_t mask = 0;
    bool ok;
    uint32_t id = leaf_class_of(lc, r, j, mask, ok);
    if (!ok) {
        atomicOr(err, 512u);  // a leaf outside its column's runs: reported, not followed
        j = j < njobs ? j : 0u;
        id = 0;
        mask = 0;
    }
    lv.slot[i] = id;
    lv.mask[i] = mask;
    if (ok) leaf_first_update(lc, f, id, i);
    return j;
}

// One thread per listed leaf (used where the expansion of level 3 runs in
// the cluster kernel; else k_expand_lb<true> resolves the leaves as it
// writes them).
__global__ void __launch_bounds__(kThreads)
    k_leaf_resolve(LevelDev lv, const uint32_t* __restrict__ counts, const JobDev* __restrict__ jobs, uint32_t njobs,
                   SegDev seg, LeafColumns lc, uint32_t* err) {
    chain_enter();
    __shared__ uint32_t s_umin[kResUniform];
    const LeafFirst f = leaf_first_begin(s_umin, lc.njobs);
    __syncthreads();
    const uint32_t n = counts[2];
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        const uint32_t j0 = lv.job[i];
        const uint32_t j = leaf_resolve_one(lv, njobs, lc, f, i, leaf_rec_fetch(lc, jobs, njobs, lv.coord[i], j0), j0, err);
        if (j != j0) lv.job[i] = j;
        leaf_segments(lv, seg, i, n, j, 2, njobs, err);
    }
    __syncthreads();
    leaf_first_flush(lc, f);
}

// --------------------------------------------------------------- bottom-up
// A child's merged identity: the hash slot its class occupies.  Equal nodes
// hash to the same start and probe the same sequence; a slot, once claimed,
// keeps its class (later equal nodes only lower the representative index in
// its lower half), so every member of a class ends on the class's slot and
// no two classes share one.  The identity is thus final as soon as the
// node's own insert returns, and the level above needs no pass that resolves
// representatives first.  CG: written by other blocks of the same launch, so
// read from L2.
template <bool CG>
__device__ __forceinline__ uint32_t child_uid(const LevelDev& child, uint32_t x) {
    return CG ? __ldcg(child.slot + x) : child.slot[x];
}

// Two leaves are the same node when their jobs and all eight slice masks
// are equal.
__device__ __forceinline__ bool same_leaf(const LevelDev& cur, uint32_t a, uint32_t b) {
    if (cur.job[a] != cur.job[b]) return false;
    const ulonglong2* sa = reinterpret_cast<const ulonglong2*>(cur.slices + (size_t)a * 8);
    const ulonglong2* sb = reinterpret_cast<const ulonglong2*>(cur.slices + (size_t)b * 8);
#pragma unroll
    for (int q = 0; q < 4; ++q) {
        const ulonglong2 x = sa[q], y = sb[q];
        if (x.x != y.x || x.y != y.y) return false;
    }
    return true;
}

// Inserts every node of level L into the table.  A slot holds
// (tag << 32 | node index); the first node of a signature class claims an
// empty slot with CAS, later equal nodes lower it with atomicMin, so the slot
// ends with the class's smallest (first-occurring) index.  The probe is
// bounded by the table size (the table is at least twice the node count).
// Node i with mask m, job j, first child f; returns its slot.
template <bool CG>
__device__ __forceinline__ uint32_t insert_inner(LevelDev& cur, const LevelDev& child, uint32_t i, uint32_t m,
                                                 uint32_t j, uint32_t f, unsigned long long* table,
                                                 uint64_t cap_mask, uint32_t* err);

template <bool LEAF>
__global__ void __launch_bounds__(kThreads)
    k_dedup_insert(LevelDev cur, LevelDev child, const uint32_t* __restrict__ counts, int L,
                   unsigned long long* table, uint64_t cap_mask, uint32_t* err) {
    chain_enter();
    const uint32_t n = counts[L];
    if (!LEAF) {
        // the next node's mask, job and first child are requested one
        // iteration ahead
        const uint32_t stride = gridDim.x * blockDim.x;
        uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
        uint32_t m_n = i < n ? cur.mask[i] : 0u, j_n = i < n ? cur.job[i] : 0u, f_n = i < n ? cur.first[i] : 0u;
        for (; i < n; i += stride) {
            const uint32_t m = m_n, j = j_n, f = f_n;
            if (i + stride < n) {
                m_n = cur.mask[i + stride];
                j_n = cur.job[i + stride];
                f_n = cur.first[i + stride];
            }
            insert_inner<false>(cur, child, i, m, j, f, table, cap_mask, err);
        }
        return;
    }
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        const uint64_t h = cur.hash[i];
        const unsigned long long key = (h & 0xFFFFFFFF00000000ull) | i;
        uint64_t s = h & cap_mask;
        bool placed = false;
        for (uint64_t probe = 0; probe <= cap_mask; ++probe) {
            unsigned long long cur_e = __ldcg(&table[s]);
            if (cur_e == kEmptySlot) {
                const unsigned long long prev = atomicCAS(&table[s], kEmptySlot, key);
                if (prev == kEmptySlot) {
                    placed = true;
                    break;
                }
                cur_e = prev;
            }
            if ((cur_e >> 32) == (key >> 32) && same_leaf(cur, i, (uint32_t)cur_e)) {
                // the slot only ever decreases: nothing to do when it already
                // holds an earlier occurrence
                if ((uint32_t)cur_e > i) atomicMin(&table[s], key);
                placed = true;
                break;
            }
            s = (s + 1) & cap_mask;
        }
        if (!placed) atomicOr(err, 16u);  // table full: the result is void, reported
        cur.slot[i] = (uint32_t)s;
    }
}

__device__ __forceinline__ uint32_t node_words(uint32_t m, bool leaf) {
    return 1u + (leaf ? 2u : 1u) * partial_children(m);
}

// Representative of every node; per-CTA (kept count, kept words).
template <bool LEAF>
__global__ void __launch_bounds__(kThreads)
    k_dedup_resolve(LevelDev cur, const uint32_t* __restrict__ counts, int L,
                    const unsigned long long* __restrict__ table, uint2* partials) {
    __shared__ uint64_t red[32];
    uint32_t b, e;
    block_chunk(counts[L], b, e);
    uint64_t kept = 0, words = 0;
    for (uint32_t i = b + threadIdx.x; i < e; i += blockDim.x) {
        const uint32_t rep = (uint32_t)table[cur.slot[i]];
        cur.uid[i] = rep;
        if (rep == i) {
            ++kept;
            words += node_words(cur.mask[i], LEAF);
        }
    }
    kept = block_sum_u64(kept, red);
    words = block_sum_u64(words, red);
    if (threadIdx.x == 0) partials[blockIdx.x] = make_uint2((uint32_t)kept, (uint32_t)words);
}

// Ranks and word offsets of the kept nodes in node order; each kept node
// writes its rank into its table slot for dedup_remap.
template <bool LEAF>
__global__ void __launch_bounds__(kThreads)
    k_dedup_scan(LevelDev cur, const uint32_t* __restrict__ counts, uint32_t* level_u, int L,
                 unsigned long long* table, const uint2* __restrict__ partials, SegDev seg) {
    __shared__ uint32_t sm[64];
    const uint32_t n = counts[L];
    uint32_t b, e;
    block_chunk(n, b, e);
    uint2 run = block_prefix_of_partials(partials, blockIdx.x, sm);
    if (blockIdx.x == gridDim.x - 1 && threadIdx.x == 0) {
        level_u[2 * L] = run.x + partials[blockIdx.x].x;
        level_u[2 * L + 1] = run.y + partials[blockIdx.x].y;
    }
    for (uint32_t t0 = b; t0 < e; t0 += blockDim.x) {
        const uint32_t i = t0 + threadIdx.x;
        const bool valid = i < e;
        const bool kept = valid && cur.uid[i] == i;
        const uint32_t w = kept ? node_words(cur.mask[i], LEAF) : 0u;
        uint2 tot;
        const uint2 p = block_exclusive_scan2(make_uint2(kept ? 1u : 0u, w), tot, sm);
        const uint2 q = make_uint2(run.x + p.x, run.y + p.y);
        if (kept) {
            cur.uniq[q.x] = i;
            cur.woff[q.x] = q.y;
            table[cur.slot[i]] = q.x;
        }
        if (valid) {
            const uint32_t j = cur.job[i];
            if (i == 0 || cur.job[i - 1] != j) {
                seg.ustart[seg_index(j, L)] = q.x;
                seg.wstart[seg_index(j, L)] = q.y;
            }
            if (i == n - 1 || cur.job[i + 1] != j) {
                seg.uend[seg_index(j, L)] = q.x + (kept ? 1u : 0u);
                seg.wend[seg_index(j, L)] = q.y + w;
            }
        }
        run.x += tot.x;
        run.y += tot.y;
    }
}

__global__ void __launch_bounds__(kThreads)
    k_dedup_remap(LevelDev cur, const uint32_t* __restrict__ counts, int L, const unsigned long long* __restrict__ table) {
    const uint32_t n = counts[L];
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
        cur.uid[i] = (uint32_t)table[cur.slot[i]];
}

// ------------------------------------------------------- single-pass levels
// Build plans run each level in as few launches as possible: the top-down
// expansion of a level is one kernel (classify, count, scan, write the
// children); its merge is the insert plus one kernel that finds the kept
// nodes (first occurrences), ranks them and assigns their word offsets.  The
// prefix across blocks is a decoupled look-back: a block takes the next tile
// by ticket, publishes its tile's aggregate, then walks back over its
// predecessors' flags until one carries an inclusive prefix.  Tiles are
// taken in order, so a block only waits on blocks that already run, and
// every wait is bounded in time (a timeout sets error bit 32).  A kept
// node's rank goes into the upper half of its hash slot (the lower half
// keeps the class representative), so the emission reads a node's rank as
// table[slot] >> 32 and no remap pass runs.  The topmost levels, which hold
// few nodes, run in one cluster launch for the expansion and one for the
// merge.

constexpr unsigned long long kFlagAgg = 1ull << 62, kFlagInc = 2ull << 62, kFlagState = 3ull << 62;
constexpr uint64_t kLookbackTimeoutNs = 200000000ull;  // 0.2 s
constexpr int kExpItems = 4;
constexpr uint32_t kExpTile = kThreads * kExpItems;
constexpr int kScanItems = 8;
constexpr uint32_t kScanTile = kThreads * kScanItems;

__device__ __forceinline__ unsigned long long ld_relaxed(const unsigned long long* p) {
    unsigned long long v;
    asm volatile("ld.relaxed.gpu.global.u64 %0, [%1];" : "=l"(v) : "l"(p) : "memory");
    return v;
}

__device__ __forceinline__ uint64_t global_ns() {
    uint64_t t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    return t;
}

// A tile's flag: state (bits 63..62: aggregate / inclusive), then two
// 31-bit sums (bits 61..31 and 30..0).  Every level's sums stay below 2^31
// (node counts are bounded by the plan, word counts by the DAG size check);
// a sum that does not fit sets error bit 64.
__device__ __forceinline__ unsigned long long pack_flag(unsigned long long state, uint2 v) {
    return state | ((unsigned long long)(v.x & 0x7FFFFFFFu) << 31) | (v.y & 0x7FFFFFFFu);
}
__device__ __forceinline__ uint2 flag_values(unsigned long long f) {
    return make_uint2((uint32_t)(f >> 31) & 0x7FFFFFFFu, (uint32_t)f & 0x7FFFFFFFu);
}

// Exclusive prefix of `agg` over tiles 0..tile-1; called by all 32 lanes of
// one warp, which read 32 predecessors' flags per step: the nearest
// inclusive flag ends the walk, aggregates before it are summed.
__device__ uint2 lookback(unsigned long long* flags, uint32_t tile, uint2 agg, uint32_t* err) {
    const int lane = threadIdx.x & 31;
    if (agg.x > 0x7FFFFFFFu || agg.y > 0x7FFFFFFFu) atomicOr(err, 64u);
    if (tile == 0) {
        if (lane == 0) atomicExch(&flags[0], pack_flag(kFlagInc, agg));
        return make_uint2(0u, 0u);
    }
    if (lane == 0) atomicExch(&flags[tile], pack_flag(kFlagAgg, agg));
    uint2 excl = make_uint2(0u, 0u);
    int64_t p = (int64_t)tile - 1;
    const uint64_t t0 = global_ns();
    for (;;) {
        const int64_t q = p - lane;
        // before tile 0: an inclusive zero
        unsigned long long f = q >= 0 ? ld_relaxed(&flags[q]) : kFlagInc;
        bool timed_out = false;
        while (__any_sync(0xffffffffu, (f & kFlagState) == 0ull)) {
            timed_out = __shfl_sync(0xffffffffu, global_ns() - t0 > kLookbackTimeoutNs, 0);
            if (timed_out) break;
            __nanosleep(32);
            if ((f & kFlagState) == 0ull) f = ld_relaxed(&flags[q]);
        }
        if (timed_out) {
            if (lane == 0) atomicOr(err, 32u);  // a predecessor never published: the result is void, reported
            break;
        }
        const unsigned inc = __ballot_sync(0xffffffffu, (f & kFlagState) == kFlagInc);
        const int stop = inc ? __ffs(inc) - 1 : 31;
        uint2 v = lane <= stop ? flag_values(f) : make_uint2(0u, 0u);
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) {
            v.x += __shfl_xor_sync(0xffffffffu, v.x, o);
            v.y += __shfl_xor_sync(0xffffffffu, v.y, o);
        }
        excl.x += v.x;
        excl.y += v.y;
        if (inc) break;
        p -= 32;
    }
    const uint2 incl = make_uint2(excl.x + agg.x, excl.y + agg.y);
    if (incl.x > 0x7FFFFFFFu || incl.y > 0x7FFFFFFFu) atomicOr(err, 64u);
    if (lane == 0) atomicExch(&flags[tile], pack_flag(kFlagInc, incl));
    return excl;
}

// 8-bit set of the partial children (bit ch) of a 16-bit class mask.
__device__ __forceinline__ uint32_t partial_set(uint32_t m) {
    uint32_t pb = 0;
#pragma unroll
    for (uint32_t ch = 0; ch < 8; ++ch) pb |= ((m >> (2u * ch + 1u)) & 1u) << ch;
    return pb;
}

// Expansion of level L into L-1 in one pass, tiles of kExpTile nodes.  Each
// thread classifies four consecutive nodes (their inputs loaded before any
// store, so the loads overlap) and records, for each of their children, the
// (parent, child slot) pair at the child's position in a shared-memory map;
// after the tile's scan and look-back, thread t writes children t, t + 256,
// ... of the tile from that map, so the child arrays are written in
// coalesced runs.
// LEAVES (level 3 into the leaf level of a leafmask build, after the leaf
// column passes): each leaf takes its class from its column's runs as it is
// written (leaf_resolve_one), instead of its coordinate, and the leaf
// level's job ranges follow from the parents' (a job's leaves are its
// level-3 nodes' children, contiguous), so no pass re-reads the leaf list.
template <bool LEAVES>
__global__ void __launch_bounds__(kThreads)
    k_expand_lb(LevelDev cur, LevelDev nxt, uint32_t* counts, const JobDev* __restrict__ jobs, uint32_t njobs,
                int L, const Injected* __restrict__ inj, uint32_t ninj, SegDev seg, uint32_t cap_next,
                unsigned int* ticket, unsigned long long* flags, LeafColumns lc, uint32_t* err) {
    chain_enter();
    __shared__ uint32_t sm[64];
    __shared__ uint32_t s_tile, s_excl;
    __shared__ uint64_t s_coord[kExpTile];
    __shared__ uint32_t s_job[kExpTile];
    __shared__ uint16_t s_child[8 * kExpTile];  // tile child c: parent (local index) << 3 | child slot
    __shared__ uint32_t s_umin[LEAVES ? kResUniform : 1];
    LeafFirst lf{};
    if (LEAVES) lf = leaf_first_begin(s_umin, lc.njobs);  // synchronised by the first ticket's barrier
    const uint32_t n = counts[L];
    const uint32_t ntiles = n ? (n + kExpTile - 1) / kExpTile : 1u;
    for (;;) {
        if (threadIdx.x == 0) s_tile = atomicAdd(ticket, 1u);
        __syncthreads();
        const uint32_t tile = s_tile;
        if (tile >= ntiles) break;
        if (tile == 0)
            for (uint32_t r = threadIdx.x; r < ninj; r += blockDim.x) {
                nxt.coord[r] = inj[r].coord;
                if (LEAVES) {
                    // a job whose root is a leaf: its leaf range is that root
                    const Injected q = inj[r];
                    const uint32_t j = leaf_resolve_one(nxt, njobs, lc, lf, r, leaf_rec_fetch(lc, jobs, njobs, q.coord, q.job),
                                                        q.job, err);
                    nxt.job[r] = j;
                    seg.nstart[seg_index(j, L - 1)] = r;
                    seg.nend[seg_index(j, L - 1)] = r + 1;
                } else {
                    nxt.job[r] = inj[r].job;
                }
            }
        const uint32_t l0 = threadIdx.x * kExpItems;  // first node of this thread within the tile
        const uint32_t b0 = tile * kExpTile + l0;
        uint32_t jv[kExpItems];
        uint64_t cv[kExpItems];
        if (b0 + kExpItems <= n) {
            const uint4 j4 = *reinterpret_cast<const uint4*>(cur.job + b0);
            const ulonglong2 c01 = *reinterpret_cast<const ulonglong2*>(cur.coord + b0);
            const ulonglong2 c23 = *reinterpret_cast<const ulonglong2*>(cur.coord + b0 + 2);
            jv[0] = j4.x; jv[1] = j4.y; jv[2] = j4.z; jv[3] = j4.w;
            cv[0] = c01.x; cv[1] = c01.y; cv[2] = c23.x; cv[3] = c23.y;
        } else {
#pragma unroll
            for (int it = 0; it < kExpItems; ++it) {
                const bool in = b0 + it < n;
                jv[it] = in ? cur.job[b0 + it] : 0u;
                cv[it] = in ? cur.coord[b0 + it] : 0ull;
            }
        }
        uint32_t m[kExpItems], ksum = 0;
        bool bad_job = false, bad_node = false;
#pragma unroll
        for (int it = 0; it < kExpItems; ++it) {
            m[it] = 0;
            if (b0 + it < n) {
                if (jv[it] < njobs) {
                    m[it] = node_mask_nf(jobs[jv[it]], L, cv[it], bad_node);
                } else {
                    bad_job = true;
                    jv[it] = 0;
                }
            }
            ksum += partial_children(m[it]);
        }
        if (bad_job) atomicOr(err, 8u);
        if (bad_node) atomicOr(err, 4u);
        uint2 tot;
        const uint32_t pre = block_exclusive_scan2(make_uint2(ksum, 0u), tot, sm).x;
        if (threadIdx.x < 32) {
            const uint32_t e = lookback(flags, tile, make_uint2(tot.x, 0u), err).x;
            if (threadIdx.x == 0) s_excl = e;
        }
        // the tile's parents and, per child, its parent and slot, for the
        // cooperative writes
        uint32_t off = pre;
#pragma unroll
        for (int it = 0; it < kExpItems; ++it) {
            s_coord[l0 + it] = cv[it];
            s_job[l0 + it] = jv[it];
            uint32_t pb = partial_set(m[it]);
            while (pb) {
                const uint32_t ch = (uint32_t)__ffs((int)pb) - 1u;
                pb &= pb - 1u;
                s_child[off++] = (uint16_t)(((l0 + it) << 3) | ch);
            }
        }
        __syncthreads();
        const uint32_t f0 = ninj + s_excl;  // first child of the tile in level L-1
        // per parent: first child, overflow, job boundaries
        uint32_t poff = pre;
#pragma unroll
        for (int it = 0; it < kExpItems; ++it) {
            const uint32_t i = b0 + it;
            if (i >= n) break;
            const uint32_t k = partial_children(m[it]);
            const uint32_t f = f0 + poff;
            poff += k;
            if (f + k > cap_next) {
                // more children than the level bound: they are not written;
                // reported, and the plan grows
                atomicOr(err, 1u);
                m[it] &= 0x5555u;
                cur.first[i] = 0;
            } else {
                cur.first[i] = f;
            }
            cur.mask[i] = m[it];
            if (jv[it] != cur.job[i]) cur.job[i] = jv[it];
            const uint32_t j = jv[it];
            const bool jfirst = i == 0 || cur.job[i - 1] != j, jlast = i == n - 1 || cur.job[i + 1] != j;
            if (jfirst) seg.nstart[seg_index(j, L)] = i;
            if (jlast) seg.nend[seg_index(j, L)] = i + 1;
            if (LEAVES) {
                // the job's leaves: from its first node's first child to
                // its last node's last child
                if (jfirst) seg.nstart[seg_index(j, L - 1)] = f;
                if (jlast) seg.nend[seg_index(j, L - 1)] = f + k;
            }
        }
        // cs::getChildCoordinates (src/CompressedShadowUtil.cpp:101-117),
        // one child per thread and step
        const uint32_t C = tot.x;
        auto child_coord = [&](uint32_t c, uint32_t& j) {
            const uint32_t e = s_child[c];
            const uint32_t lo = e >> 3, ch = e & 7u;
            const uint64_t pc = s_coord[lo];
            const uint32_t x = unpack_x(pc), y = unpack_y(pc), z = unpack_z(pc);
            j = s_job[lo];
            return pack_xyz((x + (ch & 1u)) * 2u, (y + ((ch >> 1) & 1u)) * 2u, (z + (ch >> 2)) * 2u);
        };
        const uint32_t Cw = min(C, cap_next > f0 ? cap_next - f0 : 0u);  // children that fit the level
        if (LEAVES) {
            // one leaf per thread and step (requesting several leaves'
            // column records together measured slower: the registers it
            // takes cost more occupancy than the overlap gains)
            for (uint32_t c = threadIdx.x; c < Cw; c += blockDim.x) {
                uint32_t j;
                const uint64_t cc = child_coord(c, j);
                nxt.job[f0 + c] = leaf_resolve_one(nxt, njobs, lc, lf, f0 + c, leaf_rec_fetch(lc, jobs, njobs, cc, j), j, err);
            }
        } else {
            for (uint32_t c = threadIdx.x; c < Cw; c += blockDim.x) {
                uint32_t j;
                nxt.coord[f0 + c] = child_coord(c, j);
                nxt.job[f0 + c] = j;
            }
        }
        if (tile == ntiles - 1 && threadIdx.x == 0) {
            const uint32_t total = f0 + tot.x;
            if (total > cap_next) atomicOr(err, 1u);
            counts[L - 1] = total < cap_next ? total : cap_next;
        }
        __syncthreads();
    }
    if (LEAVES) {
        __syncthreads();
        leaf_first_flush(lc, lf);
    }
}

// Hash insert of inner node i into `table` (dedup_insert's rule: the slot
// ends with the class's first occurrence); children are compared by their
// merged identities (class slots).  The node's child identities, and on a tag match
// the candidate's, are requested as independent loads before they are used,
// so a node costs two dependent round trips for its children instead of one
// per child.
template <bool CG>
__device__ __forceinline__ void load_child_ids(const LevelDev& child, uint32_t f, uint32_t k, uint32_t u[8]) {
#pragma unroll
    for (uint32_t r = 0; r < 8; ++r) u[r] = r < k ? child_uid<CG>(child, f + r) : 0u;
}

// Signature hash of an inner node: job, child mask and the k child
// identities in order.
__device__ __forceinline__ uint64_t inner_hash(uint32_t j, uint32_t m, uint32_t k, const uint32_t u[8]) {
    uint64_t h = fmix64((((uint64_t)j + 1) << 32 | m) ^ kGolden);
#pragma unroll
    for (uint32_t r = 0; r < 8; ++r)
        if (r < k) h = fmix64(h ^ ((uint64_t)u[r] + (uint64_t)(r + 1) * kGolden));
    return h;
}

template <bool CG>
__device__ __forceinline__ uint32_t insert_inner(LevelDev& cur, const LevelDev& child, uint32_t i, uint32_t m,
                                                 uint32_t j, uint32_t f, unsigned long long* table,
                                                 uint64_t cap_mask, uint32_t* err) {
    const uint32_t k = partial_children(m);
    uint32_t u[8];
    load_child_ids<CG>(child, k ? f : 0u, k, u);
    const uint64_t h = inner_hash(j, m, k, u);
    const unsigned long long key = (h & 0xFFFFFFFF00000000ull) | i;
    uint64_t s = h & cap_mask;
    bool placed = false;
    for (uint64_t probe = 0; probe <= cap_mask; ++probe) {
        unsigned long long e = __ldcg(&table[s]);
        if (e == kEmptySlot) {
            const unsigned long long prev = atomicCAS(&table[s], kEmptySlot, key);
            if (prev == kEmptySlot) {
                placed = true;
                break;
            }
            e = prev;
        }
        if ((e >> 32) == (key >> 32)) {
            // the candidate's job, mask and first child in one round of loads
            const uint32_t b = (uint32_t)e;
            const uint32_t jb = cur.job[b], mb = cur.mask[b], fb = cur.first[b];
            bool same = jb == j && mb == m;
            if (same && k) {
                uint32_t v[8];
                load_child_ids<CG>(child, fb, k, v);
#pragma unroll
                for (uint32_t r = 0; r < 8; ++r) same = same && (r >= k || u[r] == v[r]);
            }
            if (same) {
                if (b > i) atomicMin(&table[s], key);
                placed = true;
                break;
            }
        }
        s = (s + 1) & cap_mask;
    }
    if (!placed) atomicOr(err, 16u);  // table full: the result is void, reported
    cur.slot[i] = (uint32_t)s;
    return (uint32_t)s;
}

// Kept nodes of level L in node order: rank, word offset, the rank in the
// slot's upper half, job boundaries; the level's totals from the last tile.
// Each thread takes eight consecutive nodes; their slots, masks and jobs are
// loaded as vectors and all eight table entries requested before any store.
template <bool LEAF>
__global__ void __launch_bounds__(kThreads)
    k_merge_scan_lb(LevelDev cur, const uint32_t* __restrict__ counts, uint32_t* level_u, int L, SegDev seg,
                    uint32_t njobs, unsigned int* ticket, unsigned long long* flags, uint32_t* err) {
    chain_enter();
    __shared__ uint32_t sm[64];
    __shared__ uint32_t s_tile;
    __shared__ uint2 s_excl;
    const uint32_t n = counts[L];
    const uint32_t ntiles = n ? (n + kScanTile - 1) / kScanTile : 1u;
    for (;;) {
        if (threadIdx.x == 0) s_tile = atomicAdd(ticket, 1u);
        __syncthreads();
        const uint32_t tile = s_tile;
        if (tile >= ntiles) break;
        const uint32_t b0 = tile * kScanTile + threadIdx.x * kScanItems;
        const bool full = b0 + kScanItems <= n;
        uint32_t sl[kScanItems], mk[kScanItems], jb[kScanItems];
        if (full) {
#pragma unroll
            for (int h = 0; h < kScanItems; h += 4) {
                const uint4 a4 = *reinterpret_cast<const uint4*>(cur.slot + b0 + h);
                const uint4 m4 = *reinterpret_cast<const uint4*>(cur.mask + b0 + h);
                const uint4 j4 = *reinterpret_cast<const uint4*>(cur.job + b0 + h);
                sl[h] = a4.x; sl[h + 1] = a4.y; sl[h + 2] = a4.z; sl[h + 3] = a4.w;
                mk[h] = m4.x; mk[h + 1] = m4.y; mk[h + 2] = m4.z; mk[h + 3] = m4.w;
                jb[h] = j4.x; jb[h + 1] = j4.y; jb[h + 2] = j4.z; jb[h + 3] = j4.w;
            }
        } else {
#pragma unroll
            for (int it = 0; it < kScanItems; ++it) {
                const bool in = b0 + it < n;
                sl[it] = in ? cur.slot[b0 + it] : 0u;
                mk[it] = in ? cur.mask[b0 + it] : 0u;
                jb[it] = in ? cur.job[b0 + it] : 0u;
            }
        }
        const uint32_t jprev = (b0 > 0 && b0 <= n) ? cur.job[b0 - 1] : ~0u;
        const uint32_t jnext = (b0 + kScanItems < n) ? cur.job[b0 + kScanItems] : ~0u;
        uint32_t rep[kScanItems];
#pragma unroll
        for (int it = 0; it < kScanItems; ++it)
            rep[it] = b0 + it < n ? __ldcg(reinterpret_cast<const uint32_t*>(cur.table + sl[it])) : ~0u;
        uint32_t kept = 0, cnt = 0, words = 0;
#pragma unroll
        for (int it = 0; it < kScanItems; ++it)
            if (rep[it] == b0 + it) {
                kept |= 1u << it;
                ++cnt;
                words += node_words(mk[it], LEAF);
            }
        uint2 tot;
        const uint2 pre = block_exclusive_scan2(make_uint2(cnt, words), tot, sm);
        if (threadIdx.x < 32) {
            const uint2 e = lookback(flags, tile, tot, err);
            if (threadIdx.x == 0) s_excl = e;
        }
        __syncthreads();
        uint32_t qx = s_excl.x + pre.x, qy = s_excl.y + pre.y;
#pragma unroll
        for (int it = 0; it < kScanItems; ++it) {
            const uint32_t i = b0 + it;
            if (i >= n) break;
            const uint32_t j = jb[it] < njobs ? jb[it] : 0u;
            if (jb[it] >= njobs) atomicOr(err, 128u);  // a node's job out of range: reported, not followed
            const uint32_t jl = it == 0 ? jprev : jb[it - 1];
            const uint32_t jr = it == kScanItems - 1 ? jnext : jb[it + 1];
            if (i == 0 || jl != j) {
                seg.ustart[seg_index(j, L)] = qx;
                seg.wstart[seg_index(j, L)] = qy;
            }
            if (kept & (1u << it)) {
                cur.uniq[qx] = i;
                cur.woff[qx] = qy;
                reinterpret_cast<uint32_t*>(cur.table + sl[it])[1] = qx;  // upper half: the rank
                ++qx;
                qy += node_words(mk[it], LEAF);
            }
            if (i == n - 1 || jr != j) {
                seg.uend[seg_index(j, L)] = qx;
                seg.wend[seg_index(j, L)] = qy;
            }
        }
        if (tile == ntiles - 1 && threadIdx.x == 0) {
            level_u[2 * L] = s_excl.x + tot.x;
            level_u[2 * L + 1] = s_excl.y + tot.y;
        }
        __syncthreads();
    }
}

// The small top levels (at most kClusterItems * 1024 nodes per block) run as
// one thread-block cluster (up to 16 blocks of 1024 threads on one GPC) in
// one launch for the expansion and one for the merge.  Each level is split
// into contiguous per-block ranges; block totals cross the cluster through
// distributed shared memory, and a cluster barrier separates the passes and
// the levels.  Node data written by other blocks of the same launch is read
// from L2 (ld.global.cg).
constexpr int kClusterThreads = 1024;
constexpr int kClusterItems = 4;
constexpr int kClusterMaxBlocks = 16;
constexpr uint32_t kClusterLevelCap = 8192;  // default: planned nodes of a level that the cluster kernels take, at most
constexpr uint32_t kClusterCaps[] = {2048, 4096, 8192, 16384};  // the candidates a plan's tuner times

struct SmallLevels {
    uint32_t inj_off[CPVS_MAX_LEVELS];
    uint32_t ninj[CPVS_MAX_LEVELS];
    uint32_t cap[CPVS_MAX_LEVELS];
};

// Exclusive prefix of this block's `v` over the lower-ranked blocks of the
// cluster, and the cluster total (every thread calls it; `v` is uniform).
__device__ __forceinline__ uint2 cluster_prefix(cg::cluster_group& cl, uint2 v, uint2* s_tot, uint2& total) {
    const uint32_t nb = cl.num_blocks(), rank = cl.block_rank();
    if (threadIdx.x < nb) cl.map_shared_rank(s_tot, threadIdx.x)[rank] = v;
    cl.sync();
    uint2 p = make_uint2(0u, 0u), t = make_uint2(0u, 0u);
    for (uint32_t r = 0; r < nb; ++r) {
        const uint2 x = s_tot[r];
        if (r < rank) {
            p.x += x.x;
            p.y += x.y;
        }
        t.x += x.x;
        t.y += x.y;
    }
    total = t;
    return p;
}

// The topmost levels, while a level holds few enough nodes, run in the
// cluster's first block alone with the level's node data in shared memory
// (and, for one job, the top pyramid levels): a level then costs a few block
// barriers instead of several global round trips and cluster barriers.  The merge keeps its hash table in shared memory;
// every node's class slot there is also its slot in the level's global table
// (the shared table is never larger), which receives the class's rank for
// the emission.
// Expansion: a level of at most kTopNodes nodes whose children fit in
// kTopChildren runs in the first block (the children are gathered in shared
// memory and written out coalesced); the first level that does not goes to
// the cluster.  Merge: levels of at most kTopMergeNodes nodes.
constexpr uint32_t kTopNodes = 2048;
constexpr uint32_t kTopChildren = 8192;
constexpr int kTopItems = kTopNodes / kClusterThreads;
constexpr uint32_t kTopMergeNodes = 4096;
constexpr int kTopMergeItems = kTopMergeNodes / kClusterThreads;
constexpr uint32_t kTopTable = 2 * kTopMergeNodes;

constexpr uint32_t kTopPyrLog = 5;       // expansion: pyramid levels of side <= 2^5 held on chip (one job)
constexpr uint32_t kTopPyr = 1366;       // their texels: 32^2 + 16^2 + ... + 1, rounded up to even
constexpr uint32_t kTopJobs = 32;        // job tables of at most this many jobs held on chip
struct ExpandTopSmem {
    uint64_t coord[2][kTopChildren];
    uint32_t job[2][kTopChildren];
    uint32_t mask[kTopNodes], first[kTopNodes];
    float2 pyr[kTopPyr];
};
constexpr uint32_t kTopPreload = 8192;  // merge: node data of all top levels held at once
constexpr uint32_t kTopSlots = 8192;    // merge: class slots of a level (the one below the top levels included)
struct MergeTopSmem {
    unsigned long long table[kTopTable];
    uint32_t mask[kTopPreload], job[kTopPreload], first[kTopPreload];
    uint32_t slot[2][kTopSlots];
};
constexpr size_t kExpandClusterSmem = sizeof(ExpandTopSmem);
constexpr size_t kMergeClusterSmem = sizeof(MergeTopSmem);

// Expands levels Lhi, Lhi-1, ... (not below Llo) in one block, after placing
// the roots of level Lhi, while a level fits (see above); writes the highest
// level left to expand (Llo - 1 when none) to *next.
// `lvt` and `jobs` may be shared-memory copies; with Lp <= Lhi, S.pyr holds
// pyramid levels Lp.. of the single job's map.
__device__ __forceinline__ void expand_top(ExpandTopSmem& S, const LevelDev* lvt, uint32_t* counts,
                                           const JobDev* jobs, uint32_t njobs, int Lhi, int Llo,
                                           const Injected* __restrict__ inj_all, const SmallLevels& sl, SegDev seg,
                                           uint32_t* err, uint32_t* sm, uint32_t* next, int Lp) {
    const uint32_t tid = threadIdx.x;
    const uint64_t pyr_base = Lp <= Lhi ? pyramid_level_offset_dev(jobs[0].n, Lp) : 0ull;
    uint32_t n = sl.ninj[Lhi];
    {
        LevelDev top = lvt[Lhi];
        const Injected* inj = inj_all + sl.inj_off[Lhi];
        for (uint32_t r = tid; r < n; r += blockDim.x) {
            const Injected q = inj[r];
            top.coord[r] = q.coord;
            top.job[r] = q.job;
            if (r < kTopChildren) {
                S.coord[0][r] = q.coord;
                S.job[0][r] = q.job;
            }
        }
        if (tid == 0) counts[Lhi] = n;
    }
    __syncthreads();
    int b = 0, L = Lhi;
    for (; L >= Llo && n <= kTopNodes; --L) {
        LevelDev cur = lvt[L], nxt = lvt[L - 1];
        // classification: node_mask (src/CompressedShadow.cpp:270-315)
        bool bad_job = false, bad_node = false;
#pragma unroll
        for (int it = 0; it < kTopItems; ++it) {
            const uint32_t i = tid + it * kClusterThreads;
            if (i < n) {
                const uint32_t j = S.job[b][i];
                uint32_t m = 0;
                if (j < njobs) {
                    const JobDev& J = jobs[j];
                    if (L >= Lp) {
                        const uint32_t W = J.n >> L;
                        m = node_mask_at(S.pyr + (pyramid_level_offset_dev(J.n, L) - pyr_base), W,
                                         __uint2float_rn(W * J.z_num), S.coord[b][i], bad_node);
                    } else {
                        m = node_mask_nf(J, L, S.coord[b][i], bad_node);
                    }
                } else {
                    bad_job = true;
                    S.job[b][i] = 0;
                    cur.job[i] = 0;
                }
                S.mask[i] = m;
            }
        }
        if (bad_job) atomicOr(err, 8u);
        if (bad_node) atomicOr(err, 4u);
        __syncthreads();
        // children in node order: consecutive nodes per thread
        const uint32_t i0 = tid * kTopItems;
        uint32_t ksum = 0;
#pragma unroll
        for (int it = 0; it < kTopItems; ++it) ksum += i0 + it < n ? partial_children(S.mask[i0 + it]) : 0u;
        uint2 tot;
        const uint32_t pre = block_exclusive_scan2(make_uint2(ksum, 0u), tot, sm).x;
        const uint32_t ninj = sl.ninj[L - 1], cap_next = sl.cap[L - 1];
        const uint32_t total = ninj + tot.x;
        if (total > kTopChildren) break;  // uniform: the cluster takes this level
        uint32_t f = ninj + pre;
#pragma unroll
        for (int it = 0; it < kTopItems; ++it) {
            const uint32_t i = i0 + it;
            if (i < n) {
                uint32_t m = S.mask[i];
                const uint32_t k = partial_children(m);
                if (f + k > cap_next) {
                    atomicOr(err, 1u);  // more children than the level holds: not written, reported
                    S.mask[i] = m & 0x5555u;
                    S.first[i] = 0;
                } else {
                    S.first[i] = f;
                    const uint64_t c = S.coord[b][i];
                    const uint32_t j = S.job[b][i];
                    const uint32_t x = unpack_x(c), y = unpack_y(c), z = unpack_z(c);
                    uint32_t r = 0;
                    for (uint32_t ch = 0; ch < 8; ++ch)
                        if (m & (2u << (2u * ch))) {
                            // cs::getChildCoordinates (src/CompressedShadowUtil.cpp:101-117)
                            S.coord[b ^ 1][f + r] =
                                pack_xyz((x + (ch & 1u)) * 2u, (y + ((ch >> 1) & 1u)) * 2u, (z + (ch >> 2)) * 2u);
                            S.job[b ^ 1][f + r] = j;
                            ++r;
                        }
                }
                f += k;
            }
        }
        const Injected* inj = inj_all + sl.inj_off[L - 1];
        for (uint32_t r = tid; r < ninj; r += blockDim.x) {
            const Injected q = inj[r];
            S.coord[b ^ 1][r] = q.coord;
            S.job[b ^ 1][r] = q.job;
        }
        __syncthreads();
        // the level's node data and the children, coalesced
        for (uint32_t i = tid; i < n; i += blockDim.x) {
            const uint32_t j = S.job[b][i];
            cur.mask[i] = S.mask[i];
            cur.first[i] = S.first[i];
            if (i == 0 || S.job[b][i - 1] != j) seg.nstart[seg_index(j, L)] = i;
            if (i == n - 1 || S.job[b][i + 1] != j) seg.nend[seg_index(j, L)] = i + 1;
        }
        const uint32_t nn = total < cap_next ? total : cap_next;
        for (uint32_t c = tid; c < nn; c += blockDim.x) {
            nxt.coord[c] = S.coord[b ^ 1][c];
            nxt.job[c] = S.job[b ^ 1][c];
        }
        if (tid == 0) {
            if (total > cap_next) atomicOr(err, 1u);
            counts[L - 1] = nn;
        }
        n = nn;
        b ^= 1;
        __syncthreads();
    }
    if (tid == 0) *next = (uint32_t)L;
}

// Expansion of levels Lhi (whose roots this kernel writes) down to Llo, each
// into the level below it: the topmost in the first block alone, the rest
// across the cluster.
__global__ void __launch_bounds__(kClusterThreads, 1)
    k_expand_cluster(const LevelDev* __restrict__ lvt, uint32_t* counts, const JobDev* __restrict__ jobs,
                     uint32_t njobs, int Lhi, int Llo, const Injected* __restrict__ inj_all, SmallLevels sl,
                     SegDev seg, uint32_t* top_next, uint32_t* err) {
    chain_enter();
    cg::cluster_group cl = cg::this_cluster();
    const uint32_t nb = cl.num_blocks(), rank = cl.block_rank();
    extern __shared__ __align__(16) unsigned char dyn_smem[];
    __shared__ uint32_t sm[64];
    __shared__ uint2 s_tot[kClusterMaxBlocks];
    // the level table and (small) job table on chip, and for one job the
    // top pyramid levels that the first block classifies against
    __shared__ __align__(16) LevelDev s_lv[CPVS_MAX_LEVELS];
    __shared__ __align__(16) JobDev s_jobs[kTopJobs];
    fetch_async(s_lv, lvt, (uint32_t)(CPVS_MAX_LEVELS * sizeof(LevelDev)));
    if (njobs <= kTopJobs) fetch_async(s_jobs, jobs, (uint32_t)(njobs * sizeof(JobDev)));
    int Lp = CPVS_MAX_LEVELS;
    if (rank == 0 && njobs == 1) {
        ExpandTopSmem& S = *reinterpret_cast<ExpandTopSmem*>(dyn_smem);
        const float2* pyr = jobs[0].pyr;
        const uint32_t nm = jobs[0].n, lg = 31u - (uint32_t)__clz((int)nm);
        Lp = lg > kTopPyrLog ? (int)(lg - kTopPyrLog) : 1;  // side (nm >> Lp) <= 2^kTopPyrLog
        const uint64_t o = pyramid_level_offset_dev(nm, Lp);
        fetch_async(S.pyr, pyr + o, (uint32_t)((pyramid_level_offset_dev(nm, (int)lg + 1) - o) * sizeof(float2)));
    }
    fetch_wait();
    const JobDev* jt = njobs <= kTopJobs ? s_jobs : jobs;
    if (rank == 0)
        expand_top(*reinterpret_cast<ExpandTopSmem*>(dyn_smem), s_lv, counts, jt, njobs, Lhi, Llo, inj_all, sl, seg,
                   err, sm, top_next, Lp);
    cl.sync();
    const int Lstart = (int)__ldcg(top_next);
    // the cluster levels: each block takes a contiguous range of the level,
    // kClusterItems consecutive nodes per thread; its node data stays in
    // registers and shared memory, and the next level's size follows from
    // the cluster total, so a level costs two rounds of loads (node data,
    // then pyramid texels) and two cluster barriers
    uint32_t* s_job = reinterpret_cast<uint32_t*>(dyn_smem);  // [kClusterItems * kClusterThreads + 2]
    uint32_t n = Lstart >= Llo ? __ldcg(counts + Lstart) : 0u;
    for (int L = Lstart; L >= Llo; --L) {
        LevelDev cur = s_lv[L], nxt = s_lv[L - 1];
        const uint32_t per = ((n + nb - 1) / nb + 3u) & ~3u;
        const uint32_t lo = min(n, rank * per), hi = min(n, lo + per);
        if (hi - lo > (uint32_t)(kClusterItems * kClusterThreads)) atomicOr(err, 1u);  // the plan sized this level
        const uint32_t i0 = lo + threadIdx.x * kClusterItems;
        uint32_t m[kClusterItems], jv[kClusterItems], ksum = 0, badj = 0;
        uint64_t cv[kClusterItems];
        bool bad_node = false;
#pragma unroll
        for (int it = 0; it < kClusterItems; ++it) {
            const uint32_t i = i0 + it;
            jv[it] = i < hi ? __ldcg(cur.job + i) : 0u;
            cv[it] = i < hi ? __ldcg(cur.coord + i) : 0ull;
        }
        // the jobs of the range's neighbours (for the segment boundaries)
        if (threadIdx.x == 0) {
            s_job[0] = lo > 0 && lo < n ? __ldcg(cur.job + lo - 1) : ~0u;
            s_job[1 + (hi - lo)] = hi < n ? __ldcg(cur.job + hi) : ~0u;
        }
#pragma unroll
        for (int it = 0; it < kClusterItems; ++it) {
            const uint32_t i = i0 + it;
            m[it] = 0;
            if (i < hi) {
                if (jv[it] < njobs) {
                    m[it] = node_mask_nf(jt[jv[it]], L, cv[it], bad_node);
                } else {
                    badj |= 1u << it;
                    jv[it] = 0;
                }
            }
            if (i < hi) s_job[1 + threadIdx.x * kClusterItems + it] = jv[it];
            ksum += partial_children(m[it]);
        }
        if (badj) atomicOr(err, 8u);
        if (bad_node) atomicOr(err, 4u);
        uint2 btot, ctot;
        const uint32_t pre = block_exclusive_scan2(make_uint2(ksum, 0u), btot, sm).x;
        const uint2 bpre = cluster_prefix(cl, btot, s_tot, ctot);
        const uint32_t ninj = sl.ninj[L - 1], cap_next = sl.cap[L - 1];
        uint32_t f = ninj + bpre.x + pre;
#pragma unroll
        for (int it = 0; it < kClusterItems; ++it) {
            const uint32_t i = i0 + it;
            if (i >= hi) break;
            uint32_t mi = m[it];
            const uint32_t k = partial_children(mi);
            if (f + k > cap_next) {
                atomicOr(err, 1u);  // more children than the level holds: not written, reported
                mi &= 0x5555u;
                cur.first[i] = 0;
            } else {
                cur.first[i] = f;
                const uint32_t x = unpack_x(cv[it]), y = unpack_y(cv[it]), z = unpack_z(cv[it]);
                uint32_t r = 0;
#pragma unroll
                for (uint32_t ch = 0; ch < 8; ++ch)
                    if (mi & (2u << (2u * ch))) {
                        // cs::getChildCoordinates (src/CompressedShadowUtil.cpp:101-117)
                        nxt.coord[f + r] =
                            pack_xyz((x + (ch & 1u)) * 2u, (y + ((ch >> 1) & 1u)) * 2u, (z + (ch >> 2)) * 2u);
                        nxt.job[f + r] = jv[it];
                        ++r;
                    }
            }
            cur.mask[i] = mi;
            if (badj & (1u << it)) cur.job[i] = 0;
            const uint32_t j = jv[it], li = 1 + threadIdx.x * kClusterItems + it;
            if (i == 0 || s_job[li - 1] != j) seg.nstart[seg_index(j, L)] = i;
            if (i == n - 1 || s_job[li + 1] != j) seg.nend[seg_index(j, L)] = i + 1;
            f += k;
        }
        const uint32_t total = ninj + ctot.x;
        if (rank == 0) {
            const Injected* inj = inj_all + sl.inj_off[L - 1];
            for (uint32_t r = threadIdx.x; r < ninj; r += blockDim.x) {
                nxt.coord[r] = inj[r].coord;
                nxt.job[r] = inj[r].job;
            }
            if (threadIdx.x == 0) {
                if (total > cap_next) atomicOr(err, 1u);
                counts[L - 1] = total < cap_next ? total : cap_next;
            }
        }
        n = total < cap_next ? total : cap_next;
        cl.sync();
    }
}

// Merge of levels Llo..Lhi in one block (each level at most kTopMergeNodes
// nodes): insert into the shared table (the leaf level was inserted into its
// global table by the leaf kernel), then ranks and word offsets in node
// order, as the multi-block passes compute them.  The node data of all these
// levels, and the class slots of the level below them, are loaded into
// shared memory up front when they fit, so a level then runs on chip.
__device__ __forceinline__ void merge_top(MergeTopSmem& S, const LevelDev* lvt,
                                          const uint32_t* __restrict__ counts, const uint32_t* s_cnt,
                                          uint32_t* level_u, int Llo, int Lhi, int bottom, int leaf_level,
                                          SegDev seg, uint32_t* err, uint32_t* sm) {
    const uint32_t tid = threadIdx.x;
    uint32_t base[CPVS_MAX_LEVELS], total = 0;  // level offsets, multiples of four nodes
    for (int L = Llo; L <= Lhi; ++L) {
        base[L] = total;
        total += (s_cnt[L] + 3u) & ~3u;
    }
    const bool pre = total <= kTopPreload;
    if (pre)
        for (int L = Llo; L <= Lhi; ++L) {
            const LevelDev& cur = lvt[L];
            fetch_async(S.mask + base[L], cur.mask, s_cnt[L] * 4u);
            fetch_async(S.job + base[L], cur.job, s_cnt[L] * 4u);
            if (L != leaf_level) fetch_async(S.first + base[L], cur.first, s_cnt[L] * 4u);
        }
    int cb = 0;  // S.slot[cb]: class slots of the level below
    bool child_here = false;
    if (Llo > bottom) {
        const uint32_t nc = __ldcg(counts + Llo - 1);
        if (((nc + 3u) & ~3u) <= kTopSlots) {
            fetch_async(S.slot[0], lvt[Llo - 1].slot, nc * 4u);
            child_here = true;
        }
    }
    fetch_wait();
    for (int L = Llo; L <= Lhi; ++L) {
        LevelDev cur = lvt[L];
        const LevelDev child = L > bottom ? lvt[L - 1] : lvt[L];
        const bool leaf = L == leaf_level;
        const uint32_t n = s_cnt[L];
        const uint32_t off = pre ? base[L] : 0u;
        uint32_t* my_slot = S.slot[cb ^ 1];
        const uint32_t* child_slot = S.slot[cb];
        const uint32_t* mask = S.mask + off;
        const uint32_t* job = S.job + off;
        const uint32_t* first = S.first + off;
        uint32_t T = 64;
        while (T < 2 * n && T < kTopTable) T <<= 1;
        if (T > cur.table_mask + 1) T = (uint32_t)(cur.table_mask + 1);
        for (uint32_t i = tid; i < n; i += blockDim.x) {
            if (!pre) {
                S.mask[i] = __ldcg(cur.mask + i);
                S.job[i] = __ldcg(cur.job + i);
                if (!leaf) S.first[i] = __ldcg(cur.first + i);
            }
            if (leaf) my_slot[i] = __ldcg(cur.slot + i);
        }
        if (!leaf)
            for (uint32_t s = tid; s < T; s += blockDim.x) S.table[s] = kEmptySlot;
        __syncthreads();
        if (!leaf) {
            for (uint32_t i = tid; i < n; i += blockDim.x) {
                const uint32_t m = mask[i], j = job[i], k = partial_children(m);
                const uint32_t f = k ? first[i] : 0u;
                uint32_t u[8];
#pragma unroll
                for (uint32_t r = 0; r < 8; ++r)
                    u[r] = r < k ? (child_here ? child_slot[f + r] : __ldcg(child.slot + f + r)) : 0u;
                const uint64_t h = inner_hash(j, m, k, u);
                const unsigned long long key = (h & 0xFFFFFFFF00000000ull) | i;
                uint32_t s = (uint32_t)h & (T - 1);
                bool placed = false;
                for (uint32_t probe = 0; probe < T; ++probe) {
                    unsigned long long e = *reinterpret_cast<volatile unsigned long long*>(S.table + s);
                    if (e == kEmptySlot) {
                        const unsigned long long prev = atomicCAS(S.table + s, kEmptySlot, key);
                        if (prev == kEmptySlot) {
                            placed = true;
                            break;
                        }
                        e = prev;
                    }
                    if ((e >> 32) == (key >> 32)) {
                        const uint32_t bn = (uint32_t)e;
                        bool same = job[bn] == j && mask[bn] == m;
                        if (same && k) {
                            const uint32_t fb = first[bn];
#pragma unroll
                            for (uint32_t r = 0; r < 8; ++r)
                                if (r < k)
                                    same = same && u[r] == (child_here ? child_slot[fb + r]
                                                                       : __ldcg(child.slot + fb + r));
                        }
                        if (same) {
                            if (bn > i) atomicMin(S.table + s, key);
                            placed = true;
                            break;
                        }
                    }
                    s = (s + 1) & (T - 1);
                }
                if (!placed) atomicOr(err, 16u);  // table full: the result is void, reported
                my_slot[i] = s;
            }
            __syncthreads();
        }
        // kept nodes (first occurrences) in node order: consecutive nodes per thread
        const uint32_t i0 = tid * kTopMergeItems;
        uint32_t kept = 0, cnt = 0, words = 0, rep[kTopMergeItems];
#pragma unroll
        for (int it = 0; it < kTopMergeItems; ++it) {
            const uint32_t i = i0 + it;
            rep[it] = ~0u;
            if (i < n) {
                const uint32_t s = my_slot[i];
                rep[it] = leaf ? __ldcg(reinterpret_cast<const uint32_t*>(cur.table + s)) : (uint32_t)S.table[s];
                if (rep[it] == i) {
                    kept |= 1u << it;
                    ++cnt;
                    words += node_words(mask[i], leaf);
                }
            }
        }
        uint2 tot;
        const uint2 pr = block_exclusive_scan2(make_uint2(cnt, words), tot, sm);
        uint32_t qx = pr.x, qy = pr.y;
#pragma unroll
        for (int it = 0; it < kTopMergeItems; ++it) {
            const uint32_t i = i0 + it;
            if (i >= n) break;
            const uint32_t j = job[i], s = my_slot[i];
            if (i == 0 || job[i - 1] != j) {
                seg.ustart[seg_index(j, L)] = qx;
                seg.wstart[seg_index(j, L)] = qy;
            }
            if (!leaf) cur.slot[i] = s;
            if (kept & (1u << it)) {
                cur.uniq[qx] = i;
                cur.woff[qx] = qy;
                if (leaf)
                    reinterpret_cast<uint32_t*>(cur.table + s)[1] = qx;  // upper half: the rank
                else
                    cur.table[s] = ((unsigned long long)qx << 32) | rep[it];
                ++qx;
                qy += node_words(mask[i], leaf);
            }
            if (i == n - 1 || job[i + 1] != j) {
                seg.uend[seg_index(j, L)] = qx;
                seg.wend[seg_index(j, L)] = qy;
            }
        }
        if (tid == 0) {
            level_u[2 * L] = tot.x;
            level_u[2 * L + 1] = tot.y;
        }
        __syncthreads();
        cb ^= 1;
        child_here = true;
    }
}

// Merge of levels Llo..Lhi (insert, then ranks and offsets); the leaf level
// (leaf_level, or -1) was inserted by k_leaf_insert.  The lower levels run
// across the cluster, the topmost (each at most kTopMergeNodes nodes) in the
// first block alone.
__global__ void __launch_bounds__(kClusterThreads, 1)
    k_merge_cluster(const LevelDev* __restrict__ lvt, const uint32_t* __restrict__ counts, uint32_t* level_u,
                    int Llo, int Lhi, int bottom, int leaf_level, SegDev seg, uint32_t* err) {
    chain_enter();
    cg::cluster_group cl = cg::this_cluster();
    const uint32_t nb = cl.num_blocks(), rank = cl.block_rank();
    extern __shared__ __align__(16) unsigned char dyn_smem[];
    __shared__ uint32_t sm[64];
    __shared__ uint2 s_tot[kClusterMaxBlocks];
    // counts are final here (the expansion has completed); the level table
    // on chip
    __shared__ uint32_t s_cnt[CPVS_MAX_LEVELS];
    __shared__ __align__(16) LevelDev s_lv[CPVS_MAX_LEVELS];
    if (threadIdx.x < CPVS_MAX_LEVELS)
        s_cnt[threadIdx.x] = (int)threadIdx.x >= Llo && (int)threadIdx.x <= Lhi ? counts[threadIdx.x] : 0u;
    fetch_async(s_lv, lvt, (uint32_t)(CPVS_MAX_LEVELS * sizeof(LevelDev)));
    fetch_wait();
    int Ltop = Lhi + 1;
    while (Ltop - 1 >= Llo && s_cnt[Ltop - 1] <= kTopMergeNodes) --Ltop;
    // the cluster levels: each block takes a contiguous range; the insert
    // runs over it strided (one node per thread and round), and the node's
    // slot, mask and job go to shared memory for the ranking pass, which
    // takes kClusterItems consecutive nodes per thread
    constexpr uint32_t kRange = kClusterItems * kClusterThreads;
    uint32_t* s_slot = reinterpret_cast<uint32_t*>(dyn_smem);
    uint32_t* s_mask = s_slot + kRange;
    uint32_t* s_job = s_mask + kRange;  // [kRange + 2]: the range's jobs between its neighbours'
    for (int L = Llo; L < Ltop; ++L) {
        LevelDev cur = s_lv[L];
        const LevelDev child = L > bottom ? s_lv[L - 1] : s_lv[L];
        const bool leaf = L == leaf_level;
        const uint32_t n = s_cnt[L];
        const uint32_t per = ((n + nb - 1) / nb + 3u) & ~3u;
        const uint32_t lo = min(n, rank * per), hi = min(n, lo + per);
        for (uint32_t i = lo + threadIdx.x; i < hi; i += blockDim.x) {
            uint3 r;
            r.y = cur.mask[i];
            r.z = cur.job[i];
            if (!leaf)
                r.x = insert_inner<true>(cur, child, i, r.y, r.z, cur.first[i], cur.table, cur.table_mask, err);
            else
                r.x = cur.slot[i];
            s_slot[i - lo] = r.x;
            s_mask[i - lo] = r.y;
            s_job[1 + i - lo] = r.z;
        }
        if (threadIdx.x == 0) {
            s_job[0] = lo > 0 && lo < n ? cur.job[lo - 1] : ~0u;
            s_job[1 + (hi - lo)] = hi < n ? cur.job[hi] : ~0u;
        }
        cl.sync();  // every slot final
        const uint32_t i0 = lo + threadIdx.x * kClusterItems;
        uint32_t rep[kClusterItems], kept = 0, cnt = 0, words = 0;
#pragma unroll
        for (int it = 0; it < kClusterItems; ++it)
            rep[it] = i0 + it < hi ? __ldcg(reinterpret_cast<const uint32_t*>(cur.table + s_slot[i0 + it - lo])) : ~0u;
#pragma unroll
        for (int it = 0; it < kClusterItems; ++it)
            if (rep[it] == i0 + it) {
                kept |= 1u << it;
                ++cnt;
                words += node_words(s_mask[i0 + it - lo], leaf);
            }
        uint2 btot, ctot;
        const uint2 pre = block_exclusive_scan2(make_uint2(cnt, words), btot, sm);
        const uint2 bpre = cluster_prefix(cl, btot, s_tot, ctot);
        uint32_t qx = bpre.x + pre.x, qy = bpre.y + pre.y;
#pragma unroll
        for (int it = 0; it < kClusterItems; ++it) {
            const uint32_t i = i0 + it;
            if (i >= hi) break;
            const uint32_t li = i - lo, j = s_job[1 + li];
            if (i == 0 || s_job[li] != j) {
                seg.ustart[seg_index(j, L)] = qx;
                seg.wstart[seg_index(j, L)] = qy;
            }
            if (kept & (1u << it)) {
                cur.uniq[qx] = i;
                cur.woff[qx] = qy;
                reinterpret_cast<uint32_t*>(cur.table + s_slot[li])[1] = qx;  // upper half: the rank
                ++qx;
                qy += node_words(s_mask[li], leaf);
            }
            if (i == n - 1 || s_job[2 + li] != j) {
                seg.uend[seg_index(j, L)] = qx;
                seg.wend[seg_index(j, L)] = qy;
            }
        }
        if (rank == 0 && threadIdx.x == 0) {
            level_u[2 * L] = ctot.x;
            level_u[2 * L + 1] = ctot.y;
        }
        cl.sync();  // class slots visible to the level above
    }
    if (rank == 0 && Ltop <= Lhi)
        merge_top(*reinterpret_cast<MergeTopSmem*>(dyn_smem), s_lv, counts, s_cnt, level_u, Ltop, Lhi, bottom,
                  leaf_level, seg, err, sm);
}

// ------------------------------------------------------------------ layout
// Per job: level bases top-down and the DAG size; then job offsets.
struct JobLayout {
    uint64_t* job_off;  // [njobs + 1]
    uint32_t* base;     // [job * L_MAX + level]: word offset of the level in the job's DAG
};

// With `root_mask` (and `lvt`), also the root mask of every job (the first
// word of its DAG).
__global__ void k_layout(SegDev seg, JobLayout lay, const uint32_t* __restrict__ root_level, uint32_t njobs, int bottom,
                         const LevelDev* __restrict__ lvt, uint32_t* root_mask) {
    chain_enter();
    // single block: each thread sums its jobs, then a block scan over jobs in
    // rounds of blockDim
    __shared__ uint32_t sm[64];
    uint64_t carry = 0;
    for (uint32_t j0 = 0; j0 < njobs; j0 += blockDim.x) {
        const uint32_t j = j0 + threadIdx.x;
        uint64_t total = 0;
        if (j < njobs) {
            if (root_mask) {
                const int R = (int)root_level[j];
                root_mask[j] = lvt[R].mask[seg.nstart[seg_index(j, R)]];
            }
            for (int L = (int)root_level[j]; L >= bottom; --L) {
                const uint32_t s = seg_index(j, L);
                lay.base[s] = (uint32_t)total;
                total += seg.wend[s] - seg.wstart[s];
            }
        }
        // totals stay below 2^32 words per job (checked on the host)
        uint2 tot;
        const uint2 p = block_exclusive_scan2(make_uint2((uint32_t)total, 0u), tot, sm);
        if (j < njobs) lay.job_off[j] = carry + p.x;
        carry += tot.x;
    }
    if (threadIdx.x == 0) lay.job_off[njobs] = carry;
}

template <bool LEAF>
__global__ void __launch_bounds__(kThreads)
    k_emit(LevelDev cur, LevelDev child, const uint32_t* __restrict__ level_u, int L, SegDev seg, JobLayout lay,
           uint32_t* __restrict__ out, uint64_t total_words, uint32_t* err) {
    const uint32_t U = level_u[2 * L];
    for (uint32_t u = blockIdx.x * blockDim.x + threadIdx.x; u < U; u += gridDim.x * blockDim.x) {
        const uint32_t i = cur.uniq[u];
        const uint32_t j = cur.job[i];
        const uint32_t sj = seg_index(j, L);
        const uint32_t m = cur.mask[i];
        const uint64_t at = lay.job_off[j] + lay.base[sj] + (cur.woff[u] - seg.wstart[sj]);
        if (at + node_words(m, LEAF) > total_words) {
            atomicOr(err, 2u);  // layout out of range: skip, report
            continue;
        }
        uint32_t* dst = out + at;
        dst[0] = m;
        if (LEAF) {
            uint32_t r = 0;
#pragma unroll
            for (uint32_t s = 0; s < 8; ++s)
                if (((m >> (2u * s)) & 3u) == kPartial) {
                    const uint64_t v = cur.slices[(size_t)i * 8 + s];
                    dst[1 + 2 * r] = (uint32_t)v;
                    dst[2 + 2 * r] = (uint32_t)(v >> 32);
                    ++r;
                }
        } else {
            // only nodes with children touch the level below (which does not
            // exist under the bottom level)
            const uint32_t k = partial_children(m);
            if (k && L > 0) {
                const uint32_t f = cur.first[i];
                const uint32_t sc = seg_index(j, L - 1);
                const uint32_t cb = lay.base[sc] - seg.wstart[sc];
                for (uint32_t r = 0; r < k; ++r) dst[1 + r] = cb + child.woff[child.uid[f + r]];
            }
        }
    }
}


// The top level of a batch: the roots of the jobs whose root lies there.
__global__ void k_init_top(LevelDev top, uint32_t* counts, int L, const Injected* __restrict__ inj, uint32_t ninj) {
    chain_enter();
    for (uint32_t r = threadIdx.x; r < ninj; r += blockDim.x) {
        top.coord[r] = inj[r].coord;
        top.job[r] = inj[r].job;
    }
    if (threadIdx.x == 0) counts[L] = ninj;
}

// Emission of every level in one launch: global kept-node index g maps to
// level L through the per-level prefix `ustart` (levels bottom..top).
struct EmitLevels {
    uint32_t ustart[CPVS_MAX_LEVELS + 1];
};

__global__ void __launch_bounds__(kThreads)
    k_emit_all(const LevelDev* __restrict__ lvt, EmitLevels el, int bottom, int top, bool leafmasks, SegDev seg,
               JobLayout lay, uint32_t njobs, uint32_t* __restrict__ out, uint64_t total_words, uint32_t* err) {
    const uint32_t U = el.ustart[top + 1];
    for (uint32_t g = blockIdx.x * blockDim.x + threadIdx.x; g < U; g += gridDim.x * blockDim.x) {
        int L = bottom;
        while (L < top && g >= el.ustart[L + 1]) ++L;
        const uint32_t u = g - el.ustart[L];
        const LevelDev& cur = lvt[L];
        const bool leaf = leafmasks && L == 2;
        const uint32_t i = cur.uniq[u];
        const uint32_t j = cur.job[i];
        if (j >= njobs) {
            atomicOr(err, 128u);  // a node's job out of range: reported, not followed
            continue;
        }
        const uint32_t sj = seg_index(j, L);
        const uint32_t m = cur.mask[i];
        const uint64_t at = lay.job_off[j] + lay.base[sj] + (cur.woff[u] - seg.wstart[sj]);
        if (at + node_words(m, leaf) > total_words) {
            atomicOr(err, 2u);
            continue;
        }
        uint32_t* dst = out + at;
        dst[0] = m;
        if (leaf) {
            // the class's eight slices (leaf masks are stored per class id,
            // which is the leaf's slot) as four 16-byte loads, all issued first
            const ulonglong2* sp = reinterpret_cast<const ulonglong2*>(cur.slices + (size_t)cur.slot[i] * 8);
            uint64_t v[8];
#pragma unroll
            for (int q = 0; q < 4; ++q) {
                const ulonglong2 t = sp[q];
                v[2 * q] = t.x;
                v[2 * q + 1] = t.y;
            }
            uint32_t r = 0;
#pragma unroll
            for (uint32_t q = 0; q < 8; ++q)
                if (((m >> (2u * q)) & 3u) == kPartial) {
                    dst[1 + 2 * r] = (uint32_t)v[q];
                    dst[2 + 2 * r] = (uint32_t)(v[q] >> 32);
                    ++r;
                }
        } else {
            const uint32_t k = partial_children(m);
            if (k && L > 0) {
                const LevelDev& child = lvt[L - 1];
                const uint32_t f = cur.first[i];
                const uint32_t sc = seg_index(j, L - 1);
                const uint32_t cb = lay.base[sc] - seg.wstart[sc];
                // the children's slots, ranks and offsets, each as independent loads
                uint32_t x[8];
#pragma unroll
                for (uint32_t r = 0; r < 8; ++r) x[r] = r < k ? child.slot[f + r] : 0u;
#pragma unroll
                for (uint32_t r = 0; r < 8; ++r) x[r] = r < k ? (uint32_t)(__ldcg(child.table + x[r]) >> 32) : 0u;
                const uint32_t kept_below = el.ustart[L] - el.ustart[L - 1];  // ranks of the level below
#pragma unroll
                for (uint32_t r = 0; r < 8; ++r) {
                    if (r >= k) break;
                    if (x[r] >= kept_below) {
                        atomicOr(err, 256u);  // a child without a rank: reported, not followed
                        break;
                    }
                    dst[1 + r] = cb + child.woff[x[r]];
                }
            }
        }
    }
}

// --------------------------------------------------------------- host side
inline uint64_t next_pow2(uint64_t v) {
    uint64_t p = 1;
    while (p < v) p <<= 1;
    return p;
}
inline size_t align256(size_t b) { return (b + 255) & ~(size_t)255; }

// A bump allocator over one device block.
struct Arena {
    char* base = nullptr;
    size_t size = 0, used = 0;
    template <class T>
    T* take(size_t count) {
        const size_t b = align256(count * sizeof(T));
        T* p = reinterpret_cast<T*>(base + used);
        used += b;
        return p;
    }
};

// Host-visible results of one build, copied in one piece at its end.
struct ResultView {
    uint64_t* job_off;  // njobs + 1
    uint32_t* seg;      // 6 * segn: nstart, nend, ustart, uend, wstart, wend
    uint32_t* level_u;  // 2 * L_MAX
    uint32_t* err;      // 1
    uint32_t* root_mask;  // njobs
};

inline size_t result_bytes(uint32_t njobs) {
    const size_t segn = (size_t)njobs * CPVS_MAX_LEVELS;
    return align256(8 * (njobs + 1)) + align256(4 * 6 * segn) + align256(4 * 2 * CPVS_MAX_LEVELS) + align256(4) +
           align256(4 * (size_t)njobs);
}

inline ResultView result_view(char* base, uint32_t njobs) {
    const size_t segn = (size_t)njobs * CPVS_MAX_LEVELS;
    ResultView v;
    size_t o = 0;
    v.job_off = reinterpret_cast<uint64_t*>(base + o); o += align256(8 * (njobs + 1));
    v.seg = reinterpret_cast<uint32_t*>(base + o); o += align256(4 * 6 * segn);
    v.level_u = reinterpret_cast<uint32_t*>(base + o); o += align256(4 * 2 * CPVS_MAX_LEVELS);
    v.err = reinterpret_cast<uint32_t*>(base + o); o += align256(4);
    v.root_mask = reinterpret_cast<uint32_t*>(base + o);
    return v;
}

// Inputs staged per build, one contiguous block in pinned host memory and
// one on the device (one copy): job table, roots, and for leafmask plans the
// leaf column groups, the z-tile table and the column pass's counts.
struct StageLayout {
    size_t jobs, inj, groups, ztiles, meta, bytes;
};
inline StageLayout stage_layout(uint32_t njobs) {
    auto a16 = [](size_t b) { return (b + 15) & ~(size_t)15; };
    StageLayout L{};
    size_t o = 0;
    L.jobs = o; o += a16(njobs * sizeof(JobDev));
    L.inj = o; o += a16(njobs * sizeof(Injected));
    L.groups = o; o += a16(njobs * sizeof(LeafGroupDev));
    L.ztiles = o; o += a16(njobs * sizeof(uint2));
    L.meta = o; o += 32;
    L.bytes = o;
    return L;
}

}  // namespace

// A build plan: capacities, scratch and the captured launch sequence for
// one shape of batch (leafmask mode + the map side of every job).  Reused as
// long as the data fit its capacities; otherwise rebuilt larger.
struct BuildPlan {
    bool leafmasks = false;
    bool pow2 = false;  // every job's level-0 height (map side x z tiles) is a power of two
    int bottom = 0, maxR = 0;
    uint32_t njobs = 0;
    std::vector<uint32_t> job_n, root_level;
    uint64_t cap[CPVS_MAX_LEVELS] = {0}, tcap[CPVS_MAX_LEVELS] = {0}, ninj[CPVS_MAX_LEVELS] = {0};
    uint64_t inj_off[CPVS_MAX_LEVELS + 1] = {0};
    uint32_t max_grid = 0;
    uint32_t insert_grid = 0;  // one wave of the inner insert kernel
    // launch shapes (tuned on the plan's first build, or fixed by the
    // context's options): the largest level the cluster kernels take, and
    // the inner insert's grid in resident waves
    uint32_t cluster_cap = kClusterLevelCap;
    uint32_t insert_waves = 1;
    bool shapes_set = false;
    // device memory
    char* arena = nullptr;
    size_t arena_bytes = 0;
    unsigned long long* table = nullptr;
    uint64_t table_slots = 0;
    LevelDev lv[CPVS_MAX_LEVELS];
    LevelDev* lvt = nullptr;
    uint2* partials = nullptr;
    uint32_t* counts = nullptr;
    uint32_t* segbuf = nullptr;  // 7 * segn: the six SegDev arrays + JobLayout::base
    SegDev seg{};
    JobLayout lay{};
    char* res = nullptr;  // device results region (ResultView layout)
    ResultView resv{};
    uint32_t* root_dev = nullptr;
    char* stage_dev = nullptr;  // StageLayout: the per-build inputs on the device
    JobDev* jobs_dev = nullptr;
    Injected* inj_dev = nullptr;
    // leaf column pass (leafmask plans): groups and z-tiles (staged), the
    // run entries (cap[2]) and per-column records (grown to the batch's
    // columns), its counts, the class hash table (the leaf level's table
    // region; the level's own `table` is the class records)
    LeafGroupDev* groups_dev = nullptr;
    uint2* ztiles_dev = nullptr;
    uint32_t* lmeta = nullptr;  // [0] groups, [1] columns, [2] run entries reserved, [3] pending runs,
                                // [4] queued columns
    uint2* pending = nullptr;  // non-uniform runs (cap[2])
    uint4* runs = nullptr;
    uint4* colrec = nullptr;  // two per column (colrec_cap), followed by the queue of columns
    uint4* heavy = nullptr;   // that need their texels (colrec_cap)
    uint64_t colrec_cap = 0;
    unsigned long long* ltable = nullptr;
    uint64_t ltable_mask = 0;
    // pinned host staging
    char* hin = nullptr;
    size_t hin_bytes = 0;
    char* hout = nullptr;
    size_t hout_bytes = 0;
    std::vector<char> staged;  // the inputs last copied to stage_dev (empty: none)
    cudaGraphExec_t exec = nullptr;
    cudaEvent_t done = nullptr;  // recorded after the emission that last read the scratch
    // fork / join of the ranking passes' stream in the captured launch sequence
    cudaEvent_t fork[CPVS_MAX_LEVELS] = {nullptr}, join = nullptr, start = nullptr, tables = nullptr;
    bool tables_tuned = false;
    // single-pass levels: the levels >= small_lo run in the single-block
    // kernels; look-back tickets and flags (zeroed by every build)
    int small_lo = CPVS_MAX_LEVELS;
    int cluster_blocks = 0;  // blocks of the small-level cluster kernels (0: none)
    unsigned int* tickets = nullptr;     // [2 * L_MAX + 1]
    unsigned long long* flags = nullptr;
    uint64_t flags_count = 0;
    uint64_t exp_flag_off[CPVS_MAX_LEVELS] = {0}, scan_flag_off[CPVS_MAX_LEVELS] = {0};
    uint64_t scan_tiles_cap[CPVS_MAX_LEVELS] = {0};
};

struct PlanCache {
    std::vector<BuildPlan*> plans;
};

namespace {

void plan_release(Ctx& ctx, BuildPlan* P) {
    if (P->done) cudaEventSynchronize(P->done);
    if (P->exec) cudaGraphExecDestroy(P->exec);
    P->exec = nullptr;
    for (cudaEvent_t& e : P->fork)
        if (e) cudaEventDestroy(e), e = nullptr;
    for (cudaEvent_t* e : {&P->join, &P->start, &P->tables})
        if (*e) cudaEventDestroy(*e), *e = nullptr;
    if (P->arena) ctx.release(P->arena, P->arena_bytes, true, nullptr);
    if (P->colrec) ctx.release(P->colrec, P->colrec_cap * 3 * sizeof(uint4), true, nullptr);
    P->colrec = nullptr;
    P->heavy = nullptr;
    P->colrec_cap = 0;
    if (P->table) ctx.release(P->table, P->table_slots * 8, true, nullptr);
    P->arena = nullptr;
    P->table = nullptr;
    if (P->hin) cudaFreeHost(P->hin);
    if (P->hout) cudaFreeHost(P->hout);
    P->hin = P->hout = nullptr;
    P->staged.clear();
}

// Per-level table regions (consecutive, tcap[L] slots each) and the split
// between the multi-block levels and the topmost ones that run in the
// cluster kernels (a level is small when it and every level above it hold
// at most kClusterItems * 1024 nodes per cluster block).
void plan_bind_tables(BuildPlan* P) {
    // a level of more nodes runs faster as its own launches over every SM
    const uint64_t small_cap =
        std::min<uint64_t>((uint64_t)P->cluster_blocks * kClusterThreads * kClusterItems, P->cluster_cap);
    uint64_t off = 0;
    for (int L = P->bottom; L <= P->maxR; ++L) {
        P->lv[L].table = P->table + off;
        P->lv[L].table_mask = P->tcap[L] - 1;
        off += P->tcap[L];
    }
    if (P->leafmasks) {
        // the leaf classes' hash table is the level's table region; the
        // level's `table` (read by the ranking and the emission) is the
        // per-class record array
        P->ltable = P->lv[2].table;
        P->ltable_mask = P->lv[2].table_mask;
        P->lv[2].table = reinterpret_cast<unsigned long long*>(P->lv[2].hash);
        P->lv[2].table_mask = 0;
    }
    P->small_lo = P->maxR + 1;
    while (P->small_lo > P->bottom && P->cap[P->small_lo - 1] <= small_cap) --P->small_lo;
}

uint64_t plan_table_slots(const BuildPlan* P) {
    uint64_t t = 0;
    for (int L = P->bottom; L <= P->maxR; ++L) t += P->tcap[L];
    return t;
}

// Capacities -> scratch layout, pinned staging, level table.
cpvs_status plan_allocate(Ctx& ctx, BuildPlan* P, cudaStream_t st) {
    const uint32_t njobs = P->njobs;
    const size_t segn = (size_t)njobs * CPVS_MAX_LEVELS;
    size_t bytes = 0;
    auto add = [&](size_t count, size_t elem) { bytes += align256(count * elem); };
    for (int L = P->bottom; L <= P->maxR; ++L) {
        const uint64_t c = std::max<uint64_t>(P->cap[L], 1);
        for (int a = 0; a < 7; ++a) add(c, a == 0 ? 8 : 4);  // coord, job, mask, first, slot, uniq, woff
        if (P->leafmasks && L == 2) {
            const uint64_t cls = c + 9ull * njobs;  // run entries + the uniform classes
            add(cls * 8, 8);  // class slice masks
            add(cls, 8);      // class records
            add(cls, 4);      // class jobs
            add(c, 16);       // run entries
            add(c, 8);        // pending run list
        }
    }
    add(CPVS_MAX_LEVELS, sizeof(LevelDev));
    add(P->max_grid, sizeof(uint2));
    add(CPVS_MAX_LEVELS, 4);
    add(segn * 7, 4);
    bytes += result_bytes(njobs);
    add(njobs, 4);
    add(stage_layout(njobs).bytes, 1);
    // look-back flags: per level, expansion tiles and 2 x merge tiles
    P->flags_count = 0;
    for (int L = P->bottom; L <= P->maxR; ++L) {
        const uint64_t c = std::max<uint64_t>(P->cap[L], 1);
        P->exp_flag_off[L] = P->flags_count;
        P->flags_count += (c + kExpTile - 1) / kExpTile + 1;
        P->scan_tiles_cap[L] = (c + kScanTile - 1) / kScanTile + 1;
        P->scan_flag_off[L] = P->flags_count;
        P->flags_count += P->scan_tiles_cap[L];
    }
    add(2 * CPVS_MAX_LEVELS + 1, 4);
    add(P->flags_count, 8);
    P->arena_bytes = bytes;
    cpvs_status r = ctx.alloc((void**)&P->arena, bytes, true, st);
    if (r != CPVS_OK) return r;
    // one region of per-level hash tables (sized for the untuned tables;
    // tuning only shrinks them)
    P->table_slots = 0;
    for (int L = P->bottom; L <= P->maxR; ++L) P->table_slots += P->tcap[L];
    r = ctx.alloc((void**)&P->table, P->table_slots * 8, true, st);
    if (r != CPVS_OK) return r;
    Arena A;
    A.base = P->arena;
    A.size = bytes;
    std::memset(P->lv, 0, sizeof(P->lv));
    for (int L = P->bottom; L <= P->maxR; ++L) {
        const uint64_t c = std::max<uint64_t>(P->cap[L], 1);
        LevelDev& l = P->lv[L];
        l.coord = A.take<uint64_t>(c);
        l.job = A.take<uint32_t>(c);
        l.mask = A.take<uint32_t>(c);
        l.first = A.take<uint32_t>(c);
        l.slot = A.take<uint32_t>(c);
        l.uniq = A.take<uint32_t>(c);
        l.woff = A.take<uint32_t>(c);
        if (P->leafmasks && L == 2) {
            // leaf level: per class id (a run entry index) its masks, job
            // (in `uid`) and record (in `hash`); the run entries
            const uint64_t cls = c + 9ull * njobs;
            l.slices = A.take<uint64_t>(cls * 8);
            l.hash = A.take<uint64_t>(cls);
            l.uid = A.take<uint32_t>(cls);
            P->runs = A.take<uint4>(c);
            P->pending = A.take<uint2>(c);
        }
    }
    P->lvt = A.take<LevelDev>(CPVS_MAX_LEVELS);
    P->partials = A.take<uint2>(P->max_grid);
    P->counts = A.take<uint32_t>(CPVS_MAX_LEVELS);
    P->segbuf = A.take<uint32_t>(segn * 7);
    P->res = A.base + A.used;
    A.used += result_bytes(njobs);
    P->resv = result_view(P->res, njobs);
    P->root_dev = A.take<uint32_t>(njobs);
    const StageLayout SL = stage_layout(njobs);
    P->stage_dev = A.take<char>(SL.bytes);
    P->jobs_dev = reinterpret_cast<JobDev*>(P->stage_dev + SL.jobs);
    P->inj_dev = reinterpret_cast<Injected*>(P->stage_dev + SL.inj);
    P->groups_dev = reinterpret_cast<LeafGroupDev*>(P->stage_dev + SL.groups);
    P->ztiles_dev = reinterpret_cast<uint2*>(P->stage_dev + SL.ztiles);
    P->lmeta = reinterpret_cast<uint32_t*>(P->stage_dev + SL.meta);
    P->tickets = A.take<unsigned int>(2 * CPVS_MAX_LEVELS + 1);  // + the expansion's first cluster level
    P->flags = A.take<unsigned long long>(P->flags_count);
    plan_bind_tables(P);
    // the device results region carries SegDev's arrays, so the six segment
    // arrays live there (copied to the host with the rest) and segbuf keeps
    // only JobLayout::base
    uint32_t* sg = P->resv.seg;
    P->seg = SegDev{sg, sg + segn, sg + 2 * segn, sg + 3 * segn, sg + 4 * segn, sg + 5 * segn};
    P->lay = JobLayout{P->resv.job_off, P->segbuf + 6 * segn};
    // pinned staging
    P->hin_bytes = SL.bytes;
    P->hout_bytes = result_bytes(njobs);
    CPVS_CUDA(cudaMallocHost((void**)&P->hin, P->hin_bytes));
    CPVS_CUDA(cudaMallocHost((void**)&P->hout, P->hout_bytes));
    // constant per plan: level table, root levels, bound segments
    CPVS_CUDA(cudaMemcpyAsync(P->lvt, P->lv, sizeof(P->lv), cudaMemcpyHostToDevice, st));
    CPVS_CUDA(cudaMemcpyAsync(P->root_dev, P->root_level.data(), njobs * 4, cudaMemcpyHostToDevice, st));
    CPVS_CUDA(cudaStreamSynchronize(st));
    return CPVS_OK;
}

uint32_t plan_grid(const BuildPlan* P, uint64_t items, uint64_t per_block) {
    uint64_t g = (items + per_block - 1) / per_block;
    return (uint32_t)std::max<uint64_t>(1, std::min<uint64_t>(g, P->max_grid));
}

// Blocks of `kernel` (kThreads each) resident on the whole GPU at once: the
// grid of a grid-stride kernel, so that all of it runs in one wave.
template <typename K>
uint32_t resident_blocks(K kernel, int num_sms) {
    int per_sm = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kernel, kThreads, 0) != cudaSuccess || per_sm < 1) {
        cudaGetLastError();
        per_sm = 1;
    }
    return (uint32_t)(per_sm * std::max(num_sms, 1));
}

// The largest cluster (16, else 8 blocks of 1024 threads) that both
// small-level kernels can have resident on this device; 0 if none.
int probe_cluster_blocks() {
    cudaFuncSetAttribute(k_expand_cluster, cudaFuncAttributeNonPortableClusterSizeAllowed, 1);
    cudaFuncSetAttribute(k_merge_cluster, cudaFuncAttributeNonPortableClusterSizeAllowed, 1);
    if (cudaFuncSetAttribute(k_expand_cluster, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kExpandClusterSmem) !=
            cudaSuccess ||
        cudaFuncSetAttribute(k_merge_cluster, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kMergeClusterSmem) !=
            cudaSuccess) {
        cudaGetLastError();
        return 0;
    }
    cudaGetLastError();
    for (int nb : {16, 8}) {
        cudaLaunchConfig_t cfg{};
        cfg.gridDim = dim3(nb);
        cfg.blockDim = dim3(kClusterThreads);
        cudaLaunchAttribute at[1];
        at[0].id = cudaLaunchAttributeClusterDimension;
        at[0].val.clusterDim.x = nb;
        at[0].val.clusterDim.y = 1;
        at[0].val.clusterDim.z = 1;
        cfg.attrs = at;
        cfg.numAttrs = 1;
        int a = 0, b = 0;
        cfg.dynamicSmemBytes = kExpandClusterSmem;
        bool ok = cudaOccupancyMaxActiveClusters(&a, k_expand_cluster, &cfg) == cudaSuccess && a > 0;
        cfg.dynamicSmemBytes = kMergeClusterSmem;
        ok = ok && cudaOccupancyMaxActiveClusters(&b, k_merge_cluster, &cfg) == cudaSuccess && b > 0;
        cudaGetLastError();
        if (ok) return nb;
    }
    return 0;
}

// The column pass's view of a leafmask plan (all null otherwise).
LeafColumns plan_leaf_columns(const BuildPlan* P) {
    LeafColumns lc{};
    if (!P->leafmasks) return lc;
    const LevelDev& l = P->lv[2];
    lc.groups = P->groups_dev;
    lc.ztiles = P->ztiles_dev;
    lc.meta = P->lmeta;
    lc.colrec = P->colrec;
    lc.runs = P->runs;
    lc.run_cap = (uint32_t)std::max<uint64_t>(P->cap[2], 1);
    lc.run_ctr = P->lmeta + 2;
    lc.cls_slices = l.slices;
    lc.cls_job = l.uid;
    lc.crec = l.table;
    lc.table = P->ltable;
    lc.table_mask = P->ltable_mask;
    lc.njobs = P->njobs;
    lc.pending = P->pending;
    lc.pending_ctr = P->lmeta + 3;
    lc.heavy = P->heavy;
    lc.heavy_ctr = P->lmeta + 4;
    return lc;
}

// The whole device-side build after the inputs are staged: top-down
// expansion, leaves, bottom-up merge, layout, root masks, and the copy of
// the results region to pinned host memory.  Stream-ordered; capturable.
// With a second stream `rank_st` (capture only), each level's ranking pass
// runs there, beside the inserts of the levels above it, which need only the
// level's class slots; the layout waits for both streams.
cpvs_status plan_enqueue(BuildPlan* P, cudaStream_t st, cudaStream_t rank_st, Timing* tm) {
    const uint32_t njobs = P->njobs;
    const size_t segn = (size_t)njobs * CPVS_MAX_LEVELS;
    const ResultView& rv = P->resv;
    uint32_t* err = rv.err;
    const bool forked = rank_st && rank_st != st;
    if (!forked) rank_st = st;
    const bool ch = forked;  // chained launches on the captured path
    auto event = [](cudaEvent_t& e) -> cudaError_t {
        return e ? cudaSuccess : cudaEventCreateWithFlags(&e, cudaEventDisableTiming);
    };
    if (forked) {
        CPVS_CUDA(event(P->start));
        CPVS_CUDA(event(P->tables));
        CPVS_CUDA(cudaEventRecord(P->start, st));
        CPVS_CUDA(cudaStreamWaitEvent(rank_st, P->start, 0));
    }
    // every level's hash table, beside the expansion (needed from the
    // leaves on)
    {
        KernelTimer kt(tm, K_TABLE_CLEAR, rank_st);
        CPVS_CUDA(cudaMemsetAsync(P->table, 0xFF, plan_table_slots(P) * 8, rank_st));
    }
    // the leaf classes of every column, beside the expansion (they need
    // only the maps, their level-3 bounds and the cleared tables)
    const LeafColumns lc = plan_leaf_columns(P);
    if (P->leafmasks) {
        KernelTimer kt(tm, K_LEAF_COLUMNS, rank_st);
        CPVS_CUDA(cudaMemsetAsync(P->lmeta + 2, 0, 12, rank_st));
        // one block per chunk of columns (the column records are sized to
        // the batch's columns; a larger batch re-captures the sequence)
        const uint32_t cg = (uint32_t)std::max<uint64_t>(
            1, std::min<uint64_t>((P->colrec_cap + kColChunk - 1) / kColChunk, P->max_grid));
        if (P->pow2)
            k_leaf_columns<true><<<cg, kThreads, 0, rank_st>>>(lc, err);
        else
            k_leaf_columns<false><<<cg, kThreads, 0, rank_st>>>(lc, err);
        CPVS_CUDA(cudaGetLastError());
        const uint32_t hg = plan_grid(P, P->colrec_cap, kThreads);
        if (P->pow2)
            k_leaf_columns_heavy<true><<<hg, kThreads, 0, rank_st>>>(lc);
        else
            k_leaf_columns_heavy<false><<<hg, kThreads, 0, rank_st>>>(lc);
        CPVS_CUDA(cudaGetLastError());
    }
    if (P->leafmasks) {
        // the classes of the non-uniform runs (one thread each)
        KernelTimer kt(tm, K_LEAF_CLASSES, rank_st);
        k_leaf_classes<<<plan_grid(P, P->cap[2], kThreads), kThreads, 0, rank_st>>>(lc, err);
        CPVS_CUDA(cudaGetLastError());
    }
    if (forked) CPVS_CUDA(cudaEventRecord(P->tables, rank_st));
    // results, level counts, job bases, look-back tickets and flags (the
    // last two adjacent in the arena)
    {
        ClearRanges cr{};
        cr.p[0] = P->res;
        cr.n[0] = result_bytes(njobs);
        cr.p[1] = reinterpret_cast<char*>(P->counts);
        cr.n[1] = CPVS_MAX_LEVELS * 4;
        cr.p[2] = reinterpret_cast<char*>(P->segbuf + 6 * segn);
        cr.n[2] = segn * 4;
        cr.p[3] = reinterpret_cast<char*>(P->tickets);
        cr.n[3] = reinterpret_cast<const char*>(P->flags + P->flags_count) - reinterpret_cast<const char*>(P->tickets);
        uint64_t mx = 0;
        for (int k = 0; k < 4; ++k) mx = std::max<uint64_t>(mx, cr.n[k]);
        const uint32_t g = (uint32_t)std::min<uint64_t>((mx / 16 + kThreads - 1) / kThreads + 1, P->max_grid);
        CPVS_CUDA(launch_kernel(k_clear, g, kThreads, 0, st, false, 0, cr));
    }
    // top-down: the small top levels as one cluster (which also places the
    // roots), then one pass per level
    const int Ls = P->small_lo;
    const int exp_lo = std::max(Ls, P->bottom + 1);
    if (P->maxR >= exp_lo) {
        KernelTimer kt(tm, K_EXPAND_WRITE, st);
        SmallLevels sl{};
        for (int L = 0; L < CPVS_MAX_LEVELS; ++L) {
            sl.inj_off[L] = (uint32_t)P->inj_off[L];
            sl.ninj[L] = (uint32_t)P->ninj[L];
            sl.cap[L] = (uint32_t)P->cap[L];
        }
        CPVS_CUDA(launch_kernel(k_expand_cluster, (uint32_t)P->cluster_blocks, kClusterThreads, kExpandClusterSmem, st, ch,
                               (uint32_t)P->cluster_blocks, P->lvt, P->counts, P->jobs_dev, njobs, P->maxR, exp_lo,
                               P->inj_dev, sl, P->seg, P->tickets + 2 * CPVS_MAX_LEVELS, err));
    } else {
        // the top level holds only roots
        CPVS_CUDA(launch_kernel(k_init_top, 1, 256, 0, st, ch, 0, P->lv[P->maxR], P->counts, P->maxR,
                               P->inj_dev + P->inj_off[P->maxR], (uint32_t)P->ninj[P->maxR]));
    }
    // a leafmask build whose level 3 expands over every SM resolves its
    // leaves in that pass (after the leaf column passes); else k_leaf_resolve
    const bool fuse_leaves = P->leafmasks && std::min(exp_lo - 1, P->maxR) >= 3;
    for (int L = std::min(exp_lo - 1, P->maxR); L > P->bottom; --L) {
        const bool leaves = fuse_leaves && L == 3;
        if (leaves && forked) CPVS_CUDA(cudaStreamWaitEvent(st, P->tables, 0));
        KernelTimer kt(tm, K_EXPAND_WRITE, st);
        CPVS_CUDA(launch_kernel(leaves ? k_expand_lb<true> : k_expand_lb<false>, plan_grid(P, P->cap[L], kExpTile),
                               kThreads, 0, st, ch, 0, P->lv[L], P->lv[L - 1], P->counts, P->jobs_dev, njobs, L,
                               P->inj_dev + P->inj_off[L - 1], (uint32_t)P->ninj[L - 1], P->seg,
                               (uint32_t)P->cap[L - 1], P->tickets + L, P->flags + P->exp_flag_off[L], lc, err));
    }
    if (forked && !fuse_leaves) CPVS_CUDA(cudaStreamWaitEvent(st, P->tables, 0));
    if (fuse_leaves) {
        // resolved by the expansion
    } else if (P->leafmasks) {
        KernelTimer kt(tm, K_LEAF_RESOLVE, st);
        CPVS_CUDA(launch_kernel(k_leaf_resolve, plan_grid(P, P->cap[2], kThreads), kThreads, 0, st, ch, 0, P->lv[2],
                                P->counts, P->jobs_dev, njobs, P->seg, lc, err));
    } else {
        KernelTimer kt(tm, K_CLASSIFY_BOTTOM, st);
        CPVS_CUDA(launch_kernel(k_classify_bottom, plan_grid(P, P->cap[0], kThreads), kThreads, 0, st, ch, 0, P->lv[0],
                               P->counts, P->jobs_dev, njobs, 0, P->seg, err));
    }
    // bottom-up: per level an insert and the ranking pass (on rank_st), then
    // the small top levels in one cluster
    const int merge_hi = std::min(Ls - 1, P->maxR);
    for (int L = P->bottom; L <= merge_hi; ++L) {
        const bool leaf = P->leafmasks && L == 2;
        const LevelDev child = (L > P->bottom) ? P->lv[L - 1] : P->lv[L];
        if (!leaf) {
            KernelTimer kt(tm, K_INSERT_INNER, st);
            CPVS_CUDA(launch_kernel(k_dedup_insert<false>,
                                    std::min(plan_grid(P, P->cap[L], kThreads), P->insert_grid * P->insert_waves),
                                    kThreads, 0, st, ch, 0,
                                   P->lv[L], child, P->counts, L, P->lv[L].table, P->lv[L].table_mask, err));
        }
        if (forked) {
            CPVS_CUDA(event(P->fork[L]));
            CPVS_CUDA(cudaEventRecord(P->fork[L], st));
            CPVS_CUDA(cudaStreamWaitEvent(rank_st, P->fork[L], 0));
        }
        KernelTimer kt(tm, K_SCAN, rank_st);
        const uint32_t g = plan_grid(P, P->cap[L], kScanTile);
        unsigned long long* fl = P->flags + P->scan_flag_off[L];
        unsigned int* ticket = P->tickets + CPVS_MAX_LEVELS + L;
        if (leaf)
            k_merge_scan_lb<true><<<g, kThreads, 0, rank_st>>>(P->lv[L], P->counts, rv.level_u, L, P->seg, njobs, ticket,
                                                               fl, err);
        else
            k_merge_scan_lb<false><<<g, kThreads, 0, rank_st>>>(P->lv[L], P->counts, rv.level_u, L, P->seg, njobs, ticket,
                                                                fl, err);
        CPVS_CUDA(cudaGetLastError());
    }
    if (merge_hi < P->maxR) {
        KernelTimer kt(tm, K_SCAN, st);
        CPVS_CUDA(launch_kernel(k_merge_cluster, (uint32_t)P->cluster_blocks, kClusterThreads, kMergeClusterSmem, st, ch,
                               (uint32_t)P->cluster_blocks, P->lvt, P->counts, rv.level_u,
                               std::max(merge_hi + 1, P->bottom), P->maxR, P->bottom, P->leafmasks ? 2 : -1, P->seg,
                               err));
    }
    if (forked) {
        CPVS_CUDA(event(P->join));
        CPVS_CUDA(cudaEventRecord(P->join, rank_st));
        CPVS_CUDA(cudaStreamWaitEvent(st, P->join, 0));
    }
    {
        KernelTimer kt(tm, K_LAYOUT, st);
        CPVS_CUDA(launch_kernel(k_layout, 1, 1024, 0, st, ch, 0, P->seg, P->lay, P->root_dev, njobs, P->bottom,
                                static_cast<const LevelDev*>(P->lvt), rv.root_mask));
    }
    CPVS_CUDA(cudaMemcpyAsync(P->hout, P->res, result_bytes(njobs), cudaMemcpyDeviceToHost, st));
    return CPVS_OK;
}

// Captures the plan's launch sequence into P->exec.
cpvs_status plan_capture(Ctx& ctx, BuildPlan* P) {
    if (!ctx.capture_stream) CPVS_CUDA(cudaStreamCreateWithFlags(&ctx.capture_stream, cudaStreamNonBlocking));
    if (!ctx.capture_rank_stream) CPVS_CUDA(cudaStreamCreateWithFlags(&ctx.capture_rank_stream, cudaStreamNonBlocking));
    if (P->exec) {
        cudaGraphExecDestroy(P->exec);
        P->exec = nullptr;
    }
    cudaGraph_t graph = nullptr;
    CPVS_CUDA(cudaStreamBeginCapture(ctx.capture_stream, cudaStreamCaptureModeThreadLocal));
    cpvs_status r = plan_enqueue(P, ctx.capture_stream, ctx.capture_rank_stream, nullptr);
    cudaError_t ec = cudaStreamEndCapture(ctx.capture_stream, &graph);
    if (r != CPVS_OK) {
        if (graph) cudaGraphDestroy(graph);
        return r;
    }
    if (ec != cudaSuccess) return cuda_fail(ec, "cudaStreamEndCapture");
    ec = cudaGraphInstantiate(&P->exec, graph, 0);
    cudaGraphDestroy(graph);
    if (ec != cudaSuccess) return cuda_fail(ec, "cudaGraphInstantiate");
    return CPVS_OK;
}

// Launch shapes of a plan: (cluster cap, insert waves).
void plan_set_shapes(BuildPlan* P, uint32_t cap, uint32_t waves) {
    if (P->cluster_cap == cap && P->insert_waves == waves) return;
    P->cluster_cap = cap;
    P->insert_waves = waves;
    plan_bind_tables(P);  // the split between cluster and multi-block levels
    if (P->exec) {
        cudaGraphExecDestroy(P->exec);
        P->exec = nullptr;
    }
}

// The plan's autotuner: after the plan's first build (its inputs still
// staged, its hash tables sized), every (cluster cap, insert waves) pair is
// captured once, then the pairs' launch sequences are replayed in turn --
// one warm-up round and kTuneRounds CUDA-event-timed rounds on `st`, so that
// a clock ramp or a neighbour's load falls on every pair alike -- and the
// pair with the lowest replay time is kept with its graph.  A pair whose
// replay reports an internal check (a level or table overflow) is not taken.
// Runs after the current DAG build's emission in stream order; the replays only rewrite
// the plan's own scratch.
constexpr int kTuneRounds = 3;
constexpr int kTuneShapes = (int)(sizeof(kClusterCaps) / sizeof(kClusterCaps[0])) * 2;

cpvs_status plan_tune(Ctx& ctx, BuildPlan* P, cudaStream_t st, float& tuning_ms) {
    cudaEvent_t a = nullptr, b = nullptr, t0 = nullptr, t1 = nullptr;
    CPVS_CUDA(cudaEventCreate(&a));
    CPVS_CUDA(cudaEventCreate(&b));
    CPVS_CUDA(cudaEventCreate(&t0));
    CPVS_CUDA(cudaEventCreate(&t1));
    CPVS_CUDA(cudaEventRecord(t0, st));
    const uint32_t cap0 = P->cluster_cap, waves0 = P->insert_waves;
    cudaGraphExec_t exec[kTuneShapes] = {};
    uint32_t cap_of[kTuneShapes], waves_of[kTuneShapes];
    float t_min[kTuneShapes];
    bool clean[kTuneShapes];
    cpvs_status r = CPVS_OK;
    int ns = 0;
    for (uint32_t cap : kClusterCaps)
        for (uint32_t waves : {1u, 2u}) {
            if (r != CPVS_OK) break;
            plan_set_shapes(P, cap, waves);
            r = plan_capture(ctx, P);
            if (r != CPVS_OK) break;
            exec[ns] = P->exec;
            P->exec = nullptr;
            cap_of[ns] = cap;
            waves_of[ns] = waves;
            t_min[ns] = 1e30f;
            clean[ns] = true;
            ++ns;
        }
    for (int round = 0; round <= kTuneRounds && r == CPVS_OK; ++round)
        for (int i = 0; i < ns && r == CPVS_OK; ++i) {
            if (!clean[i]) continue;
            cudaEventRecord(a, st);
            cudaGraphLaunch(exec[i], st);
            cudaEventRecord(b, st);
            if (cudaEventSynchronize(b) != cudaSuccess) {
                r = cuda_fail(cudaGetLastError(), "build tuning");
                break;
            }
            clean[i] = *result_view(P->hout, P->njobs).err == 0;
            float t = 0.f;
            cudaEventElapsedTime(&t, a, b);
            if (round > 0 && t < t_min[i]) t_min[i] = t;  // round 0 warms the caches
        }
    int best = -1;
    if (r == CPVS_OK)
        for (int i = 0; i < ns; ++i)
            if (clean[i] && (best < 0 || t_min[i] < t_min[best])) best = i;
    // the plan keeps the winner's graph; with none (an error, or every pair
    // overflowing) it returns to its shapes before tuning and recaptures on
    // its next build
    plan_set_shapes(P, best >= 0 ? cap_of[best] : cap0, best >= 0 ? waves_of[best] : waves0);
    if (P->exec) cudaGraphExecDestroy(P->exec);
    P->exec = nullptr;
    for (int i = 0; i < ns; ++i) {
        if (i == best) P->exec = exec[i];
        else cudaGraphExecDestroy(exec[i]);
    }
    cudaEventRecord(t1, st);
    cudaEventSynchronize(t1);
    cudaEventElapsedTime(&tuning_ms, t0, t1);
    for (cudaEvent_t e : {a, b, t0, t1}) cudaEventDestroy(e);
    if (P->done) cudaEventRecord(P->done, st);  // the next build waits for the replays too
    return r;
}

bool same_shape(const BuildPlan* P, bool leafmasks, bool pow2, const std::vector<uint32_t>& job_n) {
    return P->leafmasks == leafmasks && P->pow2 == pow2 && P->job_n == job_n;
}

// Capacities from per-job level bounds (+25% slack) and table sizes.  A
// plan only grows: re-planning keeps every level at least as large as before,
// so batches of different maps settle on one plan.
void plan_set_capacities(BuildPlan* P, const std::vector<unsigned long long>& bounds, bool exact_tables) {
    uint64_t cap[CPVS_MAX_LEVELS] = {0};
    for (uint32_t j = 0; j < P->njobs; ++j)
        for (int L = P->bottom; L < (int)P->root_level[j]; ++L) cap[L] += bounds[(size_t)j * CPVS_MAX_LEVELS + L];
    for (int L = 0; L < CPVS_MAX_LEVELS; ++L) {
        if (cap[L]) cap[L] = cap[L] + cap[L] / 4 + 256;
        cap[L] += P->ninj[L];
        P->cap[L] = std::max(P->cap[L], cap[L]);
        if (exact_tables || !P->tcap[L] || P->tcap[L] < 1024) P->tcap[L] = next_pow2(std::max<uint64_t>(2 * P->cap[L], 1024));
    }
}

cpvs_status plan_create(Ctx& ctx, const std::vector<JobSpec>& jobs, const std::vector<SourceSpec>& sources,
                        bool leafmasks, const std::vector<uint32_t>& job_n,
                        const std::vector<unsigned long long>& bounds, cudaStream_t st, BuildPlan** out) {
    auto* P = new BuildPlan;
    P->leafmasks = leafmasks;
    P->bottom = leafmasks ? 2 : 0;
    P->njobs = (uint32_t)jobs.size();
    P->job_n = job_n;
    P->root_level.resize(P->njobs);
    P->max_grid = (uint32_t)std::max(ctx.num_sms, 1) * 8;
    P->insert_grid = std::min(P->max_grid, resident_blocks(k_dedup_insert<false>, ctx.num_sms));
    if (ctx.cluster_blocks < 0) ctx.cluster_blocks = probe_cluster_blocks();
    P->cluster_blocks = ctx.cluster_blocks;
    for (uint32_t j = 0; j < P->njobs; ++j) {
        P->root_level[j] = (uint32_t)(log2_u32(job_n[j]) - 1);
        P->maxR = std::max(P->maxR, (int)P->root_level[j]);
        P->ninj[P->root_level[j]] += 1;
    }
    uint64_t o = 0;
    for (int L = 0; L < CPVS_MAX_LEVELS; ++L) {
        P->inj_off[L] = o;
        o += P->ninj[L];
    }
    P->inj_off[CPVS_MAX_LEVELS] = o;
    plan_set_capacities(P, bounds, true);
    for (int L = 0; L < CPVS_MAX_LEVELS; ++L)
        if (P->cap[L] >= (1ull << 31)) {
            delete P;
            return fail(CPVS_ERR_BUDGET, "build: a level exceeds 2^31 nodes");
        }
    cpvs_status r = plan_allocate(ctx, P, st);
    if (r != CPVS_OK) {
        plan_release(ctx, P);
        delete P;
        return r;
    }
    *out = P;
    return CPVS_OK;
}

// Level bounds of a batch straight from its pyramids (one sync).
cpvs_status prepass_bounds(Ctx& ctx, const std::vector<SourceSpec>& sources, const std::vector<JobSpec>& jobs,
                           int lmin, cudaStream_t st, std::vector<unsigned long long>& bounds) {
    const uint32_t njobs = (uint32_t)jobs.size();
    const size_t bounds_bytes = (size_t)njobs * CPVS_MAX_LEVELS * sizeof(unsigned long long);
    unsigned long long* bounds_dev = nullptr;
    BoundJob* bj_dev = nullptr;
    cpvs_status r = ctx.alloc((void**)&bounds_dev, bounds_bytes, false, st);
    if (r != CPVS_OK) return r;
    r = ctx.alloc((void**)&bj_dev, njobs * sizeof(BoundJob), false, st);
    if (r != CPVS_OK) {
        ctx.release(bounds_dev, bounds_bytes, false, st);
        return r;
    }
    std::vector<std::vector<uint32_t>> by_src(sources.size());
    for (uint32_t j = 0; j < njobs; ++j) by_src[jobs[j].source].push_back(j);
    std::vector<BoundJob> grouped;
    std::vector<std::pair<size_t, size_t>> ranges(sources.size());
    for (size_t s = 0; s < sources.size(); ++s) {
        ranges[s] = {grouped.size(), by_src[s].size()};
        for (uint32_t j : by_src[s]) grouped.push_back(BoundJob{jobs[j].z_idx, jobs[j].z_num, j});
    }
    cudaError_t e = cudaMemsetAsync(bounds_dev, 0, bounds_bytes, st);
    if (e == cudaSuccess)
        e = cudaMemcpyAsync(bj_dev, grouped.data(), njobs * sizeof(BoundJob), cudaMemcpyHostToDevice, st);
    for (size_t s = 0; s < sources.size() && e == cudaSuccess && r == CPVS_OK; ++s) {
        if (!ranges[s].second) continue;
        KernelTimer kt(&ctx.timing, K_LEVEL_BOUNDS, st);
        r = launch_level_bounds(sources[s].levels, sources[s].n, lmin, bj_dev + ranges[s].first,
                                (int)ranges[s].second, bounds_dev, st);
    }
    bounds.assign((size_t)njobs * CPVS_MAX_LEVELS, 0);
    if (e == cudaSuccess && r == CPVS_OK)
        e = cudaMemcpyAsync(bounds.data(), bounds_dev, bounds_bytes, cudaMemcpyDeviceToHost, st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    ctx.release(bounds_dev, bounds_bytes, false, st);
    ctx.release(bj_dev, njobs * sizeof(BoundJob), false, st);
    if (e != cudaSuccess) return cuda_fail(e, "build bounds pre-pass");
    return r;
}

}  // namespace

void destroy_plans(Ctx& ctx) {
    if (!ctx.plans) return;
    for (BuildPlan* P : ctx.plans->plans) {
        plan_release(ctx, P);
        if (P->done) cudaEventDestroy(P->done);
        delete P;
    }
    delete ctx.plans;
    ctx.plans = nullptr;
}

cpvs_status build_dags(Ctx& ctx, const std::vector<SourceSpec>& sources, const std::vector<JobSpec>& jobs,
                       bool leafmasks, cudaStream_t st, BuildOutput& out) {
    NvtxRange range("cpvs build");
    const uint32_t njobs = (uint32_t)jobs.size();
    if (njobs == 0) return fail(CPVS_ERR_INVALID_ARG, "build_dags: no jobs");
    std::vector<uint32_t> job_n(njobs);
    bool pow2 = true;  // the leaf pass may then skip the depth product (exact for these heights)
    for (uint32_t j = 0; j < njobs; ++j) {
        const SourceSpec& S = sources[jobs[j].source];
        const uint64_t h0 = (uint64_t)S.n * jobs[j].z_num;
        pow2 = pow2 && (h0 & (h0 - 1)) == 0;
        const int nl = log2_u32(S.n) + 1;
        // leafmasks need numLevels-3 >= 2 (src/CompressedShadow.cpp:20-27)
        if (leafmasks && nl - 3 < 2) return fail(CPVS_ERR_INVALID_ARG, "build_dags: map too small for leafmasks");
        job_n[j] = S.n;
    }
    if (!ctx.plans) ctx.plans = new PlanCache;
    BuildPlan* P = nullptr;
    for (BuildPlan* q : ctx.plans->plans)
        if (same_shape(q, leafmasks, pow2, job_n)) P = q;
    if (!P) {
        NvtxRange plan_range("cpvs build: new plan");
        std::vector<unsigned long long> bounds;
        cpvs_status r = prepass_bounds(ctx, sources, jobs, (leafmasks ? 2 : 0) + 1, st, bounds);
        if (r != CPVS_OK) return r;
        r = plan_create(ctx, jobs, sources, leafmasks, job_n, bounds, st, &P);
        if (r == CPVS_OK) P->pow2 = pow2;
        if (r != CPVS_OK) return r;
        // keep a few shapes; drop the oldest
        if (ctx.plans->plans.size() >= 8) {
            plan_release(ctx, ctx.plans->plans.front());
            if (ctx.plans->plans.front()->done) cudaEventDestroy(ctx.plans->plans.front()->done);
            delete ctx.plans->plans.front();
            ctx.plans->plans.erase(ctx.plans->plans.begin());
        }
        ctx.plans->plans.push_back(P);
    }

    if (!P->done) CPVS_CUDA(cudaEventCreateWithFlags(&P->done, cudaEventDisableTiming));
    // launch shapes fixed by the context's options take effect at once;
    // otherwise the plan's first graph build times the candidates (below)
    if (ctx.build_cluster_cap || ctx.build_insert_waves) {
        plan_set_shapes(P, ctx.build_cluster_cap ? (uint32_t)ctx.build_cluster_cap : kClusterLevelCap,
                        ctx.build_insert_waves ? (uint32_t)ctx.build_insert_waves : 1u);
        P->shapes_set = true;
    }
    uint32_t replans = 0;
    // the previous build with this plan may still be emitting from its
    // scratch on another stream
    CPVS_CUDA(cudaStreamWaitEvent(st, P->done, 0));
    // leaf column groups: the jobs that share a map and a z_num, with
    // distinct z-tiles (a repeated z-tile starts another group)
    std::vector<uint32_t> job_group(njobs, 0);
    std::vector<uint32_t> grp_source, grp_znum;
    std::vector<uint64_t> grp_colbase;
    std::vector<std::vector<uint2>> grp_tiles;  // (z_idx, job)
    uint64_t ncols = 0;
    if (leafmasks) {
        for (uint32_t j = 0; j < njobs; ++j) {
            uint32_t g = 0;
            for (; g < grp_source.size(); ++g) {
                if (grp_source[g] != jobs[j].source || grp_znum[g] != jobs[j].z_num) continue;
                bool taken = false;
                for (const uint2& t : grp_tiles[g]) taken = taken || t.x == jobs[j].z_idx;
                if (!taken) break;
            }
            if (g == grp_source.size()) {
                grp_source.push_back(jobs[j].source);
                grp_znum.push_back(jobs[j].z_num);
                grp_tiles.emplace_back();
                grp_colbase.push_back(ncols);
                const uint64_t c = sources[jobs[j].source].n / 8;
                ncols += c * c;
            }
            grp_tiles[g].push_back(make_uint2(jobs[j].z_idx, j));
            job_group[j] = g;
        }
        for (auto& t : grp_tiles) std::sort(t.begin(), t.end(), [](uint2 a, uint2 b) { return a.x < b.x; });
        if (ncols >= (1ull << 31)) return fail(CPVS_ERR_BUDGET, "build_dags: more than 2^31 leaf columns");
    }
    ResultView hv{};
    for (int attempt = 0;; ++attempt) {
        // column records for this batch's maps (kept; grown when a batch
        // has more columns: the launch sequence is captured anew)
        if (leafmasks && ncols > P->colrec_cap) {
            if (P->colrec) {
                CPVS_CUDA(cudaStreamSynchronize(st));
                ctx.release(P->colrec, P->colrec_cap * 3 * sizeof(uint4), true, nullptr);
                P->colrec = nullptr;
                P->heavy = nullptr;
                P->colrec_cap = 0;
            }
            cpvs_status r = ctx.alloc((void**)&P->colrec, ncols * 3 * sizeof(uint4), true, st);
            if (r != CPVS_OK) return r;
            P->heavy = P->colrec + 2 * ncols;
            P->colrec_cap = ncols;
            if (P->exec) {
                cudaGraphExecDestroy(P->exec);
                P->exec = nullptr;
            }
        }
        // stage this batch's inputs (StageLayout): job table (pyramid and
        // map pointers, z-tile, column group), roots in root-level order,
        // the column groups and their z-tiles
        const StageLayout SL = stage_layout(njobs);
        std::memset(P->hin, 0, SL.bytes);
        JobDev* hj = reinterpret_cast<JobDev*>(P->hin + SL.jobs);
        Injected* hi = reinterpret_cast<Injected*>(P->hin + SL.inj);
        std::vector<uint64_t> fill(CPVS_MAX_LEVELS, 0);
        for (uint32_t j = 0; j < njobs; ++j) {
            const SourceSpec& S = sources[jobs[j].source];
            hj[j] = JobDev{S.levels,         S.depth,       S.n, P->root_level[j] + 2, jobs[j].z_idx, jobs[j].z_num,
                           job_group[j],     0,             leafmasks ? grp_colbase[job_group[j]] : 0ull};
            const int R = (int)P->root_level[j];
            hi[P->inj_off[R] + fill[R]++] = Injected{pack_xyz(0, 0, 2 * jobs[j].z_idx), j, 0};
        }
        if (leafmasks) {
            LeafGroupDev* hg = reinterpret_cast<LeafGroupDev*>(P->hin + SL.groups);
            uint2* hz = reinterpret_cast<uint2*>(P->hin + SL.ztiles);
            uint32_t* hm = reinterpret_cast<uint32_t*>(P->hin + SL.meta);
            uint32_t zo = 0;
            uint64_t cb = 0;
            for (size_t g = 0; g < grp_source.size(); ++g) {
                const SourceSpec& S = sources[grp_source[g]];
                hg[g] = LeafGroupDev{S.levels + pyramid_level_offset(S.n, 3), S.depth, S.nan_flag, S.n, grp_znum[g],
                                     zo, (uint32_t)grp_tiles[g].size(), cb};
                for (const uint2& t : grp_tiles[g]) hz[zo++] = t;
                cb += (uint64_t)(S.n / 8) * (S.n / 8);
            }
            hm[0] = (uint32_t)grp_source.size();
            hm[1] = (uint32_t)ncols;
        }
        // the device copies are read-only to the build: repeated builds of the
        // same maps (same pyramid and map addresses) skip the copy
        if (P->staged.size() != SL.bytes || std::memcmp(P->staged.data(), P->hin, SL.bytes) != 0) {
            CPVS_CUDA(cudaMemcpyAsync(P->stage_dev, P->hin, SL.bytes, cudaMemcpyHostToDevice, st));
            P->staged.assign(P->hin, P->hin + SL.bytes);
        }
        NvtxRange pass_range("cpvs build: levels");
        if (ctx.timing.on) {
            cpvs_status r = plan_enqueue(P, st, nullptr, &ctx.timing);
            if (r != CPVS_OK) return r;
        } else {
            if (!P->exec) {
                cpvs_status r = plan_capture(ctx, P);
                if (r != CPVS_OK) return r;
            }
            CPVS_CUDA(cudaGraphLaunch(P->exec, st));
        }
        CPVS_CUDA(cudaStreamSynchronize(st));
        hv = result_view(P->hout, njobs);
        const uint32_t herr = *hv.err;
        if (herr == 0) break;
        // bit 1 (a level outgrew the plan) or 16 (a hash table did): re-plan
        // from these maps' level bounds and retry; the rejected stale slots
        // that an overflow leaves behind (bits 4, 8) go with it.  Anything
        // else is an internal fault, reported as a timeout when a bounded
        // wait on another CTA gave up (bit 32).
        const bool overflow = (herr & (1u | 16u)) != 0;
        if (!overflow || (herr & 2u) || attempt >= 2)
            return fail((herr & 32u) ? CPVS_ERR_TIMEOUT : CPVS_ERR_DEVICE,
                        "build_dags: internal check " + std::to_string(herr));
        ++replans;
        std::vector<unsigned long long> bounds;
        {
            cpvs_status r = prepass_bounds(ctx, sources, jobs, (leafmasks ? 2 : 0) + 1, st, bounds);
            if (r != CPVS_OK) return r;
        }
        plan_release(ctx, P);
        plan_set_capacities(P, bounds, true);
        cpvs_status r = plan_allocate(ctx, P, st);
        if (r != CPVS_OK) return r;
    }

    const size_t segn = (size_t)njobs * CPVS_MAX_LEVELS;
    const uint32_t* hseg = hv.seg;
    const uint64_t total = hv.job_off[njobs];
    out.leafmasks = leafmasks;
    out.dag_words = total;
    out.job_offset.assign(hv.job_off, hv.job_off + njobs);
    out.job_words.resize(njobs);
    out.root_mask.assign(hv.root_mask, hv.root_mask + njobs);
    out.tree_nodes.assign(njobs, std::vector<uint64_t>());
    out.unique_nodes.assign(njobs, std::vector<uint64_t>());
    uint64_t level_unique[CPVS_MAX_LEVELS] = {0};
    for (uint32_t j = 0; j < njobs; ++j) {
        out.job_words[j] = hv.job_off[j + 1] - hv.job_off[j];
        if (out.job_words[j] >= 0xFFFFFFFEull) return fail(CPVS_ERR_BUDGET, "build_dags: DAG exceeds 2^32-2 words");
        const int nl = (int)P->root_level[j] + 2;
        out.tree_nodes[j].assign(nl, 0);
        out.unique_nodes[j].assign(nl, 0);
        for (int L = P->bottom; L <= (int)P->root_level[j]; ++L) {
            const size_t s = (size_t)j * CPVS_MAX_LEVELS + L;
            out.tree_nodes[j][L] = hseg[1 * segn + s] - hseg[0 * segn + s];
            out.unique_nodes[j][L] = hseg[3 * segn + s] - hseg[2 * segn + s];
        }
    }
    EmitLevels el{};
    for (int L = P->bottom; L <= P->maxR; ++L) {
        level_unique[L] = hv.level_u[2 * L];
        el.ustart[L + 1] = el.ustart[L] + hv.level_u[2 * L];
    }
    {
        cpvs_status r = ctx.alloc((void**)&out.dag, (total + kDagPad) * 4, true, st);
        if (r != CPVS_OK) return r;
        CPVS_CUDA(cudaMemsetAsync(out.dag + total, 0, kDagPad * 4, st));
    }
    {
        NvtxRange emit_range("cpvs build: emission");
        KernelTimer kt(&ctx.timing, K_EMIT, st);
        const uint32_t U = el.ustart[P->maxR + 1];
        if (U)
            k_emit_all<<<plan_grid(P, U, kThreads), kThreads, 0, st>>>(P->lvt, el, P->bottom, P->maxR, P->leafmasks,
                                                                       P->seg, P->lay, njobs, out.dag, total,
                                                                       P->resv.err);
        CPVS_CUDA(cudaGetLastError());
        CPVS_CUDA(cudaEventRecord(P->done, st));
    }
    // size the hash tables to the unique counts seen (3x rounded up to a
    // power of two, load <= 1/3); a later build that needs more grows them back
    if (!P->tables_tuned) {
        bool changed = false;
        for (int L = P->bottom; L <= P->maxR; ++L) {
            const uint64_t t = next_pow2(std::max<uint64_t>(3 * level_unique[L], 1024));
            const uint64_t tc = std::min<uint64_t>(t, next_pow2(std::max<uint64_t>(2 * P->cap[L], 1024)));
            if (tc != P->tcap[L]) changed = true;
            P->tcap[L] = tc;
        }
        P->tables_tuned = true;
        if (changed) {
            if (P->exec) {
                cudaGraphExecDestroy(P->exec);
                P->exec = nullptr;
            }
            // after the current DAG build's emission (stream order), which reads the
            // level table
            plan_bind_tables(P);
            CPVS_CUDA(cudaMemcpyAsync(P->lvt, P->lv, sizeof(P->lv), cudaMemcpyHostToDevice, st));
        }
    }
    float tuning_ms = 0.f;
    bool tuned = false;
    if (!P->shapes_set && !ctx.timing.on && ctx.tune_builds) {
        NvtxRange tune_range("cpvs build: tuning");
        cpvs_status r = plan_tune(ctx, P, st, tuning_ms);
        if (r != CPVS_OK) return r;
        P->shapes_set = tuned = true;
    }
    ctx.last_build.error_word = 0;
    ctx.last_build.replans = replans;
    ctx.last_build.cluster_cap = P->cluster_cap;
    ctx.last_build.insert_waves = P->insert_waves;
    ctx.last_build.tuned = tuned ? 1u : 0u;
    ctx.last_build.tuning_ms = tuning_ms;
    return CPVS_OK;
}

}  // namespace cpvs

// ---------------------------------------------------------------------------
// Allocation-free build for small maps.
//
// Some callers may not allocate device memory at all: a render loop that must
// not stall on cudaMalloc / cudaFree (both can synchronise the device and take
// unpredictable time), or a plugin running inside a host application that
// owns and pre-reserves all GPU memory.  For them, cpvs_shadow_build_noalloc
// builds a DAG with every scratch buffer (pyramid, per-level node arrays,
// hash table) carved out of the fixed array below, which each GPU that loads
// this library keeps until the process exits.  The caller passes the depth
// map and the output buffer.
//
// It does not run build_dags' launch sequence.  It uses the multi-pass
// kernels, which need no look-back flags, tickets or per-plan tables:
// k_pyramid, k_expand_count + k_expand_write per level, k_leaf_masks (or
// k_classify_bottom without leafmasks), per level k_dedup_insert,
// k_dedup_resolve, k_dedup_scan and k_dedup_remap, then k_layout and k_emit
// per level.  It is those kernels' only user, so a change to the node
// layout, the error bits or the segment bookkeeping of the main path must be
// mirrored there; tests/test_zz_no_alloc.py compares the allocation-free build word for
// word with the allocating build and with the oracle.
// ---------------------------------------------------------------------------
namespace cpvs {
namespace {

constexpr size_t kNoAllocScratchBytes = size_t(8) << 20;  // 8 MiB per device
constexpr uint32_t kNoAllocMaxSide = 256;         // with leafmasks
constexpr uint32_t kNoAllocMaxSideNoLeaf = 64;    // without: the full octree down to level 0

static __device__ __align__(256) unsigned char g_noalloc_scratch[kNoAllocScratchBytes];

// Device address of g_noalloc_scratch on the current device (host code
// cannot use the symbol itself as a device pointer).  Looked up on every
// call, with the device current: the lookup allocates nothing once the
// module is loaded, and an address kept across calls would go stale if the
// application reset the device or tore down its primary context.
cpvs_status noalloc_scratch_address(void** out) {
    void* p = nullptr;
    const cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
    if (e != cudaSuccess) return cuda_fail(e, "cudaGetSymbolAddress(g_noalloc_scratch)");
    *out = p;
    return CPVS_OK;
}

}  // namespace
}  // namespace cpvs

extern "C" CPVS_API cpvs_status cpvs_shadow_build_noalloc(const float* depth, uint32_t n, uint32_t z_tile_index,
                                                          uint32_t z_tile_num, uint32_t flags, uint32_t* dag_out,
                                                          uint64_t dag_capacity, uint64_t* dag_words,
                                                          void* stream) {
    using namespace cpvs;
    if (dag_words) *dag_words = 0;
    if (!depth) return fail(CPVS_ERR_INVALID_ARG, "noalloc: null depth map");
    if (n < 8 || n > kNoAllocMaxSide || (n & (n - 1)))
        return fail(CPVS_ERR_INVALID_ARG, "noalloc: map side must be a power of two in [8, " +
                                              std::to_string(kNoAllocMaxSide) + "], got " + std::to_string(n) +
                                              " (larger maps: cpvs_shadow_create_from_depth)");
    if (flags & ~CPVS_FLAG_LEAFMASKS)
        return fail(CPVS_ERR_INVALID_ARG, "noalloc: unknown flag bits " + std::to_string(flags & ~CPVS_FLAG_LEAFMASKS));
    if (!(flags & CPVS_FLAG_LEAFMASKS) && n > kNoAllocMaxSideNoLeaf)
        return fail(CPVS_ERR_INVALID_ARG, "noalloc: without leafmasks the map side must not exceed " +
                                              std::to_string(kNoAllocMaxSideNoLeaf) + ", got " + std::to_string(n));
    if (z_tile_num == 0 || z_tile_index >= z_tile_num)
        return fail(CPVS_ERR_INVALID_ARG, "noalloc: need z_tile_index < z_tile_num");
    if ((uint64_t)n * z_tile_num > (1ull << 23))
        return fail(CPVS_ERR_INVALID_ARG, "noalloc: n * z_tile_num must not exceed 2^23");
    cudaStream_t st = (cudaStream_t)stream;
    const int nl = log2_u32(n) + 1, R = nl - 2;
    const bool leafmasks = (flags & CPVS_FLAG_LEAFMASKS) && (nl - 3 >= 2);
    const int bottom = leafmasks ? 2 : 0;

    // full-octree capacity of every level: 8^(R-L) nodes
    uint64_t cap[CPVS_MAX_LEVELS] = {0};
    uint64_t maxcap = 1;
    for (int L = bottom; L <= R; ++L) {
        cap[L] = 1ull << (3 * (R - L));
        maxcap = std::max(maxcap, cap[L]);
    }
    uint64_t tcap = 1024;
    while (tcap < 2 * maxcap) tcap <<= 1;
    int dev = 0, sms = 0;
    CPVS_CUDA(cudaGetDevice(&dev));
    CPVS_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
    const uint32_t max_grid = (uint32_t)std::max(sms, 1) * 8;
    auto grid_for = [&](uint64_t items, uint64_t per_block) -> uint32_t {
        uint64_t g = (items + per_block - 1) / per_block;
        return (uint32_t)std::max<uint64_t>(1, std::min<uint64_t>(g, max_grid));
    };

    // carve the scratch
    void* base = nullptr;
    cpvs_status r = noalloc_scratch_address(&base);
    if (r != CPVS_OK) return r;
    Arena A;
    A.base = static_cast<char*>(base);
    A.size = kNoAllocScratchBytes;
    float2* pyr = A.take<float2>(pyramid_texels(n));
    LevelDev lv[CPVS_MAX_LEVELS];
    std::memset(lv, 0, sizeof(lv));
    for (int L = bottom; L <= R; ++L) {
        const uint64_t c = cap[L];
        lv[L].coord = A.take<uint64_t>(c);
        lv[L].job = A.take<uint32_t>(c);
        lv[L].mask = A.take<uint32_t>(c);
        lv[L].first = A.take<uint32_t>(c);
        lv[L].uid = A.take<uint32_t>(c);
        lv[L].slot = A.take<uint32_t>(c);
        lv[L].uniq = A.take<uint32_t>(c);
        lv[L].woff = A.take<uint32_t>(c);
        if (leafmasks && L == 2) {
            lv[L].slices = A.take<uint64_t>(c * 8);
            lv[L].hash = A.take<uint64_t>(c);
        }
    }
    unsigned long long* table = A.take<unsigned long long>(tcap);
    uint2* partials = A.take<uint2>(max_grid);
    uint32_t* counts = A.take<uint32_t>(CPVS_MAX_LEVELS);
    uint32_t* level_u = A.take<uint32_t>(2 * CPVS_MAX_LEVELS);
    uint32_t* err = A.take<uint32_t>(1);
    const size_t segn = CPVS_MAX_LEVELS;
    uint32_t* segbuf = A.take<uint32_t>(segn * 7);
    uint64_t* job_off = A.take<uint64_t>(2);
    uint32_t* root_dev = A.take<uint32_t>(1);
    JobDev* job_dev = A.take<JobDev>(1);
    if (A.used > A.size)
        return fail(CPVS_ERR_INVALID_ARG, "noalloc: this map needs " + std::to_string(A.used) +
                                              " scratch bytes, above the fixed " +
                                              std::to_string(kNoAllocScratchBytes) + " (use leafmasks or a smaller map)");
    SegDev seg{segbuf, segbuf + segn, segbuf + 2 * segn, segbuf + 3 * segn, segbuf + 4 * segn, segbuf + 5 * segn};
    JobLayout lay{job_off, segbuf + 6 * segn};

    // the array keeps the previous call's contents: reset what starts at zero
    CPVS_CUDA(cudaMemsetAsync(segbuf, 0, segn * 7 * sizeof(uint32_t), st));
    CPVS_CUDA(cudaMemsetAsync(counts, 0, CPVS_MAX_LEVELS * sizeof(uint32_t), st));
    CPVS_CUDA(cudaMemsetAsync(level_u, 0, 2 * CPVS_MAX_LEVELS * sizeof(uint32_t), st));
    CPVS_CUDA(cudaMemsetAsync(err, 0, sizeof(uint32_t), st));
    r = launch_pyramid(depth, n, pyr, st);
    if (r != CPVS_OK) return r;
    const JobDev jd{pyr, depth, n, (uint32_t)nl, z_tile_index, z_tile_num};
    const uint32_t root = (uint32_t)R, one = 1;
    const uint64_t root_coord = pack_xyz(0, 0, 2 * z_tile_index);
    const uint32_t zero = 0;
    CPVS_CUDA(cudaMemcpyAsync(job_dev, &jd, sizeof(jd), cudaMemcpyHostToDevice, st));
    CPVS_CUDA(cudaMemcpyAsync(root_dev, &root, 4, cudaMemcpyHostToDevice, st));
    CPVS_CUDA(cudaMemcpyAsync(lv[R].coord, &root_coord, 8, cudaMemcpyHostToDevice, st));
    CPVS_CUDA(cudaMemcpyAsync(lv[R].job, &zero, 4, cudaMemcpyHostToDevice, st));
    CPVS_CUDA(cudaMemcpyAsync(counts + R, &one, 4, cudaMemcpyHostToDevice, st));

    for (int L = R; L > bottom; --L) {
        const uint32_t g = grid_for(cap[L], kThreads * 4);
        k_expand_count<<<g, kThreads, 0, st>>>(lv[L], counts, job_dev, 1, L, partials, err);
        k_expand_write<<<g, kThreads, 0, st>>>(lv[L], lv[L - 1], counts, L, partials, nullptr, 0, seg,
                                               (uint32_t)cap[L - 1], err);
    }
    if (leafmasks)
        k_leaf_masks<<<grid_for(cap[2], kThreads), kThreads, 0, st>>>(lv[2], counts, job_dev, 1, 2, seg, err);
    else
        k_classify_bottom<<<grid_for(cap[0], kThreads), kThreads, 0, st>>>(lv[0], counts, job_dev, 1, 0, seg, err);
    for (int L = bottom; L <= R; ++L) {
        uint64_t tc = 1024;
        while (tc < 2 * cap[L]) tc <<= 1;
        const bool leaf = leafmasks && L == 2;
        const uint32_t gs = grid_for(cap[L], kThreads * 4), gi = grid_for(cap[L], kThreads);
        const LevelDev child = (L > bottom) ? lv[L - 1] : lv[L];
        CPVS_CUDA(cudaMemsetAsync(table, 0xFF, tc * sizeof(unsigned long long), st));
        if (leaf) {
            k_dedup_insert<true><<<gi, kThreads, 0, st>>>(lv[L], child, counts, L, table, tc - 1, err);
            k_dedup_resolve<true><<<gs, kThreads, 0, st>>>(lv[L], counts, L, table, partials);
            k_dedup_scan<true><<<gs, kThreads, 0, st>>>(lv[L], counts, level_u, L, table, partials, seg);
        } else {
            k_dedup_insert<false><<<gi, kThreads, 0, st>>>(lv[L], child, counts, L, table, tc - 1, err);
            k_dedup_resolve<false><<<gs, kThreads, 0, st>>>(lv[L], counts, L, table, partials);
            k_dedup_scan<false><<<gs, kThreads, 0, st>>>(lv[L], counts, level_u, L, table, partials, seg);
        }
        k_dedup_remap<<<gi, kThreads, 0, st>>>(lv[L], counts, L, table);
    }
    k_layout<<<1, 1024, 0, st>>>(seg, lay, root_dev, 1, bottom, nullptr, nullptr);
    CPVS_CUDA(cudaGetLastError());
    uint64_t hoff[2] = {0, 0};
    uint32_t hlu[2 * CPVS_MAX_LEVELS] = {0};
    uint32_t herr = 0;
    CPVS_CUDA(cudaMemcpyAsync(hoff, job_off, sizeof(hoff), cudaMemcpyDeviceToHost, st));
    CPVS_CUDA(cudaMemcpyAsync(hlu, level_u, sizeof(hlu), cudaMemcpyDeviceToHost, st));
    CPVS_CUDA(cudaMemcpyAsync(&herr, err, 4, cudaMemcpyDeviceToHost, st));
    CPVS_CUDA(cudaStreamSynchronize(st));
    if (herr) return fail(CPVS_ERR_DEVICE, "noalloc: internal check " + std::to_string(herr));
    const uint64_t total = hoff[1];
    if (dag_words) *dag_words = total;
    if (!dag_out || dag_capacity < total)
        return fail(CPVS_ERR_CAPACITY, "noalloc: the DAG has " + std::to_string(total) + " words, the output holds " +
                                           std::to_string(dag_capacity));
    for (int L = R; L >= bottom; --L) {
        if (!hlu[2 * L]) continue;
        const LevelDev child = (L > bottom) ? lv[L - 1] : lv[L];
        const uint32_t g = grid_for(hlu[2 * L], kThreads);
        if (leafmasks && L == 2)
            k_emit<true><<<g, kThreads, 0, st>>>(lv[L], child, level_u, L, seg, lay, dag_out, total, err);
        else
            k_emit<false><<<g, kThreads, 0, st>>>(lv[L], child, level_u, L, seg, lay, dag_out, total, err);
    }
    CPVS_CUDA(cudaGetLastError());
    CPVS_CUDA(cudaMemcpyAsync(&herr, err, 4, cudaMemcpyDeviceToHost, st));
    CPVS_CUDA(cudaStreamSynchronize(st));
    if (herr) return fail(CPVS_ERR_DEVICE, "noalloc: internal check " + std::to_string(herr));
    return CPVS_OK;
}
