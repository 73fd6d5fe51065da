// Min-max pyramid of a depth map, and the per-level SVO node bounds.
//
// Replaces MinMaxHierarchy (src/MinMaxHierarchy.cpp:9-97).  Level L >= 1 is
// (n>>L)^2 (min,max) float pairs; texel (x,y) of level L reduces texels
// a=(2x,2y), b=(2x+1,2y), c=(2x,2y+1), d=(2x+1,2y+1) of level L-1 as
// pred(pred(a,b), pred(c,d)) with pred = std::min<float> / std::max<float>
// (:29-49), so the result is bit-identical to the reference's, signed zeros
// and NaN included.  Level 1 reads the single-channel depth map for both min
// and max (:75-97).
//
// One CTA reduces a T x T input tile (T = 64, or the whole level when it is
// smaller) through log2(T) levels: the first level straight from global
// memory with 16-byte loads, the rest in shared memory.  Three launches cover
// an 8192^2 map (levels 1-6, 7-12, 13).  HBM-bound: the map is read once and
// every pyramid texel written once.
#include <vector>

#include "common.cuh"

namespace cpvs {
namespace {

__device__ __forceinline__ float pmin(float a, float b) { return (b < a) ? b : a; }  // std::min<float>
__device__ __forceinline__ float pmax(float a, float b) { return (a < b) ? b : a; }  // std::max<float>

constexpr int kTile = 64;
constexpr int kThreads = 256;

// in: level `L0-1` of side S (the depth map when FROM_DEPTH), out: pyramid
// level array; writes levels L0 .. L0+log2(T)-1 of this CTA's tile, those
// below `store_from` only into shared memory.  With
// `copy` (FROM_DEPTH only) the depth map is also written there as it is
// read: a map in host memory that the GPU reads in place crosses the host
// link once, while it is reduced, instead of in a separate copy first.
// Tile `tile` of the pass, with the block's shared buffers buf0
// ((kTile/2)^2 pairs) and buf1 ((kTile/4)^2 pairs).
template <bool FROM_DEPTH>
__device__ __forceinline__ void pyramid_tile(const void* __restrict__ in, uint32_t S, float2* __restrict__ out,
                                             uint32_t n, int L0, uint32_t T, float* __restrict__ copy,
                                             int store_from, uint32_t* nan_flag, uint32_t tile, float2* buf0,
                                             float2* buf1) {
    const uint32_t tiles_x = S / T;
    const uint32_t tx = tile % tiles_x, ty = tile / tiles_x;

    // first level: (T/2)^2 outputs of this tile
    uint32_t half = T / 2;
    int nan = 0;  // a NaN among the depths this thread read
    {
        const uint32_t So = S / 2;
        float2* dst = out + pyramid_level_offset_dev(n, L0);
        for (uint32_t o = threadIdx.x; o < half * half; o += blockDim.x) {
            const uint32_t ox = o % half, oy = o / half;
            const uint32_t ix = (tx * T) + 2 * ox, iy = (ty * T) + 2 * oy;
            float lo, hi;
            if (FROM_DEPTH) {
                const float* d = static_cast<const float*>(in);
                const float2 r0 = *reinterpret_cast<const float2*>(d + (size_t)iy * S + ix);
                const float2 r1 = *reinterpret_cast<const float2*>(d + (size_t)(iy + 1) * S + ix);
                if (copy) {
                    *reinterpret_cast<float2*>(copy + (size_t)iy * S + ix) = r0;
                    *reinterpret_cast<float2*>(copy + (size_t)(iy + 1) * S + ix) = r1;
                }
                lo = pmin(pmin(r0.x, r0.y), pmin(r1.x, r1.y));
                hi = pmax(pmax(r0.x, r0.y), pmax(r1.x, r1.y));
                nan |= (r0.x != r0.x) | (r0.y != r0.y) | (r1.x != r1.x) | (r1.y != r1.y);
            } else {
                const float2* p = static_cast<const float2*>(in);
                const float4 r0 = *reinterpret_cast<const float4*>(p + (size_t)iy * S + ix);
                const float4 r1 = *reinterpret_cast<const float4*>(p + (size_t)(iy + 1) * S + ix);
                lo = pmin(pmin(r0.x, r0.z), pmin(r1.x, r1.z));
                hi = pmax(pmax(r0.y, r0.w), pmax(r1.y, r1.w));
            }
            const float2 v = make_float2(lo, hi);
            if (L0 >= store_from) dst[(size_t)(ty * half + oy) * So + tx * half + ox] = v;
            buf0[o] = v;
        }
    }
    if (FROM_DEPTH && nan_flag && __any_sync(0xffffffffu, nan) && (threadIdx.x & 31u) == 0) atomicOr(nan_flag, 1u);
    // remaining levels of the tile in shared memory (ping-pong buf0 <-> buf1)
    uint32_t So = S / 2;
    int L = L0 + 1;
    float2* src = buf0;
    float2* nxt = buf1;
    while (half > 1) {
        __syncthreads();
        const uint32_t h2 = half / 2;
        So /= 2;
        float2* dst = out + pyramid_level_offset_dev(n, L);
        for (uint32_t o = threadIdx.x; o < h2 * h2; o += blockDim.x) {
            const uint32_t ox = o % h2, oy = o / h2;
            const float2 a = src[(2 * oy) * half + 2 * ox], b = src[(2 * oy) * half + 2 * ox + 1];
            const float2 c = src[(2 * oy + 1) * half + 2 * ox], d = src[(2 * oy + 1) * half + 2 * ox + 1];
            const float2 v = make_float2(pmin(pmin(a.x, b.x), pmin(c.x, d.x)), pmax(pmax(a.y, b.y), pmax(c.y, d.y)));
            if (L >= store_from) dst[(size_t)(ty * h2 + oy) * So + tx * h2 + ox] = v;
            nxt[o] = v;
        }
        // the next level reads what this one wrote: swap, and reuse the
        // larger buffer for the level after (its size only shrinks)
        float2* t = src;
        src = nxt;
        nxt = t;
        half = h2;
        ++L;
    }
}

template <bool FROM_DEPTH>
__global__ void __launch_bounds__(kThreads) k_pyramid(const void* __restrict__ in, uint32_t S, float2* __restrict__ out,
                                                      uint32_t n, int L0, uint32_t T, float* __restrict__ copy,
                                                      int store_from, uint32_t* nan_flag) {
    chain_enter();
    __shared__ float2 buf0[(kTile / 2) * (kTile / 2)];
    __shared__ float2 buf1[(kTile / 4) * (kTile / 4)];
    pyramid_tile<FROM_DEPTH>(in, S, out, n, L0, T, copy, store_from, nan_flag, blockIdx.x, buf0, buf1);
}

// Levels 1-6 of a 64x64 tile straight from the depth map, with the tile
// size fixed at compile time: each thread reduces two horizontally adjacent
// level-1 texels per step from two 16-byte loads (one per input row) and
// stores them as one 16-byte (min,max,min,max) pair; a warp covers 512
// contiguous bytes of each input row.  Levels 2-6 reduce in shared memory.
// With `copy` the map is also written there as it is read; levels below
// `store_from` stay in shared memory.
__device__ __forceinline__ void pyramid64_tile(const float* __restrict__ in, uint32_t S, float2* __restrict__ out,
                                               uint32_t n, float* __restrict__ copy, int store_from,
                                               uint32_t* nan_flag, uint32_t tile, float2* buf0, float2* buf1) {
    const uint32_t tiles_x = S >> 6;
    const uint32_t tx = tile % tiles_x, ty = tile / tiles_x;
    int nan = 0;  // a NaN among the depths this thread read
    {
        const uint32_t So = S >> 1;
        float2* dst = out;  // level 1 starts the pyramid array
#pragma unroll
        for (int k = 0; k < 2; ++k) {
            const uint32_t pidx = threadIdx.x + k * kThreads;  // 512 texel pairs: 32 rows x 16
            const uint32_t oy = pidx >> 4, px = pidx & 15u;
            const size_t r0 = (size_t)(ty * 64 + 2 * oy) * S + tx * 64 + 4 * px;
            const float4 a = *reinterpret_cast<const float4*>(in + r0);
            const float4 b = *reinterpret_cast<const float4*>(in + r0 + S);
            if (copy) {
                *reinterpret_cast<float4*>(copy + r0) = a;
                *reinterpret_cast<float4*>(copy + r0 + S) = b;
            }
            const float2 v0 = make_float2(pmin(pmin(a.x, a.y), pmin(b.x, b.y)), pmax(pmax(a.x, a.y), pmax(b.x, b.y)));
            const float2 v1 = make_float2(pmin(pmin(a.z, a.w), pmin(b.z, b.w)), pmax(pmax(a.z, a.w), pmax(b.z, b.w)));
            nan |= (a.x != a.x) | (a.y != a.y) | (a.z != a.z) | (a.w != a.w) | (b.x != b.x) | (b.y != b.y) |
                   (b.z != b.z) | (b.w != b.w);
            if (store_from <= 1)
                *reinterpret_cast<float4*>(dst + (size_t)(ty * 32 + oy) * So + tx * 32 + 2 * px) =
                    make_float4(v0.x, v0.y, v1.x, v1.y);
            buf0[oy * 32 + 2 * px] = v0;
            buf0[oy * 32 + 2 * px + 1] = v1;
        }
    }
    if (nan_flag && __any_sync(0xffffffffu, nan) && (threadIdx.x & 31u) == 0) atomicOr(nan_flag, 1u);
    uint32_t So = S >> 1;
    float2* src = buf0;
    float2* nxt = buf1;
#pragma unroll
    for (int lvl = 2; lvl <= 6; ++lvl) {
        __syncthreads();
        const uint32_t h = 64u >> lvl, lh = 6 - lvl;  // output side of this level in the tile, log2
        So >>= 1;
        float2* dst = out + pyramid_level_offset_dev(n, lvl);
        if (threadIdx.x < h * h) {
            const uint32_t o = threadIdx.x, ox = o & (h - 1), oy = o >> lh, w = 2 * h;
            const float2 a = src[(2 * oy) * w + 2 * ox], b = src[(2 * oy) * w + 2 * ox + 1];
            const float2 c = src[(2 * oy + 1) * w + 2 * ox], d = src[(2 * oy + 1) * w + 2 * ox + 1];
            const float2 v = make_float2(pmin(pmin(a.x, b.x), pmin(c.x, d.x)), pmax(pmax(a.y, b.y), pmax(c.y, d.y)));
            if (lvl >= store_from) dst[(size_t)(ty * h + oy) * So + tx * h + ox] = v;
            nxt[o] = v;
        }
        float2* t = src;
        src = nxt;
        nxt = t;
    }
}

__global__ void __launch_bounds__(kThreads)
    k_pyramid64(const float* __restrict__ in, uint32_t S, float2* __restrict__ out, uint32_t n,
                float* __restrict__ copy, int store_from, uint32_t* nan_flag) {
    chain_enter();
    __shared__ float2 buf0[32 * 32];
    __shared__ float2 buf1[16 * 16];
    pyramid64_tile(in, S, out, n, copy, store_from, nan_flag, blockIdx.x, buf0, buf1);
}

// Many maps' pyramids, one pass over all of them per launch: entry j of
// the table covers tiles [first, next entry's first) of one map's pass.
// The same per-tile code as k_pyramid64 / k_pyramid, so the bits are the
// same as the maps' own passes.
struct PyrPass {
    const void* in;     // the map (FROM_DEPTH) or its level L0 - 1
    float2* out;        // the map's pyramid
    uint32_t* nan_flag;
    uint32_t S, n, T, first;
    int L0, store_from;
};
constexpr int kPyrBatch = 256;
struct PyrPassTable {
    PyrPass p[kPyrBatch];
    uint32_t count;
};

template <bool FROM_DEPTH>
__global__ void __launch_bounds__(kThreads) k_pyramid_batch(const __grid_constant__ PyrPassTable tab) {
    chain_enter();
    __shared__ float2 buf0[(kTile / 2) * (kTile / 2)];
    __shared__ float2 buf1[(kTile / 4) * (kTile / 4)];
    uint32_t lo = 0, hi = tab.count;  // the last entry whose first tile is <= blockIdx.x
    while (hi - lo > 1) {
        const uint32_t mid = (lo + hi) >> 1;
        if (tab.p[mid].first <= blockIdx.x) lo = mid; else hi = mid;
    }
    const PyrPass& P = tab.p[lo];
    const uint32_t tile = blockIdx.x - P.first;
    if (FROM_DEPTH && P.T == (uint32_t)kTile)
        pyramid64_tile(static_cast<const float*>(P.in), P.S, P.out, P.n, nullptr, P.store_from, P.nan_flag, tile,
                       buf0, buf1);
    else
        pyramid_tile<FROM_DEPTH>(P.in, P.S, P.out, P.n, P.L0, P.T, nullptr, P.store_from, P.nan_flag, tile, buf0,
                                 buf1);
}

// Zeroes the maps' NaN flags before their first pass.
__global__ void k_zero_flags(const __grid_constant__ PyrPassTable tab) {
    for (uint32_t j = threadIdx.x; j < tab.count; j += blockDim.x)
        if (tab.p[j].nan_flag) *tab.p[j].nan_flag = 0;
}

// Partial-cell count of one texel for a z range [lo, hi): the cells z with
// NOT(z+1 <= a) and NOT(z >= b), i.e. z in [floor(a), ceil(b)), where a and
// b are the scaled min and max; a NaN bound excludes nothing (the
// comparisons against it are false, as in cs::visible).
__device__ __forceinline__ uint64_t partial_cells(float a, float b, uint64_t lo, uint64_t hi) {
    double s = (a != a) ? (double)lo : floor((double)a);
    double e = (b != b) ? (double)hi : ceil((double)b);
    if (s < (double)lo) s = (double)lo;
    if (e > (double)hi) e = (double)hi;
    return (e > s) ? (uint64_t)(e - s) : 0ull;
}

constexpr int kBoundThreads = 256;

// One block per (level, texel chunk); block_level[] maps a block to its
// pyramid level.  For every z-tile job of this map, sums the partial cells of
// the job's z range at that level.
struct BlockTable {
    uint32_t first[CPVS_MAX_LEVELS + 1];
};

__global__ void __launch_bounds__(kBoundThreads)
    k_level_bounds(const float2* __restrict__ levels, uint32_t n, int num_levels, const BlockTable bt, int lmin, const BoundJob* __restrict__ jobs, int njobs, unsigned long long* bounds) {
    __shared__ uint64_t red[32];
    int L = lmin;
    while (L + 1 <= num_levels - 2 && blockIdx.x >= bt.first[L + 1 - lmin]) ++L;
    const uint32_t W = n >> L;
    const uint64_t texels = (uint64_t)W * W;
    const uint64_t t = (uint64_t)(blockIdx.x - bt.first[L - lmin]) * blockDim.x + threadIdx.x;
    const int R = num_levels - 2;
    float2 mm = make_float2(0.f, 0.f);
    const bool valid = t < texels;
    if (valid) mm = levels[pyramid_level_offset_dev(n, L) + t];
    for (int j = 0; j < njobs; ++j) {
        const BoundJob J = jobs[j];
        const float H = __uint2float_rn((n >> L) * J.z_num);
        const uint64_t span = 2ull << (R - L);
        uint64_t c = 0;
        if (valid) c = partial_cells(__fmul_rn(mm.x, H), __fmul_rn(mm.y, H), J.z_idx * span, (J.z_idx + 1) * span);
        const uint64_t s = block_sum_u64(c, red);
        if (threadIdx.x == 0 && s) atomicAdd(&bounds[(size_t)J.out_row * CPVS_MAX_LEVELS + (L - 1)], (unsigned long long)s);
    }
}

}  // namespace

cpvs_status launch_pyramid(const float* depth, uint32_t n, float2* levels, cudaStream_t st, Timing* timing,
                           float* depth_copy, int store_from, uint32_t* nan_flag) {
    KernelTimer kt(timing, K_PYRAMID, st);
    if (nan_flag) CPVS_CUDA(cudaMemsetAsync(nan_flag, 0, sizeof(uint32_t), st));
    uint32_t S = n;
    int L0 = 1;
    bool first = true;
    while (S > 1) {
        const uint32_t T = S < (uint32_t)kTile ? S : (uint32_t)kTile;
        const uint32_t tiles = (S / T) * (S / T);
        // chained: each pass may be scheduled while the work before it in
        // the stream drains, and waits for it at its start
        if (first && T == (uint32_t)kTile)
            CPVS_CUDA(launch_kernel(k_pyramid64, tiles, kThreads, 0, st, true, 0, depth, S, levels, n, depth_copy,
                                    store_from, nan_flag));
        else if (first)
            CPVS_CUDA(launch_kernel(k_pyramid<true>, tiles, kThreads, 0, st, true, 0, static_cast<const void*>(depth), S,
                                    levels, n, L0, T, depth_copy, store_from, nan_flag));
        else
            CPVS_CUDA(launch_kernel(k_pyramid<false>, tiles, kThreads, 0, st, true, 0,
                                    static_cast<const void*>(levels + pyramid_level_offset(n, L0 - 1)), S, levels, n,
                                    L0, T, static_cast<float*>(nullptr), store_from, static_cast<uint32_t*>(nullptr)));
        first = false;
        L0 += log2_u32(T);
        S /= T;
    }
    return CPVS_OK;
}

cpvs_status launch_pyramid_batch(const std::vector<PyramidMap>& maps, cudaStream_t st, Timing* timing) {
    KernelTimer kt(timing, K_PYRAMID, st);
    // per map its passes: (S, T, L0) while S > 1, as launch_pyramid runs them
    struct MapPass {
        uint32_t S, T;
        int L0;
    };
    std::vector<std::vector<MapPass>> passes(maps.size());
    size_t npass = 0;
    for (size_t m = 0; m < maps.size(); ++m) {
        uint32_t S = maps[m].n;
        int L0 = 1;
        while (S > 1) {
            const uint32_t T = S < (uint32_t)kTile ? S : (uint32_t)kTile;
            passes[m].push_back(MapPass{S, T, L0});
            L0 += log2_u32(T);
            S /= T;
        }
        npass = std::max(npass, passes[m].size());
    }
    // pass k of every map in launches of up to kPyrBatch maps
    for (size_t m0 = 0; m0 < maps.size(); m0 += kPyrBatch) {
        const size_t m1 = std::min(maps.size(), m0 + (size_t)kPyrBatch);
        PyrPassTable flags{};
        for (size_t m = m0; m < m1; ++m) flags.p[flags.count++].nan_flag = maps[m].nan_flag;
        k_zero_flags<<<1, 256, 0, st>>>(flags);
        CPVS_CUDA(cudaGetLastError());
        for (size_t k = 0; k < npass; ++k) {
            PyrPassTable tab{};
            uint32_t tiles = 0;
            for (size_t m = m0; m < m1; ++m) {
                if (k >= passes[m].size()) continue;
                const MapPass& q = passes[m][k];
                PyrPass& P = tab.p[tab.count++];
                P.in = k == 0 ? static_cast<const void*>(maps[m].depth)
                              : static_cast<const void*>(maps[m].levels + pyramid_level_offset(maps[m].n, q.L0 - 1));
                P.out = maps[m].levels;
                P.nan_flag = k == 0 ? maps[m].nan_flag : nullptr;
                P.S = q.S;
                P.n = maps[m].n;
                P.T = q.T;
                P.L0 = q.L0;
                // the first pass stores from the map's first stored level;
                // later passes read their predecessor's last level, stored
                P.store_from = maps[m].store_from;
                P.first = tiles;
                tiles += (q.S / q.T) * (q.S / q.T);
            }
            if (!tab.count) continue;
            if (k == 0)
                CPVS_CUDA(launch_kernel(k_pyramid_batch<true>, tiles, kThreads, 0, st, true, 0, tab));
            else
                CPVS_CUDA(launch_kernel(k_pyramid_batch<false>, tiles, kThreads, 0, st, true, 0, tab));
        }
    }
    return CPVS_OK;
}

cpvs_status launch_level_bounds(const float2* levels, uint32_t n, int lmin, const BoundJob* jobs_dev, int njobs,
                                unsigned long long* bounds, cudaStream_t st) {
    const int num_levels = log2_u32(n) + 1;
    const int R = num_levels - 2;
    if (lmin > R || njobs == 0) return CPVS_OK;
    // bt.first[k] = first block of level lmin+k
    BlockTable bt{};
    uint32_t blocks = 0;
    for (int L = lmin; L <= R; ++L) {
        bt.first[L - lmin] = blocks;
        const uint64_t tex = (uint64_t)(n >> L) * (n >> L);
        blocks += (uint32_t)((tex + kBoundThreads - 1) / kBoundThreads);
    }
    bt.first[R + 1 - lmin] = blocks;
    k_level_bounds<<<blocks, kBoundThreads, 0, st>>>(levels, n, num_levels, bt, lmin, jobs_dev, njobs, bounds);
    CPVS_CUDA(cudaGetLastError());
    return CPVS_OK;
}

}  // namespace cpvs
