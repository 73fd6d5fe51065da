// Shared device and host helpers of the GB300 shadow library.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include "internal.h"

namespace cpvs {

// ------------------------------------------------------- chained launches
// Programmatic dependent launch.  Kernels launched with `chained` set may be
// scheduled while their predecessor in the stream drains; each such kernel
// first waits until that predecessor has completed and its writes are
// visible (a no-op when launched without the attribute), then lets its own
// successor be scheduled.  Every chained kernel waits at its start, so
// completion stays transitive along the chain.
__device__ __forceinline__ void chain_wait() { asm volatile("griddepcontrol.wait;" ::: "memory"); }
__device__ __forceinline__ void chain_release() { asm volatile("griddepcontrol.launch_dependents;" ::: "memory"); }
__device__ __forceinline__ void chain_enter() {
    chain_wait();
    chain_release();
}

// `smem`: dynamic shared memory bytes; `cluster` > 0: one cluster of that
// many blocks.
template <typename... Exp, typename... Act>
inline cudaError_t launch_kernel(void (*kernel)(Exp...), uint32_t grid, uint32_t block, size_t smem, cudaStream_t st,
                                 bool chained, uint32_t cluster, Act&&... args) {
    cudaLaunchConfig_t cfg{};
    cfg.gridDim = dim3(grid);
    cfg.blockDim = dim3(block);
    cfg.dynamicSmemBytes = smem;
    cfg.stream = st;
    cudaLaunchAttribute at[2];
    uint32_t na = 0;
    if (cluster) {
        at[na].id = cudaLaunchAttributeClusterDimension;
        at[na].val.clusterDim.x = cluster;
        at[na].val.clusterDim.y = 1;
        at[na].val.clusterDim.z = 1;
        ++na;
    }
    if (chained) {
        at[na].id = cudaLaunchAttributeProgrammaticStreamSerialization;
        at[na].val.programmaticStreamSerializationAllowed = 1;
        ++na;
    }
    cfg.attrs = at;
    cfg.numAttrs = na;
    return cudaLaunchKernelEx(&cfg, kernel, static_cast<Act&&>(args)...);
}

// ---------------------------------------------------------------- classes
// NodeVisibility (src/CompressedShadow.h:22-26).
constexpr uint32_t kShadow = 0, kVisible = 1, kPartial = 2;

// cs::visible (src/CompressedShadowUtil.h:35-43) for the z-cell
// [zc, zc+1) against the depth bounds already scaled by the level height.
// Every float operation is the IEEE round-to-nearest one the reference's
// CPU code performs; nothing may be contracted.
__device__ __forceinline__ uint32_t classify_cell(uint32_t zc, float dmin_scaled, float dmax_scaled) {
    const float zlo = __uint2float_rn(zc);
    const float zhi = __uint2float_rn(zc + 1u);
    if (zhi <= dmin_scaled) return kVisible;
    if (zlo >= dmax_scaled) return kShadow;
    return kPartial;
}

// cs::absoluteVisible (src/CompressedShadowUtil.h:51-57): the voxel centre
// ((zc + (zc+1)) * 0.5, in float32) against the scaled depth.
__device__ __forceinline__ bool voxel_lit(uint32_t zc, float d_scaled) {
    const float mid = __fmul_rn(__fadd_rn(__uint2float_rn(zc), __uint2float_rn(zc + 1u)), 0.5f);
    return mid <= d_scaled;
}

__host__ __device__ __forceinline__ uint32_t partial_children(uint32_t mask) {
#ifdef __CUDA_ARCH__
    return __popc(mask & 0xAAAAu);
#else
    return (uint32_t)__builtin_popcount(mask & 0xAAAAu);
#endif
}

// Float2 offset of pyramid level L (L >= 1) in the packed level array of an
// n x n map (levels 1..log2(n), (n>>l)^2 pairs each, back to back).
__host__ __device__ __forceinline__ uint64_t pyramid_level_offset_dev(uint32_t n, int L) {
    uint64_t o = 0;
    for (int l = 1; l < L; ++l) o += (uint64_t)(n >> l) * (n >> l);
    return o;
}

// ------------------------------------------------------------ coordinates
// A node coordinate packed in 64 bits: x (16) | y (16) | z (32).
__host__ __device__ __forceinline__ uint64_t pack_xyz(uint32_t x, uint32_t y, uint32_t z) {
    return (uint64_t)(x & 0xFFFFu) | ((uint64_t)(y & 0xFFFFu) << 16) | ((uint64_t)z << 32);
}
__host__ __device__ __forceinline__ uint32_t unpack_x(uint64_t c) { return (uint32_t)(c & 0xFFFFu); }
__host__ __device__ __forceinline__ uint32_t unpack_y(uint64_t c) { return (uint32_t)((c >> 16) & 0xFFFFu); }
__host__ __device__ __forceinline__ uint32_t unpack_z(uint64_t c) { return (uint32_t)(c >> 32); }

// ------------------------------------------------------------------ hash
// 64-bit finaliser of MurmurHash3 (Appleby, public domain).
__host__ __device__ __forceinline__ uint64_t fmix64(uint64_t k) {
    k ^= k >> 33;
    k *= 0xff51afd7ed558ccdULL;
    k ^= k >> 33;
    k *= 0xc4ceb9fe1a85ec53ULL;
    k ^= k >> 33;
    return k;
}
constexpr uint64_t kGolden = 0x9E3779B97F4A7C15ULL;
constexpr uint64_t kEmptySlot = 0xFFFFFFFFFFFFFFFFULL;

// ------------------------------------------------------------ block scan
// Exclusive scan of one uint32 pair per thread across a block of
// blockDim.x threads (a multiple of 32, at most 1024).  Returns the
// exclusive prefix; `total` receives the block total.  `smem` holds
// 2*32 words.
__device__ __forceinline__ uint2 block_exclusive_scan2(uint2 v, uint2& total, uint32_t* smem) {
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nwarps = blockDim.x >> 5;
    uint2 inc = v;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        uint32_t a = __shfl_up_sync(0xffffffffu, inc.x, o);
        uint32_t b = __shfl_up_sync(0xffffffffu, inc.y, o);
        if (lane >= o) {
            inc.x += a;
            inc.y += b;
        }
    }
    if (lane == 31) {
        smem[warp] = inc.x;
        smem[32 + warp] = inc.y;
    }
    __syncthreads();
    if (warp == 0) {
        uint32_t a = (lane < nwarps) ? smem[lane] : 0u;
        uint32_t b = (lane < nwarps) ? smem[32 + lane] : 0u;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            uint32_t ta = __shfl_up_sync(0xffffffffu, a, o);
            uint32_t tb = __shfl_up_sync(0xffffffffu, b, o);
            if (lane >= o) {
                a += ta;
                b += tb;
            }
        }
        smem[lane] = a;  // inclusive warp totals
        smem[32 + lane] = b;
    }
    __syncthreads();
    uint2 base = make_uint2(0u, 0u);
    if (warp > 0) {
        base.x = smem[warp - 1];
        base.y = smem[32 + warp - 1];
    }
    total = make_uint2(smem[nwarps - 1], smem[32 + nwarps - 1]);
    __syncthreads();
    return make_uint2(base.x + inc.x - v.x, base.y + inc.y - v.y);
}

// Block-wide sum of a uint64; result valid in every thread.
__device__ __forceinline__ uint64_t block_sum_u64(uint64_t v, uint64_t* smem) {
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nwarps = blockDim.x >> 5;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
    if (lane == 0) smem[warp] = v;
    __syncthreads();
    uint64_t t = 0;
    for (int w = 0; w < nwarps; ++w) t += smem[w];
    __syncthreads();
    return t;
}

// Sum of pair partials[0..b) over the block (every thread gets it).
__device__ __forceinline__ uint2 block_prefix_of_partials(const uint2* partials, uint32_t b, uint32_t* smem) {
    uint2 s = make_uint2(0u, 0u);
    for (uint32_t i = threadIdx.x; i < b; i += blockDim.x) {
        uint2 p = partials[i];
        s.x += p.x;
        s.y += p.y;
    }
    uint2 total;
    block_exclusive_scan2(s, total, smem);
    return total;
}

// Contiguous chunk [begin, end) of n items owned by block b of g blocks.
__device__ __forceinline__ void block_chunk(uint32_t n, uint32_t& begin, uint32_t& end) {
    const uint32_t g = gridDim.x, b = blockIdx.x;
    const uint32_t per = (n + g - 1) / g;
    const uint64_t s = (uint64_t)per * b, e = s + per;
    begin = (uint32_t)(s < n ? s : n);
    end = (uint32_t)(e < n ? e : n);
}

}  // namespace cpvs
