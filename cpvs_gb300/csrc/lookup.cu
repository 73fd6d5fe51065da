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
// The DAG (9.4 MB for an 8192^2 map) stays in L2; the hops are dependent
// 4-byte loads, so the kernel is latency- and L2-bound rather than HBM-bound.
// Every query issues its loads through the read-only path (__ldg).
#include "common.cuh"

namespace cpvs {
namespace {

constexpr int kThreads = 256;

__device__ __forceinline__ int32_t quantise(float v, float scale) {
    const float t = __fmul_rn(__fadd_rn(v, 1.0f), 0.5f);
    return __float2int_rz(__fmul_rn(t, scale));
}

// Descent from word `base` (the DAG's root) with pointers relative to
// `base`.  Returns true when the voxel is lit.  Every read is checked
// against `words` (the buffer's size), so a malformed DAG cannot make the
// kernel read outside it; such a query answers "shadow".
__device__ __forceinline__ bool descend(const uint32_t* __restrict__ dag, uint64_t words, uint32_t base,
                                        int num_levels, bool leafmasks, int32_t px, int32_t py, int32_t pz) {
    uint64_t off = base;
    const int min_level = leafmasks ? 3 : 0;
    for (int level = num_levels - 2; level >= min_level; --level) {
        const int32_t bit = 1 << level;
        const uint32_t c = ((px & bit) ? 1u : 0u) | ((py & bit) ? 2u : 0u) | ((pz & bit) ? 4u : 0u);
        if (off >= words) return false;
        const uint32_t m = __ldg(dag + off);
        const uint32_t v = (m >> (2u * c)) & 3u;
        if (v != kPartial) return v == kVisible;
        const uint64_t slot = off + 1u + child_rank(m, c);
        if (slot >= words) return false;
        off = (uint64_t)base + __ldg(dag + slot);
    }
    if (!leafmasks) return true;  // unreachable: level 0 has no partial children
    if (off >= words) return false;
    const uint32_t c = (uint32_t)(pz & 7);
    const uint32_t m = __ldg(dag + off);
    const uint32_t v = (m >> (2u * c)) & 3u;
    if (v != kPartial) return v == kVisible;
    const uint32_t b = (uint32_t)((px & 7) + 8 * (py & 7));
    const uint64_t idx = off + child_rank(m, c) * 2u + 1u + (b >> 5);
    if (idx >= words) return false;
    const uint32_t w = __ldg(dag + idx);
    return (w >> (b & 31u)) & 1u;
}

template <bool NDC>
__global__ void __launch_bounds__(kThreads)
    k_lookup(const uint32_t* __restrict__ dag, uint64_t words, int num_levels, bool leafmasks,
             const void* __restrict__ q, uint64_t n, uint32_t* __restrict__ bits) {
    const int lane = threadIdx.x & 31;
    const uint64_t nwords = (n + 31) / 32;
    const uint64_t nw = ((uint64_t)gridDim.x * blockDim.x) >> 5;
    const float scale = (float)((1u << (num_levels - 1)) - 1u);
    for (uint64_t w = ((uint64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5; w < nwords; w += nw) {
        const uint64_t i = w * 32 + (uint64_t)lane;
        bool lit = false;
        if (i < n) {
            int32_t px, py, pz;
            if (NDC) {
                const float* p = static_cast<const float*>(q) + 3 * i;
                px = quantise(p[0], scale);
                py = quantise(p[1], scale);
                pz = quantise(p[2], scale);
            } else {
                const int32_t* p = static_cast<const int32_t*>(q) + 3 * i;
                px = p[0];
                py = p[1];
                pz = p[2];
            }
            lit = descend(dag, words, 0u, num_levels, leafmasks, px, py, pz);
        }
        const uint32_t word = __ballot_sync(0xffffffffu, lit);
        if (lane == 0) bits[w] = word;
    }
}

// Grid routing (shader/traverse.cs:75-88): the path at resolution
// 2^(dag_levels+grid_levels-1), its top bits select the cell, the cell word
// holds the DAG offset or a uniform-cell sentinel.
__global__ void __launch_bounds__(kThreads)
    k_grid_lookup(const uint32_t* __restrict__ dag, uint64_t words, const uint32_t* __restrict__ cells, uint32_t length,
                  int dag_levels, int grid_levels, bool leafmasks, const float* __restrict__ q, uint64_t n,
                  uint32_t* __restrict__ bits) {
    const int lane = threadIdx.x & 31;
    const uint64_t nwords = (n + 31) / 32;
    const uint64_t nw = ((uint64_t)gridDim.x * blockDim.x) >> 5;
    const float scale = (float)((1u << (dag_levels + grid_levels - 1)) - 1u);
    for (uint64_t w = ((uint64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5; w < nwords; w += nw) {
        const uint64_t i = w * 32 + (uint64_t)lane;
        bool lit = false;
        if (i < n) {
            const float* p = q + 3 * i;
            const int32_t px = quantise(p[0], scale), py = quantise(p[1], scale), pz = quantise(p[2], scale);
            const int32_t gx = px >> (dag_levels - 1), gy = py >> (dag_levels - 1), gz = pz >> (dag_levels - 1);
            if (gx < 0 || gy < 0 || gz < 0 || gx >= (int32_t)length || gy >= (int32_t)length || gz >= (int32_t)length) {
                lit = true;
            } else {
                const uint32_t cell = __ldg(cells + ((size_t)gz * length + gy) * length + gx);
                if (cell == 0xFFFFFFFFu)
                    lit = false;
                else if (cell == 0xFFFFFFFEu)
                    lit = true;
                else
                    lit = descend(dag, words, cell, dag_levels, leafmasks, px, py, pz);
            }
        }
        const uint32_t word = __ballot_sync(0xffffffffu, lit);
        if (lane == 0) bits[w] = word;
    }
}

uint32_t lookup_grid(int num_sms, uint64_t n) {
    const uint64_t warps = (n + 31) / 32;
    const uint64_t blocks = (warps * 32 + kThreads - 1) / kThreads;
    const uint64_t cap = (uint64_t)(num_sms > 0 ? num_sms : 152) * 16;
    return (uint32_t)(blocks < 1 ? 1 : (blocks < cap ? blocks : cap));
}

}  // namespace

cpvs_status launch_lookup(const uint32_t* dag, uint64_t words, uint32_t num_levels, bool leafmasks, const void* xyz,
                          bool ndc, uint64_t n, uint32_t* bits, cudaStream_t st, Timing* timing) {
    if (n == 0) return CPVS_OK;
    KernelTimer kt(timing, K_LOOKUP, st);
    int dev = 0, sms = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    const uint32_t g = lookup_grid(sms, n);
    if (ndc)
        k_lookup<true><<<g, kThreads, 0, st>>>(dag, words, (int)num_levels, leafmasks, xyz, n, bits);
    else
        k_lookup<false><<<g, kThreads, 0, st>>>(dag, words, (int)num_levels, leafmasks, xyz, n, bits);
    CPVS_CUDA(cudaGetLastError());
    return CPVS_OK;
}

cpvs_status launch_grid_lookup(const uint32_t* dag, uint64_t words, const uint32_t* cells, uint32_t length,
                               uint32_t dag_levels, bool leafmasks, const float* xyz, uint64_t n, uint32_t* bits,
                               cudaStream_t st, Timing* timing) {
    if (n == 0) return CPVS_OK;
    KernelTimer kt(timing, K_GRID_LOOKUP, st);
    int dev = 0, sms = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    const uint32_t g = lookup_grid(sms, n);
    k_grid_lookup<<<g, kThreads, 0, st>>>(dag, words, cells, length, (int)dag_levels, log2_u32(length), leafmasks, xyz, n,
                                          bits);
    CPVS_CUDA(cudaGetLastError());
    return CPVS_OK;
}

}  // namespace cpvs
