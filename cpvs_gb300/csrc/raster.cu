// Depth-map producer: axis-aligned boxes and spheres over a ground plane,
// rasterised under an orthographic light straight into device memory.
//
// Replaces the reference's GL shadow pass and read-back
// (src/DeferredRenderer.cpp:110-148 renderSceneForSM / renderShadowMap,
// shader/create_sm.vert, src/ShadowMap.cpp:23-30 glGetTexImage): the map a
// build consumes is produced where the build runs.  The scene model is the
// one the synthetic workloads use (a plane plus min-combined boxes and
// spheres); every float operation matches the host rasteriser
// (cpvs_gb300/scene.py) bit for bit: pixel centre (x+0.5)/n, a box covers
// the centres in [c-h, c+h], a sphere covers the centres in its bounding
// square with dy*dy + dx*dx < r*r and contributes depth - sqrt(r*r - rho2).
//
// One CTA per 64x64 pixel tile: the primitives are streamed through shared
// memory in chunks, culled against the tile's centre range, and every thread
// min-combines the survivors into its 16 pixels.
#include <algorithm>

#include "common.cuh"

namespace cpvs {
namespace {

constexpr int kTile = 64;
constexpr int kThreads = 256;
constexpr int kChunk = 512;

__device__ __forceinline__ float centre(uint32_t i, float inv_n) {
    return __fmul_rn(__fadd_rn(__uint2float_rn(i), 0.5f), inv_n);  // (i + 0.5) / n, exact for power-of-two n
}

__global__ void __launch_bounds__(kThreads)
    k_raster(const float* __restrict__ boxes, uint32_t nb, const float* __restrict__ spheres, uint32_t ns, float plane,
             uint32_t n, uint32_t x0, uint32_t y0, uint32_t w, uint32_t h, float* __restrict__ out) {
    __shared__ float s_prim[kChunk][5];
    __shared__ uint32_t s_keep[kChunk];
    __shared__ uint32_t s_nkeep;
    const float inv_n = 1.0f / __uint2float_rn(n);
    const uint32_t tiles_x = (w + kTile - 1) / kTile;
    const uint32_t tx = blockIdx.x % tiles_x, ty = blockIdx.x / tiles_x;
    const uint32_t px0 = tx * kTile, py0 = ty * kTile;  // tile origin inside the window
    const uint32_t px1 = min(px0 + kTile, w), py1 = min(py0 + kTile, h);
    // centre range of the tile (global pixel indices x0+px, y0+py)
    const float cx_lo = centre(x0 + px0, inv_n), cx_hi = centre(x0 + px1 - 1, inv_n);
    const float cy_lo = centre(y0 + py0, inv_n), cy_hi = centre(y0 + py1 - 1, inv_n);
    constexpr int kPer = kTile * kTile / kThreads;  // 16 pixels per thread
    float d[kPer];
#pragma unroll
    for (int k = 0; k < kPer; ++k) d[k] = plane;

    for (int pass = 0; pass < 2; ++pass) {
        const bool is_box = pass == 0;
        const uint32_t np = is_box ? nb : ns;
        const float* src = is_box ? boxes : spheres;
        const int stride = is_box ? 5 : 4;
        for (uint32_t base = 0; base < np; base += kChunk) {
            const uint32_t cnt = min((uint32_t)kChunk, np - base);
            if (threadIdx.x == 0) s_nkeep = 0;
            __syncthreads();
            for (uint32_t i = threadIdx.x; i < cnt; i += blockDim.x) {
                const float* p = src + (size_t)(base + i) * stride;
                float lox, hix, loy, hiy;
                if (is_box) {
                    lox = __fsub_rn(p[0], p[2]);
                    hix = __fadd_rn(p[0], p[2]);
                    loy = __fsub_rn(p[1], p[3]);
                    hiy = __fadd_rn(p[1], p[3]);
                } else {
                    lox = __fsub_rn(p[0], p[2]);
                    hix = __fadd_rn(p[0], p[2]);
                    loy = __fsub_rn(p[1], p[2]);
                    hiy = __fadd_rn(p[1], p[2]);
                }
                // keep primitives whose window contains a centre of this tile
                if (lox <= cx_hi && hix >= cx_lo && loy <= cy_hi && hiy >= cy_lo) {
                    const uint32_t slot = atomicAdd(&s_nkeep, 1u);
                    s_keep[slot] = i;
                    for (int q = 0; q < stride; ++q) s_prim[i][q] = p[q];
                }
            }
            __syncthreads();
            const uint32_t nk = s_nkeep;
            for (uint32_t k2 = 0; k2 < nk; ++k2) {
                const float* p = s_prim[s_keep[k2]];
#pragma unroll
                for (int k = 0; k < kPer; ++k) {
                    const uint32_t pix = threadIdx.x + (uint32_t)k * kThreads;
                    const uint32_t lx = px0 + (pix % kTile), ly = py0 + (pix / kTile);
                    if (lx >= w || ly >= h) continue;
                    const float cx = centre(x0 + lx, inv_n), cy = centre(y0 + ly, inv_n);
                    if (is_box) {
                        if (__fsub_rn(p[0], p[2]) <= cx && cx <= __fadd_rn(p[0], p[2]) && __fsub_rn(p[1], p[3]) <= cy &&
                            cy <= __fadd_rn(p[1], p[3]))
                            d[k] = (p[4] < d[k] || p[4] != p[4]) ? p[4] : d[k];  // np.minimum keeps NaN
                    } else {
                        if (__fsub_rn(p[0], p[2]) <= cx && cx <= __fadd_rn(p[0], p[2]) && __fsub_rn(p[1], p[2]) <= cy &&
                            cy <= __fadd_rn(p[1], p[2])) {
                            const float dx = __fsub_rn(cx, p[0]), dy = __fsub_rn(cy, p[1]);
                            const float rho2 = __fadd_rn(__fmul_rn(dy, dy), __fmul_rn(dx, dx));
                            const float r2 = __fmul_rn(p[2], p[2]);
                            if (rho2 < r2) {
                                const float v = __fsub_rn(p[3], __fsqrt_rn(__fsub_rn(r2, rho2)));
                                d[k] = (v < d[k] || v != v) ? v : d[k];
                            }
                        }
                    }
                }
            }
            __syncthreads();
        }
    }
#pragma unroll
    for (int k = 0; k < kPer; ++k) {
        const uint32_t pix = threadIdx.x + (uint32_t)k * kThreads;
        const uint32_t lx = px0 + (pix % kTile), ly = py0 + (pix / kTile);
        if (lx < w && ly < h) out[(size_t)ly * w + lx] = d[k];
    }
}

}  // namespace

cpvs_status launch_raster(const float* boxes, uint32_t nb, const float* spheres, uint32_t ns, float plane, uint32_t n,
                          uint32_t x0, uint32_t y0, uint32_t w, uint32_t h, float* out, cudaStream_t st,
                          Timing* timing) {
    if (!w || !h) return CPVS_OK;
    KernelTimer kt(timing, K_RASTER, st);
    const uint64_t tiles = (uint64_t)((w + kTile - 1) / kTile) * ((h + kTile - 1) / kTile);
    if (tiles >= (1ull << 31)) return fail(CPVS_ERR_INVALID_ARG, "raster: window too large");
    k_raster<<<(uint32_t)tiles, kThreads, 0, st>>>(boxes, nb, spheres, ns, plane, n, x0, y0, w, h, out);
    CPVS_CUDA(cudaGetLastError());
    return CPVS_OK;
}

}  // namespace cpvs
