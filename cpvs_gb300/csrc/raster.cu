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
#include "internal.h"

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

// ------------------------------------------------------------ triangles
// A triangle (x0,y0,d0, x1,y1,d1, x2,y2,d2; x, y in map coordinates [0,1],
// d its depth at each vertex) covers pixel centre p when p lies in its
// bounding box [min x, max x] x [min y, max y] and the three edge functions
//   e0 = (x2-x1)*(py-y1) - (y2-y1)*(px-x1)
//   e1 = (x0-x2)*(py-y2) - (y0-y2)*(px-x2)
//   e2 = (x1-x0)*(py-y0) - (y1-y0)*(px-x0)
// all have the sign of area = (e0 + e1) + e2 (zero included, area nonzero;
// either winding); its depth there is ((e0*d0 + e1*d1) + e2*d2) / area.
// Every operation is a float32 round-to-nearest one in that order (the host
// rasteriser, cpvs_gb300/scene.py, does the same), and the map keeps the
// minimum, NaN propagating -- an order-independent combination, so the
// binning order does not matter.
//
// Triangles are binned into the 64x64 tiles of the window (count per tile,
// scan, fill), then one CTA per tile streams its list through shared memory.

struct TriWindow {
    uint32_t n, x0, y0, w, h, tiles_x, tiles_y;
    float inv_n;
};

// Conservative pixel range [lo, hi] (window coordinates, clamped) whose
// centres may fall in [a, b]; false when empty.
__device__ __forceinline__ bool pixel_range(float a, float b, uint32_t base, uint32_t size, uint32_t n, int32_t& lo,
                                            int32_t& hi) {
    if (!(a <= b)) return false;  // NaN, or an empty interval
    const float fa = fmaxf(a * (float)n - 1.5f, -1.0f), fb = fminf(b * (float)n + 0.5f, (float)n + 1.0f);
    lo = max((int32_t)floorf(fa) - (int32_t)base, 0);
    hi = min((int32_t)ceilf(fb) - (int32_t)base, (int32_t)size - 1);
    return lo <= hi;
}

__device__ __forceinline__ bool tri_tiles(const float* t, const TriWindow& W, int32_t& tx0, int32_t& tx1, int32_t& ty0,
                                          int32_t& ty1) {
    const float minx = fminf(fminf(t[0], t[3]), t[6]), maxx = fmaxf(fmaxf(t[0], t[3]), t[6]);
    const float miny = fminf(fminf(t[1], t[4]), t[7]), maxy = fmaxf(fmaxf(t[1], t[4]), t[7]);
    if (t[0] != t[0] || t[3] != t[3] || t[6] != t[6] || t[1] != t[1] || t[4] != t[4] || t[7] != t[7]) return false;
    int32_t px0, px1, py0, py1;
    if (!pixel_range(minx, maxx, W.x0, W.w, W.n, px0, px1) || !pixel_range(miny, maxy, W.y0, W.h, W.n, py0, py1))
        return false;
    tx0 = px0 / kTile;
    tx1 = px1 / kTile;
    ty0 = py0 / kTile;
    ty1 = py1 / kTile;
    return true;
}

__global__ void k_tri_count(const float* __restrict__ tris, uint32_t ntris, TriWindow W, uint32_t* counts) {
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < ntris; i += gridDim.x * blockDim.x) {
        int32_t tx0, tx1, ty0, ty1;
        if (!tri_tiles(tris + 9 * (size_t)i, W, tx0, tx1, ty0, ty1)) continue;
        for (int32_t ty = ty0; ty <= ty1; ++ty)
            for (int32_t tx = tx0; tx <= tx1; ++tx) atomicAdd(&counts[(size_t)ty * W.tiles_x + tx], 1u);
    }
}

// Exclusive scan of the tile counts into offsets (one block), and the total.
__global__ void k_tri_scan(const uint32_t* __restrict__ counts, uint32_t ntiles, uint32_t* offsets, uint32_t* cursor) {
    __shared__ uint32_t sm[64];
    uint32_t carry = 0;
    for (uint32_t t0 = 0; t0 < ntiles; t0 += blockDim.x) {
        const uint32_t t = t0 + threadIdx.x;
        const uint32_t c = t < ntiles ? counts[t] : 0u;
        uint2 tot;
        const uint32_t p = block_exclusive_scan2(make_uint2(c, 0u), tot, sm).x;
        if (t < ntiles) {
            offsets[t] = carry + p;
            cursor[t] = carry + p;
        }
        carry += tot.x;
        __syncthreads();
    }
    if (threadIdx.x == 0) offsets[ntiles] = carry;
}

__global__ void k_tri_bin(const float* __restrict__ tris, uint32_t ntris, TriWindow W, uint32_t* cursor,
                          uint32_t* __restrict__ list) {
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < ntris; i += gridDim.x * blockDim.x) {
        int32_t tx0, tx1, ty0, ty1;
        if (!tri_tiles(tris + 9 * (size_t)i, W, tx0, tx1, ty0, ty1)) continue;
        for (int32_t ty = ty0; ty <= ty1; ++ty)
            for (int32_t tx = tx0; tx <= tx1; ++tx) list[atomicAdd(&cursor[(size_t)ty * W.tiles_x + tx], 1u)] = i;
    }
}

constexpr int kTriChunk = 256;

__global__ void __launch_bounds__(kThreads)
    k_tri_raster(const float* __restrict__ tris, TriWindow W, const uint32_t* __restrict__ offsets,
                 const uint32_t* __restrict__ list, float plane, float* __restrict__ out) {
    __shared__ float s_t[kTriChunk][9];
    const uint32_t tx = blockIdx.x % W.tiles_x, ty = blockIdx.x / W.tiles_x;
    const uint32_t px0 = tx * kTile, py0 = ty * kTile;
    constexpr int kPer = kTile * kTile / kThreads;  // 16 pixels per thread
    float d[kPer];
#pragma unroll
    for (int k = 0; k < kPer; ++k) d[k] = plane;
    const uint32_t b = offsets[blockIdx.x], e = offsets[blockIdx.x + 1];
    for (uint32_t c0 = b; c0 < e; c0 += kTriChunk) {
        const uint32_t cnt = min((uint32_t)kTriChunk, e - c0);
        __syncthreads();
        for (uint32_t q = threadIdx.x; q < cnt * 9; q += blockDim.x) {
            const uint32_t r = q / 9, c = q % 9;
            s_t[r][c] = tris[9 * (size_t)list[c0 + r] + c];
        }
        __syncthreads();
        for (uint32_t r = 0; r < cnt; ++r) {
            const float* t = s_t[r];
            const float minx = fminf(fminf(t[0], t[3]), t[6]), maxx = fmaxf(fmaxf(t[0], t[3]), t[6]);
            const float miny = fminf(fminf(t[1], t[4]), t[7]), maxy = fmaxf(fmaxf(t[1], t[4]), t[7]);
            const float ax = __fsub_rn(t[6], t[3]), ay = __fsub_rn(t[7], t[4]);  // edge v1 -> v2
            const float bx = __fsub_rn(t[0], t[6]), by = __fsub_rn(t[1], t[7]);  // edge v2 -> v0
            const float cx = __fsub_rn(t[3], t[0]), cy = __fsub_rn(t[4], t[1]);  // edge v0 -> v1
#pragma unroll
            for (int k = 0; k < kPer; ++k) {
                const uint32_t pix = threadIdx.x + (uint32_t)k * kThreads;
                const uint32_t lx = px0 + (pix % kTile), ly = py0 + (pix / kTile);
                if (lx >= W.w || ly >= W.h) continue;
                const float px = centre(W.x0 + lx, W.inv_n), py = centre(W.y0 + ly, W.inv_n);
                if (!(minx <= px && px <= maxx && miny <= py && py <= maxy)) continue;
                const float e0 = __fsub_rn(__fmul_rn(ax, __fsub_rn(py, t[4])), __fmul_rn(ay, __fsub_rn(px, t[3])));
                const float e1 = __fsub_rn(__fmul_rn(bx, __fsub_rn(py, t[7])), __fmul_rn(by, __fsub_rn(px, t[6])));
                const float e2 = __fsub_rn(__fmul_rn(cx, __fsub_rn(py, t[1])), __fmul_rn(cy, __fsub_rn(px, t[0])));
                const float area = __fadd_rn(__fadd_rn(e0, e1), e2);
                const bool in = (area > 0.0f && e0 >= 0.0f && e1 >= 0.0f && e2 >= 0.0f) ||
                                (area < 0.0f && e0 <= 0.0f && e1 <= 0.0f && e2 <= 0.0f);
                if (!in) continue;
                const float num = __fadd_rn(__fadd_rn(__fmul_rn(e0, t[2]), __fmul_rn(e1, t[5])), __fmul_rn(e2, t[8]));
                const float v = __fdiv_rn(num, area);
                d[k] = (v < d[k] || v != v) ? v : d[k];  // np.minimum keeps NaN
            }
        }
    }
#pragma unroll
    for (int k = 0; k < kPer; ++k) {
        const uint32_t pix = threadIdx.x + (uint32_t)k * kThreads;
        const uint32_t lx = px0 + (pix % kTile), ly = py0 + (pix / kTile);
        if (lx < W.w && ly < W.h) out[(size_t)ly * W.w + lx] = d[k];
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

namespace cpvs {

cpvs_status launch_raster_triangles(Ctx& c, const float* tris, uint32_t ntris, float plane, uint32_t n, uint32_t x0,
                                    uint32_t y0, uint32_t w, uint32_t h, float* out, cudaStream_t st) {
    if (!w || !h) return CPVS_OK;
    TriWindow W{n, x0, y0, w, h, (w + kTile - 1) / kTile, (h + kTile - 1) / kTile, 1.0f / (float)n};
    const uint64_t ntiles = (uint64_t)W.tiles_x * W.tiles_y;
    if (ntiles >= (1ull << 31)) return fail(CPVS_ERR_INVALID_ARG, "raster_triangles: window too large");
    KernelTimer kt(&c.timing, K_RASTER, st);
    const uint64_t small_bytes = (3 * ntiles + 1) * 4;
    uint32_t* buf = nullptr;
    cpvs_status r = c.alloc((void**)&buf, small_bytes, false, st);
    if (r != CPVS_OK) return r;
    uint32_t *counts = buf, *offsets = buf + ntiles, *cursor = buf + 2 * ntiles + 1;
    uint32_t* list = nullptr;
    uint64_t list_bytes = 0;
    uint32_t total = 0;
    cudaError_t e = cudaMemsetAsync(counts, 0, ntiles * 4, st);
    const uint32_t g = (uint32_t)std::min<uint64_t>((ntris + 255) / 256 + 1, 152ull * 16);
    if (e == cudaSuccess && ntris) {
        k_tri_count<<<g, 256, 0, st>>>(tris, ntris, W, counts);
        e = cudaGetLastError();
    }
    if (e == cudaSuccess) {
        k_tri_scan<<<1, 1024, 0, st>>>(counts, (uint32_t)ntiles, offsets, cursor);
        e = cudaGetLastError();
    }
    if (e == cudaSuccess) e = cudaMemcpyAsync(&total, offsets + ntiles, 4, cudaMemcpyDeviceToHost, st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);  // the list is sized by the count
    if (e == cudaSuccess && total) {
        list_bytes = (uint64_t)total * 4;
        r = c.alloc((void**)&list, list_bytes, false, st);
        if (r == CPVS_OK) {
            k_tri_bin<<<g, 256, 0, st>>>(tris, ntris, W, cursor, list);
            e = cudaGetLastError();
        }
    }
    if (e == cudaSuccess && r == CPVS_OK) {
        k_tri_raster<<<(uint32_t)ntiles, kThreads, 0, st>>>(tris, W, offsets, list, plane, out);
        e = cudaGetLastError();
    }
    if (list) c.release(list, list_bytes, false, st);
    c.release(buf, small_bytes, false, st);
    if (r != CPVS_OK) return r;
    if (e != cudaSuccess) return cuda_fail(e, "raster_triangles");
    return CPVS_OK;
}

}  // namespace cpvs
