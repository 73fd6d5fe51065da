// Deferred shading of one frame: the fragment shader the reference runs over
// a full-screen quad after evaluate (shader/shade.frag:34-56, driven by
// DeferredRenderer::doAllShading, src/DeferredRenderer.cpp:319-348), on
// device buffers instead of G-buffer textures.  One thread per pixel; the
// kernel streams normals, albedo and the visibility byte from HBM and writes
// the colour once, so it is bound by HBM bandwidth.
//
// Every float operation is one IEEE round-to-nearest operation in a fixed
// order (no contraction), so results are bit-identical to the CPU
// restatement:
//   L        = l / sqrt((lx*lx + ly*ly) + lz*lz)          normalize(light.direction)
//   diffuse  = max(0, (Nx*Lx + Ny*Ly) + Nz*Lz)            max(0.0, dot(N, L))
//   vis      = byte / 255                                  the r8 visibility image
//            | shadow-map test (renderShadow == 0):        evaluateShadowMap
//              c = M * (pos, 1) as in evaluate, s = c.xyz / c.w, s = s*0.5 + 0.5,
//              texel (floor(s.x*N), floor(s.y*N)) -- nearest filtering; outside
//              the map the border value 1.0 (src/ShadowMap.cpp:3-9) -- and
//              vis = (d < s.z) ? 0 : 1
//   colour   = ((0.15 + diffuse*vis) * albedo.rgb, albedo.a)
#include "common.cuh"

namespace cpvs {
namespace {

constexpr uint32_t kShadeThreads = 256;

struct ShadeArgs {
    float m[16];  // light view-projection, column-major
    float l[3];   // light direction as given
    const float* nrm;
    uint32_t fpn;  // floats per normal pixel
    const float* alb;
    const uint8_t* vis;
    const float* pos;
    uint32_t fpp;  // floats per position pixel
    const float* sm;
    uint32_t sm_n;
    float* out;
    uint64_t n;
};

__device__ __forceinline__ float shadow_map_test(const ShadeArgs& a, float x, float y, float z) {
    float c[4];
#pragma unroll
    for (int r = 0; r < 4; ++r)
        c[r] = __fadd_rn(__fadd_rn(__fadd_rn(__fmul_rn(a.m[r], x), __fmul_rn(a.m[4 + r], y)), __fmul_rn(a.m[8 + r], z)),
                         a.m[12 + r]);
    const float sx = __fadd_rn(__fmul_rn(__fdiv_rn(c[0], c[3]), 0.5f), 0.5f);
    const float sy = __fadd_rn(__fmul_rn(__fdiv_rn(c[1], c[3]), 0.5f), 0.5f);
    const float sz = __fadd_rn(__fmul_rn(__fdiv_rn(c[2], c[3]), 0.5f), 0.5f);
    const float side = __uint2float_rn(a.sm_n);
    const float fx = floorf(__fmul_rn(sx, side)), fy = floorf(__fmul_rn(sy, side));
    float d = 1.0f;  // border colour
    if (fx >= 0.f && fx < side && fy >= 0.f && fy < side)
        d = __ldg(a.sm + (size_t)__float2uint_rz(fy) * a.sm_n + __float2uint_rz(fx));
    return (d < sz) ? 0.f : 1.f;
}

// V4: normals (and positions, when read) are 4 floats per pixel and every
// pixel buffer is 16-byte aligned, so each pixel is one vector load per
// buffer and one vector store.
template <bool V4>
__global__ void __launch_bounds__(kShadeThreads) k_shade(ShadeArgs a) {
    const uint64_t i = (uint64_t)blockIdx.x * kShadeThreads + threadIdx.x;
    if (i >= a.n) return;
    const float len =
        __fsqrt_rn(__fadd_rn(__fadd_rn(__fmul_rn(a.l[0], a.l[0]), __fmul_rn(a.l[1], a.l[1])), __fmul_rn(a.l[2], a.l[2])));
    const float lx = __fdiv_rn(a.l[0], len), ly = __fdiv_rn(a.l[1], len), lz = __fdiv_rn(a.l[2], len);
    float nx, ny, nz;
    float4 alb;
    if (V4) {
        const float4 nv = __ldcs(reinterpret_cast<const float4*>(a.nrm) + i);
        nx = nv.x;
        ny = nv.y;
        nz = nv.z;
        alb = __ldcs(reinterpret_cast<const float4*>(a.alb) + i);
    } else {
        const float* p = a.nrm + (size_t)a.fpn * i;
        nx = __ldcs(p);
        ny = __ldcs(p + 1);
        nz = __ldcs(p + 2);
        const float* q = a.alb + 4 * i;
        alb = make_float4(__ldcs(q), __ldcs(q + 1), __ldcs(q + 2), __ldcs(q + 3));
    }
    float vis;
    if (a.vis) {
        vis = fmaxf(__fdiv_rn(__uint2float_rn(__ldcs(a.vis + i)), 255.f), 0.f);
    } else {
        float x, y, z;
        if (V4) {
            const float4 pv = __ldcs(reinterpret_cast<const float4*>(a.pos) + i);
            x = pv.x;
            y = pv.y;
            z = pv.z;
        } else {
            const float* p = a.pos + (size_t)a.fpp * i;
            x = __ldcs(p);
            y = __ldcs(p + 1);
            z = __ldcs(p + 2);
        }
        vis = shadow_map_test(a, x, y, z);
    }
    const float dot = __fadd_rn(__fadd_rn(__fmul_rn(nx, lx), __fmul_rn(ny, ly)), __fmul_rn(nz, lz));
    const float diffuse = dot > 0.f ? dot : 0.f;
    const float s = __fadd_rn(0.15f, __fmul_rn(diffuse, vis));
    const float4 o = make_float4(__fmul_rn(s, alb.x), __fmul_rn(s, alb.y), __fmul_rn(s, alb.z), alb.w);
    if (V4)
        __stcs(reinterpret_cast<float4*>(a.out) + i, o);
    else {
        float* q = a.out + 4 * i;
        __stcs(q, o.x);
        __stcs(q + 1, o.y);
        __stcs(q + 2, o.z);
        __stcs(q + 3, o.w);
    }
}

bool aligned16(const void* p) { return ((uintptr_t)p & 15u) == 0; }

}  // namespace

cpvs_status launch_shade(uint64_t n, const float* normals, uint32_t normal_floats, const float* albedo,
                         const uint8_t* visibilities, const float* positions, uint32_t position_floats,
                         const float* shadow_map, uint32_t shadow_map_side, const float* light_view_proj,
                         const float* light_direction, float* out, cudaStream_t st, Timing* timing) {
    if (n == 0) return CPVS_OK;
    KernelTimer kt(timing, K_SHADE, st);
    ShadeArgs a{};
    for (int k = 0; k < 16; ++k) a.m[k] = light_view_proj ? light_view_proj[k] : 0.f;
    for (int k = 0; k < 3; ++k) a.l[k] = light_direction[k];
    a.nrm = normals;
    a.fpn = normal_floats;
    a.alb = albedo;
    a.vis = visibilities;
    a.pos = positions;
    a.fpp = position_floats;
    a.sm = shadow_map;
    a.sm_n = shadow_map_side;
    a.out = out;
    a.n = n;
    const bool v4 = normal_floats == 4 && aligned16(normals) && aligned16(albedo) && aligned16(out) &&
                    (visibilities || (position_floats == 4 && aligned16(positions)));
    const uint64_t blocks = (n + kShadeThreads - 1) / kShadeThreads;
    if (blocks > 0x7FFFFFFFull) return fail(CPVS_ERR_INVALID_ARG, "shade: image too large");
    if (v4)
        k_shade<true><<<(uint32_t)blocks, kShadeThreads, 0, st>>>(a);
    else
        k_shade<false><<<(uint32_t)blocks, kShadeThreads, 0, st>>>(a);
    CPVS_CUDA(cudaGetLastError());
    return CPVS_OK;
}

}  // namespace cpvs
