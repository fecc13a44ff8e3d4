// pbd_sprites.cuh -- headless particle sprites (src/app/rendering/shader/particles/
// particleSpriteGeom.{vert,geom,frag}, drawn by Particles.cc:234-284), as CUDA splatting.
//
// One thread per particle: the sprite's quad (half-size sphere_radius around view * position,
// facing the camera) maps to an axis-aligned window rectangle, because all its corners share one
// view depth; uv is affine in window coordinates; a pixel is covered when its centre lies in
// [x0, x1) x [y0, y1).  Each covered pixel inside the unit disc is shaded as the fragment shader
// does and offers the key (depth bits << 32 | RGBA8) to the pixel with atomicMin: the nearest
// fragment wins (ties: the smaller colour).  Every floating-point operation is an explicit
// correctly rounded one in a fixed order (the _rn intrinsics), the same order as the oracle's
// orc_render_sprites, so both give the same bits; pow(x, 1/6) is a 32-step bisection on [0, 1]
// and pow(s, 10) repeated squaring.
#pragma once
#include <cstdint>
#include <cuda_runtime.h>
#include "../../include/pbd.h"

namespace pbd {

#define FA __fadd_rn
#define FS __fsub_rn
#define FM __fmul_rn
#define FD __fdiv_rn

struct SpriteCam {
    float V[16], Pm[16];
    float vd[3];               // -view_direction (normalised in the kernel)
    float light[3];
    float r;
    uint32_t W, H;
};

__device__ __forceinline__ float spr_root6(float x) {
    if (!(x > 0.0f)) return 0.0f;
    if (x >= 1.0f) return 1.0f;
    float lo = 0.0f, hi = 1.0f;
#pragma unroll 1
    for (int k = 0; k < 32; ++k) {
        const float m = FM(FA(lo, hi), 0.5f);
        const float m2 = FM(m, m);
        const float m6 = FM(FM(m2, m2), m2);
        if (m6 < x) lo = m; else hi = m;
    }
    return lo;
}

// column-major 4x4 times (x, y, z, w): ((m0 x + m4 y) + m8 z) + m12 w per row
__device__ __forceinline__ void spr_mat4(const float* m, float x, float y, float z, float w, float* o) {
#pragma unroll
    for (int r = 0; r < 4; ++r) o[r] = FA(FA(FA(FM(m[r], x), FM(m[4 + r], y)), FM(m[8 + r], z)), FM(m[12 + r], w));
}

__device__ __forceinline__ void spr_normalize3(float* v) {
    const float l = __fsqrt_rn(FA(FA(FM(v[0], v[0]), FM(v[1], v[1])), FM(v[2], v[2])));
    v[0] = FD(v[0], l);
    v[1] = FD(v[1], l);
    v[2] = FD(v[2], l);
}

__device__ __forceinline__ uint32_t spr_unorm8(float c) {
    c = c < 0.0f ? 0.0f : (c > 1.0f ? 1.0f : c);
    return (uint32_t)floorf(FA(FM(c, 255.0f), 0.5f));
}

// every pixel: depth 1 and the clear colour
__global__ void sprite_clear_kernel(unsigned long long* key, size_t n, float4 clear) {
    const uint32_t c = spr_unorm8(clear.x) | (spr_unorm8(clear.y) << 8) | (spr_unorm8(clear.z) << 16) |
                       (spr_unorm8(clear.w) << 24);
    const unsigned long long value = ((unsigned long long)__float_as_uint(1.0f) << 32) | c;
    for (size_t q = (size_t)blockIdx.x * blockDim.x + threadIdx.x; q < n; q += (size_t)gridDim.x * blockDim.x) key[q] = value;
}

__global__ void __launch_bounds__(256)
sprite_splat_kernel(SpriteCam cam, const float4* __restrict__ pos, const float4* __restrict__ col, uint32_t n,
                    unsigned long long* __restrict__ key) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const float4 pp = pos[i];
    float vd[3] = {cam.vd[0], cam.vd[1], cam.vd[2]};
    spr_normalize3(vd);
    const float t = spr_root6(col ? col[i].x : 0.0f);
    const float omt = FS(1.0f, t);
    const float c[3] = {FA(FM(0.95f, omt), FM(0.0f, t)), FA(FM(0.97f, omt), FM(0.0f, t)), FA(FM(0.97f, omt), FM(1.0f, t))};
    float L[3] = {FS(cam.light[0], pp.x), FS(cam.light[1], pp.y), FS(cam.light[2], pp.z)};
    spr_normalize3(L);
    float vp[4], lo[4], hi[4];
    spr_mat4(cam.V, pp.x, pp.y, pp.z, 1.0f, vp);
    spr_mat4(cam.Pm, FS(vp[0], cam.r), FS(vp[1], cam.r), vp[2], vp[3], lo);
    spr_mat4(cam.Pm, FA(vp[0], cam.r), FA(vp[1], cam.r), vp[2], vp[3], hi);
    if (!(lo[3] > 0.0f)) return;                                   // behind the eye
    const float zn = FD(lo[2], lo[3]);
    if (zn < -1.0f || zn > 1.0f) return;                           // outside the near / far planes
    const float Wf = (float)cam.W, Hf = (float)cam.H;
    const float x0 = FM(FA(FM(FD(lo[0], lo[3]), 0.5f), 0.5f), Wf), y0 = FM(FA(FM(FD(lo[1], lo[3]), 0.5f), 0.5f), Hf);
    const float x1 = FM(FA(FM(FD(hi[0], hi[3]), 0.5f), 0.5f), Wf), y1 = FM(FA(FM(FD(hi[1], hi[3]), 0.5f), 0.5f), Hf);
    if (!(x1 > x0) || !(y1 > y0)) return;
    long ix0 = (long)ceilf(FS(x0, 0.5f)), ix1 = (long)ceilf(FS(x1, 0.5f));
    long iy0 = (long)ceilf(FS(y0, 0.5f)), iy1 = (long)ceilf(FS(y1, 0.5f));
    if (ix0 < 0) ix0 = 0;
    if (iy0 < 0) iy0 = 0;
    if (ix1 > (long)cam.W) ix1 = (long)cam.W;
    if (iy1 > (long)cam.H) iy1 = (long)cam.H;
    const float sx = FD(2.0f, FS(x1, x0)), sy = FD(2.0f, FS(y1, y0));
#pragma unroll 1
    for (long iy = iy0; iy < iy1; ++iy) {
        const float v = FS(FM(FS(FA((float)iy, 0.5f), y0), sy), 1.0f);
#pragma unroll 1
        for (long ix = ix0; ix < ix1; ++ix) {
            const float u = FS(FM(FS(FA((float)ix, 0.5f), x0), sx), 1.0f);
            const float mag = FA(FM(u, u), FM(v, v));
            if (mag > 1.0f) continue;
            const float nz = __fsqrt_rn(FS(1.0f, mag));
            float dp[4];
            spr_mat4(cam.Pm, vp[0], vp[1], FA(vp[2], FM(cam.r, nz)), vp[3], dp);
            float dz = FA(FM(0.5f, FD(dp[2], dp[3])), 0.5f);
            if (dz < 0.0f) dz = 0.0f;
            if (!(dz < 1.0f)) continue;                             // GL_LESS against the cleared 1
            const size_t q = (size_t)iy * cam.W + (size_t)ix;
            const unsigned long long dkey = (unsigned long long)__float_as_uint(dz) << 32;
            if (dkey > *((volatile unsigned long long*)(key + q))) continue;   // a nearer fragment is there
            // inverse of the view rotation = its transpose: N_world[k] = sum_r V[4k + r] N[r]
            float N[3];
#pragma unroll
            for (int k = 0; k < 3; ++k) N[k] = FA(FA(FM(cam.V[4 * k], u), FM(cam.V[4 * k + 1], v)), FM(cam.V[4 * k + 2], nz));
            spr_normalize3(N);
            const float ln = FA(FA(FM(L[0], N[0]), FM(L[1], N[1])), FM(L[2], N[2]));
            float R[3];
#pragma unroll
            for (int k = 0; k < 3; ++k) R[k] = FA(-L[k], FM(FM(2.0f, ln), N[k]));
            float rv = FA(FA(FM(R[0], vd[0]), FM(R[1], vd[1])), FM(R[2], vd[2]));
            rv = rv < 0.0f ? 0.0f : (rv > 1.0f ? 1.0f : rv);
            const float s2 = FM(rv, rv), s4 = FM(s2, s2), s8 = FM(s4, s4), s10 = FM(s8, s2);
            const float diff = ln > 0.0f ? ln : 0.0f;
            uint32_t cc = 0;
#pragma unroll
            for (int k = 0; k < 3; ++k) {
                const float f = FA(FA(FM(0.3f, c[k]), FM(FM(0.7f, diff), c[k])), FM(FM(0.2f, s10), 1.0f));
                cc |= spr_unorm8(f) << (8 * k);
            }
            cc |= 255u << 24;
            atomicMin(key + q, dkey | cc);
        }
    }
}

// keys -> RGBA8 rows top-down and depth
__global__ void sprite_resolve_kernel(const unsigned long long* __restrict__ key, uint32_t W, uint32_t H,
                                      uint32_t* __restrict__ rgba, float* __restrict__ depth) {
    const size_t q = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (q >= (size_t)W * H) return;
    const uint32_t y = (uint32_t)(q / W), x = (uint32_t)(q - (size_t)y * W);
    const unsigned long long k = key[q];
    const size_t o = (size_t)(H - 1 - y) * W + x;
    if (rgba) rgba[o] = (uint32_t)k;
    if (depth) depth[o] = __uint_as_float((uint32_t)(k >> 32));
}

#undef FA
#undef FS
#undef FM
#undef FD

}  // namespace pbd
