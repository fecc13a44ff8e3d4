// pbd_device.cuh -- device-side parameter block and the per-pair arithmetic of the step.
//
// Everything here restates the reference's device helpers in our own code:
//   Morton hashing          kernel/Hash.h:10-34
//   poly6 / spiky kernels   kernel/Density.h:14-42
//   wall confinement        kernel/Forces.h:19-59
// The parameter block replaces `__constant__ SimulationParameters params`
// (kernel/Globals.h:50-77): it is passed by value to every kernel (kernel parameters live
// in the constant bank), so separate simulations never share a global.
#pragma once
#include <cstdint>
#include <cuda_runtime.h>

namespace pbd {

constexpr uint32_t kEmptyCell = 0xFFFFFFFFu;   // UINT_MAX start = empty cell (SortReorder.h:146)

// Per-scene values of the batched form (one simulation holding many independent scenes).
struct SceneParams {
    float rho0;            // Density.restDensity of this scene
    float gravity;         // Forces.gravity of this scene
    float bmin[3], bmax[3];
    uint32_t base;         // first entry of the scene's slice of the cell tables
    uint32_t cells;        // the slice's size: the Morton cube (power-of-two side) that holds its walls
};

struct DevParams {
    uint32_t N;            // numberOfParticles this frame
    uint32_t G;            // maxGrid (cells addressable by the tables)
    uint32_t M;            // maxNeighboursPerParticle (list cap)
    uint32_t K;            // kernelWidthNeighbours (cell shells)
    uint32_t active;       // PBD_ACTIVE_* bits
    uint32_t flags;        // PBD_FLAG_* bits
    int32_t  n_scorr;
    uint32_t far_pairs_zero;  // 1 when pairs beyond every kernel support contribute exactly 0
    float d;               // particleDiameter = 2 r
    float dt, gravity;
    float inv_dt;          // 1 / dt: v = (p - x) / dt as a multiply (Update.h:22)
    float rho0;
    float hs, hp;          // spiky width (x diameter already applied), poly width
    float hp2;             // hp*hp
    float hp_lim;          // hp - 0.001 (poly6's upper bound, Density.h:19)
    float k_scorr;
    float c_visc, e_vort;
    float stiffness, one_minus_stiffness;
    float pos_damp, vel_damp;
    float lambda_eps;
    float bmin[3], bmax[3];
    float poly_inv_den;    // 1 / (0.001 + 64 pi hp^9)   (Density.h:21, double there)
    float spiky_den;       // pi * hs^6                  (Density.h:37)
    float wq;              // poly6(q), the s_corr reference value (Density.h:138)
    float inv_wq;          // 1 / wq
    float inv_spiky_den;   // 1 / spiky_den
    float cut2;            // max(hp, hs, d)^2: beyond it no kernel and no contact is non-zero
    // batched form: scene of each particle (sorted order), each scene's [start, end) in the sorted
    // arrays and its parameters; cells of scene s live at s * G + morton in the tables
    uint32_t batched;
    uint32_t nscenes;
    uint32_t table_size;   // cells in the tables: G, or nscenes * G in the batched form
    const SceneParams* scenes;
    uint32_t* scene_of;
    uint32_t* scene_range;
    // an adjoint's taped frame: the vorticity pass also stores each particle's eta (its
    // sum_j |omega_j - omega_i| / (p_j - p_i + 1e-8)) here; null in every other frame
    float4* eta_tape;
};

// The scene a particle belongs to, as the walk and the per-scene constants see it.
struct SceneCtx {
    uint32_t base;   // first table entry of the scene's cells
    uint32_t end;    // one past the scene's last particle in the sorted arrays
    uint32_t n;      // particles in the scene (the reference's numberOfParticles)
    float rho0;
    uint32_t cells;  // cells of the scene's slice (Morton keys below it are in the tables)
};

__device__ __forceinline__ SceneCtx scene_ctx(const DevParams& P, uint32_t i) {
    if (!P.batched) return SceneCtx{0u, P.N, P.N, P.rho0, P.G};
    const uint32_t sc = P.scene_of[i];
    const uint32_t s = P.scene_range[2 * sc], e = P.scene_range[2 * sc + 1];
    return SceneCtx{P.scenes[sc].base, e, e - s, P.scenes[sc].rho0, P.scenes[sc].cells};
}

// The scene whose slice holds table entry `key` (slices are in scene order): binary search.
__device__ __forceinline__ uint32_t scene_of_key(const DevParams& P, uint32_t key) {
    uint32_t lo = 0, hi = P.nscenes;
    while (hi - lo > 1) {
        const uint32_t mid = (lo + hi) >> 1;
        if (P.scenes[mid].base <= key) lo = mid; else hi = mid;
    }
    return lo;
}

// ---------------------------------------------------------------- Morton (Hash.h) -----
__device__ __forceinline__ uint32_t expand_bits(uint32_t v) {
    v = (v * 0x00010001u) & 0xFF0000FFu;
    v = (v * 0x00000101u) & 0x0F00F00Fu;
    v = (v * 0x00000011u) & 0xC30C30C3u;
    v = (v * 0x00000005u) & 0x49249249u;
    return v;
}

// Per-axis part of mortonCode: clamp to [0, 1023], truncate, spread.
__device__ __forceinline__ uint32_t morton_axis(float c) {
    c = fminf(fmaxf(c, 0.0f), 1023.0f);
    return expand_bits((uint32_t)c);
}

__device__ __forceinline__ uint32_t morton(float x, float y, float z) {
    return (morton_axis(x) << 2) + (morton_axis(y) << 1) + morton_axis(z);
}

// |r|^2 over xyz with explicit rounding: x*x, then + y*y and + z*z as fused multiply-adds, in that
// order.  The compiler may contract a plain x*x + y*y + z*z differently from one kernel to
// another; this spelling gives every walker (cells, lists, staged copies) the same bits.
__device__ __forceinline__ float dist2(float rx, float ry, float rz) {
    return __fmaf_rn(rz, rz, __fmaf_rn(ry, ry, __fmul_rn(rx, rx)));
}

// ---------------------------------------------------------- pair kernels (Density.h) --
// poly6Viscosity: W = 315 t^3 t^3 / den, t = hp^2 - d^2, for 0.001 < d < hp - 0.001.
__device__ __forceinline__ float poly6(const DevParams& P, float dist) {
    if (dist > 0.001f && dist < P.hp_lim) {
        float t = __fsub_rn(P.hp2, __fmul_rn(dist, dist));
        float t3 = t * t * t;
        return (315.0f * t3 * t3) * P.poly_inv_den;
    }
    return 0.0f;
}

// Scalar part of spiky: 15 (hs - d)^2 / (pi hs^6) / |r|_4, so that grad = s * r (r = pi - pj,
// normalised over all four lanes as the float4 normalize of the reference does).
__device__ __forceinline__ float spiky_scale(const DevParams& P, float dist, float r2w) {
    if (dist > 0.0001f && (P.hs - dist) > 0.0001f) {
        float a = P.hs - dist;
        return 15.0f * (a * a * P.inv_spiky_den) * rsqrtf(r2w);
    }
    return 0.0f;
}

// Integer power by repeated multiplication (the reference's pow(float, int)): r = 1, then
// r *= x |n| times.  The usual exponents are spelled out with the same products in the same
// order (1 * x = x exactly), without the loop.
__device__ __forceinline__ float powi(float x, int n) {
    if (n == 4) return ((x * x) * x) * x;   // config.txt's nSCorr: one test before the others
    switch (n) {
        case 0: return 1.0f;
        case 1: return x;
        case 2: return x * x;
        case 3: return (x * x) * x;
        case 4: return ((x * x) * x) * x;
        default: break;
    }
    int m = n < 0 ? -n : n;
    float r = 1.0f;
    for (int k = 0; k < m; ++k) r *= x;
    return n < 0 ? 1.0f / r : r;
}

}  // namespace pbd
