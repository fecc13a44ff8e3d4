// pbd_adjoint.cuh -- reverse-mode kernels of the frame (no counterpart in the reference).
//
// The frame's map (x, v) -> (x', v') with the neighbour list, the sort permutation and the wall
// clamps held fixed (they are piecewise constant in the inputs):
//   predict   p = x + (v + g dt + f dt) dt, clamped per component to the walls   (Forces.h:65-101)
//   reorder   gather by the permutation                                           (SortReorder.h:86-115)
//   I times   lambda_i = -(rho_i/rho0 - 1) / (B_i + |S_i|^2/rho0 + eps)             (Density.h:48-93)
//             Delta_i = (1/rho0) sum_j (lambda_i + lambda_j + s_corr_ij) G_ij        (Density.h:104-145)
//             c_i = sum_contacts s_ij (1 - stiffness) (d - |r|) r_hat             (Collision.h:171-242)
//             p <- p + c - w_i Delta ;  x <- x + c
//   update    v' = (p - x)/dt ; x' = p                                              (Update.h:11-32)
//   viscosity v'' = v' + c w_i sum_j (v'_j - v'_i) W(|p_i - p_j|), when active       (Density.h:280-310)
// with r = p_i - p_j, G = spiky gradient g(|r|) r_hat, W = poly6, w_i the inverse mass (1 without
// solids; a solid's 0 holds it still) and s_ij = w_i / (w_i + w_j) its share of a contact's
// overlap (1/2 with unit masses, Collision.h:223-225).  The reverse passes scatter the
// pair terms to the partner with atomic adds (so the neighbour relation need not be symmetric)
// in 64-bit fixed point, which is associative, so the gradients do not depend on the order in
// which the atomics land: a reverse pass gives the same bits every time.  The fixed point's scale
// is set per frame from the largest gradient entering the frame's reverse pass.  A particle's own
// terms are summed in its list's order; dL/drest_density and dL/deps are summed per block in
// double into the block's own slot (one block per slot per launch, launches in stream order) and
// the slots are added in index order at the end.
#pragma once
#include "pbd_passes.cuh"

namespace pbd {

// spiky magnitude g(L) = 15 (h - L)^2 / (pi h^6) and its derivative, inside the support
__device__ __forceinline__ void spiky_g(const DevParams& P, float L, float& g, float& dg) {
    if (L > 0.0001f && (P.hs - L) > 0.0001f) {
        const float a = P.hs - L;
        const float k = 15.0f * P.inv_spiky_den;
        g = k * a * a;
        dg = -2.0f * k * a;
    } else {
        g = 0.0f;
        dg = 0.0f;
    }
}

// poly6 W(L) = 315 (hp^2 - L^2)^6 / den and dW/dL, inside the support
__device__ __forceinline__ void poly6_w(const DevParams& P, float L, float& W, float& dW) {
    if (L > 0.001f && L < P.hp - 0.001f) {
        const float t = P.hp2 - L * L;
        const float t2 = t * t, t5 = t2 * t2 * t;
        W = 315.0f * t5 * t * P.poly_inv_den;
        dW = -12.0f * L * 315.0f * t5 * P.poly_inv_den;
    } else {
        W = 0.0f;
        dW = 0.0f;
    }
}

// H v for H = dG/dr = dg rhat rhat^T + (g/L)(I - rhat rhat^T)
__device__ __forceinline__ float3 spiky_hess_mul(float g, float dg, float L, float3 rh, float3 v) {
    const float rv = rh.x * v.x + rh.y * v.y + rh.z * v.z;
    const float gl = g / L;
    return make_float3(dg * rv * rh.x + gl * (v.x - rv * rh.x), dg * rv * rh.y + gl * (v.y - rv * rh.y),
                       dg * rv * rh.z + gl * (v.z - rv * rh.z));
}

// Fixed point of the scattered terms, scaled per frame: the frame's reverse pass starts with
// adj_gmax_kernel, which takes the largest |dL/dx'| + |dL/dv'|/dt over the particles (m < 2^e);
// every scatter and take of that frame then uses the scale 2^(40 - e).  A term of magnitude a
// keeps a - 2^(e-41) of its value (relative 2^-41 of the frame's largest gradient), and the
// sums stay below 2^62 while no particle's scattered terms exceed 2^22 times that gradient.
// A fixed scale cannot serve both a loss averaged over a million particles (terms ~1e-7) and
// a summed one that has grown over many frames.
struct FixScale { float sc, inv; };
__device__ __forceinline__ FixScale fix_scale(const uint32_t* __restrict__ gmax) {
    const uint32_t be = (*gmax >> 23) & 0xFFu;                 // biased exponent of the largest gradient
    int s = (be == 0xFFu) ? 0 : 40 - ((int)be - 126);           // m < 2^(be - 126); inf/NaN: scale 1
    s = max(-120, min(120, s));
    return FixScale{__int_as_float((s + 127) << 23), __int_as_float((127 - s) << 23)};
}
__device__ __forceinline__ void fix_add(unsigned long long* a, float v, float sc) {
    atomicAdd(a, (unsigned long long)__float2ll_rn(v * sc));
}
__device__ __forceinline__ void scatter_sub3(unsigned long long* sj, float3 v, float sc) {
    fix_add(sj + 0, -v.x, sc);
    fix_add(sj + 1, -v.y, sc);
    fix_add(sj + 2, -v.z, sc);
}
// Particle i's scattered terms as floats; the slot is cleared for the next pass.
__device__ __forceinline__ float4 take_scattered(unsigned long long* scat, uint32_t i, float inv) {
    unsigned long long* s = scat + 4 * (size_t)i;
    const float4 r = make_float4(__ll2float_rn((long long)s[0]) * inv, __ll2float_rn((long long)s[1]) * inv,
                                 __ll2float_rn((long long)s[2]) * inv, __ll2float_rn((long long)s[3]) * inv);
    s[0] = s[1] = s[2] = s[3] = 0ull;
    return r;
}

// Block-reduce two doubles (in a fixed order) and add them to this block's slots acc[2b], acc[2b+1]:
// a launch has one block per slot and the launches run in stream order, so no atomics are needed
// and the sums do not depend on scheduling.
__device__ __forceinline__ void block_add2(double a, double b, double* acc) {
    __shared__ double sa[32], sb[32];
    for (int o = 16; o > 0; o >>= 1) {
        a += __shfl_down_sync(0xffffffffu, a, o);
        b += __shfl_down_sync(0xffffffffu, b, o);
    }
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    if (lane == 0) { sa[warp] = a; sb[warp] = b; }
    __syncthreads();
    if (threadIdx.x == 0) {
        double ta = 0.0, tb = 0.0;
        for (int w = 0; w < (int)(blockDim.x + 31) / 32; ++w) { ta += sa[w]; tb += sb[w]; }
        acc[2 * (size_t)blockIdx.x] += ta;
        acc[2 * (size_t)blockIdx.x + 1] += tb;
    }
}

__device__ __forceinline__ void scatter_add3(unsigned long long* sj, float3 v, float sc) {
    fix_add(sj + 0, v.x, sc);
    fix_add(sj + 1, v.y, sc);
    fix_add(sj + 2, v.z, sc);
}

// The largest |dL/dx'| + |dL/dv'|/dt entering a frame's reverse pass (non-negative floats order
// as their bit patterns), for fix_scale.  *gmax is zeroed before the launch.
__global__ void adj_gmax_kernel(const DevParams P, const float4* __restrict__ gx_out, const float4* __restrict__ gv_out,
                                uint32_t* __restrict__ gmax) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    float m = 0.0f;
    if (i < P.N) {
        const float4 a = gx_out[i], b = gv_out[i];
        const float r = P.inv_dt;
        m = fmaxf(fmaxf(fabsf(a.x) + fabsf(b.x) * r, fabsf(a.y) + fabsf(b.y) * r), fabsf(a.z) + fabsf(b.z) * r);
    }
    for (int o = 16; o > 0; o >>= 1) m = fmaxf(m, __shfl_down_sync(0xffffffffu, m, o));
    if ((threadIdx.x & 31) == 0 && m > 0.0f) atomicMax(gmax, __float_as_uint(m));
}

// XSPH viscosity backward (Density.h:280-310, Jacobi), the frame's last pass:
//   v'_i = v_i + c sum_j (v_j - v_i) W(|p_i - p_j|)   at the frame's final positions p
// vbar_i = v'bar_i (1 - c sum_j W_ij) + sum over the lists holding i of c W v'bar (scattered);
// pbar_i += sum_j c (v'bar_i . (v_j - v_i)) dW/dL rhat, pbar_j -= the same (scattered).
struct AdjViscVisit {
    struct Contrib { int dummy; };
    using Extra = float4;   // v_j before the viscosity
    const DevParams& P;
    const float4* __restrict__ vu;
    float4 pi, vi;
    float3 gvo;        // dL/dv'_i
    float c;
    unsigned long long* scat_p;   // partners' dL/dp terms (fixed point)
    unsigned long long* scat_v;   // partners' dL/dv terms (fixed point)
    float fix;                    // the frame's fixed-point scale
    float sumw;
    float3 gpi;
    __device__ __forceinline__ void end_contacts(uint32_t) {}
    __device__ static Contrib zero() { return Contrib{0}; }
    __device__ static bool effective(const Contrib&) { return false; }
    __device__ static Contrib shfl(const Contrib& c, int) { return c; }
    __device__ __forceinline__ float4 fetch(uint32_t j) const { return __ldg(vu + j); }
    __device__ __forceinline__ Contrib contrib(uint32_t j, const float4& pj, const float4& vj, bool) {
        const float rx = pi.x - pj.x, ry = pi.y - pj.y, rz = pi.z - pj.z;
        const float r2 = dist2(rx, ry, rz);
        if (r2 >= P.hp2 || r2 <= 0.0f) return zero();
        const float L = sqrtf(r2);
        float W, dW;
        poly6_w(P, L, W, dW);
        if (W == 0.0f && dW == 0.0f) return zero();
        sumw += W;
        const float cw = c * W;
        scatter_add3(scat_v + 4 * (size_t)j, make_float3(cw * gvo.x, cw * gvo.y, cw * gvo.z), fix);
        const float term = c * (gvo.x * (vj.x - vi.x) + gvo.y * (vj.y - vi.y) + gvo.z * (vj.z - vi.z)) * dW / L;
        const float3 t3 = make_float3(term * rx, term * ry, term * rz);
        gpi.x += t3.x; gpi.y += t3.y; gpi.z += t3.z;
        scatter_sub3(scat_p + 4 * (size_t)j, t3, fix);
        return zero();
    }
    __device__ __forceinline__ void add(const Contrib&, bool) {}
};

// Vorticity confinement backward (Density.h:179-221).  The frame's force f_i = e (n_i x omega_i)
// acts in the next frame's applyForces (v* = v + dt (g + f), not on solids), so dL/df_i = dt
// dL/dv_i of the next frame's input, which the next frame's reverse pass left in gv_out.  With
// eta_i = sum_j |omega_j - omega_i| / (p_j - p_i + 1e-8) (componentwise, every list entry; the
// taped frame kept it) and n = (eta + 1e-8) / (|eta| + 1e-8):
//   nbar = e omega_i x fbar,  omegabar_i = e fbar x n,
//   etabar = nbar / (|eta| + 1e-8) - eta ((eta + 1e-8) . nbar) / ((|eta| + 1e-8)^2 |eta|),
// and per entry, with D = p_j - p_i + 1e-8, u = omega_j - omega_i, l = |u|:
//   omegabar_j += (sum_a etabar_a / D_a) u / l (omegabar_i the opposite),
//   pbar_j,a -= etabar_a l / D_a^2 (pbar_i,a the opposite).
struct AdjVortVisit {   // the entries' terms for etabar
    struct Contrib { int dummy; };
    using Extra = float4;   // omega_j
    const float4* __restrict__ om;
    float4 pi, oi;
    float3 eb;          // etabar_i
    unsigned long long* scat_om;
    unsigned long long* scat_p;
    float fix;
    float3 obi = make_float3(0.f, 0.f, 0.f), pbi = make_float3(0.f, 0.f, 0.f);
    __device__ __forceinline__ void end_contacts(uint32_t) {}
    __device__ static Contrib zero() { return Contrib{0}; }
    __device__ static bool effective(const Contrib&) { return false; }
    __device__ static Contrib shfl(const Contrib& c, int) { return c; }
    __device__ __forceinline__ float4 fetch(uint32_t j) const { return __ldg(om + j); }
    __device__ __forceinline__ Contrib contrib(uint32_t j, const float4& pj, const float4& oj, bool) {
        const float ux = oj.x - oi.x, uy = oj.y - oi.y, uz = oj.z - oi.z;
        const float ol = sqrtf(dist2(ux, uy, uz));
        const float Dx = (pj.x - pi.x) + 0.00000001f, Dy = (pj.y - pi.y) + 0.00000001f, Dz = (pj.z - pi.z) + 0.00000001f;
        const float ix = 1.0f / Dx, iy = 1.0f / Dy, iz = 1.0f / Dz;
        if (ol > 0.0f) {
            const float sq = (eb.x * ix + eb.y * iy + eb.z * iz) / ol;
            const float3 du = make_float3(sq * ux, sq * uy, sq * uz);
            scatter_add3(scat_om + 4 * (size_t)j, du, fix);
            obi.x -= du.x; obi.y -= du.y; obi.z -= du.z;
        }
        const float3 tp = make_float3(-eb.x * ol * ix * ix, -eb.y * ol * iy * iy, -eb.z * ol * iz * iz);
        scatter_add3(scat_p + 4 * (size_t)j, tp, fix);
        pbi.x -= tp.x; pbi.y -= tp.y; pbi.z -= tp.z;
        return zero();
    }
    __device__ __forceinline__ void add(const Contrib&, bool) {}
};

// Particle i's entries of the frame's list: from the full list the taped forward recorded (meta
// fm), or from the anchors' cells when it has none for i (a list longer than its slots, a walk
// that met a long cell range, or no list recorded).  The same entries either way.
template <class V>
__device__ __forceinline__ void walk_frame_list(const DevParams& P, const SceneCtx& S, uint32_t i, float4 anchor,
                                                const float4* __restrict__ p, const uint32_t* __restrict__ cs,
                                                const uint32_t* __restrict__ ce, const NbList& F, uint32_t fm, V& vis) {
    if (fm != kListOff) {
        walk_list(F, i, fm, p, vis);
    } else {
        bool deferred = false;
        walk_seq(P, S, i, anchor, p, cs, ce, vis, false, &deferred);
    }
}

// Both per-entry visitors in one walk, each with its own neighbour data.
template <class A, class B>
struct BothVisit {
    struct Contrib { int dummy; };
    struct Extra { typename ExtraOf<A>::type a; typename ExtraOf<B>::type b; };
    A& va;
    B& vb;
    __device__ __forceinline__ void end_contacts(uint32_t n) { va.end_contacts(n); vb.end_contacts(n); }
    __device__ static Contrib zero() { return Contrib{0}; }
    __device__ static bool effective(const Contrib&) { return false; }
    __device__ static Contrib shfl(const Contrib& c, int) { return c; }
    __device__ __forceinline__ Extra fetch(uint32_t j) const { return Extra{fetch_extra(va, j), fetch_extra(vb, j)}; }
    __device__ __forceinline__ Contrib contrib(uint32_t j, const float4& pj, const Extra& ex, bool contact) {
        contrib_of(va, j, pj, ex.a, contact);
        contrib_of(vb, j, pj, ex.b, contact);
        return zero();
    }
    __device__ __forceinline__ void add(const Contrib&, bool) {}
};

// The reverse of the passes after updatePositions, the viscosity's and the vorticity force's
// terms in one walk of the frame's list (the anchors' cells at the final positions):
//   gx = dL/dx' + their own dL/dp terms, gv_u = dL/dv before the viscosity (own terms),
//   gom = each particle's own dL/domega (vorticity);
// the partners' terms go to scat_p, scat_v and scat_om.  omega's own reverse runs after it.
__global__ void __launch_bounds__(128)
adj_visc_vort_kernel(DevParams P, const float4* __restrict__ pf, const float4* __restrict__ pa,
                     const float4* __restrict__ vu, const float4* __restrict__ om, const float4* __restrict__ eta,
                     const float4* __restrict__ gx_out, const float4* __restrict__ gv_out, const float* __restrict__ w,
                     float4* __restrict__ gx, float4* __restrict__ gv_u, float4* __restrict__ gom,
                     unsigned long long* __restrict__ scat_p, unsigned long long* __restrict__ scat_v,
                     unsigned long long* __restrict__ scat_om, const uint32_t* __restrict__ cs,
                     const uint32_t* __restrict__ ce, const uint32_t* __restrict__ gmax, int do_visc, int do_vort,
                     NbList Ft) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= P.N) return;
    const SceneCtx S = scene_ctx(P, i);
    const float fix = fix_scale(gmax).sc;
    const float4 g = gv_out[i], x0 = gx_out[i], pi = pf[i];
    // viscosity: v'' = v' + c w_i sum_j (v'_j - v'_i) W_ij
    const float ci = w ? w[i] * P.c_visc : P.c_visc;   // a solid's coefficient is 0
    AdjViscVisit vis{P, vu, pi, vu[i], make_float3(g.x, g.y, g.z), ci, scat_p, scat_v, fix, 0.f,
                     make_float3(0.f, 0.f, 0.f)};
    // vorticity: dL/df = dt dL/dv of the next frame (zero for the last frame and for solids)
    const float k = (w && w[i] == 0.0f) ? 0.0f : P.dt;
    const float3 fb = make_float3(g.x * k, g.y * k, g.z * k);
    const bool vort = do_vort && (fb.x != 0.0f || fb.y != 0.0f || fb.z != 0.0f);
    float3 ob = make_float3(0.f, 0.f, 0.f), eb = ob;
    float4 oi = make_float4(0.f, 0.f, 0.f, 0.f);
    if (vort) {
        oi = om[i];
        const float4 et = eta[i];
        const float e = P.e_vort, EPS = 0.00000001f;
        const float gl = sqrtf(et.x * et.x + et.y * et.y + et.z * et.z), ge = gl + EPS;
        const float3 nv = make_float3((et.x + EPS) / ge, (et.y + EPS) / ge, (et.z + EPS) / ge);
        const float3 nb = make_float3(e * (oi.y * fb.z - oi.z * fb.y), e * (oi.z * fb.x - oi.x * fb.z),
                                      e * (oi.x * fb.y - oi.y * fb.x));
        ob = make_float3(e * (fb.y * nv.z - fb.z * nv.y), e * (fb.z * nv.x - fb.x * nv.z), e * (fb.x * nv.y - fb.y * nv.x));
        const float c2 = gl > 0.0f ? ((et.x + EPS) * nb.x + (et.y + EPS) * nb.y + (et.z + EPS) * nb.z) / (ge * ge * gl) : 0.0f;
        eb = make_float3(nb.x / ge - et.x * c2, nb.y / ge - et.y * c2, nb.z / ge - et.z * c2);
    }
    AdjVortVisit vv{om, pi, oi, eb, scat_om, scat_p, fix};
    const uint32_t fm = Ft.list ? Ft.meta[i] : kListOff;   // the taped full list, else the cells
    if (do_visc && vort) {
        BothVisit<AdjViscVisit, AdjVortVisit> both{vis, vv};
        walk_frame_list(P, S, i, pa[i], pf, cs, ce, Ft, fm, both);
    } else if (do_visc) {
        walk_frame_list(P, S, i, pa[i], pf, cs, ce, Ft, fm, vis);
    } else if (vort) {
        walk_frame_list(P, S, i, pa[i], pf, cs, ce, Ft, fm, vv);
    }
    gx[i] = make_float4(x0.x + vis.gpi.x + vv.pbi.x, x0.y + vis.gpi.y + vv.pbi.y, x0.z + vis.gpi.z + vv.pbi.z, 0.f);
    const float kv = do_visc ? 1.0f - ci * vis.sumw : 1.0f;
    gv_u[i] = make_float4(g.x * kv, g.y * kv, g.z * kv, 0.f);
    if (do_vort) gom[i] = make_float4(ob.x + vv.obi.x, ob.y + vv.obi.y, ob.z + vv.obi.z, 0.f);
}

// computeOmega backward (Density.h:232-269): omega_i = sum_j (v_j - v_i) x G_ij, G = g(|r|) rhat,
// r = p_i - p_j (the pairs within the spiky support), at the final positions and the velocities
// before the viscosity.  With obar_i (own + partners'): vbar_j += G x obar_i (vbar_i the
// opposite), pbar_i += H (obar_i x (v_j - v_i)) (pbar_j the opposite), H = dG/dr.  Own terms go
// into gv_u and gx, partners' terms to scat_v and scat_p.
struct AdjOmegaVisit {
    struct Contrib { int dummy; };
    using Extra = float4;   // v_j
    const DevParams& P;
    const float4* __restrict__ vu;
    float4 pi, vi;
    float3 ob;
    unsigned long long* scat_v;
    unsigned long long* scat_p;
    float fix;
    float3 vbi = make_float3(0.f, 0.f, 0.f), pbi = make_float3(0.f, 0.f, 0.f);
    __device__ __forceinline__ void end_contacts(uint32_t) {}
    __device__ static Contrib zero() { return Contrib{0}; }
    __device__ static bool effective(const Contrib&) { return false; }
    __device__ static Contrib shfl(const Contrib& c, int) { return c; }
    __device__ __forceinline__ float4 fetch(uint32_t j) const { return __ldg(vu + j); }
    __device__ __forceinline__ Contrib contrib(uint32_t j, const float4& pj, const float4& vj, bool) {
        const float rx = pi.x - pj.x, ry = pi.y - pj.y, rz = pi.z - pj.z;
        const float r2 = dist2(rx, ry, rz);
        if (r2 >= P.cut2 || r2 <= 0.0f) return zero();
        const float L = sqrtf(r2);
        float g, dg;
        spiky_g(P, L, g, dg);
        if (g == 0.0f && dg == 0.0f) return zero();
        const float3 rh = make_float3(rx / L, ry / L, rz / L);
        const float3 G = make_float3(g * rh.x, g * rh.y, g * rh.z);
        const float3 gG = make_float3(G.y * ob.z - G.z * ob.y, G.z * ob.x - G.x * ob.z, G.x * ob.y - G.y * ob.x);
        scatter_add3(scat_v + 4 * (size_t)j, gG, fix);
        vbi.x -= gG.x; vbi.y -= gG.y; vbi.z -= gG.z;
        const float ux = vj.x - vi.x, uy = vj.y - vi.y, uz = vj.z - vi.z;
        const float3 ou = make_float3(ob.y * uz - ob.z * uy, ob.z * ux - ob.x * uz, ob.x * uy - ob.y * ux);
        const float3 rb = spiky_hess_mul(g, dg, L, rh, ou);
        pbi.x += rb.x; pbi.y += rb.y; pbi.z += rb.z;
        scatter_sub3(scat_p + 4 * (size_t)j, rb, fix);
        return zero();
    }
    __device__ __forceinline__ void add(const Contrib&, bool) {}
};

__global__ void __launch_bounds__(128)
adj_omega_kernel(DevParams P, const float4* __restrict__ pf, const float4* __restrict__ pa, const float4* __restrict__ vu,
                 const float4* __restrict__ gom, unsigned long long* __restrict__ scat_om, float4* __restrict__ gx,
                 float4* __restrict__ gv_u, unsigned long long* __restrict__ scat_v, unsigned long long* __restrict__ scat_p,
                 const uint32_t* __restrict__ cs, const uint32_t* __restrict__ ce, const uint32_t* __restrict__ gmax,
                 NbList Ft) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= P.N) return;
    const FixScale fs = fix_scale(gmax);
    const float4 t = take_scattered(scat_om, i, fs.inv), o0 = gom[i];
    const float3 ob = make_float3(o0.x + t.x, o0.y + t.y, o0.z + t.z);
    if (ob.x == 0.0f && ob.y == 0.0f && ob.z == 0.0f) return;
    const SceneCtx S = scene_ctx(P, i);
    AdjOmegaVisit vis{P, vu, pf[i], vu[i], ob, scat_v, scat_p, fs.sc};
    walk_frame_list(P, S, i, pa[i], pf, cs, ce, Ft, Ft.list ? Ft.meta[i] : kListOff, vis);
    const float4 a = gx[i], b = gv_u[i];
    gx[i] = make_float4(a.x + vis.pbi.x, a.y + vis.pbi.y, a.z + vis.pbi.z, 0.f);
    gv_u[i] = make_float4(b.x + vis.vbi.x, b.y + vis.vbi.y, b.z + vis.vbi.z, 0.f);
}

// update backward after the viscosity's: the partners' terms added to the own ones first
__global__ void adj_update_visc_kernel(const DevParams P, float4* __restrict__ gx_mod, const float4* __restrict__ gv_u,
                                       float4* __restrict__ gp, unsigned long long* __restrict__ scat_p,
                                       unsigned long long* __restrict__ scat_v, const uint32_t* __restrict__ gmax) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= P.N) return;
    const float inv = fix_scale(gmax).inv;
    const float4 tp = take_scattered(scat_p, i, inv), tv = take_scattered(scat_v, i, inv);
    const float4 a0 = gx_mod[i], b0 = gv_u[i];
    const float4 a = make_float4(a0.x + tp.x, a0.y + tp.y, a0.z + tp.z, 0.f);
    const float4 b = make_float4(b0.x + tv.x, b0.y + tv.y, b0.z + tv.z, 0.f);
    const float r = P.inv_dt;
    gp[i] = make_float4(a.x + b.x * r, a.y + b.y * r, a.z + b.z * r, 0.f);
    gx_mod[i] = make_float4(-b.x * r, -b.y * r, -b.z * r, 0.f);   // becomes dL/dx
}

// update backward: pbar = xbar + vbar/dt, xbar = -vbar/dt   (sorted order of the frame)
__global__ void adj_update_kernel(const DevParams P, const float4* __restrict__ gx_out, const float4* __restrict__ gv_out,
                                  float4* __restrict__ gp, float4* __restrict__ gx) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= P.N) return;
    const float4 a = gx_out[i], b = gv_out[i];
    const float r = P.inv_dt;
    gp[i] = make_float4(a.x + b.x * r, a.y + b.y * r, a.z + b.z * r, 0.f);
    gx[i] = make_float4(-b.x * r, -b.y * r, -b.z * r, 0.f);
}

// Delta + contact backward for one iteration.  gp_in = dL/dp^{it+1}, gx = dL/dx^{it+1};
// gp_out (pre-filled with gp_in) receives J^T terms; glam receives dL/dlambda (pre-zeroed).
struct AdjDeltaVisit {
    struct Contrib { int dummy; };
    const DevParams& P;
    const float* __restrict__ lambda;
    const float* __restrict__ w;   // inverse masses (solids), or null
    float wi;
    float4 pi;
    float li;
    float3 a;          // Delta-bar / rho0 (w_i scales the density correction)
    float3 cbar;       // dL/dc_i = gp_in + gx
    unsigned long long* scat;   // per particle: x, y, z of dL/dp, dL/dlambda (fixed point)
    float fix;         // the frame's fixed-point scale
    float3 gpi;        // this particle's own accumulated term
    float3 sdelta;     // sum coef * G (for the rho0 term)
    float glami;
    bool collide;      // solveCollisions runs (collisionType 0)
    __device__ __forceinline__ void end_contacts(uint32_t) {}
    __device__ static Contrib zero() { return Contrib{0}; }
    __device__ static bool effective(const Contrib&) { return false; }
    __device__ static Contrib shfl(const Contrib& c, int) { return c; }
    __device__ __forceinline__ Contrib contrib(uint32_t j, const float4& pj, bool contact) {
        const float rx = pi.x - pj.x, ry = pi.y - pj.y, rz = pi.z - pj.z;
        const float r2 = dist2(rx, ry, rz);
        if (r2 >= P.cut2 || r2 <= 0.0f) return zero();
        const float L = sqrtf(r2);
        const float3 rh = make_float3(rx / L, ry / L, rz / L);
        float3 rbar = make_float3(0.f, 0.f, 0.f);
        float g, dg;
        spiky_g(P, L, g, dg);
        if (g != 0.0f) {
            float W, dW;
            poly6_w(P, L, W, dW);
            const float q = W * P.inv_wq;
            const float sc = -P.k_scorr * powi(q, P.n_scorr);
            const float dsc = P.n_scorr != 0 ? -P.k_scorr * (float)P.n_scorr * powi(q, P.n_scorr - 1) * dW * P.inv_wq : 0.0f;
            const float lj = __ldg(lambda + j);
            const float coef = li + lj + sc;
            const float3 G = make_float3(g * rh.x, g * rh.y, g * rh.z);
            const float gd = G.x * a.x + G.y * a.y + G.z * a.z;
            glami += gd;
            fix_add(scat + 4 * (size_t)j + 3, gd, fix);
            const float3 Ha = spiky_hess_mul(g, dg, L, rh, a);
            rbar.x += coef * Ha.x + gd * dsc * rh.x;
            rbar.y += coef * Ha.y + gd * dsc * rh.y;
            rbar.z += coef * Ha.z + gd * dsc * rh.z;
            sdelta.x += coef * G.x; sdelta.y += coef * G.y; sdelta.z += coef * G.z;
        }
        if (contact && collide) {
            const float overlap = P.d - L;
            // this particle's share of the overlap: w_i / (w_i + w_j), 1/2 with unit masses
            float share = 0.5f;
            if (w) {
                const float wj = __ldg(w + j);
                share = (wi + wj) > 0.0f ? wi / (wi + wj) : 0.0f;
            }
            if (overlap > 0.0f && L > 0.00001f && share != 0.0f) {
                // f = ac (d - L) rhat, df/dr = ac [ -rhat rhat^T + (d - L)/L (I - rhat rhat^T) ]
                const float ac = share * P.one_minus_stiffness;
                const float rc = rh.x * cbar.x + rh.y * cbar.y + rh.z * cbar.z;
                const float ol = overlap / L;
                rbar.x += ac * (-rc * rh.x + ol * (cbar.x - rc * rh.x));
                rbar.y += ac * (-rc * rh.y + ol * (cbar.y - rc * rh.y));
                rbar.z += ac * (-rc * rh.z + ol * (cbar.z - rc * rh.z));
            }
        }
        gpi.x += rbar.x; gpi.y += rbar.y; gpi.z += rbar.z;
        scatter_sub3(scat + 4 * (size_t)j, rbar, fix);
        return zero();
    }
    __device__ __forceinline__ void add(const Contrib&, bool) {}
};

__global__ void __launch_bounds__(128)
adj_delta_kernel(DevParams P, const float4* __restrict__ p, const float4* __restrict__ pa, const float* __restrict__ lambda,
                 const float4* __restrict__ gp_in, const float4* __restrict__ gx, float4* __restrict__ gp_out,
                 float* __restrict__ glam, unsigned long long* __restrict__ scat, unsigned long long* __restrict__ scat_in,
                 const uint32_t* __restrict__ cs, const uint32_t* __restrict__ ce, double* acc, bool collide,
                 NbList Lt, const uint32_t* __restrict__ gmax, const float* __restrict__ w,
                 const float4* __restrict__ gfin) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    double drho = 0.0;
    if (i < P.N) {
        const SceneCtx S = scene_ctx(P, i);
        const FixScale fs = fix_scale(gmax);
        const float4 g0 = gp_in[i], t = take_scattered(scat_in, i, fs.inv), gxi = gx[i];   // + the pass after's partners
        const float4 gpin = make_float4(g0.x + t.x, g0.y + t.y, g0.z + t.z, 0.f);
        // the density correction is applied after the iteration's last contact pass: its terms take
        // the iteration's final gradient (gfin, with later contact passes), else this pass's
        const float4 gd = gfin ? gfin[i] : gpin;
        const float wi = w ? w[i] : 1.0f;
        const float inv = 1.0f / S.rho0, winv = wi * inv;
        AdjDeltaVisit vis{P, lambda, w, wi, p[i], lambda[i],
                          make_float3(-gd.x * winv, -gd.y * winv, -gd.z * winv),
                          make_float3(gpin.x + gxi.x, gpin.y + gxi.y, gpin.z + gxi.z), scat, fs.sc,
                          make_float3(0.f, 0.f, 0.f), make_float3(0.f, 0.f, 0.f), 0.f, collide};
        // the forward's near list of this iteration (the pairs within the cut), else the cells
        const uint32_t meta = Lt.list ? Lt.meta[i] : kListOff;
        bool deferred = false;
        if (meta != kListOff) walk_list(Lt, i, meta, p, vis);
        else walk_seq(P, S, i, pa[i], p, cs, ce, vis, false, &deferred);
        // own terms: this thread alone writes slot i (the partners' terms are in scat)
        gp_out[i] = make_float4(gpin.x + vis.gpi.x, gpin.y + vis.gpi.y, gpin.z + vis.gpi.z, 0.f);
        glam[i] = vis.glami;
        // Delta_i = sdelta / rho0 (applied as w_i Delta_i): d/drho0 = -w_i sdelta / rho0^2, Delta-bar = -w_i gp_in
        drho = (double)(gd.x * vis.sdelta.x + gd.y * vis.sdelta.y + gd.z * vis.sdelta.z) * (double)(inv * inv) *
               (double)wi;
    }
    block_add2(drho, 0.0, acc);
}

// A contact pass after the iteration's first (stabilizationIterations > 1; Collision.h:171-242 run
// again on the positions the pass before left): p' = p + c(p), x' = x + c(p).  gp_out = gp_in
// (own + the pass after's partners) + the contacts' own J^T terms, the partners' to scat;
// gd_out, when given, keeps the complete gp_in (the iteration's final gradient).
struct AdjCollideVisit {
    struct Contrib { int dummy; };
    const DevParams& P;
    const float* __restrict__ w;
    float wi;
    float4 pi;
    float3 cbar;       // dL/dc_i = gp_in + gx
    unsigned long long* scat;
    float fix;
    float3 gpi = make_float3(0.f, 0.f, 0.f);
    __device__ __forceinline__ void end_contacts(uint32_t) {}
    __device__ static Contrib zero() { return Contrib{0}; }
    __device__ static bool effective(const Contrib&) { return false; }
    __device__ static Contrib shfl(const Contrib& c, int) { return c; }
    __device__ __forceinline__ Contrib contrib(uint32_t j, const float4& pj, bool contact) {
        if (!contact) return zero();
        const float rx = pi.x - pj.x, ry = pi.y - pj.y, rz = pi.z - pj.z;
        const float r2 = dist2(rx, ry, rz);
        if (r2 >= P.cut2 || r2 <= 0.0f) return zero();
        const float L = sqrtf(r2);
        const float overlap = P.d - L;
        float share = 0.5f;
        if (w) {
            const float wj = __ldg(w + j);
            share = (wi + wj) > 0.0f ? wi / (wi + wj) : 0.0f;
        }
        if (!(overlap > 0.0f && L > 0.00001f && share != 0.0f)) return zero();
        const float3 rh = make_float3(rx / L, ry / L, rz / L);
        const float ac = share * P.one_minus_stiffness;
        const float rc = rh.x * cbar.x + rh.y * cbar.y + rh.z * cbar.z;
        const float ol = overlap / L;
        const float3 rb = make_float3(ac * (-rc * rh.x + ol * (cbar.x - rc * rh.x)), ac * (-rc * rh.y + ol * (cbar.y - rc * rh.y)),
                                      ac * (-rc * rh.z + ol * (cbar.z - rc * rh.z)));
        gpi.x += rb.x; gpi.y += rb.y; gpi.z += rb.z;
        scatter_sub3(scat + 4 * (size_t)j, rb, fix);
        return zero();
    }
    __device__ __forceinline__ void add(const Contrib&, bool) {}
};

__global__ void __launch_bounds__(128)
adj_collide_kernel(DevParams P, const float4* __restrict__ p, const float4* __restrict__ pa,
                   const float4* __restrict__ gp_in, const float4* __restrict__ gx, float4* __restrict__ gp_out,
                   unsigned long long* __restrict__ scat_in, unsigned long long* __restrict__ scat,
                   float4* __restrict__ gd_out, const uint32_t* __restrict__ cs, const uint32_t* __restrict__ ce,
                   const uint32_t* __restrict__ gmax, const float* __restrict__ w) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= P.N) return;
    const SceneCtx S = scene_ctx(P, i);
    const FixScale fs = fix_scale(gmax);
    const float4 g0 = gp_in[i], t = take_scattered(scat_in, i, fs.inv), gxi = gx[i];
    const float4 g = make_float4(g0.x + t.x, g0.y + t.y, g0.z + t.z, 0.f);
    if (gd_out) gd_out[i] = g;
    AdjCollideVisit vis{P, w, w ? w[i] : 1.0f, p[i], make_float3(g.x + gxi.x, g.y + gxi.y, g.z + gxi.z), scat, fs.sc};
    bool deferred = false;
    walk_seq(P, S, i, pa[i], p, cs, ce, vis, false, &deferred);
    gp_out[i] = make_float4(g.x + vis.gpi.x, g.y + vis.gpi.y, g.z + vis.gpi.z, 0.f);
}

// lambda backward for one iteration: glam complete; adds J^T terms to gp_out, d/drho0, d/deps.
// rho, B and S come from the forward's own sums (LambdaVisit::store_aux), so only the scatter
// walk remains.
struct AdjLambdaBwd {
    struct Contrib { int dummy; };
    const DevParams& P;
    float4 pi;
    float cbar_w;      // Cbar / rho0
    float dbar2;       // 2 Dbar / rho0
    float3 Sg;
    unsigned long long* scat;
    float fix;         // the frame's fixed-point scale
    float3 gpi;
    __device__ __forceinline__ void end_contacts(uint32_t) {}
    __device__ static Contrib zero() { return Contrib{0}; }
    __device__ static bool effective(const Contrib&) { return false; }
    __device__ static Contrib shfl(const Contrib& c, int) { return c; }
    __device__ __forceinline__ Contrib contrib(uint32_t j, const float4& pj, bool) {
        const float rx = pi.x - pj.x, ry = pi.y - pj.y, rz = pi.z - pj.z;
        const float r2 = dist2(rx, ry, rz);
        if (r2 >= P.cut2 || r2 <= 0.0f) return zero();
        const float L = sqrtf(r2);
        const float3 rh = make_float3(rx / L, ry / L, rz / L);
        float g, dg, W, dW;
        spiky_g(P, L, g, dg);
        poly6_w(P, L, W, dW);
        float3 rbar = make_float3(cbar_w * dW * rh.x, cbar_w * dW * rh.y, cbar_w * dW * rh.z);
        if (g != 0.0f) {
            const float3 v = make_float3(g * rh.x + Sg.x, g * rh.y + Sg.y, g * rh.z + Sg.z);
            const float3 Hv = spiky_hess_mul(g, dg, L, rh, v);
            rbar.x += dbar2 * Hv.x; rbar.y += dbar2 * Hv.y; rbar.z += dbar2 * Hv.z;
        }
        gpi.x += rbar.x; gpi.y += rbar.y; gpi.z += rbar.z;
        scatter_sub3(scat + 4 * (size_t)j, rbar, fix);
        return zero();
    }
    __device__ __forceinline__ void add(const Contrib&, bool) {}
};

__global__ void __launch_bounds__(128)
adj_lambda_kernel(DevParams P, const float4* __restrict__ p, const float4* __restrict__ pa, const float4* __restrict__ aux,
                  const float* __restrict__ glam, float4* __restrict__ gp_out, unsigned long long* __restrict__ scat,
                  unsigned long long* __restrict__ scat_in, const uint32_t* __restrict__ cs,
                  const uint32_t* __restrict__ ce, double* acc, NbList Lt, const uint32_t* __restrict__ gmax) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    double drho = 0.0, deps = 0.0;
    if (i < P.N) {
        const SceneCtx S = scene_ctx(P, i);
        const FixScale fs = fix_scale(gmax);
        const float4 t = take_scattered(scat_in, i, fs.inv);   // the delta pass's partners' terms
        const float4 g0 = gp_out[i];
        const float4 g = make_float4(g0.x + t.x, g0.y + t.y, g0.z + t.z, 0.f);
        const float lb = glam[i] + t.w;
        const float4 s0 = aux[i], s1 = aux[P.N + i];   // (rho, B, S.x, S.y), (S.z, S.w, 0, 0)
        const float rho0 = S.rho0;
        const float C = s0.x / rho0 - 1.0f;
        const float BS = s0.y + (s0.z * s0.z + s0.w * s0.w + s1.x * s1.x + s1.y * s1.y);
        const float D = BS / rho0 + P.lambda_eps;
        const float Cbar = -lb / D;
        const float Dbar = lb * C / (D * D);
        const double r02 = (double)rho0 * rho0;
        drho = (double)Cbar * (-(double)s0.x / r02) + (double)Dbar * (-(double)BS / r02);
        deps = (double)Dbar;
        if (lb != 0.0f) {
            AdjLambdaBwd b{P, p[i], Cbar / rho0, 2.0f * Dbar / rho0, make_float3(s0.z, s0.w, s1.x), scat, fs.sc,
                           make_float3(0.f, 0.f, 0.f)};
            const uint32_t meta = Lt.list ? Lt.meta[i] : kListOff;
            bool deferred = false;
            if (meta != kListOff) walk_list(Lt, i, meta, p, b);
            else walk_seq(P, S, i, pa[i], p, cs, ce, b, false, &deferred);
            gp_out[i] = make_float4(g.x + b.gpi.x, g.y + b.gpi.y, g.z + b.gpi.z, 0.f);   // this thread alone writes slot i
        } else {
            gp_out[i] = g;
        }
    }
    block_add2(drho, deps, acc);
}

// re-order + applyForces backward, fused: sorted slot i came from pre-sort slot o = perm[i];
// p = x + v* dt unless the wall clamp fired on that axis, and x is damped toward p when it did.
__global__ void adj_predict_kernel(DevParams P, const uint32_t* __restrict__ perm, const float4* __restrict__ x_in,
                                   const float4* __restrict__ v_in, const float4* __restrict__ fext,
                                   const float4* __restrict__ gp, const float4* __restrict__ gxp,
                                   float4* __restrict__ gx_out, float4* __restrict__ gv_out,
                                   unsigned long long* __restrict__ scat_in, const uint32_t* __restrict__ gmax) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= P.N) return;
    const uint32_t o = perm[i];
    const float4 xx = x_in[o], f = fext[o];
    float4 vv = v_in[o];
    const float dt = P.dt;
    vv.y = __fmaf_rn(P.gravity, dt, vv.y);
    vv.x = __fmaf_rn(f.x, dt, vv.x);
    vv.y = __fmaf_rn(f.y, dt, vv.y);
    vv.z = __fmaf_rn(f.z, dt, vv.z);
    const float px = __fmaf_rn(vv.x, dt, xx.x), py = __fmaf_rn(vv.y, dt, xx.y), pz = __fmaf_rn(vv.z, dt, xx.z);
    const float mx = (px < P.bmin[0] || px > P.bmax[0]) ? 0.f : 1.f;
    const float my = (py < P.bmin[1] || py > P.bmax[1]) ? 0.f : 1.f;
    const float mz = (pz < P.bmin[2] || pz > P.bmax[2]) ? 0.f : 1.f;
    const float4 g0 = gp[i], t = take_scattered(scat_in, i, fix_scale(gmax).inv), gx = gxp[i];   // + the last lambda pass's partners
    const float4 g = make_float4(g0.x + t.x, g0.y + t.y, g0.z + t.z, 0.f);
    // enclosurePositionDamping (Forces.h:56-58): a particle clamped on some axis takes
    // x' = x + pd (p - x) on every axis, so dx'/dx = 1 - k + k m and dx'/dv* = k m dt per axis
    // (k = pd when clamped, m the axis's clamp mask; gx is dL/dx')
    const float k = (mx == 0.f || my == 0.f || mz == 0.f) ? P.pos_damp : 0.f;
    gx_out[o] = make_float4(mx * g.x + gx.x * (1.f - k + k * mx), my * g.y + gx.y * (1.f - k + k * my),
                            mz * g.z + gx.z * (1.f - k + k * mz), 0.f);
    gv_out[o] = make_float4(mx * (g.x + k * gx.x) * dt, my * (g.y + k * gx.y) * dt, mz * (g.z + k * gx.z) * dt, 0.f);
}

// Rebuild the cell tables of a taped frame from its sorted keys (computeCellInfo,
// SortReorder.h:160-188).  clear_keys/clear_n: the keys whose cells the tables hold now.
__global__ void adj_clear_cells_kernel(const uint32_t* __restrict__ keys, uint32_t n, uint32_t* __restrict__ cs,
                                       uint32_t table_size) {
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        const uint32_t k = keys[i];
        if (k < table_size) cs[k] = kEmptyCell;
    }
}

__global__ void adj_set_cells_kernel(const uint32_t* __restrict__ skeys, uint32_t n, uint32_t* __restrict__ cs,
                                     uint32_t* __restrict__ ce, uint32_t table_size) {
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        const uint32_t k = skeys[i];
        if (k >= table_size) continue;
        if (i == 0 || skeys[i - 1] != k) cs[k] = i;
        if (i == n - 1 || skeys[i + 1] != k) ce[k] = i + 1;
    }
}

}  // namespace pbd
