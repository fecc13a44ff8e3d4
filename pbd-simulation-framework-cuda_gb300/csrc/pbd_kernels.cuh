// pbd_kernels.cuh -- the per-particle kernels of one frame.
//
// Reference frame (Fluid.cu:14-97) and where each piece lands here:
//   applyForces + initializeCellIds (+ digit histograms, + clearing last frame's cells)
//                                                  -> predict_key_kernel
//   sortIds (CUB SortPairs)                        -> onesweep_pass x P   (pbd_sort.cuh)
//   copy + reorder + resetCellInfo + computeCellInfo -> reorder_cells_kernel
//   findContacts / findNeighbours                  -> no stored list: every neighbour pass
//                                                     re-walks the cells in the list's order
//   computeLambda                                  -> lambda_kernel
//   computeDeltaPositions + solveCollisions + applyDeltaPositions (+ updatePositions on the
//   last iteration)                                -> delta_kernel
//   updatePositions (when it cannot be fused)      -> update_kernel
//   computeOmega                                   -> omega_kernel
//   computeVorticity + computeViscosity            -> vort_visc_kernel
//
// Particle state is float4 SoA in Morton-sorted order.  Every neighbour pass reads a
// snapshot buffer and writes another (Jacobi), so no pass races with itself.
#pragma once
#include "pbd_device.cuh"
#include "pbd_sort.cuh"
#include "../../include/pbd.h"

namespace pbd {

// --------------------------------------------------------------------------------------
// Neighbour walk: visits exactly the entries the reference's list would hold, in its order
// (findContacts: x offset outer, y, z inner, kernel/Collision.h:43-71; then the shells of
// findNeighbours, :126-155), skipping self and stopping at the cap M.  The visitor is told
// whether the entry belongs to the 27-cell part (the "contacts" that solveCollisions uses).
// --------------------------------------------------------------------------------------
template <class V>
__device__ __forceinline__ uint32_t walk_neighbours(const DevParams& P, uint32_t i, float4 pi,
                                                    const uint32_t* __restrict__ cs,
                                                    const uint32_t* __restrict__ ce, V& vis) {
    const uint32_t N = P.N, M = P.M;
    const bool quirk = (P.flags & PBD_FLAG_CELL_END_QUIRK) && N >= 2;
    uint32_t cnt = 0;
    if (M == 0) return 0;
    if (P.active & PBD_ACTIVE_FIND_CONTACTS) {
        uint32_t mz[3];
#pragma unroll
        for (int c = 0; c < 3; ++c) mz[c] = morton_axis(__fmaf_rn((float)(c - 1), P.d, pi.z));
#pragma unroll 1
        for (int a = -1; a <= 1; ++a) {
            const uint32_t hx = morton_axis(__fmaf_rn((float)a, P.d, pi.x)) << 2;
#pragma unroll 1
            for (int b = -1; b <= 1; ++b) {
                const uint32_t hxy = hx + (morton_axis(__fmaf_rn((float)b, P.d, pi.y)) << 1);
#pragma unroll
                for (int c = 0; c < 3; ++c) {
                    const uint32_t h = hxy + mz[c];
                    if (h >= P.G) continue;
                    const uint32_t s = __ldg(cs + h);
                    if (s >= N) continue;
                    uint32_t e = __ldg(ce + h);
                    if ((quirk && h == N - 1) || e > N) e = N;   // entries >= N are skipped (Collision.h:59)
                    for (uint32_t j = s; j < e; ++j) {
                        if (j != i) {
                            vis(j, true);
                            if (++cnt == M) return cnt;
                        }
                    }
                }
            }
        }
    }
    vis.end_contacts(cnt);
    if (P.active & PBD_ACTIVE_FIND_NEIGHBOURS) {
        const int K = (int)P.K;
#pragma unroll 1
        for (int sh = 2; sh <= K; ++sh) {
#pragma unroll 1
            for (int a = -sh; a <= sh; ++a) {
                const uint32_t hx = morton_axis(__fmaf_rn((float)a, P.d, pi.x)) << 2;
#pragma unroll 1
                for (int b = -sh; b <= sh; ++b) {
                    const uint32_t hy = morton_axis(__fmaf_rn((float)b, P.d, pi.y)) << 1;
                    const bool edge_ab = (a == sh || a == -sh || b == sh || b == -sh);
                    const int cstep = edge_ab ? 1 : 2 * sh;   // interior columns: only c = +-sh
#pragma unroll 1
                    for (int c = -sh; c <= sh; c += cstep) {
                        const uint32_t h = hx + hy + morton_axis(__fmaf_rn((float)c, P.d, pi.z));
                        if (h >= P.G) continue;
                        const uint32_t s = __ldg(cs + h);
                        uint32_t e = __ldg(ce + h);
                        if (s == kEmptyCell) continue;
                        if ((quirk && h == N - 1) || e > N) e = N;   // entries >= N are skipped (Collision.h:142)
                        for (uint32_t j = s; j < e; ++j) {
                            if (j != i) {
                                vis(j, false);
                                if (++cnt == M) return cnt;
                            }
                        }
                    }
                }
            }
        }
    }
    return cnt;
}

// --------------------------------------------------------------------------------------
// applyForces (Forces.h:65-101) + initializeCellIds (SortReorder.h:13-28), fused with the
// digit histograms of the radix sort and with clearing the cells the previous frame wrote
// (instead of resetting all maxGrid cells, SortReorder.h:135-149).
// The a*b+c forms are written as explicit FMAs: this is how nvcc contracts the reference's
// expressions, and the CPU oracle uses the same FMAs, so p* and the keys match bit for bit.
// --------------------------------------------------------------------------------------
__global__ void __launch_bounds__(256)
predict_key_kernel(DevParams P, float4* __restrict__ x, float4* __restrict__ v, float4* __restrict__ p,
                   const float4* __restrict__ fext, uint32_t* keys, const uint32_t* old_keys,
                   const uint32_t* __restrict__ table_n, uint32_t* __restrict__ cell_start,
                   uint32_t* __restrict__ hist, int npasses, uint32_t* __restrict__ err) {
    __shared__ uint32_t sh[kMaxPasses * kRadix];
    for (int b = threadIdx.x; b < kMaxPasses * kRadix; b += blockDim.x) sh[b] = 0u;
    __syncthreads();
    const uint32_t N = P.N;
    const uint32_t old_n = *table_n;            // sorted keys whose cells the tables still hold
    const uint32_t total = N > old_n ? N : old_n;
    const bool forces = (P.active & PBD_ACTIVE_APPLY_FORCES) != 0;
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < total; i += gridDim.x * blockDim.x) {
        if (i < old_n) {                        // last frame's cell of slot i: mark empty
            const uint32_t oc = old_keys[i];
            if (oc < P.G) cell_start[oc] = kEmptyCell;
        }
        if (i >= N) continue;
        float4 pp;
        if (forces) {
            float4 vv = v[i];
            const float4 f = fext[i];
            float4 xx = x[i];
            const float dt = P.dt;
            vv.y = __fmaf_rn(P.gravity, dt, vv.y);
            vv.x = __fmaf_rn(f.x, dt, vv.x);
            vv.y = __fmaf_rn(f.y, dt, vv.y);
            vv.z = __fmaf_rn(f.z, dt, vv.z);
            vv.w = __fmaf_rn(f.w, dt, vv.w);
            pp = make_float4(__fmaf_rn(vv.x, dt, xx.x), __fmaf_rn(vv.y, dt, xx.y),
                             __fmaf_rn(vv.z, dt, xx.z), __fmaf_rn(vv.w, dt, xx.w));
            bool upd = false;
            // confineToBox (Forces.h:26-54)
            if (pp.x < P.bmin[0]) { vv.x = __fmul_rn(P.vel_damp, vv.x); pp.x = __fadd_rn(P.bmin[0], 0.001f); upd = true; }
            else if (pp.x > P.bmax[0]) { vv.x = __fmul_rn(P.vel_damp, vv.x); pp.x = __fsub_rn(P.bmax[0], 0.001f); upd = true; }
            if (pp.y < P.bmin[1]) { vv.y = __fmul_rn(P.vel_damp, vv.y); pp.y = __fadd_rn(P.bmin[1], 0.001f); upd = true; }
            else if (pp.y > P.bmax[1]) { vv.y = __fmul_rn(P.vel_damp, vv.y); pp.y = __fsub_rn(P.bmax[1], 0.001f); upd = true; }
            if (pp.z < P.bmin[2]) { vv.z = __fmul_rn(P.vel_damp, vv.z); pp.z = __fadd_rn(P.bmin[2], 0.001f); upd = true; }
            else if (pp.z > P.bmax[2]) { vv.z = __fmul_rn(P.vel_damp, vv.z); pp.z = __fsub_rn(P.bmax[2], 0.001f); upd = true; }
            if (upd) {
                const float pd = P.pos_damp;
                xx.x = __fmaf_rn(pd, __fsub_rn(pp.x, xx.x), xx.x);
                xx.y = __fmaf_rn(pd, __fsub_rn(pp.y, xx.y), xx.y);
                xx.z = __fmaf_rn(pd, __fsub_rn(pp.z, xx.z), xx.z);
                xx.w = __fmaf_rn(pd, __fsub_rn(pp.w, xx.w), xx.w);
                x[i] = xx;
            }
            v[i] = vv;
            pp.w = 1.0f;                         // Forces.h:94
            p[i] = pp;
        } else {
            pp = p[i];
        }
        const uint32_t key = morton(pp.x, pp.y, pp.z);
        keys[i] = key;
        for (int ps = 0; ps < npasses; ++ps) atomicAdd(&sh[ps * kRadix + ((key >> (ps * kRadixBits)) & (kRadix - 1))], 1u);
        if (npasses < kMaxPasses && (key >> (npasses * kRadixBits)) != 0u) atomicOr(err, kErrKeyBits);
    }
    __syncthreads();
    for (int b = threadIdx.x; b < npasses * kRadix; b += blockDim.x)
        if (sh[b]) atomicAdd(&hist[b], sh[b]);
}

// --------------------------------------------------------------------------------------
// copy + reorder (SortReorder.h:53-129) as one gather, fused with computeCellInfo
// (:160-188).  Also returns the sort scratch to zero for the next frame.
// --------------------------------------------------------------------------------------
struct ReorderArgs {
    const uint32_t* skeys;   // sorted keys
    const uint32_t* perm;    // sorted values = index before the sort
    const float4 *xi, *pi, *vi, *ci;
    float4 *xo, *po, *vo, *co;
    const uint32_t* idi;
    uint32_t* ido;
    uint32_t* cell_start;
    uint32_t* cell_end;
    uint32_t* table_n;       // set to N: the cells of these sorted keys are now in the tables
};

__global__ void __launch_bounds__(256)
reorder_cells_kernel(DevParams P, ReorderArgs A, SortScratch S, int npasses, uint32_t ntiles) {
    const uint32_t N = P.N;
    const uint32_t tid = blockIdx.x * blockDim.x + threadIdx.x;
    // zero the sort scratch: the last pass's look-back rows, histograms, tile counters
    const uint32_t nstat = ntiles * kRadix;
    uint32_t* last = S.status + (size_t)(npasses - 1) * S.max_tiles * kRadix;
    for (uint32_t k = tid; k < nstat; k += gridDim.x * blockDim.x) last[k] = 0u;
    if (blockIdx.x == 0) {
        for (int b = threadIdx.x; b < kMaxPasses * kRadix; b += blockDim.x) S.hist[b] = 0u;
        if (threadIdx.x < kMaxPasses) S.tile_counter[threadIdx.x] = 0u;
        if (threadIdx.x == 0) *A.table_n = N;
    }
    for (uint32_t i = tid; i < N; i += gridDim.x * blockDim.x) {
        uint32_t o = A.perm[i];
        if (o >= N) { atomicOr(S.err, kErrSortTimeout); o = i; }   // only after a failed sort
        A.xo[i] = A.xi[o];
        A.po[i] = A.pi[o];
        A.vo[i] = A.vi[o];
        if (A.co) A.co[i] = A.ci[o];
        if (A.ido) A.ido[i] = A.idi[o];
        const uint32_t k = A.skeys[i];
        if (k < P.G) {
            if (i == 0 || A.skeys[i - 1] != k) A.cell_start[k] = i;
            if (i == N - 1 || A.skeys[i + 1] != k) A.cell_end[k] = i + 1;
        }
    }
}

// --------------------------------------------------------------------------------------
// computeLambda (Density.h:48-93)
// --------------------------------------------------------------------------------------
struct LambdaVisit {
    const DevParams& P;
    const float4* __restrict__ p;
    float4 pi;
    float A, B, Cx, Cy, Cz, Cw;
    __device__ __forceinline__ void end_contacts(uint32_t) {}
    __device__ __forceinline__ void operator()(uint32_t j, bool) {
        const float4 pj = __ldg(p + j);
        const float rx = pi.x - pj.x, ry = pi.y - pj.y, rz = pi.z - pj.z, rw = pi.w - pj.w;
        const float r2 = rx * rx + ry * ry + rz * rz;
        if (r2 >= P.cut2) return;      // every kernel is exactly 0 there
        const float dist = sqrtf(r2);
        A += poly6(P, dist);
        const float s = spiky_scale(P, dist, r2 + rw * rw);
        const float gx = s * rx, gy = s * ry, gz = s * rz, gw = s * rw;
        B += gx * gx + gy * gy + gz * gz + gw * gw;
        Cx += gx; Cy += gy; Cz += gz; Cw += gw;
    }
};

__global__ void __launch_bounds__(128)
lambda_kernel(DevParams P, const float4* __restrict__ p, const uint32_t* __restrict__ cs,
              const uint32_t* __restrict__ ce, float* __restrict__ lambda) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= P.N) return;
    LambdaVisit vis{P, p, p[i], 0.f, 0.f, 0.f, 0.f, 0.f, 0.f};
    walk_neighbours(P, i, vis.pi, cs, ce, vis);
    const float a = vis.A / P.rho0 - 1.0f;
    const float b = vis.B / P.rho0;
    const float c = (vis.Cx * vis.Cx + vis.Cy * vis.Cy + vis.Cz * vis.Cz + vis.Cw * vis.Cw) / P.rho0;
    lambda[i] = -a / (b + c + P.lambda_eps);
}

// --------------------------------------------------------------------------------------
// computeDeltaPositions (Density.h:104-145) + solveCollisions type 0 (Collision.h:171-242,
// Jacobi: contacts read the frame's snapshot, the adds of particle i apply in list order)
// + applyDeltaPositions (Density.h:156-168) + updatePositions (Update.h:11-32).
// --------------------------------------------------------------------------------------
enum DeltaMode : uint32_t {
    kDoDelta = 1u << 0,      // compute delta p from lambda
    kDoCollide = 1u << 1,    // one solveCollisions pass over the contacts
    kDoApply = 1u << 2,      // p -= delta
    kLoadDelta = 1u << 3,    // delta from the buffer (not computed in this pass)
    kStoreDelta = 1u << 4,   // keep delta in the buffer
    kDoUpdate = 1u << 5,     // v = (p - x)/dt; x = p
};

struct DeltaVisit {
    const DevParams& P;
    const float4* __restrict__ p;
    const float* __restrict__ lambda;
    float4 pi;
    float li;
    bool do_delta, do_collide, all_pairs;
    float ax, ay, az, aw;        // sum of (li + lj + sCorr) * grad
    float4 pacc, xacc;           // positions with the contact corrections added in order
    __device__ __forceinline__ void end_contacts(uint32_t) {}
    __device__ __forceinline__ void operator()(uint32_t j, bool contact) {
        const float4 pj = __ldg(p + j);
        const float rx = pi.x - pj.x, ry = pi.y - pj.y, rz = pi.z - pj.z, rw = pi.w - pj.w;
        const float r2 = rx * rx + ry * ry + rz * rz;
        if (!all_pairs && r2 >= P.cut2) return;
        const float dist = sqrtf(r2);
        if (do_delta) {
            const float s = spiky_scale(P, dist, r2 + rw * rw);
            if (s != 0.0f || all_pairs) {
                const float W = poly6(P, dist);
                const float sc = -P.k_scorr * powi(__fdiv_rn(W, P.wq), P.n_scorr);
                const float coef = (li + __ldg(lambda + j) + sc) * s;
                ax += coef * rx; ay += coef * ry; az += coef * rz; aw += coef * rw;
            }
        }
        if (contact && do_collide) {
            const float overlap = P.d - dist;
            if (overlap > 0.0f && dist > 0.00001f) {
                const float sc = -0.5f * overlap;
                const float cx = (sc * __fdiv_rn(-rx, dist)) * P.one_minus_stiffness;
                const float cy = (sc * __fdiv_rn(-ry, dist)) * P.one_minus_stiffness;
                const float cz = (sc * __fdiv_rn(-rz, dist)) * P.one_minus_stiffness;
                pacc.x += cx; xacc.x += cx;
                pacc.y += cy; xacc.y += cy;
                pacc.z += cz; xacc.z += cz;
            }
        }
    }
};

__global__ void __launch_bounds__(128)
delta_kernel(DevParams P, uint32_t mode, const float4* __restrict__ pin, float4* __restrict__ pout,
             float4* __restrict__ x, float4* __restrict__ v, const float* __restrict__ lambda,
             float4* __restrict__ delta, const uint32_t* __restrict__ cs, const uint32_t* __restrict__ ce) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= P.N) return;
    const float4 pi = pin[i];
    const bool need_x = (mode & (kDoCollide | kDoUpdate)) != 0;
    const float4 xi = need_x ? x[i] : make_float4(0.f, 0.f, 0.f, 0.f);
    DeltaVisit vis{P, pin, lambda, pi, (mode & kDoDelta) ? lambda[i] : 0.f,
                   (mode & kDoDelta) != 0, (mode & kDoCollide) != 0, P.far_pairs_zero == 0u,
                   0.f, 0.f, 0.f, 0.f, pi, xi};
    if (mode & (kDoDelta | kDoCollide)) walk_neighbours(P, i, pi, cs, ce, vis);
    float4 pn = vis.pacc, xn = vis.xacc;
    float4 dp = make_float4(0.f, 0.f, 0.f, 0.f);
    if (mode & kDoDelta) dp = make_float4(vis.ax / P.rho0, vis.ay / P.rho0, vis.az / P.rho0, vis.aw / P.rho0);
    else if (mode & kLoadDelta) dp = delta[i];
    if (mode & kStoreDelta) delta[i] = dp;
    if (mode & kDoApply) { pn.x -= dp.x; pn.y -= dp.y; pn.z -= dp.z; pn.w -= dp.w; }
    if (mode & kDoUpdate) {
        const float dt = P.dt;
        v[i] = make_float4(__fdiv_rn(pn.x - xn.x, dt), __fdiv_rn(pn.y - xn.y, dt),
                           __fdiv_rn(pn.z - xn.z, dt), __fdiv_rn(pn.w - xn.w, dt));
        xn = pn;
    }
    pout[i] = pn;
    if (need_x) x[i] = xn;
}

// updatePositions on its own (Update.h:11-32), when no delta pass can carry it.
__global__ void __launch_bounds__(256)
update_kernel(DevParams P, const float4* __restrict__ p, float4* __restrict__ x, float4* __restrict__ v) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= P.N) return;
    const float4 pp = p[i], xx = x[i];
    const float dt = P.dt;
    v[i] = make_float4(__fdiv_rn(pp.x - xx.x, dt), __fdiv_rn(pp.y - xx.y, dt), __fdiv_rn(pp.z - xx.z, dt),
                       __fdiv_rn(pp.w - xx.w, dt));
    x[i] = pp;
}

// --------------------------------------------------------------------------------------
// computeOmega (Density.h:232-269): omega_i = sum_j (v_j - v_i) x spiky(p_i, p_j)
// --------------------------------------------------------------------------------------
struct OmegaVisit {
    const DevParams& P;
    const float4* __restrict__ p;
    const float4* __restrict__ v;
    float4 pi, vi;
    float ox, oy, oz;
    __device__ __forceinline__ void end_contacts(uint32_t) {}
    __device__ __forceinline__ void operator()(uint32_t j, bool) {
        const float4 pj = __ldg(p + j);
        const float rx = pi.x - pj.x, ry = pi.y - pj.y, rz = pi.z - pj.z, rw = pi.w - pj.w;
        const float r2 = rx * rx + ry * ry + rz * rz;
        if (r2 >= P.cut2) return;
        const float dist = sqrtf(r2);
        const float s = spiky_scale(P, dist, r2 + rw * rw);
        if (s == 0.0f) return;
        const float4 vj = __ldg(v + j);
        const float wx = vj.x - vi.x, wy = vj.y - vi.y, wz = vj.z - vi.z;
        const float gx = s * rx, gy = s * ry, gz = s * rz;
        ox += wy * gz - wz * gy;
        oy += wz * gx - wx * gz;
        oz += wx * gy - wy * gx;
    }
};

__global__ void __launch_bounds__(128)
omega_kernel(DevParams P, const float4* __restrict__ p, const float4* __restrict__ v,
             const uint32_t* __restrict__ cs, const uint32_t* __restrict__ ce, float4* __restrict__ omega) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= P.N) return;
    OmegaVisit vis{P, p, v, p[i], v[i], 0.f, 0.f, 0.f};
    walk_neighbours(P, i, vis.pi, cs, ce, vis);
    omega[i] = make_float4(vis.ox, vis.oy, vis.oz, 0.f);
}

// --------------------------------------------------------------------------------------
// computeVorticity (Density.h:179-221) + computeViscosity (Density.h:280-310, Jacobi).
// Vorticity sums |omega_j - omega_i| / (p_j - p_i + 1e-8) componentwise over EVERY list
// entry (no kernel weight), so with vorticity on no pair may be skipped.
// --------------------------------------------------------------------------------------
struct VortViscVisit {
    const DevParams& P;
    const float4* __restrict__ p;
    const float4* __restrict__ v;
    const float4* __restrict__ omega;
    float4 pi, vi, oi;
    bool vort, visc;
    float gx, gy, gz;
    float sx, sy, sz, sw;
    __device__ __forceinline__ void end_contacts(uint32_t) {}
    __device__ __forceinline__ void operator()(uint32_t j, bool) {
        const float4 pj = __ldg(p + j);
        if (vort) {
            const float4 oj = __ldg(omega + j);
            const float dx = oj.x - oi.x, dy = oj.y - oi.y, dz = oj.z - oi.z;
            const float ol = sqrtf(dx * dx + dy * dy + dz * dz);
            gx += __fdiv_rn(ol, (pj.x - pi.x) + 0.00000001f);
            gy += __fdiv_rn(ol, (pj.y - pi.y) + 0.00000001f);
            gz += __fdiv_rn(ol, (pj.z - pi.z) + 0.00000001f);
        }
        if (visc) {
            const float rx = pi.x - pj.x, ry = pi.y - pj.y, rz = pi.z - pj.z;
            const float r2 = rx * rx + ry * ry + rz * rz;
            if (r2 >= P.hp2) return;
            const float W = poly6(P, sqrtf(r2));
            if (W == 0.0f) return;
            const float4 vj = __ldg(v + j);
            sx += (vj.x - vi.x) * W; sy += (vj.y - vi.y) * W;
            sz += (vj.z - vi.z) * W; sw += (vj.w - vi.w) * W;
        }
    }
};

__global__ void __launch_bounds__(128)
vort_visc_kernel(DevParams P, const float4* __restrict__ p, const float4* __restrict__ vin,
                 float4* __restrict__ vout, const float4* __restrict__ omega, float4* __restrict__ fext,
                 const uint32_t* __restrict__ cs, const uint32_t* __restrict__ ce, int do_vort, int do_visc) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= P.N) return;
    const float4 oi = do_vort ? omega[i] : make_float4(0.f, 0.f, 0.f, 0.f);
    VortViscVisit vis{P, p, vin, omega, p[i], vin[i], oi, do_vort != 0, do_visc != 0,
                      0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f};
    walk_neighbours(P, i, vis.pi, cs, ce, vis);
    if (do_vort) {
        const float EPS = 0.00000001f;
        const float gl = sqrtf(vis.gx * vis.gx + vis.gy * vis.gy + vis.gz * vis.gz);
        const float inv = 1.0f / (gl + EPS);
        const float nx = inv * (vis.gx + EPS), ny = inv * (vis.gy + EPS), nz = inv * (vis.gz + EPS);
        const float e = P.e_vort;
        fext[i] = make_float4(e * (ny * oi.z - nz * oi.y), e * (nz * oi.x - nx * oi.z), e * (nx * oi.y - ny * oi.x), 0.f);
    }
    if (do_visc) {
        const float c = P.c_visc;
        const float4 vi = vis.vi;
        vout[i] = make_float4(vi.x + c * vis.sx, vi.y + c * vis.sy, vi.z + c * vis.sz, vi.w + c * vis.sw);
    }
}

// --------------------------------------------------------------------------------------
// Debug: materialise the neighbour list (findContacts + findNeighbours, Collision.h:11-160)
// --------------------------------------------------------------------------------------
struct ListVisit {
    uint32_t* out;
    uint32_t cap, n, contacts;
    __device__ __forceinline__ void end_contacts(uint32_t c) { contacts = c; }
    __device__ __forceinline__ void operator()(uint32_t j, bool) {
        if (n < cap) out[n] = j;
        ++n;
    }
};

__global__ void list_kernel(DevParams P, const float4* __restrict__ p, const uint32_t* __restrict__ cs,
                            const uint32_t* __restrict__ ce, uint32_t cap, uint32_t* list,
                            uint32_t* count, uint32_t* contacts, float4* col) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= P.N) return;
    ListVisit vis{list + (size_t)i * cap, cap, 0u, 0u};
    vis.contacts = 0xFFFFFFFFu;
    const uint32_t n = walk_neighbours(P, i, p[i], cs, ce, vis);
    if (vis.contacts == 0xFFFFFFFFu) vis.contacts = n;   // cap reached inside the 27 cells
    count[i] = n;
    contacts[i] = vis.contacts;
    if (col) {
        const float f = (float)n / (float)P.M;
        col[i] = make_float4(f, f, f, 1.0f);
    }
}

// Mark empty every cell the tables hold (used when the sorted-key buffer moves).
__global__ void clear_cells_kernel(const uint32_t* __restrict__ old_keys, const uint32_t* __restrict__ table_n,
                                   uint32_t* __restrict__ cell_start, uint32_t G) {
    const uint32_t n = *table_n;
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        const uint32_t oc = old_keys[i];
        if (oc < G) cell_start[oc] = kEmptyCell;
    }
}

__global__ void fill_ids_kernel(uint32_t* ids, uint32_t first, uint32_t n) {
    const uint32_t k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k < n) ids[first + k] = first + k;
}

__global__ void add_one_kernel(float4* x, float4* v, float4* col, uint32_t* ids, uint32_t at,
                               float px, float py, float pz, float dx, float dy, float dz) {
    x[at] = make_float4(px, py, pz, 0.0f);
    v[at] = make_float4(50.0f * dx, 50.0f * dy, 50.0f * dz, 0.0f);   // Communication.h:27
    if (col) col[at] = make_float4(1.0f, 0.0f, 0.0f, 1.0f);
    if (ids) ids[at] = at;
}

}  // namespace pbd
