// pbd_kernels.cuh -- the per-particle kernels of one frame.
//
// Reference frame (Fluid.cu:14-97) and where each piece lands here:
//   applyForces + initializeCellIds (+ digit histograms, + clearing last frame's cells)
//                                                  -> predict_key_kernel
//   sortIds (CUB SortPairs)                        -> onesweep_pass x P   (pbd_sort.cuh)
//   copy + reorder + resetCellInfo + computeCellInfo -> reorder_cells_kernel
//   findContacts / findNeighbours                  -> the frame's first lambda pass walks the
//                                                     cells in the list's order and stores the
//                                                     full list; later passes read it
//   computeLambda, computeDeltaPositions + solveCollisions + applyDeltaPositions
//   (+ updatePositions), computeOmega, computeVorticity + computeViscosity
//                                                  -> pbd_passes.cuh
//
// Particle state is float4 SoA in Morton-sorted order.  Every neighbour pass reads a
// snapshot buffer and writes another (Jacobi), so no pass races with itself.
#pragma once
#include "pbd_device.cuh"
#include "pbd_sort.cuh"
#include "pbd_passes.cuh"
#include "../../include/pbd.h"

namespace pbd {

// --------------------------------------------------------------------------------------
// applyForces (Forces.h:65-101) + initializeCellIds (SortReorder.h:13-28), fused with the
// digit histograms of the radix sort and with clearing the cells the previous frame wrote
// (instead of resetting all maxGrid cells, SortReorder.h:135-149).
// The a*b+c forms are written as explicit FMAs: this is how nvcc contracts the reference's
// expressions, and the CPU oracle uses the same FMAs, so p* and the keys match bit for bit.
// --------------------------------------------------------------------------------------
__global__ void __launch_bounds__(256)
predict_key_kernel(DevParams P, float4* __restrict__ x, float4* __restrict__ v, float4* __restrict__ p,
                   const float4* __restrict__ fext, const float* __restrict__ w, uint32_t* keys, const uint32_t* old_keys,
                   const uint32_t* __restrict__ table_n, uint32_t* __restrict__ cell_start,
                   uint32_t* __restrict__ hist, int npasses, uint32_t* __restrict__ err, uint32_t* __restrict__ clear_word) {
    __shared__ uint32_t sh[kMaxPasses * kRadix];
    for (int b = threadIdx.x; b < kMaxPasses * kRadix; b += blockDim.x) sh[b] = 0u;
    __syncthreads();
    const uint32_t N = P.N;
    const uint32_t old_n = *table_n;            // sorted keys whose cells the tables still hold
    const uint32_t total = N > old_n ? N : old_n;
    const bool forces = (P.active & PBD_ACTIVE_APPLY_FORCES) != 0;
    if (clear_word && blockIdx.x == 0 && threadIdx.x == 0) *clear_word = 0u;   // a set the frame refills
    if (P.batched && blockIdx.x == 0)           // scene ranges are rebuilt by the re-order
        for (uint32_t k = threadIdx.x; k < 2 * P.nscenes; k += blockDim.x) P.scene_range[k] = 0u;
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < total; i += gridDim.x * blockDim.x) {
        if (i < old_n) {                        // last frame's cell of slot i: mark empty
            const uint32_t oc = old_keys[i];
            if (oc < P.table_size) cell_start[oc] = kEmptyCell;
        }
        if (i >= N) continue;
        float4 pp;
        uint32_t sc = 0;
        float gravity = P.gravity;
        const float* bmin = P.bmin;
        const float* bmax = P.bmax;
        if (P.batched) {                         // this particle's scene: own gravity and walls
            sc = P.scene_of[i];
            gravity = P.scenes[sc].gravity;
            bmin = P.scenes[sc].bmin;
            bmax = P.scenes[sc].bmax;
        }
        if (forces) {
            float4 vv = v[i];
            float4 xx = x[i];
            const float dt = P.dt;
            if (!w || w[i] != 0.0f) {           // solids (inverse mass 0) take no forces
                const float4 f = fext[i];
                vv.y = __fmaf_rn(gravity, dt, vv.y);
                vv.x = __fmaf_rn(f.x, dt, vv.x);
                vv.y = __fmaf_rn(f.y, dt, vv.y);
                vv.z = __fmaf_rn(f.z, dt, vv.z);
                vv.w = __fmaf_rn(f.w, dt, vv.w);
            }
            pp = make_float4(__fmaf_rn(vv.x, dt, xx.x), __fmaf_rn(vv.y, dt, xx.y),
                             __fmaf_rn(vv.z, dt, xx.z), __fmaf_rn(vv.w, dt, xx.w));
            bool upd = false;
            // confineToBox (Forces.h:26-54)
            if (pp.x < bmin[0]) { vv.x = __fmul_rn(P.vel_damp, vv.x); pp.x = __fadd_rn(bmin[0], 0.001f); upd = true; }
            else if (pp.x > bmax[0]) { vv.x = __fmul_rn(P.vel_damp, vv.x); pp.x = __fsub_rn(bmax[0], 0.001f); upd = true; }
            if (pp.y < bmin[1]) { vv.y = __fmul_rn(P.vel_damp, vv.y); pp.y = __fadd_rn(bmin[1], 0.001f); upd = true; }
            else if (pp.y > bmax[1]) { vv.y = __fmul_rn(P.vel_damp, vv.y); pp.y = __fsub_rn(bmax[1], 0.001f); upd = true; }
            if (pp.z < bmin[2]) { vv.z = __fmul_rn(P.vel_damp, vv.z); pp.z = __fadd_rn(bmin[2], 0.001f); upd = true; }
            else if (pp.z > bmax[2]) { vv.z = __fmul_rn(P.vel_damp, vv.z); pp.z = __fsub_rn(bmax[2], 0.001f); upd = true; }
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
        uint32_t key = morton(pp.x, pp.y, pp.z);
        if (P.batched) {                         // the scene's slice: scenes sort apart
            const uint32_t cells = P.scenes[sc].cells;
            if (key >= cells) { atomicOr(err, kErrKeyBits); key = cells - 1u; }
            key += P.scenes[sc].base;
        }
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
    const float* wi;         // inverse masses (solids), or null
    float* wo;
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
        if (A.wo) A.wo[i] = A.wi[o];
        const uint32_t k = A.skeys[i];
        if (k < P.table_size) {
            if (i == 0 || A.skeys[i - 1] != k) A.cell_start[k] = i;
            if (i == N - 1 || A.skeys[i + 1] != k) A.cell_end[k] = i + 1;
        }
        if (P.batched) {                         // scene of each sorted slot and each scene's range
            const uint32_t sc = scene_of_key(P, k);
            const uint32_t lo = P.scenes[sc].base, hi = lo + P.scenes[sc].cells;
            P.scene_of[i] = sc;
            if (i == 0 || A.skeys[i - 1] < lo) P.scene_range[2 * sc] = i;
            if (i == N - 1 || A.skeys[i + 1] >= hi) P.scene_range[2 * sc + 1] = i + 1;
        }
    }
}

// Mark empty every cell the tables hold (used when the sorted-key buffer moves).
__global__ void clear_cells_kernel(const uint32_t* __restrict__ old_keys, const uint32_t* __restrict__ table_n,
                                   uint32_t* __restrict__ cell_start, uint32_t table_size) {
    const uint32_t n = *table_n;
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        const uint32_t oc = old_keys[i];
        if (oc < table_size) cell_start[oc] = kEmptyCell;
    }
}

__global__ void fill_u32_kernel(uint32_t* a, uint32_t value, uint32_t first, uint32_t n) {
    for (uint32_t k = blockIdx.x * blockDim.x + threadIdx.x; k < n; k += gridDim.x * blockDim.x) a[first + k] = value;
}

__global__ void fill_float_kernel(float* a, float value, uint32_t n) {
    for (uint32_t k = blockIdx.x * blockDim.x + threadIdx.x; k < n; k += gridDim.x * blockDim.x) a[k] = value;
}

// New particles: ids first..first+n-1 and inverse mass 1 unless given.
__global__ void fill_new_kernel(uint32_t* ids, float* w, int keep_w, uint32_t first, uint32_t n) {
    const uint32_t k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k < n) {
        ids[first + k] = first + k;
        if (!keep_w) w[first + k] = 1.0f;
    }
}

__global__ void add_one_kernel(float4* x, float4* v, float4* col, uint32_t* ids, float* w, uint32_t at,
                               float px, float py, float pz, float dx, float dy, float dz) {
    w[at] = 1.0f;
    x[at] = make_float4(px, py, pz, 0.0f);
    v[at] = make_float4(50.0f * dx, 50.0f * dy, 50.0f * dz, 0.0f);   // Communication.h:27
    if (col) col[at] = make_float4(1.0f, 0.0f, 0.0f, 1.0f);
    if (ids) ids[at] = at;
}

}  // namespace pbd
