// pbd_staged.cuh -- neighbour passes over a shared-memory copy of each block's neighbourhood.
//
// With kernel widths of a few cells (the reference's config.txt regime: poly6 4.1, spiky a few
// particle diameters, kernelWidthNeighbours 2) every particle's list holds ~100-125 entries and
// every entry lies within the kernels' reach.  Reading those entries from the stored list costs
// an index load and a dependent gather per pair.  Here a block of kStageThreads consecutive
// (Morton-sorted) particles instead copies the particles of every cell its members' lists can
// reach -- the box spanned by their anchor cells, widened by the shell count -- into shared
// memory once: positions, the pass's per-neighbour value (lambda_j, v_j) and the sorted index.
// Each thread then walks its own list in the reference's order (findContacts' 27 cells with the
// x offset outer and z inner, then the shells of findNeighbours, Collision.h:11-160; within a cell
// ascending index; self skipped; cap M) over that copy.  The box is laid out with z fastest, so
// the cells of one (x, y) column that follow each other in list order are one contiguous run.
//
// Same entries, same order, same visitor arithmetic as the list walk: the sums are bit-identical.
// A block whose box is too large, holds too many particles or meets a cell range longer than
// kLongRange (the cellEndings[N-1] = N range of SortReorder.h:183-184) walks the stored full list
// instead; particles without a full list are walked by the leading cooperative blocks as in the
// list kernels.
#pragma once
#include "pbd_passes.cuh"

namespace pbd {

constexpr int kStageThreads = 128;
constexpr uint32_t kStageMaxCells = 2048;     // box cells a block may stage
constexpr uint32_t kStageMaxParts = 1216;     // particles a block may stage (6 blocks of 128 threads per SM)
constexpr int kStageMaxReach = 3;             // shells the staged walk supports

// Integer cell coordinate of a position component, as morton_axis computes it before spreading.
__device__ __forceinline__ int cell_coord(float c) { return (int)(uint32_t)fminf(fmaxf(c, 0.0f), 1023.0f); }

// Shells a particle's list reaches (0 = empty list).
__device__ __forceinline__ int list_reach(const DevParams& P) {
    int r = (P.active & PBD_ACTIVE_FIND_CONTACTS) ? 1 : 0;
    if ((P.active & PBD_ACTIVE_FIND_NEIGHBOURS) && (int)P.K > r) r = (int)P.K;
    return r;
}

template <class Ex>
struct StageSmem {
    uint16_t off[kStageMaxCells + 1];   // first staged slot of each box cell (z fastest); off[n] = total
    uint32_t start[kStageMaxCells];     // the cell's first sorted index
    float4 pos[kStageMaxParts];
    Ex ex[kStageMaxParts];
    int box[6];                         // x0, y0, z0, nx, ny, nz
    uint32_t wsum[kStageThreads / 32];
    int red[kStageThreads / 32][6];
    uint32_t box_too_large;             // set before the first barrier that reads it,
    uint32_t long_range;                // each by its own phase: no thread writes a flag others may still read
};

// Stage the neighbourhood of particles [i0, i0 + kStageThreads).  Returns false (for the whole
// block) when the block must walk its stored lists instead.  `fetch(j)` loads the per-neighbour
// value the pass needs.
template <class Ex, class Fetch>
__device__ __forceinline__ bool stage_block(const DevParams& P, uint32_t i0, const float4* __restrict__ pa,
                                            const float4* __restrict__ p, const uint32_t* __restrict__ cs,
                                            const uint32_t* __restrict__ ce, StageSmem<Ex>& sm, Fetch fetch,
                                            uint32_t& own) {
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const uint32_t N = P.N;
    const uint32_t i = i0 + tid;
    const int R = list_reach(P);
    int v[6] = {INT_MAX, INT_MAX, INT_MAX, INT_MIN, INT_MIN, INT_MIN};   // lo xyz, hi xyz
    if (i < N) {
        const float4 a = pa[i];
        v[0] = cell_coord(__fmaf_rn((float)-R, P.d, a.x));
        v[1] = cell_coord(__fmaf_rn((float)-R, P.d, a.y));
        v[2] = cell_coord(__fmaf_rn((float)-R, P.d, a.z));
        v[3] = cell_coord(__fmaf_rn((float)R, P.d, a.x));
        v[4] = cell_coord(__fmaf_rn((float)R, P.d, a.y));
        v[5] = cell_coord(__fmaf_rn((float)R, P.d, a.z));
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
#pragma unroll
        for (int k = 0; k < 3; ++k) v[k] = min(v[k], __shfl_xor_sync(kFullMask, v[k], o));
#pragma unroll
        for (int k = 3; k < 6; ++k) v[k] = max(v[k], __shfl_xor_sync(kFullMask, v[k], o));
    }
    if (lane == 0)
#pragma unroll
        for (int k = 0; k < 6; ++k) sm.red[warp][k] = v[k];
    if (tid == 0) { sm.box_too_large = 0u; sm.long_range = 0u; }
    __syncthreads();
    if (tid == 0) {
        int b[6];
#pragma unroll
        for (int k = 0; k < 6; ++k) b[k] = sm.red[0][k];
        for (int w = 1; w < kStageThreads / 32; ++w) {
            for (int k = 0; k < 3; ++k) b[k] = min(b[k], sm.red[w][k]);
            for (int k = 3; k < 6; ++k) b[k] = max(b[k], sm.red[w][k]);
        }
        const int nx = b[3] - b[0] + 1, ny = b[4] - b[1] + 1, nz = b[5] - b[2] + 1;
        sm.box[0] = b[0]; sm.box[1] = b[1]; sm.box[2] = b[2];
        sm.box[3] = nx; sm.box[4] = ny; sm.box[5] = nz;
        if ((uint64_t)nx * ny * nz > kStageMaxCells) sm.box_too_large = 1u;
    }
    __syncthreads();
    if (sm.box_too_large) return false;
    const int x0 = sm.box[0], y0 = sm.box[1], z0 = sm.box[2], ny = sm.box[4], nz = sm.box[5];
    const uint32_t ncells = (uint32_t)(sm.box[3] * ny * nz);
    const bool quirk = (P.flags & PBD_FLAG_CELL_END_QUIRK) && N >= 2;
    // cell ranges: each thread a contiguous chunk of cells, then a block scan of the chunk sums
    const uint32_t chunk = (ncells + kStageThreads - 1) / kStageThreads;
    const uint32_t c0 = min((uint32_t)tid * chunk, ncells), c1 = min(c0 + chunk, ncells);
    uint32_t mine = 0, bad = 0;
    for (uint32_t c = c0; c < c1; ++c) {
        const int z = (int)(c % (uint32_t)nz), t = (int)(c / (uint32_t)nz), y = t % ny, x = t / ny;
        const uint32_t h = (expand_bits((uint32_t)(x0 + x)) << 2) + (expand_bits((uint32_t)(y0 + y)) << 1) +
                           expand_bits((uint32_t)(z0 + z));
        uint32_t s = kEmptyCell, len = 0;
        if (h < P.G) {
            s = __ldg(cs + h);
            if (s < N) {
                uint32_t e = __ldg(ce + h);
                if ((quirk && h == N - 1) || e > N) e = N;   // entries >= N are skipped (Collision.h:59)
                len = e > s ? e - s : 0u;
            }
        }
        if (len > kLongRange) bad = 1u;
        sm.start[c] = s;
        sm.off[c] = (uint16_t)len;   // the length for now, the offset after the scan
        mine += len;
    }
    // exclusive scan of the chunk sums
    uint32_t x = mine;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const uint32_t y = __shfl_up_sync(kFullMask, x, o);
        if (lane >= o) x += y;
    }
    if (lane == 31) sm.wsum[warp] = x;
    if (bad) sm.long_range = 1u;
    __syncthreads();
    uint32_t before = 0, total = 0;
#pragma unroll
    for (int w = 0; w < kStageThreads / 32; ++w) {
        if (w < warp) before += sm.wsum[w];
        total += sm.wsum[w];
    }
    if (sm.long_range || total > kStageMaxParts) return false;
    uint32_t run = before + x - mine;
    for (uint32_t c = c0; c < c1; ++c) {
        const uint32_t len = sm.off[c];
        sm.off[c] = (uint16_t)run;
        run += len;
    }
    if (tid == kStageThreads - 1) sm.off[ncells] = (uint16_t)total;
    __syncthreads();
    // copy: one thread per slot (its cell by binary search over the offsets), loads of four slots
    // in flight at once
    for (uint32_t k0 = tid; k0 < total; k0 += 4 * kStageThreads) {
        uint32_t j[4];
#pragma unroll
        for (int u = 0; u < 4; ++u) {
            const uint32_t k = k0 + u * kStageThreads;
            j[u] = 0xFFFFFFFFu;
            if (k < total) {
                uint32_t lo = 0, hi = ncells;   // the last cell with off <= k
                while (hi - lo > 1) {
                    const uint32_t mid = (lo + hi) >> 1;
                    if (sm.off[mid] <= k) lo = mid; else hi = mid;
                }
                j[u] = sm.start[lo] + (k - sm.off[lo]);
            }
        }
#pragma unroll
        for (int u = 0; u < 4; ++u) {
            const uint32_t k = k0 + u * kStageThreads;
            if (k < total) {
                sm.pos[k] = __ldg(p + j[u]);
                sm.ex[k] = fetch(j[u]);
            }
        }
    }
    // this thread's own slot (its list skips it): its cell's first slot + its place in the cell
    own = 0xFFFFu;
    if (i < N) {
        const float4 a = pa[i];
        const int cx = cell_coord(a.x) - x0, cy = cell_coord(a.y) - y0, cz = cell_coord(a.z) - z0;
        const uint32_t c = (uint32_t)((cx * ny + cy) * nz + cz);
        const uint32_t st = sm.start[c];
        if (st <= i && i - st < (uint32_t)(sm.off[c + 1] - sm.off[c])) own = sm.off[c] + (i - st);
    }
    __syncthreads();
    return true;
}

// Particle i's list over the staged box, in the reference's order, with the cap M.  `pa_i` is
// the particle's anchor.  Returns the list length.
// Box-relative cell coordinate at offsets -R..R of one axis: base + a + R where every offset lands
// one cell after the previous one (the usual case), else computed with the reference's float rule.
struct AxisCells {
    int base;        // coordinate at offset -R
    bool regular;
    float p;
    int o;           // box origin
    __device__ __forceinline__ int at(const DevParams& P, int a, int R) const {
        return regular ? base + a + R : cell_coord(__fmaf_rn((float)a, P.d, p)) - o;
    }
};
__device__ __forceinline__ AxisCells axis_cells(const DevParams& P, float p, int o, int R) {
    AxisCells ax{cell_coord(__fmaf_rn((float)-R, P.d, p)) - o, true, p, o};
    for (int a = -R; a < R; ++a)
        ax.regular = ax.regular && cell_coord(__fmaf_rn((float)(a + 1), P.d, p)) == cell_coord(__fmaf_rn((float)a, P.d, p)) + 1;
    return ax;
}

// Particle i's list over the staged box, in the reference's order, with the cap M.  `pa_i` is
// the particle's anchor, `own` its staged slot.  Returns the list length.
template <class V, class Ex>
__device__ __forceinline__ uint32_t walk_staged(const DevParams& P, float4 pa_i, uint32_t own, const StageSmem<Ex>& sm,
                                                V& vis) {
    const uint32_t M = P.M;
    if (M == 0) return 0;
    const int R = list_reach(P);
    const int ny = sm.box[4], nz = sm.box[5];
    const AxisCells X = axis_cells(P, pa_i.x, sm.box[0], R), Y = axis_cells(P, pa_i.y, sm.box[1], R),
                    Z = axis_cells(P, pa_i.z, sm.box[2], R);
    uint32_t cnt = 0;
    // the staged slots [s0, s1); returns true when the cap is reached
    auto run = [&](uint32_t s0, uint32_t s1, bool contact) -> bool {
#pragma unroll 2
        for (uint32_t k = s0; k < s1; ++k) {
            if (k == own) continue;
            vis.add(contrib_of(vis, 0u, sm.pos[k], sm.ex[k], contact), contact);
            if (++cnt == M) return true;
        }
        return false;
    };
    // cells c_lo..c_hi (offsets) of column (a, b): one run when their cells follow each other
    auto column = [&](int a, int b, int c_lo, int c_hi, bool contact) -> bool {
        const int col = (X.at(P, a, R) * ny + Y.at(P, b, R)) * nz;
        if (Z.regular || c_lo == c_hi) {
            const int f = col + Z.at(P, c_lo, R), l = col + Z.at(P, c_hi, R);
            return run(sm.off[f], sm.off[l + 1], contact);
        }
        for (int c = c_lo; c <= c_hi; ++c) {
            const int f = col + Z.at(P, c, R);
            if (run(sm.off[f], sm.off[f + 1], contact)) return true;
        }
        return false;
    };
    if (P.active & PBD_ACTIVE_FIND_CONTACTS) {
        for (int a = -1; a <= 1; ++a)
            for (int b = -1; b <= 1; ++b)
                if (column(a, b, -1, 1, true)) return cnt;
    }
    vis.end_contacts(cnt);
    if (P.active & PBD_ACTIVE_FIND_NEIGHBOURS) {
        const int K = (int)P.K;
        for (int sh = 2; sh <= K; ++sh)
            for (int a = -sh; a <= sh; ++a)
                for (int b = -sh; b <= sh; ++b) {
                    if (a == sh || a == -sh || b == sh || b == -sh) {
                        if (column(a, b, -sh, sh, false)) return cnt;
                    } else {
                        if (column(a, b, -sh, -sh, false)) return cnt;
                        if (column(a, b, sh, sh, false)) return cnt;
                    }
                }
    }
    return cnt;
}

// Whether the staged kernels may take a frame's passes: one scene, reach within kStageMaxReach.
__host__ __forceinline__ bool staged_supported(const DevParams& P) {
    int r = (P.active & PBD_ACTIVE_FIND_CONTACTS) ? 1 : 0;
    if ((P.active & PBD_ACTIVE_FIND_NEIGHBOURS) && (int)P.K > r) r = (int)P.K;
    return !P.batched && r >= 1 && r <= kStageMaxReach;
}

// computeLambda over the staged neighbourhood (the frame's later lambda passes).
__global__ void __launch_bounds__(kStageThreads, 6)
lambda_staged_kernel(DevParams P, const float4* __restrict__ p, const float4* __restrict__ pa,
                     const uint32_t* __restrict__ cs, const uint32_t* __restrict__ ce, float* __restrict__ lambda,
                     CoopSet C, NbList F) {
    __shared__ StageSmem<NoExtra> sm;
    if (blockIdx.x < C.blocks) {
        run_coop_set(C, [&](uint32_t i) { coop_lambda(P, p, pa, cs, ce, lambda, nullptr, i); });
        return;
    }
    const uint32_t i0 = (blockIdx.x - C.blocks) * kStageThreads;
    uint32_t own;
    const bool staged = stage_block(P, i0, pa, p, cs, ce, sm, [&](uint32_t) { return NoExtra{}; }, own);
    const uint32_t i = i0 + threadIdx.x;
    if (i >= P.N) return;
    const uint32_t fm = F.meta[i];
    if (fm == kListOff) return;   // walked by the cooperative blocks
    const float4 pi = p[i];
    LambdaVisit vis(P, pi);
    if (staged) walk_staged(P, pa[i], own, sm, vis);
    else walk_list(F, i, fm, p, vis);
    lambda[i] = vis.finish(P.rho0);
}

// computeDeltaPositions + solveCollisions + applyDeltaPositions (+ updatePositions) over the
// staged neighbourhood.
template <uint32_t kMode>
__global__ void __launch_bounds__(kStageThreads, 6)
delta_staged_kernel(DevParams P, uint32_t mode_rt, const float4* __restrict__ pin, const float4* __restrict__ pa,
                    float4* __restrict__ pout, float4* __restrict__ x, float4* __restrict__ v,
                    const float* __restrict__ lambda, const float* __restrict__ w, float4* __restrict__ delta,
                    const uint32_t* __restrict__ cs, const uint32_t* __restrict__ ce, CoopSet C, NbList F) {
    __shared__ StageSmem<float> sm;
    const uint32_t mode = kMode ? kMode : mode_rt;
    if (blockIdx.x < C.blocks) {
        run_coop_set(C, [&](uint32_t i) { coop_delta(P, mode, pin, pa, pout, x, v, lambda, w, delta, cs, ce, i); });
        return;
    }
    const uint32_t i0 = (blockIdx.x - C.blocks) * kStageThreads;
    const bool dd = (mode & kDoDelta) != 0;
    uint32_t own;
    const bool staged = stage_block(P, i0, pa, pin, cs, ce, sm,
                                    [&](uint32_t j) { return dd ? __ldg(lambda + j) : 0.0f; }, own);
    const uint32_t i = i0 + threadIdx.x;
    if (i >= P.N) return;
    const uint32_t fm = F.meta[i];
    if (fm == kListOff) return;   // walked by the cooperative blocks
    const float4 pi = pin[i];
    const bool need_x = (mode & (kDoCollide | kDoUpdate)) != 0;
    const float4 xi = need_x ? x[i] : make_float4(0.f, 0.f, 0.f, 0.f);
    const float li = dd ? lambda[i] : 0.f;
    DeltaVisit vis(P, lambda, w, pi, li, w ? w[i] : 1.0f, dd, (mode & kDoCollide) != 0, xi);
    if (staged) walk_staged(P, pa[i], own, sm, vis);
    else walk_list<false, kListBatch>(F, i, fm, pin, vis);
    delta_finish(P, P.rho0, mode, i, vis, pout, x, v, delta);
}

}  // namespace pbd
