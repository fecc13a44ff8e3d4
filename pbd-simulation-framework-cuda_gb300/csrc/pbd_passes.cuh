// pbd_passes.cuh -- the neighbour passes of a frame.
//
// The reference builds an explicit N x M list once per frame (findContacts +
// findNeighbours, kernel/Collision.h:11-160) and every density/vorticity/viscosity kernel
// loops over it (kernel/Density.h).  Here the frame's first lambda pass walks the cells in
// exactly the order the list would hold them (27 cells with the x offset outer and z inner,
// then the shells of findNeighbours), skipping self and stopping at the cap M, and stores the
// result (the full list); later passes read the stored lists, so sums run in the list's order.
//
// Each pass is split into a per-candidate contribution (`contrib`) and an in-order
// accumulation (`add`); a visitor may also name per-neighbour data (`Extra`, loaded by
// `fetch(j)`) that the walkers load together with the neighbour's position.  Three walkers
// drive them:
//  - walk_seq: one thread per particle over the cells;
//  - walk_coop: one warp per particle.  Lanes evaluate 32 candidates at once and the
//    contributions are added in list order through shuffles, so the result is bit-identical
//    to walk_seq.  It takes the particles whose walk meets a cell range longer than
//    kLongRange -- in practice the range that SortReorder.h:183-184 extends to N (up to M
//    entries) -- which would otherwise serialise a whole warp behind one thread;
//  - walk_list: one thread per particle over a stored list.
#pragma once
#include <type_traits>
#include "pbd_device.cuh"
#include "../../include/pbd.h"

namespace pbd {

// Per-neighbour data a visitor loads with the neighbour's position: V::Extra and V::fetch(j)
// when the visitor declares them, nothing otherwise.
struct NoExtra {};
template <class V, class = void> struct ExtraOf { using type = NoExtra; static constexpr bool has = false; };
template <class V> struct ExtraOf<V, std::void_t<typename V::Extra>> {
    using type = typename V::Extra;
    static constexpr bool has = true;
};
template <class V>
__device__ __forceinline__ typename ExtraOf<V>::type fetch_extra(const V& vis, uint32_t j) {
    if constexpr (ExtraOf<V>::has) return vis.fetch(j);
    else return NoExtra{};
}
template <class V>
__device__ __forceinline__ typename V::Contrib contrib_of(V& vis, uint32_t j, const float4& pj,
                                                          const typename ExtraOf<V>::type& ex, bool contact) {
    if constexpr (ExtraOf<V>::has) return vis.contrib(j, pj, ex, contact);
    else return vis.contrib(j, pj, contact);
}

constexpr uint32_t kLongRange = 32;
constexpr uint32_t kFullMask = 0xffffffffu;

__device__ __forceinline__ uint32_t lane_id() { return threadIdx.x & 31u; }
__device__ __forceinline__ uint32_t lanemask_lt_u() {
    uint32_t m;
    asm("mov.u32 %0, %%lanemask_lt;" : "=r"(m));
    return m;
}

// Particles whose walk is handed to the warp-cooperative kernel.
struct DeferList {
    uint32_t* items;
    uint32_t* count;
    uint32_t* done;
    uint32_t cap;
};

// Stored lists, both in the reference's list order, slot-major.
//  - The full list: the frame's first lambda pass walks the cells once (the cells come from the
//    frame's anchors, so the list is fixed for the frame) and stores every entry, up to the cap
//    M; the later lambda passes, omega and vorticity read it instead of the cell tables.
//  - The near list: a lambda or omega pass keeps the entries within the cut (r^2 < cut2 at the
//    positions it read); the pass right after it reads the same positions (delta after lambda,
//    viscosity after omega), so every entry left out adds an exact zero there and the short
//    list gives the full walk's sums bit for bit.
// A particle whose list does not fit (or whose walk met a long cell range) walks the cells.
constexpr uint32_t kListOff = 0x80000000u;   // meta: this particle walks the cells
struct NbList {
    uint32_t* list;      // kmax x stride entries, slot-major (slot k of particle i at k * stride + i)
    uint32_t* meta;      // per particle: count | contacts << 8, or kListOff
    uint32_t stride;
    uint32_t kmax;       // <= 255
};

// Enumerate the non-empty cell ranges [s, e) of particle i's list in the reference's
// order.  f(s, e, contact) returns true to stop; end_contacts(n) marks the end of the
// 27-cell part (Collision.h:38-39).  `pi` is the particle's anchor: its predicted position
// right after the frame's re-order, from which the reference builds the list once per frame
// (findContacts/findNeighbours run before the solver loop, Fluid.cu:41-47); passes later in
// the frame use the moved positions for the physics but the anchor's cells.
template <class F, class G>
__device__ __forceinline__ void for_each_range(const DevParams& P, const SceneCtx& S, float4 pi, const uint32_t* __restrict__ cs,
                                               const uint32_t* __restrict__ ce, F& f, G& end_contacts) {
    const uint32_t N = P.N;     // table starts >= N mark empty cells
    const bool quirk = (P.flags & PBD_FLAG_CELL_END_QUIRK) && S.n >= 2;
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
                // the column's three cells: all six table loads in flight before the walk
                uint32_t h[3], cs3[3], ce3[3];
#pragma unroll
                for (int c = 0; c < 3; ++c) {
                    h[c] = hxy + mz[c];
                    cs3[c] = h[c] < S.cells ? __ldg(cs + S.base + h[c]) : kEmptyCell;
                }
#pragma unroll
                for (int c = 0; c < 3; ++c) ce3[c] = h[c] < S.cells ? __ldg(ce + S.base + h[c]) : 0u;
#pragma unroll
                for (int c = 0; c < 3; ++c) {
                    if (cs3[c] >= N) continue;
                    const uint32_t e = ((quirk && h[c] == S.n - 1) || ce3[c] > S.end) ? S.end : ce3[c];
                    if (f(cs3[c], e, true)) return;
                }
            }
        }
    }
    if (end_contacts()) return;
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
                        if (h >= S.cells) continue;
                        const uint32_t s = __ldg(cs + S.base + h);
                        uint32_t e = __ldg(ce + S.base + h);
                        if (s >= N) continue;
                        if ((quirk && h == S.n - 1) || e > S.end) e = S.end;   // entries >= N are skipped (Collision.h:142)
                        if (f(s, e, false)) return;
                    }
                }
            }
        }
    }
}

// One thread per particle.  Returns the list length; sets *deferred (and stops) when a
// range longer than kLongRange is met and `defer` is set.  `anchor` selects the cells, `p`
// holds the current positions.
template <class V>
__device__ __forceinline__ uint32_t walk_seq(const DevParams& P, const SceneCtx& S, uint32_t i, float4 anchor,
                                             const float4* __restrict__ p, const uint32_t* __restrict__ cs,
                                             const uint32_t* __restrict__ ce, V& vis, bool defer, bool* deferred) {
    const uint32_t M = P.M;
    uint32_t cnt = 0;
    if (M == 0) return 0;
    auto range = [&](uint32_t s, uint32_t e, bool contact) -> bool {
        if (defer && e - s > kLongRange) { *deferred = true; return true; }
        for (uint32_t j = s; j < e; ++j) {
            if (j == i) continue;
            vis.add(contrib_of(vis, j, __ldg(p + j), fetch_extra(vis, j), contact), contact);
            if (++cnt == M) return true;
        }
        return false;
    };
    auto endc = [&]() -> bool { vis.end_contacts(cnt); return false; };
    for_each_range(P, S, anchor, cs, ce, range, endc);
    return cnt;
}

// One warp per particle (all 32 lanes call it with the same i).  Same list, same order.
template <class V>
__device__ __forceinline__ uint32_t walk_coop(const DevParams& P, const SceneCtx& S, uint32_t i, float4 anchor,
                                              const float4* __restrict__ p, const uint32_t* __restrict__ cs,
                                              const uint32_t* __restrict__ ce, V& vis) {
    const uint32_t M = P.M;
    const uint32_t lane = lane_id(), lt = lanemask_lt_u();
    uint32_t cnt = 0;
    if (M == 0) return 0;
    auto range = [&](uint32_t s, uint32_t e, bool contact) -> bool {
        for (uint32_t c0 = s; c0 < e; c0 += 32u) {
            const uint32_t j = c0 + lane;
            bool valid = j < e && j != i;
            const uint32_t b = __ballot_sync(kFullMask, valid);
            valid = valid && __popc(b & lt) < M - cnt;
            typename V::Contrib c = valid ? contrib_of(vis, j, __ldg(p + j), fetch_extra(vis, j), contact) : V::zero();
            const uint32_t n = __popc(__ballot_sync(kFullMask, valid));
            // only entries whose contribution changes a sum are added (in order); the others
            // are exact no-ops of add() and still count toward the cap
            uint32_t take = __ballot_sync(kFullMask, valid && V::effective(c));
            while (take) {
                const int k = __ffs(take) - 1;
                take &= take - 1u;
                vis.add(V::shfl(c, k), contact);
            }
            cnt += n;
            if (cnt == M) return true;
        }
        return false;
    };
    auto endc = [&]() -> bool { vis.end_contacts(cnt); return false; };
    for_each_range(P, S, anchor, cs, ce, range, endc);
    return cnt;
}

// One thread per particle over a stored list (meta not kListOff): the contact entries, then
// end_contacts, then the rest.  Entries go in batches of B: the batch's position (and extra)
// loads are all in flight before the first contribution, and the next batch's indices are
// loaded while this one is summed.
// Every visitor adds its contributions with explicitly rounded operations (__fadd_rn, or
// __fmaf_rn where a product goes into the sum), which the compiler never contracts, so the sums
// get the same bits whichever walker (cells, stored list, cooperative warp) and whichever loop
// shape the compiler sees.
//
// kOwn: the list was written by this thread in this kernel, so it is read with ordinary
// (coherent) loads rather than through the read-only path.  Otherwise the list entries are
// read with the streaming hint (ld.global.cs: evict first): each is read once per pass, and
// the cache lines they would take are worth more to the neighbour positions gathered next
// (3% off the frame on fluid_1m).
// Batch sizes measured on fluid_1m (1M particles, GB300): full lists 4 (2, 3, 6 and 8 were
// slower), near lists 1 (2, 3 and 8 slower; a deeper software pipeline too).
constexpr uint32_t kListBatch = 4;   // full lists (~32 entries)
constexpr uint32_t kNearBatch = 1;   // near lists (~6 entries)
template <bool kOwn = false, uint32_t B = kListBatch, class V>
__device__ __forceinline__ void walk_list_part(const NbList& L, uint32_t i, uint32_t k0, uint32_t k1, bool contact,
                                               const float4* __restrict__ p, V& vis) {
    const size_t st = L.stride;
    const uint32_t* e = L.list + i + (size_t)k0 * st;   // entry k0; each batch moves it by B entries
    uint32_t jn[B];
#pragma unroll
    for (uint32_t b = 0; b < B; ++b) {
        const uint32_t* a = e + b * st;
        jn[b] = (k0 + b < k1) ? (kOwn ? *a : __ldcs(a)) : i;
    }
#pragma unroll 1
    for (uint32_t kb = k0; kb < k1; kb += B) {
        uint32_t j[B];
        float4 pj[B];
        typename ExtraOf<V>::type ex[B];
#pragma unroll
        for (uint32_t b = 0; b < B; ++b) j[b] = jn[b];
#pragma unroll
        for (uint32_t b = 0; b < B; ++b) {
            pj[b] = __ldg(p + j[b]);
            ex[b] = fetch_extra(vis, j[b]);
        }
        e += B * st;
#pragma unroll
        for (uint32_t b = 0; b < B; ++b) {
            const uint32_t* a = e + b * st;
            jn[b] = (kb + B + b < k1) ? (kOwn ? *a : __ldcs(a)) : i;
        }
#pragma unroll
        for (uint32_t b = 0; b < B; ++b)
            if (kb + b < k1) vis.add(contrib_of(vis, j[b], pj[b], ex[b], contact), contact);
    }
}
template <bool kOwn = false, uint32_t B = kListBatch, class V>
__device__ __forceinline__ void walk_list(const NbList& L, uint32_t i, uint32_t meta, const float4* __restrict__ p, V& vis) {
    const uint32_t n = meta & 0xFFu, nc = (meta >> 8) & 0xFFu;
    walk_list_part<kOwn, B>(L, i, 0u, nc, true, p, vis);
    vis.end_contacts(nc);
    walk_list_part<kOwn, B>(L, i, nc, n, false, p, vis);
}
// A near list (~6 entries): one entry at a time, the next entry's index in flight.
template <bool kOwn = false, class V>
__device__ __forceinline__ void walk_near(const NbList& L, uint32_t i, uint32_t meta, const float4* __restrict__ p, V& vis) {
    walk_list<kOwn, kNearBatch>(L, i, meta, p, vis);
}

// Particle i's near list from its full list (meta fm): the entries with r^2 < cut2 at p, in
// list order, the boundary of the contact entries kept.  No sums: a pass then walks the near
// list alone (every entry left out adds an exact zero to every sum of a lambda, omega or delta
// pass), so the warp runs the kernel arithmetic for ~6 entries per particle instead of ~32.
// Returns the near list's meta (kListOff when it does not fit).
// kStepped: entry and output addresses stepped by the strides instead of a product per entry
// (lambda_list_kernel: 7.6% faster on fluid_1m; omega_list_kernel's 40-register budget takes
// the two extra pointers badly: 8.8% slower there, so it keeps the products).
template <bool kOwn = false, bool kStepped = false>
__device__ __forceinline__ uint32_t filter_list(const NbList& F, uint32_t fm, const NbList& L, uint32_t i,
                                                const float4& pi, float cut2, const float4* __restrict__ p) {
    const uint32_t n = fm & 0xFFu, nc = (fm >> 8) & 0xFFu;
    const size_t st = F.stride, ost = L.stride;
    const uint32_t* e = F.list + i;
    uint32_t* o = L.list + i;
    uint32_t m = 0, mc = 0;
    uint32_t jn[kListBatch];
#pragma unroll
    for (uint32_t b = 0; b < kListBatch; ++b) {
        const uint32_t* a = e + b * st;
        jn[b] = (b < n) ? (kOwn ? *a : __ldcs(a)) : i;
    }
#pragma unroll 1
    for (uint32_t kb = 0; kb < n; kb += kListBatch) {
        uint32_t j[kListBatch];
        float4 pj[kListBatch];
#pragma unroll
        for (uint32_t b = 0; b < kListBatch; ++b) j[b] = jn[b];
#pragma unroll
        for (uint32_t b = 0; b < kListBatch; ++b) pj[b] = __ldg(p + j[b]);
        if constexpr (kStepped) e += kListBatch * st;
#pragma unroll
        for (uint32_t b = 0; b < kListBatch; ++b) {
            const uint32_t* a = kStepped ? e + b * st : F.list + i + (size_t)(kb + kListBatch + b) * F.stride;
            jn[b] = (kb + kListBatch + b < n) ? (kOwn ? *a : __ldcs(a)) : i;
        }
#pragma unroll
        for (uint32_t b = 0; b < kListBatch; ++b) {
            if (kb + b == nc) mc = m;
            if (kb + b < n) {
                const float rx = pi.x - pj[b].x, ry = pi.y - pj[b].y, rz = pi.z - pj[b].z;
                if (dist2(rx, ry, rz) < cut2) {
                    if (m < L.kmax) {
                        if constexpr (kStepped) { *o = j[b]; o += ost; }
                        else L.list[(size_t)m * L.stride + i] = j[b];
                    }
                    ++m;
                }
            }
        }
    }
    if (nc >= n) mc = m;
    return m > L.kmax ? kListOff : (m | (mc << 8));
}

// Wraps the visitor of a walking pass and keeps particle i's near list (when `list` is set)
// and its full list (when `flist` is set) as the walk goes.  Holds everything by value so the
// visitor stays in registers.
template <class V>
struct Recorder {
    using Contrib = typename V::Contrib;
    using Extra = typename ExtraOf<V>::type;
    V inner;
    uint32_t* list;
    uint32_t* flist;
    uint32_t stride, fstride, kmax, fkmax, i;
    float4 pi;
    float cut2;
    uint32_t n = 0, nc = 0xFFFFFFFFu, fn = 0, fnc = 0xFFFFFFFFu;
    __device__ Recorder(const V& v, const NbList& L, const NbList& F, bool full, uint32_t i_, float4 p_i, float c2)
        : inner(v), list(L.list), flist(full ? F.list : nullptr), stride(L.stride), fstride(F.stride), kmax(L.kmax),
          fkmax(F.kmax), i(i_), pi(p_i), cut2(c2) {}
    __device__ static Contrib zero() { return V::zero(); }
    __device__ __forceinline__ void end_contacts(uint32_t c) { nc = n; fnc = fn; inner.end_contacts(c); }
    __device__ __forceinline__ Extra fetch(uint32_t j) const { return fetch_extra(inner, j); }
    __device__ __forceinline__ Contrib contrib(uint32_t j, const float4& pj, const Extra& ex, bool contact) {
        if (flist) {
            if (fn < fkmax) flist[(size_t)fn * fstride + i] = j;
            ++fn;
        }
        if (list) {
            const float rx = pi.x - pj.x, ry = pi.y - pj.y, rz = pi.z - pj.z;
            if (dist2(rx, ry, rz) < cut2) {
                if (n < kmax) list[(size_t)n * stride + i] = j;
                ++n;
            }
        }
        return contrib_of(inner, j, pj, ex, contact);
    }
    __device__ __forceinline__ void add(const Contrib& c, bool contact) { inner.add(c, contact); }
    __device__ __forceinline__ uint32_t meta() const {
        const uint32_t c = nc == 0xFFFFFFFFu ? n : nc;
        return n > kmax ? kListOff : (n | (c << 8));
    }
    __device__ __forceinline__ uint32_t fmeta() const {
        const uint32_t c = fnc == 0xFFFFFFFFu ? fn : fnc;
        return fn > fkmax ? kListOff : (fn | (c << 8));
    }
};

// A walk that only stores particle i's full list: indices, no positions (the walk's position
// loads are dead and vanish), the boundary of the contact entries kept.
struct ListRecorder {
    struct Contrib {};
    uint32_t* list;
    uint32_t stride, kmax, i;
    uint32_t n = 0, nc = 0xFFFFFFFFu;
    __device__ ListRecorder(const NbList& F, uint32_t i_) : list(F.list), stride(F.stride), kmax(F.kmax), i(i_) {}
    __device__ static Contrib zero() { return Contrib{}; }
    __device__ static bool effective(const Contrib&) { return false; }
    __device__ static Contrib shfl(const Contrib& c, int) { return c; }
    __device__ __forceinline__ void end_contacts(uint32_t) { nc = n; }
    __device__ __forceinline__ Contrib contrib(uint32_t j, const float4&, bool) {
        if (n < kmax) list[(size_t)n * stride + i] = j;
        ++n;
        return Contrib{};
    }
    __device__ __forceinline__ void add(const Contrib&, bool) {}
    __device__ __forceinline__ uint32_t meta() const {
        const uint32_t c = nc == 0xFFFFFFFFu ? n : nc;
        return n > kmax ? kListOff : (n | (c << 8));
    }
};


// The frame's full list of particle i for a 27-cell neighbourhood (kernelWidthNeighbours 1,
// findContacts on), indices only: the entries, order, cap M, self-skip and long-range hand-over
// of walk_seq over for_each_range, with the three cells of a column stored by one loop.
// Returns the list's meta (kListOff when it does not fit or the particle is handed over; then
// *deferred tells which).
__device__ __forceinline__ uint32_t store_full_list(const DevParams& P, const SceneCtx& S, uint32_t i, float4 pa,
                                                    const uint32_t* __restrict__ cs, const uint32_t* __restrict__ ce,
                                                    const NbList& F, bool* deferred) {
    const uint32_t N = P.N, M = P.M;
    if (M == 0) return 0u;
    const bool quirk = (P.flags & PBD_FLAG_CELL_END_QUIRK) && S.n >= 2;
    uint32_t mx[3], my[3], mz[3];
#pragma unroll
    for (int c = 0; c < 3; ++c) {
        mx[c] = morton_axis(__fmaf_rn((float)(c - 1), P.d, pa.x)) << 2;
        my[c] = morton_axis(__fmaf_rn((float)(c - 1), P.d, pa.y)) << 1;
        mz[c] = morton_axis(__fmaf_rn((float)(c - 1), P.d, pa.z));
    }
    uint32_t* out = F.list + i;
    uint32_t n = 0;
#pragma unroll 1
    for (int col = 0; col < 9; ++col) {
        const int a = col / 3, b = col - 3 * (col / 3);
        const uint32_t hxy = (a == 0 ? mx[0] : (a == 1 ? mx[1] : mx[2])) + (b == 0 ? my[0] : (b == 1 ? my[1] : my[2]));
        uint32_t h[3], s3[3], e3[3];
#pragma unroll
        for (int c = 0; c < 3; ++c) {
            h[c] = hxy + mz[c];
            s3[c] = h[c] < S.cells ? __ldg(cs + S.base + h[c]) : kEmptyCell;
        }
#pragma unroll
        for (int c = 0; c < 3; ++c) e3[c] = h[c] < S.cells ? __ldg(ce + S.base + h[c]) : 0u;
        uint32_t len[3];
        uint32_t reach = n;   // entries stored before the cell: the walk reaches it while below the cap
#pragma unroll
        for (int c = 0; c < 3; ++c) {
            const bool valid = s3[c] < N;
            const uint32_t e = ((quirk && h[c] == S.n - 1) || e3[c] > S.end) ? S.end : e3[c];
            len[c] = valid ? e - s3[c] : 0u;
            if (valid && reach < M && len[c] > kLongRange) { *deferred = true; return kListOff; }
            reach += len[c] - ((valid && s3[c] <= i && i < e) ? 1u : 0u);
        }
        const uint32_t l01 = len[0] + len[1], T = l01 + len[2];
        if (reach < M && reach <= F.kmax) {   // the column fits below the cap and the list's room
            uint32_t* o = out + (size_t)n * F.stride;
#pragma unroll 1
            for (uint32_t t = 0; t < T; ++t) {
                const uint32_t j = t < len[0] ? s3[0] + t : (t < l01 ? s3[1] + (t - len[0]) : s3[2] + (t - l01));
                if (j == i) continue;
                *o = j;
                o += F.stride;
            }
            n = reach;
            continue;
        }
#pragma unroll 1
        for (uint32_t t = 0; t < T; ++t) {
            const uint32_t j = t < len[0] ? s3[0] + t : (t < l01 ? s3[1] + (t - len[0]) : s3[2] + (t - l01));
            if (j == i) continue;
            if (n < F.kmax) out[(size_t)n * F.stride] = j;
            if (++n == M) return n > F.kmax ? kListOff : (n | (n << 8));
        }
    }
    return n > F.kmax ? kListOff : (n | (n << 8));
}

// The cells of one group of particle i's list (the 3 cells of a findContacts column, or the cells
// of a findNeighbours column: 2 sh + 1 on an edge column, 2 otherwise), stored into the full list:
// all table loads in flight first, then the entries in list order, skipping self, with the cap M,
// the list's room and the long-range hand-over of walk_seq.  Returns true when the walk ends here
// (cap reached or handed over).
template <int kMax>
__device__ __forceinline__ bool store_cell_group(const DevParams& P, const SceneCtx& S, uint32_t i, const uint32_t* h,
                                                 int ncell, const uint32_t* __restrict__ cs,
                                                 const uint32_t* __restrict__ ce, const NbList& F, bool quirk,
                                                 uint32_t& n, bool* deferred) {
    const uint32_t N = P.N, M = P.M;
    uint32_t s[kMax], e[kMax], len[kMax];
#pragma unroll
    for (int c = 0; c < kMax; ++c) s[c] = (c < ncell && h[c] < S.cells) ? __ldg(cs + S.base + h[c]) : kEmptyCell;
#pragma unroll
    for (int c = 0; c < kMax; ++c) e[c] = (c < ncell && h[c] < S.cells) ? __ldg(ce + S.base + h[c]) : 0u;
    uint32_t reach = n;   // entries stored before the cell: the walk reaches it while below the cap
#pragma unroll
    for (int c = 0; c < kMax; ++c) {
        const bool valid = c < ncell && s[c] < N;
        const uint32_t ec = ((quirk && h[c] == S.n - 1) || e[c] > S.end) ? S.end : e[c];
        len[c] = valid ? ec - s[c] : 0u;
        if (valid && reach < M && len[c] > kLongRange) { *deferred = true; return true; }
        reach += len[c] - ((valid && s[c] <= i && i < ec) ? 1u : 0u);
    }
    uint32_t* out = F.list + i;
    if (reach < M && reach <= F.kmax) {   // the group fits below the cap and the list's room
        uint32_t* o = out + (size_t)n * F.stride;
#pragma unroll
        for (int c = 0; c < kMax; ++c)
#pragma unroll 1
            for (uint32_t t = 0; t < len[c]; ++t) {
                const uint32_t j = s[c] + t;
                if (j == i) continue;
                *o = j;
                o += F.stride;
            }
        n = reach;
        return false;
    }
#pragma unroll
    for (int c = 0; c < kMax; ++c)
#pragma unroll 1
        for (uint32_t t = 0; t < len[c]; ++t) {
            const uint32_t j = s[c] + t;
            if (j == i) continue;
            if (n < F.kmax) out[(size_t)n * F.stride] = j;
            if (++n == M) return true;
        }
    return false;
}

// The frame's full list of particle i with findNeighbours' shells (kernelWidthNeighbours 2 or 3,
// findContacts on): the 27 cells, then each shell, by cell groups (store_cell_group).  Returns the
// list's meta (kListOff when it does not fit or the particle is handed over; *deferred tells which).
__device__ __forceinline__ uint32_t store_full_list_shells(const DevParams& P, const SceneCtx& S, uint32_t i, float4 pa,
                                                           const uint32_t* __restrict__ cs,
                                                           const uint32_t* __restrict__ ce, const NbList& F,
                                                           bool* deferred) {
    const uint32_t M = P.M;
    if (M == 0) return 0u;
    const bool quirk = (P.flags & PBD_FLAG_CELL_END_QUIRK) && S.n >= 2;
    const int K = (int)P.K;
    uint32_t n = 0, nc = 0xFFFFFFFFu;
    auto meta = [&]() -> uint32_t {
        const uint32_t c = nc == 0xFFFFFFFFu ? n : nc;
        return n > F.kmax ? kListOff : (n | (c << 8));
    };
    uint32_t h[7];
    for (int a = -1; a <= 1; ++a) {
        const uint32_t hx = morton_axis(__fmaf_rn((float)a, P.d, pa.x)) << 2;
        for (int b = -1; b <= 1; ++b) {
            const uint32_t hxy = hx + (morton_axis(__fmaf_rn((float)b, P.d, pa.y)) << 1);
#pragma unroll
            for (int c = 0; c < 3; ++c) h[c] = hxy + morton_axis(__fmaf_rn((float)(c - 1), P.d, pa.z));
            if (store_cell_group<3>(P, S, i, h, 3, cs, ce, F, quirk, n, deferred)) return *deferred ? kListOff : meta();
        }
    }
    nc = n;
    for (int sh = 2; sh <= K; ++sh)
        for (int a = -sh; a <= sh; ++a) {
            const uint32_t hx = morton_axis(__fmaf_rn((float)a, P.d, pa.x)) << 2;
            for (int b = -sh; b <= sh; ++b) {
                const uint32_t hxy = hx + (morton_axis(__fmaf_rn((float)b, P.d, pa.y)) << 1);
                const bool edge = (a == sh || a == -sh || b == sh || b == -sh);
                const int m = edge ? 2 * sh + 1 : 2;   // interior columns: only c = -sh and c = +sh
#pragma unroll
                for (int t = 0; t < 7; ++t) {
                    const int c = edge ? t - sh : (t == 0 ? -sh : sh);
                    h[t] = hxy + morton_axis(__fmaf_rn((float)c, P.d, pa.z));
                }
                if (store_cell_group<7>(P, S, i, h, m, cs, ce, F, quirk, n, deferred)) return *deferred ? kListOff : meta();
            }
        }
    return meta();
}

// A visitor that sums nothing: a walk with Recorder<NullVisit> only stores the lists.
struct NullVisit {
    struct Contrib {};
    __device__ static Contrib zero() { return Contrib{}; }
    __device__ static bool effective(const Contrib&) { return false; }
    __device__ static Contrib shfl(const Contrib& c, int) { return c; }
    __device__ __forceinline__ void end_contacts(uint32_t) {}
    __device__ __forceinline__ Contrib contrib(uint32_t, const float4&, bool) const { return Contrib{}; }
    __device__ __forceinline__ void add(const Contrib&, bool) {}
};

__device__ __forceinline__ float shfl_f(float v, int k) { return __shfl_sync(kFullMask, v, k); }
__device__ __forceinline__ uint32_t shfl_u(uint32_t v, int k) { return __shfl_sync(kFullMask, v, k); }

// Hand particle i to the cooperative kernel; if the list is full, walk it here.
__device__ __forceinline__ bool defer_particle(const DeferList& D, uint32_t i) {
    const uint32_t k = atomicAdd(D.count, 1u);
    if (k < D.cap) { D.items[k] = i; return true; }
    return false;
}

// Grid-stride loop of the cooperative kernels over the deferred particles, then the last
// block to finish empties the list for the next pass.
template <class F>
__device__ __forceinline__ void for_each_deferred(const DeferList& D, F&& f) {
    const uint32_t n = min(*((volatile uint32_t*)D.count), D.cap);
    const uint32_t warps = gridDim.x * (blockDim.x >> 5);
    for (uint32_t w = blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5); w < n; w += warps) f(D.items[w]);
    __syncthreads();
    if (threadIdx.x == 0) {
        __threadfence();
        if (atomicAdd(D.done, 1u) == gridDim.x - 1) {
            *D.count = 0u;
            *D.done = 0u;
            __threadfence();
        }
    }
}

// The leading `blocks` blocks of a list kernel walk a set of particles over the cells (one warp
// per particle, walk_coop) while the other blocks walk the stored lists.  The particles without
// a list are known before such a kernel starts (the frame's first lambda pass, or the pass
// that recorded the near lists), so their long walks run beside the list walks instead of in a
// kernel after them.  With `reset`, the last of these blocks empties the set for its producer.
struct CoopSet {
    const uint32_t* items;
    uint32_t* count;
    uint32_t* done;
    uint32_t cap;
    uint32_t blocks;
    uint32_t reset;
};
template <class F>
__device__ __forceinline__ void run_coop_set(const CoopSet& C, F&& f) {
    const uint32_t n = min(*((volatile uint32_t*)C.count), C.cap);
    const uint32_t wpb = blockDim.x >> 5;
    const uint32_t warps = C.blocks * wpb;
    for (uint32_t w = blockIdx.x * wpb + (threadIdx.x >> 5); w < n; w += warps) f(C.items[w]);
    if (C.reset) {
        __syncthreads();
        if (threadIdx.x == 0) {
            __threadfence();
            if (atomicAdd(C.done, 1u) == C.blocks - 1) {
                *C.count = 0u;
                *C.done = 0u;
                __threadfence();
            }
        }
    }
}
// Append i to a set when the set is given (items non-null).
__device__ __forceinline__ void note_particle(const DeferList& D, uint32_t i) {
    if (D.items) defer_particle(D, i);
}

// ======================================================================================
// computeLambda (Density.h:48-93)
// ======================================================================================
struct LambdaVisit {
    // a = W, b = |grad|^2 = s^2 |r|^2; the gradient sum takes s * r by explicit FMAs, so every
    // walker rounds it the same way
    struct Contrib { float a, b, s, rx, ry, rz, rw; uint32_t near; };
    const DevParams& P;
    float4 pi;
    float A = 0.f, B = 0.f, Cx = 0.f, Cy = 0.f, Cz = 0.f, Cw = 0.f;
    __device__ LambdaVisit(const DevParams& P_, float4 pi_) : P(P_), pi(pi_) {}
    __device__ void reset() { A = B = Cx = Cy = Cz = Cw = 0.f; }
    __device__ static Contrib zero() { return Contrib{0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0u}; }
    __device__ static bool effective(const Contrib& c) { return c.near != 0u; }
    __device__ static Contrib shfl(const Contrib& c, int k) {
        return Contrib{shfl_f(c.a, k), shfl_f(c.b, k), shfl_f(c.s, k), shfl_f(c.rx, k), shfl_f(c.ry, k),
                       shfl_f(c.rz, k), shfl_f(c.rw, k), shfl_u(c.near, k)};
    }
    __device__ __forceinline__ void end_contacts(uint32_t) {}
    __device__ __forceinline__ Contrib contrib(uint32_t, const float4& pj, bool) const {
        const float rx = pi.x - pj.x, ry = pi.y - pj.y, rz = pi.z - pj.z, rw = pi.w - pj.w;
        const float r2 = dist2(rx, ry, rz);
        if (r2 >= P.cut2) return zero();      // every kernel is exactly 0 there
        const float dist = sqrtf(r2);
        const float r2w = __fmaf_rn(rw, rw, r2);
        const float s = spiky_scale(P, dist, r2w);
        return Contrib{poly6(P, dist), __fmul_rn(__fmul_rn(s, s), r2w), s, rx, ry, rz, rw, 1u};
    }
    __device__ __forceinline__ void add(const Contrib& c, bool) {
        if (!c.near) return;
        A = __fadd_rn(A, c.a); B = __fadd_rn(B, c.b);
        Cx = __fmaf_rn(c.s, c.rx, Cx); Cy = __fmaf_rn(c.s, c.ry, Cy);
        Cz = __fmaf_rn(c.s, c.rz, Cz); Cw = __fmaf_rn(c.s, c.rw, Cw);
    }
    // the sums the reverse pass needs: aux[i] = (rho, B, S.x, S.y), aux[N + i] = (S.z, S.w, 0, 0)
    __device__ __forceinline__ void store_aux(float4* __restrict__ aux, uint32_t N, uint32_t i) const {
        aux[i] = make_float4(A, B, Cx, Cy);
        aux[N + i] = make_float4(Cz, Cw, 0.f, 0.f);
    }
    __device__ __forceinline__ float finish(float rho0) const {
        // correctly rounded: every kernel that finishes a lambda gets the same bits
        const float a = __fsub_rn(__fdiv_rn(A, rho0), 1.0f);
        const float b = __fdiv_rn(B, rho0);
        const float s2 = __fadd_rn(__fadd_rn(__fmul_rn(Cx, Cx), __fmul_rn(Cy, Cy)), __fadd_rn(__fmul_rn(Cz, Cz), __fmul_rn(Cw, Cw)));
        const float c = __fdiv_rn(s2, rho0);
        return __fdiv_rn(-a, __fadd_rn(__fadd_rn(b, c), P.lambda_eps));
    }
};

__global__ void __launch_bounds__(256)
lambda_kernel(DevParams P, const float4* __restrict__ p, const float4* __restrict__ pa, const uint32_t* __restrict__ cs,
              const uint32_t* __restrict__ ce, float* __restrict__ lambda, DeferList D, float4* __restrict__ aux,
              NbList L, NbList F, DeferList DF, DeferList DN) {
    // walks the cells; L.list: record the near lists for the delta pass that follows (the
    // particles left without one noted in DN); F.list: store the full lists (the frame's first
    // lambda pass; the particles left without one noted in DF)
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= P.N) return;
    const SceneCtx S = scene_ctx(P, i);
    const float4 pi = p[i];
    LambdaVisit vis(P, pi);
    bool deferred = false;
    if (F.list) {
        // the walk stores the full list (indices only), the filter the near list; the sums then
        // run over the shortest list that fits
        uint32_t fm;
        const bool shells = (P.active & PBD_ACTIVE_FIND_NEIGHBOURS) && P.K >= 2;
        if (!shells && (P.active & PBD_ACTIVE_FIND_CONTACTS)) {
            fm = store_full_list(P, S, i, pa[i], cs, ce, F, &deferred);
        } else if (shells && P.K <= 3 && (P.active & PBD_ACTIVE_FIND_CONTACTS)) {
            fm = store_full_list_shells(P, S, i, pa[i], cs, ce, F, &deferred);
        } else {
            ListRecorder rec(F, i);
            walk_seq(P, S, i, pa[i], p, cs, ce, rec, true, &deferred);
            fm = deferred ? kListOff : rec.meta();
        }
        F.meta[i] = fm;
        if (fm == kListOff) note_particle(DF, i);
        const uint32_t lm = (L.list && fm != kListOff) ? filter_list<true>(F, fm, L, i, pi, P.cut2, p) : kListOff;
        if (L.list) {
            L.meta[i] = lm;
            if (lm == kListOff) note_particle(DN, i);
        }
        if (!deferred) {
            if (lm != kListOff) walk_near<true>(L, i, lm, p, vis);
            else if (fm != kListOff) walk_list<true>(F, i, fm, p, vis);
            else walk_seq(P, S, i, pa[i], p, cs, ce, vis, false, &deferred);
            lambda[i] = vis.finish(S.rho0);
            if (aux) vis.store_aux(aux, P.N, i);
            return;
        }
    } else if (L.list) {
        // the walk stores the near list; the sums then run over it when it fits
        Recorder<NullVisit> rec(NullVisit{}, L, F, false, i, pi, P.cut2);
        walk_seq(P, S, i, pa[i], p, cs, ce, rec, true, &deferred);
        const uint32_t lm = deferred ? kListOff : rec.meta();
        L.meta[i] = lm;
        if (lm == kListOff) note_particle(DN, i);
        if (!deferred) {
            if (lm != kListOff) walk_near<true>(L, i, lm, p, vis);
            else walk_seq(P, S, i, pa[i], p, cs, ce, vis, false, &deferred);
            lambda[i] = vis.finish(S.rho0);
            if (aux) vis.store_aux(aux, P.N, i);
            return;
        }
    } else {
        walk_seq(P, S, i, pa[i], p, cs, ce, vis, true, &deferred);
    }
    if (deferred) {
        if (defer_particle(D, i)) return;
        vis.reset();
        walk_seq(P, S, i, pa[i], p, cs, ce, vis, false, &deferred);
    }
    lambda[i] = vis.finish(S.rho0);
    if (aux) vis.store_aux(aux, P.N, i);
}

// One warp computes lambda_i over the cells.
__device__ __noinline__ void coop_lambda(const DevParams& P, const float4* __restrict__ p, const float4* __restrict__ pa,
                                            const uint32_t* __restrict__ cs, const uint32_t* __restrict__ ce,
                                            float* __restrict__ lambda, float4* __restrict__ aux, uint32_t i) {
    const SceneCtx S = scene_ctx(P, i);
    LambdaVisit vis(P, p[i]);
    walk_coop(P, S, i, pa[i], p, cs, ce, vis);
    if (lane_id() == 0) {
        lambda[i] = vis.finish(S.rho0);
        if (aux) vis.store_aux(aux, P.N, i);
    }
}

__global__ void __launch_bounds__(128)
lambda_coop_kernel(DevParams P, const float4* __restrict__ p, const float4* __restrict__ pa, const uint32_t* __restrict__ cs,
                   const uint32_t* __restrict__ ce, float* __restrict__ lambda, DeferList D, float4* __restrict__ aux) {
    for_each_deferred(D, [&](uint32_t i) { coop_lambda(P, p, pa, cs, ce, lambda, aux, i); });
}

// The frame's later lambda passes: read the full list (no cell tables), record the near list.
// The particles without a full list (the set C) are walked by the leading blocks; the ones left
// without a near list are noted in DN for the delta pass.  Kept apart from lambda_kernel so that
// its register budget is the list walk's alone.
__global__ void __launch_bounds__(256, 5)
lambda_list_kernel(DevParams P, const float4* __restrict__ p, const float4* __restrict__ pa,
                   const uint32_t* __restrict__ cs, const uint32_t* __restrict__ ce, float* __restrict__ lambda,
                   CoopSet C, DeferList DN, float4* __restrict__ aux, NbList L, NbList F) {
    if (blockIdx.x < C.blocks) {
        run_coop_set(C, [&](uint32_t i) { coop_lambda(P, p, pa, cs, ce, lambda, aux, i); });
        return;
    }
    const uint32_t i = (blockIdx.x - C.blocks) * blockDim.x + threadIdx.x;
    if (i >= P.N) return;
    const uint32_t fm = F.meta[i];
    if (fm == kListOff) {
        if (L.list) {
            L.meta[i] = kListOff;
            note_particle(DN, i);
        }
        return;
    }
    const SceneCtx S = scene_ctx(P, i);
    const float4 pi = p[i];
    LambdaVisit vis(P, pi);
    const uint32_t lm = L.list ? filter_list<false, true>(F, fm, L, i, pi, P.cut2, p) : kListOff;
    if (L.list) {
        L.meta[i] = lm;
        if (lm == kListOff) note_particle(DN, i);
    }
    if (lm != kListOff) walk_near<true>(L, i, lm, p, vis);
    else walk_list(F, i, fm, p, vis);
    lambda[i] = vis.finish(S.rho0);
    if (aux) vis.store_aux(aux, P.N, i);
}

// ======================================================================================
// computeDeltaPositions (Density.h:104-145) + solveCollisions type 0 (Collision.h:171-242,
// Jacobi: contacts read the frame's snapshot, the adds of particle i apply in list order)
// + applyDeltaPositions (Density.h:156-168) + updatePositions (Update.h:11-32).
// ======================================================================================
enum DeltaMode : uint32_t {
    kDoDelta = 1u << 0,      // compute delta p from lambda
    kDoCollide = 1u << 1,    // one solveCollisions pass over the contacts
    kDoApply = 1u << 2,      // p -= delta
    kLoadDelta = 1u << 3,    // delta from the buffer (not computed in this pass)
    kStoreDelta = 1u << 4,   // keep delta in the buffer
    kDoUpdate = 1u << 5,     // v = (p - x)/dt; x = p
};

struct DeltaVisit {
    // coef * r is the density part, t * (-r) the contact part; add() applies both with explicit
    // FMAs, so every walker (cells, lists, cooperative warp) rounds them the same way
    struct Contrib { float coef, rx, ry, rz, rw, t; uint32_t flags; };   // flags: 1 delta part, 2 contact part
    const DevParams& P;
    const float* __restrict__ lambda;
    const float* __restrict__ w;       // inverse masses, or null (all 1, the reference)
    float4 pi;
    float li, wi;
    bool do_delta, do_collide, all_pairs;
    float ax = 0.f, ay = 0.f, az = 0.f, aw = 0.f;   // sum of (li + lj + sCorr) * grad
    float4 pacc, xacc;                               // positions with the contact corrections added in order
    float4 xi;
    __device__ DeltaVisit(const DevParams& P_, const float* lam, const float* w_, float4 pi_, float li_, float wi_,
                          bool dd, bool dc, float4 xi_)
        : P(P_), lambda(lam), w(w_), pi(pi_), li(li_), wi(wi_), do_delta(dd), do_collide(dc),
          all_pairs(P_.far_pairs_zero == 0u), pacc(pi_), xacc(xi_), xi(xi_) {}
    __device__ void reset() { ax = ay = az = aw = 0.f; pacc = pi; xacc = xi; }
    __device__ static Contrib zero() { return Contrib{0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0u}; }
    __device__ static bool effective(const Contrib& c) { return c.flags != 0u; }
    __device__ static Contrib shfl(const Contrib& c, int k) {
        return Contrib{shfl_f(c.coef, k), shfl_f(c.rx, k), shfl_f(c.ry, k), shfl_f(c.rz, k), shfl_f(c.rw, k),
                       shfl_f(c.t, k), shfl_u(c.flags, k)};
    }
    __device__ __forceinline__ void end_contacts(uint32_t) {}
    using Extra = float;   // lambda_j
    __device__ __forceinline__ float fetch(uint32_t j) const { return do_delta ? __ldg(lambda + j) : 0.f; }
    __device__ __forceinline__ Contrib contrib(uint32_t j, const float4& pj, float lj, bool contact) const {
        Contrib c = zero();
        const float rx = pi.x - pj.x, ry = pi.y - pj.y, rz = pi.z - pj.z, rw = pi.w - pj.w;
        c.rx = rx; c.ry = ry; c.rz = rz; c.rw = rw;
        const float r2 = dist2(rx, ry, rz);
        if (!all_pairs && r2 >= P.cut2) return c;
        const float dist = sqrtf(r2);
        if (do_delta) {
            const float s = spiky_scale(P, dist, __fmaf_rn(rw, rw, r2));
            if (s != 0.0f || all_pairs) {
                const float W = poly6(P, dist);
                const float sc = __fmul_rn(-P.k_scorr, powi(__fmul_rn(W, P.inv_wq), P.n_scorr));
                c.coef = __fmul_rn(__fadd_rn(__fadd_rn(li, lj), sc), s);
                c.flags |= 1u;
            }
        }
        if (contact && do_collide) {
            const float overlap = P.d - dist;
            // share of the overlap this particle takes: inverseMass1 / (inverseMass1 + inverseMass2)
            // (Collision.h:223-225, where both are forced to 1); solids have inverse mass 0
            float share = 0.5f;
            if (w) {
                const float wj = __ldg(w + j);
                share = (wi + wj) > 0.0f ? wi / (wi + wj) : 0.0f;
            }
            if (overlap > 0.0f && dist > 0.00001f && share != 0.0f) {
                // -share * overlap * (1 - stiffness) along -r / |r|
                c.t = __fmul_rn(__fmul_rn(-share * overlap, 1.0f / dist), P.one_minus_stiffness);
                c.flags |= 2u;
            }
        }
        return c;
    }
    __device__ __forceinline__ void add(const Contrib& c, bool) {
        if (c.flags & 1u) {
            ax = __fmaf_rn(c.coef, c.rx, ax); ay = __fmaf_rn(c.coef, c.ry, ay);
            az = __fmaf_rn(c.coef, c.rz, az); aw = __fmaf_rn(c.coef, c.rw, aw);
        }
        if (c.flags & 2u) {
            pacc.x = __fmaf_rn(-c.rx, c.t, pacc.x); xacc.x = __fmaf_rn(-c.rx, c.t, xacc.x);
            pacc.y = __fmaf_rn(-c.ry, c.t, pacc.y); xacc.y = __fmaf_rn(-c.ry, c.t, xacc.y);
            pacc.z = __fmaf_rn(-c.rz, c.t, pacc.z); xacc.z = __fmaf_rn(-c.rz, c.t, xacc.z);
        }
    }
};

__device__ __forceinline__ void delta_finish(const DevParams& P, float rho0, uint32_t mode, uint32_t i, const DeltaVisit& vis,
                                             float4* __restrict__ pout, float4* __restrict__ x, float4* __restrict__ v,
                                             float4* __restrict__ delta) {
    // a solid (inverse mass 0) takes no density correction
    float4 pn = vis.pacc, xn = vis.xacc;
    float4 dp = make_float4(0.f, 0.f, 0.f, 0.f);
    if (mode & kDoDelta)   // correctly rounded: the list and the walking kernels store the same bits
        dp = make_float4(__fdiv_rn(vis.ax, rho0), __fdiv_rn(vis.ay, rho0), __fdiv_rn(vis.az, rho0), __fdiv_rn(vis.aw, rho0));
    else if (mode & kLoadDelta) dp = delta[i];
    if (mode & kStoreDelta) delta[i] = dp;
    if (mode & kDoApply) {
        if (vis.w) { dp.x *= vis.wi; dp.y *= vis.wi; dp.z *= vis.wi; dp.w *= vis.wi; }
        pn.x -= dp.x; pn.y -= dp.y; pn.z -= dp.z; pn.w -= dp.w;
    }
    if (mode & kDoUpdate) {
        const float r = P.inv_dt;
        v[i] = make_float4((pn.x - xn.x) * r, (pn.y - xn.y) * r, (pn.z - xn.z) * r, (pn.w - xn.w) * r);
        xn = pn;
    }
    pout[i] = pn;
    if (mode & (kDoCollide | kDoUpdate)) x[i] = xn;
}

__global__ void __launch_bounds__(256, 2)
delta_kernel(DevParams P, uint32_t mode, const float4* __restrict__ pin, const float4* __restrict__ pa, float4* __restrict__ pout,
             float4* __restrict__ x, float4* __restrict__ v, const float* __restrict__ lambda, const float* __restrict__ w,
             float4* __restrict__ delta, const uint32_t* __restrict__ cs, const uint32_t* __restrict__ ce,
             DeferList D) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= P.N) return;
    const float4 pi = pin[i];
    const bool need_x = (mode & (kDoCollide | kDoUpdate)) != 0;
    const float4 xi = need_x ? x[i] : make_float4(0.f, 0.f, 0.f, 0.f);
    const float li = (mode & kDoDelta) ? lambda[i] : 0.f;
    const SceneCtx S = scene_ctx(P, i);
    DeltaVisit vis(P, lambda, w, pi, li, w ? w[i] : 1.0f, (mode & kDoDelta) != 0, (mode & kDoCollide) != 0, xi);
    if (mode & (kDoDelta | kDoCollide)) {
        bool deferred = false;
        walk_seq(P, S, i, pa[i], pin, cs, ce, vis, true, &deferred);
        if (deferred) {
            if (defer_particle(D, i)) return;
            vis.reset();
            walk_seq(P, S, i, pa[i], pin, cs, ce, vis, false, &deferred);
        }
    }
    delta_finish(P, S.rho0, mode, i, vis, pout, x, v, delta);
}

// One warp runs the delta pass for particle i over the cells.
__device__ __noinline__ void coop_delta(const DevParams& P, uint32_t mode, const float4* __restrict__ pin,
                                           const float4* __restrict__ pa, float4* __restrict__ pout, float4* __restrict__ x,
                                           float4* __restrict__ v, const float* __restrict__ lambda, const float* __restrict__ w,
                                           float4* __restrict__ delta, const uint32_t* __restrict__ cs,
                                           const uint32_t* __restrict__ ce, uint32_t i) {
    const float4 pi = pin[i];
    const bool need_x = (mode & (kDoCollide | kDoUpdate)) != 0;
    const float4 xi = need_x ? x[i] : make_float4(0.f, 0.f, 0.f, 0.f);
    const float li = (mode & kDoDelta) ? lambda[i] : 0.f;
    const SceneCtx S = scene_ctx(P, i);
    DeltaVisit vis(P, lambda, w, pi, li, w ? w[i] : 1.0f, (mode & kDoDelta) != 0, (mode & kDoCollide) != 0, xi);
    walk_coop(P, S, i, pa[i], pin, cs, ce, vis);
    if (lane_id() == 0) delta_finish(P, S.rho0, mode, i, vis, pout, x, v, delta);
}

// delta pass 0 of an iteration over the near lists its lambda pass recorded (kB = kNearBatch), or
// any delta pass over the frame's full list when there are no near lists (kB = kListBatch); the
// particles without one (the set C) walk the cells.  kMode != 0: the pass
// mode fixed at compile time (the two passes of a fluid frame), kMode = 0: `mode` at run time.
// Blocks per SM by the list it walks (measured on GB300): 6 over the near lists (fluid_1m: 2%
// faster than 5), 5 over the full lists of the density-active workload (6 was 15% slower).
template <uint32_t kMode, uint32_t kB = kNearBatch>
__global__ void __launch_bounds__(256, kB == kNearBatch ? 6 : 5)
delta_list_kernel(DevParams P, uint32_t mode_rt, const float4* __restrict__ pin, const float4* __restrict__ pa,
                  float4* __restrict__ pout, float4* __restrict__ x, float4* __restrict__ v,
                  const float* __restrict__ lambda, const float* __restrict__ w, float4* __restrict__ delta,
                  const uint32_t* __restrict__ cs, const uint32_t* __restrict__ ce, CoopSet C, NbList L) {
    const uint32_t mode = kMode ? kMode : mode_rt;
    if (blockIdx.x < C.blocks) {
        run_coop_set(C, [&](uint32_t i) { coop_delta(P, mode, pin, pa, pout, x, v, lambda, w, delta, cs, ce, i); });
        return;
    }
    const uint32_t i = (blockIdx.x - C.blocks) * blockDim.x + threadIdx.x;
    if (i >= P.N) return;
    const uint32_t meta = L.meta[i];
    if (meta == kListOff) return;
    const float4 pi = pin[i];
    const bool need_x = (mode & (kDoCollide | kDoUpdate)) != 0;
    const float4 xi = need_x ? x[i] : make_float4(0.f, 0.f, 0.f, 0.f);
    const float li = (mode & kDoDelta) ? lambda[i] : 0.f;
    const SceneCtx S = scene_ctx(P, i);
    DeltaVisit vis(P, lambda, w, pi, li, w ? w[i] : 1.0f, (mode & kDoDelta) != 0, (mode & kDoCollide) != 0, xi);
    walk_list<false, kB>(L, i, meta, pin, vis);
    delta_finish(P, S.rho0, mode, i, vis, pout, x, v, delta);
}

__global__ void __launch_bounds__(128)
delta_coop_kernel(DevParams P, uint32_t mode, const float4* __restrict__ pin, const float4* __restrict__ pa, float4* __restrict__ pout,
                  float4* __restrict__ x, float4* __restrict__ v, const float* __restrict__ lambda, const float* __restrict__ w,
                  float4* __restrict__ delta, const uint32_t* __restrict__ cs, const uint32_t* __restrict__ ce,
                  DeferList D) {
    for_each_deferred(D, [&](uint32_t i) { coop_delta(P, mode, pin, pa, pout, x, v, lambda, w, delta, cs, ce, i); });
}

// updatePositions on its own (Update.h:11-32), when no delta pass can carry it.
__global__ void __launch_bounds__(256)
update_kernel(DevParams P, const float4* __restrict__ p, float4* __restrict__ x, float4* __restrict__ v) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= P.N) return;
    const float4 pp = p[i], xx = x[i];
    const float r = P.inv_dt;
    v[i] = make_float4((pp.x - xx.x) * r, (pp.y - xx.y) * r, (pp.z - xx.z) * r, (pp.w - xx.w) * r);
    x[i] = pp;
}

// ======================================================================================
// computeOmega (Density.h:232-269): omega_i = sum_j (v_j - v_i) x spiky(p_i, p_j)
// ======================================================================================
struct OmegaVisit {
    struct Contrib { float ox, oy, oz; uint32_t near; };
    const DevParams& P;
    const float4* __restrict__ v;
    float4 pi, vi;
    float ox = 0.f, oy = 0.f, oz = 0.f;
    __device__ OmegaVisit(const DevParams& P_, const float4* v_, float4 pi_, float4 vi_) : P(P_), v(v_), pi(pi_), vi(vi_) {}
    __device__ void reset() { ox = oy = oz = 0.f; }
    __device__ static Contrib zero() { return Contrib{0.f, 0.f, 0.f, 0u}; }
    __device__ static bool effective(const Contrib& c) { return c.near != 0u; }
    __device__ static Contrib shfl(const Contrib& c, int k) {
        return Contrib{shfl_f(c.ox, k), shfl_f(c.oy, k), shfl_f(c.oz, k), shfl_u(c.near, k)};
    }
    __device__ __forceinline__ void end_contacts(uint32_t) {}
    using Extra = float4;   // v_j
    __device__ __forceinline__ float4 fetch(uint32_t j) const { return __ldg(v + j); }
    __device__ __forceinline__ Contrib contrib(uint32_t, const float4& pj, const float4& vj, bool) const {
        const float rx = pi.x - pj.x, ry = pi.y - pj.y, rz = pi.z - pj.z, rw = pi.w - pj.w;
        const float r2 = dist2(rx, ry, rz);
        if (r2 >= P.cut2) return zero();
        const float dist = sqrtf(r2);
        const float s = spiky_scale(P, dist, __fmaf_rn(rw, rw, r2));
        if (s == 0.0f) return zero();
        const float wx = vj.x - vi.x, wy = vj.y - vi.y, wz = vj.z - vi.z;
        const float gx = s * rx, gy = s * ry, gz = s * rz;
        return Contrib{__fsub_rn(__fmul_rn(wy, gz), __fmul_rn(wz, gy)), __fsub_rn(__fmul_rn(wz, gx), __fmul_rn(wx, gz)),
                       __fsub_rn(__fmul_rn(wx, gy), __fmul_rn(wy, gx)), 1u};
    }
    __device__ __forceinline__ void add(const Contrib& c, bool) {
        if (!c.near) return;
        ox = __fadd_rn(ox, c.ox); oy = __fadd_rn(oy, c.oy); oz = __fadd_rn(oz, c.oz);
    }
};

__global__ void __launch_bounds__(256)
omega_kernel(DevParams P, const float4* __restrict__ p, const float4* __restrict__ pa, const float4* __restrict__ v,
             const uint32_t* __restrict__ cs, const uint32_t* __restrict__ ce, float4* __restrict__ omega, DeferList D,
             NbList L, DeferList DN) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= P.N) return;
    const SceneCtx S = scene_ctx(P, i);
    // walks the cells; L.list: record the near lists for a viscosity pass without vorticity (the
    // particles left without one noted in DN when DN is given)
    const float4 pi = p[i];
    OmegaVisit vis(P, v, pi, v[i]);
    bool deferred = false;
    if (L.list) {
        Recorder<OmegaVisit> rec(vis, L, L, false, i, pi, P.cut2);
        walk_seq(P, S, i, pa[i], p, cs, ce, rec, true, &deferred);
        L.meta[i] = deferred ? kListOff : rec.meta();
        if (L.meta[i] == kListOff) note_particle(DN, i);
        if (!deferred) {
            omega[i] = make_float4(rec.inner.ox, rec.inner.oy, rec.inner.oz, 0.f);
            return;
        }
    } else {
        walk_seq(P, S, i, pa[i], p, cs, ce, vis, true, &deferred);
    }
    if (deferred) {
        if (defer_particle(D, i)) return;
        vis.reset();
        walk_seq(P, S, i, pa[i], p, cs, ce, vis, false, &deferred);
    }
    omega[i] = make_float4(vis.ox, vis.oy, vis.oz, 0.f);
}

// One warp computes omega_i over the cells.
__device__ __noinline__ void coop_omega(const DevParams& P, const float4* __restrict__ p, const float4* __restrict__ pa,
                                           const float4* __restrict__ v, const uint32_t* __restrict__ cs,
                                           const uint32_t* __restrict__ ce, float4* __restrict__ omega, uint32_t i) {
    const SceneCtx S = scene_ctx(P, i);
    OmegaVisit vis(P, v, p[i], v[i]);
    walk_coop(P, S, i, pa[i], p, cs, ce, vis);
    if (lane_id() == 0) omega[i] = make_float4(vis.ox, vis.oy, vis.oz, 0.f);
}

// omega over the full list (recording the near list when L.list, and noting the particles left
// without one in DN when DN is given); the particles without a full list (the set C) are walked
// by the leading blocks.
// kNear: the pass filters the full list into omega's near list (the fluid workloads: 5 blocks
// per SM, 2.5% faster than 6 on fluid_1m); else it walks the full list (the density-active
// workload: 6, 5 was 3.8% slower).
template <bool kNear>
__global__ void __launch_bounds__(256, kNear ? 5 : 6)
omega_list_kernel(DevParams P, const float4* __restrict__ p, const float4* __restrict__ pa, const float4* __restrict__ v,
                  const uint32_t* __restrict__ cs, const uint32_t* __restrict__ ce, float4* __restrict__ omega,
                  CoopSet C, DeferList DN, NbList L, NbList F) {
    if (blockIdx.x < C.blocks) {
        run_coop_set(C, [&](uint32_t i) { coop_omega(P, p, pa, v, cs, ce, omega, i); });
        return;
    }
    const uint32_t i = (blockIdx.x - C.blocks) * blockDim.x + threadIdx.x;
    if (i >= P.N) return;
    const uint32_t fm = F.meta[i];
    if (fm == kListOff) {
        if (L.list) {
            L.meta[i] = kListOff;
            note_particle(DN, i);
        }
        return;
    }
    const float4 pi = p[i];
    OmegaVisit vis(P, v, pi, v[i]);
    const uint32_t lm = L.list ? filter_list(F, fm, L, i, pi, P.cut2, p) : kListOff;
    if (L.list) {
        L.meta[i] = lm;
        if (lm == kListOff) note_particle(DN, i);
    }
    if (lm != kListOff) walk_near<true>(L, i, lm, p, vis);
    else walk_list<false, 2>(F, i, fm, p, vis);
    omega[i] = make_float4(vis.ox, vis.oy, vis.oz, 0.f);
}

__global__ void __launch_bounds__(128)
omega_coop_kernel(DevParams P, const float4* __restrict__ p, const float4* __restrict__ pa, const float4* __restrict__ v,
                  const uint32_t* __restrict__ cs, const uint32_t* __restrict__ ce, float4* __restrict__ omega,
                  DeferList D) {
    for_each_deferred(D, [&](uint32_t i) { coop_omega(P, p, pa, v, cs, ce, omega, i); });
}

// ======================================================================================
// computeVorticity (Density.h:179-221) + computeViscosity (Density.h:280-310, Jacobi).
// Vorticity sums |omega_j - omega_i| / (p_j - p_i + 1e-8) componentwise over EVERY list
// entry (no kernel weight), so with vorticity on no pair may be skipped.
// ======================================================================================
// kTerms: the terms this visitor may run (1 vorticity, 2 viscosity, 3 either, as the run-time
// flags say); a visitor for one term loads one neighbour vector per entry.
template <uint32_t T> struct VortViscExtra { float4 oj, vj; };
template <> struct VortViscExtra<1u> { float4 oj; };
template <> struct VortViscExtra<2u> { float4 vj; };
template <uint32_t kTerms = 3u>
struct VortViscVisitT {
    struct Contrib { float gx, gy, gz, sx, sy, sz, sw; uint32_t flags; };   // 1 vorticity, 2 viscosity
    const DevParams& P;
    const float4* __restrict__ v;
    const float4* __restrict__ omega;
    float4 pi, vi, oi;
    bool vort, visc;
    float gx = 0.f, gy = 0.f, gz = 0.f;
    float sx = 0.f, sy = 0.f, sz = 0.f, sw = 0.f;
    __device__ VortViscVisitT(const DevParams& P_, const float4* v_, const float4* om, float4 pi_, float4 vi_, float4 oi_,
                              bool vo, bool vs)
        : P(P_), v(v_), omega(om), pi(pi_), vi(vi_), oi(oi_), vort(vo && (kTerms & 1u)), visc(vs && (kTerms & 2u)) {}
    __device__ void reset() { gx = gy = gz = sx = sy = sz = sw = 0.f; }
    __device__ static Contrib zero() { return Contrib{0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0u}; }
    __device__ static bool effective(const Contrib& c) { return c.flags != 0u; }
    __device__ static Contrib shfl(const Contrib& c, int k) {
        return Contrib{shfl_f(c.gx, k), shfl_f(c.gy, k), shfl_f(c.gz, k), shfl_f(c.sx, k),
                       shfl_f(c.sy, k), shfl_f(c.sz, k), shfl_f(c.sw, k), shfl_u(c.flags, k)};
    }
    __device__ __forceinline__ void end_contacts(uint32_t) {}
    using Extra = VortViscExtra<kTerms>;
    __device__ __forceinline__ Extra fetch(uint32_t j) const {
        Extra e;
        if constexpr ((kTerms & 1u) != 0u) e.oj = vort ? __ldg(omega + j) : make_float4(0.f, 0.f, 0.f, 0.f);
        if constexpr ((kTerms & 2u) != 0u) e.vj = visc ? __ldg(v + j) : make_float4(0.f, 0.f, 0.f, 0.f);
        return e;
    }
    __device__ __forceinline__ Contrib contrib(uint32_t, const float4& pj, const Extra& ex, bool) const {
        Contrib c = zero();
        if constexpr ((kTerms & 1u) != 0u) if (vort) {
            const float4 oj = ex.oj;
            const float dx = oj.x - oi.x, dy = oj.y - oi.y, dz = oj.z - oi.z;
            const float ol = sqrtf(dist2(dx, dy, dz));
            // the fast division: the divisors (position differences + 1e-8) stay far below 2^126
            c.gx = __fdividef(ol, (pj.x - pi.x) + 0.00000001f);
            c.gy = __fdividef(ol, (pj.y - pi.y) + 0.00000001f);
            c.gz = __fdividef(ol, (pj.z - pi.z) + 0.00000001f);
            c.flags |= 1u;
        }
        if constexpr ((kTerms & 2u) != 0u) if (visc) {
            const float rx = pi.x - pj.x, ry = pi.y - pj.y, rz = pi.z - pj.z;
            const float r2 = dist2(rx, ry, rz);
            if (r2 >= P.hp2) return c;
            const float W = poly6(P, sqrtf(r2));
            if (W == 0.0f) return c;
            const float4 vj = ex.vj;
            c.sx = (vj.x - vi.x) * W; c.sy = (vj.y - vi.y) * W;
            c.sz = (vj.z - vi.z) * W; c.sw = (vj.w - vi.w) * W;
            c.flags |= 2u;
        }
        return c;
    }
    __device__ __forceinline__ void add(const Contrib& c, bool) {
        if (c.flags & 1u) { gx = __fadd_rn(gx, c.gx); gy = __fadd_rn(gy, c.gy); gz = __fadd_rn(gz, c.gz); }
        if (c.flags & 2u) { sx = __fadd_rn(sx, c.sx); sy = __fadd_rn(sy, c.sy); sz = __fadd_rn(sz, c.sz); sw = __fadd_rn(sw, c.sw); }
    }
};

using VortViscVisit = VortViscVisitT<3u>;

// The vorticity force from the vorticity sums of `vo` and the viscosity update from the sums of
// `vs` (the same visitor when one walk summed both terms).  Explicitly rounded, so every kernel
// that finishes a particle stores the same bits.  `vhost` (mapped pinned host memory, or null)
// also receives the new velocity: a frame that reads its state back gets v without a copy after
// the pass.
template <class VO, class VS>
__device__ __forceinline__ void vort_visc_finish(const DevParams& P, uint32_t i, const VO& vo, const VS& vs,
                                                 float4* __restrict__ vout, float4* __restrict__ fext,
                                                 const float* __restrict__ w, float4* __restrict__ vhost = nullptr) {
    if (vo.vort) {
        if (P.eta_tape) P.eta_tape[i] = make_float4(vo.gx, vo.gy, vo.gz, 0.f);
        const float EPS = 0.00000001f;
        const float gl = sqrtf(__fmaf_rn(vo.gz, vo.gz, __fmaf_rn(vo.gy, vo.gy, __fmul_rn(vo.gx, vo.gx))));
        const float inv = 1.0f / __fadd_rn(gl, EPS);
        const float nx = __fmul_rn(inv, __fadd_rn(vo.gx, EPS)), ny = __fmul_rn(inv, __fadd_rn(vo.gy, EPS)),
                    nz = __fmul_rn(inv, __fadd_rn(vo.gz, EPS));
        const float e = P.e_vort;
        const float4 oi = vo.oi;
        fext[i] = make_float4(__fmul_rn(e, __fmaf_rn(ny, oi.z, -__fmul_rn(nz, oi.y))),
                              __fmul_rn(e, __fmaf_rn(nz, oi.x, -__fmul_rn(nx, oi.z))),
                              __fmul_rn(e, __fmaf_rn(nx, oi.y, -__fmul_rn(ny, oi.x))), 0.f);
    }
    if (vs.visc) {
        const float c = w ? __fmul_rn(w[i], P.c_visc) : P.c_visc;   // a solid keeps its velocity
        const float4 vi = vs.vi;
        const float4 vn = make_float4(__fmaf_rn(c, vs.sx, vi.x), __fmaf_rn(c, vs.sy, vi.y), __fmaf_rn(c, vs.sz, vi.z),
                                      __fmaf_rn(c, vs.sw, vi.w));
        vout[i] = vn;
        if (vhost) vhost[i] = vn;
    }
}

__global__ void __launch_bounds__(256, 2)
vort_visc_kernel(DevParams P, const float4* __restrict__ p, const float4* __restrict__ pa, const float4* __restrict__ vin,
                 float4* __restrict__ vout, const float4* __restrict__ omega, float4* __restrict__ fext,
                 const uint32_t* __restrict__ cs, const uint32_t* __restrict__ ce, int do_vort, int do_visc,
                 const float* __restrict__ w, DeferList D) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= P.N) return;
    const float4 oi = do_vort ? omega[i] : make_float4(0.f, 0.f, 0.f, 0.f);
    const SceneCtx S = scene_ctx(P, i);
    VortViscVisit vis(P, vin, omega, p[i], vin[i], oi, do_vort != 0, do_visc != 0);
    bool deferred = false;
    walk_seq(P, S, i, pa[i], p, cs, ce, vis, true, &deferred);
    if (deferred) {
        if (defer_particle(D, i)) return;
        vis.reset();
        walk_seq(P, S, i, pa[i], p, cs, ce, vis, false, &deferred);
    }
    vort_visc_finish(P, i, vis, vis, vout, fext, w);
}

// One warp runs vorticity + viscosity for particle i over the cells.
__device__ __noinline__ void coop_vort_visc(const DevParams& P, const float4* __restrict__ p, const float4* __restrict__ pa,
                                               const float4* __restrict__ vin, float4* __restrict__ vout,
                                               const float4* __restrict__ omega, float4* __restrict__ fext,
                                               const uint32_t* __restrict__ cs, const uint32_t* __restrict__ ce,
                                               int do_vort, int do_visc, const float* __restrict__ w, uint32_t i,
                                               float4* __restrict__ vhost) {
    const float4 oi = do_vort ? omega[i] : make_float4(0.f, 0.f, 0.f, 0.f);
    const SceneCtx S = scene_ctx(P, i);
    VortViscVisit vis(P, vin, omega, p[i], vin[i], oi, do_vort != 0, do_visc != 0);
    walk_coop(P, S, i, pa[i], p, cs, ce, vis);
    if (lane_id() == 0) vort_visc_finish(P, i, vis, vis, vout, fext, w, vhost);
}

// vorticity + viscosity over a stored list (the full list with vorticity, else the omega pass's
// near list); the particles without one (the set C) are walked by the leading blocks.  With both
// terms and the omega pass's near list Ln at hand, vorticity runs over the full list and
// viscosity over the near list (its entries beyond the cut add exact zeros): the two sums keep
// their own order.
// kNear: viscosity over omega's near list (the fluid workloads: 6 blocks per SM, 6.6% faster
// than 5 on fluid_1m); else both terms over the full list (the density-active workload's ~125
// entries: 5 blocks per SM, 6 was 36% slower).
template <bool kNear>
__global__ void __launch_bounds__(256, kNear ? 6 : 5)
vort_visc_list_kernel(DevParams P, const float4* __restrict__ p, const float4* __restrict__ pa,
                      const float4* __restrict__ vin, float4* __restrict__ vout, const float4* __restrict__ omega,
                      float4* __restrict__ fext, const uint32_t* __restrict__ cs, const uint32_t* __restrict__ ce,
                      int do_vort, int do_visc, const float* __restrict__ w, CoopSet C, NbList Lv, NbList Ln,
                      float4* __restrict__ vhost) {
    if (blockIdx.x < C.blocks) {
        run_coop_set(C, [&](uint32_t i) {
            coop_vort_visc(P, p, pa, vin, vout, omega, fext, cs, ce, do_vort, do_visc, w, i, vhost);
        });
        return;
    }
    const uint32_t i = (blockIdx.x - C.blocks) * blockDim.x + threadIdx.x;
    if (i >= P.N) return;
    const uint32_t meta = Lv.meta[i];
    if (meta == kListOff) return;
    const float4 oi = do_vort ? omega[i] : make_float4(0.f, 0.f, 0.f, 0.f);
    const uint32_t nm = (do_vort && do_visc && Ln.list) ? Ln.meta[i] : kListOff;
    if (nm != kListOff) {
        VortViscVisitT<1u> vo(P, vin, omega, p[i], vin[i], oi, true, false);
        walk_list<false, 2>(Lv, i, meta, p, vo);   // position + omega per entry: batches of 2 fit the registers
        VortViscVisitT<2u> vs(P, vin, omega, p[i], vin[i], oi, false, true);
        walk_near(Ln, i, nm, p, vs);
        vort_visc_finish(P, i, vo, vs, vout, fext, w, vhost);
        return;
    }
    VortViscVisit vis(P, vin, omega, p[i], vin[i], oi, do_vort != 0, do_visc != 0);
    walk_list<false, 2>(Lv, i, meta, p, vis);
    vort_visc_finish(P, i, vis, vis, vout, fext, w, vhost);
}

__global__ void __launch_bounds__(128)
vort_visc_coop_kernel(DevParams P, const float4* __restrict__ p, const float4* __restrict__ pa, const float4* __restrict__ vin,
                      float4* __restrict__ vout, const float4* __restrict__ omega, float4* __restrict__ fext,
                      const uint32_t* __restrict__ cs, const uint32_t* __restrict__ ce, int do_vort, int do_visc,
                      const float* __restrict__ w, DeferList D) {
    for_each_deferred(D, [&](uint32_t i) {
        coop_vort_visc(P, p, pa, vin, vout, omega, fext, cs, ce, do_vort, do_visc, w, i, nullptr);
    });
}

// ======================================================================================
// Density constraint after a frame: C_i = rho_i / rho0 - 1 with rho_i the poly6 sum over the
// frame's list (no self term, Density.h:67-84) at the current positions.
// ======================================================================================
struct DensityVisit {
    struct Contrib { float a; uint32_t near; };
    const DevParams& P;
    float4 pi;
    float A = 0.f;
    __device__ DensityVisit(const DevParams& P_, float4 pi_) : P(P_), pi(pi_) {}
    __device__ static Contrib zero() { return Contrib{0.f, 0u}; }
    __device__ static bool effective(const Contrib& c) { return c.near != 0u; }
    __device__ static Contrib shfl(const Contrib& c, int k) { return Contrib{shfl_f(c.a, k), shfl_u(c.near, k)}; }
    __device__ __forceinline__ void end_contacts(uint32_t) {}
    __device__ __forceinline__ Contrib contrib(uint32_t, const float4& pj, bool) const {
        const float rx = pi.x - pj.x, ry = pi.y - pj.y, rz = pi.z - pj.z;
        const float r2 = dist2(rx, ry, rz);
        if (r2 >= P.cut2) return zero();
        return Contrib{poly6(P, sqrtf(r2)), 1u};
    }
    __device__ __forceinline__ void add(const Contrib& c, bool) { if (c.near) A = __fadd_rn(A, c.a); }
};

// err[i] = C_i; acc[0] += |C_i| (double), acc[1] = max |C_i| (double bits, non-negative); over the
// interior particles (list length >= min_nb and position at least `margin` inside the enclosure on
// every axis: their kernel support lies in the fluid) acc[2] += |C_i|, acc[3] = max |C_i|,
// acc[4] += 1.
__global__ void __launch_bounds__(128)
density_error_kernel(DevParams P, const float4* __restrict__ p, const float4* __restrict__ pa,
                     const uint32_t* __restrict__ cs, const uint32_t* __restrict__ ce, float* __restrict__ err,
                     double* acc, uint32_t min_nb, float margin) {
    __shared__ double sred[5][4];
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    double a = 0.0, ai = 0.0, ni = 0.0;
    if (i < P.N) {
        const SceneCtx S = scene_ctx(P, i);
        const float4 pi = p[i];
        DensityVisit vis(P, pi);
        bool deferred = false;
        const uint32_t n = walk_seq(P, S, i, pa[i], p, cs, ce, vis, false, &deferred);
        const float c = vis.A / S.rho0 - 1.0f;
        err[i] = c;
        a = fabs((double)c);
        const float* bmn = P.batched ? P.scenes[P.scene_of[i]].bmin : P.bmin;
        const float* bmx = P.batched ? P.scenes[P.scene_of[i]].bmax : P.bmax;
        const bool inside = pi.x > bmn[0] + margin && pi.x < bmx[0] - margin && pi.y > bmn[1] + margin &&
                            pi.y < bmx[1] - margin && pi.z > bmn[2] + margin && pi.z < bmx[2] - margin;
        if (inside && n >= min_nb) { ai = a; ni = 1.0; }
    }
    double sm = a, mx = a, smi = ai, mxi = ai, cnt = ni;
    for (int o = 16; o > 0; o >>= 1) {
        sm += __shfl_down_sync(0xffffffffu, sm, o);
        mx = fmax(mx, __shfl_down_sync(0xffffffffu, mx, o));
        smi += __shfl_down_sync(0xffffffffu, smi, o);
        mxi = fmax(mxi, __shfl_down_sync(0xffffffffu, mxi, o));
        cnt += __shfl_down_sync(0xffffffffu, cnt, o);
    }
    if ((threadIdx.x & 31u) == 0u) {
        const int w = threadIdx.x >> 5;
        sred[0][w] = sm; sred[1][w] = mx; sred[2][w] = smi; sred[3][w] = mxi; sred[4][w] = cnt;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        double t = 0.0, m = 0.0, ti = 0.0, mi = 0.0, c = 0.0;
        for (int w = 0; w < (int)(blockDim.x >> 5); ++w) {
            t += sred[0][w]; m = fmax(m, sred[1][w]); ti += sred[2][w]; mi = fmax(mi, sred[3][w]); c += sred[4][w];
        }
        atomicAdd(acc, t);
        atomicMax(reinterpret_cast<unsigned long long*>(acc + 1), (unsigned long long)__double_as_longlong(m));
        atomicAdd(acc + 2, ti);
        atomicMax(reinterpret_cast<unsigned long long*>(acc + 3), (unsigned long long)__double_as_longlong(mi));
        atomicAdd(acc + 4, c);
    }
}

// ======================================================================================
// Debug: materialise the neighbour list (findContacts + findNeighbours, Collision.h:11-160)
// ======================================================================================
struct ListVisit {
    struct Contrib { uint32_t j; };
    uint32_t* out;
    uint32_t cap, n = 0, contacts = 0xFFFFFFFFu;
    __device__ ListVisit(uint32_t* o, uint32_t c) : out(o), cap(c) {}
    __device__ static Contrib zero() { return Contrib{0u}; }
    __device__ static bool effective(const Contrib&) { return true; }
    __device__ static Contrib shfl(const Contrib& c, int k) { return Contrib{shfl_u(c.j, k)}; }
    __device__ __forceinline__ void end_contacts(uint32_t c) { contacts = c; }
    __device__ __forceinline__ Contrib contrib(uint32_t j, const float4&, bool) const { return Contrib{j}; }
    __device__ __forceinline__ void add(const Contrib& c, bool) {
        if (n < cap) out[n] = c.j;
        ++n;
    }
};

__global__ void list_kernel(DevParams P, const float4* __restrict__ p, const uint32_t* __restrict__ cs,
                            const uint32_t* __restrict__ ce, uint32_t cap, uint32_t* list,
                            uint32_t* count, uint32_t* contacts, float4* col, int coop) {
    // coop = 0: one thread per particle; coop = 1: one warp per particle (checks walk_coop)
    const uint32_t i = coop ? (blockIdx.x * blockDim.x + threadIdx.x) >> 5 : blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= P.N) return;
    ListVisit vis(list + (size_t)i * cap, cap);
    uint32_t n;
    if (coop) {
        ListVisit lv(lane_id() == 0 ? list + (size_t)i * cap : nullptr, lane_id() == 0 ? cap : 0u);
        n = walk_coop(P, scene_ctx(P, i), i, p[i], p, cs, ce, lv);
        vis.contacts = lv.contacts;
        if (lane_id() != 0) return;
    } else {
        bool deferred = false;
        n = walk_seq(P, scene_ctx(P, i), i, p[i], p, cs, ce, vis, false, &deferred);
    }
    if (vis.contacts == 0xFFFFFFFFu) vis.contacts = n;   // cap reached inside the 27 cells
    count[i] = n;
    contacts[i] = vis.contacts;
    if (col) {
        const float f = (float)n / (float)P.M;
        col[i] = make_float4(f, f, f, 1.0f);
    }
}

}  // namespace pbd
