// pbd_contacts.cuh -- collisionType 1: contact constraints solved in batches of disjoint pairs
// (kernel/Collision.h:288-436, Fluid.cu:37-38,65-72).
//
// The reference claims contacts with a __syncthreads inside divergent code and lets blocks race
// on the claims, so its batches are undefined across blocks.  Here the batches are defined as
// locally dominant matching:
//  - the constraints are the frame's list entries c = i * M + k (partner = entry k of particle
//    i's list; the reference fills the same array, findContacts + findNeighbours);
//  - in each batch, a constraint not yet solved in this stabilization pass competes when its
//    particles overlap at the batch's start (diameter - |p_j - p_i| > 0, |p_j - p_i| > 1e-5, a
//    movable particle); its key is lowbias32(c + 1) (C. Wellons' published 32-bit integer mix)
//    above c; every particle takes its highest competing key (atomicMax over both ends) and a
//    constraint both of whose particles took it is solved -- a batch is a matching, so its
//    projections touch disjoint particles and run in parallel (Gauss-Seidel across batches);
//  - solving follows setupCollisionConstraintBatchesCheck (Collision.h:389-436): d = p2 - p1
//    (w = 0), half = (diameter - |d|) / 2, p1 and x1 move by -n half (1 - stiffness), p2 and x2 by
//    +n half (1 - stiffness), and both p* are written back with w = 0.  With unified solids the
//    overlap is split by inverse mass (1/2 each for unit masses, the same bits as half).
// The oracle (solve_collisions_batched) restates the same definition.
#pragma once
#include "pbd_passes.cuh"

namespace pbd {

struct ContactStore {
    uint32_t* list;      // M x stride partner indices, slot-major
    uint32_t* count;     // entries per particle
    uint32_t* solved;    // ceil(M / 32) x stride words: bit k of particle i = constraint (i, k) solved
    unsigned long long* best;   // each particle's chosen constraint key in this batch (0: none)
    unsigned long long* best_next;   // the next batch's keys: cleared by this batch's solve pass
    uint32_t* long_items;   // particles with more than kClaimLong entries (any order)
    uint32_t* long_count;   // zeroed before the frame's contact_list_kernel
    uint32_t stride;
    uint32_t M;
};

// Lanes per particle in the claim pass: entry k of a list goes to lane k mod kClaimLanes.  Lists
// longer than kClaimLong (up to M = 512 entries where the cell-end quirk stretches a cell's
// range, against ~26 on average) go to a whole warp in the pass's leading blocks instead, so they
// do not hold up the pass.
constexpr uint32_t kClaimLanes = 1;
constexpr uint32_t kClaimBatch = 4;    // entries per lane per step
constexpr uint32_t kClaimLong = 64;
constexpr uint32_t kClaimCoopBlocks = 4;

__device__ __forceinline__ uint32_t lowbias32(uint32_t x) {
    x ^= x >> 16;
    x *= 0x7feb352du;
    x ^= x >> 15;
    x *= 0x846ca68bu;
    x ^= x >> 16;
    return x;
}

// |p_j - p_i| of a contact pair, with explicit FMAs: the claim and the solve pass round it the
// same way, so they agree on which contacts act.
__device__ __forceinline__ float contact_len(float dx, float dy, float dz) {
    return sqrtf(__fmaf_rn(dz, dz, __fmaf_rn(dy, dy, __fmul_rn(dx, dx))));
}
// Whether the contact of i and j at distance len acts: an overlap, not coincident, and not two
// immovable particles.
__device__ __forceinline__ bool contact_acts(const DevParams& P, const float* __restrict__ w, uint32_t i, uint32_t j,
                                             float len) {
    if (w && !(w[i] + w[j] > 0.f)) return false;
    const float overlap = P.d - len;
    return (overlap * 0.5f > 0.f) && len > 0.00001f;
}

// The contact between particles i and j at the current positions: false when it does not act.
__device__ __forceinline__ bool contact_geometry(const DevParams& P, const float4* __restrict__ p,
                                                 const float* __restrict__ w, uint32_t i, uint32_t j,
                                                 float4& n, float& h1, float& h2) {
    const float4 p1 = p[i], p2 = p[j];
    const float dx = p2.x - p1.x, dy = p2.y - p1.y, dz = p2.z - p1.z;
    const float len = contact_len(dx, dy, dz);
    if (!contact_acts(P, w, i, j, len)) return false;
    float s1 = 0.5f, s2 = 0.5f;
    if (w) {
        const float w1 = w[i], w2 = w[j];
        s1 = w1 / (w1 + w2);
        s2 = w2 / (w1 + w2);
    }
    const float overlap = P.d - len;
    n = make_float4(dx / len, dy / len, dz / len, 0.f);
    h1 = overlap * s1;
    h2 = overlap * s2;
    return true;
}

// Every entry of particle i's list, in list order, up to the cap M.
struct ContactListVisit {
    struct Contrib { uint32_t j; };
    uint32_t* list;
    uint32_t stride, i, n = 0;
    __device__ ContactListVisit(uint32_t* l, uint32_t s, uint32_t i_) : list(l), stride(s), i(i_) {}
    __device__ static Contrib zero() { return Contrib{0u}; }
    __device__ static bool effective(const Contrib&) { return true; }
    __device__ static Contrib shfl(const Contrib& c, int k) { return Contrib{shfl_u(c.j, k)}; }
    __device__ __forceinline__ void end_contacts(uint32_t) {}
    __device__ __forceinline__ Contrib contrib(uint32_t j, const float4&, bool) const { return Contrib{j}; }
    __device__ __forceinline__ void add(const Contrib& c, bool) { list[(size_t)n * stride + i] = c.j; ++n; }
};

__device__ __forceinline__ void contact_list_done(const ContactStore& C, uint32_t i, uint32_t n) {
    C.count[i] = n;
    if (n > kClaimLong) C.long_items[atomicAdd(C.long_count, 1u)] = i;
}

// After the re-order: each particle's constraint list (the walk stops at the cap M itself).  A
// particle whose walk meets a cell range longer than one thread's walk takes is listed again by
// a warp of its block (walk_coop: the same entries in the same order) once the block's threads
// are done.  Blocks of 256 threads.
__global__ void __launch_bounds__(256)
contact_list_kernel(DevParams P, const float4* __restrict__ pa, const uint32_t* __restrict__ cs,
                    const uint32_t* __restrict__ ce, ContactStore C) {
    __shared__ uint32_t left[256];
    __shared__ uint32_t nleft;
    if (threadIdx.x == 0) nleft = 0u;
    __syncthreads();
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < P.N) {
        ContactListVisit vis(C.list, C.stride, i);
        bool deferred = false;
        walk_seq(P, scene_ctx(P, i), i, pa[i], pa, cs, ce, vis, true, &deferred);
        if (deferred) left[atomicAdd(&nleft, 1u)] = i;
        else contact_list_done(C, i, vis.n);
    }
    __syncthreads();
    const uint32_t nl = nleft;
    for (uint32_t k = threadIdx.x >> 5; k < nl; k += blockDim.x >> 5) {
        const uint32_t q = left[k];
        ContactListVisit vis(C.list, C.stride, q);
        walk_coop(P, scene_ctx(P, q), q, pa[q], pa, cs, ce, vis);
        if (lane_id() == 0) contact_list_done(C, q, vis.n);
    }
}

// Offer the keys of particle i's pending overlapping constraints k = t, t + L, t + 2L, ... (lane t
// of L lanes) to both particles; returns the highest key offered to i itself.  Each lane takes B
// entries per step (index loads, then position loads, in flight together, the next step's
// indices loaded meanwhile); a cheap squared-distance test (a superset of the overlap test,
// |r| < diameter) skips most entries before the exact one.
template <uint32_t L, uint32_t B>
__device__ __forceinline__ unsigned long long claim_entries(const DevParams& P, const ContactStore& C,
                                                            const float4* __restrict__ p, const float* __restrict__ w,
                                                            uint32_t i, uint32_t t, uint32_t n) {
    constexpr uint32_t kStep = B * L;
    static_assert((kStep <= 32u && (32u % kStep) == 0u) || (L == 32u && B == 2u), "a step's solved words");
    const float4 pi = p[i];
    const float reach2 = P.d * P.d * 1.0001f;
    const uint32_t* __restrict__ e = C.list + i;
    unsigned long long own = 0ull;
    uint32_t word[B];   // solved bits of the word holding each of this step's entries
    uint32_t jn[B];     // the next step's entries, loaded while this step is tested
#pragma unroll
    for (uint32_t b = 0; b < B; ++b) {
        word[b] = 0u;
        jn[b] = (t + b * L < n) ? __ldcs(e + (size_t)(t + b * L) * C.stride) : i;
    }
#pragma unroll 1
    for (uint32_t k0 = 0; k0 < n; k0 += kStep) {
        if (kStep <= 32u) {                      // a step stays inside one 32-entry word
            if ((k0 & 31u) == 0u) {
                const uint32_t v = C.solved[(size_t)(k0 >> 5) * C.stride + i];
#pragma unroll
                for (uint32_t b = 0; b < B; ++b) word[b] = v;
            }
        } else {                                 // 64 entries a step: entry b of a lane is in word k0/32 + b
#pragma unroll
            for (uint32_t b = 0; b < B; ++b)
                word[b] = (k0 + b * 32u < n) ? C.solved[(size_t)((k0 >> 5) + b) * C.stride + i] : 0u;
        }
        uint32_t j[B];
        float4 pj[B];
#pragma unroll
        for (uint32_t b = 0; b < B; ++b) j[b] = jn[b];
#pragma unroll
        for (uint32_t b = 0; b < B; ++b) pj[b] = (k0 + t + b * L < n) ? __ldg(p + j[b]) : pi;
#pragma unroll
        for (uint32_t b = 0; b < B; ++b) {
            const uint32_t k = k0 + kStep + t + b * L;
            jn[b] = (k < n) ? __ldcs(e + (size_t)k * C.stride) : i;
        }
#pragma unroll
        for (uint32_t b = 0; b < B; ++b) {
            const uint32_t k = k0 + t + b * L;
            if (k >= n || ((word[b] >> (k & 31u)) & 1u)) continue;
            const float dx = pj[b].x - pi.x, dy = pj[b].y - pi.y, dz = pj[b].z - pi.z;
            if (!(dx * dx + dy * dy + dz * dz < reach2)) continue;
            if (!contact_acts(P, w, i, j[b], contact_len(dx, dy, dz))) continue;
            const uint32_t c = i * C.M + k;
            const unsigned long long key = ((unsigned long long)lowbias32(c + 1u) << 32) | c;
            own = key > own ? key : own;          // i's own offers: one atomic per particle
            atomicMax(C.best + j[b], key);        // the partner's (no read first: fire and forget)
        }
    }
    return own;
}

// Maximum over groups of L lanes (L a power of two dividing 32); every lane of the warp calls it.
template <uint32_t L>
__device__ __forceinline__ unsigned long long group_max(unsigned long long v) {
#pragma unroll
    for (uint32_t s = 1; s < L; s <<= 1) {
        const unsigned long long o = __shfl_xor_sync(0xffffffffu, v, s);
        v = o > v ? o : v;
    }
    return v;
}

// Each pending overlapping constraint offers its key to both of its particles; the particle's
// own offers are reduced over its lanes into one atomic.  The first kClaimCoopBlocks blocks take
// the long lists, a warp each; the others take every other particle, kClaimLanes lanes each.
__global__ void __launch_bounds__(256, 6)
contact_claim_kernel(DevParams P, ContactStore C, const float4* __restrict__ p, const float* __restrict__ w) {
    if (blockIdx.x < kClaimCoopBlocks) {
        const uint32_t nl = *C.long_count;
        const uint32_t wpb = blockDim.x >> 5, lane = threadIdx.x & 31u;
        for (uint32_t q = blockIdx.x * wpb + (threadIdx.x >> 5); q < nl; q += kClaimCoopBlocks * wpb) {
            const uint32_t i = C.long_items[q];
            const unsigned long long own = group_max<32>(claim_entries<32, 2>(P, C, p, w, i, lane, C.count[i]));
            if (lane == 0 && own) atomicMax(C.best + i, own);
        }
        return;
    }
    constexpr uint32_t L = kClaimLanes;
    const uint32_t i = (blockIdx.x - kClaimCoopBlocks) * (blockDim.x / L) + threadIdx.x / L, t = threadIdx.x % L;
    uint32_t n = i < P.N ? C.count[i] : 0u;
    if (n > kClaimLong) n = 0u;                  // a long list: a leading block's warp takes it
    // no early exit: the lanes meet in the shuffles below
    const unsigned long long own = group_max<L>(n ? claim_entries<L, kClaimBatch>(P, C, p, w, i, t, n) : 0ull);
    if (t == 0 && own) atomicMax(C.best + i, own);
}

// A constraint both of whose particles took it is solved by its partner's thread: the key holds
// the constraint c = a * M + k, so the partner finds the owner a without reading the list.  Each
// thread also clears its particle's key for the next batch (that buffer was the previous batch's
// and is read by no one here).
__global__ void __launch_bounds__(256)
contact_solve_kernel(DevParams P, ContactStore C, float4* __restrict__ p, float4* __restrict__ x,
                     const float* __restrict__ w) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= P.N) return;
    C.best_next[i] = 0ull;
    const unsigned long long key = C.best[i];
    if (key == 0ull) return;
    const uint32_t c = (uint32_t)key;
    const uint32_t a = c / C.M;                  // the owner; i is its partner unless a == i
    if (a == i || C.best[a] != key) return;
    const uint32_t k = c - a * C.M;
    C.solved[(size_t)(k >> 5) * C.stride + a] |= 1u << (k & 31u);   // a is in one solved constraint
    float4 n;
    float h1, h2;
    if (!contact_geometry(P, p, w, a, i, n, h1, h2)) return;
    const float om = P.one_minus_stiffness;
    const float4 a1 = make_float4(-n.x * h1 * om, -n.y * h1 * om, -n.z * h1 * om, -n.w * h1 * om);
    const float4 a2 = make_float4(n.x * h2 * om, n.y * h2 * om, n.z * h2 * om, n.w * h2 * om);
    const float4 p1 = p[a], p2 = p[i];
    p[a] = make_float4(p1.x + a1.x, p1.y + a1.y, p1.z + a1.z, 0.f + a1.w);
    p[i] = make_float4(p2.x + a2.x, p2.y + a2.y, p2.z + a2.z, 0.f + a2.w);
    const float4 x1 = x[a], x2 = x[i];
    x[a] = make_float4(x1.x + a1.x, x1.y + a1.y, x1.z + a1.z, x1.w + a1.w);
    x[i] = make_float4(x2.x + a2.x, x2.y + a2.y, x2.z + a2.z, x2.w + a2.w);
}

}  // namespace pbd
