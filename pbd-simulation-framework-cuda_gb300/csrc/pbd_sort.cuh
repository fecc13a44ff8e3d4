// pbd_sort.cuh -- stable LSD radix sort of (Morton key, particle index) pairs.
//
// Replaces cub::DeviceRadixSort::SortPairs (kernel/SortReorder.h:39-47, temp storage
// :221-238).  CUB's sort is a stable LSD radix sort; this one is too, so the permutation is
// the one any stable sort by the uint32 key gives (checked bit for bit against the oracle).
//
// Design (one kernel per 8-bit digit, "onesweep" style):
//  - The digit histograms of every pass are counted once, fused into the predict kernel
//    (shared-memory histograms flushed with one global atomic per non-empty bin).
//  - Each pass kernel takes a tile of kSortTile keys.  Tiles are numbered by an atomic
//    counter in launch order, so a tile only ever waits on tiles that are already running.
//  - Inside a tile every warp ranks its items with __match_any_sync (stable: item order is
//    warp, then register slot, then lane); warp counts are scanned per digit in shared
//    memory.
//  - Tile digit counts are chained across tiles with decoupled look-back (status word =
//    2 flag bits + 30 count bits).  Every wait is bounded: after SortScratch::spin_limit polls
//    (kSpinLimit by default, a few seconds) the tile records PBD device error bit
//    kErrSortTimeout and carries on, so a lost predecessor can never hang the GPU.  For tests
//    of that path, SortScratch::hold makes the first tile of every pass withhold its status
//    (a predecessor that never publishes): every wait on it runs out.
//  - Keys are scattered to shared memory in tile order first, then written out so that
//    each digit's run lands on consecutive global addresses.
#pragma once
#include <cstdint>
#include <cuda_runtime.h>

namespace pbd {

constexpr int kRadixBits = 8;
constexpr int kRadix = 1 << kRadixBits;
constexpr int kMaxPasses = 4;
constexpr int kSortThreads = 256;          // == kRadix: thread d owns digit d
constexpr int kSortWarps = kSortThreads / 32;
constexpr int kSortItems = 16;
constexpr int kSortTile = kSortThreads * kSortItems;   // 4096 keys per tile (2048 and 3072 were slower)
constexpr uint32_t kFlagAggregate = 1u << 30;
constexpr uint32_t kFlagPrefix = 2u << 30;
constexpr uint32_t kValueMask = (1u << 30) - 1u;
constexpr uint32_t kSpinLimit = 1u << 22;

// device error word bits
constexpr uint32_t kErrSortTimeout = 1u << 0;
constexpr uint32_t kErrKeyBits = 1u << 1;

struct SortScratch {
    uint32_t* hist;          // [kMaxPasses][kRadix] digit counts of the whole array
    uint32_t* status;        // [kMaxPasses][max_tiles][kRadix] look-back words
    uint32_t* tile_counter;  // [kMaxPasses]
    uint32_t* err;           // device error word
    uint32_t max_tiles;
    uint32_t spin_limit = kSpinLimit;   // polls of one look-back wait before it gives up
    uint32_t hold = 0;                  // 1: the first tile of each pass never publishes (tests)
    uint32_t key_bits = 32;             // only bits [0, key_bits) order the keys
};

// The digit of `key` in pass `pass`, counting only the bits below key_bits.
__device__ __forceinline__ uint32_t sort_digit(uint32_t key, int pass, uint32_t key_bits) {
    const uint32_t shift = (uint32_t)pass * kRadixBits;
    const uint32_t bits = key_bits - shift;          // >= 1 for every pass the sort runs
    const uint32_t mask = bits >= (uint32_t)kRadixBits ? (uint32_t)(kRadix - 1) : ((1u << bits) - 1u);
    return (key >> shift) & mask;
}

__device__ __forceinline__ uint32_t ld_relaxed(const uint32_t* p) {
    uint32_t v;
    asm volatile("ld.relaxed.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
    return v;
}
__device__ __forceinline__ void st_relaxed(uint32_t* p, uint32_t v) {
    asm volatile("st.relaxed.gpu.global.u32 [%0], %1;" ::"l"(p), "r"(v) : "memory");
}
__device__ __forceinline__ uint32_t lanemask_lt() {
    uint32_t m;
    asm("mov.u32 %0, %%lanemask_lt;" : "=r"(m));
    return m;
}

// Exclusive scan of one value per thread over a 256-thread block.  `warp_tot` is 8 words of
// shared memory.  Returns the exclusive prefix; the block total is written to *total.
__device__ __forceinline__ uint32_t block_exclusive_scan256(uint32_t v, uint32_t* warp_tot, uint32_t* total) {
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    uint32_t x = v;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        uint32_t y = __shfl_up_sync(0xffffffffu, x, o);
        if (lane >= o) x += y;
    }
    if (lane == 31) warp_tot[warp] = x;
    __syncthreads();
    if (warp == 0) {
        uint32_t t = lane < kSortWarps ? warp_tot[lane] : 0u;
#pragma unroll
        for (int o = 1; o < kSortWarps; o <<= 1) {
            uint32_t y = __shfl_up_sync(0xffffffffu, t, o);
            if (lane >= o) t += y;
        }
        if (lane < kSortWarps) warp_tot[lane] = t;   // inclusive warp totals
    }
    __syncthreads();
    uint32_t base = warp > 0 ? warp_tot[warp - 1] : 0u;
    if (total) *total = warp_tot[kSortWarps - 1];
    return base + x - v;
}

// One LSD pass over digit `pass` (bits 8*pass .. 8*pass+7).  kFirst: values are the
// identity (initializeParticleIds, SortReorder.h:199-210) and are generated, not loaded.
template <bool kFirst>
__global__ void __launch_bounds__(kSortThreads)
onesweep_pass(const uint32_t* __restrict__ kin, const uint32_t* __restrict__ vin,
              uint32_t* __restrict__ kout, uint32_t* __restrict__ vout, uint32_t n, int pass,
              SortScratch S) {
    __shared__ uint32_t s_whist[kSortWarps][kRadix];
    __shared__ uint32_t s_keys[kSortTile];
    __shared__ uint32_t s_vals[kSortTile];
    __shared__ uint32_t s_goff[kRadix];
    __shared__ uint32_t s_start[kRadix];
    __shared__ uint32_t s_wtot[kSortWarps];
    __shared__ uint32_t s_tile;

    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    if (tid == 0) s_tile = atomicAdd(&S.tile_counter[pass], 1u);
    for (int k = tid; k < kSortWarps * kRadix; k += kSortThreads) (&s_whist[0][0])[k] = 0u;
    __syncthreads();
    const uint32_t tile = s_tile;
    // The previous pass has finished (stream order): clear its look-back row for this tile.
    if (pass > 0) S.status[((size_t)(pass - 1) * S.max_tiles + tile) * kRadix + tid] = 0u;

    const uint32_t base = tile * (uint32_t)kSortTile;
    uint32_t key[kSortItems], val[kSortItems], rank[kSortItems];
#pragma unroll
    for (int k = 0; k < kSortItems; ++k) {
        const uint32_t idx = base + warp * (32 * kSortItems) + k * 32 + lane;
        const bool valid = idx < n;
        key[k] = valid ? kin[idx] : 0xFFFFFFFFu;
        val[k] = kFirst ? idx : (valid ? vin[idx] : 0u);
    }
    // ---- warp-level stable ranking
    uint32_t* wh = s_whist[warp];
    const uint32_t lt = lanemask_lt();
#pragma unroll
    for (int k = 0; k < kSortItems; ++k) {
        const uint32_t idx = base + warp * (32 * kSortItems) + k * 32 + lane;
        const bool valid = idx < n;
        const uint32_t digit = sort_digit(key[k], pass, S.key_bits);
        const uint32_t peers = __match_any_sync(0xffffffffu, valid ? digit : (uint32_t)kRadix);
        const uint32_t before = valid ? wh[digit] : 0u;
        __syncwarp();
        if (valid && (peers & lt) == 0u) wh[digit] = before + __popc(peers);
        __syncwarp();
        rank[k] = before + __popc(peers & lt);
    }
    __syncthreads();
    // ---- per digit (thread d): warp offsets, tile count, look-back
    const uint32_t d = tid;
    uint32_t run = 0;
#pragma unroll
    for (int w = 0; w < kSortWarps; ++w) {
        uint32_t c = s_whist[w][d];
        s_whist[w][d] = run;
        run += c;
    }
    uint32_t* st = S.status + (size_t)pass * S.max_tiles * kRadix;
    uint32_t excl = 0;
    if (tile == 0) {
        if (!S.hold) st_relaxed(&st[d], kFlagPrefix | run);
    } else {
        st_relaxed(&st[(size_t)tile * kRadix + d], kFlagAggregate | run);
        int t = (int)tile - 1;
        while (t >= 0) {
            uint32_t w = 0, spins = 0;
            for (;;) {
                w = ld_relaxed(&st[(size_t)t * kRadix + d]);
                if (w >> 30) break;
                if (++spins > S.spin_limit) {
                    atomicOr(S.err, kErrSortTimeout);
                    w = kFlagPrefix;
                    break;
                }
                __nanosleep(32);
            }
            excl += w & kValueMask;
            if ((w >> 30) == 2u) break;
            --t;
        }
        st_relaxed(&st[(size_t)tile * kRadix + d], kFlagPrefix | (excl + run));
    }
    // ---- global digit base (exclusive scan of the whole-array histogram) and tile starts
    const uint32_t hx = block_exclusive_scan256(S.hist[pass * kRadix + d], s_wtot, nullptr);
    __syncthreads();
    const uint32_t rx = block_exclusive_scan256(run, s_wtot, nullptr);
    s_goff[d] = hx + excl - rx;
    s_start[d] = rx;
    __syncthreads();
    // ---- scatter to shared memory in tile order
#pragma unroll
    for (int k = 0; k < kSortItems; ++k) {
        const uint32_t idx = base + warp * (32 * kSortItems) + k * 32 + lane;
        if (idx < n) {
            const uint32_t digit = sort_digit(key[k], pass, S.key_bits);
            const uint32_t pos = s_start[digit] + s_whist[warp][digit] + rank[k];
            s_keys[pos] = key[k];
            s_vals[pos] = val[k];
        }
    }
    __syncthreads();
    const uint32_t tile_n = (n - base) < (uint32_t)kSortTile ? (n - base) : (uint32_t)kSortTile;
    for (uint32_t i = tid; i < tile_n; i += kSortThreads) {
        const uint32_t kk = s_keys[i];
        const uint32_t o = s_goff[sort_digit(kk, pass, S.key_bits)] + i;
        if (o < n) {            // always true unless a look-back wait gave up (error word set)
            kout[o] = kk;
            vout[o] = s_vals[i];
        }
    }
}

}  // namespace pbd
