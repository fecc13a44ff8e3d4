// pbd_noalloc.cu -- the Morton-key radix sort as an entry point that allocates nothing.
//
// Some hosts cannot call cudaMalloc from the place where they sort: a renderer or game
// engine that sizes all of its device memory once at start-up and hands out pieces of its own
// pools, or a frame loop that must not call cudaMalloc because it can synchronise the device
// and stall the frame.  pbd_sort_keys_noalloc gives them the step's stable LSD radix sort
// (the replacement of cub::DeviceRadixSort::SortPairs in the reference's sortIds) with every
// byte of working memory taken from one fixed array compiled into this library.
//
// The working memory is the file-scope array below: kNoAllocMaxKeys keys at most
// (1,048,576), kScratchWords * 4 = 9,441,536 bytes (9.0 MiB).  Every GPU that loads the library
// keeps that array until the process exits.  All calls share it and it keeps the last call's
// contents, so each call first zeroes the parts that must start at zero; calls whose GPU work
// overlaps (different streams, or different host threads) race on it and must be serialised by
// the caller.  Its error word holds the outcome of the last call on the device:
// pbd_sort_noalloc_status reads it.
//
// Host code cannot use the array's name as a device address.  The first call on each device,
// with that device current, looks the address up with cudaGetSymbolAddress and caches it;
// make that first call before any stream capture.
#include <algorithm>
#include <cstdint>
#include <cstring>
#include <mutex>
#include <string>

#include <cuda_runtime.h>

#include "../../include/pbd.h"
#include "pbd_internal.h"
#include "pbd_sort.cuh"

namespace {

using namespace pbd;

constexpr uint32_t kNoAllocMaxKeys = 1u << 20;
constexpr uint32_t kNoAllocMaxTiles = (kNoAllocMaxKeys + kSortTile - 1) / kSortTile;
// word offsets inside the array
constexpr size_t kOffKeys = 0;
constexpr size_t kOffVals = kOffKeys + kNoAllocMaxKeys;
constexpr size_t kOffHist = kOffVals + kNoAllocMaxKeys;
constexpr size_t kOffStatus = kOffHist + (size_t)kMaxPasses * kRadix;
constexpr size_t kOffTiles = kOffStatus + (size_t)kMaxPasses * kNoAllocMaxTiles * kRadix;
constexpr size_t kOffErr = kOffTiles + kMaxPasses;
constexpr size_t kScratchWords = (kOffErr + 1 + 63) & ~size_t(63);

static_assert(kScratchWords * 4 == 9441536, "the fixed array's size is stated in pbd.h");
static __device__ __align__(256) uint32_t g_sort_scratch[kScratchWords];

constexpr int kMaxDevices = 64;
std::mutex g_setup_mutex;
uint32_t* g_scratch_ptr[kMaxDevices] = {};
// look-back wait settings (pbd_debug_set_wait_limit with a null simulation)
uint32_t g_spin_limit = kSpinLimit;
uint32_t g_hold = 0;

// Zero the histograms, the look-back rows the call will use, the tile counters and the error word.
__global__ void noalloc_clear_kernel(uint32_t* base, uint32_t ntiles) {
    const uint32_t t = blockIdx.x * blockDim.x + threadIdx.x, stride = gridDim.x * blockDim.x;
    for (uint32_t k = t; k < kMaxPasses * kRadix; k += stride) base[kOffHist + k] = 0u;
    for (uint32_t pass = 0; pass < kMaxPasses; ++pass)
        for (uint32_t k = t; k < ntiles * kRadix; k += stride)
            base[kOffStatus + (size_t)pass * kNoAllocMaxTiles * kRadix + k] = 0u;
    if (t < kMaxPasses) base[kOffTiles + t] = 0u;
    if (t == 0) base[kOffErr] = 0u;
}

// Digit histograms of every pass (the sim counts them in its predict kernel).
__global__ void noalloc_hist_kernel(const uint32_t* __restrict__ keys, uint32_t n, uint32_t* __restrict__ hist,
                                    int npasses, uint32_t key_bits) {
    __shared__ uint32_t sh[kMaxPasses * kRadix];
    for (int b = threadIdx.x; b < kMaxPasses * kRadix; b += blockDim.x) sh[b] = 0u;
    __syncthreads();
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        const uint32_t key = keys[i];
        for (int ps = 0; ps < npasses; ++ps) atomicAdd(&sh[ps * kRadix + sort_digit(key, ps, key_bits)], 1u);
    }
    __syncthreads();
    for (int b = threadIdx.x; b < npasses * kRadix; b += blockDim.x)
        if (sh[b]) atomicAdd(&hist[b], sh[b]);
}

int scratch_for_current_device(uint32_t** out) {
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) { set_error(std::string("pbd_sort_keys_noalloc: cudaGetDevice: ") + cudaGetErrorString(e)); return PBD_ERR_CUDA; }
    if (dev < 0 || dev >= kMaxDevices) { set_error("pbd_sort_keys_noalloc: device index out of range"); return PBD_ERR_UNSUPPORTED; }
    std::lock_guard<std::mutex> lock(g_setup_mutex);
    if (!g_scratch_ptr[dev]) {
        void* p = nullptr;
        e = cudaGetSymbolAddress(&p, g_sort_scratch);
        if (e != cudaSuccess || !p) {
            set_error(std::string("pbd_sort_keys_noalloc: cudaGetSymbolAddress: ") + cudaGetErrorString(e));
            return PBD_ERR_CUDA;
        }
        g_scratch_ptr[dev] = static_cast<uint32_t*>(p);
    }
    *out = g_scratch_ptr[dev];
    return PBD_OK;
}

}  // namespace

using pbd::clear_error;
using pbd::set_error;

int pbd_noalloc_set_wait_limit(unsigned int spins, int hold_first_tile) {
    std::lock_guard<std::mutex> lock(g_setup_mutex);
    g_spin_limit = spins ? spins : kSpinLimit;
    g_hold = hold_first_tile ? 1u : 0u;
    return PBD_OK;
}

extern "C" int pbd_sort_keys_noalloc(const uint32_t* d_keys_in, uint32_t* d_keys_out, uint32_t* d_perm_out,
                                     uint32_t n, uint32_t key_bits, void* stream) {
    clear_error();
    if (!d_keys_in || !d_keys_out || !d_perm_out) {
        set_error("pbd_sort_keys_noalloc: null device pointer");
        return PBD_ERR_INVALID_ARG;
    }
    if (key_bits == 0 || key_bits > 32) {
        set_error("pbd_sort_keys_noalloc: key_bits must be in [1, 32]");
        return PBD_ERR_INVALID_ARG;
    }
    if (n > kNoAllocMaxKeys) {
        set_error("pbd_sort_keys_noalloc: " + std::to_string(n) + " keys exceed the fixed working memory, which holds at most " +
                  std::to_string(kNoAllocMaxKeys) + " keys");
        return PBD_ERR_CAPACITY;
    }
    if (n == 0) return PBD_OK;
    uint32_t* base = nullptr;
    if (int rc = scratch_for_current_device(&base)) return rc;
    cudaStream_t st = (cudaStream_t)stream;
    const int npasses = (int)((key_bits + kRadixBits - 1) / kRadixBits);
    const uint32_t ntiles = (n + kSortTile - 1) / kSortTile;
    SortScratch S{base + kOffHist, base + kOffStatus, base + kOffTiles, base + kOffErr, kNoAllocMaxTiles};
    {
        std::lock_guard<std::mutex> lock(g_setup_mutex);
        S.spin_limit = g_spin_limit;
        S.hold = g_hold;
    }
    S.key_bits = key_bits;

    noalloc_clear_kernel<<<32, 256, 0, st>>>(base, ntiles);
    const uint32_t gh = std::min<uint32_t>((n + 255) / 256, 1024u);
    noalloc_hist_kernel<<<gh, 256, 0, st>>>(d_keys_in, n, S.hist, npasses, key_bits);
    // Ping-pong between the caller's outputs and the fixed array so that the last pass
    // writes the outputs: pass p writes the outputs when (npasses - 1 - p) is even.
    uint32_t* tmp_k = base + kOffKeys;
    uint32_t* tmp_v = base + kOffVals;
    const uint32_t* src_k = d_keys_in;
    const uint32_t* src_v = nullptr;
    for (int pass = 0; pass < npasses; ++pass) {
        const bool to_out = ((npasses - 1 - pass) % 2) == 0;
        uint32_t* dk = to_out ? d_keys_out : tmp_k;
        uint32_t* dv = to_out ? d_perm_out : tmp_v;
        if (pass == 0)
            onesweep_pass<true><<<ntiles, kSortThreads, 0, st>>>(src_k, src_v, dk, dv, n, pass, S);
        else
            onesweep_pass<false><<<ntiles, kSortThreads, 0, st>>>(src_k, src_v, dk, dv, n, pass, S);
        src_k = dk;
        src_v = dv;
    }
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) {
        set_error(std::string("pbd_sort_keys_noalloc: launch: ") + cudaGetErrorString(e));
        return PBD_ERR_CUDA;
    }
    return PBD_OK;
}

extern "C" int pbd_sort_noalloc_status(void* stream) {
    clear_error();
    uint32_t* base = nullptr;
    if (int rc = scratch_for_current_device(&base)) return rc;
    cudaError_t e = cudaStreamSynchronize((cudaStream_t)stream);
    uint32_t err = 0;
    if (e == cudaSuccess) e = cudaMemcpy(&err, base + kOffErr, sizeof(err), cudaMemcpyDeviceToHost);
    if (e != cudaSuccess) {
        set_error(std::string("pbd_sort_noalloc_status: ") + cudaGetErrorString(e));
        return PBD_ERR_CUDA;
    }
    if (err & kErrSortTimeout) {
        set_error("pbd_sort_keys_noalloc: a bounded look-back wait gave up; the output is not sorted");
        return PBD_ERR_TIMEOUT;
    }
    return PBD_OK;
}
