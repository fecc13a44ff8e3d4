// pbd_internal.h -- helpers shared by the translation units of libpbd (not installed).
#pragma once
#include <string>

#include <cstddef>
#ifdef __CUDACC__
#include <cuda_runtime.h>
#endif

namespace pbd {
// Thread-local text returned by pbd_last_error().
void set_error(const std::string& msg);
void clear_error();
#ifdef __CUDACC__
// Every device and pinned-host allocation of the library goes through these two, so that
// pbd_debug_fail_allocations can make them fail as an out-of-memory GPU would.
cudaError_t lib_malloc(void** p, size_t bytes);
cudaError_t lib_host_alloc(void** p, size_t bytes, unsigned int flags);
#endif
}  // namespace pbd

// The no-allocation sort's wait settings (pbd_debug_set_wait_limit with a null simulation).
int pbd_noalloc_set_wait_limit(unsigned int spins, int hold_first_tile);
