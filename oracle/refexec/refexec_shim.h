/* refexec_shim.h -- lets the reference's own kernel sources (kernel/{Globals,Hash,SortReorder,
 * Forces,Collision,Density,Update}.h) run on the CPU.  TEST INFRASTRUCTURE ONLY: it builds the
 * checker oracle/_ref/librefexec.so, never the product.
 *
 * It stands in for what current CUDA and a headless machine no longer provide:
 *  - texture/surface references (removed from CUDA; Globals.h:5-13): a `surface` template over a
 *    row-major float4 array with the reference's byte-offset x addressing (x = column * 16);
 *  - the GL/console headers of Kernels.h and Globals.h (their include guards are predefined and
 *    Communication is an empty type);
 *  - the CUDA execution model: kernels become plain functions, a launch runs every thread of the
 *    grid in order (block by block, thread by thread), with threadIdx/blockIdx as globals;
 *  - atomicAdd and surf2Dwrite can be logged during a launch and applied after it, which runs a
 *    kernel as if every thread read before any thread wrote (used for solveCollisions and
 *    computeViscosity, the two kernels whose reads race with other threads' writes).
 * CUDA's own vector types and constructors (vector_types.h / vector_functions.h) are used as
 * they are; the reference's float4 helper header is included from the reference tree.
 */
#pragma once
#include <algorithm>
#include <climits>
#include <cmath>
#include <cstddef>
#include <cstdint>
#include <cstdlib>
#include <cstring>
#include <functional>
#include <vector>

#include <vector_types.h>
#include <vector_functions.h>

#undef __host__
#undef __device__
#undef __forceinline__
#define __host__
#define __device__
#define __global__
#define __constant__
#define __forceinline__ inline

/* headers of the reference that need OpenGL or the console: skipped */
#define CUDA_H
#define CUDA_UTIL_H
#define GL_CL_SHARED_H
#define COMMUNICATION_H
#define CUDA(call) (call)
struct Communication { void initialize() {} };

/* float math the device code calls */
inline float rsqrtf(float x) { return 1.0f / sqrtf(x); }
inline float min(float a, float b) { return fminf(a, b); }
inline float max(float a, float b) { return fmaxf(a, b); }

/* the reference's float4 helpers, with their own host block skipped (it redefines fminf) */
#define __CUDACC__ 1
#include "cuda/Cuda_Helper_Math.h"
#undef __CUDACC__

/* ---- runtime ----------------------------------------------------------------------- */
/* cudaError_t, cudaMemcpyKind and cudaSurfaceType2D come with vector_types.h's builtin types */
inline cudaError_t cudaMalloc(void** p, size_t n) { *p = calloc(n ? n : 1, 1); return cudaSuccess; }
template <class T> inline cudaError_t cudaMalloc(T** p, size_t n) { return cudaMalloc((void**)p, n); }
inline cudaError_t cudaFree(void* p) { free(p); return cudaSuccess; }
inline cudaError_t cudaMemset(void* p, int v, size_t n) { memset(p, v, n); return cudaSuccess; }
inline cudaError_t cudaMemcpy(void* d, const void* s, size_t n, cudaMemcpyKind) { memcpy(d, s, n); return cudaSuccess; }
inline void __syncthreads() {}

namespace refx {
extern uint3 g_threadIdx, g_blockIdx;
extern dim3 g_blockDim, g_gridDim;
struct FloatAdd { float* at; float v; };
struct SurfWrite { float4* at; float4 v; };
extern bool defer_atomics, defer_surface_writes;
extern std::vector<FloatAdd> atomic_log;
extern std::vector<SurfWrite> surface_log;
}  // namespace refx
#define threadIdx refx::g_threadIdx
#define blockIdx refx::g_blockIdx
#define blockDim refx::g_blockDim
#define gridDim refx::g_gridDim

inline float atomicAdd(float* p, float v) {
    const float old = *p;
    if (refx::defer_atomics) refx::atomic_log.push_back({p, v});
    else *p = old + v;
    return old;
}

/* ---- surfaces ------------------------------------------------------------------------ */
template <class T, int D>
struct surface {
    float4* data = nullptr;
    unsigned width = 0;   /* texels per row */
};
template <class S, class X, class Y>
inline void surf2Dread(float4* out, const S& s, X x, Y y) {
    *out = s.data[(size_t)(unsigned)y * s.width + (unsigned)x / 16u];
}
template <class S, class X, class Y>
inline void surf2Dwrite(float4 v, const S& s, X x, Y y) {
    float4* at = &s.data[(size_t)(unsigned)y * s.width + (unsigned)x / 16u];
    if (refx::defer_surface_writes) refx::surface_log.push_back({at, v});
    else *at = v;
}

/* ---- launches ------------------------------------------------------------------------ */
namespace refx {
inline void launch(dim3 grid, dim3 block, const std::function<void()>& body) {
    g_gridDim = grid;
    g_blockDim = block;
    for (unsigned bx = 0; bx < grid.x; ++bx)
        for (unsigned tx = 0; tx < block.x; ++tx) {
            g_blockIdx = make_uint3(bx, 0, 0);
            g_threadIdx = make_uint3(tx, 0, 0);
            body();
        }
    for (const FloatAdd& a : atomic_log) *a.at += a.v;          /* in thread order */
    atomic_log.clear();
    for (const SurfWrite& w : surface_log) *w.at = w.v;
    surface_log.clear();
}
}  // namespace refx
