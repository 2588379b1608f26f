// Small helpers shared by the kernel translation units.
#pragma once
#include <cuda_runtime.h>
#include <cstdint>
#include "kernels.cuh"

namespace uhm_gpu {

template <typename T> __device__ __forceinline__ T* arena(const DevCtx& c);
template <> __device__ __forceinline__ double* arena<double>(const DevCtx& c) { return c.a64; }
template <> __device__ __forceinline__ float* arena<float>(const DevCtx& c) { return c.a32; }

__device__ __forceinline__ double load_src(const DevCtx& c, const SrcDev& s, int64_t idx) {
  if (!s.is_child) return c.emat[s.off + idx];
  return s.dtype == F64 ? c.a64[s.off + idx] : (double)c.a32[s.off + idx];
}

template <typename T> __device__ __forceinline__ T my_sqrt(T x);
template <> __device__ __forceinline__ double my_sqrt<double>(double x) { return sqrt(x); }
template <> __device__ __forceinline__ float my_sqrt<float>(float x) { return sqrtf(x); }

template <typename T> __device__ __forceinline__ T my_abs(T x);
template <> __device__ __forceinline__ double my_abs<double>(double x) { return fabs(x); }
template <> __device__ __forceinline__ float my_abs<float>(float x) { return fabsf(x); }

__device__ __forceinline__ void set_status(const DevCtx& c, int front, int st) {
  if (c.status) atomicCAS(&c.status[front], 0, st);
}

inline int ceil_div(int a, int b) { return (a + b - 1) / b; }

#define UHM_CUDA_LAUNCH_CHECK() do { cudaError_t e__ = cudaGetLastError(); (void)e__; } while (0)

// Iteration limit of the bounded spin-waits in one translation unit's kernels
// (flag hand-offs, grid barriers, mbarrier waits).  Each unit that waits
// defines its own copy with UHM_DEFINE_WAIT_LIMIT(setter, default) and reads
// g_wait_limit once per wait.  The default keeps every wait under about a
// second; uhm_gpu_set_wait_limit lowers it (0: a wait that is not satisfied
// on its first look gives up) so that tests can make a wait run out on the
// GPU and check the status it returns.  setter(v): v < 0 restores the default.
#define UHM_DEFINE_WAIT_LIMIT(setter, dflt)                                        \
  static __device__ uint32_t g_wait_limit = (dflt);                                \
  int setter(long long v) {                                                        \
    const uint32_t u = v < 0 ? (uint32_t)(dflt) : v > 0xFFFFFFFFll ? 0xFFFFFFFFu : (uint32_t)v; \
    return cudaMemcpyToSymbol(g_wait_limit, &u, sizeof(u)) == cudaSuccess ? 0 : 7; \
  }

// setters of the units that wait (k_factor.cu, k_solve.cu, k_tc_gemm.cu, k_noalloc.cu, k_chol_tc.cu)
int set_wait_limit_factor(long long v);
int set_wait_limit_solve(long long v);
int set_wait_limit_tc(long long v);
int set_wait_limit_noalloc(long long v);
int set_wait_limit_chol_tc(long long v);

}  // namespace uhm_gpu
