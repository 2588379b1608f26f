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

}  // namespace uhm_gpu
