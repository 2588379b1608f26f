// Dense SPD solve from a caller-held Cholesky factor, allocating nothing.
//
// Who this is for: code that owns all device memory itself and may not call
// cudaMalloc / cudaFree - a host application that hands this library a fixed
// memory pool, a real-time loop where an allocation's implicit device
// synchronisation is not allowed, a process whose device memory is already
// fully reserved by another framework.  Such callers hold the factor and the
// right-hand side in their own device buffers and need x = (L L^T)^{-1} b.
//
// The work is the flag-driven block solve of the multifrontal path (one CTA
// per 64-row block; a CTA publishes its block of the solution and raises a
// completion flag that later blocks wait on) in one kernel for both sweeps:
// tickets 0..nb-1 run the forward blocks in order, tickets nb..2nb-1 the
// backward blocks from the last one down.  Its only scratch is a ticket
// counter, an error word and two flags per block, held in a fixed file-scope
// device array (STATIC_WORDS ints, 32 KB, owned by every GPU that loads this
// library until the process exits).
#include <cuda_runtime.h>

#include <cstdint>
#include <mutex>

#include "k_common.cuh"

namespace uhm_gpu {
UHM_DEFINE_WAIT_LIMIT(set_wait_limit_noalloc, 1u << 22)   // bounded waits (~0.5 s)
}  // namespace uhm_gpu

namespace {
using uhm_gpu::g_wait_limit;

constexpr int NA_FB = 64;                          // rows per block
constexpr int NA_MAX_BLOCKS = 4096;                // largest system: 262144 rows
constexpr int NA_MAX_N = NA_FB * NA_MAX_BLOCKS;
constexpr int STATIC_WORDS = 2 + 2 * NA_MAX_BLOCKS;
constexpr int NA_THREADS = 256;

// [0] ticket, [1] error word, then flags: 2b = forward block b done,
// 2b + 1 = backward block b done.  The first 2 + 2 nb words must be zero
// when a solve starts; the entry point clears them on the caller's stream.
static __device__ __align__(256) int g_noalloc_scratch[STATIC_WORDS];

__device__ __forceinline__ int na_ld_acquire(const int* p) {
  int v;
  asm volatile("ld.acquire.gpu.global.b32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
  return v;
}
__device__ __forceinline__ void na_st_release(int* p, int v) {
  asm volatile("st.release.gpu.global.b32 [%0], %1;" ::"l"(p), "r"(v) : "memory");
}

// thread 0 waits for *flag (bounded); the block learns whether to go on.
// The leading barrier keeps thread 0 from overwriting *s_ok while a slower
// warp has not yet read the previous wait's answer, so every thread of the
// block takes the same branch after each wait.
__device__ bool na_wait(const int* flag, int* err, int* s_ok) {
  __syncthreads();
  if (threadIdx.x == 0) {
    bool ok = na_ld_acquire(err) == 0;
    if (ok) {
      ok = false;
      const uint32_t lim = g_wait_limit;
      for (uint32_t it = 0; it < lim; ++it) {
        if (na_ld_acquire(flag) == 1) { ok = true; break; }
        if ((it & 255) == 255 && na_ld_acquire(err) != 0) break;
        __nanosleep(64);
      }
      if (!ok) atomicExch(err, 1);
    }
    *s_ok = ok;
  }
  __syncthreads();
  return *s_ok != 0;
}

__global__ void __launch_bounds__(NA_THREADS) k_dense_chol_solve_noalloc(const double* __restrict__ L, int n,
                                                                        int ld, double* x, int* scratch) {
  __shared__ double buf[NA_FB * (NA_FB + 1)];   // reduction, then the diagonal block
  __shared__ double v[NA_FB];
  __shared__ int s_t, s_ok;
  int* ticket = scratch;
  int* err = scratch + 1;
  int* flags = scratch + 2;
  if (threadIdx.x == 0) s_t = atomicAdd(ticket, 1);
  __syncthreads();
  const int nb = (n + NA_FB - 1) / NA_FB;
  const bool forward = s_t < nb;
  const int b = forward ? s_t : 2 * nb - 1 - s_t;
  const int r0 = b * NA_FB, kb = min(NA_FB, n - r0);
  const int lane = threadIdx.x % NA_FB, grp = threadIdx.x / NA_FB;   // 64 lanes x 4 groups
  double acc[16];
#pragma unroll
  for (int u = 0; u < 16; ++u) acc[u] = 0.0;
  bool go = true;

  if (forward) {
    // v = b_blk - sum_{j < b} L[blk, j] y_j ; thread (lane = row, grp = 16 columns)
    const int row = r0 + lane;
    for (int j = 0; j < b && go; ++j) {
      go = na_wait(flags + 2 * j, err, &s_ok);
      if (!go) break;
#pragma unroll
      for (int u = 0; u < 16; ++u) {
        const int c = j * NA_FB + grp * 16 + u;
        if (lane < kb) acc[0] += L[row + (int64_t)c * ld] * __ldcg(x + c);
      }
    }
    buf[grp * NA_FB + lane] = acc[0];
    __syncthreads();
    if (threadIdx.x < NA_FB)
      v[lane] = lane < kb ? __ldcg(x + row) - (buf[lane] + buf[NA_FB + lane] + buf[2 * NA_FB + lane] +
                                                buf[3 * NA_FB + lane])
                          : 0.0;
  } else {
    // v = y_blk - sum_{rows below the block} L[r, blk]^T x_r ; thread (lane = row of
    // a block below, grp = 16 columns of this block), then a reduction over lanes
    go = na_wait(flags + 2 * (nb - 1), err, &s_ok);   // every forward block is done
    for (int j = nb - 1; j > b && go; --j) {
      go = na_wait(flags + 2 * j + 1, err, &s_ok);
      if (!go) break;
      const int r = j * NA_FB + lane;
      if (r < n) {
        const double xr = __ldcg(x + r);
#pragma unroll
        for (int u = 0; u < 16; ++u) {
          const int c = grp * 16 + u;
          if (c < kb) acc[u] += L[r + (int64_t)(r0 + c) * ld] * xr;
        }
      }
    }
#pragma unroll
    for (int u = 0; u < 16; ++u) buf[lane * (NA_FB + 1) + grp * 16 + u] = acc[u];
    __syncthreads();
    if (threadIdx.x < NA_FB) {
      double s = 0.0;
      for (int r = 0; r < NA_FB; ++r) s += buf[r * (NA_FB + 1) + threadIdx.x];
      v[threadIdx.x] = threadIdx.x < kb ? __ldcg(x + r0 + threadIdx.x) - s : 0.0;
    }
  }
  __syncthreads();
  // the diagonal block, row-major with a padded row: buf[i * 65 + j] = L[r0 + i][r0 + j]
  for (int idx = threadIdx.x; idx < NA_FB * NA_FB; idx += NA_THREADS) {
    const int i = idx % NA_FB, j = idx / NA_FB;
    buf[i * (NA_FB + 1) + j] = (i < kb && j <= i) ? L[(r0 + i) + (int64_t)(r0 + j) * ld] : 0.0;
  }
  __syncthreads();
  if (forward) {
    for (int k = 0; k < kb; ++k) {                 // L_bb y = v
      if (threadIdx.x == k) v[k] /= buf[k * (NA_FB + 1) + k];
      __syncthreads();
      if (threadIdx.x > k && threadIdx.x < kb) v[threadIdx.x] -= buf[threadIdx.x * (NA_FB + 1) + k] * v[k];
      __syncthreads();
    }
  } else {
    for (int k = kb - 1; k >= 0; --k) {            // L_bb^T x = v
      if (threadIdx.x == k) v[k] /= buf[k * (NA_FB + 1) + k];
      __syncthreads();
      if (threadIdx.x < k) v[threadIdx.x] -= buf[k * (NA_FB + 1) + threadIdx.x] * v[k];
      __syncthreads();
    }
  }
  if (threadIdx.x < kb) x[r0 + threadIdx.x] = v[threadIdx.x];
  __threadfence();
  __syncthreads();
  if (threadIdx.x == 0) na_st_release(flags + 2 * b + (forward ? 0 : 1), 1);
}

// per-device address of the scratch array (host code cannot use the symbol
// itself as a device pointer)
std::mutex g_setup_mutex;
int* g_scratch_ptr[64] = {};

}  // namespace

extern "C" int uhm_gpu_dense_chol_solve_noalloc(const double* L, int n, int ld, double* x, void* stream) {
  if (!L || !x || n <= 0 || ld < n) return 7;
  if (n > NA_MAX_N) return 30;
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 64) return 7;
  int* scratch = nullptr;
  {
    std::lock_guard<std::mutex> lk(g_setup_mutex);
    if (!g_scratch_ptr[dev]) {
      void* p = nullptr;
      if (cudaGetSymbolAddress(&p, g_noalloc_scratch) != cudaSuccess || !p) return 7;
      g_scratch_ptr[dev] = static_cast<int*>(p);
    }
    scratch = g_scratch_ptr[dev];
  }
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  const int nb = (n + NA_FB - 1) / NA_FB;
  if (cudaMemsetAsync(scratch, 0, sizeof(int) * (2 + 2 * (size_t)nb), s) != cudaSuccess) return 7;
  k_dense_chol_solve_noalloc<<<2 * nb, NA_THREADS, 0, s>>>(L, n, ld, x, scratch);
  if (cudaGetLastError() != cudaSuccess) return 7;
  int h_err = 0;
  if (cudaMemcpyAsync(&h_err, scratch + 1, sizeof(int), cudaMemcpyDeviceToHost, s) != cudaSuccess) return 7;
  if (cudaStreamSynchronize(s) != cudaSuccess) return 7;
  return h_err ? 14 : 0;
}
