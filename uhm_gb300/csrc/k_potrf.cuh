// The 64 x 64 diagonal-block Cholesky shared by the blocked factor kernels
// (k_factor.cu) and the cooperative panel kernel of tensor-core fronts
// (k_chol_tc.cu): a tile-owned right-looking factorisation that forms the
// block's inverse in the same phases.
#pragma once
#include <cuda_runtime.h>
#include <cstdint>

namespace uhm_gpu {

template <typename T> __device__ __forceinline__ void pivot_root(T s, T& d, T& rd);
template <> __device__ __forceinline__ void pivot_root<float>(float s, float& d, float& rd) {
  rd = rsqrtf(s);
  d = s * rd;
}
template <> __device__ __forceinline__ void pivot_root<double>(double s, double& d, double& rd) {
  d = sqrt(s);
  rd = 1.0 / d;
}

template <typename T> struct Vec4;
template <> struct Vec4<float> {
  static __device__ __forceinline__ void ld(const float* p, float (&v)[4]) {
    const float4 q = *reinterpret_cast<const float4*>(p);
    v[0] = q.x; v[1] = q.y; v[2] = q.z; v[3] = q.w;
  }
  static __device__ __forceinline__ void st(float* p, const float (&v)[4]) {
    *reinterpret_cast<float4*>(p) = make_float4(v[0], v[1], v[2], v[3]);
  }
};
template <> struct Vec4<double> {
  static __device__ __forceinline__ void ld(const double* p, double (&v)[4]) {
    const double2 q0 = *reinterpret_cast<const double2*>(p);
    const double2 q1 = *reinterpret_cast<const double2*>(p + 2);
    v[0] = q0.x; v[1] = q0.y; v[2] = q1.x; v[3] = q1.y;
  }
  static __device__ __forceinline__ void st(double* p, const double (&v)[4]) {
    *reinterpret_cast<double2*>(p) = make_double2(v[0], v[1]);
    *reinterpret_cast<double2*>(p + 2) = make_double2(v[2], v[3]);
  }
};

template <typename T>
struct PotrfShared {
  T V[64][64];      // V[p][i]: column p of the reduced block (zero above p)
  T XR[8][4][8];    // per warp: rows P..P+3 of its block of X, finished
};

// Factor the 64 x 64 block at G (leading dimension n, kb <= 64 valid rows and
// columns) in shared memory; on return x holds this thread's tile of L^{-1}
// and, when Lout is not null, the lower triangle of L has been written there
// (leading dimension n); bad is set when a pivot was not positive.  Ends
// with a block barrier.
template <typename T>
__device__ __forceinline__ void potrf_block(const T* __restrict__ G, int n, int kb, PotrfShared<T>& sh,
                                            T (&x)[4][4], bool& bad, T* __restrict__ Lout) {
  const int tid = threadIdx.x, w = tid >> 5;
  const int ti = tid & 15, tj = tid >> 4, h = tj & 1;
  const int r0 = 4 * ti, c0 = 4 * tj, cb0 = 8 * w;
  {
    // stage the lower triangle (coalesced column reads, all loads in flight
    // before the shared stores), identity padding
    T g[16];
#pragma unroll
    for (int u = 0; u < 16; ++u) {
      const int idx = tid + 256 * u, i = idx & 63, j = idx >> 6;
      g[u] = (i >= j && i < kb && j < kb) ? G[i + (int64_t)j * n] : (i == j ? T(1) : T(0));
    }
#pragma unroll
    for (int u = 0; u < 16; ++u) {
      const int idx = tid + 256 * u, i = idx & 63, j = idx >> 6;
      if (i >= j) sh.V[j][i] = g[u];
    }
  }
  __syncthreads();
  T a[4][4];
#pragma unroll
  for (int u = 0; u < 4; ++u)
#pragma unroll
    for (int v = 0; v < 4; ++v) {
      const int i = r0 + u, j = c0 + v;
      a[u][v] = i >= j ? sh.V[j][i] : sh.V[i][j];
      x[u][v] = i == j ? T(1) : T(0);
    }
  __syncthreads();   // tiles read before any column is republished; columns 0..3 stay as staged
  bad = false;
#pragma unroll 1
  for (int q = 0; q < 16; ++q) {
    const int P = 4 * q;
    // the pivot block (every thread factors it) and this thread's rows / columns
    T bk[4][4], lr[4][4], lc[4][4];   // bk[j][i] = v_{P+j}[P+i]; lr[u][j], lc[v][j]: factor entries
#pragma unroll
    for (int j = 0; j < 4; ++j) {
      T t4[4];
      Vec4<T>::ld(&sh.V[P + j][P], bk[j]);
      Vec4<T>::ld(&sh.V[P + j][r0], t4);
#pragma unroll
      for (int u = 0; u < 4; ++u) lr[u][j] = t4[u];
      Vec4<T>::ld(&sh.V[P + j][c0], t4);
#pragma unroll
      for (int v = 0; v < 4; ++v) lc[v][j] = t4[v];
    }
    T lb[4][4], rd[4];
#pragma unroll
    for (int j = 0; j < 4; ++j) {
      T s = bk[j][j];
#pragma unroll
      for (int m = 0; m < j; ++m) s -= lb[j][m] * lb[j][m];
      if (!(s > T(0))) { bad = true; s = T(1); }
      T d;
      pivot_root<T>(s, d, rd[j]);
      lb[j][j] = d;
#pragma unroll
      for (int i = j + 1; i < 4; ++i) {
        T t = bk[j][i];
#pragma unroll
        for (int m = 0; m < j; ++m) t -= lb[i][m] * lb[j][m];
        lb[i][j] = t * rd[j];
      }
    }
#pragma unroll
    for (int j = 0; j < 4; ++j)
#pragma unroll
      for (int u = 0; u < 4; ++u) {
        T t = lr[u][j], tc = lc[u][j];
#pragma unroll
        for (int m = 0; m < j; ++m) { t -= lr[u][m] * lb[j][m]; tc -= lc[u][m] * lb[j][m]; }
        lr[u][j] = t * rd[j];
        lc[u][j] = tc * rd[j];
      }
    if (P <= cb0 + 3) {
#pragma unroll
      for (int u = 0; u < 4; ++u)
#pragma unroll
        for (int v = 0; v < 4; ++v)
#pragma unroll
          for (int j = 0; j < 4; ++j) a[u][v] -= lr[u][j] * lc[v][j];
      if (P + 4 < 64 && tj == q + 1) {
        // publish columns P+4..P+7 (zero above their diagonal)
#pragma unroll
        for (int v = 0; v < 4; ++v) {
          T wv[4];
#pragma unroll
          for (int u = 0; u < 4; ++u) wv[u] = (r0 + u >= P + 4 + v) ? a[u][v] : T(0);
          Vec4<T>::st(&sh.V[P + 4 + v][r0], wv);
        }
      }
    }
    if (Lout && tj == q) {
#pragma unroll
      for (int j = 0; j < 4; ++j)
#pragma unroll
        for (int u = 0; u < 4; ++u) {
          const int i = r0 + u, k = P + j;
          if (i >= k && i < kb && k < kb) Lout[i + (int64_t)k * n] = lr[u][j];
        }
    }
    if (P + 3 >= cb0) {
      if (ti == q) {
        // rows P..P+3 of X: their last substitution, then published to the warp
#pragma unroll
        for (int i = 0; i < 4; ++i) {
#pragma unroll
          for (int m = 0; m < i; ++m)
#pragma unroll
            for (int v = 0; v < 4; ++v) x[i][v] -= lb[i][m] * x[m][v];
#pragma unroll
          for (int v = 0; v < 4; ++v) x[i][v] *= rd[i];
          Vec4<T>::st(&sh.XR[w][i][4 * h], x[i]);
        }
      }
      __syncwarp();
      T xr[4][4];
#pragma unroll
      for (int j = 0; j < 4; ++j) Vec4<T>::ld(&sh.XR[w][j][4 * h], xr[j]);
#pragma unroll
      for (int u = 0; u < 4; ++u)
        if (r0 + u > P + 3) {
#pragma unroll
          for (int j = 0; j < 4; ++j)
#pragma unroll
            for (int v = 0; v < 4; ++v) x[u][v] -= lr[u][j] * xr[j][v];
        }
    }
    __syncthreads();
  }
}

// the inverse, column-major with 128-bit stores (Dinv[j * 64 + i] = X[i][j]), into D
template <typename T>
__device__ __forceinline__ void potrf_store_inverse(int kb, const T (&x)[4][4], T* __restrict__ D) {
  const int tid = threadIdx.x;
  const int r0 = 4 * (tid & 15), c0 = 4 * (tid >> 4);
#pragma unroll
  for (int v = 0; v < 4; ++v) {
    const int j = c0 + v;
    T wv[4];
#pragma unroll
    for (int u = 0; u < 4; ++u) wv[u] = (r0 + u < kb && j < kb) ? x[u][v] : T(0);
    Vec4<T>::st(D + (int64_t)j * 64 + r0, wv);
  }
}

}  // namespace uhm_gpu

namespace uhm_gpu {

// ---------------------------------------------------------------------------
// The same factorisation with a lookahead: only the 16 threads that hold the
// next pivot columns (one half warp) factor the 4 x 4 pivot block and form
// the L rows of those columns; they write them to shared memory and arrive on
// the step's mbarrier.  Every thread waits only for that barrier, applies the
// rank-4 update to its tile and advances its part of the inverse, so the
// chain from one step to the next is the half warp's update, pivot and row
// solve, not a block-wide barrier after every thread's whole step.
// ---------------------------------------------------------------------------
template <typename T>
struct PotrfLaShared {
  union {
    T V[64][64];                   // the staged block (lower triangle), until every tile is loaded
    T Lf[64][64];                  // then L, column-major: Lf[k][i] = L[i][k] (zero above the diagonal)
  };
  T pv[16][16];                    // step q's pivot block from its diagonal thread: pv[q][4 j + i] = a(P+i, P+j)
  T lbr[16][20];                   // step q's pivot factor: lb[i][j] at 4 i + j, 1 / L(P+j, P+j) at 16 + j
  T XR[8][4][8];                   // per warp: rows P..P+3 of its block of X, finished
  unsigned long long bar[16];      // step q's columns of L written (16 arrivals)
};

constexpr uint32_t POTRF_LA_WAIT = 1u << 22;

__device__ __forceinline__ bool la_wait(const unsigned long long* bar) {
  const uint32_t b = static_cast<uint32_t>(__cvta_generic_to_shared(bar));
  for (uint32_t i = 0; i < POTRF_LA_WAIT; ++i) {
    uint32_t ok;
    asm volatile(
        "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], 0;\n"
        " selp.b32 %0, 1, 0, p;\n}\n"
        : "=r"(ok)
        : "r"(b)
        : "memory");
    if (ok) return true;
  }
  return false;
}

// the half warp of tile column q1: factor the pivot block (its tile of the
// diagonal thread, ti == q1), solve its rows' L entries of columns 4 q1 ..,
// publish them and arrive
template <typename T>
__device__ __forceinline__ void la_pivot(PotrfLaShared<T>& sh, int q1, const T (&a)[4][4], int ti, int r0,
                                         bool& bad) {
  const int P1 = 4 * q1;
  const unsigned hmask = (threadIdx.x & 16) ? 0xFFFF0000u : 0x0000FFFFu;
  if (ti == q1) {
#pragma unroll
    for (int j = 0; j < 4; ++j) {
      T col[4];
#pragma unroll
      for (int i = 0; i < 4; ++i) col[i] = a[i][j];
      Vec4<T>::st(&sh.pv[q1][4 * j], col);
    }
  }
  __syncwarp(hmask);
  T bk[4][4];                      // bk[j][i] = a(P1+i, P1+j)
#pragma unroll
  for (int j = 0; j < 4; ++j) Vec4<T>::ld(&sh.pv[q1][4 * j], bk[j]);
  T lb[4][4], rd[4];
#pragma unroll
  for (int j = 0; j < 4; ++j) {
    T s = bk[j][j];
#pragma unroll
    for (int m = 0; m < j; ++m) s -= lb[j][m] * lb[j][m];
    if (!(s > T(0))) { bad = true; s = T(1); }
    T d;
    pivot_root<T>(s, d, rd[j]);
    lb[j][j] = d;
#pragma unroll
    for (int i = j + 1; i < 4; ++i) {
      T t = bk[j][i];
#pragma unroll
      for (int m = 0; m < j; ++m) t -= lb[i][m] * lb[j][m];
      lb[i][j] = t * rd[j];
    }
  }
  T l[4][4];                       // l[u][j] = L(r0+u, P1+j)
#pragma unroll
  for (int u = 0; u < 4; ++u)
#pragma unroll
    for (int j = 0; j < 4; ++j) l[u][j] = T(0);
  if (ti > q1) {
#pragma unroll
    for (int j = 0; j < 4; ++j)
#pragma unroll
      for (int u = 0; u < 4; ++u) {
        T t = a[u][j];
#pragma unroll
        for (int m = 0; m < j; ++m) t -= l[u][m] * lb[j][m];
        l[u][j] = t * rd[j];
      }
  } else if (ti == q1) {
#pragma unroll
    for (int u = 0; u < 4; ++u)
#pragma unroll
      for (int j = 0; j < 4; ++j) l[u][j] = u >= j ? lb[u][j] : T(0);
#pragma unroll
    for (int i = 0; i < 4; ++i)
#pragma unroll
      for (int j = 0; j < 4; ++j) sh.lbr[q1][4 * i + j] = lb[i][j];
#pragma unroll
    for (int j = 0; j < 4; ++j) sh.lbr[q1][16 + j] = rd[j];
  }
#pragma unroll
  for (int j = 0; j < 4; ++j) {
    T col[4];
#pragma unroll
    for (int u = 0; u < 4; ++u) col[u] = l[u][j];
    Vec4<T>::st(&sh.Lf[P1 + j][r0], col);
  }
  asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(
                   static_cast<uint32_t>(__cvta_generic_to_shared(&sh.bar[q1])))
               : "memory");
}

// Factor the 64 x 64 block at G (leading dimension n, kb <= 64 valid rows and
// columns) as potrf_block does: on return x holds this thread's tile of
// L^{-1}, the lower triangle of L has been written to Lout (leading dimension
// n) when it is not null, and bad (the same in every thread) is set when a
// pivot was not positive.  Ends with a block barrier.
template <typename T>
__device__ __forceinline__ void potrf_block_la(const T* __restrict__ G, int n, int kb, PotrfLaShared<T>& sh,
                                               T (&x)[4][4], bool& bad, T* __restrict__ Lout) {
  const int tid = threadIdx.x, w = tid >> 5;
  const int ti = tid & 15, tj = tid >> 4, h = tj & 1;
  const int r0 = 4 * ti, c0 = 4 * tj, cb0 = 8 * w;
  if (tid == 0) {
#pragma unroll 1
    for (int q = 0; q < 16; ++q)
      asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(
                       static_cast<uint32_t>(__cvta_generic_to_shared(&sh.bar[q]))),
                   "r"(16));
  }
  {
    T g[16];
#pragma unroll
    for (int u = 0; u < 16; ++u) {
      const int idx = tid + 256 * u, i = idx & 63, j = idx >> 6;
      g[u] = (i >= j && i < kb && j < kb) ? G[i + (int64_t)j * n] : (i == j ? T(1) : T(0));
    }
#pragma unroll
    for (int u = 0; u < 16; ++u) {
      const int idx = tid + 256 * u, i = idx & 63, j = idx >> 6;
      if (i >= j) sh.V[j][i] = g[u];
    }
  }
  __syncthreads();
  T a[4][4];
#pragma unroll
  for (int u = 0; u < 4; ++u)
#pragma unroll
    for (int v = 0; v < 4; ++v) {
      const int i = r0 + u, j = c0 + v;
      a[u][v] = i >= j ? sh.V[j][i] : sh.V[i][j];
      x[u][v] = i == j ? T(1) : T(0);
    }
  __syncthreads();   // every tile loaded before L overwrites the staged block
  bad = false;
  if (tj == 0) la_pivot<T>(sh, 0, a, ti, r0, bad);
#pragma unroll 1
  for (int q = 0; q < 16; ++q) {
    const int P = 4 * q;
    if (!la_wait(&sh.bar[q])) bad = true;
    T lr[4][4], lc[4][4];          // lr[u][j] = L(r0+u, P+j), lc[v][j] = L(c0+v, P+j)
#pragma unroll
    for (int j = 0; j < 4; ++j) {
      T t4[4];
      Vec4<T>::ld(&sh.Lf[P + j][r0], t4);
#pragma unroll
      for (int u = 0; u < 4; ++u) lr[u][j] = t4[u];
      Vec4<T>::ld(&sh.Lf[P + j][c0], t4);
#pragma unroll
      for (int v = 0; v < 4; ++v) lc[v][j] = t4[v];
    }
    if (tj > q) {
#pragma unroll
      for (int u = 0; u < 4; ++u)
#pragma unroll
        for (int v = 0; v < 4; ++v)
#pragma unroll
          for (int j = 0; j < 4; ++j) a[u][v] -= lr[u][j] * lc[v][j];
      if (tj == q + 1) la_pivot<T>(sh, q + 1, a, ti, r0, bad);
    }
    if (P + 3 >= cb0) {
      if (ti == q) {
        // rows P..P+3 of X: their last substitution, then published to the warp
        T lb[4][4], rd[4];
#pragma unroll
        for (int i = 0; i < 4; ++i) Vec4<T>::ld(&sh.lbr[q][4 * i], lb[i]);
        Vec4<T>::ld(&sh.lbr[q][16], rd);
#pragma unroll
        for (int i = 0; i < 4; ++i) {
#pragma unroll
          for (int m = 0; m < i; ++m)
#pragma unroll
            for (int v = 0; v < 4; ++v) x[i][v] -= lb[i][m] * x[m][v];
#pragma unroll
          for (int v = 0; v < 4; ++v) x[i][v] *= rd[i];
          Vec4<T>::st(&sh.XR[w][i][4 * h], x[i]);
        }
      }
      __syncwarp();
      T xr[4][4];
#pragma unroll
      for (int j = 0; j < 4; ++j) Vec4<T>::ld(&sh.XR[w][j][4 * h], xr[j]);
      __syncwarp();
#pragma unroll
      for (int u = 0; u < 4; ++u)
        if (r0 + u > P + 3) {
#pragma unroll
          for (int j = 0; j < 4; ++j)
#pragma unroll
            for (int v = 0; v < 4; ++v) x[u][v] -= lr[u][j] * xr[j][v];
        }
    }
  }
  bad = __syncthreads_or(bad);
  if (Lout) {
    for (int idx = tid; idx < 64 * 64; idx += 256) {
      const int i = idx & 63, k = idx >> 6;
      if (i >= k && i < kb && k < kb) Lout[i + (int64_t)k * n] = sh.Lf[k][i];
    }
  }
  if (tid == 0) {
#pragma unroll 1
    for (int q = 0; q < 16; ++q)
      asm volatile("mbarrier.inval.shared::cta.b64 [%0];" ::"r"(
          static_cast<uint32_t>(__cvta_generic_to_shared(&sh.bar[q]))));
  }
  __syncthreads();
}

}  // namespace uhm_gpu
