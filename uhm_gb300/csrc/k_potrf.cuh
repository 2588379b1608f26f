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
  T aux[512];       // potrf_block2: inverse pivot tiles, then one tile row of X
  int bad_flag;
};

// Factor the 64 x 64 block at G (leading dimension n, kb <= 64 valid rows and
// columns) in shared memory; on return x holds this thread's tile of L^{-1}
// and, when Lout is not null, the lower triangle of L has been written there
// (leading dimension n); bad is set when a pivot was not positive.  Ends
// with a block barrier.
template <typename T>
__device__ __forceinline__ void potrf_block_interleaved(const T* __restrict__ G, int n, int kb,
                                                        PotrfShared<T>& sh, T (&x)[4][4], bool& bad,
                                                        T* __restrict__ Lout) {
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

// The factorisation the kernels use, same contract as
// potrf_block_interleaved (which forms X in the same phases as L and is about
// twice as slow):
// x = this thread's tile of L^{-1}, L into Lout, bad on a non-positive pivot,
// ends with a block barrier.  Two passes instead of one interleaved pass:
//  1. L: 16 phases of 4 columns; the 4 x 4 tiles are thread-owned (thread
//     (ti, tj) = rows 4 ti .., columns 4 tj .., lower tiles only).  In phase q
//     the owners of tile column q factor the pivot tile (each redundantly,
//     read from shared memory), form their tile of L and publish it; after a
//     barrier every tile right of the column subtracts its rank-4 product,
//     the owners of the next tile column publishing their updated tiles.
//  2. L^{-1}: right-looking block substitution on L X = I: in step k the
//     tiles (k, j) become X[k][j] = L_kk^{-1} B[k][j] and are published, then
//     every tile (i > k, j <= k) subtracts L[i][k] X[k][j] from its B.
// Two barriers per phase or step, no sequential work beyond a 4 x 4 tile.
template <typename T>
__device__ __forceinline__ void potrf_block(const T* __restrict__ G, int n, int kb, PotrfShared<T>& sh,
                                            T (&x)[4][4], bool& bad, T* __restrict__ Lout) {
  const int tid = threadIdx.x;
  const int ti = tid & 15, tj = tid >> 4;
  const int r0 = 4 * ti, c0 = 4 * tj;
  const bool low = ti >= tj;
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
      a[u][v] = low ? (i >= j ? sh.V[j][i] : sh.V[i][j]) : T(0);
    }
  T* DI = sh.aux;                       // 16 inverse pivot tiles, DI[q * 16 + u * 4 + v]
  bool my_bad = false;
  if (tid == 0) sh.bad_flag = 0;
  __syncthreads();
#pragma unroll 1
  for (int q = 0; q < 16; ++q) {
    const int P = 4 * q;
    if (tj == q && low) {
      // the pivot tile (columns P..P+3 of V hold the current tile column)
      T bk[4][4];
#pragma unroll
      for (int v = 0; v < 4; ++v) {
        T t4[4];
        Vec4<T>::ld(&sh.V[P + v][P], t4);
#pragma unroll
        for (int u = 0; u < 4; ++u) bk[u][v] = t4[u];
      }
      T lb[4][4], rd[4];
#pragma unroll
      for (int v = 0; v < 4; ++v) {
        T s = bk[v][v];
#pragma unroll
        for (int m = 0; m < v; ++m) s -= lb[v][m] * lb[v][m];
        if (!(s > T(0))) { my_bad = true; s = T(1); }
        T d;
        pivot_root<T>(s, d, rd[v]);
        lb[v][v] = d;
#pragma unroll
        for (int u = v + 1; u < 4; ++u) {
          T t = bk[u][v];
#pragma unroll
          for (int m = 0; m < v; ++m) t -= lb[u][m] * lb[v][m];
          lb[u][v] = t * rd[v];
        }
#pragma unroll
        for (int u = 0; u < v; ++u) lb[u][v] = T(0);
      }
      T l[4][4];
      if (ti == q) {
#pragma unroll
        for (int u = 0; u < 4; ++u)
#pragma unroll
          for (int v = 0; v < 4; ++v) l[u][v] = lb[u][v];
        // the pivot tile's inverse, for the second pass
        T w[4][4];
#pragma unroll
        for (int cc = 0; cc < 4; ++cc)
#pragma unroll
          for (int u = 0; u < 4; ++u) {
            T t = (u == cc) ? T(1) : T(0);
#pragma unroll
            for (int m = 0; m < u; ++m) t -= lb[u][m] * w[m][cc];
            w[u][cc] = (u >= cc) ? t * rd[u] : T(0);
          }
#pragma unroll
        for (int u = 0; u < 4; ++u)
#pragma unroll
          for (int v = 0; v < 4; ++v) DI[q * 16 + u * 4 + v] = w[u][v];
      } else {
#pragma unroll
        for (int u = 0; u < 4; ++u)
#pragma unroll
          for (int v = 0; v < 4; ++v) {
            T t = a[u][v];
#pragma unroll
            for (int m = 0; m < v; ++m) t -= l[u][m] * lb[v][m];
            l[u][v] = t * rd[v];
          }
      }
#pragma unroll
      for (int v = 0; v < 4; ++v) {
        T wv[4];
#pragma unroll
        for (int u = 0; u < 4; ++u) wv[u] = l[u][v];
        Vec4<T>::st(&sh.V[P + v][r0], wv);
      }
      if (Lout) {
#pragma unroll
        for (int u = 0; u < 4; ++u)
#pragma unroll
          for (int v = 0; v < 4; ++v) {
            const int i = r0 + u, k = P + v;
            if (i >= k && i < kb && k < kb) Lout[i + (int64_t)k * n] = l[u][v];
          }
      }
    }
    __syncthreads();
    if (low && tj > q) {
      T li[4][4], lj[4][4];
#pragma unroll
      for (int m = 0; m < 4; ++m) {
        Vec4<T>::ld(&sh.V[P + m][r0], li[m]);
        Vec4<T>::ld(&sh.V[P + m][c0], lj[m]);
      }
#pragma unroll
      for (int u = 0; u < 4; ++u)
#pragma unroll
        for (int v = 0; v < 4; ++v)
#pragma unroll
          for (int m = 0; m < 4; ++m) a[u][v] -= li[m][u] * lj[m][v];
      if (tj == q + 1) {
#pragma unroll
        for (int v = 0; v < 4; ++v) {
          T wv[4];
#pragma unroll
          for (int u = 0; u < 4; ++u) wv[u] = a[u][v];
          Vec4<T>::st(&sh.V[c0 + v][r0], wv);
        }
      }
    }
    __syncthreads();
  }
  // pass 2: X = L^{-1}; B starts as the identity, x holds B then X
#pragma unroll
  for (int u = 0; u < 4; ++u)
#pragma unroll
    for (int v = 0; v < 4; ++v) x[u][v] = (ti == tj && u == v) ? T(1) : T(0);
  if (my_bad) sh.bad_flag = 1;
  T* XB = sh.aux + 256;                 // row k of X: tile j at XB[j * 16 + u * 4 + v]
#pragma unroll 1
  for (int k = 0; k < 16; ++k) {
    if (ti == k && tj <= k) {
      T y[4][4];
#pragma unroll
      for (int u = 0; u < 4; ++u)
#pragma unroll
        for (int v = 0; v < 4; ++v) {
          T t = T(0);
#pragma unroll
          for (int m = 0; m < 4; ++m) t += DI[k * 16 + u * 4 + m] * x[m][v];
          y[u][v] = t;
        }
#pragma unroll
      for (int u = 0; u < 4; ++u)
#pragma unroll
        for (int v = 0; v < 4; ++v) {
          x[u][v] = y[u][v];
          XB[tj * 16 + u * 4 + v] = y[u][v];
        }
    }
    __syncthreads();
    if (ti > k && tj <= k) {
      T lk[4][4], xk[4][4];
#pragma unroll
      for (int m = 0; m < 4; ++m) Vec4<T>::ld(&sh.V[4 * k + m][r0], lk[m]);   // lk[m][u] = L[r0+u][4k+m]
#pragma unroll
      for (int m = 0; m < 4; ++m)
#pragma unroll
        for (int v = 0; v < 4; ++v) xk[m][v] = XB[tj * 16 + m * 4 + v];
#pragma unroll
      for (int u = 0; u < 4; ++u)
#pragma unroll
        for (int v = 0; v < 4; ++v)
#pragma unroll
          for (int m = 0; m < 4; ++m) x[u][v] -= lk[m][u] * xk[m][v];
    }
    __syncthreads();
  }
  bad = sh.bad_flag != 0;
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
