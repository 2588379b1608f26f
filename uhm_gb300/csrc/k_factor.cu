// Front assembly (extend-add) and partial factorisation kernels, SIMT path.
//
// Reference steps restated here:
//   extend-add      Helper_::_merge_A -> Matrix_FLA_::merge (FLA_Axpy of
//                   sub-blocks), UHM/include/uhm/matrix/uhm/helper.hxx:191-222,
//                   UHM/src/matrix/uhm/fla/matrix.cxx:284-303; element scatter
//                   of Mesh_::copy_in, UHM/src/mesh/interf.cxx:108-204
//   Cholesky front  chol_hier, UHM/src/matrix/uhm/fla/chol/decompose.cxx:85-98
//                   (LINAL/src/dense/chol.cxx:46-92, trsm.cxx:221-247, syrk.cxx:58-90)
//   LU fronts       lu_piv_hier / lu_nopiv_hier, fla/lu_piv/decompose.cxx:124-153,
//                   fla/lu_nopiv/decompose.cxx:95-121 (pivot search restricted to
//                   the ATL rows, LINAL/src/dense/lu_piv.cxx:47-111)
//
// The extend-add is a parent-centric gather: every parent entry is written
// exactly once as  0 + sum over sources in source order  (element
// contributions, then children in child order), which is the reference's
// summation order onto a zeroed parent; no atomics, bitwise reproducible.
#include <cstdio>
#include <stdexcept>
#include "k_common.cuh"

namespace uhm_gpu {

// ---------------------------------------------------------------------------
// assembly
// ---------------------------------------------------------------------------
constexpr int ASM_TJ = 16;
constexpr int ASM_MAXSRC = 64;

template <typename T>
__global__ void __launch_bounds__(256) k_assemble(DevCtx c, const Item* __restrict__ items,
                                                  int lower) {
  __shared__ SrcDev s_src[ASM_MAXSRC];
  const Item it = items[blockIdx.x];
  const FrontDev f = c.fronts[it.front];
  const int n = f.n;
  const int nsrc = f.nsrc;
  for (int s = threadIdx.x; s < nsrc && s < ASM_MAXSRC; s += blockDim.x) s_src[s] = c.srcs[f.src0 + s];
  __syncthreads();
  T* __restrict__ P = arena<T>(c) + f.off;
  const int64_t* __restrict__ cp = c.colptr + f.colptr_off;
  const int32_t* __restrict__ inv = c.inv + f.inv_off;
  const int J0 = it.a;
  const int J1 = min(J0 + ASM_TJ, n);
  for (int J = J0; J < J1; ++J) {
    const int64_t k0 = cp[J], k1 = cp[J + 1];
    const int istart = lower ? J : 0;
    for (int I = istart + threadIdx.x; I < n; I += blockDim.x) {
      double acc = 0.0;
      for (int64_t k = k0; k < k1; ++k) {
        const int2 cs = c.colsrc[k];
        const int is = inv[(int64_t)cs.x * n + I];
        if (is >= 0) {
          const SrcDev sd = cs.x < ASM_MAXSRC ? s_src[cs.x] : c.srcs[f.src0 + cs.x];
          int r = is, cc = cs.y;
          if (sd.is_child && c.symmetric && r < cc) { int t = r; r = cc; cc = t; }
          acc += load_src(c, sd, r + (int64_t)cc * sd.ld);
        }
      }
      P[I + (int64_t)J * n] = (T)acc;
    }
  }
}

void launch_assemble(const DevCtx& c, const Item* items, int n_items, int dtype, int lower,
                     cudaStream_t s) {
  if (!n_items) return;
  if (dtype == F64) k_assemble<double><<<n_items, 256, 0, s>>>(c, items, lower);
  else k_assemble<float><<<n_items, 256, 0, s>>>(c, items, lower);
}

// ---------------------------------------------------------------------------
// block-wide argmax |v| (ties -> smaller index), for partial pivoting
// ---------------------------------------------------------------------------
template <typename T, int NT>
__device__ int block_argmax(T best, int bi, T* s_v, int* s_i) {
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    T ov = __shfl_down_sync(0xffffffffu, best, o);
    int oi = __shfl_down_sync(0xffffffffu, bi, o);
    if (ov > best || (ov == best && oi < bi)) { best = ov; bi = oi; }
  }
  if (lane == 0) { s_v[warp] = best; s_i[warp] = bi; }
  __syncthreads();
  if (warp == 0) {
    best = lane < NT / 32 ? s_v[lane] : (T)-1;
    bi = lane < NT / 32 ? s_i[lane] : 0x7fffffff;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
      T ov = __shfl_down_sync(0xffffffffu, best, o);
      int oi = __shfl_down_sync(0xffffffffu, bi, o);
      if (ov > best || (ov == best && oi < bi)) { best = ov; bi = oi; }
    }
    if (lane == 0) s_i[0] = bi;
  }
  __syncthreads();
  int r = s_i[0];
  __syncthreads();
  return r;
}

// ---------------------------------------------------------------------------
// whole-front partial factorisation in shared memory (one CTA per front)
// ---------------------------------------------------------------------------
template <typename T, int NT>
__global__ void __launch_bounds__(NT) k_small_factor(DevCtx c, const Item* __restrict__ items,
                                                     int method) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  T* A = reinterpret_cast<T*>(smem_raw);
  __shared__ T s_v[NT / 32];
  __shared__ int s_i[NT / 32];
  const Item it = items[blockIdx.x];
  const FrontDev f = c.fronts[it.front];
  const int n = f.n, fs = f.fs;
  T* __restrict__ G = arena<T>(c) + f.off;
  const bool chol = method == M_CHOL;
  const bool pivot = method == M_LU_PIV;
  const int64_t nn = (int64_t)n * n;
  for (int64_t idx = threadIdx.x; idx < nn; idx += NT) {
    const int i = (int)(idx % n), j = (int)(idx / n);
    if (!chol || i >= j) A[idx] = G[idx];
  }
  __syncthreads();
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  constexpr int NW = NT / 32;
  for (int k = 0; k < fs; ++k) {
    if (chol) {
      if (threadIdx.x == 0) {
        T d = A[k + (int64_t)k * n];
        if (!(d > (T)0)) { set_status(c, it.front, d != d ? ST_NAN : ST_NOT_SPD); d = (T)1; }
        A[k + (int64_t)k * n] = my_sqrt<T>(d);
      }
      __syncthreads();
      const T dkk = A[k + (int64_t)k * n];
      for (int i = k + 1 + threadIdx.x; i < n; i += NT) A[i + (int64_t)k * n] /= dkk;
      __syncthreads();
      for (int j = k + 1 + warp; j < n; j += NW) {
        const T ajk = A[j + (int64_t)k * n];
        T* __restrict__ col = A + (int64_t)j * n;
        const T* __restrict__ colk = A + (int64_t)k * n;
        for (int i = j + lane; i < n; i += 32) col[i] -= colk[i] * ajk;
      }
      __syncthreads();
    } else {
      if (pivot) {
        T best = (T)-1;
        int bi = k;
        for (int i = k + threadIdx.x; i < fs; i += NT) {
          const T v = my_abs<T>(A[i + (int64_t)k * n]);
          if (v > best) { best = v; bi = i; }
        }
        const int p = block_argmax<T, NT>(best, bi, s_v, s_i);
        if (threadIdx.x == 0) c.piv[f.piv_off + k] = p;
        if (p != k)
          for (int j = threadIdx.x; j < n; j += NT) {
            T t = A[k + (int64_t)j * n];
            A[k + (int64_t)j * n] = A[p + (int64_t)j * n];
            A[p + (int64_t)j * n] = t;
          }
        __syncthreads();
      }
      T akk = A[k + (int64_t)k * n];
      if (akk == (T)0 || akk != akk) {
        if (threadIdx.x == 0) set_status(c, it.front, akk != akk ? ST_NAN : ST_ZERO_PIVOT);
        akk = (T)1;
      }
      for (int i = k + 1 + threadIdx.x; i < n; i += NT) A[i + (int64_t)k * n] /= akk;
      __syncthreads();
      for (int j = k + 1 + warp; j < n; j += NW) {
        const T akj = A[k + (int64_t)j * n];
        T* __restrict__ col = A + (int64_t)j * n;
        const T* __restrict__ colk = A + (int64_t)k * n;
        for (int i = k + 1 + lane; i < n; i += 32) col[i] -= colk[i] * akj;
      }
      __syncthreads();
    }
  }
  for (int64_t idx = threadIdx.x; idx < nn; idx += NT) {
    const int i = (int)(idx % n), j = (int)(idx / n);
    if (!chol || i >= j) G[idx] = A[idx];
  }
}

void launch_small_factor(const DevCtx& c, const Item* items, int n_items, int dtype, int method,
                         int max_n, cudaStream_t s) {
  if (!n_items) return;
  if (dtype == F64) {
    size_t sm = (size_t)max_n * max_n * sizeof(double);
    cudaFuncSetAttribute(k_small_factor<double, 256>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                         (int)sm);
    k_small_factor<double, 256><<<n_items, 256, sm, s>>>(c, items, method);
  } else {
    size_t sm = (size_t)max_n * max_n * sizeof(float);
    cudaFuncSetAttribute(k_small_factor<float, 256>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                         (int)sm);
    k_small_factor<float, 256><<<n_items, 256, sm, s>>>(c, items, method);
  }
}

// ---------------------------------------------------------------------------
// blocked large-front Cholesky: diagonal block, panel TRSM, trailing update
// item: front, a = k0 (step start), b = row block / tile row, c = tile col
// ---------------------------------------------------------------------------
// Cholesky of one diagonal block (kb <= 64) and the inverse of its factor.
// 64 threads; thread i keeps row i of the block in registers (fully unrolled,
// compile-time register indices) and publishes every finished entry L[i][k]
// into a row-major shared copy.  Left-looking: the entry (i, k) is
//   L[i][k] = (A[i][k] - sum_{j<k} L[i][j] L[k][j]) / L[k][k],
// with row k read from shared memory as 128-bit vectors.  One barrier per
// column: before it, every thread has all terms j < k-1 (row k's entries up
// to k-2 are visible since the previous barrier) and thread k has its pivot
// (its own row is in registers); after it, the single missing term j = k-1
// is added.  Blocks narrower than 64 are padded with the identity.  The
// inverse L^{-1} (used by the panel TRSM and by the flag-driven solves) is
// formed column per thread by forward substitution over the shared rows and
// stored column-major with 128-bit stores.  FP32 pivots use rsqrt (the
// factor is refined in FP64 by the mixed path); FP64 uses sqrt and a divide.
template <typename T> struct PotrfVec;
template <> struct PotrfVec<float> { using V = float4; static constexpr int W = 4, RL = 68; };
template <> struct PotrfVec<double> { using V = double2; static constexpr int W = 2, RL = 66; };

template <typename T> __device__ __forceinline__ void pivot_root(T s, T& d, T& rd);
template <> __device__ __forceinline__ void pivot_root<float>(float s, float& d, float& rd) {
  rd = rsqrtf(s);
  d = s * rd;
}
template <> __device__ __forceinline__ void pivot_root<double>(double s, double& d, double& rd) {
  d = sqrt(s);
  rd = 1.0 / d;
}

// s - sum_{j < CNT} x[j] * row[j]; row 16-byte aligned; W partial sums
template <int CNT, typename T>
__device__ __forceinline__ T potrf_dot(T s, const T (&x)[64], const T* __restrict__ row) {
  constexpr int W = PotrfVec<T>::W;
  using V = typename PotrfVec<T>::V;
  T acc[W];
#pragma unroll
  for (int u = 0; u < W; ++u) acc[u] = T(0);
#pragma unroll
  for (int j = 0; j + W <= CNT; j += W) {
    const V v = *reinterpret_cast<const V*>(row + j);
    const T* pv = reinterpret_cast<const T*>(&v);
#pragma unroll
    for (int u = 0; u < W; ++u) acc[u] += x[j + u] * pv[u];
  }
#pragma unroll
  for (int j = (CNT / W) * W; j < CNT; ++j) acc[0] += x[j] * row[j];
  T t = acc[0];
#pragma unroll
  for (int u = 1; u < W; ++u) t += acc[u];
  return s - t;
}

template <int K, typename T>
struct PotrfColumn {
  static __device__ __forceinline__ void run(T (&a)[64], T* Ls, T* sd, T* srd, int i, bool& bad) {
    constexpr int RL = PotrfVec<T>::RL;
    const T* rk = Ls + K * RL;
    T s = potrf_dot<(K > 0 ? K - 1 : 0)>(a[K], a, rk);
    if (i == K) {
      if (K > 0) s -= a[K - 1] * a[K - 1];
      T piv = s;
      if (!(piv > T(0))) { bad = true; piv = T(1); }
      T d, rd;
      pivot_root<T>(piv, d, rd);
      sd[K] = d;
      srd[K] = rd;
    }
    __syncthreads();
    if (K > 0) s -= a[K - 1] * rk[K - 1];
    const T l = (i > K) ? s * srd[K] : (i == K ? sd[K] : T(0));
    a[K] = l;
    if (i > K) Ls[i * RL + K] = l;
    PotrfColumn<K + 1, T>::run(a, Ls, sd, srd, i, bad);
  }
};
template <typename T>
struct PotrfColumn<64, T> {
  static __device__ __forceinline__ void run(T (&)[64], T*, T*, T*, int, bool&) {}
};

template <int R, typename T>
struct InverseRow {
  static __device__ __forceinline__ void run(T (&x)[64], const T* Ls, const T* srd, int jc) {
    constexpr int RL = PotrfVec<T>::RL;
    x[R] = potrf_dot<R>((R == jc) ? T(1) : T(0), x, Ls + R * RL) * srd[R];
    InverseRow<R + 1, T>::run(x, Ls, srd, jc);
  }
};
template <typename T>
struct InverseRow<64, T> {
  static __device__ __forceinline__ void run(T (&)[64], const T*, const T*, int) {}
};

template <typename T>
__global__ void __launch_bounds__(64) k_potrf_diag(DevCtx c, const Item* __restrict__ items, int nb) {
  constexpr int RL = PotrfVec<T>::RL;
  __shared__ __align__(16) T Ls[64 * RL];
  __shared__ T sd[64], srd[64];
  const Item it = items[blockIdx.x];
  const FrontDev f = c.fronts[it.front];
  const int n = f.n, k0 = it.a;
  const int kb = min(nb, f.fs - k0);
  T* __restrict__ G = arena<T>(c) + f.off + k0 + (int64_t)k0 * n;
  const int i = threadIdx.x;
  T a[64];
  {
    const T* p = G + i;
#pragma unroll
    for (int j = 0; j < 64; ++j) {
      const bool in = i < kb && j < kb;
      a[j] = in ? (j <= i ? p[(int64_t)j * n] : T(0)) : (i == j ? T(1) : T(0));
    }
  }
  bool bad = false;
  PotrfColumn<0, T>::run(a, Ls, sd, srd, i, bad);
  if (bad) set_status(c, it.front, ST_NOT_SPD);
  {
    T* p = G + i;
#pragma unroll
    for (int j = 0; j < 64; ++j)
      if (i < kb && j < kb && j <= i) p[(int64_t)j * n] = a[j];
  }
  T* Dinv = (sizeof(T) == 8 ? (T*)c.dinv64 : (T*)c.dinv32);
  if (nb != 64 || !Dinv) return;
  __syncthreads();   // every row of Ls is complete
  const int jc = i;
  T x[64];
  InverseRow<0, T>::run(x, Ls, srd, jc);
  using V = typename PotrfVec<T>::V;
  constexpr int W = PotrfVec<T>::W;
  V* D = reinterpret_cast<V*>(Dinv + f.dinv_off + (int64_t)(k0 / 64) * 4096 + jc * 64);
#pragma unroll
  for (int r = 0; r < 64; r += W) {
    V v;
    T* pv = reinterpret_cast<T*>(&v);
#pragma unroll
    for (int u = 0; u < W; ++u) pv[u] = (r + u < kb && jc < kb) ? x[r + u] : T(0);
    D[r / W] = v;
  }
}

void launch_potrf_diag(const DevCtx& c, const Item* items, int n_items, int dtype, int nb,
                       cudaStream_t s) {
  if (!n_items) return;
  if (dtype == F64)
    k_potrf_diag<double><<<n_items, 64, 0, s>>>(c, items, nb);
  else
    k_potrf_diag<float><<<n_items, 64, 0, s>>>(c, items, nb);
}

constexpr int TRSM_RB = 64;   // rows per panel-TRSM block

// X (rows r0..r0+RB of columns k0..k0+kb) <- X * L11^{-T}
template <typename T, int NT>
__global__ void __launch_bounds__(NT) k_trsm_panel(DevCtx c, const Item* __restrict__ items,
                                                   int nb) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const Item it = items[blockIdx.x];
  const FrontDev f = c.fronts[it.front];
  const int n = f.n, k0 = it.a, r0 = it.b;
  const int kb = min(nb, f.fs - k0);
  const int rb = min(TRSM_RB, n - r0);
  T* L = reinterpret_cast<T*>(smem_raw);        // kb x kb (or 64 x 65 padded inverse)
  T* X = L + 64 * 65;                           // TRSM_RB x kb, ld TRSM_RB
  T* __restrict__ G = arena<T>(c) + f.off;
  const T* Dinv = (sizeof(T) == 8 ? (const T*)c.dinv64 : (const T*)c.dinv32);
  if (nb == 64 && Dinv) {
    // X <- X * L11^{-T} as a product with the inverse computed by the
    // diagonal-block kernel (stored column-major 64 x 64): no sequential
    // sweep.  Both tiles are loaded in one batch of registers.
    static_assert(NT == 256 && TRSM_RB == 64, "64 x 64 tiles over 256 threads");
    Dinv += f.dinv_off + (int64_t)(k0 / 64) * 4096;
    T xv[16], dv[16];
#pragma unroll
    for (int u = 0; u < 16; ++u) {
      const int idx = threadIdx.x + NT * u, i = idx % TRSM_RB, j = idx / TRSM_RB;
      xv[u] = (i < rb && j < kb) ? G[(r0 + i) + (int64_t)(k0 + j) * n] : (T)0;
      dv[u] = Dinv[idx];
    }
#pragma unroll
    for (int u = 0; u < 16; ++u) {
      const int idx = threadIdx.x + NT * u;
      // Dinv is column-major: Dinv[t * 64 + j] = Linv[j][t]; keep it as
      // rows t of length 64 padded to 65, so that L[t * 65 + j] = Linv[j][t]
      const int t = idx / 64, j = idx % 64;
      X[idx] = xv[u];
      L[t * 65 + j] = (t < kb && j < kb) ? dv[u] : T(0);
    }
    __syncthreads();
    const int i = threadIdx.x % TRSM_RB, jg = threadIdx.x / TRSM_RB;   // 4 column groups of 16
    T acc[16];
#pragma unroll
    for (int u = 0; u < 16; ++u) acc[u] = T(0);
    for (int t = 0; t < kb; ++t) {
      const T x = X[i + t * TRSM_RB];
#pragma unroll
      for (int u = 0; u < 16; ++u) acc[u] += x * L[t * 65 + jg * 16 + u];
    }
#pragma unroll
    for (int u = 0; u < 16; ++u) {
      const int j = jg * 16 + u;
      if (i < rb && j < kb) G[(r0 + i) + (int64_t)(k0 + j) * n] = acc[u];
    }
    return;
  }
  for (int idx = threadIdx.x; idx < kb * kb; idx += NT) {
    const int i = idx % kb, j = idx / kb;
    L[idx] = i >= j ? G[(k0 + i) + (int64_t)(k0 + j) * n] : (T)0;
  }
  for (int idx = threadIdx.x; idx < TRSM_RB * kb; idx += NT) {
    const int i = idx % TRSM_RB, j = idx / TRSM_RB;
    X[idx] = i < rb ? G[(r0 + i) + (int64_t)(k0 + j) * n] : (T)0;
  }
  __syncthreads();
  for (int j = 0; j < kb; ++j) {
    const T ljj = L[j + j * kb];
    for (int i = threadIdx.x; i < TRSM_RB; i += NT) X[i + j * TRSM_RB] /= ljj;
    __syncthreads();
    const int w = kb - j - 1;
    for (int idx = threadIdx.x; idx < TRSM_RB * w; idx += NT) {
      const int i = idx % TRSM_RB, t = j + 1 + idx / TRSM_RB;
      X[i + t * TRSM_RB] -= X[i + j * TRSM_RB] * L[t + j * kb];
    }
    __syncthreads();
  }
  for (int idx = threadIdx.x; idx < TRSM_RB * kb; idx += NT) {
    const int i = idx % TRSM_RB, j = idx / TRSM_RB;
    if (i < rb) G[(r0 + i) + (int64_t)(k0 + j) * n] = X[idx];
  }
}

void launch_trsm_panel(const DevCtx& c, const Item* items, int n_items, int dtype, int nb,
                       cudaStream_t s) {
  if (!n_items) return;
  if (dtype == F64) {
    size_t sm = (size_t)(64 * 65 + TRSM_RB * nb) * sizeof(double);
    cudaFuncSetAttribute(k_trsm_panel<double, 256>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm);
    k_trsm_panel<double, 256><<<n_items, 256, sm, s>>>(c, items, nb);
  } else {
    size_t sm = (size_t)(64 * 65 + TRSM_RB * nb) * sizeof(float);
    cudaFuncSetAttribute(k_trsm_panel<float, 256>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm);
    k_trsm_panel<float, 256><<<n_items, 256, sm, s>>>(c, items, nb);
  }
}

// Trailing update of one BM x BN tile of the front:
//   C[rows, cols] -= A[rows, k0:k0+kb] * B,  B = A[cols, k0:k0+kb]^T  (ROWPANEL=false: SYRK)
//                                            B = A[k0:k0+kb, cols]    (ROWPANEL=true: LU GEMM)
// item: front, a = k0, b = tile row, c = tile col (tiles counted from k0+kb)
template <typename T, int BM, int BN, int BK, int TM, int TN, bool ROWPANEL>
__global__ void __launch_bounds__((BM / TM) * (BN / TN))
k_tile_update(DevCtx c, const Item* __restrict__ items, int nb, int nbo) {
  constexpr int NTX = BN / TN, NTY = BM / TM, NT = NTX * NTY;
  __shared__ T As[BK][BM + 1];
  __shared__ T Bs[BK][BN + 1];
  const Item it = items[blockIdx.x];
  const FrontDev f = c.fronts[it.front];
  const int n = f.n, k0 = it.a;
  const int kb = min(nb, f.fs - k0);
  const int base = k0 + kb;
  const int R0 = base + it.b * BM, C0 = base + it.c * BN;
  // nbo > 0: update only the columns of the current outer panel (two-level blocking)
  const int cmax = nbo > 0 ? min((k0 / nbo) * nbo + nbo, f.fs) : n;
  T* __restrict__ G = arena<T>(c) + f.off;
  const int tx = threadIdx.x % NTX, ty = threadIdx.x / NTX;
  T acc[TM][TN];
#pragma unroll
  for (int i = 0; i < TM; ++i)
#pragma unroll
    for (int j = 0; j < TN; ++j) acc[i][j] = (T)0;
  // All K-chunks of both operands are loaded into registers in one batch
  // (stores to shared memory between global loads would serialise them),
  // then staged chunk by chunk.
  constexpr int KCH = 4;                                  // chunks of BK (kb <= KCH * BK)
  constexpr int PA = BK * BM / NT, PB = BK * BN / NT;    // elements per thread and chunk
  static_assert(BK * BM % NT == 0 && BK * BN % NT == 0, "whole chunks per thread");
  T ra[KCH][PA], rb[KCH][PB];
#pragma unroll
  for (int ch = 0; ch < KCH; ++ch) {
    const int kk = ch * BK;
#pragma unroll
    for (int e = 0; e < PA; ++e) {
      const int idx = threadIdx.x + NT * e, r = idx % BM, t = idx / BM;
      const int gr = R0 + r, gt = kk + t;
      ra[ch][e] = (gr < n && gt < kb) ? G[gr + (int64_t)(k0 + gt) * n] : (T)0;
    }
#pragma unroll
    for (int e = 0; e < PB; ++e) {
      const int idx = threadIdx.x + NT * e;
      if (!ROWPANEL) {
        const int r = idx % BN, t = idx / BN;
        const int gr = C0 + r, gt = kk + t;
        rb[ch][e] = (gr < n && gt < kb) ? G[gr + (int64_t)(k0 + gt) * n] : (T)0;
      } else {
        const int t = idx % BK, r = idx / BK;
        const int gr = C0 + r, gt = kk + t;
        rb[ch][e] = (gr < n && gt < kb) ? G[(k0 + gt) + (int64_t)gr * n] : (T)0;
      }
    }
  }
  for (int kk = 0; kk < kb; kk += BK) {
    const int ch = kk / BK;
#pragma unroll
    for (int cc = 0; cc < KCH; ++cc) {
      if (cc != ch) continue;
#pragma unroll
      for (int e = 0; e < PA; ++e) {
        const int idx = threadIdx.x + NT * e;
        As[idx / BM][idx % BM] = ra[cc][e];
      }
#pragma unroll
      for (int e = 0; e < PB; ++e) {
        const int idx = threadIdx.x + NT * e;
        if (!ROWPANEL) Bs[idx / BN][idx % BN] = rb[cc][e];
        else Bs[idx % BK][idx / BK] = rb[cc][e];
      }
    }
    __syncthreads();
#pragma unroll 4
    for (int t = 0; t < BK; ++t) {
      T a[TM], b[TN];
#pragma unroll
      for (int i = 0; i < TM; ++i) a[i] = As[t][ty + i * NTY];
#pragma unroll
      for (int j = 0; j < TN; ++j) b[j] = Bs[t][tx + j * NTX];
#pragma unroll
      for (int i = 0; i < TM; ++i)
#pragma unroll
        for (int j = 0; j < TN; ++j) acc[i][j] += a[i] * b[j];
    }
    __syncthreads();
  }
  // C -= acc: every C value is read before any is written back
  T cv[TM][TN];
#pragma unroll
  for (int i = 0; i < TM; ++i) {
    const int gr = R0 + ty + i * NTY;
#pragma unroll
    for (int j = 0; j < TN; ++j) {
      const int gc = C0 + tx + j * NTX;
      const bool ok = gr < n && gc < cmax && (ROWPANEL || gr >= gc);
      cv[i][j] = ok ? G[gr + (int64_t)gc * n] : (T)0;
    }
  }
#pragma unroll
  for (int i = 0; i < TM; ++i) {
    const int gr = R0 + ty + i * NTY;
#pragma unroll
    for (int j = 0; j < TN; ++j) {
      const int gc = C0 + tx + j * NTX;
      const bool ok = gr < n && gc < cmax && (ROWPANEL || gr >= gc);
      if (ok) G[gr + (int64_t)gc * n] = cv[i][j] - acc[i][j];
    }
  }
}

void launch_syrk_update(const DevCtx& c, const Item* items, int n_items, int dtype, int nb,
                        int nbo, cudaStream_t s) {
  if (!n_items) return;
  if (nb > 64) throw std::invalid_argument("trailing update: panel width above 64");
  if (dtype == F64) k_tile_update<double, 64, 64, 16, 4, 4, false><<<n_items, 256, 0, s>>>(c, items, nb, nbo);
  else k_tile_update<float, 64, 64, 16, 4, 4, false><<<n_items, 256, 0, s>>>(c, items, nb, nbo);
}

void launch_gemm_update(const DevCtx& c, const Item* items, int n_items, int dtype, int nb,
                        cudaStream_t s) {
  if (nb > 64) throw std::invalid_argument("trailing update: panel width above 64");
  if (!n_items) return;
  if (dtype == F64) k_tile_update<double, 64, 64, 16, 4, 4, true><<<n_items, 256, 0, s>>>(c, items, nb, 0);
  else k_tile_update<float, 64, 64, 16, 4, 4, true><<<n_items, 256, 0, s>>>(c, items, nb, 0);
}

// ---------------------------------------------------------------------------
// blocked large-front LU: panel (with pivot search restricted to rows < fs),
// row-panel solve U12 = L11^{-1} A12, trailing GEMM (k_tile_update<..., true>)
// ---------------------------------------------------------------------------
template <typename T, int NT>
__global__ void __launch_bounds__(NT) k_getrf_panel(DevCtx c, const Item* __restrict__ items,
                                                    int nb, int pivot) {
  __shared__ T s_v[NT / 32];
  __shared__ int s_i[NT / 32];
  const Item it = items[blockIdx.x];
  const FrontDev f = c.fronts[it.front];
  const int n = f.n, fs = f.fs, k0 = it.a;
  const int kb = min(nb, fs - k0);
  T* __restrict__ G = arena<T>(c) + f.off;
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  constexpr int NW = NT / 32;
  for (int k = k0; k < k0 + kb; ++k) {
    if (pivot) {
      T best = (T)-1;
      int bi = k;
      for (int i = k + threadIdx.x; i < fs; i += NT) {
        const T v = my_abs<T>(G[i + (int64_t)k * n]);
        if (v > best) { best = v; bi = i; }
      }
      const int p = block_argmax<T, NT>(best, bi, s_v, s_i);
      if (threadIdx.x == 0) c.piv[f.piv_off + k] = p;
      if (p != k)
        for (int j = threadIdx.x; j < n; j += NT) {
          T t = G[k + (int64_t)j * n];
          G[k + (int64_t)j * n] = G[p + (int64_t)j * n];
          G[p + (int64_t)j * n] = t;
        }
      __syncthreads();
    }
    T akk = G[k + (int64_t)k * n];
    if (akk == (T)0 || akk != akk) {
      if (threadIdx.x == 0) set_status(c, it.front, akk != akk ? ST_NAN : ST_ZERO_PIVOT);
      akk = (T)1;
    }
    __syncthreads();
    for (int i = k + 1 + threadIdx.x; i < n; i += NT) G[i + (int64_t)k * n] /= akk;
    __syncthreads();
    for (int j = k + 1 + warp; j < k0 + kb; j += NW) {
      const T akj = G[k + (int64_t)j * n];
      for (int i = k + 1 + lane; i < n; i += 32) G[i + (int64_t)j * n] -= G[i + (int64_t)k * n] * akj;
    }
    __syncthreads();
  }
}

void launch_getrf_panel(const DevCtx& c, const Item* items, int n_items, int dtype, int nb,
                        int pivot, cudaStream_t s) {
  if (!n_items) return;
  if (dtype == F64) k_getrf_panel<double, 512><<<n_items, 512, 0, s>>>(c, items, nb, pivot);
  else k_getrf_panel<float, 512><<<n_items, 512, 0, s>>>(c, items, nb, pivot);
}

constexpr int LUROW_CB = 64;   // columns per row-panel block

// A[k0:k0+kb, cols] <- L11^{-1} A[k0:k0+kb, cols]  (unit lower), cols >= k0+kb
template <typename T, int NT>
__global__ void __launch_bounds__(NT) k_lu_row_update(DevCtx c, const Item* __restrict__ items,
                                                      int nb) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const Item it = items[blockIdx.x];
  const FrontDev f = c.fronts[it.front];
  const int n = f.n, k0 = it.a, c0 = it.b;
  const int kb = min(nb, f.fs - k0);
  const int cb = min(LUROW_CB, n - c0);
  T* L = reinterpret_cast<T*>(smem_raw);      // kb x kb
  T* X = L + nb * nb;                         // kb x LUROW_CB, ld nb
  T* __restrict__ G = arena<T>(c) + f.off;
  for (int idx = threadIdx.x; idx < kb * kb; idx += NT) {
    const int i = idx % kb, j = idx / kb;
    L[idx] = i > j ? G[(k0 + i) + (int64_t)(k0 + j) * n] : (T)0;
  }
  for (int idx = threadIdx.x; idx < nb * LUROW_CB; idx += NT) {
    const int i = idx % nb, j = idx / nb;
    X[idx] = (i < kb && j < cb) ? G[(k0 + i) + (int64_t)(c0 + j) * n] : (T)0;
  }
  __syncthreads();
  for (int k = 0; k < kb; ++k) {
    const int h = kb - k - 1;
    for (int idx = threadIdx.x; idx < h * LUROW_CB; idx += NT) {
      const int i = k + 1 + idx % h, j = idx / h;
      X[i + j * nb] -= L[i + k * kb] * X[k + j * nb];
    }
    __syncthreads();
  }
  for (int idx = threadIdx.x; idx < nb * LUROW_CB; idx += NT) {
    const int i = idx % nb, j = idx / nb;
    if (i < kb && j < cb) G[(k0 + i) + (int64_t)(c0 + j) * n] = X[idx];
  }
}

void launch_lu_row_update(const DevCtx& c, const Item* items, int n_items, int dtype, int nb,
                          int pivot, cudaStream_t s) {
  (void)pivot;
  if (!n_items) return;
  if (dtype == F64) {
    size_t sm = (size_t)(nb * nb + nb * LUROW_CB) * sizeof(double);
    cudaFuncSetAttribute(k_lu_row_update<double, 256>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm);
    k_lu_row_update<double, 256><<<n_items, 256, sm, s>>>(c, items, nb);
  } else {
    size_t sm = (size_t)(nb * nb + nb * LUROW_CB) * sizeof(float);
    cudaFuncSetAttribute(k_lu_row_update<float, 256>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm);
    k_lu_row_update<float, 256><<<n_items, 256, sm, s>>>(c, items, nb);
  }
}

// ---------------------------------------------------------------------------
// FP64 <-> FP32 panel conversion (mixed precision bookkeeping)
// ---------------------------------------------------------------------------
__global__ void k_convert(DevCtx c, const Item* __restrict__ items, int to_f32) {
  const Item it = items[blockIdx.y];
  const FrontDev f = c.fronts[it.front];
  const int64_t nn = (int64_t)f.n * f.n;
  const int64_t o64 = ((int64_t)it.a << 32) | (uint32_t)it.b;   // FP64 shadow offset
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < nn;
       i += (int64_t)gridDim.x * blockDim.x) {
    if (to_f32) c.a32[f.off + i] = (float)c.a64[o64 + i];
    else c.a64[o64 + i] = (double)c.a32[f.off + i];
  }
}

void launch_convert_panels(const DevCtx& c, const Item* items, int n_items, int to_f32,
                           cudaStream_t s) {
  if (!n_items) return;
  dim3 g(64, n_items);
  k_convert<<<g, 256, 0, s>>>(c, items, to_f32);
}

}  // namespace uhm_gpu
