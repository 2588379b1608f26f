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
// The sum is formed in the front's precision: FP64 fronts in FP64, FP32
// fronts in FP32 (FP64 arithmetic runs at a small fraction of the FP32 rate
// on this GPU, and the FP32 front stores the sum in FP32 either way).
#include <cstdio>
#include <stdexcept>
#include <string>
#include "k_common.cuh"
#include "k_potrf.cuh"

namespace uhm_gpu {

// ---------------------------------------------------------------------------
// assembly
// ---------------------------------------------------------------------------
constexpr int ASM_TJ = 16;
constexpr int ASM_MAXSRC = 64;

// Extend-add of a front below ASM_SCATTER_MIN rows: 16 parent columns per
// CTA, one thread per parent row, the column's sources walked in summation
// order (element first, then the children in child order) through their
// inverse row maps.  Each parent entry is written once; a child's
// lower-stored Schur block is read transposed where the parent row falls
// above its diagonal.  (Forms with several rows per thread, or a warp per
// column with the sources decoded once per pass, issued more instructions
// per entry on these front sizes and measured slower.)
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
      T acc = T(0);
      for (int64_t k = k0; k < k1; ++k) {
        const int2 cs = c.colsrc[k];
        const int is = inv[(int64_t)cs.x * n + I];
        if (is >= 0) {
          const SrcDev sd = cs.x < ASM_MAXSRC ? s_src[cs.x] : c.srcs[f.src0 + cs.x];
          int r = is, cc = cs.y;
          if (sd.is_child && c.symmetric && r < cc) { int t = r; r = cc; cc = t; }
          acc += (T)load_src(c, sd, r + (int64_t)cc * sd.ld);
        }
      }
      P[I + (int64_t)J * n] = acc;
    }
  }
}

// Extend-add of a large front, one parent column J per CTA.  The column is
// accumulated in shared memory (in the front's precision): zero, then each source holding
// column J in source order (the element, then the children in child order)
// scatters its column through its row map (an injective map, so a source
// never hits the same entry twice and one barrier between sources keeps the
// order); then the column is written once.  Every entry therefore gets the
// same sum in the same order as in k_assemble (bit-identical), but each
// source entry is read once instead of every parent row looking up every
// source.  NT threads, four rows each per pass.  EARLY: a child's stored
// part of its column (rows at or below its diagonal, every row of an
// unsymmetric child) is read beside the row-map look-up instead of after it
// (only rows stored transposed, and element rows, wait for their parent row
// to be known); it paid on the root's launch (fronts above ASM_EARLY_MIN
// rows, 512 threads) and not on the levels below.
constexpr int ASM_EARLY_MIN = 8192;

template <typename T, int NT, bool EARLY>
__global__ void __launch_bounds__(NT) k_assemble_scatter(DevCtx c, const Item* __restrict__ items, int lower) {
  extern __shared__ __align__(16) unsigned char sc_raw[];
  T* s_col = reinterpret_cast<T*>(sc_raw);
  const Item it = items[blockIdx.x];
  const FrontDev f = c.fronts[it.front];
  const int n = f.n, J = it.a;
  const int istart = lower ? J : 0;
  for (int I = istart + threadIdx.x; I < n; I += NT) s_col[I] = T(0);
  const int64_t* __restrict__ cp = c.colptr + f.colptr_off;
  const int64_t k0 = cp[J], k1 = cp[J + 1];
  __syncthreads();
  for (int64_t k = k0; k < k1; ++k) {
    const int2 cs = c.colsrc[k];
    const SrcDev sd = c.srcs[f.src0 + cs.x];
    const int32_t* __restrict__ fw = c.fwd + sd.fwd_off;
    const bool sym = sd.is_child && c.symmetric;
    // the source decoded once; per pass every thread issues all its map
    // look-ups, then all its loads, then the shared-memory adds
    const double* __restrict__ b64 = !sd.is_child ? c.emat + sd.off : (sd.dtype == F64 ? c.a64 + sd.off : nullptr);
    const float* __restrict__ b32 = (sd.is_child && sd.dtype != F64) ? c.a32 + sd.off : nullptr;
    const int cc = cs.y;
    // rows r >= rs are stored in column cc and read at once (EARLY)
    const int rs = !EARLY ? sd.m : (sd.is_child ? (sym ? cc : 0) : sd.m);
    for (int r0 = 0; r0 < sd.m; r0 += 4 * NT) {
      int I[4];
      T v[4];
#pragma unroll
      for (int u = 0; u < 4; ++u) {
        const int r = r0 + threadIdx.x + NT * u;
        I[u] = r < sd.m ? __ldg(fw + r) : -1;
      }
#pragma unroll
      for (int u = 0; u < 4; ++u) {
        const int r = r0 + threadIdx.x + NT * u;
        v[u] = T(0);
        if (r < sd.m && r >= rs) {
          const int64_t idx = r + (int64_t)cc * sd.ld;
          v[u] = b32 ? (T)b32[idx] : (T)b64[idx];
        }
      }
#pragma unroll
      for (int u = 0; u < 4; ++u) {
        const int r = r0 + threadIdx.x + NT * u;
        if (I[u] >= istart) {
          if (r < rs) {
            int rr = r, cl = cc;
            if (sym && rr < cl) { const int t = rr; rr = cl; cl = t; }
            const int64_t idx = rr + (int64_t)cl * sd.ld;
            v[u] = b32 ? (T)b32[idx] : (T)b64[idx];
          }
          s_col[I[u]] += v[u];
        }
      }
    }
    __syncthreads();
  }
  T* __restrict__ P = arena<T>(c) + f.off + (int64_t)J * n;
  for (int I = istart + threadIdx.x; I < n; I += NT) P[I] = s_col[I];
}

template <typename T>
static void assemble_scatter_t(const DevCtx& c, const Item* items, int n_items, int lower, int n_max,
                               cudaStream_t s) {
  const size_t sm = sizeof(T) * (size_t)n_max;
  if (n_max >= ASM_EARLY_MIN) {
    cudaFuncSetAttribute(k_assemble_scatter<T, 512, true>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm);
    k_assemble_scatter<T, 512, true><<<n_items, 512, sm, s>>>(c, items, lower);
  } else {
    cudaFuncSetAttribute(k_assemble_scatter<T, 256, false>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm);
    k_assemble_scatter<T, 256, false><<<n_items, 256, sm, s>>>(c, items, lower);
  }
}

void launch_assemble_scatter(const DevCtx& c, const Item* items, int n_items, int dtype, int lower,
                             int n_max, cudaStream_t s) {
  if (!n_items) return;
  if (dtype == F64) assemble_scatter_t<double>(c, items, n_items, lower, n_max, s);
  else assemble_scatter_t<float>(c, items, n_items, lower, n_max, s);
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
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  constexpr int NW = NT / 32;
  // the front in (its lower triangle for Cholesky): a warp per column, no
  // index division
  for (int j = warp; j < n; j += NW)
    for (int i = (chol ? j : 0) + lane; i < n; i += 32) A[i + (int64_t)j * n] = G[i + (int64_t)j * n];
  __syncthreads();
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
  for (int j = warp; j < n; j += NW)
    for (int i = (chol ? j : 0) + lane; i < n; i += 32) G[i + (int64_t)j * n] = A[i + (int64_t)j * n];
}

// Cholesky fronts in shared memory, one CTA per front: the lower triangle is
// staged with eight loads in flight per thread; the fs factor columns are
// factored column by column as in k_small_factor, but each step updates only
// the panel's later columns; the Schur block is then updated once from the
// factor panel in 4 x 4 register tiles, subtracting the fs products in
// column order -- the same operations in the same order as k_small_factor's
// rank-1 steps (bit-identical), with one shared-memory read and write per
// Schur entry instead of one per entry and step.
template <typename T, int NT>
__global__ void __launch_bounds__(NT) k_small_chol(DevCtx c, const Item* __restrict__ items) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  T* A = reinterpret_cast<T*>(smem_raw);
  const Item it = items[blockIdx.x];
  const FrontDev f = c.fronts[it.front];
  const int n = f.n, fs = f.fs;
  T* __restrict__ G = arena<T>(c) + f.off;
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  constexpr int NW = NT / 32;
  const int nn = n * n;
  // flat index e = i + j n walked in steps of NT with (i, j) kept by carry
  const int qs = NT / n, rs = NT % n;
  {
    int i0 = threadIdx.x % n, j0 = threadIdx.x / n;
    for (int e0 = 0; e0 < nn; e0 += 8 * NT) {
      T v[8];
      int i = i0, j = j0;
#pragma unroll
      for (int u = 0; u < 8; ++u) {
        const int e = e0 + threadIdx.x + u * NT;
        v[u] = (e < nn && i >= j) ? G[e] : T(0);
        i += rs; j += qs;
        if (i >= n) { i -= n; ++j; }
      }
      i = i0; j = j0;
#pragma unroll
      for (int u = 0; u < 8; ++u) {
        const int e = e0 + threadIdx.x + u * NT;
        if (e < nn && i >= j) A[e] = v[u];
        i += rs; j += qs;
        if (i >= n) { i -= n; ++j; }
      }
      i0 = i; j0 = j;
    }
  }
  __syncthreads();
  for (int k = 0; k < fs; ++k) {
    if (threadIdx.x == 0) {
      T d = A[k + k * n];
      if (!(d > (T)0)) { set_status(c, it.front, d != d ? ST_NAN : ST_NOT_SPD); d = (T)1; }
      A[k + k * n] = my_sqrt<T>(d);
    }
    __syncthreads();
    const T dkk = A[k + k * n];
    for (int i = k + 1 + threadIdx.x; i < n; i += NT) A[i + k * n] /= dkk;
    __syncthreads();
    for (int j = k + 1 + warp; j < fs; j += NW) {
      const T ajk = A[j + k * n];
      T* __restrict__ col = A + j * n;
      const T* __restrict__ colk = A + k * n;
      for (int i = j + lane; i < n; i += 32) col[i] -= colk[i] * ajk;
    }
    __syncthreads();
  }
  // Schur block S (rows / columns fs .. n-1): S -= L21 L21^T by 4 x 4 tiles
  // of its lower triangle, tile t -> (ti, tj), ti >= tj
  const int m = n - fs, tm = (m + 3) / 4, ntile = tm * (tm + 1) / 2;
  for (int t = threadIdx.x; t < ntile; t += NT) {
    int ti = (int)((sqrtf(8.f * (float)t + 1.f) - 1.f) * 0.5f);
    while (ti * (ti + 1) / 2 > t) --ti;
    while ((ti + 1) * (ti + 2) / 2 <= t) ++ti;
    const int tj = t - ti * (ti + 1) / 2;
    const int r0 = fs + 4 * ti, c0 = fs + 4 * tj;
    T acc[4][4];
#pragma unroll
    for (int u = 0; u < 4; ++u)
#pragma unroll
      for (int v = 0; v < 4; ++v) {
        const int i = r0 + u, j = c0 + v;
        acc[u][v] = (i < n && j < n && i >= j) ? A[i + j * n] : T(0);
      }
    for (int k = 0; k < fs; ++k) {
      const T* __restrict__ colk = A + k * n;
      T x[4], y[4];
#pragma unroll
      for (int u = 0; u < 4; ++u) {
        x[u] = r0 + u < n ? colk[r0 + u] : T(0);
        y[u] = c0 + u < n ? colk[c0 + u] : T(0);
      }
#pragma unroll
      for (int u = 0; u < 4; ++u)
#pragma unroll
        for (int v = 0; v < 4; ++v) acc[u][v] -= x[u] * y[v];
    }
#pragma unroll
    for (int u = 0; u < 4; ++u)
#pragma unroll
      for (int v = 0; v < 4; ++v) {
        const int i = r0 + u, j = c0 + v;
        if (i < n && j < n && i >= j) A[i + j * n] = acc[u][v];
      }
  }
  __syncthreads();
  {
    int i0 = threadIdx.x % n, j0 = threadIdx.x / n;
    for (int e0 = 0; e0 < nn; e0 += 8 * NT) {
      int i = i0, j = j0;
#pragma unroll
      for (int u = 0; u < 8; ++u) {
        const int e = e0 + threadIdx.x + u * NT;
        if (e < nn && i >= j) G[e] = A[e];
        i += rs; j += qs;
        if (i >= n) { i -= n; ++j; }
      }
      i0 = i; j0 = j;
    }
  }
}

void launch_small_factor(const DevCtx& c, const Item* items, int n_items, int dtype, int method,
                         int max_n, cudaStream_t s) {
  if (!n_items) return;
  if (method == M_CHOL) {
    if (dtype == F64) {
      const size_t sm = (size_t)max_n * max_n * sizeof(double);
      cudaFuncSetAttribute(k_small_chol<double, 256>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm);
      k_small_chol<double, 256><<<n_items, 256, sm, s>>>(c, items);
    } else {
      const size_t sm = (size_t)max_n * max_n * sizeof(float);
      cudaFuncSetAttribute(k_small_chol<float, 256>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm);
      k_small_chol<float, 256><<<n_items, 256, sm, s>>>(c, items);
    }
    return;
  }
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
// Cholesky of one diagonal block (kb <= 64) and the inverse of its factor,
// 256 threads = 8 warps (potrf_block, shared by k_potrf_diag and the fused
// k_potrf_trsm).  Warp w owns the column block 8w..8w+7 of the symmetric
// 64 x 64 block and of the inverse X = L^{-1} being formed; lane (ti, h)
// keeps the 4 x 4 tile at rows 4 ti.., columns 8w + 4h.. of both in
// registers.  Right-looking, four columns P..P+3 per phase: the columns, as
// reduced by all earlier phases, were published in shared memory (V[P+j]);
// every thread factors their 4 x 4 pivot block itself, forms the factor
// entries of its 4 rows and 4 columns by a 4-step substitution
//   l_rj = (v_{P+j}[r] - sum_{m<j} l_rm l_{P+j,P+m}) / l_{P+j,P+j},
// and applies the rank-4 update A -= L_r L_c^T to its tile; the owners of
// columns P+4..P+7 then publish them.  In the same phase the owners of rows
// P..P+3 of X finish them with the pivot block's substitution and the other
// rows take the rank-4 update X -= L[:, P:P+4] X[P:P+4, :] (column blocks of
// X are independent, so rows go through shared memory per warp).  One block
// barrier per phase, 16 in all.  A warp does only the factor work that
// reaches its columns and only the inverse work whose rows are nonzero in
// them.  Blocks narrower than 64 are padded with the identity.  FP32 pivots
// use rsqrt (the factor is refined in FP64 by the mixed path); FP64 uses sqrt
// and a divide.  Measured alternatives: one column per phase (64 barriers)
// took 2x as long; a fully unrolled left-looking version (one row per
// thread, ~100 KB of straight-line code) was bound by instruction fetch;
// hand-offs between warps on mbarriers or shared flags instead of the block
// barrier were slower (their wake-up latency).
template <typename T>
__global__ void __launch_bounds__(256) k_potrf_diag(DevCtx c, const Item* __restrict__ items, int nb) {
  __shared__ __align__(16) PotrfShared<T> sh;
  const Item it = items[blockIdx.x];
  const FrontDev f = c.fronts[it.front];
  const int n = f.n, k0 = it.a;
  const int kb = min(nb, f.fs - k0);
  T* __restrict__ G = arena<T>(c) + f.off + k0 + (int64_t)k0 * n;
  T x[4][4];
  bool bad;
  // L is written over the block in place: only this CTA reads it
  potrf_block<T>(G, n, kb, sh, x, bad, G);
  if (bad && threadIdx.x == 0) set_status(c, it.front, ST_NOT_SPD);
  T* Dinv = (sizeof(T) == 8 ? (T*)c.dinv64 : (T*)c.dinv32);
  if (nb == 64 && Dinv) potrf_store_inverse<T>(kb, x, Dinv + f.dinv_off + (int64_t)(k0 / 64) * 4096);
}

void launch_potrf_diag(const DevCtx& c, const Item* items, int n_items, int dtype, int nb,
                       cudaStream_t s) {
  if (!n_items) return;
  if (nb > 64) throw std::invalid_argument("potrf_diag: block wider than 64");
  if (dtype == F64)
    k_potrf_diag<double><<<n_items, 256, 0, s>>>(c, items, nb);
  else
    k_potrf_diag<float><<<n_items, 256, 0, s>>>(c, items, nb);
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
  T* L = reinterpret_cast<T*>(smem_raw);        // kb x kb (or 64 x 68 padded inverse)
  T* X = L + 64 * 68;                           // TRSM_RB x kb, ld TRSM_RB
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
      // rows t of length 64 padded to 68 (16-byte rows), L[t * 68 + j] = Linv[j][t]
      const int t = idx / 64, j = idx % 64;
      X[idx] = xv[u];
      L[t * 68 + j] = (t < kb && j < kb) ? dv[u] : T(0);
    }
    __syncthreads();
    const int i = threadIdx.x % TRSM_RB, jg = threadIdx.x / TRSM_RB;   // 4 column groups of 16
    T acc[16];
#pragma unroll
    for (int u = 0; u < 16; ++u) acc[u] = T(0);
    for (int t = 0; t < kb; ++t) {
      const T x = X[i + t * TRSM_RB];
#pragma unroll
      for (int u4 = 0; u4 < 16; u4 += 4) {
        T l4[4];
        Vec4<T>::ld(&L[t * 68 + jg * 16 + u4], l4);
#pragma unroll
        for (int e = 0; e < 4; ++e) acc[u4 + e] += x * l4[e];
      }
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
    size_t sm = (size_t)(64 * 68 + TRSM_RB * nb) * sizeof(double);
    cudaFuncSetAttribute(k_trsm_panel<double, 256>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm);
    k_trsm_panel<double, 256><<<n_items, 256, sm, s>>>(c, items, nb);
  } else {
    size_t sm = (size_t)(64 * 68 + TRSM_RB * nb) * sizeof(float);
    cudaFuncSetAttribute(k_trsm_panel<float, 256>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm);
    k_trsm_panel<float, 256><<<n_items, 256, sm, s>>>(c, items, nb);
  }
}

// Diagonal block and panel TRSM of one 64-column step in one launch.  Every
// CTA factors the diagonal block and forms its inverse itself (potrf_block;
// the SMs would otherwise idle through that latency-bound step), then
// applies X <- X L^{-T} = X (L^{-1})^T to its 64-row block of the panel.  The
// CTA flagged in the item writes the inverse, which is how the factor's
// diagonal block is kept: the flag-driven solves and this TRSM use only the
// inverse, and writing L over the block in place would race with other
// CTAs still reading A's block, so the arena keeps A's diagonal block.  A CTA
// takes several consecutive row blocks, so that a step's launch is one wave.
// Item: front, a = k0, b = first row of the first block (n: none),
// c = writer (bit 0) + 2 * number of row blocks.
constexpr int PT_LD = 68;   // row length of the transposed inverse in shared memory (16-byte rows)

template <typename T>
__global__ void __launch_bounds__(256) k_potrf_trsm(DevCtx c, const Item* __restrict__ items) {
  extern __shared__ __align__(16) unsigned char pt_smem[];
  PotrfShared<T>& sh = *reinterpret_cast<PotrfShared<T>*>(pt_smem);
  T* Lt = reinterpret_cast<T*>(pt_smem + ((sizeof(PotrfShared<T>) + 15) / 16) * 16);   // 64 x PT_LD
  const Item it = items[blockIdx.x];
  const FrontDev f = c.fronts[it.front];
  const int n = f.n, k0 = it.a;
  const int kb = min(64, f.fs - k0);
  T* __restrict__ A = arena<T>(c) + f.off;
  T* __restrict__ G = A + k0 + (int64_t)k0 * n;
  const int tid = threadIdx.x;
  T x[4][4];
  bool bad;
  potrf_block<T>(G, n, kb, sh, x, bad, nullptr);
  const bool writer = it.c & 1;
  const int nrb = it.c >> 1;
  if (writer) {
    if (bad && tid == 0) set_status(c, it.front, ST_NOT_SPD);
    T* Dinv = (sizeof(T) == 8 ? (T*)c.dinv64 : (T*)c.dinv32);
    potrf_store_inverse<T>(kb, x, Dinv + f.dinv_off + (int64_t)(k0 / 64) * 4096);
  }
  if (it.b >= n || nrb == 0) return;
  // L^{-1} transposed into Lt (Lt[t * PT_LD + j] = Linv[j][t]); the panel
  // blocks into V in turn (its factor values are no longer needed)
  {
    const int ti = tid & 15, tj = tid >> 4;
#pragma unroll
    for (int u = 0; u < 4; ++u)
#pragma unroll
      for (int v = 0; v < 4; ++v) {
        const int j = 4 * ti + u, t = 4 * tj + v;   // x[u][v] = Linv[j][t]
        Lt[t * PT_LD + j] = (j < kb && t < kb) ? x[u][v] : T(0);
      }
  }
  T* X = &sh.V[0][0];   // 64 x 64, column-major
  const int i = tid % TRSM_RB, jg = tid / TRSM_RB;   // 4 column groups of 16
  for (int blk = 0; blk < nrb; ++blk) {
    const int r0 = it.b + blk * TRSM_RB;
    if (r0 >= n) break;
    const int rb = min(TRSM_RB, n - r0);
    {
      T xv[16];
#pragma unroll
      for (int u = 0; u < 16; ++u) {
        const int idx = tid + 256 * u, ii = idx % TRSM_RB, j = idx / TRSM_RB;
        xv[u] = (ii < rb && j < kb) ? A[(r0 + ii) + (int64_t)(k0 + j) * n] : (T)0;
      }
      __syncthreads();   // the previous block's reads of X are done
#pragma unroll
      for (int u = 0; u < 16; ++u) X[tid + 256 * u] = xv[u];
    }
    __syncthreads();
    T acc[16];
#pragma unroll
    for (int u = 0; u < 16; ++u) acc[u] = T(0);
    for (int t = 0; t < kb; ++t) {
      const T xt = X[i + t * TRSM_RB];
#pragma unroll
      for (int u4 = 0; u4 < 16; u4 += 4) {
        T l4[4];
        Vec4<T>::ld(&Lt[t * PT_LD + jg * 16 + u4], l4);
#pragma unroll
        for (int e = 0; e < 4; ++e) acc[u4 + e] += xt * l4[e];
      }
    }
#pragma unroll
    for (int u = 0; u < 16; ++u) {
      const int j = jg * 16 + u;
      if (i < rb && j < kb) A[(r0 + i) + (int64_t)(k0 + j) * n] = acc[u];
    }
  }
}

void launch_potrf_trsm(const DevCtx& c, const Item* items, int n_items, int dtype, cudaStream_t s) {
  if (!n_items) return;
  if (dtype == F64) {
    const size_t sm = ((sizeof(PotrfShared<double>) + 15) / 16) * 16 + sizeof(double) * 64 * PT_LD;
    cudaFuncSetAttribute(k_potrf_trsm<double>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm);
    k_potrf_trsm<double><<<n_items, 256, sm, s>>>(c, items);
  } else {
    const size_t sm = ((sizeof(PotrfShared<float>) + 15) / 16) * 16 + sizeof(float) * 64 * PT_LD;
    cudaFuncSetAttribute(k_potrf_trsm<float>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm);
    k_potrf_trsm<float><<<n_items, 256, sm, s>>>(c, items);
  }
}

// Trailing update of one BM x BN tile of the front:
//   C[rows, cols] -= A[rows, k0:k0+kb] * B,  B = A[cols, k0:k0+kb]^T  (ROWPANEL=false: SYRK)
//                                            B = A[k0:k0+kb, cols]    (ROWPANEL=true: LU GEMM)
// item: front, a = k0, b = tile row, c = tile col (tiles counted from k0+kb).
// With two-level blocking (nbo > 0) B = K0 + min(nbo, fs - K0) is the first
// row / column of the current outer panel's trailing block, and region
// selects what is updated: 0 every entry, 1 columns < B (inside the outer
// panel), 2 rows < B and columns >= B (the outer panel's rows right of it).
template <typename T, int BM, int BN, int BK, int TM, int TN, bool ROWPANEL>
__global__ void __launch_bounds__((BM / TM) * (BN / TN))
k_tile_update(DevCtx c, const Item* __restrict__ items, int nb, int nbo, int region) {
  constexpr int NTX = BN / TN, NTY = BM / TM, NT = NTX * NTY;
  __shared__ T As[BK][BM + 1];
  __shared__ T Bs[BK][BN + 1];
  const Item it = items[blockIdx.x];
  const FrontDev f = c.fronts[it.front];
  const int n = f.n, k0 = it.a;
  const int kb = min(nb, f.fs - k0);
  const int base = k0 + kb;
  const int R0 = base + it.b * BM, C0 = base + it.c * BN;
  const int Bnd = nbo > 0 ? min((k0 / nbo) * nbo + nbo, f.fs) : n;
  const int rmax = region == 2 ? Bnd : n;
  const int cmin = region == 2 ? Bnd : 0;
  const int cmax = region == 1 ? Bnd : n;
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
  // FP32: the C tile does not depend on the arithmetic, so its loads go out
  // with the operands' and their latency overlaps the products (FP64 keeps
  // them after the products: the extra registers would halve its occupancy)
  constexpr bool EARLY_C = sizeof(T) == 4;
  T cv[TM][TN];
  auto load_c = [&]() {
#pragma unroll
    for (int i = 0; i < TM; ++i) {
      const int gr = R0 + ty + i * NTY;
#pragma unroll
      for (int j = 0; j < TN; ++j) {
        const int gc = C0 + tx + j * NTX;
        const bool ok = gr < rmax && gc >= cmin && gc < cmax && (ROWPANEL || gr >= gc);
        cv[i][j] = ok ? G[gr + (int64_t)gc * n] : (T)0;
      }
    }
  };
  if constexpr (EARLY_C) load_c();
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
  if constexpr (!EARLY_C) load_c();
#pragma unroll
  for (int i = 0; i < TM; ++i) {
    const int gr = R0 + ty + i * NTY;
#pragma unroll
    for (int j = 0; j < TN; ++j) {
      const int gc = C0 + tx + j * NTX;
      const bool ok = gr < rmax && gc >= cmin && gc < cmax && (ROWPANEL || gr >= gc);
      if (ok) G[gr + (int64_t)gc * n] = cv[i][j] - acc[i][j];
    }
  }
}

void launch_syrk_update(const DevCtx& c, const Item* items, int n_items, int dtype, int nb,
                        int nbo, cudaStream_t s) {
  if (!n_items) return;
  if (nb > 64) throw std::invalid_argument("trailing update: panel width above 64");
  const int region = nbo > 0 ? 1 : 0;
  if (dtype == F64) k_tile_update<double, 64, 64, 16, 4, 4, false><<<n_items, 256, 0, s>>>(c, items, nb, nbo, region);
  else k_tile_update<float, 64, 64, 16, 4, 4, false><<<n_items, 256, 0, s>>>(c, items, nb, nbo, region);
}

void launch_gemm_update(const DevCtx& c, const Item* items, int n_items, int dtype, int nb, int nbo,
                        int region, cudaStream_t s) {
  if (nb > 64) throw std::invalid_argument("trailing update: panel width above 64");
  if (!n_items) return;
  if (dtype == F64) k_tile_update<double, 64, 64, 16, 4, 4, true><<<n_items, 256, 0, s>>>(c, items, nb, nbo, region);
  else k_tile_update<float, 64, 64, 16, 4, 4, true><<<n_items, 256, 0, s>>>(c, items, nb, nbo, region);
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
  const int jend = it.b > 0 ? min(it.b, n) : n;   // rows are swapped in columns < jend
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
        for (int j = threadIdx.x; j < jend; j += NT) {
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

// ---------------------------------------------------------------------------
// LU panel of a tall front on many CTAs (cooperative launch)
// ---------------------------------------------------------------------------
// The panel (rows k0..n-1, columns k0..k0+kb-1) of each item is split into
// row chunks of R rows, one per CTA, held in shared memory (column-major,
// leading dimension R).  For each column k of the panel, every CTA
//   1. finds its candidate pivot: the largest |a| in column k among its rows
//      in [k0+k, fs) (the reference searches the eliminated rows only), ties
//      to the lowest row, and publishes value, row and the row's kb values
//      in the exchange buffer; the CTA holding row k0+k also publishes that
//      row;
//   2. passes one grid barrier (the exchange buffers alternate by column
//      parity, so a barrier per column is enough);
//   3. picks the item's pivot from all its CTAs' candidates (same rule: the
//      largest value, the lowest row on ties; this is the first maximum of a
//      sequential search), swaps the two rows in its chunk when it holds
//      them, and applies l_r = a_rk / a_kk, a_rj -= l_r u_j to its rows below
//      the pivot row.
// The result is the reference's partial pivoting (FLA_LU_piv inside the
// eliminated block) exactly; only the panel's own columns are swapped here,
// the other columns of the front by k_laswp afterwards.  Item: front,
// a = k0, b = first CTA, c = number of CTAs.  The grid barrier is an arrival
// counter with a bounded spin; a CTA that gives up raises the abort word and
// the error flag, and every CTA then skips the remaining barriers.
constexpr int GC_THREADS = 256;

UHM_DEFINE_WAIT_LIMIT(set_wait_limit_factor, 1u << 22)

__device__ __forceinline__ unsigned int gc_ld_acquire(const unsigned int* p) {
  unsigned int v;
  asm volatile("ld.acquire.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
  return v;
}

// barrier number `round` (1, 2, ...) of a launch of `total` CTAs; false once
// any CTA gave up
__device__ __forceinline__ bool gc_grid_barrier(unsigned int* ctr, unsigned int round, unsigned int total,
                                                int* err, int* s_ok) {
  __syncthreads();
  if (threadIdx.x == 0) {
    bool ok = *s_ok != 0;
    if (ok) {
      __threadfence();
      atomicAdd(ctr, 1u);
      const unsigned int target = round * total;
      ok = false;
      const uint32_t lim = g_wait_limit;
      for (uint32_t i = 0; i < lim; ++i) {
        if (gc_ld_acquire(ctr) >= target) { ok = true; break; }
        if (gc_ld_acquire(ctr + 1)) break;          // another CTA gave up
        __nanosleep(20);
      }
      if (!ok) {
        atomicExch(ctr + 1, 1u);
        atomicExch(err, 3);
      }
      __threadfence();
    }
    *s_ok = ok ? 1 : 0;
  }
  __syncthreads();
  return *s_ok != 0;
}

template <typename T>
__global__ void __launch_bounds__(GC_THREADS) k_getrf_coop(DevCtx c, const Item* __restrict__ items, int n_items,
                                                           int nb, int pivot, int rmax, double* __restrict__ xbuf,
                                                           unsigned int* ctr, int* err) {
  extern __shared__ __align__(16) unsigned char gc_smem[];
  T* S = reinterpret_cast<T*>(gc_smem);        // chunk, column-major, leading dimension R
  __shared__ T s_u[64], s_old[64];
  __shared__ double s_cv[GC_THREADS / 32];
  __shared__ int s_ci[GC_THREADS / 32];
  __shared__ int s_ok, s_item, s_p, s_w;
  const unsigned int total = gridDim.x;
  if (threadIdx.x == 0) {
    s_ok = 1;
    int k = 0;
    while (k + 1 < n_items && (int)blockIdx.x >= items[k + 1].b) ++k;
    s_item = k;
  }
  __syncthreads();
  const Item it = items[s_item];
  const FrontDev f = c.fronts[it.front];
  const int n = f.n, fs = f.fs, k0 = it.a;
  const int kb = min(nb, fs - k0);
  const int P = it.c, q = blockIdx.x - it.b;
  const int rows = n - k0;
  const int R = (rows + P - 1) / P;
  const int rbeg = k0 + q * R, rend = min(rbeg + R, n);   // my rows [rbeg, rend)
  const int nr_my = max(0, rend - rbeg);
  T* __restrict__ G = arena<T>(c) + f.off;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  // exchange buffer: per parity, per CTA {value, row, kb values}, then per item the row k0+k
  constexpr int XS = 66;
  auto cand = [&](int par, int b) { return xbuf + ((size_t)par * total + b) * XS; };
  auto diag_row = [&](int par, int itx) { return xbuf + (size_t)2 * total * XS + ((size_t)par * n_items + itx) * 64; };
  for (int idx = threadIdx.x; idx < nr_my * kb; idx += GC_THREADS) {
    const int r = idx % nr_my, j = idx / nr_my;
    S[j * rmax + r] = G[(rbeg + r) + (int64_t)(k0 + j) * n];
  }
  __syncthreads();
  for (int k = 0; k < kb; ++k) {
    const int gk = k0 + k, par = k & 1;
    // 1. candidate of this chunk
    double bv = -1.0;
    int bi = 0x7fffffff;
    if (pivot) {
      const int lo = max(rbeg, gk), hi = min(rend, fs);
      for (int r = lo + threadIdx.x; r < hi; r += GC_THREADS) {
        const double v = (double)my_abs<T>(S[k * rmax + (r - rbeg)]);
        if (v > bv) { bv = v; bi = r; }
      }
#pragma unroll
      for (int o = 16; o > 0; o >>= 1) {
        const double ov = __shfl_down_sync(0xffffffffu, bv, o);
        const int oi = __shfl_down_sync(0xffffffffu, bi, o);
        if (ov > bv || (ov == bv && oi < bi)) { bv = ov; bi = oi; }
      }
      if (lane == 0) { s_cv[warp] = bv; s_ci[warp] = bi; }
      __syncthreads();
      if (threadIdx.x == 0) {
        for (int w = 1; w < GC_THREADS / 32; ++w)
          if (s_cv[w] > bv || (s_cv[w] == bv && s_ci[w] < bi)) { bv = s_cv[w]; bi = s_ci[w]; }
        s_ci[0] = bi;
        double* cb = cand(par, blockIdx.x);
        cb[0] = bv;
        cb[1] = (double)bi;
      }
      __syncthreads();
      bi = s_ci[0];
      if (bi != 0x7fffffff && threadIdx.x < kb) cand(par, blockIdx.x)[2 + threadIdx.x] = (double)S[threadIdx.x * rmax + (bi - rbeg)];
    }
    if (gk >= rbeg && gk < rend && threadIdx.x < kb)
      diag_row(par, s_item)[threadIdx.x] = (double)S[threadIdx.x * rmax + (gk - rbeg)];
    // 2. one grid barrier per column
    if (!gc_grid_barrier(ctr, (unsigned int)(k + 1), total, err, &s_ok)) return;
    // 3. the item's pivot
    if (warp == 0) {
      double v = -1.0;
      int r = 0x7fffffff, w = -1;
      if (pivot) {
        for (int b = lane; b < P; b += 32) {
          const double* cb = cand(par, it.b + b);
          const double cv = __ldcg(cb);
          const int ci = (int)__ldcg(cb + 1);
          if (cv > v || (cv == v && ci < r)) { v = cv; r = ci; w = it.b + b; }
        }
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) {
          const double ov = __shfl_down_sync(0xffffffffu, v, o);
          const int oi = __shfl_down_sync(0xffffffffu, r, o);
          const int ow = __shfl_down_sync(0xffffffffu, w, o);
          if (ov > v || (ov == v && oi < r)) { v = ov; r = oi; w = ow; }
        }
      }
      if (lane == 0) {
        if (!pivot || r == 0x7fffffff) { r = gk; w = -1; }
        s_p = r;
        s_w = w;
      }
    }
    __syncthreads();
    const int p = s_p;
    if (threadIdx.x < kb) {
      const double* dr = diag_row(par, s_item);
      s_old[threadIdx.x] = (T)__ldcg(dr + threadIdx.x);                        // old row gk
      s_u[threadIdx.x] = p == gk ? s_old[threadIdx.x] : (T)__ldcg(cand(par, s_w) + 2 + threadIdx.x);
    }
    __syncthreads();
    if (threadIdx.x < kb) {
      if (gk >= rbeg && gk < rend) S[threadIdx.x * rmax + (gk - rbeg)] = s_u[threadIdx.x];
      if (p != gk && p >= rbeg && p < rend) S[threadIdx.x * rmax + (p - rbeg)] = s_old[threadIdx.x];
    }
    if (q == 0 && threadIdx.x == 0) c.piv[f.piv_off + gk] = p;
    __syncthreads();
    T akk = s_u[k];
    if (akk == (T)0 || akk != akk) {
      if (q == 0 && threadIdx.x == 0) set_status(c, it.front, akk != akk ? ST_NAN : ST_ZERO_PIVOT);
      akk = (T)1;
    }
    const T rinv = (T)1 / akk;
    // rows below the pivot row: multiplier and rank-1 update of the panel's later columns
    for (int r = max(rbeg, gk + 1) + threadIdx.x; r < rend; r += GC_THREADS) {
      const int rl = r - rbeg;
      const T l = S[k * rmax + rl] * rinv;
      S[k * rmax + rl] = l;
      for (int j = k + 1; j < kb; ++j) S[j * rmax + rl] -= l * s_u[j];
    }
    __syncthreads();
  }
  for (int idx = threadIdx.x; idx < nr_my * kb; idx += GC_THREADS) {
    const int r = idx % nr_my, j = idx / nr_my;
    G[(rbeg + r) + (int64_t)(k0 + j) * n] = S[j * rmax + r];
  }
}

void launch_getrf_coop(const DevCtx& c, const Item* items, int n_items, int n_ctas, int dtype, int nb, int pivot,
                       int rmax, double* xbuf, unsigned int* ctr, int* err, cudaStream_t s) {
  if (!n_items) return;
  if (nb > 64) throw std::invalid_argument("getrf_coop: panel wider than 64");
  cudaMemsetAsync(ctr, 0, 2 * sizeof(unsigned int), s);
  const size_t smem = (size_t)rmax * nb * (dtype == F64 ? sizeof(double) : sizeof(float));
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3(n_ctas);
  cfg.blockDim = dim3(GC_THREADS);
  cfg.dynamicSmemBytes = smem;
  cfg.stream = s;
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributeCooperative;
  attr[0].val.cooperative = 1;
  cfg.attrs = attr;
  cfg.numAttrs = 1;
  cudaError_t e;
  if (dtype == F64) {
    cudaFuncSetAttribute(k_getrf_coop<double>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    e = cudaLaunchKernelEx(&cfg, k_getrf_coop<double>, c, items, n_items, nb, pivot, rmax, xbuf, ctr, err);
  } else {
    cudaFuncSetAttribute(k_getrf_coop<float>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    e = cudaLaunchKernelEx(&cfg, k_getrf_coop<float>, c, items, n_items, nb, pivot, rmax, xbuf, ctr, err);
  }
  if (e != cudaSuccess)
    throw std::runtime_error(std::string("cooperative LU panel launch failed: ") + cudaGetErrorString(e));
}

// Row interchanges of a panel (pivots of rows k0..k0+kb-1, kb = min(nb,
// fs - k0), applied in order) on the front's columns outside the panel and
// below a column limit.  Item: front, a = k0, b = first column of a
// 256-column chunk, c = column limit (0: n); one thread per column.
template <typename T>
__global__ void __launch_bounds__(256) k_laswp(DevCtx c, const Item* __restrict__ items, int nb) {
  const Item it = items[blockIdx.x];
  const FrontDev f = c.fronts[it.front];
  const int n = f.n, k0 = it.a;
  const int kb = min(nb, f.fs - k0);
  const int j = it.b + threadIdx.x;
  const int jend = it.c > 0 ? min(it.c, n) : n;
  if (j >= jend || (j >= k0 && j < k0 + kb)) return;
  T* __restrict__ col = arena<T>(c) + f.off + (int64_t)j * n;
  const int32_t* __restrict__ pv = c.piv + f.piv_off;
  for (int k = k0; k < k0 + kb; ++k) {
    const int p = pv[k];
    if (p != k) {
      const T t = col[k];
      col[k] = col[p];
      col[p] = t;
    }
  }
}

void launch_laswp(const DevCtx& c, const Item* items, int n_items, int dtype, int nb, cudaStream_t s) {
  if (!n_items) return;
  if (dtype == F64) k_laswp<double><<<n_items, 256, 0, s>>>(c, items, nb);
  else k_laswp<float><<<n_items, 256, 0, s>>>(c, items, nb);
}

constexpr int LUROW_CB = 64;   // columns per row-panel block

// A[k0:k0+kb, cols] <- L11^{-1} A[k0:k0+kb, cols]  (unit lower), cols >= k0+kb;
// item: front, a = k0, b = first column of the chunk, c = column limit (0: n)
template <typename T, int NT>
__global__ void __launch_bounds__(NT) k_lu_row_update(DevCtx c, const Item* __restrict__ items,
                                                      int nb) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const Item it = items[blockIdx.x];
  const FrontDev f = c.fronts[it.front];
  const int n = f.n, k0 = it.a, c0 = it.b;
  const int kb = min(nb, f.fs - k0);
  const int cend = it.c > 0 ? min(it.c, n) : n;    // columns < cend (item c; 0: all)
  const int cb = min(LUROW_CB, cend - c0);
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
