// Tree forward/backward solves and the element-wise residual.
//
// Reference steps restated here:
//   forward   solve_chol_1_hier / solve_lu_piv_1_hier + Helper_::merge_rhs_x
//             (UHM/src/matrix/uhm/fla/chol/solve.cxx:152-168,
//              fla/lu_piv/solve.cxx:161-187, helper.hxx:253-301)
//   backward  solve_chol_2_hier / solve_lu_piv_2_hier + Helper_::branch_rhs_x
//             (chol/solve.cxx:187-202, lu_piv/solve.cxx:211-231, helper.hxx:302-331)
// The right-hand side lives in a global vector in elimination order; the
// dofs eliminated at front f are g[g0 .. g0+fs).  A child's updated bottom
// block (xb) is gathered into its parent exactly like the matrix extend-add.
//
// Residual: r = b - sum_e P_e^T A_e P_e x on the retained FP64 element
// matrices (the unassembled operator), followed by a deterministic per-dof
// gather in element order.  This replaces the factor-based check_* of
// UHM/src/matrix/uhm/fla/chol/check.cxx:40-111.
#include "k_common.cuh"

namespace uhm_gpu {

// the empty value of the flag-driven solves' hand-off words (a signalling
// NaN: no arithmetic result or conversion produces it)
constexpr unsigned long long HAND_EMPTY = 0x7FF4DEAD7FF4DEADull;

// z = [g[g0 .. g0+fs); 0] + sum over children of their xb (extend-add);
// item: front, a = first row, b = rows (0: all), c = 1 for a front of the
// 64-row flag-driven solves
__global__ void __launch_bounds__(256) k_fwd_gather(DevCtx c, const Item* __restrict__ items,
                                                    const double* __restrict__ g, int64_t ldg,
                                                    int method) {
  const Item it = items[blockIdx.x];
  const FrontDev f = c.fronts[it.front];
  const int n = f.n;
  double* __restrict__ z = c.vec + f.voff;
  double* __restrict__ y = z + (int64_t)n * c.n_rhs;
  double* __restrict__ w = y + (int64_t)n * c.n_rhs;
  const int32_t* __restrict__ inv = c.inv + f.inv_off;
  // rows [it.a, it.a + it.b) of the front (it.b == 0: all rows; only then
  // are pivots applied, which needs the whole gathered vector)
  const int I0 = it.a, I1 = it.b > 0 ? min(n, it.a + it.b) : n;
  // the sources decoded once per CTA (in source order): a child's updated
  // bottom block and its leading dimension, null for an element source
  constexpr int GMAXSRC = 64;
  __shared__ const double* s_xb[GMAXSRC];
  __shared__ int s_ld[GMAXSRC];
  const int ns = min(f.nsrc, GMAXSRC);
  for (int s = threadIdx.x; s < ns; s += blockDim.x) {
    const SrcDev sd = c.srcs[f.src0 + s];
    if (sd.is_child) {
      const FrontDev ch = c.fronts[sd.slot];
      s_xb[s] = c.vec + ch.voff + ch.fs;
      s_ld[s] = ch.n;
    } else {
      s_xb[s] = nullptr;
      s_ld[s] = 0;
    }
  }
  __syncthreads();
  for (int q = 0; q < c.n_rhs; ++q) {
    for (int I = I0 + threadIdx.x; I < I1; I += blockDim.x) {
      double acc = I < f.fs ? g[(f.g0 + I) + q * ldg] : 0.0;
      for (int s = 0; s < ns; ++s) {
        const double* xb = s_xb[s];
        if (!xb) continue;
        const int is = inv[(int64_t)s * n + I];
        if (is >= 0) acc += xb[is + (int64_t)q * s_ld[s]];
      }
      for (int s = ns; s < f.nsrc; ++s) {
        const SrcDev sd = c.srcs[f.src0 + s];
        if (!sd.is_child) continue;
        const int is = inv[(int64_t)s * n + I];
        if (is >= 0) {
          const FrontDev ch = c.fronts[sd.slot];
          acc += c.vec[ch.voff + ch.fs + is + (int64_t)q * ch.n];
        }
      }
      z[I + (int64_t)q * n] = acc;
      // fronts of the 64-row flag-driven and chain solves: their y factor
      // rows (solutions) and w factor rows (partial sums) are forward
      // hand-offs, emptied here (the forward launch comes after)
      if (it.c && I < f.fs) {
        y[I + (int64_t)q * n] = __longlong_as_double((long long)HAND_EMPTY);
        w[I + (int64_t)q * n] = __longlong_as_double((long long)HAND_EMPTY);
      }
    }
  }
  __syncthreads();
  if (method == M_LU_PIV && it.b == 0 && threadIdx.x < c.n_rhs) {
    // FLA_Apply_pivots(LEFT, NO_TRANSPOSE, p, xt): sequential interchanges
    const int q = threadIdx.x;
    const int32_t* __restrict__ piv = c.piv + f.piv_off;
    double* zq = z + (int64_t)q * n;
    for (int k = 0; k < f.fs; ++k) {
      const int p = piv[k];
      if (p != k) { double t = zq[k]; zq[k] = zq[p]; zq[p] = t; }
    }
  }
}

void launch_fwd_gather(const DevCtx& c, const Item* items, int n_items, const double* g,
                       int64_t ldg, int method, cudaStream_t s) {
  if (!n_items) return;
  k_fwd_gather<<<n_items, 256, 0, s>>>(c, items, g, ldg, method);
}

// whole-front forward sweep: z_t <- L^{-1} z_t ; z_b <- z_b - ABL z_t
template <typename T, int NT>
__global__ void __launch_bounds__(NT) k_fwd_small(DevCtx c, const Item* __restrict__ items,
                                                  int method) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  double* z = reinterpret_cast<double*>(smem_raw);
  const Item it = items[blockIdx.x];
  const FrontDev f = c.fronts[it.front];
  const int n = f.n, fs = f.fs, nr = c.n_rhs;
  const T* __restrict__ G = arena<T>(c) + f.off;
  double* __restrict__ zg = c.vec + f.voff;
  for (int idx = threadIdx.x; idx < n * nr; idx += NT) z[idx] = zg[idx];
  __syncthreads();
  const bool unit = method != M_CHOL;
  for (int j = 0; j < fs; ++j) {
    if (!unit) {
      const double d = (double)G[j + (int64_t)j * n];
      if (threadIdx.x < nr) z[j + threadIdx.x * n] /= d;
      __syncthreads();
    }
    const int h = n - j - 1;
    for (int idx = threadIdx.x; idx < h * nr; idx += NT) {
      const int i = j + 1 + idx % h, q = idx / h;
      z[i + q * n] -= (double)G[i + (int64_t)j * n] * z[j + q * n];
    }
    __syncthreads();
  }
  // y (second slab) receives the eliminated part, z keeps the updated bottom
  double* __restrict__ yg = zg + (int64_t)n * nr;
  for (int idx = threadIdx.x; idx < n * nr; idx += NT) {
    const int i = idx % n;
    if (i < fs) yg[idx] = z[idx];
    else zg[idx] = z[idx];
  }
}

// Cholesky small fronts with the factor panel (n x fs) staged in shared
// memory by one batch of loads: every column step then works on shared data
// (one barrier per column instead of a global round trip per column).  The
// right-hand sides are solved in the factor's precision (as in the
// flag-driven solves of large fronts): FP32 fronts take no FP64 arithmetic,
// which runs at a small fraction of the FP32 rate on this GPU.
template <typename T, int NT>
__global__ void __launch_bounds__(NT) k_fwd_small_staged(DevCtx c, const Item* __restrict__ items) {
  using CT = T;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const Item it = items[blockIdx.x];
  const FrontDev f = c.fronts[it.front];
  const int n = f.n, fs = f.fs, nr = c.n_rhs;
  CT* z = reinterpret_cast<CT*>(smem_raw);
  T* Ls = z + (size_t)n * nr;
  const T* __restrict__ G = arena<T>(c) + f.off;
  double* __restrict__ zg = c.vec + f.voff;
  const int tot = n * fs;
  for (int i0 = 0; i0 < tot; i0 += 8 * NT) {
    T v[8];
#pragma unroll
    for (int u = 0; u < 8; ++u) {
      const int idx = i0 + threadIdx.x + u * NT;
      v[u] = idx < tot ? G[idx] : T(0);        // columns 0..fs-1 are contiguous (ld n)
    }
#pragma unroll
    for (int u = 0; u < 8; ++u) {
      const int idx = i0 + threadIdx.x + u * NT;
      if (idx < tot) Ls[idx] = v[u];
    }
  }
  for (int idx = threadIdx.x; idx < n * nr; idx += NT) z[idx] = (CT)zg[idx];
  __syncthreads();
  for (int j = 0; j < fs; ++j) {
    if (threadIdx.x < nr) z[j + threadIdx.x * n] /= (CT)Ls[j + j * n];
    __syncthreads();
    const int h = n - j - 1;
    for (int q = 0; q < nr; ++q) {
      const CT zj = z[j + q * n];
      for (int i = j + 1 + threadIdx.x; i < n; i += NT) z[i + q * n] -= (CT)Ls[i + j * n] * zj;
    }
    (void)h;
    __syncthreads();
  }
  double* __restrict__ yg = zg + (int64_t)n * nr;
  for (int q = 0; q < nr; ++q)
    for (int i = threadIdx.x; i < n; i += NT) {
      if (i < fs) yg[i + (int64_t)q * n] = (double)z[i + q * n];
      else zg[i + (int64_t)q * n] = (double)z[i + q * n];
    }
}

// x_F = L_FF^{-T} (y_F - L_SF^T x_S): the Schur-row products for all factor
// columns at once, then the small triangular solve column by column.
template <typename T, int NT>
__global__ void __launch_bounds__(NT) k_bwd_small_staged(DevCtx c, const Item* __restrict__ items,
                                                         double* __restrict__ g, int64_t ldg) {
  using CT = T;                       // the factor's precision, as in the forward sweep
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const Item it = items[blockIdx.x];
  const FrontDev f = c.fronts[it.front];
  const int n = f.n, fs = f.fs, nr = c.n_rhs;
  CT* z = reinterpret_cast<CT*>(smem_raw);
  CT* w = z + (size_t)n * nr;
  T* Ls = w + fs;
  const T* __restrict__ G = arena<T>(c) + f.off;
  double* __restrict__ zg = c.vec + f.voff + (int64_t)n * nr;   // y slab
  const int tot = n * fs;
  for (int i0 = 0; i0 < tot; i0 += 8 * NT) {
    T v[8];
#pragma unroll
    for (int u = 0; u < 8; ++u) {
      const int idx = i0 + threadIdx.x + u * NT;
      v[u] = idx < tot ? G[idx] : T(0);
    }
#pragma unroll
    for (int u = 0; u < 8; ++u) {
      const int idx = i0 + threadIdx.x + u * NT;
      if (idx < tot) Ls[idx] = v[u];
    }
  }
  for (int idx = threadIdx.x; idx < n * nr; idx += NT) z[idx] = (CT)zg[idx];
  __syncthreads();
  for (int q = 0; q < nr; ++q) {
    CT* zq = z + q * n;
    for (int j = threadIdx.x; j < fs; j += NT) {
      CT sacc = CT(0);
      const T* col = Ls + (size_t)j * n;
      for (int i = fs; i < n; ++i) sacc += (CT)col[i] * zq[i];
      w[j] = zq[j] - sacc;
    }
    __syncthreads();
    for (int j = fs - 1; j >= 0; --j) {
      const CT xj = w[j] / (CT)Ls[j + j * n];
      for (int i = threadIdx.x; i < j; i += NT) w[i] -= (CT)Ls[j + i * n] * xj;
      if (threadIdx.x == 0) zq[j] = xj;
      __syncthreads();
    }
  }
  for (int q = 0; q < nr; ++q)
    for (int i = threadIdx.x; i < fs; i += NT) g[(f.g0 + i) + q * ldg] = (double)z[i + q * n];
}

void launch_fwd_small(const DevCtx& c, const Item* items, int n_items, int dtype, int method,
                      int staged_bytes, cudaStream_t s) {
  if (!n_items) return;
  if (method == M_CHOL && staged_bytes > 0) {
    if (dtype == F64) {
      cudaFuncSetAttribute(k_fwd_small_staged<double, 128>, cudaFuncAttributeMaxDynamicSharedMemorySize, staged_bytes);
      k_fwd_small_staged<double, 128><<<n_items, 128, staged_bytes, s>>>(c, items);
    } else {
      cudaFuncSetAttribute(k_fwd_small_staged<float, 128>, cudaFuncAttributeMaxDynamicSharedMemorySize, staged_bytes);
      k_fwd_small_staged<float, 128><<<n_items, 128, staged_bytes, s>>>(c, items);
    }
    return;
  }
  // the largest small front bounds the shared slab; 64 KB covers n*n_rhs <= 8192
  size_t sm = 8192 * sizeof(double);
  if (dtype == F64) {
    cudaFuncSetAttribute(k_fwd_small<double, 256>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm);
    k_fwd_small<double, 256><<<n_items, 256, sm, s>>>(c, items, method);
  } else {
    cudaFuncSetAttribute(k_fwd_small<float, 256>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm);
    k_fwd_small<float, 256><<<n_items, 256, sm, s>>>(c, items, method);
  }
}

// backward: xb <- g[schur dofs]
__global__ void __launch_bounds__(256) k_bwd_prepare(DevCtx c, const Item* __restrict__ items,
                                                     const double* __restrict__ g, int64_t ldg) {
  const Item it = items[blockIdx.x];
  const FrontDev f = c.fronts[it.front];
  double* __restrict__ y = c.vec + f.voff + (int64_t)f.n * c.n_rhs;
  const int32_t* __restrict__ sgi = c.sgi + f.sgi_off;
  for (int q = 0; q < c.n_rhs; ++q)
    for (int j = threadIdx.x; j < f.ss; j += blockDim.x)
      y[f.fs + j + (int64_t)q * f.n] = g[sgi[j] + q * ldg];
}

void launch_bwd_prepare(const DevCtx& c, const Item* items, int n_items, int dtype, int method,
                        const double* g, int64_t ldg, cudaStream_t s) {
  (void)dtype; (void)method;
  if (!n_items) return;
  k_bwd_prepare<<<n_items, 256, 0, s>>>(c, items, g, ldg);
}

template <int NT>
__device__ double block_sum(double v, double* s_red) {
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
  if (lane == 0) s_red[warp] = v;
  __syncthreads();
  double r = 0.0;
  if (threadIdx.x == 0) {
    for (int w = 0; w < NT / 32; ++w) r += s_red[w];
    s_red[NT / 32] = r;
  }
  __syncthreads();
  r = s_red[NT / 32];
  __syncthreads();
  return r;
}

// whole-front backward sweep and store of x_t into g
template <typename T, int NT>
__global__ void __launch_bounds__(NT) k_bwd_small(DevCtx c, const Item* __restrict__ items,
                                                  int method, double* __restrict__ g, int64_t ldg) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  __shared__ double s_red[NT / 32 + 1];
  double* z = reinterpret_cast<double*>(smem_raw);
  const Item it = items[blockIdx.x];
  const FrontDev f = c.fronts[it.front];
  const int n = f.n, fs = f.fs, nr = c.n_rhs;
  const T* __restrict__ G = arena<T>(c) + f.off;
  double* __restrict__ zg = c.vec + f.voff + (int64_t)n * nr;   // y slab
  for (int idx = threadIdx.x; idx < n * nr; idx += NT) z[idx] = zg[idx];
  __syncthreads();
  const bool chol = method == M_CHOL;
  for (int q = 0; q < nr; ++q) {
    double* zq = z + q * n;
    for (int j = fs - 1; j >= 0; --j) {
      double part = 0.0;
      if (chol)
        for (int i = j + 1 + threadIdx.x; i < n; i += NT) part += (double)G[i + (int64_t)j * n] * zq[i];
      else
        for (int t = j + 1 + threadIdx.x; t < n; t += NT) part += (double)G[j + (int64_t)t * n] * zq[t];
      const double s = block_sum<NT>(part, s_red);
      if (threadIdx.x == 0) zq[j] = (zq[j] - s) / (double)G[j + (int64_t)j * n];
      __syncthreads();
    }
  }
  for (int q = 0; q < nr; ++q)
    for (int i = threadIdx.x; i < fs; i += NT) g[(f.g0 + i) + q * ldg] = z[i + q * n];
}

void launch_bwd_small(const DevCtx& c, const Item* items, int n_items, int dtype, int method,
                      double* g, int64_t ldg, int staged_bytes, cudaStream_t s) {
  if (!n_items) return;
  if (method == M_CHOL && staged_bytes > 0) {
    if (dtype == F64) {
      cudaFuncSetAttribute(k_bwd_small_staged<double, 128>, cudaFuncAttributeMaxDynamicSharedMemorySize, staged_bytes);
      k_bwd_small_staged<double, 128><<<n_items, 128, staged_bytes, s>>>(c, items, g, ldg);
    } else {
      cudaFuncSetAttribute(k_bwd_small_staged<float, 128>, cudaFuncAttributeMaxDynamicSharedMemorySize, staged_bytes);
      k_bwd_small_staged<float, 128><<<n_items, 128, staged_bytes, s>>>(c, items, g, ldg);
    }
    return;
  }
  size_t sm = 8192 * sizeof(double);
  if (dtype == F64) {
    cudaFuncSetAttribute(k_bwd_small<double, 256>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm);
    k_bwd_small<double, 256><<<n_items, 256, sm, s>>>(c, items, method, g, ldg);
  } else {
    cudaFuncSetAttribute(k_bwd_small<float, 256>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm);
    k_bwd_small<float, 256><<<n_items, 256, sm, s>>>(c, items, method, g, ldg);
  }
}

// ---------------------------------------------------------------------------
// Large fronts, blocked by SB = 64 columns.
// Forward step k (item: front, a = k0, b = row chunk): every CTA solves the
// diagonal block x_k = L_kk^{-1} z_k (warp-synchronous substitution, unit
// diagonal for LU), chunk 0 stores x_k in the y slab, and each CTA updates
// its chunk of rows below:  z[r] -= L[r, k-block] x_k.  Step k reads only
// z_k and writes only rows >= k0+kb and y_k, so CTAs never race.
// Backward step k (item: front, a = k0, b = chunk, c = number of chunks):
// each CTA forms partial dot products of its tail chunk (Chol: L^T, LU: U)
// with y; the last CTA to arrive (threadfence reduction) sums the partials in
// chunk order -- deterministic -- and solves the diagonal block into y_k.
// ---------------------------------------------------------------------------
constexpr int SB = 64;          // diagonal block of the blocked solves
constexpr int FWD_RB = 256;     // rows per forward-update CTA
constexpr int BWD_RB = 512;     // tail rows per backward partial CTA
constexpr int NR_MAX = 16;      // right-hand sides of large fronts

// lower-triangular substitution of one diagonal block by one warp;
// x (shared, length kb) in, solution out
template <typename T, typename CT>
__device__ __forceinline__ void warp_lower_solve(const T* D, int kb, CT* x, bool unit) {
  const int lane = threadIdx.x & 31;
  CT v0 = lane < kb ? x[lane] : CT(0), v1 = lane + 32 < kb ? x[lane + 32] : CT(0);
  for (int j = 0; j < kb; ++j) {
    CT xj = __shfl_sync(0xffffffffu, j < 32 ? v0 : v1, j & 31);
    if (!unit) xj /= (CT)D[j + j * SB];
    if (lane == (j & 31)) { if (j < 32) v0 = xj; else v1 = xj; }
    if (lane > j && lane < kb) v0 -= (CT)D[lane + j * SB] * xj;
    if (lane + 32 > j && lane + 32 < kb) v1 -= (CT)D[lane + 32 + j * SB] * xj;
  }
  if (lane < kb) x[lane] = v0;
  if (lane + 32 < kb) x[lane + 32] = v1;
}

// upper substitution: Chol uses L_kk^T (A(i,j) = D[j,i]), LU uses U_kk
template <typename T, typename CT>
__device__ __forceinline__ void warp_upper_solve(const T* D, int kb, CT* x, bool chol) {
  const int lane = threadIdx.x & 31;
  CT v0 = lane < kb ? x[lane] : CT(0), v1 = lane + 32 < kb ? x[lane + 32] : CT(0);
  for (int j = kb - 1; j >= 0; --j) {
    CT xj = __shfl_sync(0xffffffffu, j < 32 ? v0 : v1, j & 31);
    xj /= (CT)D[j + j * SB];
    if (lane == (j & 31)) { if (j < 32) v0 = xj; else v1 = xj; }
    if (lane < j) v0 -= (CT)(chol ? D[j + lane * SB] : D[lane + j * SB]) * xj;
    if (lane + 32 < j) v1 -= (CT)(chol ? D[j + (lane + 32) * SB] : D[lane + 32 + j * SB]) * xj;
  }
  if (lane < kb) x[lane] = v0;
  if (lane + 32 < kb) x[lane + 32] = v1;
}

template <typename T, int NT>
__global__ void __launch_bounds__(NT) k_fwd_step(DevCtx c, const Item* __restrict__ items, int method) {
  using CT = T;   // compute in the storage precision of the factor
  __shared__ T D[SB * SB];
  __shared__ CT xk[SB * NR_MAX];
  const Item it = items[blockIdx.x];
  const FrontDev f = c.fronts[it.front];
  const int n = f.n, k0 = it.a, nr = c.n_rhs;
  const int kb = min(SB, f.fs - k0);
  const T* __restrict__ G = arena<T>(c) + f.off;
  double* __restrict__ z = c.vec + f.voff;
  double* __restrict__ y = z + (int64_t)n * nr;
  for (int idx = threadIdx.x; idx < SB * kb; idx += NT) {
    const int i = idx % SB, j = idx / SB;
    D[idx] = i < kb ? G[(k0 + i) + (int64_t)(k0 + j) * n] : T(0);
  }
  for (int idx = threadIdx.x; idx < kb * nr; idx += NT) {
    const int i = idx % kb, q = idx / kb;
    xk[i + q * SB] = (CT)z[(k0 + i) + (int64_t)q * n];
  }
  __syncthreads();
  const int warp = threadIdx.x >> 5;
  for (int q = warp; q < nr; q += NT / 32) warp_lower_solve<T, CT>(D, kb, xk + q * SB, method != M_CHOL);
  __syncthreads();
  if (it.b == 0)
    for (int idx = threadIdx.x; idx < kb * nr; idx += NT) {
      const int i = idx % kb, q = idx / kb;
      y[(k0 + i) + (int64_t)q * n] = (double)xk[i + q * SB];
    }
  const int r0 = k0 + kb + it.b * FWD_RB;
  const int r1 = min(r0 + FWD_RB, n);
  for (int r = r0 + threadIdx.x; r < r1; r += NT) {
    for (int q = 0; q < nr; ++q) {
      CT acc = CT(0);
      for (int t = 0; t < kb; ++t) acc += (CT)G[r + (int64_t)(k0 + t) * n] * xk[t + q * SB];
      z[r + (int64_t)q * n] -= (double)acc;
    }
  }
}

template <typename T, int NT>
__global__ void __launch_bounds__(NT) k_bwd_step(DevCtx c, const Item* __restrict__ items, int method,
                                                 double* __restrict__ scratch,
                                                 const int64_t* __restrict__ scr_off,
                                                 int* __restrict__ counters) {
  using CT = T;
  // the diagonal block (last CTA) and the partial-sum tile (all CTAs) share storage
  __shared__ __align__(16) unsigned char s_raw[sizeof(CT) * SB * (SB + 1)];
  T* D = reinterpret_cast<T*>(s_raw);
  CT (*tileT)[SB + 1] = reinterpret_cast<CT (*)[SB + 1]>(s_raw);
  __shared__ CT part[4][SB];
  __shared__ CT xk[SB * NR_MAX];
  __shared__ CT ys[SB];
  __shared__ int s_last;
  const Item it = items[blockIdx.x];
  const FrontDev f = c.fronts[it.front];
  const int n = f.n, k0 = it.a, nr = c.n_rhs;
  const int kb = min(SB, f.fs - k0);
  const T* __restrict__ G = arena<T>(c) + f.off;
  double* __restrict__ y = c.vec + f.voff + (int64_t)n * nr;
  const int t0 = k0 + kb;
  const int nch = it.c;
  const bool chol = method == M_CHOL;
  double* __restrict__ sc = scratch + scr_off[it.front];
  if (nch > 0) {
    const int c0 = t0 + it.b * BWD_RB, c1 = min(c0 + BWD_RB, n);
    const int i = threadIdx.x % SB, g = threadIdx.x / SB;   // NT = 256: 4 groups
    for (int q = 0; q < nr; ++q) {
      CT acc = CT(0);
      if (chol) {
        // rows of the chunk in tiles of 64: load L[rows, k-block] coalesced
        // along rows, then thread (i, g) sums 16 rows of column i
        for (int t0r = c0; t0r < c1; t0r += SB) {
          __syncthreads();
          for (int idx = threadIdx.x; idx < SB * SB; idx += NT) {
            const int rr = idx % SB, cc = idx / SB;
            tileT[rr][cc] = (t0r + rr < c1 && cc < kb) ? (CT)G[(t0r + rr) + (int64_t)(k0 + cc) * n] : CT(0);
          }
          for (int rr = threadIdx.x; rr < SB; rr += NT)
            ys[rr] = t0r + rr < c1 ? (CT)y[t0r + rr + (int64_t)q * n] : CT(0);
          __syncthreads();
#pragma unroll 4
          for (int rr = g * 16; rr < g * 16 + 16; ++rr) acc += tileT[rr][i] * ys[rr];
        }
      } else if (i < kb) {
        {
          for (int cc = c0 + g; cc < c1; cc += 4)
            acc += (CT)G[(k0 + i) + (int64_t)cc * n] * (CT)y[cc + (int64_t)q * n];
        }
      }
      part[g][i] = acc;
      __syncthreads();
      if (threadIdx.x < SB)
        sc[((int64_t)it.b * nr + q) * SB + threadIdx.x] =
            (double)(part[0][threadIdx.x] + part[1][threadIdx.x] + part[2][threadIdx.x] + part[3][threadIdx.x]);
      __syncthreads();
    }
    __threadfence();
    if (threadIdx.x == 0) s_last = (atomicAdd(&counters[it.front], 1) == nch - 1);
    __syncthreads();
    if (!s_last) return;
    __threadfence();
    if (threadIdx.x == 0) counters[it.front] = 0;
  }
  // last CTA (or the only one): sum partials in chunk order, solve the block
  for (int idx = threadIdx.x; idx < SB * kb; idx += NT) {
    const int ii = idx % SB, j = idx / SB;
    D[idx] = ii < kb ? G[(k0 + ii) + (int64_t)(k0 + j) * n] : T(0);
  }
  for (int idx = threadIdx.x; idx < kb * nr; idx += NT) {
    const int ii = idx % kb, q = idx / kb;
    double s = 0.0;
    for (int ch = 0; ch < nch; ++ch) s += sc[((int64_t)ch * nr + q) * SB + ii];
    xk[ii + q * SB] = (CT)(y[(k0 + ii) + (int64_t)q * n] - s);
  }
  __syncthreads();
  const int warp = threadIdx.x >> 5;
  for (int q = warp; q < nr; q += NT / 32) warp_upper_solve<T, CT>(D, kb, xk + q * SB, chol);
  __syncthreads();
  for (int idx = threadIdx.x; idx < kb * nr; idx += NT) {
    const int ii = idx % kb, q = idx / kb;
    y[(k0 + ii) + (int64_t)q * n] = (double)xk[ii + q * SB];
  }
}

void launch_fwd_step(const DevCtx& c, const Item* items, int n_items, int dtype, int method,
                     cudaStream_t s) {
  if (!n_items) return;
  if (dtype == F64) k_fwd_step<double, 256><<<n_items, 256, 0, s>>>(c, items, method);
  else k_fwd_step<float, 256><<<n_items, 256, 0, s>>>(c, items, method);
}

void launch_bwd_step(const DevCtx& c, const Item* items, int n_items, int dtype, int method,
                     double* scratch, const int64_t* scr_off, int* counters, cudaStream_t s) {
  if (!n_items) return;
  if (dtype == F64)
    k_bwd_step<double, 256><<<n_items, 256, 0, s>>>(c, items, method, scratch, scr_off, counters);
  else
    k_bwd_step<float, 256><<<n_items, 256, 0, s>>>(c, items, method, scratch, scr_off, counters);
}

__global__ void __launch_bounds__(256) k_bwd_store(DevCtx c, const Item* __restrict__ items,
                                                   double* __restrict__ g, int64_t ldg) {
  const Item it = items[blockIdx.x];
  const FrontDev f = c.fronts[it.front];
  const double* __restrict__ z = c.vec + f.voff + (int64_t)f.n * c.n_rhs;   // y slab
  for (int q = 0; q < c.n_rhs; ++q)
    for (int i = threadIdx.x; i < f.fs; i += blockDim.x) g[(f.g0 + i) + q * ldg] = z[i + (int64_t)q * f.n];
}

void launch_bwd_store(const DevCtx& c, const Item* items, int n_items, double* g, int64_t ldg,
                      cudaStream_t s) {
  if (!n_items) return;
  k_bwd_store<<<n_items, 256, 0, s>>>(c, items, g, ldg);
}

// ---------------------------------------------------------------------------
// element-wise residual
// ---------------------------------------------------------------------------
// y_e = A_e x_e  for every element (one CTA per element)
__global__ void __launch_bounds__(256) k_elem_gemv(const double* __restrict__ emat,
                                                   const int64_t* __restrict__ emat_off,
                                                   const int* __restrict__ elem_m,
                                                   const int64_t* __restrict__ emap_off,
                                                   const int32_t* __restrict__ emap,
                                                   const double* __restrict__ x, int64_t ldx,
                                                   double* __restrict__ y,
                                                   const int64_t* __restrict__ y_off, int n_rhs) {
  __shared__ double s_x[1024];
  const int e = blockIdx.x;
  const int m = elem_m[e];
  const double* __restrict__ A = emat + emat_off[e];
  const int32_t* __restrict__ map = emap + emap_off[e];
  double* __restrict__ ye = y + y_off[e];
  for (int q = 0; q < n_rhs; ++q) {
    for (int j0 = 0; j0 < m; j0 += 1024) {
      const int jn = min(1024, m - j0);
      __syncthreads();
      for (int j = threadIdx.x; j < jn; j += blockDim.x) s_x[j] = x[map[j0 + j] + q * ldx];
      __syncthreads();
      for (int i = threadIdx.x; i < m; i += blockDim.x) {
        double acc = j0 ? ye[i + (int64_t)q * m] : 0.0;
        for (int j = 0; j < jn; ++j) acc += A[i + (int64_t)(j0 + j) * m] * s_x[j];
        ye[i + (int64_t)q * m] = acc;
      }
    }
  }
}

void launch_elem_gemv(const double* emat, const int64_t* emat_off, const int* elem_m,
                      const int64_t* emap_off, const int32_t* emap, const double* x, int64_t ldx,
                      double* y, const int64_t* y_off, int n_elem, int n_rhs, cudaStream_t s) {
  if (!n_elem) return;
  k_elem_gemv<<<n_elem, 128, 0, s>>>(emat, emat_off, elem_m, emap_off, emap, x, ldx, y, y_off,
                                     n_rhs);
}

// r[i] = (sub_from_b ? b[i] - sum : sum), sum over the (element, row) list of dof i in order.
// idx entries index the flattened per-element y buffer (offset of row 0 of rhs 0 + row).
__global__ void k_dof_gather(const int64_t* __restrict__ ptr, const int64_t* __restrict__ idx,
                             const double* __restrict__ y, const double* __restrict__ b,
                             int64_t ldb, double* __restrict__ r, int64_t N, int n_rhs,
                             int sub_from_b, const int* __restrict__ dummy) {
  (void)dummy;
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < N;
       i += (int64_t)gridDim.x * blockDim.x) {
    for (int q = 0; q < n_rhs; ++q) {
      double s = 0.0;
      for (int64_t k = ptr[i]; k < ptr[i + 1]; ++k) {
        // idx encodes (element y offset + row) and the element's row count in the high bits
        const int64_t v = idx[k];
        const int64_t off = v & ((1LL << 40) - 1);
        const int64_t m = v >> 40;
        s += y[off + q * m];
      }
      r[i + q * ldb] = sub_from_b ? b[i + q * ldb] - s : s;
    }
  }
}

void launch_dof_gather(const int64_t* ptr, const int64_t* idx, const double* y, const double* b,
                       int64_t ldb, double* r, int64_t N, int n_rhs, int sub_from_b,
                       cudaStream_t s) {
  if (!N) return;
  int blocks = (int)std::min<int64_t>((N + 255) / 256, 152 * 16);
  k_dof_gather<<<blocks, 256, 0, s>>>(ptr, idx, y, b, ldb, r, N, n_rhs, sub_from_b, nullptr);
}

// out[0] = max |v| (single-pass, deterministic: per-block max then a final block)
// max(a, b) of non-negative values that keeps a NaN (fmax drops it), so that
// a NaN anywhere in the vector reaches the result
__device__ __forceinline__ double nanmax(double a, double b) { return (b > a || b != b) ? b : a; }

__global__ void k_absmax_partial(const double* __restrict__ v, int64_t n, double* __restrict__ part) {
  __shared__ double s[256];
  double m = 0.0;
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x)
    m = nanmax(m, fabs(v[i]));
  s[threadIdx.x] = m;
  __syncthreads();
  for (int o = 128; o > 0; o >>= 1) {
    if (threadIdx.x < o) s[threadIdx.x] = nanmax(s[threadIdx.x], s[threadIdx.x + o]);
    __syncthreads();
  }
  if (threadIdx.x == 0) part[blockIdx.x] = s[0];
}

__global__ void k_absmax_final(const double* __restrict__ part, int np, double* __restrict__ out) {
  __shared__ double s[256];
  double m = 0.0;
  for (int i = threadIdx.x; i < np; i += blockDim.x) m = nanmax(m, part[i]);
  s[threadIdx.x] = m;
  __syncthreads();
  for (int o = 128; o > 0; o >>= 1) {
    if (threadIdx.x < o) s[threadIdx.x] = nanmax(s[threadIdx.x], s[threadIdx.x + o]);
    __syncthreads();
  }
  if (threadIdx.x == 0) out[0] = s[0];
}

// out must hold 1 + 304 doubles (result, then partials)
void launch_absmax(const double* v, int64_t n, double* out, cudaStream_t s) {
  const int np = 304;
  k_absmax_partial<<<np, 256, 0, s>>>(v, n, out + 1);
  k_absmax_final<<<1, 256, 0, s>>>(out + 1, np, out);
}

// Maximum |v| per tree of a forest.  v holds n_rhs columns of ng dofs;
// tree[i] is the tree of dof i.  The dofs of one tree are not contiguous
// (numbering runs generation by generation over all trees) but come in long
// runs (a front's factor dofs are consecutive), so each thread scans 32
// consecutive entries and flushes its running maximum with one atomicMax on
// the bit pattern (non-negative doubles order like their bits; NaN, kept by
// the comparison below, orders above every number) whenever the tree changes.
// out[t] must be zeroed before the launch.
__global__ void k_absmax_tree(const double* __restrict__ v, int64_t nv, int64_t ng,
                              const int* __restrict__ tree, unsigned long long* __restrict__ out) {
  const int64_t i0 = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) * 32;
  if (i0 >= nv) return;
  const int64_t i1 = i0 + 32 < nv ? i0 + 32 : nv;
  int64_t row = i0 % ng;
  int cur = -1;
  double m = 0.0;
  for (int64_t i = i0; i < i1; ++i) {
    const int t = tree[row];
    if (t != cur) {
      if (cur >= 0) atomicMax(&out[cur], (unsigned long long)__double_as_longlong(m));
      cur = t;
      m = 0.0;
    }
    const double a = fabs(v[i]);
    if (a > m || a != a) m = a;
    if (++row == ng) row = 0;
  }
  atomicMax(&out[cur], (unsigned long long)__double_as_longlong(m));
}

void launch_absmax_tree(const double* v, int64_t nv, int64_t ng, const int* tree, int n_trees,
                        unsigned long long* out, cudaStream_t s) {
  cudaMemsetAsync(out, 0, sizeof(unsigned long long) * n_trees, s);
  if (!nv) return;
  const int64_t threads = (nv + 31) / 32;
  k_absmax_tree<<<(unsigned)((threads + 255) / 256), 256, 0, s>>>(v, nv, ng, tree, out);
}

__global__ void k_axpy(double* __restrict__ y, const double* __restrict__ x, int64_t n, double a) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x)
    y[i] += a * x[i];
}

void launch_axpy(double* y, const double* x, int64_t n, double alpha, cudaStream_t s) {
  if (!n) return;
  int blocks = (int)std::min<int64_t>((n + 255) / 256, 152 * 8);
  k_axpy<<<blocks, 256, 0, s>>>(y, x, n, alpha);
}

}  // namespace uhm_gpu

namespace uhm_gpu {

// ||A||_inf of the assembled operator A = sum_e P_e^T A_e P_e, exactly, on the
// device.  Entry (i, J) of A is summed over the elements that contain both
// dofs; the element of smallest index among them (the "owner") computes that
// sum and adds |A(i, J)| to its partial row sum for row i.  Partial sums are
// then gathered per dof in element order (k_dof_gather), so the result is
// deterministic.  dof_el lists, per dof, (element, local row) sorted by element.
__global__ void __launch_bounds__(128) k_anorm_partial(const double* __restrict__ emat,
                                                       const int64_t* __restrict__ emat_off,
                                                       const int* __restrict__ elem_m,
                                                       const int64_t* __restrict__ emap_off,
                                                       const int32_t* __restrict__ emap,
                                                       const int64_t* __restrict__ dof_ptr,
                                                       const int2* __restrict__ dof_el,
                                                       double* __restrict__ part,
                                                       const int64_t* __restrict__ y_off) {
  const int e = blockIdx.x;
  const int m = elem_m[e];
  const int32_t* __restrict__ map = emap + emap_off[e];
  for (int l = threadIdx.x; l < m; l += blockDim.x) {
    const int32_t i = map[l];
    const int64_t a0 = dof_ptr[i], a1 = dof_ptr[i + 1];
    double s = 0.0;
    for (int j = 0; j < m; ++j) {
      const int32_t J = map[j];
      const int64_t b0 = dof_ptr[J], b1 = dof_ptr[J + 1];
      // merge-intersect the two element lists
      int64_t a = a0, b = b0;
      int owner = -1;
      double v = 0.0;
      while (a < a1 && b < b1) {
        const int2 pa = dof_el[a], pb = dof_el[b];
        if (pa.x < pb.x) ++a;
        else if (pb.x < pa.x) ++b;
        else {
          if (owner < 0) owner = pa.x;
          const int me = elem_m[pa.x];
          v += emat[emat_off[pa.x] + pa.y + (int64_t)pb.y * me];
          ++a;
          ++b;
        }
      }
      if (owner == e) s += fabs(v);
    }
    part[y_off[e] + l] = s;
  }
}

void launch_anorm_partial(const double* emat, const int64_t* emat_off, const int* elem_m,
                          const int64_t* emap_off, const int32_t* emap, const int64_t* dof_ptr,
                          const int2* dof_el, double* part, const int64_t* y_off, int n_elem,
                          cudaStream_t s) {
  if (!n_elem) return;
  k_anorm_partial<<<n_elem, 128, 0, s>>>(emat, emat_off, elem_m, emap_off, emap, dof_ptr, dof_el,
                                         part, y_off);
}

}  // namespace uhm_gpu

namespace uhm_gpu {

// ===========================================================================
// Flag-driven level solves of large Cholesky fronts.
//
// One launch covers every large front of a level.  The rows of a front are cut
// into 64-row blocks: factor blocks [64b, min(64b+64, fs)) and ABL blocks
// starting at fs.  A CTA takes a ticket (atomic counter) and processes the
// item of that rank; items are ordered so that each CTA only waits for blocks
// owned by CTAs with smaller tickets, which are already running -- progress
// is guaranteed whatever the residency.  The 64-row kernels publish a
// finished block's solution as self-validating hand-off words (below); the
// 256-row kernels publish it, then a release-store of the block's flag, and
// readers acquire the flag before reading.  Every wait is bounded (error
// flag, no hang).
// Forward:  x_b = L_bb^{-1} (z_b - sum_{j<b} L_bj x_j)
// Backward: x_b = L_bb^{-T} (y_b - sum_{r > block b} L_rb^T x_r)
// with L_bb^{-1} precomputed at factorisation (64 x 64, dinv arenas).
// ===========================================================================
constexpr int FB = 64;
constexpr int SF_NR = FLAG_NR;    // right-hand sides handled by one launch

UHM_DEFINE_WAIT_LIMIT(set_wait_limit_solve, 1u << 22)

template <typename T> __device__ __forceinline__ const T* dinv_arena(const DevCtx& c);
template <> __device__ __forceinline__ const double* dinv_arena<double>(const DevCtx& c) { return c.dinv64; }
template <> __device__ __forceinline__ const float* dinv_arena<float>(const DevCtx& c) { return c.dinv32; }

// Hand-off words of the 64-row flag-driven solves.  A block's solution is
// published as plain FP64 words that carry their own completion: before the
// launch every word of the hand-off holds HAND_EMPTY, a signalling NaN that
// no arithmetic result or conversion can produce, and the solving CTA
// overwrites it with the value (one relaxed 8-byte store per entry, single-
// copy atomic).  A reader polls the words themselves: once none of them is
// HAND_EMPTY it holds the values, with no flag, no fence on the writer's side
// and no second round trip on the reader's.  The forward hand-off is the y
// slab's factor rows (filled by the gather before the launch), the backward
// one the z slab's factor rows (filled by the forward CTA of the block, after
// its last read of them).
__device__ __forceinline__ unsigned long long ld_hand(const double* p) {
  unsigned long long v;
  asm volatile("ld.relaxed.gpu.global.b64 %0, [%1];" : "=l"(v) : "l"(p) : "memory");
  return v;
}
__device__ __forceinline__ void st_hand(double* p, double v) {
  asm volatile("st.relaxed.gpu.global.b64 [%0], %1;" ::"l"(p), "l"(__double_as_longlong(v)) : "memory");
}

// Where the first hand-off wait of a solve gave up (0: none): kind * 10^8 +
// awaited block * 10^4 + the waiting block (kind 1 forward rows, 2 backward
// columns, 3 forward chain, 4 backward chain), read and cleared by the host
// with the error word.
__device__ int g_solve_where = 0;
__device__ __forceinline__ int wait_code(int kind, int awaited, int own) {
  return kind * 100000000 + min(awaited, 9999) * 10000 + min(own, 9999);
}
int solve_wait_where() {
  int v = 0;
  const int zero = 0;
  if (cudaMemcpyFromSymbol(&v, g_solve_where, sizeof(int)) != cudaSuccess) return -1;
  if (v) cudaMemcpyToSymbol(g_solve_where, &zero, sizeof(int));
  return v;
}

// Warp 0 of a CTA: the 64 hand-off words of one block and right-hand side
// (entries lane and lane + 32; entries at or past kb read as 0).
struct HandWords {
  unsigned long long w0, w1;
  __device__ __forceinline__ void load(const double* base, int kb) {
    const int lane = threadIdx.x & 31;
    w0 = lane < kb ? ld_hand(base + lane) : 0ull;
    w1 = lane + 32 < kb ? ld_hand(base + lane + 32) : 0ull;
  }
  __device__ __forceinline__ bool full() const {
    return __all_sync(0xffffffffu, w0 != HAND_EMPTY && w1 != HAND_EMPTY);
  }
  // bounded wait until every word is written; false (and *err = 2, where
  // recorded) when the limit runs out
  __device__ __forceinline__ bool wait(const double* base, int kb, int* err, int where) {
    const uint32_t lim = g_wait_limit;
    for (uint32_t i = 0; !full(); ++i) {
      if (i >= lim) {
        if ((threadIdx.x & 31) == 0) {
          atomicExch(err, 2);
          atomicCAS(&g_solve_where, 0, where);
        }
        return false;
      }
      __nanosleep(32);
      load(base, kb);
    }
    return true;
  }
  template <typename CT>
  __device__ __forceinline__ void stage(CT* dst) const {
    const int lane = threadIdx.x & 31;
    dst[lane] = (CT)__longlong_as_double(w0);
    dst[lane + 32] = (CT)__longlong_as_double(w1);
  }
};

// acc[q] += sum over the column blocks j < jend of L[row, block j] y_j for
// the CTA's rows (thread: row lane tid % 64, column group tid / 64), y_j read
// from its hand-off words: warp 0 polls and stages them (the next block's
// words already in flight), the other warps wait at the block barrier.
template <typename T, int NQ>
__device__ __forceinline__ void fwd_gather_blocks(const DevCtx& c, const FrontDev& f, int row, bool rv, int jend,
                                                  int q0, int nq, int* err, T (&acc)[NQ], T (*ysh)[NQ][FB]) {
  using CT = T;
  const int n = f.n, fs = f.fs, g = threadIdx.x / FB;
  const T* __restrict__ G = arena<T>(c) + f.off;
  const double* __restrict__ y = c.vec + f.voff + (int64_t)n * c.n_rhs;
  // The factor tile of block column j does not depend on y: it is loaded one
  // block ahead, so that only the loads of y_j follow the wait.
  CT tile[16];
  auto load_tile = [&](int j) {
    const int kbj = min(FB, fs - j * FB);
#pragma unroll
    for (int u = 0; u < 16; ++u) {
      const int cc = g * 16 + u;
      tile[u] = (rv && cc < kbj) ? (CT)G[row + (int64_t)(j * FB + cc) * n] : CT(0);
    }
  };
  const bool w0 = threadIdx.x < 32;
  HandWords hw;
  bool live = true;      // warp 0: false once a wait has run out (no more waiting)
  if (jend > 0) {
    load_tile(0);
    if (w0) hw.load(y + (int64_t)q0 * n, min(FB, fs));
  }
  for (int j = 0; j < jend; ++j) {
    const int buf = j & 1;
    if (w0) {
      // y_j is read by every later block of the front at once: one warp
      // per CTA polls and stages it (the next block's words already in flight)
      const int kbj = min(FB, fs - j * FB);
      const double* yj = y + j * FB;
      if (live) live = hw.wait(yj + (int64_t)q0 * n, kbj, err, wait_code(1, j, row / FB));
      hw.stage(ysh[buf][0]);
      for (int q = 1; q < nq; ++q) {
        HandWords hq;
        hq.load(yj + (int64_t)(q0 + q) * n, kbj);
        if (live) live = hq.wait(yj + (int64_t)(q0 + q) * n, kbj, err, wait_code(1, j, row / FB));
        hq.stage(ysh[buf][q]);
      }
      if (j + 1 < jend) hw.load(y + (j + 1) * FB + (int64_t)q0 * n, min(FB, fs - (j + 1) * FB));
    }
    CT cur[16];
#pragma unroll
    for (int u = 0; u < 16; ++u) cur[u] = tile[u];
    if (j + 1 < jend) load_tile(j + 1);
    __syncthreads();
#pragma unroll
    for (int u = 0; u < 16; ++u) {
#pragma unroll
      for (int q = 0; q < NQ; ++q)
        if (q < nq) acc[q] += cur[u] * ysh[buf][q][g * 16 + u];
    }
  }
}

// item: front, a = block index (factor blocks 0..nfb-1, ABL blocks nfb..);
// right-hand sides q0 .. q0+nq-1, nq <= NQ <= SF_NR (more are solved by
// further launches); NQ is the launch's right-hand sides rounded up to 1, 2
// or 4, so that a launch for one right-hand side issues no products for
// absent ones
template <typename T, int NQ>
__global__ void __launch_bounds__(256, sizeof(T) == 4 ? 3 : 2) k_fwd_flags(DevCtx c, const Item* __restrict__ items,
                                                   int* ticket, int* err, int q0) {
  using CT = T;
  __shared__ int s_t;
  __shared__ CT red[4][FB][NQ];
  __shared__ CT v[FB][NQ];
  __shared__ T dsh[FB * (FB + 1)];     // inverse diagonal block, staged before any wait
  // y_j staged by warp 0, two buffers alternating by block: one barrier per block
  __shared__ CT ysh[2][NQ][FB];
  if (threadIdx.x == 0) s_t = atomicAdd(ticket, 1);
  __syncthreads();
  const Item it = items[s_t];
  const FrontDev f = c.fronts[it.front];
  const int n = f.n, fs = f.fs, nr = c.n_rhs, b = it.a;
  const int nq = min(NQ, nr - q0);
  const int nfb = (fs + FB - 1) / FB;
  const bool factor_block = b < nfb;
  if (factor_block) {
    const T* __restrict__ Dg = dinv_arena<T>(c) + f.dinv_off + (int64_t)b * FB * FB;
    for (int idx = threadIdx.x; idx < FB * FB; idx += 256) dsh[(idx / FB) * (FB + 1) + idx % FB] = Dg[idx];
  }
  const int r0 = factor_block ? b * FB : fs + (b - nfb) * FB;
  const int r1 = factor_block ? min(r0 + FB, fs) : min(r0 + FB, n);
  double* __restrict__ z = c.vec + f.voff;
  double* __restrict__ y = z + (int64_t)n * nr;
  const int i = threadIdx.x % FB, g = threadIdx.x / FB;
  const int row = r0 + i;
  const bool rv = row < r1;
  CT acc[NQ], zr[NQ];
#pragma unroll
  for (int q = 0; q < NQ; ++q) {
    acc[q] = CT(0);
    zr[q] = (rv && q < nq && g == 0) ? (CT)z[row + (int64_t)(q0 + q) * n] : CT(0);   // before any wait
  }
  // the factor rows of z are not read again: they become the backward
  // solve's hand-off words for this block
  if (factor_block && rv && g == 0) {
#pragma unroll
    for (int q = 0; q < NQ; ++q)
      if (q < nq) z[row + (int64_t)(q0 + q) * n] = __longlong_as_double((long long)HAND_EMPTY);
  }
  fwd_gather_blocks<T, NQ>(c, f, row, rv, factor_block ? b : nfb, q0, nq, err, acc, ysh);
#pragma unroll
  for (int q = 0; q < NQ; ++q) red[g][i][q] = acc[q];
  __syncthreads();
  if (threadIdx.x < FB) {
#pragma unroll
    for (int q = 0; q < NQ; ++q)
      v[i][q] = (rv && q < nq) ? zr[q] - (red[0][i][q] + red[1][i][q] + red[2][i][q] + red[3][i][q]) : CT(0);
  }
  __syncthreads();
  if (factor_block) {
    // y = Dinv v on all 256 threads: column group g sums t in [16 g, 16 g + 16),
    // then the four partial sums are added in group order; this takes the
    // 64-step dependent chain of one thread per row off the hand-off to the
    // next block.  The stored inverse is zero above its diagonal and past the
    // block's kb rows and columns, so every thread runs the same unbranched
    // loop (its loads issued together) and the sums equal the skipped-term
    // ones exactly.
    CT xp[NQ];
#pragma unroll
    for (int q = 0; q < NQ; ++q) xp[q] = CT(0);
#pragma unroll
    for (int u = 0; u < 16; ++u) {
      const int t = g * 16 + u;
      const CT d = (CT)dsh[t * (FB + 1) + i];     // Dinv[i][t], column t staged as row t
#pragma unroll
      for (int q = 0; q < NQ; ++q) xp[q] += d * v[t][q];
    }
#pragma unroll
    for (int q = 0; q < NQ; ++q) red[g][i][q] = xp[q];
    __syncthreads();
    if (threadIdx.x < FB && rv) {
#pragma unroll
      for (int q = 0; q < NQ; ++q)
        if (q < nq)
          st_hand(y + row + (int64_t)(q0 + q) * n,
                  (double)(red[0][i][q] + red[1][i][q] + red[2][i][q] + red[3][i][q]));
    }
  } else if (threadIdx.x < FB && rv) {
#pragma unroll
    for (int q = 0; q < NQ; ++q)
      if (q < nq) z[row + (int64_t)(q0 + q) * n] = (double)v[i][q];
  }
}

// Forward solve of large Cholesky fronts with 256-row CTAs.  Item: front,
// a = B: B < nfb4 (= ceil(nfb / 4)) the factor rows 256 B .. (64-row blocks
// 4 B .. 4 B + 3, solved here in turn), otherwise the ABL rows
// fs + 256 (B - nfb4) ...  One thread per row; the row's 64 factor entries of
// the next column block are loaded into registers before that block's
// solution is waited for.  Column blocks left of the CTA come from other
// CTAs as hand-off words (warp 0 polls and stages them, the next block's
// words already in flight); the CTA's own blocks are solved in turn on all
// its threads (v = z - sum on the block's rows, y = Dinv v by four column
// groups, summed in group order), each published at once as hand-off words,
// and every later row of the CTA adds its product with y.  One hand-off
// between CTAs per 256 rows instead of per 64.  Tickets in item order: every
// CTA waits only on smaller tickets.
constexpr int F4_ROWS = 256;

template <typename T>
__global__ void __launch_bounds__(256, 1) k_fwd_hand4(DevCtx c, const Item* __restrict__ items, int* ticket, int* err,
                                                      int q0) {
  using CT = T;
  extern __shared__ __align__(16) unsigned char f4_dyn[];
  T* dsh = reinterpret_cast<T*>(f4_dyn);          // own inverse diagonal blocks, dsh[s][t * 65 + i] = Dinv_s[i][t]
  __shared__ int s_t;
  __shared__ CT ysh[2][SF_NR][FB];
  __shared__ CT vsh[SF_NR][FB];
  __shared__ CT red[4][FB][SF_NR];
  const int tid = threadIdx.x;
  if (tid == 0) s_t = atomicAdd(ticket, 1);
  __syncthreads();
  const Item it = items[s_t];
  const FrontDev f = c.fronts[it.front];
  const int n = f.n, fs = f.fs, nr = c.n_rhs;
  const int nq = min(SF_NR, nr - q0);
  const int nfb = (fs + FB - 1) / FB, nfb4 = (nfb + 3) / 4;
  const bool factor_cta = it.a < nfb4;
  const int b0 = factor_cta ? 4 * it.a : nfb;                 // first own 64-row block (factor CTAs)
  const int ns = factor_cta ? min(4, nfb - b0) : 0;           // own blocks
  const int r0 = factor_cta ? F4_ROWS * it.a : fs + F4_ROWS * (it.a - nfb4);
  const int r1 = factor_cta ? min(r0 + F4_ROWS, fs) : min(r0 + F4_ROWS, n);
  const int row = r0 + tid;
  const bool rv = row < r1;
  const int sub = tid >> 6;                                   // own block of this row (factor CTAs)
  const T* __restrict__ G = arena<T>(c) + f.off;
  double* __restrict__ z = c.vec + f.voff;
  double* __restrict__ y = z + (int64_t)n * nr;
  if (factor_cta) {
    const T* __restrict__ Dg = dinv_arena<T>(c) + f.dinv_off + (int64_t)b0 * FB * FB;
    for (int idx = tid; idx < ns * FB * FB; idx += 256) {
      const int s2 = idx / (FB * FB), e = idx % (FB * FB);
      dsh[s2 * FB * (FB + 1) + (e / FB) * (FB + 1) + e % FB] = Dg[idx];
    }
  }
  CT acc[SF_NR], zr[SF_NR];
#pragma unroll
  for (int q = 0; q < SF_NR; ++q) {
    acc[q] = CT(0);
    zr[q] = (rv && q < nq) ? (CT)z[row + (int64_t)(q0 + q) * n] : CT(0);
  }
  // the factor rows of z are not read again: they become the backward
  // solve's hand-off words
  if (factor_cta && rv) {
#pragma unroll
    for (int q = 0; q < SF_NR; ++q)
      if (q < nq) z[row + (int64_t)(q0 + q) * n] = __longlong_as_double((long long)HAND_EMPTY);
  }
  const int jext = b0;                    // column blocks solved by other CTAs
  // the row's entries of column block j, where this row needs them
  CT tile[FB];
  auto load_tile = [&](int j) {
    const bool need = rv && (j < jext || sub > j - b0);
    const int kbj = min(FB, fs - j * FB);
#pragma unroll
    for (int u = 0; u < FB; ++u) tile[u] = (need && u < kbj) ? (CT)G[row + (int64_t)(j * FB + u) * n] : CT(0);
  };
  const int jlast = factor_cta ? b0 + ns - 1 : nfb;          // tiles needed: blocks 0 .. jlast - 1
  if (jlast > 0) load_tile(0);
  const bool w0 = tid < 32;
  HandWords hw;
  bool live = true;      // warp 0: false once a wait has run out (no more waiting)
  if (jext > 0 && w0) hw.load(y + (int64_t)q0 * n, min(FB, fs));
  for (int j = 0; j < jext; ++j) {
    const int buf = j & 1;
    if (w0) {
      const int kbj = min(FB, fs - j * FB);
      const double* yj = y + j * FB;
      if (live) live = hw.wait(yj + (int64_t)q0 * n, kbj, err, wait_code(1, j, b0));
      hw.stage(ysh[buf][0]);
      for (int q = 1; q < nq; ++q) {
        HandWords hq;
        hq.load(yj + (int64_t)(q0 + q) * n, kbj);
        if (live) live = hq.wait(yj + (int64_t)(q0 + q) * n, kbj, err, wait_code(1, j, b0));
        hq.stage(ysh[buf][q]);
      }
      if (j + 1 < jext) hw.load(y + (j + 1) * FB + (int64_t)q0 * n, min(FB, fs - (j + 1) * FB));
    }
    __syncthreads();
    if constexpr (sizeof(T) == 4) {
      // FP32: the next block's loads are issued before this block's products
      CT cur[FB];
#pragma unroll
      for (int u = 0; u < FB; ++u) cur[u] = tile[u];
      if (j + 1 < jlast) load_tile(j + 1);
      if (rv) {
#pragma unroll
        for (int u = 0; u < FB; ++u)
#pragma unroll
          for (int q = 0; q < SF_NR; ++q) acc[q] += cur[u] * ysh[buf][q][u];
      }
    } else {
      // FP64 (register budget): products first, then the next block's loads
      if (rv) {
#pragma unroll
        for (int u = 0; u < FB; ++u)
#pragma unroll
          for (int q = 0; q < SF_NR; ++q) acc[q] += tile[u] * ysh[buf][q][u];
      }
      if (j + 1 < jlast) load_tile(j + 1);
    }
  }
  // own blocks s: v = z - acc on its rows, y = Dinv_s v, published; the rows
  // below add their products with y
  for (int s = 0; s < ns; ++s) {
    const int j = b0 + s, kbj = min(FB, fs - j * FB);
    if (sub == s) {
#pragma unroll
      for (int q = 0; q < SF_NR; ++q) vsh[q][tid & 63] = rv ? zr[q] - acc[q] : CT(0);
    }
    // FP32: the next block's tile is loaded before this block's solve (the
    // rows below need it right after); FP64 (register budget) loads it after
    // the products
    CT cur[sizeof(T) == 4 ? FB : 1];
    if constexpr (sizeof(T) == 4) {
#pragma unroll
      for (int u = 0; u < FB; ++u) cur[u] = tile[u];
      if (j + 1 < jlast) load_tile(j + 1);
    }
    __syncthreads();
    {
      // y = Dinv v: column group g sums t in [16 g, 16 g + 16) (Dinv is
      // lower triangular: t <= i)
      const int i = tid & 63, g = tid >> 6;
      const T* Ds = dsh + s * FB * (FB + 1);
      CT xp[SF_NR];
#pragma unroll
      for (int q = 0; q < SF_NR; ++q) xp[q] = CT(0);
#pragma unroll
      for (int u = 0; u < 16; ++u) {
        const int t = g * 16 + u;
        if (t <= i && t < kbj) {
          const CT d = (CT)Ds[t * (FB + 1) + i];
#pragma unroll
          for (int q = 0; q < SF_NR; ++q) xp[q] += d * vsh[q][t];
        }
      }
#pragma unroll
      for (int q = 0; q < SF_NR; ++q) red[g][i][q] = xp[q];
    }
    __syncthreads();
    if (tid < FB) {
      const int i = tid, r = r0 + FB * s + i;
#pragma unroll
      for (int q = 0; q < SF_NR; ++q) {
        const CT yv = red[0][i][q] + red[1][i][q] + red[2][i][q] + red[3][i][q];
        ysh[0][q][i] = i < kbj ? yv : CT(0);
        if (i < kbj && q < nq) st_hand(y + r + (int64_t)(q0 + q) * n, (double)yv);
      }
    }
    __syncthreads();
    if constexpr (sizeof(T) == 4) {
      if (rv && sub > s) {
#pragma unroll
        for (int u = 0; u < FB; ++u)
#pragma unroll
          for (int q = 0; q < SF_NR; ++q) acc[q] += cur[u] * ysh[0][q][u];
      }
    } else {
      (void)cur;
      if (rv && sub > s) {
#pragma unroll
        for (int u = 0; u < FB; ++u)
#pragma unroll
          for (int q = 0; q < SF_NR; ++q) acc[q] += tile[u] * ysh[0][q][u];
      }
      if (j + 1 < jlast) load_tile(j + 1);
    }
  }
  if (!factor_cta && rv) {
#pragma unroll
    for (int q = 0; q < SF_NR; ++q)
      if (q < nq) z[row + (int64_t)(q0 + q) * n] = (double)(zr[q] - acc[q]);
  }
}

void launch_fwd_flags4(const DevCtx& c, const Item* items, int n_items, int dtype, int* ticket, int* err, int q0,
                       cudaStream_t s) {
  if (!n_items) return;
  cudaMemsetAsync(ticket, 0, sizeof(int), s);
  if (dtype == F64) {
    const int sm = (int)(sizeof(double) * 4 * FB * (FB + 1));
    cudaFuncSetAttribute(k_fwd_hand4<double>, cudaFuncAttributeMaxDynamicSharedMemorySize, sm);
    k_fwd_hand4<double><<<n_items, 256, sm, s>>>(c, items, ticket, err, q0);
  } else {
    const int sm = (int)(sizeof(float) * 4 * FB * (FB + 1));
    cudaFuncSetAttribute(k_fwd_hand4<float>, cudaFuncAttributeMaxDynamicSharedMemorySize, sm);
    k_fwd_hand4<float><<<n_items, 256, sm, s>>>(c, items, ticket, err, q0);
  }
}

// acc[q][u] += sum over the rows r below the factor block (the ABL rows, x
// known from the parent, then the factor blocks j = nfb - 1 down to stop + 1
// as their hand-off words arrive) of L[r, 64 b + 16 g + u] x_r, for column
// block b (thread: row lane tid % 64, column group tid / 64).  Warp 0 polls
// and stages x_j (the next block's words already in flight).
template <typename T, int NQ>
__device__ __forceinline__ void bwd_gather_rows(const DevCtx& c, const FrontDev& f, int b, int stop, int q0, int nq,
                                                int* err, T (&acc)[NQ][16], T (*xsh)[NQ][FB]) {
  using CT = T;
  const int n = f.n, fs = f.fs, nr = c.n_rhs;
  const int nfb = (fs + FB - 1) / FB;
  const int c0 = b * FB, kb = min(FB, fs - c0);
  const T* __restrict__ G = arena<T>(c) + f.off;
  const double* __restrict__ hx = c.vec + f.voff;                  // hand-off: the z slab's factor rows
  const double* __restrict__ y = hx + (int64_t)n * nr;
  const int rl = threadIdx.x % FB, g = threadIdx.x / FB;
  // rows below block b: the ABL part (known) first, two row blocks per
  // round with all loads issued before the arithmetic, then factor blocks
  // from the last one down (they complete in that order)
  for (int rs = fs; rs < n; rs += 2 * FB) {
    CT xr[2][NQ], gv[2][16];
#pragma unroll
    for (int h = 0; h < 2; ++h) {
      const int r = rs + h * FB + rl;
#pragma unroll
      for (int q = 0; q < NQ; ++q) xr[h][q] = (r < n && q < nq) ? (CT)y[r + (int64_t)(q0 + q) * n] : CT(0);
#pragma unroll
      for (int u = 0; u < 16; ++u) {
        const int cc = g * 16 + u;
        gv[h][u] = (r < n && cc < kb) ? (CT)G[r + (int64_t)(c0 + cc) * n] : CT(0);
      }
    }
#pragma unroll
    for (int h = 0; h < 2; ++h)
#pragma unroll
      for (int u = 0; u < 16; ++u)
#pragma unroll
        for (int q = 0; q < NQ; ++q) acc[q][u] += gv[h][u] * xr[h][q];
  }
  // the factor tile of row block j does not depend on x: loaded one block
  // ahead, so that only the loads of x_j follow the wait
  CT tile[16];
  auto load_tile = [&](int j) {
    const int r = j * FB + rl;
    const bool in = r < min(j * FB + FB, fs);
#pragma unroll
    for (int u = 0; u < 16; ++u) {
      const int cc = g * 16 + u;
      tile[u] = (in && cc < kb) ? (CT)G[r + (int64_t)(c0 + cc) * n] : CT(0);
    }
  };
  const bool w0 = threadIdx.x < 32;
  HandWords hw;
  bool live = true;      // warp 0: false once a wait has run out (no more waiting)
  if (nfb - 1 > stop) {
    load_tile(nfb - 1);
    if (w0) hw.load(hx + (nfb - 1) * FB + (int64_t)q0 * n, min(FB, fs - (nfb - 1) * FB));
  }
  for (int j = nfb - 1, k = 0; j > stop; --j, ++k) {
    const int buf = k & 1;
    if (w0) {
      const int kbj = min(FB, fs - j * FB);
      const double* xj = hx + j * FB;
      if (live) live = hw.wait(xj + (int64_t)q0 * n, kbj, err, wait_code(2, j, b));
      hw.stage(xsh[buf][0]);
      for (int q = 1; q < nq; ++q) {
        HandWords hq;
        hq.load(xj + (int64_t)(q0 + q) * n, kbj);
        if (live) live = hq.wait(xj + (int64_t)(q0 + q) * n, kbj, err, wait_code(2, j, b));
        hq.stage(xsh[buf][q]);
      }
      if (j - 1 > stop) hw.load(hx + (j - 1) * FB + (int64_t)q0 * n, min(FB, fs - (j - 1) * FB));
    }
    CT cur[16];
#pragma unroll
    for (int u = 0; u < 16; ++u) cur[u] = tile[u];
    if (j - 1 > stop) load_tile(j - 1);
    __syncthreads();
    const int r = j * FB + rl;
    if (r < min(j * FB + FB, fs)) {
#pragma unroll
      for (int u = 0; u < 16; ++u)
#pragma unroll
        for (int q = 0; q < NQ; ++q) acc[q][u] += cur[u] * xsh[buf][q][rl];
    }
  }
}

// item: front, a = factor block index, tickets in descending block order;
// right-hand sides q0 .. q0+NQ-1, accumulated in the same pass over the
// factor tiles (a pass per right-hand side would put NQ-1 un-overlapped
// re-reads of the whole block column on the chain of hand-offs)
template <typename T, int NQ>
__global__ void __launch_bounds__(256) k_bwd_flags(DevCtx c, const Item* __restrict__ items,
                                                   int* ticket, int* err, int q0) {
  using CT = T;
  __shared__ int s_t;
  extern __shared__ __align__(16) unsigned char bwd_dyn[];
  CT (*red)[FB + 1] = reinterpret_cast<CT (*)[FB + 1]>(bwd_dyn);   // [row lane][column]
  __shared__ CT v[FB][NQ];
  __shared__ T dsh[FB * (FB + 1)];
  // x_j staged by warp 0, two buffers alternating by block: one barrier per block
  __shared__ CT xsh[2][NQ][FB];
  if (threadIdx.x == 0) s_t = atomicAdd(ticket, 1);
  __syncthreads();
  const Item it = items[s_t];
  const FrontDev f = c.fronts[it.front];
  const int n = f.n, fs = f.fs, nr = c.n_rhs, b = it.a;
  const int nq = min(NQ, nr - q0);
  const int c0 = b * FB, kb = min(FB, fs - c0);
  {
    const T* __restrict__ Dg = dinv_arena<T>(c) + f.dinv_off + (int64_t)b * FB * FB;
    for (int idx = threadIdx.x; idx < FB * FB; idx += 256) dsh[(idx / FB) * (FB + 1) + idx % FB] = Dg[idx];
  }
  double* __restrict__ hx = c.vec + f.voff;                  // hand-off: the z slab's factor rows
  double* __restrict__ y = hx + (int64_t)n * nr;
  const int rl = threadIdx.x % FB, g = threadIdx.x / FB;   // row lane, column group
  CT acc[NQ][16];
#pragma unroll
  for (int q = 0; q < NQ; ++q)
#pragma unroll
    for (int u = 0; u < 16; ++u) acc[q][u] = CT(0);
  // this block's right-hand sides, loaded before any wait
  CT yb[NQ];
#pragma unroll
  for (int q = 0; q < NQ; ++q)
    yb[q] = (threadIdx.x < kb && q < nq) ? (CT)y[c0 + threadIdx.x + (int64_t)(q0 + q) * n] : CT(0);
  bwd_gather_rows<T, NQ>(c, f, b, b, q0, nq, err, acc, xsh);
  // the column sums over the 64 row lanes: four parts of 16 rows on all
  // 256 threads (the loads issued together), then the parts in order
  __shared__ CT part[4][FB];
#pragma unroll
  for (int q = 0; q < NQ; ++q) {
    __syncthreads();
#pragma unroll
    for (int u = 0; u < 16; ++u) red[rl][g * 16 + u] = acc[q][u];
    __syncthreads();
    {
      const int col = threadIdx.x % FB, pr = threadIdx.x / FB;
      CT sp = CT(0);
#pragma unroll
      for (int r = 0; r < 16; ++r) sp += red[16 * pr + r][col];
      part[pr][col] = sp;
    }
    __syncthreads();
    if (threadIdx.x < FB) {
      const CT sum = part[0][threadIdx.x] + part[1][threadIdx.x] + part[2][threadIdx.x] + part[3][threadIdx.x];
      v[threadIdx.x][q] = (threadIdx.x < kb && q < nq) ? yb[q] - sum : CT(0);
    }
  }
  __syncthreads();
  // x = Dinv^T v : x_i = sum_{t >= i} Dinv[t, i] v_t   (column i of Dinv, staged at start),
  // on all 256 threads: group gg sums t in [16 gg, 16 gg + 16), partial sums
  // added in group order
  {
    const int ii = threadIdx.x % FB, gg = threadIdx.x / FB;
#pragma unroll
    for (int q = 0; q < NQ; ++q) {
      CT xp = CT(0);
      // Dinv[t][ii] is zero for t < ii and past kb: the unbranched sum is exact
#pragma unroll
      for (int u = 0; u < 16; ++u) {
        const int t = gg * 16 + u;
        xp += (CT)dsh[ii * (FB + 1) + t] * v[t][q];
      }
      red[gg * NQ + q][ii] = xp;
    }
  }
  __syncthreads();
  if (threadIdx.x < kb) {
    const int ii = threadIdx.x;
#pragma unroll
    for (int q = 0; q < NQ; ++q) {
      if (q >= nq) break;
      const double x = (double)(red[q][ii] + red[NQ + q][ii] + red[2 * NQ + q][ii] + red[3 * NQ + q][ii]);
      y[c0 + ii + (int64_t)(q0 + q) * n] = x;
      st_hand(hx + c0 + ii + (int64_t)(q0 + q) * n, x);
    }
  }
}

void launch_fwd_flags(const DevCtx& c, const Item* items, int n_items, int dtype, int* ticket,
                      int* flag_base, int n_flags, int* err, int q0, cudaStream_t s) {
  if (!n_items) return;
  (void)flag_base; (void)n_flags;     // hand-off words, no flags
  cudaMemsetAsync(ticket, 0, sizeof(int), s);
  const int nq = c.n_rhs - q0 < FLAG_NR ? c.n_rhs - q0 : FLAG_NR;
  // NQ covers every right-hand side of the group (3 of them take the 4-wide kernel)
  if (dtype == F64) {
    if (nq >= 3) k_fwd_flags<double, 4><<<n_items, 256, 0, s>>>(c, items, ticket, err, q0);
    else if (nq == 2) k_fwd_flags<double, 2><<<n_items, 256, 0, s>>>(c, items, ticket, err, q0);
    else k_fwd_flags<double, 1><<<n_items, 256, 0, s>>>(c, items, ticket, err, q0);
  } else {
    if (nq >= 3) k_fwd_flags<float, 4><<<n_items, 256, 0, s>>>(c, items, ticket, err, q0);
    else if (nq == 2) k_fwd_flags<float, 2><<<n_items, 256, 0, s>>>(c, items, ticket, err, q0);
    else k_fwd_flags<float, 1><<<n_items, 256, 0, s>>>(c, items, ticket, err, q0);
  }
}

template <typename T, int NQ>
static void bwd_flags_nq(const DevCtx& c, const Item* items, int n_items, int* ticket, int* err, int q0,
                         cudaStream_t s) {
  const size_t dyn = sizeof(T) * FB * (FB + 1);
  cudaFuncSetAttribute(k_bwd_flags<T, NQ>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)dyn);
  k_bwd_flags<T, NQ><<<n_items, 256, dyn, s>>>(c, items, ticket, err, q0);
}

template <typename T>
static void bwd_flags_t(const DevCtx& c, const Item* items, int n_items, int* ticket, int* err, int q0,
                        int nq, cudaStream_t s) {
  if (nq >= 3) bwd_flags_nq<T, 4>(c, items, n_items, ticket, err, q0, s);
  else if (nq == 2) bwd_flags_nq<T, 2>(c, items, n_items, ticket, err, q0, s);
  else bwd_flags_nq<T, 1>(c, items, n_items, ticket, err, q0, s);
}

void launch_bwd_flags(const DevCtx& c, const Item* items, int n_items, int dtype, int* ticket,
                      int* flag_base, int n_flags, int* err, int q0, cudaStream_t s) {
  if (!n_items) return;
  (void)flag_base; (void)n_flags;     // hand-off words, no flags
  cudaMemsetAsync(ticket, 0, sizeof(int), s);
  // right-hand sides of this launch: FLAG_NR, or FLAG_NR_BWD_F64 in FP64
  // (register budget of the NQ x 16 accumulators)
  const int grp = dtype == F64 ? FLAG_NR_BWD_F64 : FLAG_NR;
  const int nq = c.n_rhs - q0 < grp ? c.n_rhs - q0 : grp;
  if (dtype == F64) bwd_flags_t<double>(c, items, n_items, ticket, err, q0, nq, s);
  else bwd_flags_t<float>(c, items, n_items, ticket, err, q0, nq, s);
}

// ===========================================================================
// Chain solves of large FP32 Cholesky fronts.
//
// In the flag-driven solves every 64-row block waits for its neighbour's
// solution to cross from one SM to another (a store, the reader's poll, its
// load): that latency is paid once per block along the whole diagonal.  Here
// one CTA per front (the chain) solves all diagonal blocks in turn from its
// own shared memory, and other CTAs (helpers) feed it:
//
//   forward   x_b = Dinv_b (z_b - P_b - sum_{j = b-K}^{b-1} L_bj x_j)
//             P_b = sum_{j < b-K} L_bj x_j            (helper of row block b)
//   backward  x_b = Dinv_b^T (y_b - P_b - sum_{r = b+1}^{b+K} L_rb^T x_r)
//             P_b = sum_{r > b+K} L_rb^T x_r + (ABL rows) (helper of column block b)
//
// The chain applies the K = CH_K blocks next to the diagonal itself, so a
// helper's partial sum for block b needs solutions at least K + 1 blocks
// back: it has K chain steps to arrive.  Solutions and partial sums travel
// as hand-off words (HAND_EMPTY until written): x in y's factor rows
// (forward) and z's (backward), P in the third slab w.  The chain stages its
// window of blocks and the diagonal inverse with cp.async, CH_STAGES - 1
// steps ahead (asking L2 for them CH_L2_AHEAD steps ahead), and loads each
// step's right-hand side and partial sum a step ahead; the helpers stream their blocks through shared memory CH_HS - 1
// ahead.  Rows of ABL (forward) are finished by their own CTAs once every
// x_j is out.
//
// Items: front, a = block, b = role.  Tickets: the chains first, then the
// helpers in the order their sums are needed, then the ABL rows.  A chain
// waits on helpers with larger tickets, but a helper needs only chain steps
// that in turn need only helpers with smaller tickets: as long as the
// chains and one more CTA fit on the GPU together (at most CH_MAX_CHAINS
// chains per launch, one CTA per SM), the lowest unfinished helper can
// always run and finish, and every wait ends.
// ===========================================================================
constexpr int CH_STAGES = 3;
constexpr int CH_LD = 68;           // floats per staged block column: 64 + room for the 16-byte alignment shift
constexpr int CH_TILE = 64 * CH_LD;
constexpr int CH_HS = 8;            // shared-memory stages of a helper's blocks
constexpr int CH_HW = 4;            // blocks of hand-off words warp 0 of a helper keeps in flight
constexpr int CH_L2_AHEAD = 12;     // steps ahead whose blocks the chain asks L2 for

struct ChainSmem {
  float L[CH_STAGES][CH_K + 1][CH_TILE];   // per stage: the window's blocks, the diagonal inverse (slot CH_K)
  float xs[CH_K][SF_NR][FB];               // the window's solutions (block j at j % CH_K)
  float ts[SF_NR][FB];
};
struct ChainRowSmem {
  float L[CH_HS][CH_TILE];
  float vsh[2][SF_NR][FB];          // the staged solution values of the current block
  float red[4][FB][SF_NR];
  float redb[FB][FB + 1];
};
constexpr size_t CH_SMEM = sizeof(ChainSmem) > sizeof(ChainRowSmem) ? sizeof(ChainSmem) : sizeof(ChainRowSmem);

__device__ __forceinline__ void ch_cp16(float* dst, const float* src) {
  const uint32_t s = (uint32_t)__cvta_generic_to_shared(dst);
  asm volatile("cp.async.cg.shared.global [%0], [%1], 16;" ::"r"(s), "l"(src) : "memory");
}
__device__ __forceinline__ void ch_commit() { asm volatile("cp.async.commit_group;" ::: "memory"); }
template <int N>
__device__ __forceinline__ void ch_wait() { asm volatile("cp.async.wait_group %0;" ::"n"(N) : "memory"); }
__device__ __forceinline__ void ch_l2(const float* p) { asm volatile("prefetch.global.L2 [%0];" ::"l"(p)); }

// The 64 x 64 block of the panel G (ld n) at rows r0.., columns c0.. (c0 a
// multiple of 64), its first ncols columns staged as columns of CH_LD
// floats: column cc starts at the 16-byte boundary at or before entry
// (r0, c0 + cc), so entry (i, cc) is at dst[cc * CH_LD + ch_sh(r0, cc, n) + i].
// Two columns per warp and pass, 17 chunks of 16 bytes each.  Callers stage
// only columns left of column n - 1 with r0 < n, n > 66: the up to 3 extra
// entries either side lie in the neighbouring columns of the same panel.
__device__ __forceinline__ void ch_stage_block(float* dst, const float* G, int64_t r0, int64_t c0, int64_t n,
                                               int ncols = 64) {
  const int lane = threadIdx.x & 31, p = lane & 15;
  for (int k = threadIdx.x >> 5; 2 * k < ncols; k += blockDim.x >> 5) {
    const int cc = 2 * k + (lane >> 4);
    if (cc < ncols) {
      const int64_t s0 = r0 + (c0 + cc) * n;
      const float* src = G + (s0 & ~(int64_t)3);
      float* d = dst + cc * CH_LD;
      ch_cp16(d + 4 * p, src + 4 * p);
      if (p == 0) ch_cp16(d + 64, src + 64);
    }
  }
}
// the alignment shift of staged column cc (c0 a multiple of 4)
__device__ __forceinline__ int ch_sh(int64_t r0, int cc, int64_t n) {
  return (int)(((r0 & 3) + (int64_t)(cc & 3) * (n & 3)) & 3);
}
// the lower triangle of the 64 x 64 diagonal inverse (column-major, 16-byte
// aligned): entry (i, t), i >= t, at dst[t * CH_LD + i]; the 16-byte chunks
// wholly above the diagonal are not copied
__device__ __forceinline__ void ch_stage_dinv(float* dst, const float* D) {
  for (int e = threadIdx.x; e < 64 * 16; e += blockDim.x) {
    const int t = e >> 4, p = e & 15;
    if (4 * p + 3 >= t) ch_cp16(dst + t * CH_LD + 4 * p, D + 4 * e);
  }
}
__device__ __forceinline__ void ch_l2_dinv(const float* D) {
  for (int e = threadIdx.x; e < 128; e += blockDim.x) ch_l2(D + 32 * e);
}
__device__ __forceinline__ void ch_l2_block(const float* G, int64_t r0, int64_t c0, int64_t n) {
  for (int e = threadIdx.x; e < 64 * 3; e += blockDim.x) {
    const int cc = e / 3, p = e - 3 * cc;
    ch_l2(G + r0 + (c0 + cc) * n + (p == 2 ? 63 : 32 * p));
  }
}
__device__ __forceinline__ float ch_sum4(float v) {
  v += __shfl_xor_sync(0xffffffffu, v, 1);
  return v + __shfl_xor_sync(0xffffffffu, v, 2);
}

// Bounded wait of a warp until the lanes' hand-off words (w[q], q < cnt,
// where need) are written; reloads the missing ones.  Returns false (and
// sets *err) when the limit runs out.
template <int NQ>
__device__ __forceinline__ bool ch_wait_words(unsigned long long (&w)[NQ], const double* const (&p)[NQ], int cnt,
                                              bool need, int* err, int where) {
  const uint32_t lim = g_wait_limit;
  for (uint32_t it = 0;; ++it) {
    bool ok = true;
#pragma unroll
    for (int q = 0; q < NQ; ++q)
      if (need && q < cnt && w[q] == HAND_EMPTY) ok = false;
    if (__all_sync(0xffffffffu, ok)) return true;
    if (it >= lim) {
      if ((threadIdx.x & 31) == 0) {
        atomicExch(err, 2);
        atomicCAS(&g_solve_where, 0, where);
      }
      return false;
    }
    __nanosleep(32);
#pragma unroll
    for (int q = 0; q < NQ; ++q)
      if (need && q < cnt && w[q] == HAND_EMPTY) w[q] = ld_hand(p[q]);
  }
}

// forward chain of one front (thread: row i = tid / 4, column phase g = tid % 4);
// right-hand sides q0 .. q0 + nq - 1, nq <= NQ
template <int NQ>
__device__ void fwd_chain(const DevCtx& c, const FrontDev& f, int q0, int nq, int* err, ChainSmem& S) {
  const int tid = threadIdx.x, i = tid >> 2, g = tid & 3;
  const int64_t n = f.n;
  const int fs = f.fs, nr = c.n_rhs, nfb = (fs + FB - 1) / FB;
  const float* __restrict__ G = c.a32 + f.off;
  const float* __restrict__ Dg = c.dinv32 + f.dinv_off;
  double* __restrict__ z = c.vec + f.voff;
  double* __restrict__ y = z + n * nr;
  double* __restrict__ w = y + n * nr;
  // every column this thread reads in a staged block (cc = 4 u + g) has the same shift
  const int sh = ch_sh(0, g, n);
  auto stage = [&](int b) {
    if (b >= nfb) return;
    float* St = &S.L[b % CH_STAGES][0][0];
    for (int k = 0; k < CH_K && b - 1 - k >= 0; ++k)
      ch_stage_block(St + k * CH_TILE, G, (int64_t)b * FB, (int64_t)(b - 1 - k) * FB, n);
    ch_stage_dinv(St + CH_K * CH_TILE, Dg + (int64_t)b * FB * FB);
  };
  auto l2_ahead = [&](int b) {
    if (b >= nfb) return;
    for (int k = 0; k < CH_K && b - 1 - k >= 0; ++k) ch_l2_block(G, (int64_t)b * FB, (int64_t)(b - 1 - k) * FB, n);
    ch_l2_dinv(Dg + (int64_t)b * FB * FB);
  };
  for (int b = CH_STAGES - 1; b < CH_L2_AHEAD; ++b) l2_ahead(b);
  for (int b = 0; b < CH_STAGES - 1; ++b) {
    stage(b);
    ch_commit();
  }
  // the right-hand side and the helper's words of a step are loaded a step
  // ahead, so that their round trip is off the chain
  double zn[NQ];
  unsigned long long pn[NQ];
  auto load_rhs = [&](int b) {
    const int row = b * FB + i;
    const bool on = b < nfb && g == 0 && i < min(FB, fs - b * FB);
#pragma unroll
    for (int q = 0; q < NQ; ++q) {
      zn[q] = (on && q < nq) ? z[row + (int64_t)(q0 + q) * n] : 0.0;
      pn[q] = (on && q < nq && b > CH_K) ? ld_hand(w + row + (int64_t)(q0 + q) * n) : 0ull;
    }
  };
  load_rhs(0);
  bool live = true;
  for (int b = 0; b < nfb; ++b) {
    const int kb = min(FB, fs - b * FB), row = b * FB + i;
    const bool rv = i < kb, lead = g == 0, helped = b > CH_K;
    double zq[NQ];
    unsigned long long pw[NQ];
    const double* pp[NQ];
#pragma unroll
    for (int q = 0; q < NQ; ++q) {
      pp[q] = w + row + (int64_t)(q0 + q) * n;
      zq[q] = zn[q];
      pw[q] = pn[q];
    }
    load_rhs(b + 1);
    ch_wait<CH_STAGES - 2>();
    __syncthreads();                      // step b's blocks staged, x of step b - 1 visible, stage (b - 1) free
    stage(b + CH_STAGES - 1);
    ch_commit();
    l2_ahead(b + CH_L2_AHEAD);
    const float* St = &S.L[b % CH_STAGES][0][0];
    float acc[NQ];
#pragma unroll
    for (int q = 0; q < NQ; ++q) acc[q] = 0.f;
    for (int k = 0; k < CH_K; ++k) {
      const int j = b - 1 - k;
      if (j < 0) break;
      const float* T = St + k * CH_TILE + sh + i;
      const float* xj = &S.xs[j % CH_K][0][0];
#pragma unroll
      for (int u = 0; u < 16; ++u) {
        const int cc = 4 * u + g;
        const float l = T[cc * CH_LD];
#pragma unroll
        for (int q = 0; q < NQ; ++q) acc[q] += l * xj[q * FB + cc];
      }
    }
#pragma unroll
    for (int q = 0; q < NQ; ++q) acc[q] = ch_sum4(acc[q]);
    if (helped && live) live = ch_wait_words<NQ>(pw, pp, nq, lead && rv, err, wait_code(3, b, b));
    if (lead) {
#pragma unroll
      for (int q = 0; q < NQ; ++q) {
        const bool on = rv && q < nq;
        const float p = helped ? (float)__longlong_as_double((long long)pw[q]) : 0.f;
        S.ts[q][i] = on ? (float)zq[q] - p - acc[q] : 0.f;
        if (on) {
          // the right-hand side and the partial sum are consumed: their words
          // become the backward solve's hand-offs
          z[row + (int64_t)(q0 + q) * n] = __longlong_as_double((long long)HAND_EMPTY);
          w[row + (int64_t)(q0 + q) * n] = __longlong_as_double((long long)HAND_EMPTY);
        }
      }
    }
    __syncthreads();
    // x_b = Dinv_b t (Dinv lower triangular)
    const float* Dm = St + CH_K * CH_TILE + i;
    float xp[NQ];
#pragma unroll
    for (int q = 0; q < NQ; ++q) xp[q] = 0.f;
#pragma unroll
    for (int u = 0; u < 16; ++u) {
      const int t = 4 * u + g;
      if (t <= i) {
        const float d = Dm[t * CH_LD];
#pragma unroll
        for (int q = 0; q < NQ; ++q) xp[q] += d * S.ts[q][t];
      }
    }
#pragma unroll
    for (int q = 0; q < NQ; ++q) xp[q] = ch_sum4(xp[q]);
    if (lead) {
#pragma unroll
      for (int q = 0; q < NQ; ++q) {
        const bool on = rv && q < nq;
        S.xs[b % CH_K][q][i] = on ? xp[q] : 0.f;
        if (on) st_hand(y + row + (int64_t)(q0 + q) * n, (double)xp[q]);
      }
    }
  }
  ch_wait<0>();
}

// backward chain of one front (thread: column cc = tid / 4 of the block, row phase g = tid % 4)
template <int NQ>
__device__ void bwd_chain(const DevCtx& c, const FrontDev& f, int q0, int nq, int* err, ChainSmem& S) {
  const int tid = threadIdx.x, cc = tid >> 2, g = tid & 3;
  const int64_t n = f.n;
  const int fs = f.fs, nr = c.n_rhs, nfb = (fs + FB - 1) / FB;
  const float* __restrict__ G = c.a32 + f.off;
  const float* __restrict__ Dg = c.dinv32 + f.dinv_off;
  double* __restrict__ hx = c.vec + f.voff;       // backward hand-off: the z slab's factor rows
  double* __restrict__ y = hx + n * nr;
  double* __restrict__ w = y + n * nr;
  const bool has_abl = fs < f.n;
  const int sh = ch_sh(0, cc, n);                 // this thread's column in every staged block
  // step s solves block b = nfb - 1 - s; its window: row blocks b + 1 .. b + CH_K
  auto stage = [&](int s) {
    const int b = nfb - 1 - s;
    if (b < 0) return;
    float* St = &S.L[s % CH_STAGES][0][0];
    for (int k = 0; k < CH_K && b + 1 + k < nfb; ++k)
      ch_stage_block(St + k * CH_TILE, G, (int64_t)(b + 1 + k) * FB, (int64_t)b * FB, n);
    ch_stage_dinv(St + CH_K * CH_TILE, Dg + (int64_t)b * FB * FB);
  };
  auto l2_ahead = [&](int s) {
    const int b = nfb - 1 - s;
    if (b < 0) return;
    for (int k = 0; k < CH_K && b + 1 + k < nfb; ++k) ch_l2_block(G, (int64_t)(b + 1 + k) * FB, (int64_t)b * FB, n);
    ch_l2_dinv(Dg + (int64_t)b * FB * FB);
  };
  for (int s = CH_STAGES - 1; s < CH_L2_AHEAD; ++s) l2_ahead(s);
  for (int s = 0; s < CH_STAGES - 1; ++s) {
    stage(s);
    ch_commit();
  }
  // the forward solution and the helper's words of a step, a step ahead
  double yn[NQ];
  unsigned long long pn[NQ];
  auto load_rhs = [&](int s) {
    const int b = nfb - 1 - s, col = b * FB + cc;
    const bool on = b >= 0 && g == 0 && cc < min(FB, fs - b * FB);
    const bool helped = has_abl || b + CH_K + 1 <= nfb - 1;
#pragma unroll
    for (int q = 0; q < NQ; ++q) {
      yn[q] = (on && q < nq) ? y[col + (int64_t)(q0 + q) * n] : 0.0;
      pn[q] = (on && q < nq && helped) ? ld_hand(w + col + (int64_t)(q0 + q) * n) : 0ull;
    }
  };
  load_rhs(0);
  bool live = true;
  for (int s = 0; s < nfb; ++s) {
    const int b = nfb - 1 - s;
    const int kb = min(FB, fs - b * FB), col = b * FB + cc;
    const bool cv = cc < kb, lead = g == 0;
    const bool helped = has_abl || b + CH_K + 1 <= nfb - 1;
    double yq[NQ];
    unsigned long long pw[NQ];
    const double* pp[NQ];
#pragma unroll
    for (int q = 0; q < NQ; ++q) {
      pp[q] = w + col + (int64_t)(q0 + q) * n;
      yq[q] = yn[q];
      pw[q] = pn[q];
    }
    load_rhs(s + 1);
    ch_wait<CH_STAGES - 2>();
    __syncthreads();
    stage(s + CH_STAGES - 1);
    ch_commit();
    l2_ahead(s + CH_L2_AHEAD);
    const float* St = &S.L[s % CH_STAGES][0][0];
    float acc[NQ];
#pragma unroll
    for (int q = 0; q < NQ; ++q) acc[q] = 0.f;
    for (int k = 0; k < CH_K; ++k) {
      const int r = b + 1 + k;
      if (r >= nfb) break;
      const int kbr = min(FB, fs - r * FB);
      const float* T = St + k * CH_TILE + cc * CH_LD + sh;
      const float* xr = &S.xs[r % CH_K][0][0];
#pragma unroll
      for (int u = 0; u < 16; ++u) {
        const int ii = 4 * u + g;
        // rows past the factor block hold other data: skipped, not multiplied by 0
        const float l = ii < kbr ? T[ii] : 0.f;
#pragma unroll
        for (int q = 0; q < NQ; ++q) acc[q] += l * xr[q * FB + ii];
      }
    }
#pragma unroll
    for (int q = 0; q < NQ; ++q) acc[q] = ch_sum4(acc[q]);
    if (helped && live) live = ch_wait_words<NQ>(pw, pp, nq, lead && cv, err, wait_code(4, b, b));
    if (lead) {
#pragma unroll
      for (int q = 0; q < NQ; ++q) {
        const bool on = cv && q < nq;
        const float p = helped ? (float)__longlong_as_double((long long)pw[q]) : 0.f;
        S.ts[q][cc] = on ? (float)yq[q] - p - acc[q] : 0.f;
      }
    }
    __syncthreads();
    // x_b = Dinv_b^T t: x[cc] = sum_{t >= cc} Dinv[t][cc] t[t]
    const float* Dm = St + CH_K * CH_TILE + cc * CH_LD;
    float xp[NQ];
#pragma unroll
    for (int q = 0; q < NQ; ++q) xp[q] = 0.f;
#pragma unroll
    for (int u = 0; u < 16; ++u) {
      const int t = 4 * u + g;
      if (t >= cc) {
        const float d = Dm[t];
#pragma unroll
        for (int q = 0; q < NQ; ++q) xp[q] += d * S.ts[q][t];
      }
    }
#pragma unroll
    for (int q = 0; q < NQ; ++q) xp[q] = ch_sum4(xp[q]);
    if (lead) {
#pragma unroll
      for (int q = 0; q < NQ; ++q) {
        const bool on = cv && q < nq;
        S.xs[b % CH_K][q][cc] = on ? xp[q] : 0.f;
        if (on) {
          y[col + (int64_t)(q0 + q) * n] = (double)xp[q];
          st_hand(hx + col + (int64_t)(q0 + q) * n, (double)xp[q]);
        }
      }
    }
  }
  ch_wait<0>();
}

// Helper and ABL rows of the forward chain: acc[q] = sum over column blocks
// j < jend of L[row, block j] x_j for the CTA's 64 rows r0.. (thread: row
// lane tid % 64, column group tid / 64).  The blocks stream through
// shared memory CH_HS - 1 ahead (cp.async); warp 0 keeps the hand-off words
// of CH_HW blocks in flight, waits (bounded) for each block's words and
// stages their values.
template <int NQ>
__device__ __forceinline__ void chain_fwd_rows(const DevCtx& c, const FrontDev& f, int r0, int jend, int q0, int nq,
                                               int* err, float (&acc)[NQ], ChainRowSmem& S) {
  const int64_t n = f.n;
  const int fs = f.fs, i = threadIdx.x % FB, g = threadIdx.x / FB;
  const float* __restrict__ G = c.a32 + f.off;
  const double* __restrict__ y = c.vec + f.voff + n * c.n_rhs;
  const bool w0 = threadIdx.x < 32;
  int sh[4];                        // shift of the staged columns cc with cc % 4 = 0, 1, 2, 3
#pragma unroll
  for (int k = 0; k < 4; ++k) sh[k] = ch_sh(r0, k, n);
  auto kbj = [&](int j) { return min(FB, fs - j * FB); };
  auto stage = [&](int j) {
    if (j < jend) ch_stage_block(S.L[j % CH_HS], G, r0, (int64_t)j * FB, n, kbj(j));
  };
  for (int j = 0; j < CH_HS - 1; ++j) {
    stage(j);
    ch_commit();
  }
  HandWords hw[CH_HW];
  bool live = true;
  if (w0) {
#pragma unroll
    for (int u = 0; u < CH_HW; ++u)
      if (u < jend) hw[u].load(y + u * FB + (int64_t)q0 * n, kbj(u));
  }
  for (int J = 0; J < jend; J += CH_HW) {
#pragma unroll
    for (int u = 0; u < CH_HW; ++u) {
      const int j = J + u;
      if (j >= jend) break;
      const int kb = kbj(j);
      if (w0) {
        const double* yj = y + j * FB;
        if (live) live = hw[u].wait(yj + (int64_t)q0 * n, kb, err, wait_code(1, j, r0 / FB));
        hw[u].stage(S.vsh[j & 1][0]);
        for (int q = 1; q < nq; ++q) {
          HandWords hq;
          hq.load(yj + (int64_t)(q0 + q) * n, kb);
          if (live) live = hq.wait(yj + (int64_t)(q0 + q) * n, kb, err, wait_code(1, j, r0 / FB));
          hq.stage(S.vsh[j & 1][q]);
        }
        if (j + CH_HW < jend) hw[u].load(y + (j + CH_HW) * FB + (int64_t)q0 * n, kbj(j + CH_HW));
      }
      ch_wait<CH_HS - 2>();
      __syncthreads();
      stage(j + CH_HS - 1);
      ch_commit();
      const float* T = S.L[j % CH_HS] + i;
      const float* v = &S.vsh[j & 1][0][0];
#pragma unroll
      for (int uu = 0; uu < 16; ++uu) {
        const int cc = g * 16 + uu;
        // columns past the factor block hold other data: skipped
        const float l = cc < kb ? T[cc * CH_LD + sh[uu & 3]] : 0.f;
#pragma unroll
        for (int q = 0; q < NQ; ++q) acc[q] += l * v[q * FB + cc];
      }
    }
  }
  ch_wait<0>();
}

// Helper rows of the backward chain for column block b: acc[q][u] = sum over
// the row blocks below the chain's window (the ABL rows, x from the parent,
// then the factor blocks nfb - 1 down to b + CH_K + 1, x from the hand-off
// words) of L[r, 64 b + 16 g + u] x_r (thread: row lane tid % 64, column
// group tid / 64); staged as in chain_fwd_rows.
template <int NQ>
__device__ __forceinline__ void chain_bwd_rows(const DevCtx& c, const FrontDev& f, int b, int q0, int nq, int* err,
                                               float (&acc)[NQ][16], ChainRowSmem& S) {
  const int64_t n = f.n;
  const int fs = f.fs, nfb = (fs + FB - 1) / FB, rl = threadIdx.x % FB, g = threadIdx.x / FB;
  const int kbc = min(FB, fs - b * FB);
  const float* __restrict__ G = c.a32 + f.off;
  const double* __restrict__ hx = c.vec + f.voff;
  const double* __restrict__ y = hx + n * c.n_rhs;
  const int nab = (int)((n - fs + FB - 1) / FB);
  const int nfar = max(0, nfb - 1 - (b + CH_K));
  const int tend = nab + nfar;
  // row block t: the ABL blocks first, then factor blocks from the last one up
  auto r0_of = [&](int t) { return t < nab ? fs + t * FB : (nfb - 1 - (t - nab)) * FB; };
  auto rend_of = [&](int t) { return t < nab ? (int)n : min((nfb - 1 - (t - nab)) * FB + FB, fs); };
  auto src_of = [&](int t) -> const double* { return t < nab ? y : hx; };
  auto stage = [&](int t) {
    if (t < tend) ch_stage_block(S.L[t % CH_HS], G, r0_of(t), (int64_t)b * FB, n, kbc);
  };
  for (int t = 0; t < CH_HS - 1; ++t) {
    stage(t);
    ch_commit();
  }
  const bool w0 = threadIdx.x < 32;
  HandWords hw[CH_HW];
  bool live = true;
  if (w0) {
#pragma unroll
    for (int u = 0; u < CH_HW; ++u)
      if (u < tend) hw[u].load(src_of(u) + r0_of(u) + (int64_t)q0 * n, rend_of(u) - r0_of(u));
  }
  for (int T0 = 0; T0 < tend; T0 += CH_HW) {
#pragma unroll
    for (int u = 0; u < CH_HW; ++u) {
      const int t = T0 + u;
      if (t >= tend) break;
      const int r0 = r0_of(t), kr = rend_of(t) - r0;
      if (w0) {
        const double* xr = src_of(t) + r0;
        if (live) live = hw[u].wait(xr + (int64_t)q0 * n, kr, err, wait_code(2, r0 / FB, b));
        hw[u].stage(S.vsh[t & 1][0]);
        for (int q = 1; q < nq; ++q) {
          HandWords hq;
          hq.load(xr + (int64_t)(q0 + q) * n, kr);
          if (live) live = hq.wait(xr + (int64_t)(q0 + q) * n, kr, err, wait_code(2, r0 / FB, b));
          hq.stage(S.vsh[t & 1][q]);
        }
        if (t + CH_HW < tend)
          hw[u].load(src_of(t + CH_HW) + r0_of(t + CH_HW) + (int64_t)q0 * n, rend_of(t + CH_HW) - r0_of(t + CH_HW));
      }
      ch_wait<CH_HS - 2>();
      __syncthreads();
      stage(t + CH_HS - 1);
      ch_commit();
      if (rl < kr) {
        // rows past the block (or the front) hold other data: skipped
        const float* Tt = S.L[t % CH_HS] + rl;
        int sh[4];
#pragma unroll
        for (int k = 0; k < 4; ++k) sh[k] = ch_sh(r0, k, n);
        float xv[NQ];
#pragma unroll
        for (int q = 0; q < NQ; ++q) xv[q] = S.vsh[t & 1][q][rl];
#pragma unroll
        for (int uu = 0; uu < 16; ++uu) {
          const int cc = g * 16 + uu;
          const float l = cc < kbc ? Tt[cc * CH_LD + sh[uu & 3]] : 0.f;
#pragma unroll
          for (int q = 0; q < NQ; ++q) acc[q][uu] += l * xv[q];
        }
      }
    }
  }
  ch_wait<0>();
}

template <int NQ>
__device__ __forceinline__ void fwd_chain_cta(const DevCtx& c, const Item& it, const FrontDev& f, int q0, int nq,
                                              int* err, unsigned char* raw) {
  if (it.b == CH_CHAIN) {
    fwd_chain<NQ>(c, f, q0, nq, err, *reinterpret_cast<ChainSmem*>(raw));
    return;
  }
  ChainRowSmem& H = *reinterpret_cast<ChainRowSmem*>(raw);
  const int n = f.n, fs = f.fs, nfb = (fs + FB - 1) / FB, b = it.a;
  const bool helper = it.b == CH_HELPER;      // else CH_ABL
  const int r0 = helper ? b * FB : fs + (b - nfb) * FB;
  const int r1 = helper ? min(r0 + FB, fs) : min(r0 + FB, n);
  const int i = threadIdx.x % FB, gg = threadIdx.x / FB, row = r0 + i;
  const bool rv = row < r1;
  double* __restrict__ z = c.vec + f.voff;
  double* __restrict__ w = z + 2 * (int64_t)n * c.n_rhs;
  if (helper) {
    // the chain reads this row block's CH_K blocks next to the diagonal and
    // its inverse from one SM: start them towards L2 long before
    for (int k = 1; k <= CH_K; ++k) ch_l2_block(c.a32 + f.off, (int64_t)b * FB, (int64_t)(b - k) * FB, n);
    ch_l2_dinv(c.dinv32 + f.dinv_off + (int64_t)b * FB * FB);
  }
  float zr[NQ], acc[NQ];
#pragma unroll
  for (int q = 0; q < NQ; ++q) {
    acc[q] = 0.f;
    zr[q] = (!helper && rv && q < nq && gg == 0) ? (float)z[row + (int64_t)(q0 + q) * n] : 0.f;
  }
  chain_fwd_rows<NQ>(c, f, r0, helper ? b - CH_K : nfb, q0, nq, err, acc, H);
#pragma unroll
  for (int q = 0; q < NQ; ++q) H.red[gg][i][q] = acc[q];
  __syncthreads();
  if (threadIdx.x < FB && rv) {
#pragma unroll
    for (int q = 0; q < NQ; ++q) {
      if (q >= nq) break;
      const float sum = H.red[0][i][q] + H.red[1][i][q] + H.red[2][i][q] + H.red[3][i][q];
      if (helper) st_hand(w + row + (int64_t)(q0 + q) * n, (double)sum);
      else z[row + (int64_t)(q0 + q) * n] = (double)(zr[q] - sum);
    }
  }
}

template <int NQ>
__device__ __forceinline__ void bwd_chain_cta(const DevCtx& c, const Item& it, const FrontDev& f, int q0, int nq,
                                              int* err, unsigned char* raw) {
  if (it.b == CH_CHAIN) {
    bwd_chain<NQ>(c, f, q0, nq, err, *reinterpret_cast<ChainSmem*>(raw));
    return;
  }
  ChainRowSmem& H = *reinterpret_cast<ChainRowSmem*>(raw);
  const int n = f.n, fs = f.fs, b = it.a;
  const int c0 = b * FB, kb = min(FB, fs - c0);
  double* __restrict__ w = c.vec + f.voff + 2 * (int64_t)n * c.n_rhs;
  const int rl = threadIdx.x % FB, gg = threadIdx.x / FB;
  {
    // the chain's blocks below this column block's diagonal and its inverse, towards L2
    const int nfb = (fs + FB - 1) / FB;
    for (int k = 1; k <= CH_K && b + k < nfb; ++k) ch_l2_block(c.a32 + f.off, (int64_t)(b + k) * FB, (int64_t)b * FB, n);
    ch_l2_dinv(c.dinv32 + f.dinv_off + (int64_t)b * FB * FB);
  }
  float acc[NQ][16];
#pragma unroll
  for (int q = 0; q < NQ; ++q)
#pragma unroll
    for (int u = 0; u < 16; ++u) acc[q][u] = 0.f;
  chain_bwd_rows<NQ>(c, f, b, q0, nq, err, acc, H);
  // column sums over the 64 row lanes, one right-hand side at a time
#pragma unroll
  for (int q = 0; q < NQ; ++q) {
    if (q >= nq) break;
    __syncthreads();
#pragma unroll
    for (int u = 0; u < 16; ++u) H.redb[rl][gg * 16 + u] = acc[q][u];
    __syncthreads();
    if (threadIdx.x < kb) {
      float s = 0.f;
      for (int r = 0; r < FB; ++r) s += H.redb[r][threadIdx.x];
      st_hand(w + c0 + threadIdx.x + (int64_t)(q0 + q) * n, (double)s);
    }
  }
}

// item: front, a = block, b = role; right-hand sides q0 .. q0 + SF_NR - 1
__global__ void __launch_bounds__(256, 1) k_fwd_chain(DevCtx c, const Item* __restrict__ items, int* ticket, int* err,
                                                      int q0) {
  extern __shared__ __align__(16) unsigned char ch_raw[];
  __shared__ int s_t;
  if (threadIdx.x == 0) s_t = atomicAdd(ticket, 1);
  __syncthreads();
  const Item it = items[s_t];
  const FrontDev f = c.fronts[it.front];
  const int nq = min(SF_NR, c.n_rhs - q0);
  if (nq == 1) fwd_chain_cta<1>(c, it, f, q0, nq, err, ch_raw);
  else if (nq == 2) fwd_chain_cta<2>(c, it, f, q0, nq, err, ch_raw);
  else fwd_chain_cta<SF_NR>(c, it, f, q0, nq, err, ch_raw);
}

// item: front, a = column block, b = role (chain or helper); right-hand sides q0 .. q0 + SF_NR - 1
__global__ void __launch_bounds__(256, 1) k_bwd_chain(DevCtx c, const Item* __restrict__ items, int* ticket, int* err,
                                                      int q0) {
  extern __shared__ __align__(16) unsigned char ch_raw[];
  __shared__ int s_t;
  if (threadIdx.x == 0) s_t = atomicAdd(ticket, 1);
  __syncthreads();
  const Item it = items[s_t];
  const FrontDev f = c.fronts[it.front];
  const int nq = min(SF_NR, c.n_rhs - q0);
  if (nq == 1) bwd_chain_cta<1>(c, it, f, q0, nq, err, ch_raw);
  else if (nq == 2) bwd_chain_cta<2>(c, it, f, q0, nq, err, ch_raw);
  else bwd_chain_cta<SF_NR>(c, it, f, q0, nq, err, ch_raw);
}

void launch_fwd_chain(const DevCtx& c, const Item* items, int n_items, int* ticket, int* err, int q0,
                      cudaStream_t s) {
  if (!n_items) return;
  cudaMemsetAsync(ticket, 0, sizeof(int), s);
  cudaFuncSetAttribute(k_fwd_chain, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)CH_SMEM);
  k_fwd_chain<<<n_items, 256, CH_SMEM, s>>>(c, items, ticket, err, q0);
}

void launch_bwd_chain(const DevCtx& c, const Item* items, int n_items, int* ticket, int* err, int q0,
                      cudaStream_t s) {
  if (!n_items) return;
  cudaMemsetAsync(ticket, 0, sizeof(int), s);
  cudaFuncSetAttribute(k_bwd_chain, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)CH_SMEM);
  k_bwd_chain<<<n_items, 256, CH_SMEM, s>>>(c, items, ticket, err, q0);
}

}  // namespace uhm_gpu
