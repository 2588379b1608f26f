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

// z = [g[g0 .. g0+fs); 0] + sum over children of their xb (extend-add)
__global__ void __launch_bounds__(256) k_fwd_gather(DevCtx c, const Item* __restrict__ items,
                                                    const double* __restrict__ g, int64_t ldg,
                                                    int method) {
  const Item it = items[blockIdx.x];
  const FrontDev f = c.fronts[it.front];
  const int n = f.n;
  double* __restrict__ z = c.vec + f.voff;
  const int32_t* __restrict__ inv = c.inv + f.inv_off;
  for (int q = 0; q < c.n_rhs; ++q) {
    for (int I = threadIdx.x; I < n; I += blockDim.x) {
      double acc = I < f.fs ? g[(f.g0 + I) + q * ldg] : 0.0;
      for (int s = 0; s < f.nsrc; ++s) {
        const SrcDev sd = c.srcs[f.src0 + s];
        if (!sd.is_child) continue;
        const int is = inv[(int64_t)s * n + I];
        if (is >= 0) {
          const FrontDev ch = c.fronts[sd.slot];
          acc += c.vec[ch.voff + ch.fs + is + (int64_t)q * ch.n];
        }
      }
      z[I + (int64_t)q * n] = acc;
    }
  }
  __syncthreads();
  if (method == M_LU_PIV && threadIdx.x < c.n_rhs) {
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
  for (int idx = threadIdx.x; idx < n * nr; idx += NT) zg[idx] = z[idx];
}

void launch_fwd_small(const DevCtx& c, const Item* items, int n_items, int dtype, int method,
                      cudaStream_t s) {
  if (!n_items) return;
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
  double* __restrict__ z = c.vec + f.voff;
  const int32_t* __restrict__ sgi = c.sgi + f.sgi_off;
  for (int q = 0; q < c.n_rhs; ++q)
    for (int j = threadIdx.x; j < f.ss; j += blockDim.x)
      z[f.fs + j + (int64_t)q * f.n] = g[sgi[j] + q * ldg];
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
  double* __restrict__ zg = c.vec + f.voff;
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
  for (int idx = threadIdx.x; idx < n * nr; idx += NT) zg[idx] = z[idx];
  for (int q = 0; q < nr; ++q)
    for (int i = threadIdx.x; i < fs; i += NT) g[(f.g0 + i) + q * ldg] = z[i + q * n];
}

void launch_bwd_small(const DevCtx& c, const Item* items, int n_items, int dtype, int method,
                      double* g, int64_t ldg, cudaStream_t s) {
  if (!n_items) return;
  size_t sm = 8192 * sizeof(double);
  if (dtype == F64) {
    cudaFuncSetAttribute(k_bwd_small<double, 256>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm);
    k_bwd_small<double, 256><<<n_items, 256, sm, s>>>(c, items, method, g, ldg);
  } else {
    cudaFuncSetAttribute(k_bwd_small<float, 256>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm);
    k_bwd_small<float, 256><<<n_items, 256, sm, s>>>(c, items, method, g, ldg);
  }
}

// Large fronts, blocked by nb.  item: front, a = k0.
// upper == 0: forward diagonal solve  z_k <- L_kk^{-1} z_k  (unit for LU)
// upper == 1: backward diagonal solve z_k <- L_kk^{-T} z_k (Chol) / U_kk^{-1} z_k (LU)
template <typename T, int NT>
__global__ void __launch_bounds__(NT) k_trsv_block(DevCtx c, const Item* __restrict__ items,
                                                   int method, int nb, int upper) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  T* D = reinterpret_cast<T*>(smem_raw);                   // kb x kb
  double* z = reinterpret_cast<double*>(D + nb * nb);       // kb x n_rhs
  const Item it = items[blockIdx.x];
  const FrontDev f = c.fronts[it.front];
  const int n = f.n, k0 = it.a, nr = c.n_rhs;
  const int kb = min(nb, f.fs - k0);
  const T* __restrict__ G = arena<T>(c) + f.off;
  double* __restrict__ zg = c.vec + f.voff;
  for (int idx = threadIdx.x; idx < kb * kb; idx += NT) {
    const int i = idx % kb, j = idx / kb;
    D[idx] = G[(k0 + i) + (int64_t)(k0 + j) * n];
  }
  for (int idx = threadIdx.x; idx < kb * nr; idx += NT) {
    const int i = idx % kb, q = idx / kb;
    z[i + q * kb] = zg[(k0 + i) + (int64_t)q * n];
  }
  __syncthreads();
  const bool chol = method == M_CHOL;
  if (!upper) {
    for (int j = 0; j < kb; ++j) {
      if (chol && threadIdx.x < nr) z[j + threadIdx.x * kb] /= (double)D[j + j * kb];
      __syncthreads();
      const int h = kb - j - 1;
      for (int idx = threadIdx.x; idx < h * nr; idx += NT) {
        const int i = j + 1 + idx % h, q = idx / h;
        z[i + q * kb] -= (double)D[i + j * kb] * z[j + q * kb];
      }
      __syncthreads();
    }
  } else {
    for (int j = kb - 1; j >= 0; --j) {
      if (threadIdx.x < nr) z[j + threadIdx.x * kb] /= (double)D[j + j * kb];
      __syncthreads();
      for (int idx = threadIdx.x; idx < j * nr; idx += NT) {
        const int i = idx % j, q = idx / j;
        // chol: L^T(i, j) = L(j, i); LU: U(i, j)
        const double a = chol ? (double)D[j + i * kb] : (double)D[i + j * kb];
        z[i + q * kb] -= a * z[j + q * kb];
      }
      __syncthreads();
    }
  }
  for (int idx = threadIdx.x; idx < kb * nr; idx += NT) {
    const int i = idx % kb, q = idx / kb;
    zg[(k0 + i) + (int64_t)q * n] = z[i + q * kb];
  }
}

void launch_trsv_block(const DevCtx& c, const Item* items, int n_items, int dtype, int method,
                       int nb, int upper, cudaStream_t s) {
  if (!n_items) return;
  if (dtype == F64) {
    size_t sm = (size_t)nb * nb * sizeof(double) + (size_t)nb * c.n_rhs * sizeof(double);
    cudaFuncSetAttribute(k_trsv_block<double, 256>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm);
    k_trsv_block<double, 256><<<n_items, 256, sm, s>>>(c, items, method, nb, upper);
  } else {
    size_t sm = (size_t)nb * nb * sizeof(float) + (size_t)nb * c.n_rhs * sizeof(double) + 16;
    cudaFuncSetAttribute(k_trsv_block<float, 256>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm);
    k_trsv_block<float, 256><<<n_items, 256, sm, s>>>(c, items, method, nb, upper);
  }
}

constexpr int GEMV_RB = 256;

// upper == 0 (forward): item front, a = k0, b = r0:  z[r0..r0+RB) -= A[r0.., k0..k0+kb) z_k
// upper == 1 (backward): item front, a = k0:  z_k -= A_tail^T z_tail (Chol: L[k0+kb:n, k]^T;
//                        LU: U[k, k0+kb:n]) ; one CTA per step, reduction over the tail
template <typename T, int NT>
__global__ void __launch_bounds__(NT) k_gemv_panel(DevCtx c, const Item* __restrict__ items,
                                                   int method, int nb, int upper) {
  __shared__ double s_z[64 * 16];
  __shared__ double s_red[NT / 32 + 1];
  const Item it = items[blockIdx.x];
  const FrontDev f = c.fronts[it.front];
  const int n = f.n, k0 = it.a, nr = c.n_rhs;
  const int kb = min(nb, f.fs - k0);
  const T* __restrict__ G = arena<T>(c) + f.off;
  double* __restrict__ zg = c.vec + f.voff;
  if (!upper) {
    const int r0 = it.b;
    for (int idx = threadIdx.x; idx < kb * nr; idx += NT) {
      const int i = idx % kb, q = idx / kb;
      s_z[i + q * 64] = zg[(k0 + i) + (int64_t)q * n];
    }
    __syncthreads();
    for (int r = r0 + threadIdx.x; r < min(r0 + GEMV_RB, n); r += NT) {
      for (int q = 0; q < nr; ++q) {
        double acc = 0.0;
        for (int t = 0; t < kb; ++t) acc += (double)G[r + (int64_t)(k0 + t) * n] * s_z[t + q * 64];
        zg[r + (int64_t)q * n] -= acc;
      }
    }
  } else {
    const bool chol = method == M_CHOL;
    const int t0 = k0 + kb;
    for (int q = 0; q < nr; ++q) {
      for (int i = 0; i < kb; ++i) {
        double part = 0.0;
        if (chol)
          for (int r = t0 + threadIdx.x; r < n; r += NT)
            part += (double)G[r + (int64_t)(k0 + i) * n] * zg[r + (int64_t)q * n];
        else
          for (int r = t0 + threadIdx.x; r < n; r += NT)
            part += (double)G[(k0 + i) + (int64_t)r * n] * zg[r + (int64_t)q * n];
        const double sum = block_sum<NT>(part, s_red);
        if (threadIdx.x == 0) zg[(k0 + i) + (int64_t)q * n] -= sum;
      }
    }
  }
}

void launch_gemv_panel(const DevCtx& c, const Item* items, int n_items, int dtype, int method,
                       int nb, int upper, cudaStream_t s) {
  if (!n_items) return;
  if (dtype == F64) k_gemv_panel<double, 256><<<n_items, 256, 0, s>>>(c, items, method, nb, upper);
  else k_gemv_panel<float, 256><<<n_items, 256, 0, s>>>(c, items, method, nb, upper);
}

__global__ void __launch_bounds__(256) k_bwd_store(DevCtx c, const Item* __restrict__ items,
                                                   double* __restrict__ g, int64_t ldg) {
  const Item it = items[blockIdx.x];
  const FrontDev f = c.fronts[it.front];
  const double* __restrict__ z = c.vec + f.voff;
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
__global__ void k_absmax_partial(const double* __restrict__ v, int64_t n, double* __restrict__ part) {
  __shared__ double s[256];
  double m = 0.0;
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x)
    m = fmax(m, fabs(v[i]));
  s[threadIdx.x] = m;
  __syncthreads();
  for (int o = 128; o > 0; o >>= 1) {
    if (threadIdx.x < o) s[threadIdx.x] = fmax(s[threadIdx.x], s[threadIdx.x + o]);
    __syncthreads();
  }
  if (threadIdx.x == 0) part[blockIdx.x] = s[0];
}

__global__ void k_absmax_final(const double* __restrict__ part, int np, double* __restrict__ out) {
  __shared__ double s[256];
  double m = 0.0;
  for (int i = threadIdx.x; i < np; i += blockDim.x) m = fmax(m, part[i]);
  s[threadIdx.x] = m;
  __syncthreads();
  for (int o = 128; o > 0; o >>= 1) {
    if (threadIdx.x < o) s[threadIdx.x] = fmax(s[threadIdx.x], s[threadIdx.x + o]);
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
