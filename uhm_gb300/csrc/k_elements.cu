// Element matrices of hp-FEM meshes generated on the device: the step before
// the multifrontal path (the element matrices a caller would otherwise build
// on the host and copy in), written straight into the engine's element
// buffer.
//
// For a uniform quad / hex mesh with tensor-product integrated-Legendre
// (Lobatto) modes of order p, every element matrix is a combination of
// Kronecker products of the 1D reference matrices M (mass), K (stiffness) and
// C (convection) of its order, restricted to the element's retained modes:
//   3D  A = kappa (h/2) (M(x)M(x)K + M(x)K(x)M + K(x)M(x)M) [+ c (h/2)^3 M(x)M(x)M]
//           [+ sum_a beta_a (h/2)^2 (the term with C on axis a)]
//   2D  A = kappa (M(x)K + K(x)M) [+ c (h/2)^2 M(x)M] [+ sum_a beta_a (h/2) ...]
// (axis x varies fastest in the flat mode index mi[0] + mi[1] (p+1) + ...).
// Each entry is formed with the same products and sums in the same order as
// the host generator (uhm_gb300/hpfem.py build_mesh), with no fused
// multiply-add, so the matrices are bit-identical to the host ones.  FP64
// arithmetic is scarce on this GPU, so everything but the per-element
// coefficients is formed once per order in tables over all mode pairs; the
// per-element pass is then one multiply (plus one multiply-add pair per
// optional term) and a store per entry.
#include <cstdint>
#include <cuda_runtime.h>
#include "kernels.cuh"

namespace uhm_gpu {

constexpr int GEN_MAXM = 512;   // retained modes per element ((p+1)^3 for p <= 7)

// Per order p, every element-independent factor of an entry, over all pairs
// (ga, gb) of tensor-grid modes (G = (p+1)^dim of them), column-major
// (ga fastest), table after table:
//   S  = hh ((t1 + t2) + t3)            (3D; 2D: M K + K M)
//   Rm = cmass (M (M M))                 when the mesh has a reaction term
//   Ca = cconv (the term with C on axis a), a < dim, when it has convection
// An entry of element e is then kappa_e S [+ react_e Rm] [+ beta_a Ca ...],
// the host generator's products and sums in its order.
__global__ void __launch_bounds__(256) k_gen_tables(double* __restrict__ tab, const double* __restrict__ R, int q,
                                                    int dim, double hh, double cmass, double cconv, int has_react,
                                                    int has_beta) {
  const int G = dim == 3 ? q * q * q : q * q;
  const int64_t GG = (int64_t)G * G;
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= GG) return;
  const int ga = (int)(i % G), gb = (int)(i / G);
  const int xa = (ga % q) * q + gb % q;
  const int ya = ((ga / q) % q) * q + (gb / q) % q;
  const int za = (ga / (q * q)) * q + gb / (q * q);
  const double* __restrict__ M = R;
  const double* __restrict__ K = R + q * q;
  const double* __restrict__ C = R + 2 * q * q;
  double* t = tab;
  if (dim == 3) {
    const double t1 = __dmul_rn(M[za], __dmul_rn(M[ya], K[xa]));
    const double t2 = __dmul_rn(M[za], __dmul_rn(K[ya], M[xa]));
    const double t3 = __dmul_rn(K[za], __dmul_rn(M[ya], M[xa]));
    t[i] = __dmul_rn(hh, __dadd_rn(__dadd_rn(t1, t2), t3));
    t += GG;
    if (has_react) {
      t[i] = __dmul_rn(cmass, __dmul_rn(M[za], __dmul_rn(M[ya], M[xa])));
      t += GG;
    }
    if (has_beta) {
      t[i] = __dmul_rn(cconv, __dmul_rn(M[za], __dmul_rn(M[ya], C[xa])));
      t[i + GG] = __dmul_rn(cconv, __dmul_rn(M[za], __dmul_rn(C[ya], M[xa])));
      t[i + 2 * GG] = __dmul_rn(cconv, __dmul_rn(C[za], __dmul_rn(M[ya], M[xa])));
    }
  } else {
    t[i] = __dadd_rn(__dmul_rn(M[ya], K[xa]), __dmul_rn(K[ya], M[xa]));
    t += GG;
    if (has_react) {
      t[i] = __dmul_rn(cmass, __dmul_rn(M[ya], M[xa]));
      t += GG;
    }
    if (has_beta) {
      t[i] = __dmul_rn(cconv, __dmul_rn(M[ya], C[xa]));
      t[i + GG] = __dmul_rn(cconv, __dmul_rn(C[ya], M[xa]));
    }
  }
}

// one CTA per element: warps over columns, lanes over rows (coalesced stores)
__global__ void __launch_bounds__(256, 4) k_gen_lobatto(double* __restrict__ emat, const int64_t* __restrict__ emat_off,
                                                     const int* __restrict__ p_el, const double* __restrict__ kappa,
                                                     const double* __restrict__ react, const double* __restrict__ beta,
                                                     const int64_t* __restrict__ sel_ptr,
                                                     const int32_t* __restrict__ sel, const double* __restrict__ tab,
                                                     const int64_t* __restrict__ tab_off, int dim) {
  __shared__ int s_sel[GEN_MAXM];
  const int e = blockIdx.x;
  const int p = p_el[e], q = p + 1;
  const int G = dim == 3 ? q * q * q : q * q;
  const int64_t GG = (int64_t)G * G;
  const int64_t s0 = sel_ptr[e];
  const int m = (int)(sel_ptr[e + 1] - s0);
  for (int a = threadIdx.x; a < m; a += blockDim.x) s_sel[a] = sel[s0 + a];
  __syncthreads();
  const double kap = kappa[e];
  const double rea = react ? react[e] : 0.0;
  const double* __restrict__ S = tab + tab_off[p];
  const double* __restrict__ Rm = S + GG;
  const double* __restrict__ Cv = react ? S + 2 * GG : S + GG;
  double* __restrict__ out = emat + emat_off[e];
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31, nw = blockDim.x >> 5;
  // a warp takes columns b and b + nw, its lanes 4 rows of each per pass:
  // eight independent table loads in flight before the stores
  constexpr int RU = 4;
  for (int b0 = warp; b0 < m; b0 += 2 * nw) {
    const int b1 = b0 + nw;
    const bool has1 = b1 < m;
    // table indices fit 32 bits: G <= 512, so G * G <= 2^18
    const int cb0 = s_sel[b0] * G, cb1 = has1 ? s_sel[b1] * G : cb0;
    double* __restrict__ col0 = out + (int64_t)b0 * m;
    double* __restrict__ col1 = out + (int64_t)(has1 ? b1 : b0) * m;
    for (int a0 = lane; a0 < m; a0 += 32 * RU) {
      int k0[RU], k1[RU];
      double v0[RU], v1[RU];
#pragma unroll
      for (int u = 0; u < RU; ++u) {
        const int a = a0 + 32 * u;
        const int sa = a < m ? s_sel[a] : 0;
        k0[u] = sa + cb0;
        k1[u] = sa + cb1;
        v0[u] = __ldg(S + k0[u]);
        v1[u] = __ldg(S + k1[u]);
      }
#pragma unroll
      for (int u = 0; u < RU; ++u) {
        v0[u] = __dmul_rn(kap, v0[u]);
        v1[u] = __dmul_rn(kap, v1[u]);
      }
      if (rea != 0.0) {
#pragma unroll
        for (int u = 0; u < RU; ++u) {
          v0[u] = __dadd_rn(v0[u], __dmul_rn(rea, __ldg(Rm + k0[u])));
          v1[u] = __dadd_rn(v1[u], __dmul_rn(rea, __ldg(Rm + k1[u])));
        }
      }
      if (beta)
        for (int d = 0; d < dim; ++d) {
          const double bd = beta[d];
          const double* __restrict__ Cd = Cv + d * GG;
#pragma unroll
          for (int u = 0; u < RU; ++u) {
            v0[u] = __dadd_rn(v0[u], __dmul_rn(bd, __ldg(Cd + k0[u])));
            v1[u] = __dadd_rn(v1[u], __dmul_rn(bd, __ldg(Cd + k1[u])));
          }
        }
#pragma unroll
      for (int u = 0; u < RU; ++u) {
        const int a = a0 + 32 * u;
        if (a < m) {
          col0[a] = v0[u];
          if (has1) col1[a] = v1[u];
        }
      }
    }
  }
}

int64_t gen_table_doubles(int p, int dim, int has_react, int has_beta) {
  const int64_t q = p + 1, G = dim == 3 ? q * q * q : q * q;
  return G * G * (1 + (has_react ? 1 : 0) + (has_beta ? dim : 0));
}

void launch_gen_tables(double* tab, const double* ref_p, int p, int dim, double hh, double cmass, double cconv,
                       int has_react, int has_beta, cudaStream_t s) {
  const int64_t q = p + 1, G = dim == 3 ? q * q * q : q * q, GG = G * G;
  k_gen_tables<<<(unsigned)((GG + 255) / 256), 256, 0, s>>>(tab, ref_p, (int)q, dim, hh, cmass, cconv, has_react,
                                                            has_beta);
}

void launch_gen_lobatto(double* emat, const int64_t* emat_off, int n_el, const int* p_el, const double* kappa,
                        const double* react, const double* beta, const int64_t* sel_ptr, const int32_t* sel,
                        const double* tab, const int64_t* tab_off, int dim, cudaStream_t s) {
  if (n_el <= 0) return;
  k_gen_lobatto<<<n_el, 256, 0, s>>>(emat, emat_off, p_el, kappa, react, beta, sel_ptr, sel, tab, tab_off, dim);
}

}  // namespace uhm_gpu
