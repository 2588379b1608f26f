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
// multiply-add, so the matrices are bit-identical to the host ones.
#include <cstdint>
#include <cuda_runtime.h>
#include "kernels.cuh"

namespace uhm_gpu {

constexpr int GEN_MAXM = 512;   // retained modes per element ((p+1)^3 for p <= 7)
constexpr int GEN_MAXQ = 8;     // p + 1

// one CTA per element; entries in column-major order (coalesced stores)
__global__ void __launch_bounds__(256) k_gen_lobatto(double* __restrict__ emat, const int64_t* __restrict__ emat_off,
                                                     const int* __restrict__ p_el, const double* __restrict__ kappa,
                                                     const double* __restrict__ react, const double* __restrict__ beta,
                                                     const int64_t* __restrict__ sel_ptr,
                                                     const int32_t* __restrict__ sel, const double* __restrict__ ref,
                                                     const int64_t* __restrict__ ref_off, int dim, double hh,
                                                     double cmass, double cconv) {
  __shared__ unsigned char s_x[GEN_MAXM], s_y[GEN_MAXM], s_z[GEN_MAXM];
  __shared__ double s_M[GEN_MAXQ * GEN_MAXQ], s_K[GEN_MAXQ * GEN_MAXQ], s_C[GEN_MAXQ * GEN_MAXQ];
  const int e = blockIdx.x;
  const int p = p_el[e], q = p + 1;
  const int64_t s0 = sel_ptr[e];
  const int m = (int)(sel_ptr[e + 1] - s0);
  const double* __restrict__ R = ref + ref_off[p];
  for (int i = threadIdx.x; i < q * q; i += blockDim.x) {
    s_M[i] = R[i];
    s_K[i] = R[q * q + i];
    s_C[i] = R[2 * q * q + i];
  }
  for (int a = threadIdx.x; a < m; a += blockDim.x) {
    const int f = sel[s0 + a];
    s_x[a] = (unsigned char)(f % q);
    s_y[a] = (unsigned char)((f / q) % q);
    s_z[a] = (unsigned char)(f / (q * q));
  }
  __syncthreads();
  const double kap = kappa[e];
  const double rea = react ? react[e] : 0.0;
  double* __restrict__ out = emat + emat_off[e];
  for (int idx = threadIdx.x; idx < m * m; idx += blockDim.x) {
    const int a = idx % m, b = idx / m;
    const int xa = s_x[a] * q + s_x[b], ya = s_y[a] * q + s_y[b], za = s_z[a] * q + s_z[b];
    double v;
    if (dim == 3) {
      const double t1 = __dmul_rn(s_M[za], __dmul_rn(s_M[ya], s_K[xa]));
      const double t2 = __dmul_rn(s_M[za], __dmul_rn(s_K[ya], s_M[xa]));
      const double t3 = __dmul_rn(s_K[za], __dmul_rn(s_M[ya], s_M[xa]));
      v = __dmul_rn(kap, __dmul_rn(hh, __dadd_rn(__dadd_rn(t1, t2), t3)));
      if (rea != 0.0)
        v = __dadd_rn(v, __dmul_rn(rea, __dmul_rn(cmass, __dmul_rn(s_M[za], __dmul_rn(s_M[ya], s_M[xa])))));
      if (beta) {
        v = __dadd_rn(v, __dmul_rn(beta[0], __dmul_rn(cconv, __dmul_rn(s_M[za], __dmul_rn(s_M[ya], s_C[xa])))));
        v = __dadd_rn(v, __dmul_rn(beta[1], __dmul_rn(cconv, __dmul_rn(s_M[za], __dmul_rn(s_C[ya], s_M[xa])))));
        v = __dadd_rn(v, __dmul_rn(beta[2], __dmul_rn(cconv, __dmul_rn(s_C[za], __dmul_rn(s_M[ya], s_M[xa])))));
      }
    } else {
      v = __dmul_rn(kap, __dadd_rn(__dmul_rn(s_M[ya], s_K[xa]), __dmul_rn(s_K[ya], s_M[xa])));
      if (rea != 0.0) v = __dadd_rn(v, __dmul_rn(rea, __dmul_rn(cmass, __dmul_rn(s_M[ya], s_M[xa]))));
      if (beta) {
        v = __dadd_rn(v, __dmul_rn(beta[0], __dmul_rn(cconv, __dmul_rn(s_M[ya], s_C[xa]))));
        v = __dadd_rn(v, __dmul_rn(beta[1], __dmul_rn(cconv, __dmul_rn(s_C[ya], s_M[xa]))));
      }
    }
    out[idx] = v;
  }
}

void launch_gen_lobatto(double* emat, const int64_t* emat_off, int n_el, const int* p_el, const double* kappa,
                        const double* react, const double* beta, const int64_t* sel_ptr, const int32_t* sel,
                        const double* ref, const int64_t* ref_off, int dim, double hh, double cmass,
                        double cconv, cudaStream_t s) {
  if (n_el <= 0) return;
  k_gen_lobatto<<<n_el, 256, 0, s>>>(emat, emat_off, p_el, kappa, react, beta, sel_ptr, sel, ref, ref_off, dim,
                                     hh, cmass, cconv);
}

}  // namespace uhm_gpu
