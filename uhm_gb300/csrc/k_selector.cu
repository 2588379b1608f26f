// Learned per-front precision selector: element statistics for its features,
// and a 12 -> 64 -> 64 -> 3 MLP (ReLU, softmax) with hand-written inference,
// training (forward, backward, Adam) kernels.
//
// Classes: 0 = FP64 front, 1 = FP32 front, 2 = BF16-split front (tensor-core
// Schur update where the front is large enough, FP32 elsewhere).
//
// Parameter layout (floats): W1[64][12], b1[64], W2[64][64], b2[64],
// W3[3][64], b3[3]; weights row-major (output, input).
#include <cuda_runtime.h>

#include <cmath>
#include <cstdint>
#include <vector>

#include "selector.hpp"

namespace uhm_gpu {

namespace {

constexpr int OFF_W1 = 0, OFF_B1 = OFF_W1 + SEL_H * SEL_F, OFF_W2 = OFF_B1 + SEL_H,
              OFF_B2 = OFF_W2 + SEL_H * SEL_H, OFF_W3 = OFF_B2 + SEL_H, OFF_B3 = OFF_W3 + SEL_C * SEL_H;
static_assert(OFF_B3 + SEL_C == SEL_NPARAMS, "parameter layout");

// ---------------------------------------------------------------------------
// per-element statistics: one block per element matrix (m x m, column-major)
//   out[4e + 0] = mean |a_jj|
//   out[4e + 1] = sum a_ij / sum |a_ij|            (signed mass of the matrix)
//   out[4e + 2] = min_j (|a_jj| - sum_{i!=j} |a_ij|) / |a_jj|   (column dominance)
//   out[4e + 3] = mean_j of the same ratio
// ---------------------------------------------------------------------------
__global__ void __launch_bounds__(128) k_elem_stats(const double* __restrict__ emat, const int64_t* __restrict__ off,
                                                    const int* __restrict__ msz, int n_el, float* __restrict__ out) {
  const int e = blockIdx.x;
  if (e >= n_el) return;
  const int m = msz[e];
  const double* A = emat + off[e];
  double s_sum = 0, s_abs = 0, d_sum = 0, dom_sum = 0, dom_min = 1e300;
  for (int j = threadIdx.x; j < m; j += blockDim.x) {
    double cs = 0, ca = 0;
    for (int i = 0; i < m; ++i) {
      const double v = A[i + (int64_t)j * m];
      cs += v;
      ca += fabs(v);
    }
    const double d = fabs(A[j + (int64_t)j * m]);
    s_sum += cs;
    s_abs += ca;
    d_sum += d;
    const double r = d > 0 ? (2.0 * d - ca) / d : -1e300;
    dom_sum += r;
    dom_min = fmin(dom_min, r);
  }
  __shared__ double sh[5][128];
  sh[0][threadIdx.x] = s_sum;
  sh[1][threadIdx.x] = s_abs;
  sh[2][threadIdx.x] = d_sum;
  sh[3][threadIdx.x] = dom_sum;
  sh[4][threadIdx.x] = dom_min;
  __syncthreads();
  for (int o = 64; o > 0; o >>= 1) {
    if (threadIdx.x < o) {
      for (int q = 0; q < 4; ++q) sh[q][threadIdx.x] += sh[q][threadIdx.x + o];
      sh[4][threadIdx.x] = fmin(sh[4][threadIdx.x], sh[4][threadIdx.x + o]);
    }
    __syncthreads();
  }
  if (threadIdx.x == 0) {
    const double mm = m > 0 ? m : 1;
    out[4 * e + 0] = (float)(sh[2][0] / mm);
    out[4 * e + 1] = (float)(sh[1][0] > 0 ? sh[0][0] / sh[1][0] : 0.0);
    out[4 * e + 2] = (float)fmax(-1e30, sh[4][0]);
    out[4 * e + 3] = (float)(sh[3][0] / mm);
  }
}

// ---------------------------------------------------------------------------
// MLP
// ---------------------------------------------------------------------------
__device__ __forceinline__ void mlp_forward_one(const float* __restrict__ P, const float* x, float* h1, float* h2,
                                                float* z) {
  for (int j = 0; j < SEL_H; ++j) {
    float s = P[OFF_B1 + j];
#pragma unroll
    for (int k = 0; k < SEL_F; ++k) s += P[OFF_W1 + j * SEL_F + k] * x[k];
    h1[j] = s > 0.f ? s : 0.f;
  }
  for (int j = 0; j < SEL_H; ++j) {
    float s = P[OFF_B2 + j];
    for (int k = 0; k < SEL_H; ++k) s += P[OFF_W2 + j * SEL_H + k] * h1[k];
    h2[j] = s > 0.f ? s : 0.f;
  }
  for (int c = 0; c < SEL_C; ++c) {
    float s = P[OFF_B3 + c];
    for (int k = 0; k < SEL_H; ++k) s += P[OFF_W3 + c * SEL_H + k] * h2[k];
    z[c] = s;
  }
}

// inference: one thread per sample, parameters staged in shared memory
__global__ void __launch_bounds__(128) k_mlp_infer(const float* __restrict__ X, int N, const float* __restrict__ params,
                                                   int* __restrict__ cls, float* __restrict__ prob) {
  __shared__ float P[SEL_NPARAMS];
  for (int i = threadIdx.x; i < SEL_NPARAMS; i += blockDim.x) P[i] = params[i];
  __syncthreads();
  const int s = blockIdx.x * blockDim.x + threadIdx.x;
  if (s >= N) return;
  float x[SEL_F], h1[SEL_H], h2[SEL_H], z[SEL_C];
#pragma unroll
  for (int k = 0; k < SEL_F; ++k) x[k] = X[(int64_t)s * SEL_F + k];
  mlp_forward_one(P, x, h1, h2, z);
  float zm = z[0];
  int best = 0;
  for (int c = 1; c < SEL_C; ++c)
    if (z[c] > zm) { zm = z[c]; best = c; }
  float den = 0.f;
  for (int c = 0; c < SEL_C; ++c) den += __expf(z[c] - zm);
  if (cls) cls[s] = best;
  if (prob)
    for (int c = 0; c < SEL_C; ++c) prob[(int64_t)s * SEL_C + c] = __expf(z[c] - zm) / den;
}

// training forward + activation gradients for a minibatch (one thread per sample)
//   loss = (1/B) sum_b w[y_b] * (-log softmax(z_b)[y_b])
__global__ void __launch_bounds__(128) k_mlp_fwd_bwd(const float* __restrict__ X, const int* __restrict__ Y,
                                                     const float* __restrict__ wc, const int* __restrict__ idx, int B,
                                                     const float* __restrict__ params, float* __restrict__ H1,
                                                     float* __restrict__ H2, float* __restrict__ dZ,
                                                     float* __restrict__ dH1, float* __restrict__ dH2,
                                                     float* __restrict__ loss) {
  __shared__ float P[SEL_NPARAMS];
  for (int i = threadIdx.x; i < SEL_NPARAMS; i += blockDim.x) P[i] = params[i];
  __syncthreads();
  const int b = blockIdx.x * blockDim.x + threadIdx.x;
  if (b >= B) return;
  const int s = idx ? idx[b] : b;
  float x[SEL_F], h1[SEL_H], h2[SEL_H], z[SEL_C];
#pragma unroll
  for (int k = 0; k < SEL_F; ++k) x[k] = X[(int64_t)s * SEL_F + k];
  mlp_forward_one(P, x, h1, h2, z);
  const int y = Y[s];
  const float w = wc ? wc[y] : 1.f;
  float zm = z[0];
  for (int c = 1; c < SEL_C; ++c) zm = fmaxf(zm, z[c]);
  float den = 0.f;
  for (int c = 0; c < SEL_C; ++c) den += expf(z[c] - zm);
  const float lse = zm + logf(den);
  atomicAdd(loss, w * (lse - z[y]) / B);
  float dz[SEL_C];
  for (int c = 0; c < SEL_C; ++c) dz[c] = w * (expf(z[c] - lse) - (c == y ? 1.f : 0.f)) / B;
  float dh2[SEL_H];
  for (int k = 0; k < SEL_H; ++k) {
    float s2 = 0.f;
    for (int c = 0; c < SEL_C; ++c) s2 += P[OFF_W3 + c * SEL_H + k] * dz[c];
    dh2[k] = h2[k] > 0.f ? s2 : 0.f;
  }
  for (int k = 0; k < SEL_H; ++k) {
    float s1 = 0.f;
    for (int j = 0; j < SEL_H; ++j) s1 += P[OFF_W2 + j * SEL_H + k] * dh2[j];
    dH1[(int64_t)b * SEL_H + k] = h1[k] > 0.f ? s1 : 0.f;
    H1[(int64_t)b * SEL_H + k] = h1[k];
    H2[(int64_t)b * SEL_H + k] = h2[k];
    dH2[(int64_t)b * SEL_H + k] = dh2[k];
  }
  for (int c = 0; c < SEL_C; ++c) dZ[(int64_t)b * SEL_C + c] = dz[c];
}

// parameter gradients: one thread per parameter, summed over the batch in order
__global__ void __launch_bounds__(256) k_mlp_wgrad(const float* __restrict__ X, const int* __restrict__ idx, int B,
                                                   const float* __restrict__ H1, const float* __restrict__ H2,
                                                   const float* __restrict__ dZ, const float* __restrict__ dH1,
                                                   const float* __restrict__ dH2, float* __restrict__ grad) {
  const int p = blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= SEL_NPARAMS) return;
  float g = 0.f;
  if (p < OFF_B1) {
    const int j = p / SEL_F, k = p % SEL_F;
    for (int b = 0; b < B; ++b) {
      const int s = idx ? idx[b] : b;
      g += dH1[(int64_t)b * SEL_H + j] * X[(int64_t)s * SEL_F + k];
    }
  } else if (p < OFF_W2) {
    const int j = p - OFF_B1;
    for (int b = 0; b < B; ++b) g += dH1[(int64_t)b * SEL_H + j];
  } else if (p < OFF_B2) {
    const int j = (p - OFF_W2) / SEL_H, k = (p - OFF_W2) % SEL_H;
    for (int b = 0; b < B; ++b) g += dH2[(int64_t)b * SEL_H + j] * H1[(int64_t)b * SEL_H + k];
  } else if (p < OFF_W3) {
    const int j = p - OFF_B2;
    for (int b = 0; b < B; ++b) g += dH2[(int64_t)b * SEL_H + j];
  } else if (p < OFF_B3) {
    const int c = (p - OFF_W3) / SEL_H, k = (p - OFF_W3) % SEL_H;
    for (int b = 0; b < B; ++b) g += dZ[(int64_t)b * SEL_C + c] * H2[(int64_t)b * SEL_H + k];
  } else {
    const int c = p - OFF_B3;
    for (int b = 0; b < B; ++b) g += dZ[(int64_t)b * SEL_C + c];
  }
  grad[p] = g;
}

__global__ void k_adam(float* __restrict__ P, const float* __restrict__ g, float* __restrict__ m,
                       float* __restrict__ v, int n, float lr, float b1, float b2, float eps, float c1, float c2) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const float gi = g[i];
  const float mi = b1 * m[i] + (1.f - b1) * gi;
  const float vi = b2 * v[i] + (1.f - b2) * gi * gi;
  m[i] = mi;
  v[i] = vi;
  P[i] -= lr * (mi / c1) / (sqrtf(vi / c2) + eps);
}

}  // namespace

// ---------------------------------------------------------------------------
// launchers
// ---------------------------------------------------------------------------
void launch_elem_stats(const double* emat, const int64_t* off, const int* msz, int n_el, float* out,
                       cudaStream_t s) {
  if (n_el > 0) k_elem_stats<<<n_el, 128, 0, s>>>(emat, off, msz, n_el, out);
}

void launch_mlp_infer(const float* X, int N, const float* params, int* cls, float* prob, cudaStream_t s) {
  if (N > 0) k_mlp_infer<<<(N + 127) / 128, 128, 0, s>>>(X, N, params, cls, prob);
}

void launch_mlp_grad(const float* X, const int* Y, const float* wc, const int* idx, int B, const float* params,
                     SelectorWork& w, float* grad, float* loss, cudaStream_t s) {
  cudaMemsetAsync(loss, 0, sizeof(float), s);
  k_mlp_fwd_bwd<<<(B + 127) / 128, 128, 0, s>>>(X, Y, wc, idx, B, params, w.H1, w.H2, w.dZ, w.dH1, w.dH2, loss);
  k_mlp_wgrad<<<(SEL_NPARAMS + 255) / 256, 256, 0, s>>>(X, idx, B, w.H1, w.H2, w.dZ, w.dH1, w.dH2, grad);
}

void launch_adam(float* params, const float* grad, float* m, float* v, float lr, int t, cudaStream_t s) {
  const float b1 = 0.9f, b2 = 0.999f, eps = 1e-8f;
  const float c1 = 1.f - powf(b1, (float)t), c2 = 1.f - powf(b2, (float)t);
  k_adam<<<(SEL_NPARAMS + 255) / 256, 256, 0, s>>>(params, grad, m, v, SEL_NPARAMS, lr, b1, b2, eps, c1, c2);
}

}  // namespace uhm_gpu

// ---------------------------------------------------------------------------
// C ABI for training and inference on caller-supplied samples (host arrays)
// ---------------------------------------------------------------------------
namespace {

template <typename T>
T* dev_copy(const T* h, size_t n, cudaError_t& err) {
  T* d = nullptr;
  if (err == cudaSuccess) err = cudaMalloc(&d, sizeof(T) * (n ? n : 1));
  if (err == cudaSuccess && h && n) err = cudaMemcpy(d, h, sizeof(T) * n, cudaMemcpyHostToDevice);
  return d;
}

struct DevBufs {
  std::vector<void*> ptrs;
  ~DevBufs() {
    for (void* p : ptrs) cudaFree(p);
  }
  template <typename T>
  T* add(T* p) {
    ptrs.push_back(p);
    return p;
  }
};

int alloc_work(uhm_gpu::SelectorWork& w, int B, DevBufs& keep) {
  cudaError_t e = cudaSuccess;
  w.H1 = keep.add(dev_copy<float>(nullptr, (size_t)B * uhm_gpu::SEL_H, e));
  w.H2 = keep.add(dev_copy<float>(nullptr, (size_t)B * uhm_gpu::SEL_H, e));
  w.dH1 = keep.add(dev_copy<float>(nullptr, (size_t)B * uhm_gpu::SEL_H, e));
  w.dH2 = keep.add(dev_copy<float>(nullptr, (size_t)B * uhm_gpu::SEL_H, e));
  w.dZ = keep.add(dev_copy<float>(nullptr, (size_t)B * uhm_gpu::SEL_C, e));
  return e == cudaSuccess ? 0 : 4;
}

uint64_t splitmix(uint64_t& s) {
  uint64_t z = (s += 0x9E3779B97F4A7C15ull);
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
  return z ^ (z >> 31);
}

}  // namespace

extern "C" {

int uhm_gpu_mlp_n_params(void) { return uhm_gpu::SEL_NPARAMS; }
int uhm_gpu_mlp_n_features(void) { return uhm_gpu::SEL_F; }

int uhm_gpu_mlp_predict(const float* X, int N, const float* params, int* cls, float* prob) {
  if (N < 0 || !params || (N > 0 && !X)) return 7;
  if (N == 0) return 0;
  DevBufs keep;
  cudaError_t e = cudaSuccess;
  float* dX = keep.add(dev_copy(X, (size_t)N * uhm_gpu::SEL_F, e));
  float* dP = keep.add(dev_copy(params, (size_t)uhm_gpu::SEL_NPARAMS, e));
  int* dC = keep.add(dev_copy<int>(nullptr, (size_t)N, e));
  float* dPr = keep.add(dev_copy<float>(nullptr, (size_t)N * uhm_gpu::SEL_C, e));
  if (e != cudaSuccess) return 4;
  uhm_gpu::launch_mlp_infer(dX, N, dP, dC, dPr, 0);
  if (cudaGetLastError() != cudaSuccess) return 7;
  if (cls && cudaMemcpy(cls, dC, sizeof(int) * N, cudaMemcpyDeviceToHost) != cudaSuccess) return 7;
  if (prob && cudaMemcpy(prob, dPr, sizeof(float) * N * uhm_gpu::SEL_C, cudaMemcpyDeviceToHost) != cudaSuccess)
    return 7;
  return 0;
}

// loss and gradient over all N samples (one batch), for checking the kernels
int uhm_gpu_mlp_gradient(const float* X, const int* Y, const float* wc, int N, const float* params, float* grad,
                         float* loss) {
  if (N <= 0 || !X || !Y || !params || !grad || !loss) return 7;
  DevBufs keep;
  cudaError_t e = cudaSuccess;
  float* dX = keep.add(dev_copy(X, (size_t)N * uhm_gpu::SEL_F, e));
  int* dY = keep.add(dev_copy(Y, (size_t)N, e));
  float* dW = wc ? keep.add(dev_copy(wc, (size_t)uhm_gpu::SEL_C, e)) : nullptr;
  float* dP = keep.add(dev_copy(params, (size_t)uhm_gpu::SEL_NPARAMS, e));
  float* dG = keep.add(dev_copy<float>(nullptr, (size_t)uhm_gpu::SEL_NPARAMS, e));
  float* dL = keep.add(dev_copy<float>(nullptr, 1, e));
  if (e != cudaSuccess) return 4;
  uhm_gpu::SelectorWork w;
  if (alloc_work(w, N, keep)) return 4;
  uhm_gpu::launch_mlp_grad(dX, dY, dW, nullptr, N, dP, w, dG, dL, 0);
  if (cudaGetLastError() != cudaSuccess) return 7;
  if (cudaMemcpy(grad, dG, sizeof(float) * uhm_gpu::SEL_NPARAMS, cudaMemcpyDeviceToHost) != cudaSuccess) return 7;
  if (cudaMemcpy(loss, dL, sizeof(float), cudaMemcpyDeviceToHost) != cudaSuccess) return 7;
  return 0;
}

// Adam on shuffled minibatches; params updated in place; loss_hist[epoch] =
// mean minibatch loss of that epoch
int uhm_gpu_mlp_train(const float* X, const int* Y, const float* wc, int N, float* params, int epochs, int batch,
                      float lr, unsigned long long seed, float* loss_hist) {
  if (N <= 0 || !X || !Y || !params || epochs < 0 || batch <= 0) return 7;
  const int B = batch < N ? batch : N;
  const int nb = N / B;
  DevBufs keep;
  cudaError_t e = cudaSuccess;
  float* dX = keep.add(dev_copy(X, (size_t)N * uhm_gpu::SEL_F, e));
  int* dY = keep.add(dev_copy(Y, (size_t)N, e));
  float* dW = wc ? keep.add(dev_copy(wc, (size_t)uhm_gpu::SEL_C, e)) : nullptr;
  float* dP = keep.add(dev_copy(params, (size_t)uhm_gpu::SEL_NPARAMS, e));
  float* dG = keep.add(dev_copy<float>(nullptr, (size_t)uhm_gpu::SEL_NPARAMS, e));
  std::vector<float> zeros(uhm_gpu::SEL_NPARAMS, 0.f);
  float* dM = keep.add(dev_copy(zeros.data(), zeros.size(), e));
  float* dV = keep.add(dev_copy(zeros.data(), zeros.size(), e));
  float* dL = keep.add(dev_copy<float>(nullptr, (size_t)nb, e));
  int* dI = keep.add(dev_copy<int>(nullptr, (size_t)N, e));
  if (e != cudaSuccess) return 4;
  uhm_gpu::SelectorWork w;
  if (alloc_work(w, B, keep)) return 4;
  std::vector<int> perm(N);
  std::vector<float> lb(nb);
  uint64_t st = seed;
  int t = 0;
  for (int ep = 0; ep < epochs; ++ep) {
    for (int i = 0; i < N; ++i) perm[i] = i;
    for (int i = N - 1; i > 0; --i) {
      const int j = (int)(splitmix(st) % (uint64_t)(i + 1));
      const int tmp = perm[i];
      perm[i] = perm[j];
      perm[j] = tmp;
    }
    if (cudaMemcpy(dI, perm.data(), sizeof(int) * N, cudaMemcpyHostToDevice) != cudaSuccess) return 7;
    for (int b = 0; b < nb; ++b) {
      uhm_gpu::launch_mlp_grad(dX, dY, dW, dI + (size_t)b * B, B, dP, w, dG, dL + b, 0);
      uhm_gpu::launch_adam(dP, dG, dM, dV, lr, ++t, 0);
    }
    if (cudaGetLastError() != cudaSuccess) return 7;
    if (cudaMemcpy(lb.data(), dL, sizeof(float) * nb, cudaMemcpyDeviceToHost) != cudaSuccess) return 7;
    double s = 0;
    for (float v : lb) s += v;
    if (loss_hist) loss_hist[ep] = (float)(s / (nb ? nb : 1));
  }
  if (cudaMemcpy(params, dP, sizeof(float) * uhm_gpu::SEL_NPARAMS, cudaMemcpyDeviceToHost) != cudaSuccess) return 7;
  return 0;
}

}  // extern "C"
