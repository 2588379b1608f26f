// Learned per-front precision selector: shapes and device entry points.
#pragma once

#include <cstdint>
#include <cuda_runtime.h>

namespace uhm_gpu {

constexpr int SEL_F = 12;    // features per front
constexpr int SEL_H = 64;    // hidden width (two hidden layers)
constexpr int SEL_C = 3;     // classes: 0 FP64, 1 FP32, 2 BF16-split
constexpr int SEL_NPARAMS = SEL_H * SEL_F + SEL_H + SEL_H * SEL_H + SEL_H + SEL_C * SEL_H + SEL_C;

// per-sample activations of one minibatch (device, B x SEL_H or B x SEL_C)
struct SelectorWork {
  float *H1 = nullptr, *H2 = nullptr, *dZ = nullptr, *dH1 = nullptr, *dH2 = nullptr;
};

void launch_elem_stats(const double* emat, const int64_t* off, const int* msz, int n_el, float* out,
                       cudaStream_t s);
void launch_mlp_infer(const float* X, int N, const float* params, int* cls, float* prob, cudaStream_t s);
// loss and parameter gradient of the class-weighted mean cross-entropy over
// the samples idx[0..B) (idx == nullptr: samples 0..B)
void launch_mlp_grad(const float* X, const int* Y, const float* wc, const int* idx, int B, const float* params,
                     SelectorWork& w, float* grad, float* loss, cudaStream_t s);
void launch_adam(float* params, const float* grad, float* m, float* v, float lr, int t, cudaStream_t s);

}  // namespace uhm_gpu
