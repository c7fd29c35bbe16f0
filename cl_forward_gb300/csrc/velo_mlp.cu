// velo_mlp.cu -- the doublet scorer: a 10 -> 32 -> 32 -> 2 ReLU MLP trained in
// FP32 with hand-written forward / backward / Adam kernels; inference
// (velo_mlp_forward and the learned seeding) runs in FP16 on the tensor cores
// (velo_mlp_warp.cuh).
//
// Outputs per (h0, h1) doublet: a keep logit and the half-width (mm) of the
// x window around the straight-line prediction at module f-4 in which the
// doublet's h2 lies.  Loss per sample: binary cross-entropy of the logit
// against the label (1 = the plain seeding chose this doublet for h0 and its
// tracklet survived into an output track) plus, for positives only,
// kWidthWeight * (width - target)^2.
//
// Parameters are one flat FP32 array of VELO_MLP_PARAMS values:
//   W1[32][10] b1[32] W2[32][32] b2[32] W3[2][32] b3[2]
// (row-major, out x in).
#include <cuda_runtime.h>
#include <math.h>

#include <cstring>
#include <vector>

#include "velo_internal.h"
#include "velo_mlp_warp.cuh"

namespace velo {

constexpr float kWidthWeight = 0.1f;
constexpr int kTrainThreads = 128;

// forward pass of one sample; keeps the hidden activations for backward
__device__ __forceinline__ void mlp_forward_sample(const float* __restrict__ w, const float* x, float* a1,
                                                   float* a2, float* out) {
  const float* W1 = w + kMlpW1;
  const float* b1 = w + kMlpB1;
  const float* W2 = w + kMlpW2;
  const float* b2 = w + kMlpB2;
  const float* W3 = w + kMlpW3;
  const float* b3 = w + kMlpB3;
#pragma unroll 4
  for (int j = 0; j < kMlpHidden; ++j) {
    float s = b1[j];
#pragma unroll
    for (int i = 0; i < kMlpIn; ++i) s += W1[j * kMlpIn + i] * x[i];
    a1[j] = s > 0.f ? s : 0.f;
  }
#pragma unroll 4
  for (int j = 0; j < kMlpHidden; ++j) {
    float s = b2[j];
#pragma unroll 8
    for (int i = 0; i < kMlpHidden; ++i) s += W2[j * kMlpHidden + i] * a1[i];
    a2[j] = s > 0.f ? s : 0.f;
  }
#pragma unroll
  for (int k = 0; k < kMlpOut; ++k) {
    float s = b3[k];
#pragma unroll 8
    for (int i = 0; i < kMlpHidden; ++i) s += W3[k * kMlpHidden + i] * a2[i];
    out[k] = s;
  }
}

// BCE-with-logits (stable form) + masked squared width error
__device__ __forceinline__ float sample_loss(const float* out, float label, float target, float* dz, float* dw) {
  const float z = out[0];
  const float p = 1.f / (1.f + expf(-z));
  const float bce = fmaxf(z, 0.f) - z * label + log1pf(expf(-fabsf(z)));
  *dz = p - label;
  const float e = out[1] - target;
  *dw = label * 2.f * kWidthWeight * e;
  return bce + label * kWidthWeight * e * e;
}

// One CTA: forward + backward for kTrainThreads samples, gradients summed in
// shared memory, then added to the global gradient (scaled by 1/n_batch).
__global__ void __launch_bounds__(kTrainThreads) mlp_grad_kernel(const float* __restrict__ w,
                                                                 const float* __restrict__ x,
                                                                 const float* __restrict__ label,
                                                                 const float* __restrict__ target,
                                                                 const int64_t* __restrict__ index, int64_t n,
                                                                 float scale, float* __restrict__ grad,
                                                                 float* __restrict__ loss_sum) {
  __shared__ float sw[VELO_MLP_PARAMS];
  __shared__ float sg[VELO_MLP_PARAMS];
  __shared__ float sloss;
  for (int i = threadIdx.x; i < VELO_MLP_PARAMS; i += blockDim.x) {
    sw[i] = w[i];
    sg[i] = 0.f;
  }
  if (threadIdx.x == 0) sloss = 0.f;
  __syncthreads();
  const int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (k < n) {
    const int64_t r = index ? index[k] : k;
    float xi[kMlpIn], a1[kMlpHidden], a2[kMlpHidden], out[kMlpOut];
#pragma unroll
    for (int i = 0; i < kMlpIn; ++i) xi[i] = x[r * kMlpIn + i];
    mlp_forward_sample(sw, xi, a1, a2, out);
    float dz, dw;
    const float l = sample_loss(out, label[r], target[r], &dz, &dw);
    atomicAdd(&sloss, l * scale);
    const float d3[kMlpOut] = {dz * scale, dw * scale};
    // layer 3
    float d2[kMlpHidden];
#pragma unroll 8
    for (int i = 0; i < kMlpHidden; ++i) d2[i] = 0.f;
#pragma unroll
    for (int o = 0; o < kMlpOut; ++o) {
      atomicAdd(&sg[kMlpB3 + o], d3[o]);
      for (int i = 0; i < kMlpHidden; ++i) {
        atomicAdd(&sg[kMlpW3 + o * kMlpHidden + i], d3[o] * a2[i]);
        d2[i] += sw[kMlpW3 + o * kMlpHidden + i] * d3[o];
      }
    }
    // layer 2
    float d1[kMlpHidden];
#pragma unroll 8
    for (int i = 0; i < kMlpHidden; ++i) d1[i] = 0.f;
    for (int j = 0; j < kMlpHidden; ++j) {
      const float g = a2[j] > 0.f ? d2[j] : 0.f;
      if (g == 0.f) continue;
      atomicAdd(&sg[kMlpB2 + j], g);
      for (int i = 0; i < kMlpHidden; ++i) {
        atomicAdd(&sg[kMlpW2 + j * kMlpHidden + i], g * a1[i]);
        d1[i] += sw[kMlpW2 + j * kMlpHidden + i] * g;
      }
    }
    // layer 1
    for (int j = 0; j < kMlpHidden; ++j) {
      const float g = a1[j] > 0.f ? d1[j] : 0.f;
      if (g == 0.f) continue;
      atomicAdd(&sg[kMlpB1 + j], g);
#pragma unroll
      for (int i = 0; i < kMlpIn; ++i) atomicAdd(&sg[kMlpW1 + j * kMlpIn + i], g * xi[i]);
    }
  }
  __syncthreads();
  for (int i = threadIdx.x; i < VELO_MLP_PARAMS; i += blockDim.x)
    if (sg[i] != 0.f) atomicAdd(&grad[i], sg[i]);
  if (threadIdx.x == 0 && loss_sum) atomicAdd(loss_sum, sloss);
}

// Adam (Kingma & Ba), bias-corrected, one thread per parameter.
__global__ void adam_kernel(float* __restrict__ w, const float* __restrict__ g, float* __restrict__ m,
                            float* __restrict__ v, float lr, float beta1, float beta2, float eps, float c1,
                            float c2) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= VELO_MLP_PARAMS) return;
  const float gi = g[i];
  const float mi = beta1 * m[i] + (1.f - beta1) * gi;
  const float vi = beta2 * v[i] + (1.f - beta2) * gi * gi;
  m[i] = mi;
  v[i] = vi;
  w[i] -= lr * (mi / c1) / (sqrtf(vi / c2) + eps);
}

// Inference as the learned seeding does it (FP16 tensor-core MMA, one warp
// per 32 samples), so the threshold calibrated on its outputs is the one the
// search applies.
__global__ void __launch_bounds__(256) mlp_forward_kernel(const float* __restrict__ w, const float* __restrict__ x,
                                                          int64_t n, float* __restrict__ out) {
  __shared__ MlpFrag frag;
  stage_mlp_fragments(w, &frag);
  __syncthreads();
  const int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;   // whole warps stay in the kernel
  float xi[kMlpIn];
#pragma unroll
  for (int i = 0; i < kMlpIn; ++i) xi[i] = k < n ? x[k * kMlpIn + i] : 0.f;
  float logit, width;
  mlp_eval_warp(frag, xi, &logit, &width);
  if (k < n) {
    out[2 * k] = logit;
    out[2 * k + 1] = width;
  }
}

namespace {

struct DevArrays {
  std::vector<void*> ptrs;
  ~DevArrays() {
    for (void* p : ptrs) cudaFree(p);
  }
  template <typename T>
  cudaError_t alloc(T** p, size_t count) {
    cudaError_t e = cudaMalloc((void**)p, sizeof(T) * (count ? count : 1));
    if (e == cudaSuccess) ptrs.push_back(*p);
    return e;
  }
};

#define MLP_CHECK(call)                      \
  do {                                       \
    cudaError_t e_ = (call);                 \
    if (e_ != cudaSuccess) return VELO_ERR_CUDA; \
  } while (0)

// splitmix64 for the host-side batch sampling
uint64_t mix(uint64_t& s) {
  uint64_t z = (s += 0x9E3779B97F4A7C15ull);
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
  return z ^ (z >> 31);
}

}  // namespace
}  // namespace velo

using namespace velo;

extern "C" velo_status velo_mlp_grad(const float* weights, const float* x, const float* label, const float* target,
                                     int64_t n, float* grad_out, float* loss_out) {
  if (!weights || !x || !label || !target || n <= 0 || !grad_out) return VELO_ERR_INVALID_ARGUMENT;
  DevArrays d;
  float *dw, *dx, *dl, *dt, *dg, *dloss;
  MLP_CHECK(d.alloc(&dw, VELO_MLP_PARAMS));
  MLP_CHECK(d.alloc(&dx, (size_t)n * kMlpIn));
  MLP_CHECK(d.alloc(&dl, (size_t)n));
  MLP_CHECK(d.alloc(&dt, (size_t)n));
  MLP_CHECK(d.alloc(&dg, VELO_MLP_PARAMS));
  MLP_CHECK(d.alloc(&dloss, 1));
  MLP_CHECK(cudaMemcpy(dw, weights, sizeof(float) * VELO_MLP_PARAMS, cudaMemcpyHostToDevice));
  MLP_CHECK(cudaMemcpy(dx, x, sizeof(float) * n * kMlpIn, cudaMemcpyHostToDevice));
  MLP_CHECK(cudaMemcpy(dl, label, sizeof(float) * n, cudaMemcpyHostToDevice));
  MLP_CHECK(cudaMemcpy(dt, target, sizeof(float) * n, cudaMemcpyHostToDevice));
  MLP_CHECK(cudaMemset(dg, 0, sizeof(float) * VELO_MLP_PARAMS));
  MLP_CHECK(cudaMemset(dloss, 0, sizeof(float)));
  const int blocks = (int)((n + kTrainThreads - 1) / kTrainThreads);
  mlp_grad_kernel<<<blocks, kTrainThreads>>>(dw, dx, dl, dt, nullptr, n, 1.f / (float)n, dg, dloss);
  MLP_CHECK(cudaGetLastError());
  MLP_CHECK(cudaMemcpy(grad_out, dg, sizeof(float) * VELO_MLP_PARAMS, cudaMemcpyDeviceToHost));
  if (loss_out) MLP_CHECK(cudaMemcpy(loss_out, dloss, sizeof(float), cudaMemcpyDeviceToHost));
  return VELO_OK;
}

extern "C" velo_status velo_mlp_forward(const float* weights, const float* x, int64_t n, float* out) {
  if (!weights || !x || n <= 0 || !out) return VELO_ERR_INVALID_ARGUMENT;
  DevArrays d;
  float *dw, *dx, *dout;
  MLP_CHECK(d.alloc(&dw, VELO_MLP_PARAMS));
  MLP_CHECK(d.alloc(&dx, (size_t)n * kMlpIn));
  MLP_CHECK(d.alloc(&dout, (size_t)n * 2));
  MLP_CHECK(cudaMemcpy(dw, weights, sizeof(float) * VELO_MLP_PARAMS, cudaMemcpyHostToDevice));
  MLP_CHECK(cudaMemcpy(dx, x, sizeof(float) * n * kMlpIn, cudaMemcpyHostToDevice));
  mlp_forward_kernel<<<(int)((n + 255) / 256), 256>>>(dw, dx, n, dout);
  MLP_CHECK(cudaGetLastError());
  MLP_CHECK(cudaMemcpy(out, dout, sizeof(float) * n * 2, cudaMemcpyDeviceToHost));
  return VELO_OK;
}

extern "C" velo_status velo_mlp_train(const float* x, const float* label, const float* target, int64_t n,
                                      int32_t steps, int32_t batch, float lr, uint64_t seed, float* weights_inout,
                                      float* loss_per_step) {
  if (!x || !label || !target || n <= 0 || steps <= 0 || batch <= 0 || !weights_inout)
    return VELO_ERR_INVALID_ARGUMENT;
  DevArrays d;
  float *dw, *dx, *dl, *dt, *dg, *dm, *dv, *dloss;
  int64_t* didx;
  MLP_CHECK(d.alloc(&dw, VELO_MLP_PARAMS));
  MLP_CHECK(d.alloc(&dx, (size_t)n * kMlpIn));
  MLP_CHECK(d.alloc(&dl, (size_t)n));
  MLP_CHECK(d.alloc(&dt, (size_t)n));
  MLP_CHECK(d.alloc(&dg, VELO_MLP_PARAMS));
  MLP_CHECK(d.alloc(&dm, VELO_MLP_PARAMS));
  MLP_CHECK(d.alloc(&dv, VELO_MLP_PARAMS));
  MLP_CHECK(d.alloc(&dloss, (size_t)steps));
  MLP_CHECK(d.alloc(&didx, (size_t)steps * batch));
  MLP_CHECK(cudaMemcpy(dw, weights_inout, sizeof(float) * VELO_MLP_PARAMS, cudaMemcpyHostToDevice));
  MLP_CHECK(cudaMemcpy(dx, x, sizeof(float) * n * kMlpIn, cudaMemcpyHostToDevice));
  MLP_CHECK(cudaMemcpy(dl, label, sizeof(float) * n, cudaMemcpyHostToDevice));
  MLP_CHECK(cudaMemcpy(dt, target, sizeof(float) * n, cudaMemcpyHostToDevice));
  MLP_CHECK(cudaMemset(dm, 0, sizeof(float) * VELO_MLP_PARAMS));
  MLP_CHECK(cudaMemset(dv, 0, sizeof(float) * VELO_MLP_PARAMS));
  MLP_CHECK(cudaMemset(dloss, 0, sizeof(float) * steps));
  // epoch-wise shuffled sample order
  std::vector<int64_t> order((size_t)n), idx((size_t)steps * batch);
  for (int64_t i = 0; i < n; ++i) order[(size_t)i] = i;
  uint64_t s = seed;
  int64_t pos = n;
  for (size_t k = 0; k < idx.size(); ++k) {
    if (pos == n) {
      for (int64_t i = n - 1; i > 0; --i) std::swap(order[(size_t)i], order[(size_t)(mix(s) % (uint64_t)(i + 1))]);
      pos = 0;
    }
    idx[k] = order[(size_t)pos++];
  }
  MLP_CHECK(cudaMemcpy(didx, idx.data(), sizeof(int64_t) * idx.size(), cudaMemcpyHostToDevice));
  const float beta1 = 0.9f, beta2 = 0.999f, eps = 1e-8f;
  double p1 = 1.0, p2 = 1.0;
  const int blocks = (batch + kTrainThreads - 1) / kTrainThreads;
  for (int32_t t = 0; t < steps; ++t) {
    MLP_CHECK(cudaMemsetAsync(dg, 0, sizeof(float) * VELO_MLP_PARAMS));
    mlp_grad_kernel<<<blocks, kTrainThreads>>>(dw, dx, dl, dt, didx + (size_t)t * batch, batch, 1.f / (float)batch,
                                               dg, dloss + t);
    p1 *= beta1;
    p2 *= beta2;
    adam_kernel<<<(VELO_MLP_PARAMS + 255) / 256, 256>>>(dw, dg, dm, dv, lr, beta1, beta2, eps, (float)(1.0 - p1),
                                                        (float)(1.0 - p2));
  }
  MLP_CHECK(cudaGetLastError());
  MLP_CHECK(cudaMemcpy(weights_inout, dw, sizeof(float) * VELO_MLP_PARAMS, cudaMemcpyDeviceToHost));
  if (loss_per_step) MLP_CHECK(cudaMemcpy(loss_per_step, dloss, sizeof(float) * steps, cudaMemcpyDeviceToHost));
  return VELO_OK;
}
