// Learned tile cost model: a 12 -> 64 -> 32 -> 1 ReLU MLP (the reference's
// PyTorchMLP, my_cost_model.py:1010-1029, has the same 64 / 32 hidden
// widths over 18 features) that predicts the log of an ELL tile's cost per
// wave from standardised tile features.  Inference scores every candidate
// of a search step in one launch; training runs on the GPU with the
// kernels below (per-sample forward / backward, weight-gradient reduction,
// Adam), so the network learns from timings of this package's own kernels.
//
// Parameter layout (floats): W1 [12][64], b1 [64], W2 [64][32], b2 [32],
// W3 [32], b3.
#include <cuda_runtime.h>
#include <stdint.h>

#include "../../include/stile_gb300.h"
#include "spmm.cuh"

namespace stile {

constexpr int kIn = STILE_MLP_FEATURES, kH1 = 64, kH2 = 32;
constexpr int kW1 = 0, kB1 = kW1 + kIn * kH1, kW2 = kB1 + kH1, kB2 = kW2 + kH1 * kH2, kW3 = kB2 + kH2,
              kB3 = kW3 + kH2, kParams = kB3 + 1;
static_assert(kParams == STILE_MLP_PARAMS, "parameter count");
// per-sample work record of the backward pass: h1 | h2 | dh1 | dh2
constexpr int kOffH1 = 0, kOffH2 = kH1, kOffDh1 = kH1 + kH2, kOffDh2 = 2 * kH1 + kH2;
constexpr int kWork = 2 * kH1 + 2 * kH2;

__device__ __forceinline__ void load_params(const float* __restrict__ params, float* sp) {
  for (int i = threadIdx.x; i < kParams; i += blockDim.x) sp[i] = __ldg(params + i);
  __syncthreads();
}

// forward of one sample; h1 / h2 are the post-ReLU activations
__device__ __forceinline__ float mlp_forward_one(const float* sp, const float* __restrict__ x, float (&h1)[kH1],
                                                 float (&h2)[kH2]) {
  float xi[kIn];
#pragma unroll
  for (int k = 0; k < kIn; ++k) xi[k] = __ldg(x + k);
#pragma unroll
  for (int j = 0; j < kH1; ++j) {
    float a = sp[kB1 + j];
#pragma unroll
    for (int k = 0; k < kIn; ++k) a = fmaf(xi[k], sp[kW1 + k * kH1 + j], a);
    h1[j] = fmaxf(a, 0.f);
  }
#pragma unroll
  for (int j = 0; j < kH2; ++j) {
    float a = sp[kB2 + j];
#pragma unroll
    for (int i = 0; i < kH1; ++i) a = fmaf(h1[i], sp[kW2 + i * kH2 + j], a);
    h2[j] = fmaxf(a, 0.f);
  }
  float y = sp[kB3];
#pragma unroll
  for (int j = 0; j < kH2; ++j) y = fmaf(h2[j], sp[kW3 + j], y);
  return y;
}

__global__ void __launch_bounds__(128) mlp_forward_kernel(const float* __restrict__ params,
                                                          const float* __restrict__ x, long n,
                                                          float* __restrict__ y) {
  __shared__ float sp[kParams];
  load_params(params, sp);
  const long s = (long)blockIdx.x * blockDim.x + threadIdx.x;
  if (s >= n) return;
  float h1[kH1], h2[kH2];
  y[s] = mlp_forward_one(sp, x + s * kIn, h1, h2);
}

// Loss = sum_s (y_s - t_s)^2 / n.  Per sample: forward, then the
// back-propagated signals dh2 = dL/d(pre-activation 2) and dh1 = dL/d(pre-
// activation 1); the activations and signals go to the work record for the
// weight-gradient reduction.  dy_s = 2 (y_s - t_s) / n lands in dy.
__global__ void __launch_bounds__(128) mlp_backward_kernel(const float* __restrict__ params,
                                                           const float* __restrict__ x,
                                                           const float* __restrict__ t, long n,
                                                           float* __restrict__ work, float* __restrict__ dy_out,
                                                           float* __restrict__ loss) {
  __shared__ float sp[kParams];
  __shared__ float block_loss;
  if (threadIdx.x == 0) block_loss = 0.f;
  load_params(params, sp);
  const long s = (long)blockIdx.x * blockDim.x + threadIdx.x;
  if (s < n) {
    float h1[kH1], h2[kH2];
    const float y = mlp_forward_one(sp, x + s * kIn, h1, h2);
    const float d = y - __ldg(t + s);
    atomicAdd(&block_loss, d * d / (float)n);
    const float dy = 2.f * d / (float)n;
    dy_out[s] = dy;
    float* w = work + s * kWork;
    float dh2[kH2];
#pragma unroll
    for (int j = 0; j < kH2; ++j) dh2[j] = h2[j] > 0.f ? dy * sp[kW3 + j] : 0.f;
#pragma unroll
    for (int i = 0; i < kH1; ++i) {
      float a = 0.f;
#pragma unroll
      for (int j = 0; j < kH2; ++j) a = fmaf(dh2[j], sp[kW2 + i * kH2 + j], a);
      w[kOffDh1 + i] = h1[i] > 0.f ? a : 0.f;
      w[kOffH1 + i] = h1[i];
    }
#pragma unroll
    for (int j = 0; j < kH2; ++j) {
      w[kOffH2 + j] = h2[j];
      w[kOffDh2 + j] = dh2[j];
    }
  }
  __syncthreads();
  if (threadIdx.x == 0) atomicAdd(loss, block_loss);
}

// One thread per parameter: sum over the samples of the parameter's
// per-sample gradient (a deterministic order, no atomics).
__global__ void mlp_weight_grad_kernel(const float* __restrict__ x, const float* __restrict__ work,
                                       const float* __restrict__ dy, long n, float* __restrict__ grad) {
  const int p = blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= kParams) return;
  float g = 0.f;
  if (p < kB1) {  // W1[k][j]: x_k * dh1_j
    const int k = p / kH1, j = p % kH1;
    for (long s = 0; s < n; ++s) g = fmaf(__ldg(x + s * kIn + k), __ldg(work + s * kWork + kOffDh1 + j), g);
  } else if (p < kW2) {  // b1[j]: dh1_j
    const int j = p - kB1;
    for (long s = 0; s < n; ++s) g += __ldg(work + s * kWork + kOffDh1 + j);
  } else if (p < kB2) {  // W2[i][j]: h1_i * dh2_j
    const int i = (p - kW2) / kH2, j = (p - kW2) % kH2;
    for (long s = 0; s < n; ++s)
      g = fmaf(__ldg(work + s * kWork + kOffH1 + i), __ldg(work + s * kWork + kOffDh2 + j), g);
  } else if (p < kW3) {  // b2[j]: dh2_j
    const int j = p - kB2;
    for (long s = 0; s < n; ++s) g += __ldg(work + s * kWork + kOffDh2 + j);
  } else if (p < kB3) {  // W3[j]: h2_j * dy
    const int j = p - kW3;
    for (long s = 0; s < n; ++s) g = fmaf(__ldg(work + s * kWork + kOffH2 + j), __ldg(dy + s), g);
  } else {  // b3: dy
    for (long s = 0; s < n; ++s) g += __ldg(dy + s);
  }
  grad[p] = g;
}

__global__ void mlp_adam_kernel(float* __restrict__ params, const float* __restrict__ grad, float* __restrict__ m,
                                float* __restrict__ v, long count, float lr, float b1, float b2, float eps,
                                float c1, float c2) {
  const long i = (long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= count) return;
  const float g = grad[i];
  const float mi = b1 * m[i] + (1.f - b1) * g;
  const float vi = b2 * v[i] + (1.f - b2) * g * g;
  m[i] = mi;
  v[i] = vi;
  params[i] -= lr * (mi / c1) / (sqrtf(vi / c2) + eps);
}

}  // namespace stile

extern "C" {

int stile_mlp_forward(const float* params, const float* x, int64_t n, float* y, void* stream) {
  if (n < 0 || (n > 0 && (!params || !x || !y))) return stile::report_error(STILE_E_INVALID, "bad MLP forward arguments");
  if (n == 0) return STILE_OK;
  stile::mlp_forward_kernel<<<(unsigned)((n + 127) / 128), 128, 0, static_cast<cudaStream_t>(stream)>>>(params, x, n, y);
  const cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return stile::report_error(STILE_E_CUDA, cudaGetErrorString(e));
  stile::note_launches(1);
  return STILE_OK;
}

int stile_mlp_gradient(const float* params, const float* x, const float* t, int64_t n, float* work, float* dy,
                       float* grad, float* loss, void* stream) {
  if (n <= 0 || !params || !x || !t || !work || !dy || !grad || !loss)
    return stile::report_error(STILE_E_INVALID, "bad MLP gradient arguments");
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  cudaError_t e = cudaMemsetAsync(loss, 0, sizeof(float), st);
  if (e != cudaSuccess) return stile::report_error(STILE_E_CUDA, cudaGetErrorString(e));
  stile::mlp_backward_kernel<<<(unsigned)((n + 127) / 128), 128, 0, st>>>(params, x, t, n, work, dy, loss);
  stile::mlp_weight_grad_kernel<<<(stile::kParams + 127) / 128, 128, 0, st>>>(x, work, dy, n, grad);
  e = cudaGetLastError();
  if (e != cudaSuccess) return stile::report_error(STILE_E_CUDA, cudaGetErrorString(e));
  stile::note_launches(2);
  return STILE_OK;
}

int stile_mlp_adam(float* params, const float* grad, float* m, float* v, int64_t count, float lr, float beta1,
                   float beta2, float eps, int32_t step, void* stream) {
  if (count <= 0 || !params || !grad || !m || !v || step < 1)
    return stile::report_error(STILE_E_INVALID, "bad Adam arguments");
  const float c1 = 1.f - powf(beta1, (float)step), c2 = 1.f - powf(beta2, (float)step);
  stile::mlp_adam_kernel<<<(unsigned)((count + 255) / 256), 256, 0, static_cast<cudaStream_t>(stream)>>>(
      params, grad, m, v, count, lr, beta1, beta2, eps, c1, c2);
  const cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return stile::report_error(STILE_E_CUDA, cudaGetErrorString(e));
  stile::note_launches(1);
  return STILE_OK;
}

}  // extern "C"
