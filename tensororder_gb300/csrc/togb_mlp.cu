// The learned cost model's network on the GPU: a multilayer perceptron
// F -> H -> H -> 1 with ReLU hidden layers, FP32, trained by mean squared
// error with Adam.  Forward, backward and the update are this file's kernels;
// no library routine is involved.
//
// Parameter layout (one FP32 buffer, `togb_mlp_param_count` entries):
//   W1 [F][H]  b1 [H]  W2 [H][H]  b2 [H]  W3 [H]  b3 [1]
// A layer computes y[b][o] = b[o] + sum_i x[b][i] * W[i][o].
//
// Activations of the forward pass (kept for the backward pass) live in a
// caller buffer of `togb_mlp_scratch_floats(B, H)` floats:
//   A1 [B][H]  A2 [B][H]  Y [B]  dZ2 [B][H]  dZ1 [B][H]  dY [B]
// Weight gradients reduce over the batch in a fixed order (one thread per
// weight), so results are deterministic run to run.
#include <cuda_runtime.h>

#include <cstdint>

#include "togb.h"
#include "togb_internal.h"

namespace togb {
namespace {

constexpr int kT = 256;

int blocks_for(int64_t n) { return (int)((n + kT - 1) / kT); }

// y[b][o] = act(b[o] + sum_i x[b][i] W[i][o]); one thread per output.
__global__ void k_dense_fwd(const float* __restrict__ x, const float* __restrict__ W, const float* __restrict__ bias,
                            float* __restrict__ y, int B, int in, int out, int relu) {
  const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= (int64_t)B * out) return;
  const int b = (int)(t / out), o = (int)(t % out);
  float acc = bias[o];
  const float* xr = x + (int64_t)b * in;
  for (int i = 0; i < in; ++i) acc = fmaf(xr[i], W[(int64_t)i * out + o], acc);
  y[t] = relu ? fmaxf(acc, 0.f) : acc;
}

// dY = 2 (Y - T) / B and the batch loss, summed per block then atomically.
__global__ void k_loss_grad(const float* __restrict__ y, const float* __restrict__ target, float* __restrict__ dy,
                            float* __restrict__ loss, int B) {
  __shared__ float part[kT];
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  float l = 0.f;
  if (t < B) {
    const float d = y[t] - target[t];
    dy[t] = 2.f * d / (float)B;
    l = d * d / (float)B;
  }
  part[threadIdx.x] = l;
  __syncthreads();
  for (int s = kT / 2; s > 0; s >>= 1) {
    if (threadIdx.x < s) part[threadIdx.x] += part[threadIdx.x + s];
    __syncthreads();
  }
  if (threadIdx.x == 0 && loss) atomicAdd(loss, part[0]);
}

// dx[b][i] = (sum_o dz[b][o] W[i][o]) * (a[b][i] > 0): back through a layer
// into the pre-activation gradient of the ReLU layer below it.
__global__ void k_dense_bwd_input(const float* __restrict__ dz, const float* __restrict__ W,
                                  const float* __restrict__ a, float* __restrict__ dx, int B, int in, int out) {
  const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= (int64_t)B * in) return;
  const int b = (int)(t / in), i = (int)(t % in);
  float acc = 0.f;
  const float* dzr = dz + (int64_t)b * out;
  const float* Wr = W + (int64_t)i * out;
  for (int o = 0; o < out; ++o) acc = fmaf(dzr[o], Wr[o], acc);
  dx[t] = a[t] > 0.f ? acc : 0.f;
}

// dW[i][o] = sum_b x[b][i] dz[b][o]; db[o] = sum_b dz[b][o] (threads i == in).
__global__ void k_dense_bwd_weight(const float* __restrict__ x, const float* __restrict__ dz, float* __restrict__ dW,
                                   float* __restrict__ db, int B, int in, int out) {
  const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= (int64_t)(in + 1) * out) return;
  const int i = (int)(t / out), o = (int)(t % out);
  float acc = 0.f;
  if (i < in) {
    for (int b = 0; b < B; ++b) acc = fmaf(x[(int64_t)b * in + i], dz[(int64_t)b * out + o], acc);
    dW[(int64_t)i * out + o] = acc;
  } else {
    for (int b = 0; b < B; ++b) acc += dz[(int64_t)b * out + o];
    db[o] = acc;
  }
}

__global__ void k_adam(float* __restrict__ p, const float* __restrict__ g, float* __restrict__ m,
                       float* __restrict__ v, int64_t n, float lr, float b1, float b2, float eps, float c1,
                       float c2) {
  const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= n) return;
  const float gi = g[t];
  const float mi = b1 * m[t] + (1.f - b1) * gi;
  const float vi = b2 * v[t] + (1.f - b2) * gi * gi;
  m[t] = mi;
  v[t] = vi;
  p[t] -= lr * (mi / c1) / (sqrtf(vi / c2) + eps);
}

struct Layout {
  const float *W1, *b1, *W2, *b2, *W3, *b3;
};

Layout layout(const float* p, int F, int H) {
  Layout L;
  L.W1 = p;
  L.b1 = L.W1 + (int64_t)F * H;
  L.W2 = L.b1 + H;
  L.b2 = L.W2 + (int64_t)H * H;
  L.W3 = L.b2 + H;
  L.b3 = L.W3 + H;
  return L;
}

bool bad_dims(int F, int H, int B) { return F < 1 || F > 64 || H < 1 || H > 1024 || B < 1; }

cudaError_t forward(const float* params, int F, int H, const float* x, int B, float* scratch, cudaStream_t st) {
  const Layout L = layout(params, F, H);
  float* A1 = scratch;
  float* A2 = A1 + (int64_t)B * H;
  float* Y = A2 + (int64_t)B * H;
  k_dense_fwd<<<blocks_for((int64_t)B * H), kT, 0, st>>>(x, L.W1, L.b1, A1, B, F, H, 1);
  k_dense_fwd<<<blocks_for((int64_t)B * H), kT, 0, st>>>(A1, L.W2, L.b2, A2, B, H, H, 1);
  k_dense_fwd<<<blocks_for(B), kT, 0, st>>>(A2, L.W3, L.b3, Y, B, H, 1, 0);
  return cudaGetLastError();
}

}  // namespace
}  // namespace togb

extern "C" {

int64_t togb_mlp_param_count(int F, int H) { return (int64_t)F * H + H + (int64_t)H * H + H + H + 1; }

int64_t togb_mlp_scratch_floats(int B, int H) { return 4 * (int64_t)B * H + 2 * (int64_t)B; }

togb_status togb_mlp_forward(const float* params, int F, int H, const float* x, int B, float* y, float* scratch,
                             void* stream) {
  using namespace togb;
  if (!params || !x || !y || !scratch || bad_dims(F, H, B)) return report(TOGB_ERR_INVALID, "bad MLP arguments");
  cudaStream_t st = (cudaStream_t)stream;
  cudaError_t e = forward(params, F, H, x, B, scratch, st);
  if (e == cudaSuccess)
    e = cudaMemcpyAsync(y, scratch + 2 * (int64_t)B * H, (size_t)B * 4, cudaMemcpyDeviceToDevice, st);
  if (e != cudaSuccess) return report(TOGB_ERR_CUDA, cudaGetErrorString(e));
  return TOGB_OK;
}

togb_status togb_mlp_loss_grad(const float* params, int F, int H, const float* x, const float* target, int B,
                               float* grads, float* loss, float* scratch, void* stream) {
  using namespace togb;
  if (!params || !x || !target || !grads || !scratch || bad_dims(F, H, B))
    return report(TOGB_ERR_INVALID, "bad MLP arguments");
  cudaStream_t st = (cudaStream_t)stream;
  cudaError_t e = forward(params, F, H, x, B, scratch, st);
  if (e != cudaSuccess) return report(TOGB_ERR_CUDA, cudaGetErrorString(e));
  const Layout L = layout(params, F, H);
  float* A1 = scratch;
  float* A2 = A1 + (int64_t)B * H;
  float* Y = A2 + (int64_t)B * H;
  float* dZ2 = Y + B;
  float* dZ1 = dZ2 + (int64_t)B * H;
  float* dY = dZ1 + (int64_t)B * H;
  float* gW1 = grads;
  float* gb1 = gW1 + (int64_t)F * H;
  float* gW2 = gb1 + H;
  float* gb2 = gW2 + (int64_t)H * H;
  float* gW3 = gb2 + H;
  float* gb3 = gW3 + H;
  if (loss && (e = cudaMemsetAsync(loss, 0, 4, st)) != cudaSuccess) return report(TOGB_ERR_CUDA, cudaGetErrorString(e));
  k_loss_grad<<<blocks_for(B), kT, 0, st>>>(Y, target, dY, loss, B);
  k_dense_bwd_weight<<<blocks_for((int64_t)(H + 1) * 1), kT, 0, st>>>(A2, dY, gW3, gb3, B, H, 1);
  k_dense_bwd_input<<<blocks_for((int64_t)B * H), kT, 0, st>>>(dY, L.W3, A2, dZ2, B, H, 1);
  k_dense_bwd_weight<<<blocks_for((int64_t)(H + 1) * H), kT, 0, st>>>(A1, dZ2, gW2, gb2, B, H, H);
  k_dense_bwd_input<<<blocks_for((int64_t)B * H), kT, 0, st>>>(dZ2, L.W2, A1, dZ1, B, H, H);
  k_dense_bwd_weight<<<blocks_for((int64_t)(F + 1) * H), kT, 0, st>>>(x, dZ1, gW1, gb1, B, F, H);
  e = cudaGetLastError();
  if (e != cudaSuccess) return report(TOGB_ERR_CUDA, cudaGetErrorString(e));
  return TOGB_OK;
}

togb_status togb_mlp_adam(float* params, const float* grads, float* m, float* v, int64_t n, float lr, float beta1,
                          float beta2, float eps, int32_t step, void* stream) {
  using namespace togb;
  if (!params || !grads || !m || !v || n <= 0 || step < 1) return report(TOGB_ERR_INVALID, "bad Adam arguments");
  const float c1 = 1.f - powf(beta1, (float)step), c2 = 1.f - powf(beta2, (float)step);
  k_adam<<<blocks_for(n), kT, 0, (cudaStream_t)stream>>>(params, grads, m, v, n, lr, beta1, beta2, eps, c1, c2);
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return report(TOGB_ERR_CUDA, cudaGetErrorString(e));
  return TOGB_OK;
}

}  // extern "C"
