// mlp.cu -- training of the early-exit network (no counterpart in the
// reference).  Network 5 -> 32 -> 32 -> 1 with ReLU, trained with a weighted
// binary cross-entropy on logits by hand-written kernels:
//
//   fwd_bwd_kernel   one warp per chunk of samples; lane j owns hidden unit j
//                    of both layers (row j and column j of W2 in registers),
//                    runs forward and backward for each sample and accumulates
//                    its gradient rows in registers; each warp writes one
//                    partial gradient (no atomics, so results are
//                    deterministic).
//   reduce_kernel    sums the partial gradients in a fixed order and scales by
//                    1 / (sum of sample weights in the batch).
//   adam_kernel      Adam update of the FP32 parameters.
//
// Parameter layout (MLP_NPARAM FP32): W1[32][5], b1[32], W2[32][32], b2[32],
// w3[32], b3 -- the same layout the search kernel reads (as BF16).
#include <cuda_runtime.h>

#include <cmath>
#include <cstdint>
#include <vector>

#include "internal.h"
#include "search_kernel.cuh"
#include "song_gb300.h"

namespace song {
namespace {

constexpr int CHUNK = 32;         // samples per warp per step
constexpr int PARTIAL = MLP_NPARAM + 2;  // gradient + loss + weight sum

__global__ void fwd_bwd_kernel(const float *__restrict__ x, const float *__restrict__ y,
                               const float *__restrict__ sw, const int32_t *__restrict__ idx,
                               int64_t first, int64_t count, const float *__restrict__ params,
                               float *__restrict__ partial, float *__restrict__ logits) {
  const int lane = threadIdx.x & 31;
  const int64_t warp = (static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x) >> 5;
  const int64_t s0 = warp * CHUNK;
  if (s0 >= count) return;
  const int64_t s1 = s0 + CHUNK < count ? s0 + CHUNK : count;

  float w1[MLP_IN], w2r[MLP_H], w2c[MLP_H];
#pragma unroll
  for (int i = 0; i < MLP_IN; ++i) w1[i] = params[MLP_W1 + lane * MLP_IN + i];
#pragma unroll
  for (int i = 0; i < MLP_H; ++i) {
    w2r[i] = params[MLP_W2 + lane * MLP_H + i];
    w2c[i] = params[MLP_W2 + i * MLP_H + lane];
  }
  const float b1 = params[MLP_B1 + lane], b2 = params[MLP_B2 + lane];
  const float w3 = params[MLP_W3 + lane], b3 = params[MLP_B3];

  float g1[MLP_IN], g2[MLP_H];
#pragma unroll
  for (int i = 0; i < MLP_IN; ++i) g1[i] = 0.0f;
#pragma unroll
  for (int i = 0; i < MLP_H; ++i) g2[i] = 0.0f;
  float gb1 = 0.0f, gb2 = 0.0f, gw3 = 0.0f, gb3 = 0.0f, loss = 0.0f, wsum = 0.0f;

  for (int64_t s = s0; s < s1; ++s) {
    const int64_t r = idx ? static_cast<int64_t>(idx[first + s]) : first + s;
    float xi[MLP_IN];
#pragma unroll
    for (int i = 0; i < MLP_IN; ++i) xi[i] = x[r * MLP_IN + i];
    const float yy = y ? y[r] : 0.0f;
    const float ww = sw ? sw[r] : 1.0f;
    float a1 = b1;
#pragma unroll
    for (int i = 0; i < MLP_IN; ++i) a1 = fmaf(w1[i], xi[i], a1);
    const float h1 = fmaxf(a1, 0.0f);
    float a2 = b2;
#pragma unroll
    for (int i = 0; i < MLP_H; ++i) a2 = fmaf(w2r[i], __shfl_sync(FULL, h1, i), a2);
    const float h2 = fmaxf(a2, 0.0f);
    float z = w3 * h2;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) z += __shfl_xor_sync(FULL, z, o);
    z += b3;
    if (logits) {
      if (lane == 0) logits[r] = z;
      continue;
    }
    // weighted BCE on the logit: softplus(z) - y z; d/dz = sigmoid(z) - y
    const float sp = fmaxf(z, 0.0f) + log1pf(expf(-fabsf(z)));
    const float p = 1.0f / (1.0f + expf(-z));
    loss += ww * (sp - yy * z);
    wsum += ww;
    const float dz = ww * (p - yy);
    gb3 += dz;
    gw3 = fmaf(dz, h2, gw3);
    const float da2 = a2 > 0.0f ? dz * w3 : 0.0f;
    gb2 += da2;
#pragma unroll
    for (int i = 0; i < MLP_H; ++i) g2[i] = fmaf(da2, __shfl_sync(FULL, h1, i), g2[i]);
    float dh1 = 0.0f;
#pragma unroll
    for (int i = 0; i < MLP_H; ++i) dh1 = fmaf(w2c[i], __shfl_sync(FULL, da2, i), dh1);
    const float da1 = a1 > 0.0f ? dh1 : 0.0f;
    gb1 += da1;
#pragma unroll
    for (int i = 0; i < MLP_IN; ++i) g1[i] = fmaf(da1, xi[i], g1[i]);
  }
  if (logits) return;
  float *out = partial + warp * PARTIAL;
#pragma unroll
  for (int i = 0; i < MLP_IN; ++i) out[MLP_W1 + lane * MLP_IN + i] = g1[i];
  out[MLP_B1 + lane] = gb1;
#pragma unroll
  for (int i = 0; i < MLP_H; ++i) out[MLP_W2 + lane * MLP_H + i] = g2[i];
  out[MLP_B2 + lane] = gb2;
  out[MLP_W3 + lane] = gw3;
  if (lane == 0) {
    out[MLP_B3] = gb3;
    out[MLP_NPARAM] = loss;
    out[MLP_NPARAM + 1] = wsum;
  }
}

// grad[p] = sum_w partial[w][p] / sum_w weight[w]; loss likewise.
__global__ void reduce_kernel(const float *__restrict__ partial, int nwarps, float *__restrict__ grad,
                              float *__restrict__ loss_out) {
  __shared__ float wtot;
  if (threadIdx.x == 0) {
    float t = 0.0f;
    for (int w = 0; w < nwarps; ++w) t += partial[static_cast<int64_t>(w) * PARTIAL + MLP_NPARAM + 1];
    wtot = t > 0.0f ? t : 1.0f;
  }
  __syncthreads();
  for (int pi = blockIdx.x * blockDim.x + threadIdx.x; pi <= MLP_NPARAM; pi += gridDim.x * blockDim.x) {
    float t = 0.0f;
    for (int w = 0; w < nwarps; ++w) t += partial[static_cast<int64_t>(w) * PARTIAL + pi];
    if (pi < MLP_NPARAM) grad[pi] = t / wtot;
    else if (loss_out) *loss_out = t / wtot;
  }
}

__global__ void adam_kernel(float *__restrict__ params, const float *__restrict__ grad, float *__restrict__ m,
                            float *__restrict__ v, float lr, float b1, float b2, float eps, float c1,
                            float c2) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= MLP_NPARAM) return;
  const float g = grad[i];
  const float mi = b1 * m[i] + (1.0f - b1) * g;
  const float vi = b2 * v[i] + (1.0f - b2) * g * g;
  m[i] = mi;
  v[i] = vi;
  params[i] -= lr * (mi / c1) / (sqrtf(vi / c2) + eps);
}

int run_step(const float *x, const float *y, const float *sw, const int32_t *idx, int64_t first,
             int64_t count, const float *params, float *partial, float *grad, float *loss,
             cudaStream_t s) {
  const int64_t nwarps = (count + CHUNK - 1) / CHUNK;
  const int threads = 128;
  const int64_t blocks = (nwarps * 32 + threads - 1) / threads;
  fwd_bwd_kernel<<<static_cast<unsigned>(blocks), threads, 0, s>>>(x, y, sw, idx, first, count, params,
                                                                   partial, nullptr);
  reduce_kernel<<<(MLP_NPARAM + 256) / 256, 256, 0, s>>>(partial, static_cast<int>(nwarps), grad, loss);
  return cudaGetLastError();
}

}  // namespace
}  // namespace song

using song::MLP_NPARAM;

extern "C" {

int song_mlp_train_device(const float *d_x, const float *d_y, const float *d_w, int64_t n,
                          const int32_t *d_perm, int epochs, int batch, float lr, float *d_params,
                          float *d_loss, void *stream) {
  song::clear_error();
  if (!d_x || !d_y || !d_params || n < 1 || epochs < 1 || batch < 1 || lr <= 0.0f)
    return song::fail(SONG_ERR_ARG, "bad training arguments");
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  const int64_t nwarps = (static_cast<int64_t>(batch) + song::CHUNK - 1) / song::CHUNK;
  float *partial = nullptr, *grad = nullptr, *m = nullptr, *v = nullptr, *lossbuf = nullptr;
  const int64_t steps = (n + batch - 1) / batch;
  cudaError_t e = song::dev_malloc(&partial, sizeof(float) * nwarps * song::PARTIAL);
  if (e == cudaSuccess) e = song::dev_malloc(&grad, sizeof(float) * MLP_NPARAM);
  if (e == cudaSuccess) e = song::dev_malloc(&m, sizeof(float) * MLP_NPARAM);
  if (e == cudaSuccess) e = song::dev_malloc(&v, sizeof(float) * MLP_NPARAM);
  if (e == cudaSuccess) e = song::dev_malloc(&lossbuf, sizeof(float) * steps);
  if (e == cudaSuccess) e = cudaMemsetAsync(m, 0, sizeof(float) * MLP_NPARAM, s);
  if (e == cudaSuccess) e = cudaMemsetAsync(v, 0, sizeof(float) * MLP_NPARAM, s);
  int rc = SONG_OK;
  const float b1 = 0.9f, b2 = 0.999f, eps = 1e-8f;
  int64_t t = 0;
  for (int ep = 0; ep < epochs && e == cudaSuccess && rc == SONG_OK; ++ep) {
    const int32_t *perm = d_perm ? d_perm + static_cast<int64_t>(ep) * n : nullptr;
    for (int64_t st = 0; st < steps && e == cudaSuccess; ++st) {
      const int64_t first = st * batch;
      const int64_t count = first + batch <= n ? batch : n - first;
      int le = song::run_step(d_x, d_y, d_w, perm, first, count, d_params, partial, grad, lossbuf + st, s);
      if (le != 0) {
        e = static_cast<cudaError_t>(le);
        break;
      }
      ++t;
      const float c1 = 1.0f - std::pow(b1, static_cast<float>(t));
      const float c2 = 1.0f - std::pow(b2, static_cast<float>(t));
      song::adam_kernel<<<(MLP_NPARAM + 255) / 256, 256, 0, s>>>(d_params, grad, m, v, lr, b1, b2, eps, c1, c2);
      e = cudaGetLastError();
    }
    if (e == cudaSuccess && d_loss) {
      // mean step loss of the epoch, reduced on the host after the epoch
      std::vector<float> hl(static_cast<size_t>(steps));
      e = cudaMemcpyAsync(hl.data(), lossbuf, sizeof(float) * steps, cudaMemcpyDeviceToHost, s);
      if (e == cudaSuccess) e = cudaStreamSynchronize(s);
      double acc = 0.0;
      for (float f : hl) acc += f;
      const float mean = static_cast<float>(acc / static_cast<double>(steps));
      if (e == cudaSuccess) e = cudaMemcpyAsync(d_loss + ep, &mean, sizeof(float), cudaMemcpyHostToDevice, s);
      if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    }
  }
  if (e == cudaSuccess) e = cudaStreamSynchronize(s);
  cudaFree(partial);
  cudaFree(grad);
  cudaFree(m);
  cudaFree(v);
  cudaFree(lossbuf);
  if (e != cudaSuccess)
    return song::fail(e == cudaErrorMemoryAllocation ? SONG_ERR_OOM : SONG_ERR_CUDA, "mlp training: %s",
                      cudaGetErrorString(e));
  return rc;
}

int song_mlp_grad(const float *x, const float *y, const float *w, int n, const float *params,
                  float *grad_out, float *loss_out) {
  song::clear_error();
  if (!x || !y || !params || !grad_out || n < 1) return song::fail(SONG_ERR_ARG, "bad arguments");
  const int64_t nwarps = (static_cast<int64_t>(n) + song::CHUNK - 1) / song::CHUNK;
  float *dx = nullptr, *dy = nullptr, *dw = nullptr, *dp = nullptr, *partial = nullptr, *grad = nullptr,
        *loss = nullptr;
  cudaError_t e = song::dev_malloc(&dx, sizeof(float) * n * song::MLP_IN);
  if (e == cudaSuccess) e = song::dev_malloc(&dy, sizeof(float) * n);
  if (e == cudaSuccess && w) e = song::dev_malloc(&dw, sizeof(float) * n);
  if (e == cudaSuccess) e = song::dev_malloc(&dp, sizeof(float) * MLP_NPARAM);
  if (e == cudaSuccess) e = song::dev_malloc(&partial, sizeof(float) * nwarps * song::PARTIAL);
  if (e == cudaSuccess) e = song::dev_malloc(&grad, sizeof(float) * MLP_NPARAM);
  if (e == cudaSuccess) e = song::dev_malloc(&loss, sizeof(float));
  if (e == cudaSuccess) e = cudaMemcpy(dx, x, sizeof(float) * n * song::MLP_IN, cudaMemcpyHostToDevice);
  if (e == cudaSuccess) e = cudaMemcpy(dy, y, sizeof(float) * n, cudaMemcpyHostToDevice);
  if (e == cudaSuccess && w) e = cudaMemcpy(dw, w, sizeof(float) * n, cudaMemcpyHostToDevice);
  if (e == cudaSuccess) e = cudaMemcpy(dp, params, sizeof(float) * MLP_NPARAM, cudaMemcpyHostToDevice);
  if (e == cudaSuccess) {
    int le = song::run_step(dx, dy, dw, nullptr, 0, n, dp, partial, grad, loss, 0);
    e = static_cast<cudaError_t>(le);
  }
  if (e == cudaSuccess) e = cudaMemcpy(grad_out, grad, sizeof(float) * MLP_NPARAM, cudaMemcpyDeviceToHost);
  if (e == cudaSuccess && loss_out) e = cudaMemcpy(loss_out, loss, sizeof(float), cudaMemcpyDeviceToHost);
  cudaFree(dx);
  cudaFree(dy);
  cudaFree(dw);
  cudaFree(dp);
  cudaFree(partial);
  cudaFree(grad);
  cudaFree(loss);
  if (e != cudaSuccess) return song::fail(SONG_ERR_CUDA, "mlp grad: %s", cudaGetErrorString(e));
  return SONG_OK;
}

int song_mlp_forward(const float *x, int n, const float *params, float *logits_out) {
  song::clear_error();
  if (!x || !params || !logits_out || n < 1) return song::fail(SONG_ERR_ARG, "bad arguments");
  float *dx = nullptr, *dp = nullptr, *dl = nullptr;
  cudaError_t e = song::dev_malloc(&dx, sizeof(float) * n * song::MLP_IN);
  if (e == cudaSuccess) e = song::dev_malloc(&dp, sizeof(float) * MLP_NPARAM);
  if (e == cudaSuccess) e = song::dev_malloc(&dl, sizeof(float) * n);
  if (e == cudaSuccess) e = cudaMemcpy(dx, x, sizeof(float) * n * song::MLP_IN, cudaMemcpyHostToDevice);
  if (e == cudaSuccess) e = cudaMemcpy(dp, params, sizeof(float) * MLP_NPARAM, cudaMemcpyHostToDevice);
  if (e == cudaSuccess) {
    const int64_t nwarps = (static_cast<int64_t>(n) + song::CHUNK - 1) / song::CHUNK;
    song::fwd_bwd_kernel<<<static_cast<unsigned>((nwarps * 32 + 127) / 128), 128>>>(
        dx, nullptr, nullptr, nullptr, 0, n, dp, nullptr, dl);
    e = cudaGetLastError();
  }
  if (e == cudaSuccess) e = cudaMemcpy(logits_out, dl, sizeof(float) * n, cudaMemcpyDeviceToHost);
  cudaFree(dx);
  cudaFree(dp);
  cudaFree(dl);
  if (e != cudaSuccess) return song::fail(SONG_ERR_CUDA, "mlp forward: %s", cudaGetErrorString(e));
  return SONG_OK;
}

}  // extern "C"
