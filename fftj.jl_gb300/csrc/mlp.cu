// Learned schedule cost model: a 2-hidden-layer ReLU MLP (in -> H -> H -> 1,
// FP32) trained and evaluated on the GPU by the kernels below. No
// counterpart in the reference. It maps a candidate schedule's features
// (fftj_plan_features) to its predicted log time, so that planning an unseen
// size scores the candidates instead of timing them all.
//
// Parameters, flattened: W1[H][D], b1[H], W2[H][H], b2[H], w3[H], b3.
// Loss: mean over the minibatch of (f(x) - y)^2. One CTA of H threads runs
// samples one at a time: thread j owns hidden unit j of both layers, keeps
// its rows of W1 and the gradient rows of W1 and W2 in registers, and reads
// W2 from shared memory (row-padded so that row and column walks are
// conflict-free). Gradients are summed over the CTA's samples in registers
// and added to the global gradient once per CTA.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstring>
#include <vector>

#include "../../include/fftj.h"
#include "fftj_internal.h"

namespace fftj {

constexpr int kMlpMaxIn = 32;
constexpr int kMlpH = 64;  // hidden width (the kernels' CTA size)

struct MlpLayout {
  int D;
  int64_t w1, b1, w2, b2, w3, b3, total;
};

static MlpLayout mlp_layout(int D) {
  MlpLayout L;
  L.D = D;
  L.w1 = 0;
  L.b1 = L.w1 + (int64_t)kMlpH * D;
  L.w2 = L.b1 + kMlpH;
  L.b2 = L.w2 + (int64_t)kMlpH * kMlpH;
  L.w3 = L.b2 + kMlpH;
  L.b3 = L.w3 + kMlpH;
  L.total = L.b3 + 1;
  return L;
}

// Forward (and, with GRAD, backward) over samples idx[s0 .. s1) of X.
// grads (GRAD only) accumulate d(loss)/d(param) with loss = sum (f - y)^2 *
// inv_nb; loss_acc accumulates sum (f - y)^2; pred (forward only) gets f.
template <bool GRAD>
__global__ void __launch_bounds__(kMlpH) k_mlp(const float* __restrict__ P, int D, const float* __restrict__ X,
                                               const float* __restrict__ y, const int* __restrict__ idx,
                                               int64_t base, int64_t count, int per_cta, float inv_nb,
                                               float* __restrict__ G, double* __restrict__ loss_acc,
                                               float* __restrict__ pred) {
  const MlpLayout L = {D, 0, (int64_t)kMlpH * D, (int64_t)kMlpH * D + kMlpH,
                       (int64_t)kMlpH * D + kMlpH + kMlpH * kMlpH, (int64_t)kMlpH * D + 2 * kMlpH + kMlpH * kMlpH,
                       (int64_t)kMlpH * D + 3 * kMlpH + kMlpH * kMlpH, 0};
  __shared__ float W2s[kMlpH * (kMlpH + 1)];
  __shared__ float xs[kMlpMaxIn];
  __shared__ float h1s[kMlpH];
  __shared__ float d2s[kMlpH];
  __shared__ float red[2];
  const int j = threadIdx.x;
  for (int e = j; e < kMlpH * kMlpH; e += kMlpH) W2s[(e / kMlpH) * (kMlpH + 1) + e % kMlpH] = P[L.w2 + e];
  float w1[kMlpMaxIn];
#pragma unroll
  for (int i = 0; i < kMlpMaxIn; ++i) w1[i] = i < D ? P[L.w1 + (int64_t)j * D + i] : 0.f;
  const float b1 = P[L.b1 + j], b2 = P[L.b2 + j], w3 = P[L.w3 + j], b3 = P[L.b3];
  float gw1[kMlpMaxIn];
  float gw2[kMlpH];
#pragma unroll
  for (int i = 0; i < kMlpMaxIn; ++i) gw1[i] = 0.f;
#pragma unroll
  for (int k = 0; k < kMlpH; ++k) gw2[k] = 0.f;
  float gb1 = 0.f, gb2 = 0.f, gw3 = 0.f, gb3 = 0.f;
  double lsum = 0;
  __syncthreads();

  const int64_t s0 = (int64_t)blockIdx.x * per_cta;
  const int64_t s1 = count < s0 + per_cta ? count : s0 + per_cta;
  for (int64_t s = s0; s < s1; ++s) {
    const int64_t row = idx ? (int64_t)idx[base + s] : base + s;
    if (j < D) xs[j] = X[row * D + j];
    __syncthreads();
    float a1 = b1;
#pragma unroll
    for (int i = 0; i < kMlpMaxIn; ++i)
      if (i < D) a1 = fmaf(w1[i], xs[i], a1);
    const float h1 = fmaxf(a1, 0.f);
    h1s[j] = h1;
    __syncthreads();
    float a2 = b2;
#pragma unroll 16
    for (int k = 0; k < kMlpH; ++k) a2 = fmaf(W2s[j * (kMlpH + 1) + k], h1s[k], a2);
    const float h2 = fmaxf(a2, 0.f);
    // f = b3 + sum_j w3_j h2_j: warp sums, then the two warps' partials
    float part = w3 * h2;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) part += __shfl_xor_sync(0xffffffffu, part, o);
    if ((j & 31) == 0) red[j >> 5] = part;
    __syncthreads();
    const float f = b3 + red[0] + red[1];
    if (!GRAD) {
      if (j == 0) pred[row] = f;
      __syncthreads();
      continue;
    }
    const float e = f - y[row];
    lsum += (double)e * e;
    const float dout = 2.f * e * inv_nb;
    gw3 = fmaf(dout, h2, gw3);
    gb3 += dout;
    const float d2 = a2 > 0.f ? dout * w3 : 0.f;
    d2s[j] = d2;
    gb2 += d2;
#pragma unroll
    for (int k = 0; k < kMlpH; ++k) gw2[k] = fmaf(d2, h1s[k], gw2[k]);
    __syncthreads();
    float d1 = 0.f;
#pragma unroll 16
    for (int k = 0; k < kMlpH; ++k) d1 = fmaf(W2s[k * (kMlpH + 1) + j], d2s[k], d1);
    d1 = a1 > 0.f ? d1 : 0.f;
    gb1 += d1;
#pragma unroll
    for (int i = 0; i < kMlpMaxIn; ++i)
      if (i < D) gw1[i] = fmaf(d1, xs[i], gw1[i]);
    __syncthreads();  // xs, h1s, d2s, red are rewritten by the next sample
  }
  if (!GRAD || s0 >= s1) return;
#pragma unroll
  for (int i = 0; i < kMlpMaxIn; ++i)
    if (i < D) atomicAdd(&G[L.w1 + (int64_t)j * D + i], gw1[i]);
  atomicAdd(&G[L.b1 + j], gb1);
#pragma unroll
  for (int k = 0; k < kMlpH; ++k) atomicAdd(&G[L.w2 + (int64_t)j * kMlpH + k], gw2[k]);
  atomicAdd(&G[L.b2 + j], gb2);
  atomicAdd(&G[L.w3 + j], gw3);
  if (j == 0) atomicAdd(&G[L.b3], gb3);
  // the loss is the same in every thread's copy: thread 0 adds it
  if (j == 0) atomicAdd(loss_acc, lsum);
}

// Adam (Kingma & Ba 2015) with bias correction; step t = *t0 + k + 1 (the
// step count lives in device memory so that a captured epoch stays valid).
__global__ void k_adam(float* __restrict__ P, const float* __restrict__ G, float* __restrict__ M,
                       float* __restrict__ V, int64_t n, float lr, float beta1, float beta2, float eps,
                       const int64_t* __restrict__ t0, int k) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const float t = (float)(*t0 + k + 1);
  const float g = G[i];
  const float m = beta1 * M[i] + (1.f - beta1) * g;
  const float v = beta2 * V[i] + (1.f - beta2) * g * g;
  M[i] = m;
  V[i] = v;
  const float mh = m / (1.f - powf(beta1, t));
  const float vh = v / (1.f - powf(beta2, t));
  P[i] -= lr * mh / (sqrtf(vh) + eps);
}

__global__ void k_advance(int64_t* t0, int64_t steps) { *t0 += steps; }

}  // namespace fftj

struct fftj_mlp_s {
  int D = 0;
  fftj::MlpLayout L;
  float* P = nullptr;  // params
  float* G = nullptr;  // gradient
  float* M = nullptr;  // Adam moments
  float* V = nullptr;
  double* loss = nullptr;
  ~fftj_mlp_s() {
    cudaFree(P);
    cudaFree(G);
    cudaFree(M);
    cudaFree(V);
    cudaFree(loss);
  }
};

namespace {

int mlp_fail(int code, const char* msg) {
  fftj::set_error(msg);
  return code;
}

uint64_t splitmix(uint64_t& s) {
  uint64_t z = (s += 0x9E3779B97F4A7C15ull);
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
  return z ^ (z >> 31);
}
double unif(uint64_t& s) { return (double)(splitmix(s) >> 11) * (1.0 / 9007199254740992.0); }

// device copies of the training set, freed on scope exit
struct DevSet {
  float* X = nullptr;
  float* y = nullptr;
  int* idx = nullptr;
  ~DevSet() {
    cudaFree(X);
    cudaFree(y);
    cudaFree(idx);
  }
};

int upload_set(DevSet& d, const float* X, const float* y, int64_t n, int D, bool with_idx) {
  if (cudaMalloc(&d.X, (size_t)n * D * sizeof(float)) != cudaSuccess) return FFTJ_ERR_CUDA;
  if (cudaMemcpy(d.X, X, (size_t)n * D * sizeof(float), cudaMemcpyHostToDevice) != cudaSuccess) return FFTJ_ERR_CUDA;
  if (y) {
    if (cudaMalloc(&d.y, (size_t)n * sizeof(float)) != cudaSuccess) return FFTJ_ERR_CUDA;
    if (cudaMemcpy(d.y, y, (size_t)n * sizeof(float), cudaMemcpyHostToDevice) != cudaSuccess) return FFTJ_ERR_CUDA;
  }
  if (with_idx && cudaMalloc(&d.idx, (size_t)n * sizeof(int)) != cudaSuccess) return FFTJ_ERR_CUDA;
  return FFTJ_OK;
}

constexpr int kPerCta = 16;  // samples per CTA in gradient launches

}  // namespace

extern "C" {

int fftj_mlp_create(fftj_mlp* out, int in_dim, uint64_t seed) {
  if (!out) return mlp_fail(FFTJ_ERR_ARG, "null output");
  *out = nullptr;
  if (in_dim < 1 || in_dim > fftj::kMlpMaxIn) return mlp_fail(FFTJ_ERR_ARG, "in_dim must be 1..32");
  auto* m = new fftj_mlp_s();
  m->D = in_dim;
  m->L = fftj::mlp_layout(in_dim);
  const size_t b = (size_t)m->L.total * sizeof(float);
  if (cudaMalloc(&m->P, b) != cudaSuccess || cudaMalloc(&m->G, b) != cudaSuccess ||
      cudaMalloc(&m->M, b) != cudaSuccess || cudaMalloc(&m->V, b) != cudaSuccess ||
      cudaMalloc(&m->loss, sizeof(double)) != cudaSuccess) {
    delete m;
    return mlp_fail(FFTJ_ERR_CUDA, "model allocation failed");
  }
  // He-uniform weights, zero biases
  std::vector<float> h(m->L.total, 0.f);
  uint64_t s = seed;
  auto fill = [&](int64_t off, int64_t count, int fan_in) {
    const double a = std::sqrt(6.0 / fan_in);
    for (int64_t i = 0; i < count; ++i) h[off + i] = (float)((2 * unif(s) - 1) * a);
  };
  fill(m->L.w1, (int64_t)fftj::kMlpH * in_dim, in_dim);
  fill(m->L.w2, (int64_t)fftj::kMlpH * fftj::kMlpH, fftj::kMlpH);
  fill(m->L.w3, fftj::kMlpH, fftj::kMlpH);
  if (cudaMemcpy(m->P, h.data(), b, cudaMemcpyHostToDevice) != cudaSuccess || cudaMemset(m->M, 0, b) != cudaSuccess ||
      cudaMemset(m->V, 0, b) != cudaSuccess) {
    delete m;
    return mlp_fail(FFTJ_ERR_CUDA, "model initialisation failed");
  }
  *out = m;
  fftj::set_error("");
  return FFTJ_OK;
}

int fftj_mlp_destroy(fftj_mlp m) {
  delete m;
  return FFTJ_OK;
}

int fftj_mlp_num_params(fftj_mlp m, int64_t* count) {
  if (!m || !count) return mlp_fail(FFTJ_ERR_ARG, "null argument");
  *count = m->L.total;
  return FFTJ_OK;
}

int fftj_mlp_get_params(fftj_mlp m, float* host, int64_t count) {
  if (!m || !host || count != m->L.total) return mlp_fail(FFTJ_ERR_ARG, "null argument or wrong count");
  return cudaMemcpy(host, m->P, count * sizeof(float), cudaMemcpyDeviceToHost) == cudaSuccess
             ? FFTJ_OK
             : mlp_fail(FFTJ_ERR_CUDA, "parameter copy failed");
}

int fftj_mlp_set_params(fftj_mlp m, const float* host, int64_t count) {
  if (!m || !host || count != m->L.total) return mlp_fail(FFTJ_ERR_ARG, "null argument or wrong count");
  return cudaMemcpy(m->P, host, count * sizeof(float), cudaMemcpyHostToDevice) == cudaSuccess
             ? FFTJ_OK
             : mlp_fail(FFTJ_ERR_CUDA, "parameter copy failed");
}

int fftj_mlp_grad(fftj_mlp m, const float* X, const float* y, int64_t n, float* grad, double* loss) {
  if (!m || !X || !y || !grad || n < 1) return mlp_fail(FFTJ_ERR_ARG, "null argument or n < 1");
  DevSet d;
  if (upload_set(d, X, y, n, m->D, false)) return mlp_fail(FFTJ_ERR_CUDA, "training set upload failed");
  cudaMemset(m->G, 0, (size_t)m->L.total * sizeof(float));
  cudaMemset(m->loss, 0, sizeof(double));
  const unsigned grid = (unsigned)((n + kPerCta - 1) / kPerCta);
  fftj::k_mlp<true><<<grid, fftj::kMlpH>>>(m->P, m->D, d.X, d.y, nullptr, 0, n, kPerCta, 1.f / (float)n, m->G, m->loss,
                                           nullptr);
  if (cudaGetLastError() != cudaSuccess) return mlp_fail(FFTJ_ERR_CUDA, "gradient launch failed");
  double l = 0;
  if (cudaMemcpy(grad, m->G, (size_t)m->L.total * sizeof(float), cudaMemcpyDeviceToHost) != cudaSuccess ||
      cudaMemcpy(&l, m->loss, sizeof(double), cudaMemcpyDeviceToHost) != cudaSuccess)
    return mlp_fail(FFTJ_ERR_CUDA, "gradient copy failed");
  if (loss) *loss = l / (double)n;
  fftj::set_error("");
  return FFTJ_OK;
}

// Minibatch Adam. Each epoch's shuffle is uploaded, then the epoch's launch
// sequence (per step: clear gradient, forward+backward, Adam; then advance
// the step count) runs as one CUDA graph, captured on the first epoch and
// replayed on the others. *final_loss = mean squared error over the last
// epoch, as seen by its minibatches.
int fftj_mlp_train(fftj_mlp m, const float* X, const float* y, int64_t n, int epochs, int minibatch, float lr,
                   uint64_t seed, double* final_loss) {
  if (!m || !X || !y || n < 1 || epochs < 1 || minibatch < 1 || !(lr > 0))
    return mlp_fail(FFTJ_ERR_ARG, "bad training arguments");
  DevSet d;
  if (upload_set(d, X, y, n, m->D, true)) return mlp_fail(FFTJ_ERR_CUDA, "training set upload failed");
  int64_t* tdev = nullptr;
  if (cudaMalloc(&tdev, sizeof(int64_t)) != cudaSuccess || cudaMemset(tdev, 0, sizeof(int64_t)) != cudaSuccess) {
    cudaFree(tdev);
    return mlp_fail(FFTJ_ERR_CUDA, "step counter allocation failed");
  }
  cudaStream_t st;
  if (cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking) != cudaSuccess) {
    cudaFree(tdev);
    return mlp_fail(FFTJ_ERR_CUDA, "stream creation failed");
  }
  const int64_t steps = (n + minibatch - 1) / minibatch;
  const size_t pbytes = (size_t)m->L.total * sizeof(float);
  std::vector<int> perm(n);
  for (int64_t i = 0; i < n; ++i) perm[i] = (int)i;
  uint64_t s = seed ^ 0x5DEECE66Dull;
  int rc = FFTJ_OK;
  cudaGraph_t graph = nullptr;
  cudaGraphExec_t exec = nullptr;
  double last = 0;
  for (int ep = 0; ep < epochs && rc == FFTJ_OK; ++ep) {
    for (int64_t i = n - 1; i > 0; --i) std::swap(perm[i], perm[(int64_t)(unif(s) * (double)(i + 1))]);
    if (cudaMemcpyAsync(d.idx, perm.data(), (size_t)n * sizeof(int), cudaMemcpyHostToDevice, st) != cudaSuccess) {
      rc = mlp_fail(FFTJ_ERR_CUDA, "shuffle upload failed");
      break;
    }
    if (!exec) {
      if (cudaStreamBeginCapture(st, cudaStreamCaptureModeThreadLocal) != cudaSuccess) {
        rc = mlp_fail(FFTJ_ERR_CUDA, "graph capture failed");
        break;
      }
      cudaMemsetAsync(m->loss, 0, sizeof(double), st);
      for (int64_t k = 0; k < steps; ++k) {
        const int64_t b0 = k * minibatch;
        const int64_t nb = std::min<int64_t>(minibatch, n - b0);
        cudaMemsetAsync(m->G, 0, pbytes, st);
        const unsigned grid = (unsigned)((nb + kPerCta - 1) / kPerCta);
        fftj::k_mlp<true><<<grid, fftj::kMlpH, 0, st>>>(m->P, m->D, d.X, d.y, d.idx, b0, nb, kPerCta,
                                                        1.f / (float)nb, m->G, m->loss, nullptr);
        fftj::k_adam<<<(unsigned)((m->L.total + 255) / 256), 256, 0, st>>>(m->P, m->G, m->M, m->V, m->L.total, lr,
                                                                           0.9f, 0.999f, 1e-8f, tdev, (int)k);
      }
      fftj::k_advance<<<1, 1, 0, st>>>(tdev, steps);
      if (cudaStreamEndCapture(st, &graph) != cudaSuccess || cudaGraphInstantiate(&exec, graph, 0) != cudaSuccess) {
        rc = mlp_fail(FFTJ_ERR_CUDA, "graph instantiation failed");
        break;
      }
    }
    if (cudaGraphLaunch(exec, st) != cudaSuccess) rc = mlp_fail(FFTJ_ERR_CUDA, "graph launch failed");
    if (ep + 1 == epochs && rc == FFTJ_OK &&
        cudaMemcpyAsync(&last, m->loss, sizeof(double), cudaMemcpyDeviceToHost, st) != cudaSuccess)
      rc = mlp_fail(FFTJ_ERR_CUDA, "loss copy failed");
  }
  if (cudaStreamSynchronize(st) != cudaSuccess && rc == FFTJ_OK) rc = mlp_fail(FFTJ_ERR_CUDA, "training failed");
  if (exec) cudaGraphExecDestroy(exec);
  if (graph) cudaGraphDestroy(graph);
  cudaStreamDestroy(st);
  cudaFree(tdev);
  if (rc == FFTJ_OK) {
    if (final_loss) *final_loss = last / (double)n;
    fftj::set_error("");
  }
  return rc;
}

int fftj_mlp_predict(fftj_mlp m, const float* X, int64_t n, float* out) {
  if (!m || !X || !out || n < 1) return mlp_fail(FFTJ_ERR_ARG, "null argument or n < 1");
  DevSet d;
  if (upload_set(d, X, nullptr, n, m->D, false)) return mlp_fail(FFTJ_ERR_CUDA, "input upload failed");
  float* dp = nullptr;
  if (cudaMalloc(&dp, (size_t)n * sizeof(float)) != cudaSuccess) return mlp_fail(FFTJ_ERR_CUDA, "output allocation");
  const unsigned grid = (unsigned)((n + kPerCta - 1) / kPerCta);
  fftj::k_mlp<false><<<grid, fftj::kMlpH>>>(m->P, m->D, d.X, nullptr, nullptr, 0, n, kPerCta, 0.f, nullptr, nullptr, dp);
  int rc = FFTJ_OK;
  if (cudaGetLastError() != cudaSuccess ||
      cudaMemcpy(out, dp, (size_t)n * sizeof(float), cudaMemcpyDeviceToHost) != cudaSuccess)
    rc = mlp_fail(FFTJ_ERR_CUDA, "prediction failed");
  cudaFree(dp);
  if (rc == FFTJ_OK) fftj::set_error("");
  return rc;
}

}  // extern "C"
