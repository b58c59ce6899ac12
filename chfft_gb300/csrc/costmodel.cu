// Learned plan cost model: a 3-layer MLP (features -> H -> H -> 1, ReLU,
// FP32) that predicts the log run time of a plan configuration. It is
// trained on the GPU by the kernels below (a fused forward + backward pass
// over a tile of samples, block partial gradients summed with atomics, then
// an Adam step). There is no reference counterpart: chfft picks one plan per
// length by its fixed factor order (src/prime_factorization.rs:66-113).
#include <algorithm>
#include <cmath>
#include <cstring>
#include <numeric>
#include <random>
#include <string>
#include <vector>

#include "../../include/chfft_gpu.h"
#include "plan.hpp"

namespace chfft {

int record_error(int code, const std::string& msg);

namespace cm {

constexpr int kF = CHFFT_FEATURES;
constexpr int kTile = 64;       // samples per CTA
constexpr int kMlpThreads = 256;

struct MlpShape {
  int h;
  // Offsets of the flat parameter vector.
  __host__ __device__ int w1() const { return 0; }
  __host__ __device__ int b1() const { return h * kF; }
  __host__ __device__ int w2() const { return b1() + h; }
  __host__ __device__ int b2() const { return w2() + h * h; }
  __host__ __device__ int w3() const { return b2() + h; }
  __host__ __device__ int b3() const { return w3() + h; }
  __host__ __device__ int count() const { return b3() + 1; }
};

// Shared memory of k_mlp: the parameters, the tile's inputs and both hidden
// layers (pre-activation derivatives overwrite the activations' partners).
__host__ __device__ inline size_t mlp_smem(int h) {
  const MlpShape s{h};
  return sizeof(float) * ((size_t)s.count() + (size_t)kTile * kF + 4 * (size_t)kTile * h + 2 * kTile);
}

// One CTA: forward pass of up to kTile standardised rows (rows idx[r] of X,
// or row r when idx is null). With y: adds 0.5 * sum (f - y)^2 * inv_n to
// *loss and its gradient (times inv_n) to grad. Without y: writes f to pred.
__global__ void __launch_bounds__(kMlpThreads) k_mlp(const float* __restrict__ prm, int h, const float* __restrict__ X,
                                                     const float* __restrict__ y, const int* __restrict__ idx, int n,
                                                     float inv_n, float* __restrict__ grad, float* __restrict__ loss,
                                                     float* __restrict__ pred) {
  extern __shared__ float sh[];
  const MlpShape S{h};
  float* p = sh;                       // parameters
  float* x = p + S.count();            // [kTile][kF]
  float* a1 = x + kTile * kF;          // [kTile][h] layer-1 activations
  float* a2 = a1 + kTile * h;          // [kTile][h] layer-2 activations
  float* d2 = a2 + kTile * h;          // [kTile][h] dL/d(layer-2 pre-activation)
  float* d1 = d2 + kTile * h;          // [kTile][h] dL/d(layer-1 pre-activation)
  float* e = d1 + kTile * h;           // [kTile] residual * inv_n
  float* out = e + kTile;              // [kTile]
  const int tid = threadIdx.x, nth = blockDim.x;
  const int r0 = blockIdx.x * kTile;
  const int rows = min(kTile, n - r0);
  for (int i = tid; i < S.count(); i += nth) p[i] = prm[i];
  for (int i = tid; i < kTile * kF; i += nth) {
    const int r = i / kF, f = i - r * kF;
    float v = 0.f;
    if (r < rows) {
      const long long row = idx ? idx[r0 + r] : r0 + r;
      v = X[row * kF + f];
    }
    x[i] = v;
  }
  __syncthreads();
  const float* W1 = p + S.w1();
  const float* B1 = p + S.b1();
  const float* W2 = p + S.w2();
  const float* B2 = p + S.b2();
  const float* W3 = p + S.w3();
  for (int i = tid; i < kTile * h; i += nth) {
    const int r = i / h, j = i - r * h;
    float s = B1[j];
    for (int f = 0; f < kF; f++) s = fmaf(W1[j * kF + f], x[r * kF + f], s);
    a1[i] = fmaxf(s, 0.f);
  }
  __syncthreads();
  for (int i = tid; i < kTile * h; i += nth) {
    const int r = i / h, j = i - r * h;
    float s = B2[j];
    for (int k = 0; k < h; k++) s = fmaf(W2[j * h + k], a1[r * h + k], s);
    a2[i] = fmaxf(s, 0.f);
  }
  __syncthreads();
  for (int r = tid; r < kTile; r += nth) {
    float s = p[S.b3()];
    for (int j = 0; j < h; j++) s = fmaf(W3[j], a2[r * h + j], s);
    out[r] = s;
    if (!y) {
      if (r < rows) pred[r0 + r] = s;
    } else {
      float t = 0.f;
      if (r < rows) t = y[idx ? idx[r0 + r] : r0 + r];
      e[r] = r < rows ? (s - t) * inv_n : 0.f;
    }
  }
  if (!y) return;
  __syncthreads();
  if (tid == 0) {
    float l = 0.f;
    for (int r = 0; r < rows; r++) l += 0.5f * (e[r] / inv_n) * (e[r] / inv_n) * inv_n;
    atomicAdd(loss, l);
  }
  for (int i = tid; i < kTile * h; i += nth) {
    const int r = i / h, j = i - r * h;
    d2[i] = a2[i] > 0.f ? e[r] * W3[j] : 0.f;
  }
  __syncthreads();
  for (int i = tid; i < kTile * h; i += nth) {
    const int r = i / h, k = i - r * h;
    float s = 0.f;
    for (int j = 0; j < h; j++) s = fmaf(W2[j * h + k], d2[r * h + j], s);
    d1[i] = a1[i] > 0.f ? s : 0.f;
  }
  __syncthreads();
  // Parameter gradients: sums over the tile's rows, then one atomic each.
  for (int i = tid; i < h * kF; i += nth) {
    const int j = i / kF, f = i - j * kF;
    float s = 0.f;
    for (int r = 0; r < rows; r++) s = fmaf(d1[r * h + j], x[r * kF + f], s);
    atomicAdd(&grad[S.w1() + i], s);
  }
  for (int j = tid; j < h; j += nth) {
    float s1 = 0.f, s2 = 0.f, s3 = 0.f;
    for (int r = 0; r < rows; r++) {
      s1 += d1[r * h + j];
      s2 += d2[r * h + j];
      s3 = fmaf(e[r], a2[r * h + j], s3);
    }
    atomicAdd(&grad[S.b1() + j], s1);
    atomicAdd(&grad[S.b2() + j], s2);
    atomicAdd(&grad[S.w3() + j], s3);
  }
  for (int i = tid; i < h * h; i += nth) {
    const int j = i / h, k = i - j * h;
    float s = 0.f;
    for (int r = 0; r < rows; r++) s = fmaf(d2[r * h + j], a1[r * h + k], s);
    atomicAdd(&grad[S.w2() + i], s);
  }
  if (tid == 0) {
    float s = 0.f;
    for (int r = 0; r < rows; r++) s += e[r];
    atomicAdd(&grad[S.b3()], s);
  }
}

// Adam (Kingma & Ba 2015) with bias correction; clears the gradient.
__global__ void k_adam(float* __restrict__ prm, float* __restrict__ grad, float* __restrict__ m1,
                       float* __restrict__ m2, int count, float lr, float c1, float c2) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= count) return;
  const float g = grad[i];
  const float a = 0.9f * m1[i] + 0.1f * g;
  const float b = 0.999f * m2[i] + 0.001f * g * g;
  m1[i] = a;
  m2[i] = b;
  prm[i] -= lr * (a / c1) / (sqrtf(b / c2) + 1e-8f);
  grad[i] = 0.f;
}

void check(cudaError_t e, const char* what) {
  if (e != cudaSuccess) throw Fail{CHFFT_ECUDA, std::string(what) + ": " + cudaGetErrorString(e)};
}

}  // namespace cm
}  // namespace chfft

using chfft::Fail;

struct chfft_mlp_s {
  chfft::cm::MlpShape shape{64};
  std::vector<float> mean = std::vector<float>(chfft::cm::kF, 0.f), sd = std::vector<float>(chfft::cm::kF, 1.f);
  float y_mean = 0.f, y_sd = 1.f;
  chfft::DevBuf prm, grad, m1, m2, loss;
  cudaStream_t s = nullptr;
  ~chfft_mlp_s() {
    if (s) cudaStreamDestroy(s);
  }

  __host__ __device__ int count() const { return shape.count(); }

  void standardise(const float* X, const float* y, int n, std::vector<float>& xs, std::vector<float>& ys) const {
    xs.resize((size_t)n * chfft::cm::kF);
    for (int r = 0; r < n; r++)
      for (int f = 0; f < chfft::cm::kF; f++)
        xs[(size_t)r * chfft::cm::kF + f] = (X[(size_t)r * chfft::cm::kF + f] - mean[f]) / sd[f];
    if (y) {
      ys.resize(n);
      for (int r = 0; r < n; r++) ys[r] = (y[r] - y_mean) / y_sd;
    }
  }

  // Loss and gradient sums of one pass over rows [0, n) (or idx rows).
  void pass(const float* dX, const float* dy, const int* didx, int n, float inv_n, float* dpred) {
    const size_t smem = chfft::cm::mlp_smem(shape.h);
    chfft::cm::check(cudaFuncSetAttribute(chfft::cm::k_mlp, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem), "mlp smem");
    const unsigned blocks = (unsigned)((n + chfft::cm::kTile - 1) / chfft::cm::kTile);
    chfft::cm::k_mlp<<<blocks, chfft::cm::kMlpThreads, smem, s>>>(static_cast<const float*>(prm.p), shape.h, dX, dy, didx, n,
                                                          inv_n, static_cast<float*>(grad.p),
                                                          static_cast<float*>(loss.p), dpred);
    chfft::cm::check(cudaGetLastError(), "mlp kernel");
  }
};

namespace {

template <class F>
int guard(F&& f) {
  try {
    return f();
  } catch (const Fail& e) {
    return chfft::record_error(e.code, e.msg);
  } catch (const std::exception& e) {
    return chfft::record_error(CHFFT_EINVAL, e.what());
  }
}

}  // namespace

extern "C" {

int chfft_mlp_create(int hidden, unsigned seed, chfft_mlp* out) {
  if (!out || hidden < 1 || hidden > 96) return chfft::record_error(CHFFT_EINVAL, "hidden width must be 1..96");
  return guard([&]() -> int {
    auto* m = new chfft_mlp_s();
    m->shape.h = hidden;
    try {
      chfft::cm::check(cudaStreamCreateWithFlags(&m->s, cudaStreamNonBlocking), "stream");
      const int P = m->count();
      m->prm.ensure(P * 4);
      m->grad.ensure(P * 4);
      m->m1.ensure(P * 4);
      m->m2.ensure(P * 4);
      m->loss.ensure(4);
      // He-uniform weights, zero biases.
      std::mt19937 rng(seed);
      std::vector<float> p(P, 0.f);
      auto fill = [&](int off, int cnt, int fan_in) {
        std::uniform_real_distribution<float> u(-1.f, 1.f);
        const float a = std::sqrt(6.f / (float)fan_in);
        for (int i = 0; i < cnt; i++) p[off + i] = a * u(rng);
      };
      fill(m->shape.w1(), hidden * chfft::cm::kF, chfft::cm::kF);
      fill(m->shape.w2(), hidden * hidden, hidden);
      fill(m->shape.w3(), hidden, hidden);
      chfft::cm::check(cudaMemcpy(m->prm.p, p.data(), P * 4, cudaMemcpyHostToDevice), "upload");
      chfft::cm::check(cudaMemset(m->grad.p, 0, P * 4), "memset");
      chfft::cm::check(cudaMemset(m->m1.p, 0, P * 4), "memset");
      chfft::cm::check(cudaMemset(m->m2.p, 0, P * 4), "memset");
    } catch (...) {
      delete m;
      throw;
    }
    *out = m;
    return CHFFT_OK;
  });
}

int chfft_mlp_destroy(chfft_mlp m) {
  delete m;
  return CHFFT_OK;
}

int chfft_mlp_num_params(chfft_mlp m) { return m ? m->count() : 0; }

int chfft_mlp_get_params(chfft_mlp m, float* out) {
  if (!m || !out) return chfft::record_error(CHFFT_EINVAL, "null argument");
  return guard([&]() -> int {
    chfft::cm::check(cudaMemcpy(out, m->prm.p, m->count() * 4, cudaMemcpyDeviceToHost), "download");
    return CHFFT_OK;
  });
}

int chfft_mlp_set_params(chfft_mlp m, const float* p) {
  if (!m || !p) return chfft::record_error(CHFFT_EINVAL, "null argument");
  return guard([&]() -> int {
    chfft::cm::check(cudaMemcpy(m->prm.p, p, m->count() * 4, cudaMemcpyHostToDevice), "upload");
    return CHFFT_OK;
  });
}

int chfft_mlp_set_moments(chfft_mlp m, const float* mean, const float* sd, float y_mean, float y_sd) {
  if (!m || !mean || !sd) return chfft::record_error(CHFFT_EINVAL, "null argument");
  for (int f = 0; f < chfft::cm::kF; f++) {
    m->mean[f] = mean[f];
    m->sd[f] = sd[f] > 0.f ? sd[f] : 1.f;
  }
  m->y_mean = y_mean;
  m->y_sd = y_sd > 0.f ? y_sd : 1.f;
  return CHFFT_OK;
}

int chfft_mlp_get_moments(chfft_mlp m, float* mean, float* sd, float* y_mean, float* y_sd) {
  if (!m || !mean || !sd || !y_mean || !y_sd) return chfft::record_error(CHFFT_EINVAL, "null argument");
  std::copy(m->mean.begin(), m->mean.end(), mean);
  std::copy(m->sd.begin(), m->sd.end(), sd);
  *y_mean = m->y_mean;
  *y_sd = m->y_sd;
  return CHFFT_OK;
}

int chfft_mlp_loss_grad(chfft_mlp m, const float* X, const float* y, int n, float* loss, float* grad) {
  if (!m || !X || !y || n <= 0 || !loss || !grad) return chfft::record_error(CHFFT_EINVAL, "bad argument");
  return guard([&]() -> int {
    std::vector<float> xs, ys;
    m->standardise(X, y, n, xs, ys);
    chfft::DevBuf dx, dy;
    dx.ensure(xs.size() * 4);
    dy.ensure(ys.size() * 4);
    chfft::cm::check(cudaMemcpyAsync(dx.p, xs.data(), xs.size() * 4, cudaMemcpyHostToDevice, m->s), "upload");
    chfft::cm::check(cudaMemcpyAsync(dy.p, ys.data(), ys.size() * 4, cudaMemcpyHostToDevice, m->s), "upload");
    chfft::cm::check(cudaMemsetAsync(m->grad.p, 0, m->count() * 4, m->s), "memset");
    chfft::cm::check(cudaMemsetAsync(m->loss.p, 0, 4, m->s), "memset");
    m->pass(static_cast<const float*>(dx.p), static_cast<const float*>(dy.p), nullptr, n, 1.f / n, nullptr);
    chfft::cm::check(cudaMemcpyAsync(grad, m->grad.p, m->count() * 4, cudaMemcpyDeviceToHost, m->s), "download");
    chfft::cm::check(cudaMemcpyAsync(loss, m->loss.p, 4, cudaMemcpyDeviceToHost, m->s), "download");
    chfft::cm::check(cudaMemsetAsync(m->grad.p, 0, m->count() * 4, m->s), "memset");
    chfft::cm::check(cudaStreamSynchronize(m->s), "sync");
    return CHFFT_OK;
  });
}

int chfft_mlp_train(chfft_mlp m, const float* X, const float* y, int n, int epochs, int batch, float lr,
                    unsigned seed, float* final_loss) {
  if (!m || !X || !y || n <= 1 || epochs < 0 || batch < 1) return chfft::record_error(CHFFT_EINVAL, "bad argument");
  return guard([&]() -> int {
    // Moments of the training set.
    for (int f = 0; f < chfft::cm::kF; f++) {
      double s = 0, q = 0;
      for (int r = 0; r < n; r++) s += X[(size_t)r * chfft::cm::kF + f];
      const double mu = s / n;
      for (int r = 0; r < n; r++) {
        const double d = X[(size_t)r * chfft::cm::kF + f] - mu;
        q += d * d;
      }
      const double sd = std::sqrt(q / n);
      m->mean[f] = (float)mu;
      m->sd[f] = sd > 1e-6 ? (float)sd : 1.f;
    }
    double s = 0, q = 0;
    for (int r = 0; r < n; r++) s += y[r];
    const double mu = s / n;
    for (int r = 0; r < n; r++) q += (y[r] - mu) * (y[r] - mu);
    m->y_mean = (float)mu;
    m->y_sd = std::sqrt(q / n) > 1e-6 ? (float)std::sqrt(q / n) : 1.f;
    std::vector<float> xs, ys;
    m->standardise(X, y, n, xs, ys);
    chfft::DevBuf dx, dy, didx;
    dx.ensure(xs.size() * 4);
    dy.ensure(ys.size() * 4);
    didx.ensure((size_t)n * 4);
    chfft::cm::check(cudaMemcpyAsync(dx.p, xs.data(), xs.size() * 4, cudaMemcpyHostToDevice, m->s), "upload");
    chfft::cm::check(cudaMemcpyAsync(dy.p, ys.data(), ys.size() * 4, cudaMemcpyHostToDevice, m->s), "upload");
    const int P = m->count();
    chfft::cm::check(cudaMemsetAsync(m->grad.p, 0, P * 4, m->s), "memset");
    chfft::cm::check(cudaMemsetAsync(m->m1.p, 0, P * 4, m->s), "memset");
    chfft::cm::check(cudaMemsetAsync(m->m2.p, 0, P * 4, m->s), "memset");
    std::mt19937 rng(seed);
    std::vector<int> perm(n);
    std::iota(perm.begin(), perm.end(), 0);
    long long t = 0;
    const float* fx = static_cast<const float*>(dx.p);
    const float* fy = static_cast<const float*>(dy.p);
    const int* fi = static_cast<const int*>(didx.p);
    for (int ep = 0; ep < epochs; ep++) {
      std::shuffle(perm.begin(), perm.end(), rng);
      chfft::cm::check(cudaMemcpyAsync(didx.p, perm.data(), (size_t)n * 4, cudaMemcpyHostToDevice, m->s), "upload");
      for (int b0 = 0; b0 < n; b0 += batch) {
        const int cnt = std::min(batch, n - b0);
        m->pass(fx, fy, fi + b0, cnt, 1.f / cnt, nullptr);
        t++;
        const float c1 = 1.f - std::pow(0.9f, (float)t), c2 = 1.f - std::pow(0.999f, (float)t);
        chfft::cm::k_adam<<<(P + 255) / 256, 256, 0, m->s>>>(static_cast<float*>(m->prm.p), static_cast<float*>(m->grad.p),
                                                          static_cast<float*>(m->m1.p), static_cast<float*>(m->m2.p),
                                                          P, lr, c1, c2);
        chfft::cm::check(cudaGetLastError(), "adam");
      }
      // The idx upload of the next epoch must not overtake this epoch's reads.
      chfft::cm::check(cudaStreamSynchronize(m->s), "sync");
    }
    chfft::cm::check(cudaMemsetAsync(m->loss.p, 0, 4, m->s), "memset");
    m->pass(fx, fy, nullptr, n, 1.f / n, nullptr);
    chfft::cm::check(cudaMemsetAsync(m->grad.p, 0, P * 4, m->s), "memset");
    float l = 0.f;
    chfft::cm::check(cudaMemcpyAsync(&l, m->loss.p, 4, cudaMemcpyDeviceToHost, m->s), "download");
    chfft::cm::check(cudaStreamSynchronize(m->s), "sync");
    if (final_loss) *final_loss = l;
    return CHFFT_OK;
  });
}

int chfft_mlp_predict(chfft_mlp m, const float* X, int n, float* y) {
  if (!m || !X || !y || n <= 0) return chfft::record_error(CHFFT_EINVAL, "bad argument");
  return guard([&]() -> int {
    std::vector<float> xs, ys;
    m->standardise(X, nullptr, n, xs, ys);
    chfft::DevBuf dx, dp;
    dx.ensure(xs.size() * 4);
    dp.ensure((size_t)n * 4);
    chfft::cm::check(cudaMemcpyAsync(dx.p, xs.data(), xs.size() * 4, cudaMemcpyHostToDevice, m->s), "upload");
    m->pass(static_cast<const float*>(dx.p), nullptr, nullptr, n, 1.f / n, static_cast<float*>(dp.p));
    chfft::cm::check(cudaMemcpyAsync(y, dp.p, (size_t)n * 4, cudaMemcpyDeviceToHost, m->s), "download");
    chfft::cm::check(cudaStreamSynchronize(m->s), "sync");
    for (int r = 0; r < n; r++) y[r] = y[r] * m->y_sd + m->y_mean;
    return CHFFT_OK;
  });
}

}  // extern "C"
