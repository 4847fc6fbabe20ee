// Learned CTMRG warm start (no reference counterpart).
//
// A 3-layer perceptron maps the symmetrised site tensor to a gauge-fixed
// environment (corner spectrum + edge tensor).  Everything it computes runs
// here on the GPU:
//   forward   : H_l = act(W_l·H_{l-1} + b_l), ReLU on the two hidden layers;
//   backward  : MSE loss, dW_l = dH_l·H_{l-1}ᵀ, db_l = Σ_batch dH_l,
//               dH_{l-1} = (W_lᵀ·dH_l) ∘ [H_{l-1} > 0];
//   optimiser : AdamW on the FP32 master parameters;
//   targets   : gauge fixing of converged (C, T) (eigh of C, rotation of T,
//               column signs fixed through T);
//   inference : features of a site tensor, prediction, environment build.
// All six products of a training step are BF16 tcgen05 GEMMs with FP32
// accumulation (gemm_bf16); the rest are element-wise or small reductions.
#include <cmath>
#include <memory>
#include <vector>

#include "tnad_api.h"
#include "tnad_drivers.h"
#include "tnad_energy.h"

struct tnad_mlp {
  int device = 0;
  int n_in = 0, width = 0, n_out = 0;
  int rows[4] = {0, 0, 0, 0};  // n_in, width, width, n_out
  int64_t off_w[3] = {0, 0, 0}, off_b[3] = {0, 0, 0};
  int64_t n_params = 0;
  float* P = nullptr;   // parameters (FP32 master copy)
  float* G = nullptr;   // gradient of the last backward pass
  float* M1 = nullptr;  // AdamW first moment
  float* M2 = nullptr;  // AdamW second moment
  int64_t t = 0;        // AdamW steps taken
  int cap = 0;          // batch capacity of the buffers below
  float* X = nullptr;   // n_in × cap   (staged / gathered inputs)
  float* Y = nullptr;   // n_out × cap  (staged / gathered targets)
  float* H[3] = {nullptr, nullptr, nullptr};   // layer outputs
  float* dH[3] = {nullptr, nullptr, nullptr};  // their cotangents
  int* idx = nullptr;     // device copy of the mini-batch indices
  double* red = nullptr;  // loss partial sums (1024) + total
  float* DX = nullptr;    // resident training set (tnad_mlp_set_data): n_in × n_data
  float* DY = nullptr;    //                                            n_out × n_data
  int64_t n_data = 0;
  ~tnad_mlp();  // releases every device buffer (also on a failed create)
};

namespace tnad {
namespace {

constexpr int kRedBlocks = 1024;

__device__ __forceinline__ uint64_t splitmix64(uint64_t x) {
  x += 0x9E3779B97F4A7C15ull;
  x = (x ^ (x >> 30)) * 0xBF58476D1CE4E5B9ull;
  x = (x ^ (x >> 27)) * 0x94D049BB133111EBull;
  return x ^ (x >> 31);
}

// P[i] = bound·u_i, u_i uniform in [-1, 1) from a counter-based hash
__global__ void k_init_uniform(float* __restrict__ P, int64_t n, uint64_t seed, float bound) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    const uint64_t r = splitmix64(seed * 0x2545F4914F6CDD1Dull + (uint64_t)i);
    const float u = (float)((double)(r >> 11) * (1.0 / 9007199254740992.0));  // [0, 1)
    P[i] = bound * (2.f * u - 1.f);
  }
}

// H[r, j] = act(H[r, j] + b[r])
__global__ void k_bias_act(float* __restrict__ H, const float* __restrict__ b, int rows, int64_t n, int relu) {
  for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < n; e += (int64_t)gridDim.x * blockDim.x) {
    const float v = H[e] + b[e % rows];
    H[e] = relu ? fmaxf(v, 0.f) : v;
  }
}

// dst[:, j] = src[:, idx[j]]
__global__ void k_gather_cols(const float* __restrict__ src, int rows, const int* __restrict__ idx, int B,
                              float* __restrict__ dst) {
  const int64_t n = (int64_t)rows * B;
  for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < n; e += (int64_t)gridDim.x * blockDim.x) {
    const int64_t j = e / rows, r = e % rows;
    dst[e] = src[r + (int64_t)idx[j] * rows];
  }
}

// dY = scale·(Yh − Y); per-block partial sums of (Yh − Y)² into part[blockIdx]
__global__ void k_mse(const float* __restrict__ Yh, const float* __restrict__ Y, int64_t n, float scale,
                      float* __restrict__ dY, double* __restrict__ part) {
  __shared__ double sh[32];
  double acc = 0.0;
  for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < n; e += (int64_t)gridDim.x * blockDim.x) {
    const float r = Yh[e] - Y[e];
    dY[e] = scale * r;
    acc += (double)r * (double)r;
  }
  for (int o = 16; o > 0; o >>= 1) acc += __shfl_down_sync(0xffffffffu, acc, o);
  if ((threadIdx.x & 31) == 0) sh[threadIdx.x >> 5] = acc;
  __syncthreads();
  if (threadIdx.x < 32) {
    double v = threadIdx.x < (blockDim.x >> 5) ? sh[threadIdx.x] : 0.0;
    for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
    if (threadIdx.x == 0) part[blockIdx.x] = v;
  }
}

// out[0] = Σ part[0..nb) · inv  (one block, fixed order)
__global__ void k_sum_partials(const double* __restrict__ part, int nb, double inv, double* __restrict__ out) {
  __shared__ double sh[32];
  double acc = 0.0;
  for (int i = threadIdx.x; i < nb; i += blockDim.x) acc += part[i];
  for (int o = 16; o > 0; o >>= 1) acc += __shfl_down_sync(0xffffffffu, acc, o);
  if ((threadIdx.x & 31) == 0) sh[threadIdx.x >> 5] = acc;
  __syncthreads();
  if (threadIdx.x < 32) {
    double v = threadIdx.x < (blockDim.x >> 5) ? sh[threadIdx.x] : 0.0;
    for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
    if (threadIdx.x == 0) out[0] = v * inv;
  }
}

// db[r] = Σ_j dH[r, j]
__global__ void k_rowsum(const float* __restrict__ dH, int rows, int B, float* __restrict__ db) {
  const int r = blockIdx.x * blockDim.x + threadIdx.x;
  if (r >= rows) return;
  double s = 0.0;
  for (int j = 0; j < B; ++j) s += (double)dH[r + (int64_t)j * rows];
  db[r] = (float)s;
}

// dH ∘= [H > 0]
__global__ void k_relu_mask(float* __restrict__ dH, const float* __restrict__ H, int64_t n) {
  for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < n; e += (int64_t)gridDim.x * blockDim.x)
    if (!(H[e] > 0.f)) dH[e] = 0.f;
}

struct BiasRanges {
  int64_t lo[3], hi[3];
};

// AdamW: p ← p − lr·wd·p (weights only); m, v moments; p ← p − lr·m̂/(√v̂ + ε)
__global__ void k_adamw(float* __restrict__ P, const float* __restrict__ G, float* __restrict__ M1,
                        float* __restrict__ M2, int64_t n, float lr, float wd, float b1, float b2, float eps, float bc1,
                        float bc2, BiasRanges br) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    const bool bias = (i >= br.lo[0] && i < br.hi[0]) || (i >= br.lo[1] && i < br.hi[1]) ||
                      (i >= br.lo[2] && i < br.hi[2]);
    float p = P[i];
    if (!bias) p -= lr * wd * p;
    const float g = G[i];
    const float m = b1 * M1[i] + (1.f - b1) * g;
    const float v = b2 * M2[i] + (1.f - b2) * g * g;
    M1[i] = m;
    M2[i] = v;
    const float mh = m / bc1, vh = v / bc2;
    P[i] = p - lr * mh / (sqrtf(vh) + eps);
  }
}

// Network input: x = sign(As[k*])·As (As normalised), k* the first index of max |As|.
__global__ void k_features(const double* __restrict__ As, int n, float* __restrict__ x) {
  __shared__ double sv[32];
  __shared__ int si[32];
  double best = -1.0;
  int bi = 0;
  for (int i = threadIdx.x; i < n; i += blockDim.x) {
    const double v = fabs(As[i]);
    if (v > best) {
      best = v;
      bi = i;
    }
  }
  for (int o = 16; o > 0; o >>= 1) {
    const double ov = __shfl_down_sync(0xffffffffu, best, o);
    const int oi = __shfl_down_sync(0xffffffffu, bi, o);
    if (ov > best || (ov == best && oi < bi)) {
      best = ov;
      bi = oi;
    }
  }
  if ((threadIdx.x & 31) == 0) {
    sv[threadIdx.x >> 5] = best;
    si[threadIdx.x >> 5] = bi;
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    for (int w = 1; w < (int)(blockDim.x >> 5); ++w)
      if (sv[w] > sv[0] || (sv[w] == sv[0] && si[w] < si[0])) {
        sv[0] = sv[w];
        si[0] = si[w];
      }
  }
  __syncthreads();
  const double sgn = As[si[0]] < 0.0 ? -1.0 : 1.0;
  for (int i = threadIdx.x; i < n; i += blockDim.x) x[i] = (float)(sgn * As[i]);
}

__device__ double block_sum(double v, double* sh) {
  for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
  __syncthreads();
  if ((threadIdx.x & 31) == 0) sh[threadIdx.x >> 5] = v;
  __syncthreads();
  double t = 0.0;
  for (int w = 0; w < (int)(blockDim.x >> 5); ++w) t += sh[w];
  return t;
}

// Prediction y = [λ̂ (χ) | T̂ (χ×d×χ)] → C = diag(λ̂)/‖λ̂‖, T = sym(T̂)/‖sym(T̂)‖.
// ok[0] = 1 when both norms are finite and non-zero, else 0.
__global__ void k_build_env(const float* __restrict__ y, int chi, int d, double* __restrict__ C,
                            double* __restrict__ T, int* __restrict__ ok) {
  __shared__ double sh[32];
  const int64_t nT = (int64_t)chi * d * chi, cd = (int64_t)chi * d;
  const float* yT = y + chi;
  double sc = 0.0, st = 0.0;
  for (int a = threadIdx.x; a < chi; a += blockDim.x) sc += (double)y[a] * (double)y[a];
  for (int64_t e = threadIdx.x; e < nT; e += blockDim.x) {
    const int64_t a = e % chi, i = (e / chi) % d, b = e / cd;
    const double v = 0.5 * ((double)yT[e] + (double)yT[b + i * chi + a * cd]);
    T[e] = v;
    st += v * v;
  }
  sc = block_sum(sc, sh);
  st = block_sum(st, sh);
  const bool good = sc > 0.0 && st > 0.0 && isfinite(sc) && isfinite(st);
  if (threadIdx.x == 0) ok[0] = good ? 1 : 0;
  const double ic = good ? 1.0 / sqrt(sc) : 0.0, it = good ? 1.0 / sqrt(st) : 0.0;
  for (int64_t e = threadIdx.x; e < (int64_t)chi * chi; e += blockDim.x) {
    const int64_t a = e % chi, b = e / chi;
    C[e] = a == b ? (double)y[a] * ic : 0.0;
  }
  for (int64_t e = threadIdx.x; e < nT; e += blockDim.x) T[e] *= it;
}

// Column signs of the gauge fix (one block): s_0 = 1; for a = 1..χ-1 the entry
// of largest |Tg[a,i,b]| over i < d, b < a (first in (b, i) order on ties)
// decides s_a = sign(Tg[a,i*,b*])·s_{b*}; then Tg[a,i,b] ← s_a s_b Tg[a,i,b].
__global__ void k_gauge_signs(double* __restrict__ Tg, int chi, int d) {
  extern __shared__ double smem_d[];
  double* sgn = smem_d;  // χ
  __shared__ double sv[32];
  __shared__ int si[32];
  const int64_t cd = (int64_t)chi * d;
  if (threadIdx.x == 0) sgn[0] = 1.0;
  for (int a = 1; a < chi; ++a) {
    double best = -1.0;
    int bi = 0;
    const int cnt = d * a;  // candidates (b, i), linear k = i + d·b
    for (int k = threadIdx.x; k < cnt; k += blockDim.x) {
      const int i = k % d, b = k / d;
      const double v = fabs(Tg[a + (int64_t)i * chi + (int64_t)b * cd]);
      if (v > best) {
        best = v;
        bi = k;
      }
    }
    for (int o = 16; o > 0; o >>= 1) {
      const double ov = __shfl_down_sync(0xffffffffu, best, o);
      const int oi = __shfl_down_sync(0xffffffffu, bi, o);
      if (ov > best || (ov == best && oi < bi)) {
        best = ov;
        bi = oi;
      }
    }
    __syncthreads();
    if ((threadIdx.x & 31) == 0) {
      sv[threadIdx.x >> 5] = best;
      si[threadIdx.x >> 5] = bi;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
      double bv = sv[0];
      int bk = si[0];
      for (int w = 1; w < (int)(blockDim.x >> 5); ++w)
        if (sv[w] > bv || (sv[w] == bv && si[w] < bk)) {
          bv = sv[w];
          bk = si[w];
        }
      const int i = bk % d, b = bk / d;
      const double t = Tg[a + (int64_t)i * chi + (int64_t)b * cd];
      sgn[a] = (bv > 0.0 && t < 0.0) ? -sgn[b] : sgn[b];
    }
    __syncthreads();
  }
  __syncthreads();
  const int64_t nT = cd * chi;
  for (int64_t e = threadIdx.x; e < nT; e += blockDim.x) {
    const int64_t a = e % chi, b = e / cd;
    Tg[e] *= sgn[a] * sgn[b];
  }
}

inline int nblk(int64_t n) { return (int)std::min<int64_t>((n + 255) / 256, 4096); }

float* dev_alloc_f(int64_t n) {
  void* p = nullptr;
  if (cudaMalloc(&p, (size_t)std::max<int64_t>(n, 1) * 4) != cudaSuccess)
    fail(TNAD_ERR_NOMEM, "mlp: cudaMalloc of " + std::to_string(n * 4) + " bytes failed");
  return (float*)p;
}

void free_batch_buffers(tnad_mlp* net) {
  float** fs[8] = {&net->X, &net->Y, &net->H[0], &net->H[1], &net->H[2], &net->dH[0], &net->dH[1], &net->dH[2]};
  for (float** f : fs) {
    if (*f) cudaFree(*f);
    *f = nullptr;
  }
  if (net->idx) cudaFree(net->idx);
  net->idx = nullptr;
  net->cap = 0;
}

void ensure_batch(tnad_mlp* net, int B) {
  if (B <= net->cap) return;
  free_batch_buffers(net);
  net->X = dev_alloc_f((int64_t)net->n_in * B);
  net->Y = dev_alloc_f((int64_t)net->n_out * B);
  for (int l = 0; l < 3; ++l) {
    net->H[l] = dev_alloc_f((int64_t)net->rows[l + 1] * B);
    net->dH[l] = dev_alloc_f((int64_t)net->rows[l + 1] * B);
  }
  TNAD_CK(cudaMalloc(&net->idx, (size_t)B * sizeof(int)));
  net->cap = B;
}

void mlp_forward(tnad_ctx* c, tnad_mlp* net, const float* X, int B) {
  const float* in = X;
  for (int l = 0; l < 3; ++l) {
    const int m = net->rows[l + 1], k = net->rows[l];
    gemm_bf16(c, 'N', 'N', m, B, k, 1.f, net->P + net->off_w[l], m, in, k, 0.f, net->H[l], m);
    k_bias_act<<<nblk((int64_t)m * B), 256, 0, c->stream>>>(net->H[l], net->P + net->off_b[l], m, (int64_t)m * B,
                                                            l < 2 ? 1 : 0);
    count_launch(c);
    in = net->H[l];
  }
  check_launch(c, "mlp_forward");
}

// gradient of mean((H[2] − Y)²) into net->G; loss (mean) into net->red[kRedBlocks]
void mlp_backward(tnad_ctx* c, tnad_mlp* net, const float* X, const float* Y, int B) {
  const int64_t nout = (int64_t)net->n_out * B;
  const double inv = 1.0 / (double)nout;
  k_mse<<<kRedBlocks, 256, 0, c->stream>>>(net->H[2], Y, nout, (float)(2.0 * inv), net->dH[2], net->red);
  k_sum_partials<<<1, 256, 0, c->stream>>>(net->red, kRedBlocks, inv, net->red + kRedBlocks);
  count_launch(c, 2);
  for (int l = 2; l >= 0; --l) {
    const int m = net->rows[l + 1], k = net->rows[l];
    const float* in = l > 0 ? net->H[l - 1] : X;
    gemm_bf16(c, 'N', 'T', m, k, B, 1.f, net->dH[l], m, in, k, 0.f, net->G + net->off_w[l], m);
    k_rowsum<<<(m + 255) / 256, 256, 0, c->stream>>>(net->dH[l], m, B, net->G + net->off_b[l]);
    count_launch(c);
    if (l > 0) {
      gemm_bf16(c, 'T', 'N', k, B, m, 1.f, net->P + net->off_w[l], m, net->dH[l], m, 0.f, net->dH[l - 1], k);
      k_relu_mask<<<nblk((int64_t)k * B), 256, 0, c->stream>>>(net->dH[l - 1], net->H[l - 1], (int64_t)k * B);
      count_launch(c);
    }
  }
  check_launch(c, "mlp_backward");
}

const float* stage(tnad_ctx* c, float* dst, const float* src, int64_t n, bool dev) {
  if (dev) return src;
  TNAD_CK(cudaMemcpyAsync(dst, src, (size_t)n * 4, cudaMemcpyHostToDevice, c->stream));
  return dst;
}

void check_net(const tnad_mlp* net) { TNAD_REQUIRE(net && net->P, TNAD_ERR_ARG, "mlp: null network"); }

}  // namespace

// ---- used by energy_fwd for TNAD_WARM_LEARNED ----
// Predicts (C, T) on the device for the symmetrised, normalised site tensor As;
// false (after a sync) when the prediction is zero or not finite.
bool warm_start_predict(tnad_ctx* c, tnad_mlp* net, const double* As, int n_in, int chi, int d, double* C,
                        double* T) {
  TNAD_REQUIRE(net->n_in == n_in && net->n_out == chi + chi * d * chi, TNAD_ERR_SHAPE,
               "warm start: network shape does not match (D, s, χ)");
  ensure_batch(net, 1);
  k_features<<<1, 256, 0, c->stream>>>(As, n_in, net->X);
  count_launch(c);
  mlp_forward(c, net, net->X, 1);
  int* ok = c->d_flag + 21;
  k_build_env<<<1, 1024, 0, c->stream>>>(net->H[2], chi, d, C, T, ok);
  count_launch(c);
  check_launch(c, "warm_start_predict");
  TNAD_CK(cudaMemcpyAsync(c->h_flag + 21, ok, sizeof(int), cudaMemcpyDeviceToHost, c->stream));
  TNAD_CK(cudaStreamSynchronize(c->stream));
  return c->h_flag[21] == 1;
}

}  // namespace tnad

using namespace tnad;

extern "C" int tnad_mlp_create(tnad_ctx* c, int n_in, int width, int n_out, uint64_t seed, tnad_mlp** out) {
  API_BEGIN(c)
  TNAD_REQUIRE(out && n_in > 0 && width > 0 && n_out > 0 && n_in <= (1 << 20) && width <= (1 << 16) &&
                   n_out <= (1 << 24),
               TNAD_ERR_ARG, "tnad_mlp_create: bad sizes");
  *out = nullptr;
  std::unique_ptr<tnad_mlp> net(new tnad_mlp);
  net->device = c->device;
  net->n_in = n_in;
  net->width = width;
  net->n_out = n_out;
  const int rows[4] = {n_in, width, width, n_out};
  int64_t off = 0;
  for (int l = 0; l < 4; ++l) net->rows[l] = rows[l];
  for (int l = 0; l < 3; ++l) {
    net->off_w[l] = off;
    off += (int64_t)rows[l + 1] * rows[l];
    net->off_b[l] = off;
    off += rows[l + 1];
  }
  net->n_params = off;
  net->P = dev_alloc_f(off);
  net->G = dev_alloc_f(off);
  net->M1 = dev_alloc_f(off);
  net->M2 = dev_alloc_f(off);
  void* red = nullptr;
  TNAD_CK(cudaMalloc(&red, (kRedBlocks + 8) * sizeof(double)));
  net->red = (double*)red;
  // He-uniform weights (bound √(6/fan_in)), zero biases, zero moments
  TNAD_CK(cudaMemsetAsync(net->P, 0, (size_t)off * 4, c->stream));
  TNAD_CK(cudaMemsetAsync(net->G, 0, (size_t)off * 4, c->stream));
  TNAD_CK(cudaMemsetAsync(net->M1, 0, (size_t)off * 4, c->stream));
  TNAD_CK(cudaMemsetAsync(net->M2, 0, (size_t)off * 4, c->stream));
  for (int l = 0; l < 3; ++l) {
    const int64_t nw = (int64_t)rows[l + 1] * rows[l];
    k_init_uniform<<<nblk(nw), 256, 0, c->stream>>>(net->P + net->off_w[l], nw, seed * 3 + (uint64_t)l,
                                                    (float)std::sqrt(6.0 / rows[l]));
    count_launch(c);
  }
  check_launch(c, "mlp_init");
  TNAD_CK(cudaStreamSynchronize(c->stream));
  *out = net.release();
  API_END(c)
}

tnad_mlp::~tnad_mlp() {
  cudaSetDevice(device);
  cudaDeviceSynchronize();
  free_batch_buffers(this);
  for (float* p : {P, G, M1, M2, DX, DY})
    if (p) cudaFree(p);
  if (red) cudaFree(red);
}

extern "C" void tnad_mlp_free(tnad_mlp* net) { delete net; }

extern "C" int64_t tnad_mlp_param_count(const tnad_mlp* net) { return net ? net->n_params : 0; }

extern "C" int tnad_mlp_get_params(tnad_ctx* c, const tnad_mlp* net, float* params) {
  API_BEGIN(c)
  check_net(net);
  TNAD_REQUIRE(params, TNAD_ERR_ARG, "tnad_mlp_get_params: null");
  TNAD_CK(cudaMemcpyAsync(params, net->P, (size_t)net->n_params * 4, cudaMemcpyDeviceToHost, c->stream));
  TNAD_CK(cudaStreamSynchronize(c->stream));
  API_END(c)
}

extern "C" int tnad_mlp_set_params(tnad_ctx* c, tnad_mlp* net, const float* params) {
  API_BEGIN(c)
  check_net(net);
  TNAD_REQUIRE(params, TNAD_ERR_ARG, "tnad_mlp_set_params: null");
  TNAD_CK(cudaMemcpyAsync(net->P, params, (size_t)net->n_params * 4, cudaMemcpyHostToDevice, c->stream));
  TNAD_CK(cudaMemsetAsync(net->M1, 0, (size_t)net->n_params * 4, c->stream));
  TNAD_CK(cudaMemsetAsync(net->M2, 0, (size_t)net->n_params * 4, c->stream));
  net->t = 0;
  TNAD_CK(cudaStreamSynchronize(c->stream));
  API_END(c)
}

extern "C" int tnad_mlp_forward(tnad_ctx* c, tnad_mlp* net, const float* X, int batch, float* Y, int device_ptrs) {
  API_BEGIN(c)
  check_net(net);
  TNAD_REQUIRE(X && Y && batch > 0, TNAD_ERR_ARG, "tnad_mlp_forward: bad arguments");
  ensure_batch(net, batch);
  const bool dev = device_ptrs != 0;
  const float* x = stage(c, net->X, X, (int64_t)net->n_in * batch, dev);
  mlp_forward(c, net, x, batch);
  const size_t bytes = (size_t)net->n_out * batch * 4;
  TNAD_CK(cudaMemcpyAsync(Y, net->H[2], bytes, dev ? cudaMemcpyDeviceToDevice : cudaMemcpyDeviceToHost, c->stream));
  TNAD_CK(cudaStreamSynchronize(c->stream));
  check_tc_errors(c);
  API_END(c)
}

extern "C" int tnad_mlp_gradient(tnad_ctx* c, tnad_mlp* net, const float* X, const float* Y, int batch, float* loss,
                                 float* grad, int device_ptrs) {
  API_BEGIN(c)
  check_net(net);
  TNAD_REQUIRE(X && Y && batch > 0, TNAD_ERR_ARG, "tnad_mlp_gradient: bad arguments");
  ensure_batch(net, batch);
  const bool dev = device_ptrs != 0;
  const float* x = stage(c, net->X, X, (int64_t)net->n_in * batch, dev);
  const float* y = stage(c, net->Y, Y, (int64_t)net->n_out * batch, dev);
  mlp_forward(c, net, x, batch);
  mlp_backward(c, net, x, y, batch);
  if (grad)
    TNAD_CK(cudaMemcpyAsync(grad, net->G, (size_t)net->n_params * 4,
                            dev ? cudaMemcpyDeviceToDevice : cudaMemcpyDeviceToHost, c->stream));
  TNAD_CK(cudaMemcpyAsync(c->h_pin, net->red + kRedBlocks, 8, cudaMemcpyDeviceToHost, c->stream));
  TNAD_CK(cudaStreamSynchronize(c->stream));
  check_tc_errors(c);
  if (loss) *loss = (float)c->h_pin[0];
  API_END(c)
}

extern "C" int tnad_mlp_train_step(tnad_ctx* c, tnad_mlp* net, const float* X, const float* Y, int64_t n_samples,
                                   const int32_t* idx, int batch, float lr, float weight_decay, float* loss,
                                   int device_ptrs) {
  API_BEGIN(c)
  check_net(net);
  const bool resident = !X && !Y;  // the set loaded by tnad_mlp_set_data
  if (resident) {
    TNAD_REQUIRE(net->DX && net->n_data > 0, TNAD_ERR_STATE, "tnad_mlp_train_step: no resident data set");
    n_samples = net->n_data;
  }
  TNAD_REQUIRE(idx && batch > 0 && n_samples > 0 && (resident || (X && Y)), TNAD_ERR_ARG,
               "tnad_mlp_train_step: bad arguments");
  for (int j = 0; j < batch; ++j)
    TNAD_REQUIRE(idx[j] >= 0 && idx[j] < n_samples, TNAD_ERR_ARG, "tnad_mlp_train_step: index out of range");
  ensure_batch(net, batch);
  const bool dev = device_ptrs != 0 || resident;
  WsScope scope(c);
  const float *xs = resident ? net->DX : X, *ys = resident ? net->DY : Y;
  if (!dev) {  // host data: stage the whole set once per call (small sets only)
    float* dx = ws_f(c, (int64_t)net->n_in * n_samples);
    float* dy = ws_f(c, (int64_t)net->n_out * n_samples);
    TNAD_CK(cudaMemcpyAsync(dx, X, (size_t)net->n_in * n_samples * 4, cudaMemcpyHostToDevice, c->stream));
    TNAD_CK(cudaMemcpyAsync(dy, Y, (size_t)net->n_out * n_samples * 4, cudaMemcpyHostToDevice, c->stream));
    xs = dx;
    ys = dy;
  }
  TNAD_CK(cudaMemcpyAsync(net->idx, idx, (size_t)batch * sizeof(int), cudaMemcpyHostToDevice, c->stream));
  k_gather_cols<<<nblk((int64_t)net->n_in * batch), 256, 0, c->stream>>>(xs, net->n_in, net->idx, batch, net->X);
  k_gather_cols<<<nblk((int64_t)net->n_out * batch), 256, 0, c->stream>>>(ys, net->n_out, net->idx, batch, net->Y);
  count_launch(c, 2);
  mlp_forward(c, net, net->X, batch);
  mlp_backward(c, net, net->X, net->Y, batch);
  net->t += 1;
  const float b1 = 0.9f, b2 = 0.999f;
  const float bc1 = 1.f - (float)std::pow(0.9, (double)net->t), bc2 = 1.f - (float)std::pow(0.999, (double)net->t);
  BiasRanges br;
  for (int l = 0; l < 3; ++l) {
    br.lo[l] = net->off_b[l];
    br.hi[l] = net->off_b[l] + net->rows[l + 1];
  }
  k_adamw<<<nblk(net->n_params), 256, 0, c->stream>>>(net->P, net->G, net->M1, net->M2, net->n_params, lr,
                                                      weight_decay, b1, b2, 1e-8f, bc1, bc2, br);
  count_launch(c);
  check_launch(c, "mlp_adamw");
  if (loss) {
    TNAD_CK(cudaMemcpyAsync(c->h_pin, net->red + kRedBlocks, 8, cudaMemcpyDeviceToHost, c->stream));
    TNAD_CK(cudaStreamSynchronize(c->stream));
    check_tc_errors(c);
    *loss = (float)c->h_pin[0];
  } else if (!dev) {
    TNAD_CK(cudaStreamSynchronize(c->stream));  // the staged host data lives in the workspace scope
  }
  API_END(c)
}

extern "C" int tnad_mlp_set_data(tnad_ctx* c, tnad_mlp* net, const float* X, const float* Y, int64_t n_samples) {
  API_BEGIN(c)
  check_net(net);
  TNAD_REQUIRE(n_samples >= 0 && (n_samples == 0 || (X && Y)), TNAD_ERR_ARG, "tnad_mlp_set_data: bad arguments");
  TNAD_CK(cudaStreamSynchronize(c->stream));
  if (net->DX) cudaFree(net->DX);
  if (net->DY) cudaFree(net->DY);
  net->DX = net->DY = nullptr;
  net->n_data = 0;
  if (n_samples > 0) {
    net->DX = dev_alloc_f((int64_t)net->n_in * n_samples);
    net->DY = dev_alloc_f((int64_t)net->n_out * n_samples);
    TNAD_CK(cudaMemcpyAsync(net->DX, X, (size_t)net->n_in * n_samples * 4, cudaMemcpyHostToDevice, c->stream));
    TNAD_CK(cudaMemcpyAsync(net->DY, Y, (size_t)net->n_out * n_samples * 4, cudaMemcpyHostToDevice, c->stream));
    TNAD_CK(cudaStreamSynchronize(c->stream));
    net->n_data = n_samples;
  }
  API_END(c)
}

extern "C" int tnad_env_gauge_fix(tnad_ctx* c, const double* C, const double* T, int chi, int d, double* lam,
                                  double* Tg) {
  API_BEGIN(c)
  TNAD_REQUIRE(C && T && lam && Tg && chi >= 1 && chi <= 256 && d >= 1, TNAD_ERR_ARG, "tnad_env_gauge_fix: arguments");
  WsScope scope(c);
  const int64_t nC = (int64_t)chi * chi, nT = (int64_t)chi * d * chi, cd = (int64_t)chi * d;
  double* dC = ws_d(c, nC);
  double* dT = ws_d(c, nT);
  double* W = ws_d(c, nC);
  double* dl = ws_d(c, chi);
  double* X1 = ws_d(c, nT);
  double* dTg = ws_d(c, nT);
  TNAD_CK(cudaMemcpyAsync(dC, C, nC * 8, cudaMemcpyHostToDevice, c->stream));
  TNAD_CK(cudaMemcpyAsync(dT, T, nT * 8, cudaMemcpyHostToDevice, c->stream));
  eigh_small(c, dC, chi, W, dl);  // |λ| descending
  // X1 (χ × dχ) = Wᵀ·T ; Tg ((χd) × χ) = X1·W
  gemm_f64(c, 'T', 'N', chi, cd, chi, 1.0, W, chi, dT, chi, 0.0, X1, chi);
  gemm_f64(c, 'N', 'N', cd, chi, chi, 1.0, X1, cd, W, chi, 0.0, dTg, cd);
  k_gauge_signs<<<1, 256, (size_t)chi * 8, c->stream>>>(dTg, chi, d);
  count_launch(c);
  check_launch(c, "gauge_fix");
  TNAD_CK(cudaMemcpyAsync(lam, dl, (size_t)chi * 8, cudaMemcpyDeviceToHost, c->stream));
  TNAD_CK(cudaMemcpyAsync(Tg, dTg, (size_t)nT * 8, cudaMemcpyDeviceToHost, c->stream));
  TNAD_CK(cudaStreamSynchronize(c->stream));
  API_END(c)
}

extern "C" int tnad_ctx_set_warm_start(tnad_ctx* c, tnad_mlp* net, int D, int s, int chi) {
  API_BEGIN(c)
  if (net) {
    TNAD_REQUIRE(D >= 1 && s >= 1 && chi >= 1, TNAD_ERR_ARG, "tnad_ctx_set_warm_start: sizes");
    const int64_t d = (int64_t)D * D;
    TNAD_REQUIRE(net->n_in == d * d * s && net->n_out == chi + chi * d * chi, TNAD_ERR_SHAPE,
                 "tnad_ctx_set_warm_start: network shape does not match (D, s, χ)");
  }
  c->warm_net = net;
  c->warm_D = net ? D : 0;
  c->warm_s = net ? s : 0;
  c->warm_chi = net ? chi : 0;
  c->warm_status = 0;
  API_END(c)
}

extern "C" int tnad_warm_start_features(tnad_ctx* c, const double* A, int D, int s, float* x) {
  API_BEGIN(c)
  TNAD_REQUIRE(A && x && D >= 1 && s >= 1, TNAD_ERR_ARG, "tnad_warm_start_features: arguments");
  WsScope scope(c);
  const int64_t nA = (int64_t)D * D * D * D * s;
  double* dA = ws_d(c, nA);
  double* As = ws_d(c, nA);
  double* nrm = ws_d(c, 1);
  float* fx = ws_f(c, nA);
  TNAD_CK(cudaMemcpyAsync(dA, A, nA * 8, cudaMemcpyHostToDevice, c->stream));
  symmetrize_fwd(c, dA, D, s, As, nrm);
  k_features<<<1, 256, 0, c->stream>>>(As, (int)nA, fx);
  count_launch(c);
  check_launch(c, "features");
  TNAD_CK(cudaMemcpyAsync(x, fx, nA * 4, cudaMemcpyDeviceToHost, c->stream));
  TNAD_CK(cudaStreamSynchronize(c->stream));
  API_END(c)
}

extern "C" int tnad_warm_start_env(tnad_ctx* c, const double* A, int D, int s, int chi, double* C, double* T) {
  API_BEGIN(c)
  TNAD_REQUIRE(A && C && T, TNAD_ERR_ARG, "tnad_warm_start_env: null");
  TNAD_REQUIRE(c->warm_net && c->warm_D == D && c->warm_s == s && c->warm_chi == chi, TNAD_ERR_STATE,
               "tnad_warm_start_env: no network attached for this (D, s, χ)");
  WsScope scope(c);
  const int d = D * D;
  const int64_t nA = (int64_t)D * D * D * D * s, nC = (int64_t)chi * chi, nT = (int64_t)chi * d * chi;
  double* dA = ws_d(c, nA);
  double* As = ws_d(c, nA);
  double* nrm = ws_d(c, 1);
  double* dC = ws_d(c, nC);
  double* dT = ws_d(c, nT);
  TNAD_CK(cudaMemcpyAsync(dA, A, nA * 8, cudaMemcpyHostToDevice, c->stream));
  symmetrize_fwd(c, dA, D, s, As, nrm);
  TNAD_REQUIRE(warm_start_predict(c, c->warm_net, As, (int)nA, chi, d, dC, dT), TNAD_ERR_NONFINITE,
               "tnad_warm_start_env: the network predicts a zero or non-finite environment");
  TNAD_CK(cudaMemcpyAsync(C, dC, nC * 8, cudaMemcpyDeviceToHost, c->stream));
  TNAD_CK(cudaMemcpyAsync(T, dT, nT * 8, cudaMemcpyDeviceToHost, c->stream));
  TNAD_CK(cudaStreamSynchronize(c->stream));
  check_tc_errors(c);
  API_END(c)
}

extern "C" int tnad_ctx_warm_start_status(const tnad_ctx* c) { return c ? c->warm_status : 0; }

extern "C" int tnad_gemm_bf16(tnad_ctx* c, char ta, char tb, int64_t M, int64_t N, int64_t K, float alpha,
                              const float* A, int64_t lda, const float* B, int64_t ldb, float beta, float* Cm,
                              int64_t ldc) {
  API_BEGIN(c)
  TNAD_REQUIRE(A && B && Cm && M >= 1 && N >= 1 && K >= 1, TNAD_ERR_ARG, "tnad_gemm_bf16: bad arguments");
  const bool at = (ta == 'T' || ta == 't'), bt = (tb == 'T' || tb == 't');
  TNAD_REQUIRE(lda >= (at ? K : M) && ldb >= (bt ? N : K) && ldc >= M, TNAD_ERR_ARG, "tnad_gemm_bf16: leading dims");
  WsScope scope(c);
  const int64_t na = at ? lda * M : lda * K, nb = bt ? ldb * K : ldb * N;
  float* dA = ws_f(c, na);
  float* dB = ws_f(c, nb);
  float* dC = ws_f(c, ldc * N);
  TNAD_CK(cudaMemcpyAsync(dA, A, (size_t)na * 4, cudaMemcpyHostToDevice, c->stream));
  TNAD_CK(cudaMemcpyAsync(dB, B, (size_t)nb * 4, cudaMemcpyHostToDevice, c->stream));
  TNAD_CK(cudaMemcpyAsync(dC, Cm, (size_t)ldc * N * 4, cudaMemcpyHostToDevice, c->stream));
  gemm_bf16(c, ta, tb, M, N, K, alpha, dA, lda, dB, ldb, beta, dC, ldc);
  TNAD_CK(cudaMemcpyAsync(Cm, dC, (size_t)ldc * N * 4, cudaMemcpyDeviceToHost, c->stream));
  TNAD_CK(cudaStreamSynchronize(c->stream));
  check_tc_errors(c);
  API_END(c)
}
