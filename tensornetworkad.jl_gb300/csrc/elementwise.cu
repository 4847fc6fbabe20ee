// HBM-bound elementwise, permutation and reduction kernels of libtnad.
// Reductions are deterministic: fixed grid, fixed per-thread order, warp-shuffle
// trees, then one block sums the partials in index order.
#include "tnad_internal.h"

namespace tnad {

static inline int nblocks(int64_t n, int threads, int cap = 4096) {
  int64_t b = (n + threads - 1) / threads;
  if (b < 1) b = 1;
  if (b > cap) b = cap;
  return (int)b;
}

__global__ void k_fill(double* x, int64_t n, double v) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) x[i] = v;
}

__global__ void k_axpby(int64_t n, double a, const double* __restrict__ x, double b, double* __restrict__ y) {
  // float4-style vectorisation: two doubles per 16-byte access when aligned
  int64_t tid = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  int64_t stride = (int64_t)gridDim.x * blockDim.x;
  bool al = ((((uintptr_t)x) | ((uintptr_t)y)) & 15) == 0;
  if (al) {
    int64_t n2 = n / 2;
    const double2* x2 = reinterpret_cast<const double2*>(x);
    double2* y2 = reinterpret_cast<double2*>(y);
    for (int64_t i = tid; i < n2; i += stride) {
      double2 xv = x2[i];
      double2 yv = b == 0.0 ? make_double2(0.0, 0.0) : y2[i];
      y2[i] = make_double2(a * xv.x + b * yv.x, a * xv.y + b * yv.y);
    }
    if (tid == 0 && (n & 1)) y[n - 1] = a * x[n - 1] + (b == 0.0 ? 0.0 : b * y[n - 1]);
  } else {
    for (int64_t i = tid; i < n; i += stride) y[i] = a * x[i] + (b == 0.0 ? 0.0 : b * y[i]);
  }
}

__global__ void k_scale(int64_t n, double a, double* x) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) x[i] *= a;
}

// out = x + xᵀ, 32×32 tiles through shared memory so both reads coalesce.
__global__ void k_add_transpose(int64_t n, const double* __restrict__ x, double* __restrict__ out) {
  __shared__ double tile[32][33];
  int64_t bi = blockIdx.x * 32, bj = blockIdx.y * 32;
  int tx = threadIdx.x, ty = threadIdx.y;  // 32 × 8
  // load tile (bj.., bi..) of x transposed into shared: tile[c][r] = x[bj + r, bi + c]
  for (int r = ty; r < 32; r += 8) {
    int64_t row = bj + tx, col = bi + r;
    tile[r][tx] = (row < n && col < n) ? x[row + col * n] : 0.0;  // x[bj+tx, bi+r]
  }
  __syncthreads();
  for (int r = ty; r < 32; r += 8) {
    int64_t row = bi + tx, col = bj + r;
    if (row < n && col < n) out[row + col * n] = x[row + col * n] + tile[tx][r];
  }
}

struct PermArgs {
  int nd;
  int64_t odim[10];
  int64_t istr[10];  // input stride of the input axis that becomes output axis k
};

__global__ void k_permute(PermArgs a, int64_t n, const double* __restrict__ in, double* __restrict__ out,
                          double alpha, double beta) {
  for (int64_t o = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; o < n; o += (int64_t)gridDim.x * blockDim.x) {
    int64_t rem = o, off = 0;
#pragma unroll
    for (int k = 0; k < 10; ++k) {
      if (k < a.nd) {
        int64_t ck = rem % a.odim[k];
        rem /= a.odim[k];
        off += ck * a.istr[k];
      }
    }
    double v = alpha * in[off];
    out[o] = beta == 0.0 ? v : v + beta * out[o];
  }
}

// ---- reductions ----
__device__ __forceinline__ double warp_sum(double v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
  return v;
}

template <int MODE>  // 0: Σx², 1: Σx·y
__global__ void k_reduce_partial(const double* __restrict__ x, const double* __restrict__ y, int64_t n,
                                 double* __restrict__ part) {
  double s = 0.0;
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    double v = x[i];
    s += MODE == 0 ? v * v : v * y[i];
  }
  __shared__ double sh[32];
  s = warp_sum(s);
  int w = threadIdx.x >> 5, l = threadIdx.x & 31;
  if (l == 0) sh[w] = s;
  __syncthreads();
  if (w == 0) {
    double t = l < (int)(blockDim.x >> 5) ? sh[l] : 0.0;
    t = warp_sum(t);
    if (l == 0) part[blockIdx.x] = t;
  }
}

// out[0] = Σ part[0..np); if sqrt_to != null also writes sqrt into sqrt_to[0]
__global__ void k_reduce_final(const double* __restrict__ part, int np, double* out, double* sqrt_to) {
  double s = 0.0;
  for (int i = threadIdx.x; i < np; i += blockDim.x) s += part[i];
  __shared__ double sh[32];
  s = warp_sum(s);
  int w = threadIdx.x >> 5, l = threadIdx.x & 31;
  if (l == 0) sh[w] = s;
  __syncthreads();
  if (w == 0) {
    double t = l < (int)(blockDim.x >> 5) ? sh[l] : 0.0;
    t = warp_sum(t);
    if (l == 0) {
      out[0] = t;
      if (sqrt_to) sqrt_to[0] = sqrt(t);
    }
  }
}

__global__ void k_maxabs_partial(const double* __restrict__ x, int64_t n, double* part_v, double* part_i) {
  double best = -1.0;
  int64_t bi = 0;
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    double v = fabs(x[i]);
    if (v > best) { best = v; bi = i; }
  }
  // block argmax with first-index tie break
  __shared__ double sv[256];
  __shared__ int64_t si[256];
  sv[threadIdx.x] = best;
  si[threadIdx.x] = bi;
  __syncthreads();
  for (int s = blockDim.x / 2; s > 0; s >>= 1) {
    if (threadIdx.x < s) {
      double v2 = sv[threadIdx.x + s];
      int64_t i2 = si[threadIdx.x + s];
      if (v2 > sv[threadIdx.x] || (v2 == sv[threadIdx.x] && i2 < si[threadIdx.x])) {
        sv[threadIdx.x] = v2;
        si[threadIdx.x] = i2;
      }
    }
    __syncthreads();
  }
  if (threadIdx.x == 0) {
    part_v[blockIdx.x] = sv[0];
    part_i[blockIdx.x] = (double)si[0];
  }
}

__global__ void k_maxabs_final(const double* part_v, const double* part_i, int np, double* out) {
  if (threadIdx.x == 0) {
    double best = -1.0, bi = 0.0;
    for (int i = 0; i < np; ++i) {
      double v = part_v[i];
      if (v > best || (v == best && part_i[i] < bi)) { best = v; bi = part_i[i]; }
    }
    out[0] = best;
    out[1] = bi;
  }
}

__global__ void k_div_by_dev(double* x, int64_t n, const double* s) {
  double inv = 1.0 / s[0];
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) x[i] *= inv;
}

// ----------------------------------------------------------------------------

void fill(tnad_ctx* c, double* x, int64_t n, double v) {
  if (n <= 0) return;
  k_fill<<<nblocks(n, 256), 256, 0, c->stream>>>(x, n, v);
  count_launch(c);
  check_launch(c, "fill");
}

void copy_d2d(tnad_ctx* c, double* dst, const double* src, int64_t n) {
  if (n <= 0 || dst == src) return;
  TNAD_CK(cudaMemcpyAsync(dst, src, n * 8, cudaMemcpyDeviceToDevice, c->stream));
}

void axpby(tnad_ctx* c, int64_t n, double a, const double* x, double b, double* y) {
  if (n <= 0) return;
  k_axpby<<<nblocks(n / 2 + 1, 256), 256, 0, c->stream>>>(n, a, x, b, y);
  count_launch(c);
  check_launch(c, "axpby");
}

void scale(tnad_ctx* c, int64_t n, double a, double* x) {
  if (n <= 0) return;
  k_scale<<<nblocks(n, 256), 256, 0, c->stream>>>(n, a, x);
  count_launch(c);
  check_launch(c, "scale");
}

void add_transpose(tnad_ctx* c, int64_t n, const double* x, double* out) {
  if (n <= 0) return;
  dim3 g((unsigned)((n + 31) / 32), (unsigned)((n + 31) / 32)), b(32, 8);
  k_add_transpose<<<g, b, 0, c->stream>>>(n, x, out);
  count_launch(c);
  check_launch(c, "add_transpose");
}

void permute(tnad_ctx* c, const Ten& in, const int* perm, double* out, double alpha, double beta) {
  PermArgs a;
  a.nd = in.nd;
  int64_t istr[10];
  int64_t s = 1;
  for (int k = 0; k < in.nd; ++k) {
    istr[k] = s;
    s *= in.dim[k];
  }
  bool ident = true;
  for (int k = 0; k < in.nd; ++k) {
    a.odim[k] = in.dim[perm[k]];
    a.istr[k] = istr[perm[k]];
    if (perm[k] != k) ident = false;
  }
  for (int k = in.nd; k < 10; ++k) {
    a.odim[k] = 1;
    a.istr[k] = 0;
  }
  int64_t n = in.numel();
  if (n <= 0) return;
  if (ident) {
    if (beta == 0.0 && alpha == 1.0) {
      copy_d2d(c, out, in.p, n);
    } else {
      axpby(c, n, alpha, in.p, beta, out);
    }
    return;
  }
  k_permute<<<nblocks(n, 256, 8192), 256, 0, c->stream>>>(a, n, in.p, out, alpha, beta);
  count_launch(c);
  check_launch(c, "permute");
}

static void reduce2(tnad_ctx* c, int mode, const double* x, const double* y, int64_t n, double* out,
                    double* sqrt_to) {
  int nb = nblocks(n, 256, 1024);
  double* part = c->d_red + 2048;
  if (mode == 0)
    k_reduce_partial<0><<<nb, 256, 0, c->stream>>>(x, y, n, part);
  else
    k_reduce_partial<1><<<nb, 256, 0, c->stream>>>(x, y, n, part);
  k_reduce_final<<<1, 256, 0, c->stream>>>(part, nb, out, sqrt_to);
  count_launch(c, 2);
  check_launch(c, "reduce");
}

void sumsq_dev(tnad_ctx* c, const double* x, int64_t n, double* dev_out) { reduce2(c, 0, x, nullptr, n, dev_out, nullptr); }

void dot_dev(tnad_ctx* c, const double* x, const double* y, int64_t n, double* dev_out) {
  reduce2(c, 1, x, y, n, dev_out, nullptr);
}

double norm_host(tnad_ctx* c, const double* x, int64_t n) {
  reduce2(c, 0, x, nullptr, n, c->d_red, c->d_red + 1);
  TNAD_CK(cudaMemcpyAsync(c->h_pin, c->d_red + 1, 8, cudaMemcpyDeviceToHost, c->stream));
  TNAD_CK(cudaStreamSynchronize(c->stream));
  return c->h_pin[0];
}

double dot_host(tnad_ctx* c, const double* x, const double* y, int64_t n) {
  reduce2(c, 1, x, y, n, c->d_red, nullptr);
  TNAD_CK(cudaMemcpyAsync(c->h_pin, c->d_red, 8, cudaMemcpyDeviceToHost, c->stream));
  TNAD_CK(cudaStreamSynchronize(c->stream));
  return c->h_pin[0];
}

void maxabs_dev(tnad_ctx* c, const double* x, int64_t n, double* dev_out) {
  int nb = nblocks(n, 256, 1024);
  double* pv = c->d_red + 2048;
  double* pi = c->d_red + 3072;
  k_maxabs_partial<<<nb, 256, 0, c->stream>>>(x, n, pv, pi);
  k_maxabs_final<<<1, 32, 0, c->stream>>>(pv, pi, nb, dev_out);
  count_launch(c, 2);
  check_launch(c, "maxabs");
}

void div_by_dev(tnad_ctx* c, double* x, int64_t n, const double* dev_s) {
  if (n <= 0) return;
  k_div_by_dev<<<nblocks(n, 256), 256, 0, c->stream>>>(x, n, dev_s);
  count_launch(c);
  check_launch(c, "div_by_dev");
}

void normalize_inplace(tnad_ctx* c, double* x, int64_t n, double* dev_norm_out) {
  int nb = nblocks(n, 256, 1024);
  double* part = c->d_red + 2048;
  k_reduce_partial<0><<<nb, 256, 0, c->stream>>>(x, nullptr, n, part);
  k_reduce_final<<<1, 256, 0, c->stream>>>(part, nb, c->d_red + 8, dev_norm_out);
  count_launch(c, 2);
  div_by_dev(c, x, n, dev_norm_out);
}

}  // namespace tnad
