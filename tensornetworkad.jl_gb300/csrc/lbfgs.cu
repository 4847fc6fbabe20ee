// optimiseipeps (src/variationalipeps.jl:67-75) inside the library: L-BFGS
// with m correction pairs over the site tensor, every evaluation the energy and
// its gradient of this library (energy_fwd/energy_bwd, options as for
// tnad_energy).  The iterate, gradient and the m pairs (s_k, y_k) stay on the
// device; the two-loop recursion runs in one CTA (the vectors hold D⁴·s
// values), so an iteration exchanges only scalars with the host: the energy of
// each line-search trial and gᵀd.  The line search backtracks from the unit
// step (the first iteration from 1/‖g‖∞) until the Armijo condition holds,
// halving the step; a pair with sᵀy ≤ 0 is not stored.  Optim's LBFGS (the
// reference) uses the Hager–Zhang line search instead, so trajectories differ
// while the minima they reach agree (tested on the reference's cases).
#include <cmath>
#include <cstring>
#include <memory>
#include <vector>

#include "tnad_api.h"
#include "tnad_energy.h"

namespace tnad {

namespace {

constexpr int kThreads = 512;

__device__ double block_sum(double v, double* red) {
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
  __syncthreads();
  if (lane == 0) red[w] = v;
  __syncthreads();
  double t = 0.0;
  for (int k = 0; k < (int)(blockDim.x >> 5); ++k) t += red[k];  // fixed order: deterministic
  return t;
}

// d = −H·g by the two-loop recursion over the stored pairs (oldest first in the
// ring at positions (first + i) mod m, i < cnt); out[0] = gᵀd.  One CTA.
__global__ void __launch_bounds__(kThreads) k_lbfgs_dir(const double* __restrict__ g, const double* __restrict__ S,
                                                        const double* __restrict__ Y, const double* __restrict__ rho,
                                                        int m, int first, int cnt, int64_t n, double gamma0,
                                                        double* __restrict__ q, double* __restrict__ alpha,
                                                        double* __restrict__ d, double* __restrict__ out) {
  __shared__ double red[32];
  for (int64_t e = threadIdx.x; e < n; e += blockDim.x) q[e] = g[e];
  __syncthreads();
  for (int i = cnt - 1; i >= 0; --i) {
    const int slot = (first + i) % m;
    const double* s = S + (int64_t)slot * n;
    const double* y = Y + (int64_t)slot * n;
    double p = 0.0;
    for (int64_t e = threadIdx.x; e < n; e += blockDim.x) p += s[e] * q[e];
    const double a = rho[slot] * block_sum(p, red);
    if (threadIdx.x == 0) alpha[slot] = a;
    for (int64_t e = threadIdx.x; e < n; e += blockDim.x) q[e] -= a * y[e];
    __syncthreads();
  }
  double gamma = gamma0;
  if (cnt > 0) {
    const int last = (first + cnt - 1) % m;
    const double* s = S + (int64_t)last * n;
    const double* y = Y + (int64_t)last * n;
    double sy = 0.0, yy = 0.0;
    for (int64_t e = threadIdx.x; e < n; e += blockDim.x) {
      sy += s[e] * y[e];
      yy += y[e] * y[e];
    }
    sy = block_sum(sy, red);
    yy = block_sum(yy, red);
    gamma = sy / yy;
  }
  for (int64_t e = threadIdx.x; e < n; e += blockDim.x) q[e] *= gamma;
  __syncthreads();
  for (int i = 0; i < cnt; ++i) {
    const int slot = (first + i) % m;
    const double* s = S + (int64_t)slot * n;
    const double* y = Y + (int64_t)slot * n;
    double p = 0.0;
    for (int64_t e = threadIdx.x; e < n; e += blockDim.x) p += y[e] * q[e];
    const double b = rho[slot] * block_sum(p, red);
    const double a = alpha[slot];
    for (int64_t e = threadIdx.x; e < n; e += blockDim.x) q[e] += (a - b) * s[e];
    __syncthreads();
  }
  double gd = 0.0;
  for (int64_t e = threadIdx.x; e < n; e += blockDim.x) {
    d[e] = -q[e];
    gd -= g[e] * q[e];
  }
  gd = block_sum(gd, red);
  if (threadIdx.x == 0) out[0] = gd;
}

// xt = x + a·d (one CTA)
__global__ void __launch_bounds__(kThreads) k_lbfgs_trial(const double* __restrict__ x, const double* __restrict__ d,
                                                          double a, int64_t n, double* __restrict__ xt) {
  for (int64_t e = threadIdx.x; e < n; e += blockDim.x) xt[e] = x[e] + a * d[e];
}

// stores the pair s = xt − x, y = gt − g in the slot, rho = 1/sᵀy (out[0] = sᵀy,
// out[1] = max|gt|); the caller keeps it only when sᵀy > 0
__global__ void __launch_bounds__(kThreads) k_lbfgs_pair(const double* __restrict__ x, const double* __restrict__ xt,
                                                         const double* __restrict__ g, const double* __restrict__ gt,
                                                         int64_t n, double* __restrict__ s, double* __restrict__ y,
                                                         double* __restrict__ rho_slot, double* __restrict__ out) {
  __shared__ double red[32];
  double sy = 0.0, gm = 0.0;
  for (int64_t e = threadIdx.x; e < n; e += blockDim.x) {
    const double se = xt[e] - x[e], ye = gt[e] - g[e];
    s[e] = se;
    y[e] = ye;
    sy += se * ye;
    gm = fmax(gm, fabs(gt[e]));
  }
  sy = block_sum(sy, red);
  for (int o = 16; o > 0; o >>= 1) gm = fmax(gm, __shfl_xor_sync(0xffffffffu, gm, o));
  __syncthreads();
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = gm;
  __syncthreads();
  if (threadIdx.x == 0) {
    double t = 0.0;
    for (int k = 0; k < (int)(blockDim.x >> 5); ++k) t = fmax(t, red[k]);
    rho_slot[0] = sy > 0.0 ? 1.0 / sy : 0.0;
    out[0] = sy;
    out[1] = t;
  }
}

__global__ void k_maxabs_one(const double* __restrict__ v, int64_t n, double* __restrict__ out) {
  __shared__ double red[32];
  double m = 0.0;
  for (int64_t e = threadIdx.x; e < n; e += blockDim.x) m = fmax(m, fabs(v[e]));
  for (int o = 16; o > 0; o >>= 1) m = fmax(m, __shfl_xor_sync(0xffffffffu, m, o));
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = m;
  __syncthreads();
  if (threadIdx.x == 0) {
    double t = 0.0;
    for (int k = 0; k < (int)(blockDim.x >> 5); ++k) t = fmax(t, red[k]);
    out[0] = t;
  }
}

// energy and gradient at x (device arrays), E returned
double eval_energy(tnad_ctx* c, const double* h, const double* x, int D, int s, int chi, double tol, int maxit,
                   const tnad_opts& o, double* g) {
  EnergyTape tp;
  energy_fwd(c, tp, h, x, D, s, chi, tol, maxit, o, nullptr, nullptr, true);
  energy_bwd(c, tp, 1.0, g);
  TNAD_CK(cudaStreamSynchronize(c->stream));
  return tp.E;
}

double read_scalar(tnad_ctx* c, const double* dev, int k = 0) {
  TNAD_CK(cudaMemcpyAsync(c->h_pin, dev, (k + 1) * sizeof(double), cudaMemcpyDeviceToHost, c->stream));
  TNAD_CK(cudaStreamSynchronize(c->stream));
  return c->h_pin[k];
}

}  // namespace

}  // namespace tnad

using namespace tnad;

extern "C" int tnad_optimiseipeps(tnad_ctx* c, const double* h, double* A, int D, int s, int chi, double tol,
                                  int maxit, const tnad_opts* opts, int m, int iterations, double f_tol, double g_tol,
                                  double* E_out, int* iters_out, int* evals_out) {
  API_BEGIN(c)
  TNAD_REQUIRE(h && A && D >= 1 && s >= 1 && chi >= 1 && maxit >= 0 && m >= 1 && iterations >= 0, TNAD_ERR_ARG,
               "tnad_optimiseipeps: bad arguments");
  tnad_opts o;
  tnad_opts_default(&o);
  if (opts) o = *opts;
  const bool dev = o.device_ptrs != 0;
  o.device_ptrs = 1;
  o.warm_start = TNAD_WARM_NONE;  // every evaluation starts CTMRG from :raw, as the reference does
  const int64_t n = (int64_t)D * D * D * D * s;
  WsScope scope(c);
  double* dh = ws_d(c, (int64_t)s * s * s * s);
  double* x = ws_d(c, n);
  double* xt = ws_d(c, n);
  double* g = ws_d(c, n);
  double* gt = ws_d(c, n);
  double* d = ws_d(c, n);
  double* q = ws_d(c, n);
  double* S = ws_d(c, (int64_t)m * n);
  double* Y = ws_d(c, (int64_t)m * n);
  double* rho = ws_d(c, m);
  double* alpha = ws_d(c, m);
  double* sc = ws_d(c, 4);
  TNAD_CK(cudaMemcpyAsync(dh, h, (size_t)s * s * s * s * 8, dev ? cudaMemcpyDeviceToDevice : cudaMemcpyHostToDevice,
                          c->stream));
  TNAD_CK(cudaMemcpyAsync(x, A, (size_t)n * 8, dev ? cudaMemcpyDeviceToDevice : cudaMemcpyHostToDevice, c->stream));
  int evals = 0, it = 0, first = 0, cnt = 0;
  double f = eval_energy(c, dh, x, D, s, chi, tol, maxit, o, g);
  ++evals;
  TNAD_REQUIRE(std::isfinite(f), TNAD_ERR_NONFINITE, "optimiseipeps: non-finite energy at the start");
  k_maxabs_one<<<1, kThreads, 0, c->stream>>>(g, n, sc + 2);
  count_launch(c);
  double gmax = read_scalar(c, sc, 2);
  const double c1 = 1e-4;
  for (it = 0; it < iterations && gmax > g_tol; ++it) {
    k_lbfgs_dir<<<1, kThreads, 0, c->stream>>>(g, S, Y, rho, m, first, cnt, n, 1.0, q, alpha, d, sc);
    count_launch(c);
    double gd = read_scalar(c, sc);
    if (!(gd < 0.0)) {  // not a descent direction: forget the pairs, steepest descent
      cnt = 0;
      k_lbfgs_dir<<<1, kThreads, 0, c->stream>>>(g, S, Y, rho, m, first, 0, n, 1.0, q, alpha, d, sc);
      count_launch(c);
      gd = read_scalar(c, sc);
    }
    double a = cnt == 0 ? std::min(1.0, 1.0 / std::max(gmax, 1e-300)) : 1.0;
    bool accepted = false;
    double ft = f;
    for (int ls = 0; ls < 40; ++ls) {
      k_lbfgs_trial<<<1, kThreads, 0, c->stream>>>(x, d, a, n, xt);
      count_launch(c);
      ft = eval_energy(c, dh, xt, D, s, chi, tol, maxit, o, gt);
      ++evals;
      if (std::isfinite(ft) && ft <= f + c1 * a * gd) {
        accepted = true;
        break;
      }
      a *= 0.5;
    }
    if (!accepted) break;  // the line search found no decrease: a stationary point to this precision
    const int slot = (first + cnt) % m;
    k_lbfgs_pair<<<1, kThreads, 0, c->stream>>>(x, xt, g, gt, n, S + (int64_t)slot * n, Y + (int64_t)slot * n,
                                                rho + slot, sc);
    count_launch(c);
    TNAD_CK(cudaMemcpyAsync(c->h_pin, sc, 2 * sizeof(double), cudaMemcpyDeviceToHost, c->stream));
    TNAD_CK(cudaStreamSynchronize(c->stream));
    const double sy = c->h_pin[0];
    gmax = c->h_pin[1];
    if (sy > 0.0) {
      if (cnt < m)
        ++cnt;
      else
        first = (first + 1) % m;
    }
    copy_d2d(c, x, xt, n);
    copy_d2d(c, g, gt, n);
    const double fold = f;
    f = ft;
    if (std::fabs(fold - f) <= f_tol * std::fabs(f)) {
      ++it;
      break;
    }
  }
  TNAD_CK(cudaMemcpyAsync(A, x, (size_t)n * 8, dev ? cudaMemcpyDeviceToDevice : cudaMemcpyDeviceToHost, c->stream));
  TNAD_CK(cudaStreamSynchronize(c->stream));
  TNAD_CK(cudaGetLastError());
  if (E_out) *E_out = f;
  if (iters_out) *iters_out = it;
  if (evals_out) *evals_out = evals;
  API_END(c)
}
