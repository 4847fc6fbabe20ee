// SVD adjoint of src/trg.jl:72-105 (real case).  The Lorentzian-broadened
// F-matrix F_ij = (s_j²−s_i²)/((s_j²−s_i²)²+η) is formed in FP64 inside the
// kernel that assembles res = (J+Jᵀ)S + S(K+Kᵀ) + diag(dS); the surrounding
// products Uᵀ·dU, Vᵀ·dV, U·res·Vᵀ are GEMMs.
#include "tnad_internal.h"

namespace tnad {

__global__ void k_svdback_res(int64_t n, const double* __restrict__ S, const double* __restrict__ X,
                              const double* __restrict__ Y, const double* __restrict__ dS, double eta,
                              double* __restrict__ res) {
  int64_t nn = n * n;
  for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < nn; e += (int64_t)gridDim.x * blockDim.x) {
    int64_t i = e % n, j = e / n;
    double si = S[i], sj = S[j];
    // Explicitly rounded operations (no FMA contraction): the reference forms
    // S2 = S.^2 first, so F_ii is exactly 0 and F_ji = −F_ij exactly; a fused
    // sj*sj − si*si would leave a rounding residue whose 1/d blows up.
    double d = __dsub_rn(__dmul_rn(sj, sj), __dmul_rn(si, si));  // S2' .- S2
    double f = __ddiv_rn(d, __dadd_rn(__dmul_rn(d, d), eta));     // F_ij ; F_ji = −f
    double r = 0.0;
    if (X) r = __dadd_rn(r, __dmul_rn(__dadd_rn(__dmul_rn(f, X[i + j * n]), __dmul_rn(-f, X[j + i * n])), sj));
    if (Y) r = __dadd_rn(r, __dmul_rn(si, __dadd_rn(__dmul_rn(f, Y[i + j * n]), __dmul_rn(-f, Y[j + i * n]))));
    if (dS && i == j) r = __dadd_rn(r, dS[i]);
    res[e] = r;
  }
}

__global__ void k_scale_cols(int64_t m, int64_t n, double* __restrict__ P, const double* __restrict__ S, double eta) {
  int64_t mn = m * n;
  for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < mn; e += (int64_t)gridDim.x * blockDim.x) {
    double s = S[e / m];
    P[e] *= s / (s * s + eta);
  }
}

// res blocks of svd_back when only the first k columns of dU are non-zero (and
// dS = dV = nothing): with Xk = Uᵀ·dU[:, 1:k],
//   R1[i,j] = F_ij·(Xk[i,j] − [i<k]·Xk[j,i])·s_j      (all i, j < k)
//   R2[i,j] = −F_ij·Xk[j,i]·s_j                       (i < k, j ≥ k; stored at j−k)
// kept_sym: the caller's dU makes the kept block Xk[1:k, 1:k] symmetric, so
// R1's kept block is exactly 0 and is set so (rounding in its antisymmetric part
// would otherwise be multiplied by F_ij of (near-)degenerate kept pairs).
__global__ void k_svdback_cols(int64_t n, int64_t k, const double* __restrict__ S, const double* __restrict__ Xk,
                               double eta, int kept_sym, double* __restrict__ R1, double* __restrict__ R2) {
  const int64_t n1 = n * k, n2 = k * (n - k);
  for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < n1 + n2; e += (int64_t)gridDim.x * blockDim.x) {
    int64_t i, j;
    if (e < n1) {
      i = e % n;
      j = e / n;
    } else {
      const int64_t f = e - n1;
      i = f % k;
      j = k + f / k;
    }
    const double si = S[i], sj = S[j];
    const double d = __dsub_rn(__dmul_rn(sj, sj), __dmul_rn(si, si));
    const double fij = __ddiv_rn(d, __dadd_rn(__dmul_rn(d, d), eta));
    if (e < n1) {
      if (kept_sym && i < k) {
        R1[e] = 0.0;
        continue;
      }
      const double xij = Xk[i + j * n];
      const double xji = i < k ? Xk[j + i * n] : 0.0;
      R1[e] = __dmul_rn(__dadd_rn(__dmul_rn(fij, xij), __dmul_rn(-fij, xji)), sj);
    } else {
      R2[e - n1] = __dmul_rn(__dmul_rn(-fij, Xk[j + i * n]), sj);
    }
  }
}

// svd_back for a square thin SVD with dU = [dUk, 0] (k leading columns), dS = dV = nothing.
void svd_back_cols(tnad_ctx* c, int prec, const double* U, const double* S, const double* V, int64_t n, int64_t k,
                   const double* dUk, double eta, double* dA, bool kept_sym) {
  WsScope scope(c);
  double* Xk = ws_d(c, n * k);
  gemm(c, prec, 'T', 'N', n, k, n, 1.0, U, n, dUk, n, 0.0, Xk, n);
  double* R1 = ws_d(c, n * k);
  double* R2 = ws_d(c, k * (n - k) + 1);
  const int64_t tot = n * k + k * (n - k);
  k_svdback_cols<<<(int)std::min<int64_t>((tot + 255) / 256, 4096), 256, 0, c->stream>>>(n, k, S, Xk, eta, kept_sym ? 1 : 0, R1, R2);
  count_launch(c);
  check_launch(c, "svdback_cols");
  // dA = (U·R1)·V[:, 1:k]ᵀ + U[:, 1:k]·(R2·V[:, k+1:n]ᵀ)
  double* A1 = ws_d(c, n * k);
  gemm(c, prec, 'N', 'N', n, k, n, 1.0, U, n, R1, n, 0.0, A1, n);
  gemm(c, prec, 'N', 'T', n, n, k, 1.0, A1, n, V, n, 0.0, dA, n);
  if (n > k) {
    double* B2 = ws_d(c, k * n);
    gemm(c, prec, 'N', 'T', k, n, n - k, 1.0, R2, k, V + k * n, n, 0.0, B2, k);
    gemm(c, prec, 'N', 'N', n, n, k, 1.0, U, n, B2, k, 1.0, dA, n);
  }
}

void svd_back(tnad_ctx* c, int prec, const double* U, const double* S, const double* V, int64_t m, int64_t n,
              const double* dU, const double* dS, const double* dV, double eta, double* dA) {
  WsScope scope(c);
  if (!dU && !dS && !dV) {
    fill(c, dA, m * n, 0.0);
    return;
  }
  double* X = nullptr;
  double* Y = nullptr;
  if (dU) {
    X = ws_d(c, n * n);
    gemm(c, prec, 'T', 'N', n, n, m, 1.0, U, m, dU, m, 0.0, X, n);
  }
  if (dV) {
    Y = ws_d(c, n * n);
    gemm(c, prec, 'T', 'N', n, n, n, 1.0, V, n, dV, n, 0.0, Y, n);
  }
  double* res = ws_d(c, n * n);
  int nb = (int)std::min<int64_t>((n * n + 255) / 256, 4096);
  k_svdback_res<<<nb, 256, 0, c->stream>>>(n, S, X, Y, dS, eta, res);
  count_launch(c);
  check_launch(c, "svdback_res");
  double* T1 = ws_d(c, m * n);
  gemm(c, prec, 'N', 'N', m, n, n, 1.0, U, m, res, n, 0.0, T1, m);
  gemm(c, prec, 'N', 'T', m, n, n, 1.0, T1, m, V, n, 0.0, dA, m);
  if (dU && m != n) {
    // (dU − U·(Uᵀ·dU))·diag(Sinv)·Vᵀ   src/trg.jl:98-99
    double* P = ws_d(c, m * n);
    copy_d2d(c, P, dU, m * n);
    gemm(c, prec, 'N', 'N', m, n, n, -1.0, U, m, X, n, 1.0, P, m);
    int nb2 = (int)std::min<int64_t>((m * n + 255) / 256, 4096);
    k_scale_cols<<<nb2, 256, 0, c->stream>>>(m, n, P, S, eta);
    count_launch(c);
    gemm(c, prec, 'N', 'T', m, n, n, 1.0, P, m, V, n, 1.0, dA, m);
  }
}

}  // namespace tnad
