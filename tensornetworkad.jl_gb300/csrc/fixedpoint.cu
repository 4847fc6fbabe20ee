// Implicit (fixed-point) adjoint of CTMRG.
//
// At the converged environment x* = (C*, T*) = f(x*, a) the reference's
// unrolled Zygote gradient (src/fixedpoint.jl:11-15 differentiated step by
// step) converges to  ā = (∂f/∂a)ᵀ·λ  with  λ = (I − ∂f/∂x)⁻ᵀ·x̄,  the
// implicit-function-theorem gradient used by Liao, Liu, Wang, Xiang
// (arXiv:1903.09650).  λ is obtained by the Neumann iteration
// λ ← x̄ + (∂f/∂x)ᵀ·λ, each term one step pullback (contraction adjoints +
// svd_back) at x*.  The step map is made a strict fixed point by a gauge fix:
// the full FP64 decomposition of M(x*) is computed once and the signs of its
// leading χ singular vectors are aligned with the projector that produced x*.
#include <cmath>

#include "tnad_mixed.h"

namespace tnad {

void polar_ns(tnad_ctx* c, const double* X, int64_t m, int iters, double* O, int* dev_info);
void ns_polish_f64(tnad_ctx* c, double* O, int64_t m, int iters);

__global__ void k_flip_cols(double* __restrict__ X, const double* __restrict__ dots, int64_t n, int m) {
  int64_t tot = n * m;
  for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < tot; e += (int64_t)gridDim.x * blockDim.x)
    if (dots[e / n] < 0.0) X[e] = -X[e];
}

// out = a + b ; also Σ(out − prev)² and Σ out² into acc[0], acc[1] (grid-stride, atomics-free two pass)
__global__ void k_axpy_res(int64_t n, const double* __restrict__ a, const double* __restrict__ b,
                           const double* __restrict__ prev, double* __restrict__ out) {
  for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < n; e += (int64_t)gridDim.x * blockDim.x)
    out[e] = a[e] + b[e];
}

static int nb(int64_t n) { return (int)std::min<int64_t>((n + 255) / 256, 4096); }

FixedPointInfo ctmrg_fixedpoint_adjoint(tnad_ctx* c, int prec, const double* a_, int d, int chi, const double* Cs,
                                        const double* Ts, const double* zref, const double* dC, const double* dT,
                                        double* dbulk, double tol, int maxit) {
  const int64_t n = (int64_t)chi * d;
  const int64_t nCh = (int64_t)chi * chi, nTe = (int64_t)chi * d * chi, nx = nCh + nTe;
  const int64_t na = (int64_t)d * d * d * d;
  WsScope scope(c);
  // gauge-fixed full decomposition at x*
  double* U = ws_d(c, n * n);
  double* S = ws_d(c, n);
  double* V = ws_d(c, n * n);
  {
    WsScope s2(c);
    StepFwd f;
    Ten a = make_ten(const_cast<double*>(a_), {d, d, d, d});
    Ten C = make_ten(const_cast<double*>(Cs), {chi, chi});
    Ten T = make_ten(const_cast<double*>(Ts), {chi, d, chi});
    grow(c, TNAD_PREC_FP64, a, C, T, f);
    double* M = ws_d(c, n * n);
    add_transpose(c, n, f.cp.p, M);
    svd_jacobi(c, M, n, n, U, S, V, true);
  }
  // gauge: z = U[:, 1:χ]·O with O = polar(U[:, 1:χ]ᵀ·z*), so that the step map
  // reproduces x* in the gauge it was produced in (O is held fixed: its
  // variation only moves the environment along gauge directions, which the
  // cotangents of a gauge-invariant energy annihilate)
  double* X = ws_d(c, (int64_t)chi * chi);
  double* O = ws_d(c, (int64_t)chi * chi);
  gemm_f64(c, 'T', 'N', chi, chi, n, 1.0, U, n, zref, n, 0.0, X, chi);
  polar_ns(c, X, chi, 24, O, c->d_flag + 19);
  ns_polish_f64(c, O, chi, 3);
  // λ = [λC; λT] stored contiguously
  double* g = ws_d(c, nx);
  double* lam = ws_d(c, nx);
  double* nxt = ws_d(c, nx);
  double* jt = ws_d(c, nx);
  double* scratch_a = ws_d(c, na);
  copy_d2d(c, g, dC, nCh);
  copy_d2d(c, g + nCh, dT, nTe);
  copy_d2d(c, lam, g, nx);
  FixedPointInfo info;
  const double gn = norm_host(c, g, nx);
  for (int it = 0; it < maxit; ++it) {
    ctmrg_step_bwd(c, prec, a_, d, chi, Cs, Ts, U, S, V, lam, lam + nCh, scratch_a, jt, jt + nCh, false, O, zref);
    k_axpy_res<<<nb(nx), 256, 0, c->stream>>>(nx, g, jt, lam, nxt);
    count_launch(c);
    // relative change of λ (one host sync per iteration)
    axpby(c, nx, 1.0, nxt, -1.0, lam);  // lam ← nxt − lam
    const double dn = norm_host(c, lam, nx);
    const double ln = norm_host(c, nxt, nx);
    copy_d2d(c, lam, nxt, nx);
    info.iters = it + 1;
    info.residual = dn / std::max(ln, 1e-300);
    TNAD_REQUIRE(std::isfinite(info.residual), TNAD_ERR_NONFINITE, "fixed-point adjoint: non-finite iterate");
    if (info.residual <= tol || gn == 0.0) break;
  }
  // ā += (∂f/∂a)ᵀ λ
  ctmrg_step_bwd(c, prec, a_, d, chi, Cs, Ts, U, S, V, lam, lam + nCh, dbulk, jt, jt + nCh, true, O, zref);
  return info;
}

}  // namespace tnad
