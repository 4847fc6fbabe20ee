// Mixed-precision CTMRG: the reference's ctmrgstep (src/ctmrg.jl:126-153) with
// the full SVD of the χd×χd enlarged corner replaced by a warm-started
// subspace iteration that only tracks its top-p invariant subspace
// (p = χ + max(16, χ/2), so the lag rate is |λ_{p+1}/λ_χ| instead of
// |λ_{χ+1}/λ_χ|).  Per step, with M = cp + cpᵀ and Q (n×p, orthonormal):
//     Y = M·Q                       (tensor cores, 3xTF32)
//     H = Qᵀ·Y, H = W·diag(θ)·Wᵀ    (Rayleigh–Ritz, sorted by |θ|: one-CTA FP32
//                                    Jacobi, or the multi-CTA FP64 Jacobi SVD)
//     z = Q·W[:, 1:χ]               (Ritz vectors: the projector of this step)
//     z ← z·polar(zᵀ·z_prev)        (gauge alignment with the previous projector)
//     Q ← CholeskyQR2(Y·W)          (power step on the Ritz basis, order kept)
// The dense contractions run at TF32X3 until the Ritz-value residual reaches
// ladder_tol or stalls, then the same iteration continues in FP64 (DFMA GEMMs,
// FP64 Jacobi) until ‖Δ(|θ|/|θ₁|)_{1:χ}‖₂ ≤ tol.  Any orthonormal basis of the
// top-χ subspace gives a gauge-equivalent environment, so the fixed point is
// the reference's.  The polar alignment keeps consecutive environments in one
// gauge, which the implicit adjoint needs (x* = f(x*)).  Where C's spectrum
// comes in ±λ pairs (D=4 workloads) the converged iteration still cycles
// between gauge-equivalent environments; the adjoint then re-gauges the step's
// output onto x* (fixedpoint.cu), and tnad_energy_fixed_point_residual reports
// the residual of the map it differentiates.
#include <cmath>
#include <cstdio>
#include <limits>

#include "tnad_mixed.h"

namespace tnad {

void chol_inv_upper(tnad_ctx* c, const double* G, int64_t p, double* Rinv, int* dev_fail);
void chol_inv_upper_f32(tnad_ctx* c, const double* G, int64_t p, double* Rinv, int* dev_fail);
void randn(tnad_ctx* c, double* x, int64_t n, uint64_t seed, double scale, bool accumulate,
           const double* dev_sumsq = nullptr);

static int nb(int64_t n) { return (int)std::min<int64_t>((n + 255) / 256, 4096); }

__global__ void k_symmetrize_small(double* H, int p) {
  for (int e = blockIdx.x * blockDim.x + threadIdx.x; e < p * p; e += gridDim.x * blockDim.x) {
    int i = e % p, j = e / p;
    if (i < j) {
      double v = 0.5 * (H[i + j * p] + H[j + i * p]);
      H[i + j * p] = v;
      H[j + i * p] = v;
    }
  }
}

// vals[i] = |θ_i|/|θ_0| for i < chi ; diff = ‖vals − old‖₂ (single block)
__global__ void k_ritz_vals(const double* __restrict__ lam, int chi, const double* __restrict__ old, int have_old,
                            double* __restrict__ vals, double* __restrict__ diff) {
  __shared__ double sh[256];
  double t = 0.0;
  const double l0 = fabs(lam[0]);
  for (int i = threadIdx.x; i < chi; i += blockDim.x) {
    double v = fabs(lam[i]) / l0;
    vals[i] = v;
    if (have_old) {
      double d = v - old[i];
      t += d * d;
    }
  }
  sh[threadIdx.x] = t;
  __syncthreads();
  for (int k = blockDim.x / 2; k > 0; k >>= 1) {
    if ((int)threadIdx.x < k) sh[threadIdx.x] += sh[threadIdx.x + k];
    __syncthreads();
  }
  if (threadIdx.x == 0) diff[0] = have_old ? sqrt(sh[0]) : INFINITY;
}

// flip column j of z (n×chi) when dot(zprev_j, z_j) < 0 ; dots: chi values
__global__ void k_align_cols(double* __restrict__ z, const double* __restrict__ dots, int64_t n, int chi) {
  int64_t tot = n * chi;
  for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < tot; e += (int64_t)gridDim.x * blockDim.x) {
    int64_t j = e / n;
    if (dots[j] < 0.0) z[e] = -z[e];
  }
}

// dots[j] = Σ_i a[i,j]·b[i,j] for n×m column blocks (one warp per column)
__global__ void k_coldots(const double* __restrict__ a, const double* __restrict__ b, int64_t n, int m,
                          double* __restrict__ dots) {
  int w = (blockIdx.x * blockDim.x + threadIdx.x) >> 5, lane = threadIdx.x & 31;
  if (w >= m) return;
  double s = 0.0;
  for (int64_t i = lane; i < n; i += 32) s += a[i + w * n] * b[i + w * n];
  for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
  if (lane == 0) dots[w] = s;
}

void col_dots(tnad_ctx* c, const double* a, const double* b, int64_t n, int m, double* dots) {
  k_coldots<<<(m * 32 + 255) / 256, 256, 0, c->stream>>>(a, b, n, m, dots);
  count_launch(c);
}

void align_columns(tnad_ctx* c, double* z, const double* zref, int64_t n, int chi, double* dots_scratch) {
  col_dots(c, zref, z, n, chi, dots_scratch);
  k_align_cols<<<nb(n * chi), 256, 0, c->stream>>>(z, dots_scratch, n, chi);
  count_launch(c);
}

void polar_ns(tnad_ctx* c, const double* X, int64_t m, int iters, double* O, int* dev_info);

// out = ok ? zp : z·diag(sign(diag X))
__global__ void k_select_align(const double* __restrict__ zp, const double* __restrict__ z,
                               const double* __restrict__ X, const int* __restrict__ ok, int64_t n, int chi,
                               double* __restrict__ out) {
  const int64_t tot = n * chi;
  const bool use_polar = ok[0] != 0;
  for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < tot; e += (int64_t)gridDim.x * blockDim.x) {
    const int64_t j = e / n;
    out[e] = use_polar ? zp[e] : (X[j + j * chi] < 0.0 ? -z[e] : z[e]);
  }
}

// O ← O·(3I − OᵀO)/2 in FP64 (quadratic clean-up of an almost orthogonal O)
void ns_polish_f64(tnad_ctx* c, double* O, int64_t m, int iters) {
  WsScope scope(c);
  double* G = ws_d(c, m * m);
  double* O2 = ws_d(c, m * m);
  for (int it = 0; it < iters; ++it) {
    gemm_f64(c, 'T', 'N', m, m, m, 1.0, O, m, O, m, 0.0, G, m);
    copy_d2d(c, O2, O, m * m);
    gemm_f64(c, 'N', 'N', m, m, m, -0.5, O, m, G, m, 1.5, O2, m);
    copy_d2d(c, O, O2, m * m);
  }
}

// z (n×χ) ← z·polar(zᵀ·zprev); falls back to per-column sign alignment when
// zᵀ·zprev is far from orthogonal (the subspace moved a lot: early steps).
void align_polar(tnad_ctx* c, int prec, double* z, const double* zprev, int64_t n, int chi) {
  WsScope scope(c);
  double* X = ws_d(c, (int64_t)chi * chi);
  double* O = ws_d(c, (int64_t)chi * chi);
  double* zp = ws_d(c, n * chi);
  int* ok = c->d_flag + 18;
  gemm(c, TNAD_PREC_FP64, 'T', 'N', chi, chi, n, 1.0, z, n, zprev, n, 0.0, X, chi);
  polar_ns(c, X, chi, 24, O, ok);
  ns_polish_f64(c, O, chi, 2);
  gemm(c, prec, 'N', 'N', n, chi, chi, 1.0, z, n, O, chi, 0.0, zp, n);
  k_select_align<<<nb(n * chi), 256, 0, c->stream>>>(zp, z, X, ok, n, chi, z);
  count_launch(c);
}

// Y (n×p) → Q (n×p) with orthonormal columns spanning the same nested leading
// subspaces: two CholeskyQR passes (Gram in FP64).  A tiny random component
// (relative `jitter`) keeps Y full rank when M has fewer than p non-null
// directions (the zero-padded raw environment of the first steps).  The
// first factorisation stays in FP64: CholeskyQR in FP32 (even shifted, as in
// CholeskyQR3) breaks down on these nearly rank-deficient blocks.
void cholqr2(tnad_ctx* c, int prec, const double* Y, int64_t n, int64_t p, double* Q, double jitter, uint64_t seed) {
  WsScope scope(c);
  double* G = ws_d(c, p * p);
  double* Ri = ws_d(c, p * p);
  double* t = ws_d(c, n * p);
  int* fail = c->d_flag + 16;
  copy_d2d(c, t, Y, n * p);
  if (jitter > 0.0) {
    double* ss = ws_d(c, 1);
    sumsq_dev(c, Y, n * p, ss);
    randn(c, t, n * p, seed, jitter, true, ss);  // jitter × RMS(Y), scale read on the device
  }
  const double* src = t;
  for (int pass = 0; pass < 2; ++pass) {
    gemm(c, TNAD_PREC_FP64, 'T', 'N', p, p, n, 1.0, src, n, src, n, 0.0, G, p);
    // the second Gram matrix is I + O(κ(Y)²·ε64): at TF32X3 accuracy its
    // factor is taken in FP32 (GB300's FP32 pipe is far wider than its FP64 one)
    if (pass == 1 && prec != TNAD_PREC_FP64)
      chol_inv_upper_f32(c, G, p, Ri, fail);
    else
      chol_inv_upper(c, G, p, Ri, fail);
    gemm(c, prec, 'N', 'N', n, p, p, 1.0, src, n, Ri, p, 0.0, Q, n);
    if (pass == 0) {
      copy_d2d(c, t, Q, n * p);
      src = t;
    }
  }
}

// λ_i = S_i·sign(U_i·V_i): eigenvalues of a symmetric matrix from its SVD
// (one warp per column)
__global__ void k_eig_from_svd(const double* __restrict__ U, const double* __restrict__ V,
                               const double* __restrict__ S, int p, double* __restrict__ lam) {
  const int w = (blockIdx.x * blockDim.x + threadIdx.x) >> 5, lane = threadIdx.x & 31;
  if (w >= p) return;
  double d = 0.0;
  for (int i = lane; i < p; i += 32) d += U[i + (int64_t)w * p] * V[i + (int64_t)w * p];
  for (int o = 16; o > 0; o >>= 1) d += __shfl_xor_sync(0xffffffffu, d, o);
  if (lane == 0) lam[w] = d < 0.0 ? -S[w] : S[w];
}

// FP64 eigendecomposition of the p×p Rayleigh–Ritz matrix H in the FP64 phase,
// through the multi-CTA FP64 Jacobi SVD (one CTA per column pair, sweeps
// replayed as CUDA graphs; GB300's FP64 pipe is too narrow for a one-SM FP64
// solver).  By then Q carries the previous Ritz basis, so H is nearly diagonal
// and a few sweeps suffice; λ_i = σ_i·sign(u_i·v_i), ordered by |λ| descending.
void eigh_small_fp64(tnad_ctx* c, const double* H, int64_t p, double* W, double* lam) {
  // the one-CTA FP32 solve polished by matrix products; the FP64 Jacobi SVD
  // below remains the fallback
  if (eigh_fp32_refined(c, H, p, W, lam)) return;
  WsScope scope(c);
  double* Up = ws_d(c, p * p);
  double* Sp = ws_d(c, p);
  svd_jacobi(c, H, p, p, Up, Sp, W, true, 0);
  k_eig_from_svd<<<(unsigned)((p * 32 + 255) / 256), 256, 0, c->stream>>>(Up, W, Sp, (int)p, lam);
  count_launch(c);
}

MixedRun ctmrg_run_mixed(tnad_ctx* c, const double* a_, int d, int chi, double* C, double* T, double tol, int maxit,
                         const tnad_opts& o, double* zfinal, bool judge) {
  const int64_t n = (int64_t)chi * d;
  const int64_t nCh = (int64_t)chi * chi, nTe = (int64_t)chi * d * chi;
  int64_t p = std::min<int64_t>(n, chi + std::max(16, chi / 2));
  p = std::min<int64_t>(p, 160);
  TNAD_REQUIRE(p >= chi, TNAD_ERR_SHAPE, "mixed CTMRG: χ too large for the subspace solver (p ≤ 160)");
  WsScope scope(c);
  Ten a = make_ten(const_cast<double*>(a_), {d, d, d, d});
  double* Q = ws_d(c, n * p);
  double* Y = ws_d(c, n * p);
  double* YW = ws_d(c, n * p);
  double* H = ws_d(c, p * p);
  double* Wm = ws_d(c, p * p);
  double* lam = ws_d(c, p);
  double* z = ws_d(c, n * chi);
  double* zprev = ws_d(c, n * chi);
  double* vals = ws_d(c, chi);
  double* oldv = ws_d(c, chi);
  double* diff = ws_d(c, 2);
  double* dots = ws_d(c, chi);
  double* Cn = ws_d(c, nCh);
  double* Tn = ws_d(c, nTe);
  double* M = ws_d(c, n * n);
  int prec = (o.prec == TNAD_PREC_FP64) ? TNAD_PREC_FP64 : TNAD_PREC_TF32X3;
  const bool ladder = (o.prec == TNAD_PREC_LADDER);
  // deterministic start block
  randn(c, Y, n * p, 12345, 1.0, false);
  cholqr2(c, TNAD_PREC_FP64, Y, n, p, Q, 0.0, 0);
  MixedRun run;
  PhaseTrace tr(c, "ctmrg_mixed");
  bool have_old = false, have_z = false;
  double best = std::numeric_limits<double>::infinity();
  int stall = 0;
  int counter = 0;
  double judge_ref = 0.0;
  for (int k = 1;; ++k) {
    WsScope step(c);
    StepFwd f;
    Ten Ct = make_ten(C, {chi, chi});
    Ten Tt = make_ten(T, {chi, d, chi});
    tr.mark(prec == TNAD_PREC_FP64 ? "grow_f64" : "grow_tf32");
    grow(c, prec, a, Ct, Tt, f);
    tr.mark(prec == TNAD_PREC_FP64 ? "power_f64" : "power_tf32");
    add_transpose(c, n, f.cp.p, M);
    // power steps per CTMRG step: more while the environment (hence M) still
    // moves a lot, one per step near the fixed point
    const double dprev = run.last_diff;
    const int inner = (k == 1 || dprev > 1e-2) ? 6 : (dprev > 1e-5 ? 3 : 1);
    run.power_steps += inner;
    // Relative random component added before CholeskyQR: keeps the n×p block
    // full rank (κ ≤ 1e7, so the FP64 Gram stays positive definite) while the
    // zero-padded early environments have fewer than p non-null directions; at
    // the FP64 polishing stage it is below the rounding of the result.
    const double jitter = (dprev > 1e-3 || prec != TNAD_PREC_FP64) ? 1e-7 : 1e-13;
    // the block is re-orthonormalised every second power step: two products
    // raise κ by at most (|λ₁|/|λ_p|)², far inside what FP64 CholeskyQR2 takes
    for (int it = 0; it < inner; ++it) {
      gemm(c, prec, 'N', 'N', n, p, n, 1.0, M, n, Q, n, 0.0, Y, n);
      if (it + 1 == inner) break;
      if ((inner - 1 - it) % 2 == 1)
        cholqr2(c, prec, Y, n, p, Q, jitter, 1000 + it);
      else
        copy_d2d(c, Q, Y, n * p);
    }
    // Rayleigh–Ritz in span(Q)
    tr.mark(prec == TNAD_PREC_FP64 ? "ritz_f64" : "ritz_tf32");
    gemm(c, TNAD_PREC_FP64, 'T', 'N', p, p, n, 1.0, Q, n, Y, n, 0.0, H, p);
    k_symmetrize_small<<<nb(p * p), 256, 0, c->stream>>>(H, (int)p);
    count_launch(c);
    if (prec == TNAD_PREC_FP64)
      eigh_small_fp64(c, H, p, Wm, lam);
    else
      eigh_small_prec(c, true, H, p, Wm, lam, 40, c->d_flag + 17);
    if (tr.on()) {
      TNAD_CK(cudaMemcpyAsync(c->h_flag + 17, c->d_flag + 17, sizeof(int), cudaMemcpyDeviceToHost, c->stream));
      TNAD_CK(cudaStreamSynchronize(c->stream));
      std::fprintf(stderr, "[tnad trace] step %d ritz eigh sweeps %d (inner %d)\n", k, c->h_flag[17], inner);
    }
    gemm(c, prec, 'N', 'N', n, chi, p, 1.0, Q, n, Wm, p, 0.0, z, n);
    // Gauge: rotate the Ritz basis onto the previous projector (orthogonal
    // Procrustes, z ← z·polar(zᵀ·z_prev)).  Consecutive environments then agree
    // element-wise near the fixed point, so the subspace Q carried to the next
    // step lives in the same index space as the next enlarged corner.
    tr.mark("align");
    if (have_z) align_polar(c, prec, z, zprev, n, chi);
    copy_d2d(c, zprev, z, n * chi);
    have_z = true;
    // next basis: power step applied to the Ritz basis
    tr.mark(prec == TNAD_PREC_FP64 ? "basis_f64" : "basis_tf32");
    gemm(c, prec, 'N', 'N', n, p, p, 1.0, Y, n, Wm, p, 0.0, YW, n);
    cholqr2(c, prec, YW, n, p, Q, jitter, (uint64_t)k);
    // renormalise C, T with z (src/ctmrg.jl:139-150)
    tr.mark(prec == TNAD_PREC_FP64 ? "project_f64" : "project_tf32");
    Ten zt = make_ten(z, {chi, d, chi});
    project(c, prec, a, Tt, zt, f);
    finish(c, chi, d, f, Cn, Tn);
    copy_d2d(c, C, Cn, nCh);
    copy_d2d(c, T, Tn, nTe);
    tr.mark("residual");
    k_ritz_vals<<<1, 256, 0, c->stream>>>(lam, chi, oldv, have_old ? 1 : 0, vals, diff);
    count_launch(c);
    TNAD_CK(cudaMemcpyAsync(c->h_pin, diff, 8, cudaMemcpyDeviceToHost, c->stream));
    TNAD_CK(cudaStreamSynchronize(c->stream));
    const double dv = c->h_pin[0];
    copy_d2d(c, oldv, vals, chi);
    have_old = true;
    run.steps++;
    if (prec == TNAD_PREC_FP64) run.fp64_steps++;
    run.last_diff = dv;
    counter++;
    if (counter > maxit) break;
    if (judge && k == 2) judge_ref = dv;
    if (judge && k == 4 && dv > tol && !(dv < judge_ref)) {
      run.rejected = true;
      break;
    }
    if (prec == TNAD_PREC_FP64 || !ladder) {
      if (dv <= tol) break;
    } else {
      // TF32X3 phase: hand over to FP64 once the residual reaches ladder_tol or stalls
      // a stall only counts near the TF32X3 noise floor (the early transient is
      // not monotone)
      if (dv < best * 0.7) {
        best = dv;
        stall = 0;
      } else if (dv < 1e-3) {
        ++stall;
      }
      if (dv <= o.ladder_tol || stall >= 3 || dv <= tol) {
        prec = TNAD_PREC_FP64;
        run.switch_step = k;
        best = std::numeric_limits<double>::infinity();
      }
    }
  }
  if (zfinal) copy_d2d(c, zfinal, zprev, n * chi);
  check_tc_errors(c);
  return run;
}

}  // namespace tnad
