// iPEPS energy on the device: indexperm_symmetrize (src/ipeps.jl:32-39), the
// double layer ap/a (src/variationalipeps.jl:32-34), the raw environment,
// CTMRG and expectationvalue (src/variationalipeps.jl:49-56), plus the full
// pullback dE/dA (Zygote.gradient of energy, src/variationalipeps.jl:71-73).
#include <cmath>

#include "tnad_energy.h"
#include "tnad_mixed.h"

namespace tnad {

static int nb(int64_t n) { return (int)std::min<int64_t>((n + 255) / 256, 4096); }

static const int kSymPerm[4][5] = {{0, 3, 2, 1, 4}, {2, 1, 0, 3, 4}, {1, 0, 3, 2, 4}, {3, 2, 1, 0, 4}};

__global__ void k_norm_bwd_e(int64_t n, const double* __restrict__ dy, const double* __restrict__ y,
                             const double* __restrict__ nrm, const double* __restrict__ dot, double* __restrict__ dx) {
  double inv = 1.0 / nrm[0], g = dot[0];
  for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < n; e += (int64_t)gridDim.x * blockDim.x)
    dx[e] = (dy[e] - g * y[e]) * inv;
}

void symmetrize_fwd(tnad_ctx* c, const double* A, int D, int s, double* As, double* nA_dev) {
  WsScope scope(c);
  int64_t n = (int64_t)D * D * D * D * s;
  double* x = ws_d(c, n);
  double* y = ws_d(c, n);
  copy_d2d(c, x, A, n);
  for (int k = 0; k < 4; ++k) {
    Ten t = make_ten(x, {D, D, D, D, s});
    copy_d2d(c, y, x, n);
    permute(c, t, kSymPerm[k], y, 1.0, 1.0);  // y = x + permutedims(x, p_k)
    std::swap(x, y);
  }
  copy_d2d(c, As, x, n);
  normalize_inplace(c, As, n, nA_dev);
}

// dA from dAs (all four permutations are involutions, so the pullback of
// x + permutedims(x,p) is g + permutedims(g,p)).
void symmetrize_bwd(tnad_ctx* c, const double* As, const double* nA_dev, int D, int s, const double* dAs,
                    double* dA) {
  WsScope scope(c);
  int64_t n = (int64_t)D * D * D * D * s;
  double* dot = ws_d(c, 1);
  dot_dev(c, dAs, As, n, dot);
  double* g = ws_d(c, n);
  double* h = ws_d(c, n);
  k_norm_bwd_e<<<nb(n), 256, 0, c->stream>>>(n, dAs, As, nA_dev, dot, g);
  count_launch(c);
  for (int k = 3; k >= 0; --k) {
    Ten t = make_ten(g, {D, D, D, D, s});
    copy_d2d(c, h, g, n);
    permute(c, t, kSymPerm[k], h, 1.0, 1.0);
    std::swap(g, h);
  }
  copy_d2d(c, dA, g, n);
}

// ap[(a,i),(b,j),(c,k),(d,l),x,y] = A[a,b,c,d,x]·A[i,j,k,l,y]; bulk = Σ_x ap[..,x,x]
__global__ void k_double_layer(const double* __restrict__ A, int D, int s, double* __restrict__ ap,
                               double* __restrict__ bulk) {
  const int64_t d = (int64_t)D * D;
  const int64_t d4 = d * d * d * d;
  const int64_t n = d4 * s * s;
  const int64_t D4 = (int64_t)D * D * D * D;
  for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < n; e += (int64_t)gridDim.x * blockDim.x) {
    int64_t r = e;
    int64_t ia[4], ib[4];
    for (int q = 0; q < 4; ++q) {
      int64_t al = r % d;
      r /= d;
      ia[q] = al % D;
      ib[q] = al / D;
    }
    int64_t x = r % s, y = r / s;
    int64_t offa = ia[0] + D * (ia[1] + D * (ia[2] + D * ia[3])) + D4 * x;
    int64_t offb = ib[0] + D * (ib[1] + D * (ib[2] + D * ib[3])) + D4 * y;
    ap[e] = A[offa] * A[offb];
  }
  for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < d4; e += (int64_t)gridDim.x * blockDim.x) {
    double t = 0.0;
    for (int x = 0; x < s; ++x) {
      int64_t r = e;
      int64_t offa = 0, offb = 0, mul = 1;
      for (int q = 0; q < 4; ++q) {
        int64_t al = r % d;
        r /= d;
        offa += (al % D) * mul;
        offb += (al / D) * mul;
        mul *= D;
      }
      t += A[offa + D4 * x] * A[offb + D4 * x];
    }
    bulk[e] = t;
  }
}

// dap += dbulk ⊗ δ_xy
__global__ void k_bulk_to_ap(const double* __restrict__ dbulk, int64_t d4, int s, double* __restrict__ dap) {
  for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < d4; e += (int64_t)gridDim.x * blockDim.x)
    for (int x = 0; x < s; ++x) dap[e + d4 * (x + (int64_t)s * x)] += dbulk[e];
}

// e = Σ G∘h, n = Σ_ab G[a,a,b,b], out = {e/n, e, n}
__global__ void k_energy_scalar(const double* __restrict__ G, const double* __restrict__ h, int s,
                                double* __restrict__ out) {
  if (threadIdx.x == 0 && blockIdx.x == 0) {
    int64_t s4 = (int64_t)s * s * s * s;
    double e = 0.0, nn = 0.0;
    for (int64_t q = 0; q < s4; ++q) e += G[q] * h[q];
    for (int a = 0; a < s; ++a)
      for (int b = 0; b < s; ++b) nn += G[a + s * (a + (int64_t)s * (b + (int64_t)s * b))];
    out[0] = e / nn;
    out[1] = e;
    out[2] = nn;
  }
}

// dG = (dE/n)·h − (dE·e/n²)·δ_ij δ_kl   (dE read from out[3])
__global__ void k_energy_dG(const double* __restrict__ h, const double* __restrict__ sc, double dE, int s,
                            double* __restrict__ dG) {
  int64_t s4 = (int64_t)s * s * s * s;
  double e = sc[1], nn = sc[2];
  for (int64_t q = threadIdx.x; q < s4; q += blockDim.x) {
    int i = (int)(q % s), j = (int)((q / s) % s), k = (int)((q / s / s) % s), l = (int)(q / s / s / s);
    double v = dE / nn * h[q];
    if (i == j && k == l) v -= dE * e / (nn * nn);
    dG[q] = v;
  }
}

void expect_fwd(tnad_ctx* c, int prec, const double* h, const double* ap, int d, int s, int chi, const double* C_,
                const double* T_, Expect& x) {
  const int64_t nap = (int64_t)d * d * d * d * s * s;
  x.apn = ws_d(c, nap);
  x.nap = ws_d(c, 1);
  copy_d2d(c, x.apn, ap, nap);
  normalize_inplace(c, x.apn, nap, x.nap);
  Ten C = make_ten(const_cast<double*>(C_), {chi, chi});
  Ten T = make_ten(const_cast<double*>(T_), {chi, d, chi});
  Ten apn = make_ten(x.apn, {d, d, d, d, s, s});
  x.w1 = make_ten(ws_d(c, (int64_t)chi * d * chi), {});
  contract(c, prec, C, "ab", T, "ica", x.w1, "icb");
  x.w2 = make_ten(ws_d(c, (int64_t)chi * d * d * chi), {});
  contract(c, prec, x.w1, "icb", T, "bde", x.w2, "icde");
  x.r = make_ten(ws_d(c, (int64_t)chi * d * chi), {});
  contract(c, prec, C, "eg", T, "gfk", x.r, "efk");
  x.v = make_ten(ws_d(c, (int64_t)chi * chi * d * d * s * s), {});
  contract(c, prec, x.w2, "icde", apn, "cjfdlm", x.v, "iejflm");
  x.l = make_ten(ws_d(c, (int64_t)chi * d * chi * s * s), {});
  contract(c, prec, x.v, "iejflm", x.r, "efk", x.l, "ijklm");
  x.G = make_ten(ws_d(c, (int64_t)s * s * s * s), {});
  contract(c, TNAD_PREC_FP64, x.l, "abcij", x.l, "abckl", x.G, "ijkl");
  x.sc = ws_d(c, 4);
  k_energy_scalar<<<1, 32, 0, c->stream>>>(x.G.p, h, s, x.sc);
  count_launch(c);
}

void expect_bwd(tnad_ctx* c, int prec, const double* h, int d, int s, int chi, const double* C_, const double* T_,
                const Expect& x, double dE, double* dap, double* dC, double* dT) {
  WsScope scope(c);
  const int64_t nap = (int64_t)d * d * d * d * s * s;
  Ten C = make_ten(const_cast<double*>(C_), {chi, chi});
  Ten T = make_ten(const_cast<double*>(T_), {chi, d, chi});
  Ten apn = make_ten(x.apn, {d, d, d, d, s, s});
  Ten dG = make_ten(ws_d(c, (int64_t)s * s * s * s), {s, s, s, s});
  k_energy_dG<<<1, 64, 0, c->stream>>>(h, x.sc, dE, s, dG.p);
  count_launch(c);
  Ten dl = make_ten(ws_d(c, x.l.numel()), {});
  contract(c, TNAD_PREC_FP64, x.l, "abckl", dG, "ijkl", dl, "abcij");
  contract(c, TNAD_PREC_FP64, x.l, "abcij", dG, "ijkl", dl, "abckl", 1.0, 1.0);
  Ten dv = make_ten(ws_d(c, x.v.numel()), {});
  contract(c, prec, dl, "ijklm", x.r, "efk", dv, "iejflm");
  Ten dr = make_ten(ws_d(c, x.r.numel()), {});
  contract(c, prec, x.v, "iejflm", dl, "ijklm", dr, "efk");
  Ten dw2 = make_ten(ws_d(c, x.w2.numel()), {});
  contract(c, prec, dv, "iejflm", apn, "cjfdlm", dw2, "icde");
  Ten dapn = make_ten(ws_d(c, nap), {});
  contract(c, prec, x.w2, "icde", dv, "iejflm", dapn, "cjfdlm");
  Ten dC_ = make_ten(dC, {chi, chi});
  Ten dT_ = make_ten(dT, {chi, d, chi});
  contract(c, prec, dr, "efk", T, "gfk", dC_, "eg");
  contract(c, prec, C, "eg", dr, "efk", dT_, "gfk");
  Ten dw1 = make_ten(ws_d(c, x.w1.numel()), {});
  contract(c, prec, dw2, "icde", T, "bde", dw1, "icb");
  contract(c, prec, x.w1, "icb", dw2, "icde", dT_, "bde", 1.0, 1.0);
  contract(c, prec, dw1, "icb", T, "ica", dC_, "ab", 1.0, 1.0);
  contract(c, prec, C, "ab", dw1, "icb", dT_, "ica", 1.0, 1.0);
  // ap /= norm(ap)
  double* dot = ws_d(c, 1);
  dot_dev(c, dapn.p, x.apn, nap, dot);
  k_norm_bwd_e<<<nb(nap), 256, 0, c->stream>>>(nap, dapn.p, x.apn, x.nap, dot, dap);
  count_launch(c);
}

void double_layer(tnad_ctx* c, const double* As, int D, int s, double* ap, double* bulk) {
  int64_t d = (int64_t)D * D;
  int64_t n = d * d * d * d * s * s;
  k_double_layer<<<nb(n), 256, 0, c->stream>>>(As, D, s, ap, bulk);
  count_launch(c);
  check_launch(c, "double_layer");
}

void double_layer_bwd(tnad_ctx* c, int prec, const double* As, int D, int s, double* dap, const double* dbulk,
                      double* dAs) {
  WsScope scope(c);
  int64_t d = (int64_t)D * D;
  int64_t d4 = d * d * d * d;
  k_bulk_to_ap<<<nb(d4), 256, 0, c->stream>>>(dbulk, d4, s, dap);
  count_launch(c);
  Ten g;
  g.p = dap;
  g.nd = 10;
  for (int q = 0; q < 8; ++q) g.dim[q] = D;
  g.dim[8] = s;
  g.dim[9] = s;
  Ten A = make_ten(const_cast<double*>(As), {D, D, D, D, s});
  Ten out = make_ten(dAs, {});
  contract(c, prec, g, "aibjckdlxy", A, "ijkly", out, "abcdx");
  contract(c, prec, g, "aibjckdlxy", A, "abcdx", out, "ijkly", 1.0, 1.0);
}

// ---------------------------------------------------------------------------

void energy_fwd(tnad_ctx* c, EnergyTape& tp, const double* h, const double* A, int D, int s, int chi, double tol,
                int maxit, const tnad_opts& o, const double* Cinit, const double* Tinit, bool record) {
  tp.fp64_tc = o.fp64_tc != 0;
  Fp64TcScope fp64_route(c, tp.fp64_tc);
  const int d = D * D;
  const int64_t nA = (int64_t)D * D * D * D * s;
  const int64_t nap = (int64_t)d * d * d * d * s * s;
  const int64_t d4 = (int64_t)d * d * d * d;
  tp.D = D;
  tp.s = s;
  tp.chi = chi;
  tp.d = d;
  tp.prec = o.prec == TNAD_PREC_FP64 ? TNAD_PREC_FP64 : TNAD_PREC_TF32X3;
  DevPool& P = tp.pool;
  tp.h = P.d(s * s * s * s);
  copy_d2d(c, tp.h, h, (int64_t)s * s * s * s);
  tp.As = P.d(nA);
  tp.nA = P.d(1);
  symmetrize_fwd(c, A, D, s, tp.As, tp.nA);
  TNAD_CK(cudaMemcpyAsync(c->h_pin, tp.nA, 8, cudaMemcpyDeviceToHost, c->stream));
  TNAD_CK(cudaStreamSynchronize(c->stream));
  TNAD_REQUIRE(std::isfinite(c->h_pin[0]) && c->h_pin[0] > 0.0, TNAD_ERR_NONFINITE,
               "energy: the symmetrised site tensor has a zero or non-finite norm");
  tp.ap = P.d(nap);
  tp.a = P.d(d4);
  double_layer(c, tp.As, D, s, tp.ap, tp.a);
  tp.C = P.d((int64_t)chi * chi);
  tp.T = P.d((int64_t)chi * d * chi);
  // starting environment: predicted by the attached network (vetted by the
  // residual judge below), passed in by the caller, or :raw
  bool learned = o.warm_start == TNAD_WARM_LEARNED;
  c->warm_status = 0;
  if (learned) {
    TNAD_REQUIRE(c->warm_net && c->warm_D == D && c->warm_s == s && c->warm_chi == chi, TNAD_ERR_STATE,
                 "energy: TNAD_WARM_LEARNED needs a network attached for this (D, s, χ)");
    learned = warm_start_predict(c, c->warm_net, tp.As, (int)nA, chi, d, tp.C, tp.T);
    if (!learned) {  // zero or non-finite prediction: rejected before any step
      c->warm_status = -1;
      init_raw_dev(c, tp.a, d, chi, tp.C, tp.T);
    }
  } else if (o.warm_start == TNAD_WARM_GIVEN && Cinit && Tinit) {
    copy_d2d(c, tp.C, Cinit, (int64_t)chi * chi);
    copy_d2d(c, tp.T, Tinit, (int64_t)chi * d * chi);
  } else {
    init_raw_dev(c, tp.a, d, chi, tp.C, tp.T);
  }
  tp.solver = o.solver;
  tp.adjoint = o.adjoint;
  tp.fp_tol = o.fp_tol;
  tp.fp_maxit = o.fp_maxit;
  const int64_t n = (int64_t)chi * d;
  if (o.solver == TNAD_SOLVER_SUBSPACE) {
    // mixed precision + subspace solver; the implicit adjoint needs only x* and z*
    if (record) tp.zstar = P.d(n * chi);
    MixedRun run = ctmrg_run_mixed(c, tp.a, d, chi, tp.C, tp.T, tol, maxit, o, record ? tp.zstar : nullptr, learned);
    int probe = 0;
    if (learned) {
      c->warm_status = run.rejected ? -1 : 1;
      if (run.rejected) {  // the residual did not fall: cold restart from :raw
        probe = run.steps;
        init_raw_dev(c, tp.a, d, chi, tp.C, tp.T);
        run = ctmrg_run_mixed(c, tp.a, d, chi, tp.C, tp.T, tol, maxit, o, record ? tp.zstar : nullptr);
      }
    }
    tp.steps = run.steps + probe;
    tp.fp64_steps = run.fp64_steps;
    tp.switch_step = run.switch_step;
    tp.last_diff = run.last_diff;
    TNAD_REQUIRE(!record || o.adjoint == TNAD_ADJOINT_FIXEDPOINT, TNAD_ERR_ARG,
                 "energy: the subspace solver is differentiated with the fixed-point adjoint only");
  } else {
    const bool full_tape = record && o.adjoint == TNAD_ADJOINT_UNROLLED;
    const int rprec = o.prec == TNAD_PREC_FP64 ? TNAD_PREC_FP64 : TNAD_PREC_TF32X3;
    const int64_t budget = full_tape ? o.tape_budget : (int64_t)(2 * n * n + n) * 8 * (maxit + 2);
    CtmrgRun run = ctmrg_run(c, rprec, tp.a, d, chi, tp.C, tp.T, tol, maxit, (full_tape || record) ? &tp.ct : nullptr,
                             &P, budget, learned);
    int probe = 0;
    if (learned) {
      c->warm_status = run.rejected ? -1 : 1;
      if (run.rejected) {  // the residual did not fall: cold restart from :raw
        probe = run.steps;
        tp.ct = CtmrgTape();
        init_raw_dev(c, tp.a, d, chi, tp.C, tp.T);
        run = ctmrg_run(c, rprec, tp.a, d, chi, tp.C, tp.T, tol, maxit, (full_tape || record) ? &tp.ct : nullptr, &P,
                        budget);
      }
    }
    tp.steps = run.steps + probe;
    tp.last_diff = run.last_diff;
    if (record && o.adjoint == TNAD_ADJOINT_FIXEDPOINT) {
      TNAD_REQUIRE(!tp.ct.U.empty() && tp.ct.U.back(), TNAD_ERR_STATE, "energy: missing last projector");
      tp.zstar = P.d(n * chi);
      copy_d2d(c, tp.zstar, tp.ct.U.back(), n * chi);
    }
  }
  WsScope scope(c);
  Expect x;
  expect_fwd(c, TNAD_PREC_FP64, tp.h, tp.ap, d, s, chi, tp.C, tp.T, x);
  TNAD_CK(cudaMemcpyAsync(c->h_pin, x.sc, 3 * 8, cudaMemcpyDeviceToHost, c->stream));
  TNAD_CK(cudaStreamSynchronize(c->stream));
  tp.E = c->h_pin[0];
  TNAD_REQUIRE(std::isfinite(tp.E), TNAD_ERR_NONFINITE, "energy: non-finite result");
}

void energy_bwd(tnad_ctx* c, EnergyTape& tp, double dE, double* dA) {
  Fp64TcScope fp64_route(c, tp.fp64_tc);
  const int D = tp.D, s = tp.s, chi = tp.chi, d = tp.d;
  const int64_t nap = (int64_t)d * d * d * d * s * s;
  const int64_t d4 = (int64_t)d * d * d * d;
  WsScope scope(c);
  Expect x;
  expect_fwd(c, TNAD_PREC_FP64, tp.h, tp.ap, d, s, chi, tp.C, tp.T, x);
  double* dap = ws_d(c, nap);
  double* dC = ws_d(c, (int64_t)chi * chi);
  double* dT = ws_d(c, (int64_t)chi * d * chi);
  expect_bwd(c, TNAD_PREC_FP64, tp.h, d, s, chi, tp.C, tp.T, x, dE, dap, dC, dT);
  double* dbulk = ws_d(c, d4);
  fill(c, dbulk, d4, 0.0);
  if (tp.adjoint == TNAD_ADJOINT_FIXEDPOINT) {
    const int pr = tp.prec == TNAD_PREC_FP64 ? TNAD_PREC_FP64 : TNAD_PREC_TF32X3;
    FixedPointInfo fi =
        ctmrg_fixedpoint_adjoint(c, pr, tp.a, d, chi, tp.C, tp.T, tp.zstar, dC, dT, dbulk, tp.fp_tol, tp.fp_maxit);
    tp.fp_iters = fi.iters;
    tp.fp_residual = fi.residual;
    tp.fp_fixed_point_residual = fi.fixed_point_residual;
  } else {
    ctmrg_reverse(c, tp.ct, dC, dT, dbulk);
  }
  double* dAs = ws_d(c, (int64_t)D * D * D * D * s);
  double_layer_bwd(c, TNAD_PREC_FP64, tp.As, D, s, dap, dbulk, dAs);
  symmetrize_bwd(c, tp.As, tp.nA, D, s, dAs, dA);
}

}  // namespace tnad
