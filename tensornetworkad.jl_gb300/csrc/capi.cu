// extern "C" entry points of libtnad (declared in include/tnad.h).
#include <cmath>
#include <cstring>
#include <memory>

#include "tnad_api.h"
#include "tnad_energy.h"
#include "tnad_trg.h"

using namespace tnad;

struct CtmrgOwned {
  DevPool pool;
  CtmrgTape tape;
};

struct tnad_tape {
  int kind = 0;  // 1 trg, 2 ctmrg, 3 energy
  bool dev = false;  // forward was called with device pointers
  tnad_ctx* ctx = nullptr;
  std::unique_ptr<TrgTape> trg;
  std::unique_ptr<CtmrgOwned> ct;
  std::unique_ptr<EnergyTape> en;
};

namespace {

const double* to_dev(tnad_ctx* c, const double* p, int64_t n, bool dev) {
  if (dev || !p) return p;
  double* d = ws_d(c, n);
  TNAD_CK(cudaMemcpyAsync(d, p, n * 8, cudaMemcpyHostToDevice, c->stream));
  return d;
}

void to_host(tnad_ctx* c, double* out, const double* d, int64_t n, bool dev) {
  if (!out) return;
  if (dev)
    copy_d2d(c, out, d, n);
  else
    TNAD_CK(cudaMemcpyAsync(out, d, n * 8, cudaMemcpyDeviceToHost, c->stream));
}

void finish_call(tnad_ctx* c) {
  TNAD_CK(cudaStreamSynchronize(c->stream));
  TNAD_CK(cudaGetLastError());
  check_tc_errors(c);
}

tnad_opts opts_or_default(const tnad_opts* o) {
  tnad_opts r;
  tnad_opts_default(&r);
  if (o) r = *o;
  return r;
}

}  // namespace


extern "C" void tnad_tape_free(tnad_tape* t) {
  if (!t) return;
  if (t->ctx) {
    cudaSetDevice(t->ctx->device);
    cudaStreamSynchronize(t->ctx->stream);
  }
  delete t;
}

extern "C" int tnad_model_tensor_ising(double beta, double* a, double* da) {
  if (!a) return TNAD_ERR_ARG;
  // q = 1/√2 [cβ+sβ cβ−sβ; cβ−sβ cβ+sβ], cβ = √cosh β, sβ = √sinh β;
  // a_ijkl = Σ_x q_xi q_xj q_xk q_xl   (src/exampletensors.jl:30-35)
  double cb = std::sqrt(std::cosh(beta)), sb = std::sqrt(std::sinh(beta));
  double dcb = std::sinh(beta) / (2.0 * cb), dsb = std::cosh(beta) / (2.0 * sb);
  const double r = 1.0 / std::sqrt(2.0);
  double q[2][2] = {{r * (cb + sb), r * (cb - sb)}, {r * (cb - sb), r * (cb + sb)}};
  double dq[2][2] = {{r * (dcb + dsb), r * (dcb - dsb)}, {r * (dcb - dsb), r * (dcb + dsb)}};
  for (int l = 0; l < 2; ++l)
    for (int k = 0; k < 2; ++k)
      for (int j = 0; j < 2; ++j)
        for (int i = 0; i < 2; ++i) {
          double s = 0.0, ds = 0.0;
          for (int x = 0; x < 2; ++x) {
            s += q[x][i] * q[x][j] * q[x][k] * q[x][l];
            ds += dq[x][i] * q[x][j] * q[x][k] * q[x][l] + q[x][i] * dq[x][j] * q[x][k] * q[x][l] +
                  q[x][i] * q[x][j] * dq[x][k] * q[x][l] + q[x][i] * q[x][j] * q[x][k] * dq[x][l];
          }
          int e = i + 2 * (j + 2 * (k + 2 * l));
          a[e] = s;
          if (da) da[e] = ds;
        }
  return TNAD_OK;
}

// ------------------------------------------------------------------ building blocks
extern "C" int tnad_gemm(tnad_ctx* c, int prec, char ta, char tb, int64_t M, int64_t N, int64_t K, double alpha,
                         const double* A, int64_t lda, const double* B, int64_t ldb, double beta, double* Cm,
                         int64_t ldc) {
  API_BEGIN(c)
  TNAD_REQUIRE(A && B && Cm && M >= 0 && N >= 0 && K >= 0, TNAD_ERR_ARG, "tnad_gemm: bad arguments");
  bool at = (ta == 'T' || ta == 't'), bt = (tb == 'T' || tb == 't');
  TNAD_REQUIRE(lda >= (at ? K : M) && ldb >= (bt ? N : K) && ldc >= M, TNAD_ERR_ARG, "tnad_gemm: leading dims");
  WsScope scope(c);
  int64_t na = at ? lda * M : lda * K, nbb = bt ? ldb * K : ldb * N;
  const double* dA = to_dev(c, A, na, false);
  const double* dB = to_dev(c, B, nbb, false);
  double* dC = ws_d(c, ldc * N);
  TNAD_CK(cudaMemcpyAsync(dC, Cm, ldc * N * 8, cudaMemcpyHostToDevice, c->stream));
  TNAD_REQUIRE(prec == TNAD_PREC_FP64 || prec == TNAD_PREC_TF32X3 || prec == TNAD_PREC_FP64_TC, TNAD_ERR_ARG,
               "tnad_gemm: prec");
  gemm(c, prec, ta, tb, M, N, K, alpha, dA, lda, dB, ldb, beta, dC, ldc);
  to_host(c, Cm, dC, ldc * N, false);
  finish_call(c);
  API_END(c)
}

extern "C" int tnad_contract(tnad_ctx* c, int prec, const double* A, const char* la, const int64_t* dims_a,
                             const double* B, const char* lb, const int64_t* dims_b, double* Cout, const char* lc) {
  API_BEGIN(c)
  TNAD_REQUIRE(A && B && Cout && la && lb && lc && dims_a && dims_b, TNAD_ERR_ARG, "tnad_contract: null");
  TNAD_REQUIRE(strlen(la) <= 10 && strlen(lb) <= 10 && strlen(lc) <= 10, TNAD_ERR_ARG, "tnad_contract: rank > 10");
  WsScope scope(c);
  Ten ta, tb;
  ta.nd = (int)strlen(la);
  tb.nd = (int)strlen(lb);
  for (int k = 0; k < ta.nd; ++k) ta.dim[k] = dims_a[k];
  for (int k = 0; k < tb.nd; ++k) tb.dim[k] = dims_b[k];
  ta.p = const_cast<double*>(to_dev(c, A, ta.numel(), false));
  tb.p = const_cast<double*>(to_dev(c, B, tb.numel(), false));
  Ten tc = contract_shape(ta, la, tb, lb, lc);
  tc.p = ws_d(c, tc.numel());
  contract(c, prec, ta, la, tb, lb, tc, lc);
  to_host(c, Cout, tc.p, tc.numel(), false);
  finish_call(c);
  API_END(c)
}

// ------------------------------------------------------------------ TRG
extern "C" int tnad_trg(tnad_ctx* c, const double* a, int d, int chi, int niter, double tol, double* lnZ,
                        tnad_tape** tape) {
  API_BEGIN(c)
  TNAD_REQUIRE(a && lnZ && d >= 1 && chi >= 1 && niter >= 0, TNAD_ERR_ARG, "tnad_trg: bad arguments");
  if (tape) *tape = nullptr;
  WsScope scope(c);
  const double* da = to_dev(c, a, (int64_t)d * d * d * d, false);
  auto tp = std::make_unique<TrgTape>();
  trg_fwd(c, *tp, da, d, chi, niter, tol);
  *lnZ = tp->lnZ;
  finish_call(c);
  if (tape) {
    tnad_tape* t = new tnad_tape();
    t->kind = 1;
    t->ctx = c;
    t->trg = std::move(tp);
    *tape = t;
  }
  API_END(c)
}

extern "C" int tnad_trg_backward(tnad_ctx* c, tnad_tape* tape, double dlnZ, double* da) {
  API_BEGIN(c)
  TNAD_REQUIRE(tape && tape->kind == 1 && tape->trg, TNAD_ERR_STATE, "tnad_trg_backward: not a trg tape");
  TNAD_REQUIRE(da, TNAD_ERR_ARG, "tnad_trg_backward: null output");
  WsScope scope(c);
  TrgTape& tp = *tape->trg;
  int64_t n0 = tp.it.empty() ? tp.fdims[0] * tp.fdims[1] * tp.fdims[2] * tp.fdims[3]
                             : tp.it[0].dims[0] * tp.it[0].dims[1] * tp.it[0].dims[2] * tp.it[0].dims[3];
  double* g = ws_d(c, n0);
  trg_bwd(c, tp, dlnZ, g);
  to_host(c, da, g, n0, false);
  finish_call(c);
  API_END(c)
}

extern "C" int tnad_trg_svd(tnad_ctx* c, const double* t, int d1, int d2, int d3, int d4, int chi, double tol,
                            double* u, double* v, int* k_out) {
  API_BEGIN(c)
  TNAD_REQUIRE(t && u && v && k_out && d1 > 0 && d2 > 0 && d3 > 0 && d4 > 0, TNAD_ERR_ARG, "tnad_trg_svd: bad args");
  WsScope scope(c);
  DevPool pool;
  int64_t dd[4] = {d1, d2, d3, d4};
  const double* dt = to_dev(c, t, (int64_t)d1 * d2 * d3 * d4, false);
  TrgSvd s;
  trg_svd_fwd(c, dt, dd, chi, tol, s, &pool);
  to_host(c, u, s.u, s.m * s.k, false);
  to_host(c, v, s.v, s.k * s.n, false);
  *k_out = (int)s.k;
  finish_call(c);
  API_END(c)
}

// ------------------------------------------------------------------ SVD
extern "C" int tnad_svd(tnad_ctx* c, const double* A, int m, int n, double* U, double* S, double* V) {
  API_BEGIN(c)
  TNAD_REQUIRE(A && U && S && V && m >= n && n >= 1, TNAD_ERR_ARG, "tnad_svd: needs m >= n >= 1");
  WsScope scope(c);
  const double* dA = to_dev(c, A, (int64_t)m * n, false);
  double* dU = ws_d(c, (int64_t)m * n);
  double* dS = ws_d(c, n);
  double* dV = ws_d(c, (int64_t)n * n);
  svd_jacobi(c, dA, m, n, dU, dS, dV, false);
  to_host(c, U, dU, (int64_t)m * n, false);
  to_host(c, S, dS, n, false);
  to_host(c, V, dV, (int64_t)n * n, false);
  finish_call(c);
  API_END(c)
}

extern "C" int tnad_svd_sym(tnad_ctx* c, int prec, const double* A, int n, double* U, double* S, double* V) {
  API_BEGIN(c)
  TNAD_REQUIRE(A && U && S && V && n >= 1, TNAD_ERR_ARG, "tnad_svd_sym: needs n >= 1 and non-null arrays");
  TNAD_REQUIRE(prec == TNAD_PREC_FP64 || prec == TNAD_PREC_FP64_TC, TNAD_ERR_ARG,
               "tnad_svd_sym: prec must be TNAD_PREC_FP64 or TNAD_PREC_FP64_TC");
  TNAD_REQUIRE(prec != TNAD_PREC_FP64_TC || c->tc_ok, TNAD_ERR_STATE,
               "tnad_svd_sym: TNAD_PREC_FP64_TC needs an sm_100-family GPU (tcgen05)");
  Fp64TcScope route(c, prec == TNAD_PREC_FP64_TC);
  WsScope scope(c);
  const int64_t nn = (int64_t)n * n;
  const double* dA = to_dev(c, A, nn, false);
  double* dU = ws_d(c, nn);
  double* dS = ws_d(c, n);
  double* dV = ws_d(c, nn);
  svd_jacobi(c, dA, n, n, dU, dS, dV, true, 0);
  to_host(c, U, dU, nn, false);
  to_host(c, S, dS, n, false);
  to_host(c, V, dV, nn, false);
  finish_call(c);
  API_END(c)
}

extern "C" int tnad_ctx_solver_stats(const tnad_ctx* c, int64_t* eig_refined, int64_t* eig_fallback) {
  if (!c) return TNAD_ERR_ARG;
  if (eig_refined) *eig_refined = c->eig_refined;
  if (eig_fallback) *eig_fallback = c->eig_fallback;
  return TNAD_OK;
}

extern "C" int tnad_svd_back(tnad_ctx* c, const double* U, const double* S, const double* V, int m, int n,
                             const double* dU, const double* dS, const double* dV, double eta, double* dA) {
  API_BEGIN(c)
  TNAD_REQUIRE(U && S && V && dA && m >= n && n >= 1, TNAD_ERR_ARG, "tnad_svd_back: needs m >= n >= 1");
  WsScope scope(c);
  const double* u = to_dev(c, U, (int64_t)m * n, false);
  const double* s = to_dev(c, S, n, false);
  const double* v = to_dev(c, V, (int64_t)n * n, false);
  const double* du = to_dev(c, dU, (int64_t)m * n, false);
  const double* ds = to_dev(c, dS, n, false);
  const double* dv = to_dev(c, dV, (int64_t)n * n, false);
  double* out = ws_d(c, (int64_t)m * n);
  svd_back(c, TNAD_PREC_FP64, u, s, v, m, n, du, ds, dv, eta, out);
  to_host(c, dA, out, (int64_t)m * n, false);
  finish_call(c);
  API_END(c)
}

// ------------------------------------------------------------------ CTMRG
extern "C" int tnad_init_raw(tnad_ctx* c, const double* bulk, int d, int chi, double* C, double* T) {
  API_BEGIN(c)
  TNAD_REQUIRE(bulk && C && T && d >= 1 && chi >= 1, TNAD_ERR_ARG, "tnad_init_raw: bad arguments");
  WsScope scope(c);
  const double* a = to_dev(c, bulk, (int64_t)d * d * d * d, false);
  double* dC = ws_d(c, (int64_t)chi * chi);
  double* dT = ws_d(c, (int64_t)chi * d * chi);
  init_raw_dev(c, a, d, chi, dC, dT);
  to_host(c, C, dC, (int64_t)chi * chi, false);
  to_host(c, T, dT, (int64_t)chi * d * chi, false);
  finish_call(c);
  API_END(c)
}

extern "C" int tnad_ctmrgstep(tnad_ctx* c, const double* bulk, int d, int chi, const double* C, const double* T,
                              double* Cn, double* Tn, double* vals) {
  API_BEGIN(c)
  TNAD_REQUIRE(bulk && C && T && Cn && Tn && d >= 1 && chi >= 1, TNAD_ERR_ARG, "tnad_ctmrgstep: bad arguments");
  WsScope scope(c);
  int64_t n = (int64_t)chi * d;
  const double* a = to_dev(c, bulk, (int64_t)d * d * d * d, false);
  const double* dC = to_dev(c, C, (int64_t)chi * chi, false);
  const double* dT = to_dev(c, T, (int64_t)chi * d * chi, false);
  double* oC = ws_d(c, (int64_t)chi * chi);
  double* oT = ws_d(c, (int64_t)chi * d * chi);
  double* ov = ws_d(c, n);
  double* U = ws_d(c, n * n);
  double* S = ws_d(c, n);
  double* V = ws_d(c, n * n);
  ctmrg_step_fwd(c, TNAD_PREC_FP64, a, d, chi, dC, dT, oC, oT, ov, U, S, V);
  to_host(c, Cn, oC, (int64_t)chi * chi, false);
  to_host(c, Tn, oT, (int64_t)chi * d * chi, false);
  to_host(c, vals, ov, n, false);
  finish_call(c);
  API_END(c)
}

extern "C" int tnad_ctmrgstep_backward(tnad_ctx* c, const double* bulk, int d, int chi, const double* C,
                                       const double* T, const double* dCn, const double* dTn, double* dbulk,
                                       double* dC, double* dT) {
  API_BEGIN(c)
  TNAD_REQUIRE(bulk && C && T && dCn && dTn && dbulk && dC && dT, TNAD_ERR_ARG, "tnad_ctmrgstep_backward: null");
  WsScope scope(c);
  int64_t n = (int64_t)chi * d;
  const double* a = to_dev(c, bulk, (int64_t)d * d * d * d, false);
  const double* iC = to_dev(c, C, (int64_t)chi * chi, false);
  const double* iT = to_dev(c, T, (int64_t)chi * d * chi, false);
  const double* gC = to_dev(c, dCn, (int64_t)chi * chi, false);
  const double* gT = to_dev(c, dTn, (int64_t)chi * d * chi, false);
  double* oC = ws_d(c, (int64_t)chi * chi);
  double* oT = ws_d(c, (int64_t)chi * d * chi);
  double* U = ws_d(c, n * n);
  double* S = ws_d(c, n);
  double* V = ws_d(c, n * n);
  ctmrg_step_fwd(c, TNAD_PREC_FP64, a, d, chi, iC, iT, oC, oT, nullptr, U, S, V);
  double* ga = ws_d(c, (int64_t)d * d * d * d);
  double* gC2 = ws_d(c, (int64_t)chi * chi);
  double* gT2 = ws_d(c, (int64_t)chi * d * chi);
  ctmrg_step_bwd(c, TNAD_PREC_FP64, a, d, chi, iC, iT, U, S, V, gC, gT, ga, gC2, gT2, false);
  to_host(c, dbulk, ga, (int64_t)d * d * d * d, false);
  to_host(c, dC, gC2, (int64_t)chi * chi, false);
  to_host(c, dT, gT2, (int64_t)chi * d * chi, false);
  finish_call(c);
  API_END(c)
}

extern "C" int tnad_ctmrg(tnad_ctx* c, const double* bulk, int d, int chi, const double* C0, const double* T0,
                          double tol, int maxit, const tnad_opts* opts, double* C, double* T, int* steps,
                          tnad_tape** tape) {
  API_BEGIN(c)
  TNAD_REQUIRE(bulk && C0 && T0 && C && T && d >= 1 && chi >= 1 && maxit >= 0, TNAD_ERR_ARG,
               "tnad_ctmrg: bad arguments");
  if (tape) *tape = nullptr;
  tnad_opts o = opts_or_default(opts);
  const bool dev = o.device_ptrs != 0;
  WsScope scope(c);
  auto own = std::make_unique<CtmrgOwned>();
  int64_t na = (int64_t)d * d * d * d;
  double* a = own->pool.d(na);
  const double* ain = to_dev(c, bulk, na, dev);
  copy_d2d(c, a, ain, na);
  double* wC = ws_d(c, (int64_t)chi * chi);
  double* wT = ws_d(c, (int64_t)chi * d * chi);
  copy_d2d(c, wC, to_dev(c, C0, (int64_t)chi * chi, dev), (int64_t)chi * chi);
  copy_d2d(c, wT, to_dev(c, T0, (int64_t)chi * d * chi, dev), (int64_t)chi * d * chi);
  int prec = o.prec == TNAD_PREC_FP64 ? TNAD_PREC_FP64 : TNAD_PREC_TF32X3;
  Fp64TcScope fp64_route(c, o.fp64_tc != 0);
  CtmrgRun run = ctmrg_run(c, prec, a, d, chi, wC, wT, tol, maxit, tape ? &own->tape : nullptr, &own->pool,
                           o.tape_budget);
  if (steps) *steps = run.steps;
  to_host(c, C, wC, (int64_t)chi * chi, dev);
  to_host(c, T, wT, (int64_t)chi * d * chi, dev);
  finish_call(c);
  if (tape) {
    tnad_tape* t = new tnad_tape();
    t->kind = 2;
    t->ctx = c;
    t->ct = std::move(own);
    *tape = t;
  }
  API_END(c)
}

extern "C" int tnad_ctmrg_backward(tnad_ctx* c, tnad_tape* tape, const double* dC, const double* dT, double* dbulk) {
  API_BEGIN(c)
  TNAD_REQUIRE(tape && tape->kind == 2 && tape->ct, TNAD_ERR_STATE, "tnad_ctmrg_backward: not a ctmrg tape");
  TNAD_REQUIRE(dC && dT && dbulk, TNAD_ERR_ARG, "tnad_ctmrg_backward: null argument");
  WsScope scope(c);
  const CtmrgTape& tp = tape->ct->tape;
  int d = tp.d, chi = tp.chi;
  int64_t nCh = (int64_t)chi * chi, nTe = (int64_t)chi * d * chi, na = (int64_t)d * d * d * d;
  double* gC = ws_d(c, nCh);
  double* gT = ws_d(c, nTe);
  copy_d2d(c, gC, to_dev(c, dC, nCh, false), nCh);
  copy_d2d(c, gT, to_dev(c, dT, nTe, false), nTe);
  double* ga = ws_d(c, na);
  fill(c, ga, na, 0.0);
  ctmrg_reverse(c, tp, gC, gT, ga);
  to_host(c, dbulk, ga, na, false);
  finish_call(c);
  API_END(c)
}

// ------------------------------------------------------------------ energy
extern "C" int tnad_symmetrize(tnad_ctx* c, const double* A, int D, int s, double* out) {
  API_BEGIN(c)
  TNAD_REQUIRE(A && out && D >= 1 && s >= 1, TNAD_ERR_ARG, "tnad_symmetrize: bad arguments");
  WsScope scope(c);
  int64_t n = (int64_t)D * D * D * D * s;
  const double* a = to_dev(c, A, n, false);
  double* o = ws_d(c, n);
  double* nr = ws_d(c, 1);
  symmetrize_fwd(c, a, D, s, o, nr);
  to_host(c, out, o, n, false);
  finish_call(c);
  API_END(c)
}

extern "C" int tnad_expectationvalue(tnad_ctx* c, const double* h, const double* ap, int d, int s, int chi,
                                     const double* C, const double* T, double* E) {
  API_BEGIN(c)
  TNAD_REQUIRE(h && ap && C && T && E, TNAD_ERR_ARG, "tnad_expectationvalue: null argument");
  WsScope scope(c);
  const double* dh = to_dev(c, h, (int64_t)s * s * s * s, false);
  const double* dap = to_dev(c, ap, (int64_t)d * d * d * d * s * s, false);
  const double* dC = to_dev(c, C, (int64_t)chi * chi, false);
  const double* dT = to_dev(c, T, (int64_t)chi * d * chi, false);
  Expect x;
  expect_fwd(c, TNAD_PREC_FP64, dh, dap, d, s, chi, dC, dT, x);
  TNAD_CK(cudaMemcpyAsync(c->h_pin, x.sc, 8, cudaMemcpyDeviceToHost, c->stream));
  finish_call(c);
  *E = c->h_pin[0];
  API_END(c)
}

extern "C" int tnad_energy(tnad_ctx* c, const double* h, const double* A, int D, int s, int chi, double tol,
                           int maxit, const tnad_opts* opts, const double* C_init, const double* T_init, double* E,
                           int* steps, double* C_out, double* T_out, tnad_tape** tape) {
  API_BEGIN(c)
  TNAD_REQUIRE(h && A && E && D >= 1 && s >= 1 && chi >= 1 && maxit >= 0, TNAD_ERR_ARG, "tnad_energy: bad arguments");
  if (tape) *tape = nullptr;
  tnad_opts o = opts_or_default(opts);
  const bool dev = o.device_ptrs != 0;
  const int d = D * D;
  WsScope scope(c);
  const double* dh = to_dev(c, h, (int64_t)s * s * s * s, dev);
  const double* dA = to_dev(c, A, (int64_t)D * D * D * D * s, dev);
  const double* ci = o.warm_start ? to_dev(c, C_init, (int64_t)chi * chi, dev) : nullptr;
  const double* ti = o.warm_start ? to_dev(c, T_init, (int64_t)chi * d * chi, dev) : nullptr;
  auto tp = std::make_unique<EnergyTape>();
  energy_fwd(c, *tp, dh, dA, D, s, chi, tol, maxit, o, ci, ti, tape != nullptr);
  *E = tp->E;
  if (steps) *steps = tp->steps;
  to_host(c, C_out, tp->C, (int64_t)chi * chi, dev);
  to_host(c, T_out, tp->T, (int64_t)chi * d * chi, dev);
  finish_call(c);
  if (tape) {
    tnad_tape* t = new tnad_tape();
    t->kind = 3;
    t->dev = dev;
    t->ctx = c;
    t->en = std::move(tp);
    *tape = t;
  }
  API_END(c)
}

extern "C" int tnad_energy_backward(tnad_ctx* c, tnad_tape* tape, double dE, double* dA) {
  API_BEGIN(c)
  TNAD_REQUIRE(tape && tape->kind == 3 && tape->en, TNAD_ERR_STATE, "tnad_energy_backward: not an energy tape");
  TNAD_REQUIRE(dA, TNAD_ERR_ARG, "tnad_energy_backward: null output");
  WsScope scope(c);
  EnergyTape& tp = *tape->en;
  int64_t nA = (int64_t)tp.D * tp.D * tp.D * tp.D * tp.s;
  double* g = ws_d(c, nA);
  energy_bwd(c, tp, dE, g);
  to_host(c, dA, g, nA, tape->dev);
  finish_call(c);
  API_END(c)
}

extern "C" int tnad_energy_stats(const tnad_tape* t, int* steps, int* fp64_steps, int* switch_step, int* fp_iters,
                                 double* last_diff, double* fp_residual) {
  if (!t || t->kind != 3 || !t->en) return TNAD_ERR_STATE;
  const EnergyTape& e = *t->en;
  if (steps) *steps = e.steps;
  if (fp64_steps) *fp64_steps = e.fp64_steps;
  if (switch_step) *switch_step = e.switch_step;
  if (fp_iters) *fp_iters = e.fp_iters;
  if (last_diff) *last_diff = e.last_diff;
  if (fp_residual) *fp_residual = e.fp_residual;
  return TNAD_OK;
}

extern "C" int tnad_energy_fixed_point_residual(const tnad_tape* t, double* residual) {
  if (!t || t->kind != 3 || !t->en || !residual) return TNAD_ERR_STATE;
  *residual = t->en->fp_fixed_point_residual;
  return TNAD_OK;
}
