// Energy driver state shared by energy.cu and the C ABI.
#pragma once

#include "tnad_drivers.h"

namespace tnad {

// Intermediates of expectationvalue (src/variationalipeps.jl:49-56), workspace-backed.
struct Expect {
  double* apn = nullptr;  // ap/‖ap‖
  double* nap = nullptr;  // ‖ap‖ (device scalar)
  Ten w1, w2, r, v, l, G;
  double* sc = nullptr;  // {E, e, n}
};

struct EnergyTape {
  int D = 0, s = 0, chi = 0, d = 0, steps = 0, prec = TNAD_PREC_FP64;
  int solver = TNAD_SOLVER_FULL_SVD, adjoint = TNAD_ADJOINT_UNROLLED;
  int fp64_steps = 0, switch_step = 0;  // mixed solver: FP64 polishing steps, ladder hand-over
  int fp_iters = 0;                     // fixed-point adjoint iterations used
  double fp_residual = 0.0, fp_tol = 1e-10, last_diff = 0.0;
  double fp_fixed_point_residual = 0.0;  // ‖f(x*) − x*‖/‖x*‖ of the aligned step (implicit adjoint)
  int fp_maxit = 200;
  bool fp64_tc = false;  // FP64 products as tensor-core emulation (tnad_opts.fp64_tc)
  double E = 0.0;
  DevPool pool;
  double *h = nullptr, *As = nullptr, *nA = nullptr, *ap = nullptr, *a = nullptr;
  double *C = nullptr, *T = nullptr;  // converged environment
  double* zstar = nullptr;            // projector of the last step (n×χ), fixed-point adjoint
  CtmrgTape ct;
};

void symmetrize_fwd(tnad_ctx* c, const double* A, int D, int s, double* As, double* nA_dev);
void symmetrize_bwd(tnad_ctx* c, const double* As, const double* nA_dev, int D, int s, const double* dAs,
                    double* dA);
void double_layer(tnad_ctx* c, const double* As, int D, int s, double* ap, double* bulk);
void expect_fwd(tnad_ctx* c, int prec, const double* h, const double* ap, int d, int s, int chi, const double* C,
                const double* T, Expect& x);
void expect_bwd(tnad_ctx* c, int prec, const double* h, int d, int s, int chi, const double* C, const double* T,
                const Expect& x, double dE, double* dap, double* dC, double* dT);
void energy_fwd(tnad_ctx* c, EnergyTape& tp, const double* h, const double* A, int D, int s, int chi, double tol,
                int maxit, const tnad_opts& o, const double* Cinit, const double* Tinit, bool record);
void energy_bwd(tnad_ctx* c, EnergyTape& tp, double dE, double* dA);
// Learned warm start: (C, T) predicted by net for the symmetrised, normalised
// site tensor As (n_in values), χ×χ and χ×d×χ on the device (mlp.cu); false
// when the prediction is zero or not finite.
bool warm_start_predict(tnad_ctx* c, tnad_mlp* net, const double* As, int n_in, int chi, int d, double* C,
                        double* T);

}  // namespace tnad
