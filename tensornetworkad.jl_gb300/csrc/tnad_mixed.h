// Mixed-precision CTMRG (subspace solver + precision ladder) and the implicit
// fixed-point adjoint.
#pragma once

#include <limits>

#include "tnad_drivers.h"

namespace tnad {

struct MixedRun {
  int steps = 0;
  int fp64_steps = 0;
  int switch_step = 0;  // step at which the ladder handed over to FP64 (0: never)
  int power_steps = 0;  // M·Q products in total
  double last_diff = std::numeric_limits<double>::infinity();
  bool rejected = false;  // judge: the residual did not fall from step 2 to step 4
};

// z (n×χ) ← z·polar(zᵀ·zprev) (orthogonal Procrustes gauge alignment)
void align_polar(tnad_ctx* c, int prec, double* z, const double* zprev, int64_t n, int chi);

// C/T: initial environment in, converged environment out.  zfinal (n×χ, may be
// null) receives the projector of the last step.  With judge set the run stops
// at step 4 with rejected = true unless its residual fell below that of step 2
// (used to vet a predicted starting environment).
MixedRun ctmrg_run_mixed(tnad_ctx* c, const double* a, int d, int chi, double* C, double* T, double tol, int maxit,
                         const tnad_opts& o, double* zfinal, bool judge = false);

struct FixedPointInfo {
  int iters = 0;
  double residual = 0.0;
  double tsign = 1.0;  // −1: the converged T flips sign every step
  double fixed_point_residual = 0.0;  // ‖g(x*) − x*‖/‖x*‖ of the map the adjoint differentiates
  bool regauged = false;              // g includes the re-gauge of the step's output
};

// Implicit adjoint at a converged environment (C*, T*) of bulk a: given the
// cotangents (dC, dT) of the environment, accumulates ∂/∂a of the fixed point
// into dbulk.  zref: the projector that produced (C*, T*) (gauge reference).
FixedPointInfo ctmrg_fixedpoint_adjoint(tnad_ctx* c, int prec, const double* a, int d, int chi, const double* Cs,
                                        const double* Ts, const double* zref, const double* dC, const double* dT,
                                        double* dbulk, double tol, int maxit);

void align_columns(tnad_ctx* c, double* z, const double* zref, int64_t n, int chi, double* dots_scratch);

}  // namespace tnad
