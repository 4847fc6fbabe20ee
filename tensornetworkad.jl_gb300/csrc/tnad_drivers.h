// Host-side drivers of the hot path (CTMRG, energy, TRG) and their tapes.
#pragma once

#include <memory>
#include <vector>

#include "tnad_internal.h"

namespace tnad {

// Device memory owned by a tape (freed by tnad_tape_free).
struct DevPool {
  std::vector<void*> ptrs;
  int64_t bytes = 0;
  double* d(int64_t n);
  void free_all();
  ~DevPool() { free_all(); }
};

struct CtmrgTape {
  int d = 0, chi = 0, steps = 0, prec = TNAD_PREC_FP64;
  const double* a = nullptr;           // bulk (lives in an owning pool)
  std::vector<double*> C, T;           // input environment of each step
  std::vector<double*> U, S, V;        // decomposition of each step (null: recompute)
};

struct CtmrgRun {
  int steps = 0;
  double last_diff = 0.0;
  bool rejected = false;  // judge: the residual did not fall from step 2 to step 4
};

// Intermediates of one step (workspace-backed).
struct StepFwd {
  Ten X1, X2, cp, w, y1, y2, Cn, Tn;
  double *M = nullptr, *Cs = nullptr, *Ts = nullptr;
  double *nC = nullptr, *nT = nullptr;  // device scalars
};
// cp = ein"ad,iba,dcl,jkcb -> ijlk"(C, T, T, a)                 (src/ctmrg.jl:130)
void grow(tnad_ctx* c, int prec, const Ten& a, const Ten& C, const Ten& T, StepFwd& f);
// C' = zᵀ·cp·z and T' = ein"abjcd,abi,dck -> ijk"(tp, z, z)       (src/ctmrg.jl:139-140)
void project(tnad_ctx* c, int prec, const Ten& a, const Ten& T, const Ten& z, StepFwd& f);
// symmetrise + normalise into Cout/Tout                          (src/ctmrg.jl:145-150)
void finish(tnad_ctx* c, int64_t chi, int64_t d, StepFwd& f, double* Cout, double* Tout);

// One CTMRG step (src/ctmrg.jl:126-153) on device buffers.  U/S/V: n×n, n, n×n
// buffers that receive the decomposition (may be workspace).
void ctmrg_step_fwd(tnad_ctx* c, int prec, const double* a, int d, int chi, const double* C, const double* T,
                    double* Cn, double* Tn, double* vals, double* U, double* S, double* V);
// Pullback of one step.  dbulk/dC/dT are ACCUMULATED into (beta = 1) when accumulate.
void ctmrg_step_bwd(tnad_ctx* c, int prec, const double* a, int d, int chi, const double* C, const double* T,
                    const double* U, const double* S, const double* V, const double* dCn, const double* dTn,
                    double* dbulk, double* dC, double* dT, bool accumulate_bulk, const double* O = nullptr,
                    const double* zref = nullptr, const struct StepCache* cache = nullptr);
// Forward intermediates of one step at fixed (C, T, z), reusable across many
// pullbacks (the fixed-point adjoint applies the same step Jacobian repeatedly).
struct StepCache {
  StepFwd f;
  Ten z;
  double *Cout = nullptr, *Tout = nullptr;
};
void step_cache_fill(tnad_ctx* c, int prec, const double* a, int d, int chi, const double* C, const double* T,
                     const double* U, const double* O, StepCache& sc);
// ctmrg loop with the reference stop rule; C/T hold the initial env on entry and
// the result on exit.  With tape != null every step's input and decomposition
// are recorded (pool owns the memory).
CtmrgRun ctmrg_run(tnad_ctx* c, int prec, const double* a, int d, int chi, double* C, double* T, double tol,
                   int maxit, CtmrgTape* tape, DevPool* pool, int64_t tape_budget, bool judge = false);
// Reverse pass over a recorded CTMRG: dC/dT are the cotangents of the final
// environment (overwritten as scratch); dbulk accumulates.
void ctmrg_reverse(tnad_ctx* c, const CtmrgTape& tape, double* dC, double* dT, double* dbulk);

void init_raw_dev(tnad_ctx* c, const double* a, int d, int chi, double* C, double* T);

}  // namespace tnad
