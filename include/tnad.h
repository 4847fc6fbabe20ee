/*
 * libtnad — C ABI of the GB300 (sm_103a) contraction-and-truncation path of
 * TensorNetworkAD.jl.
 *
 * Conventions (all entry points):
 *   - every array is Float64 in Julia (column-major) order, exactly as a Julia
 *     Array is laid out in memory, so `ccall` can pass Julia arrays unchanged;
 *   - pointers are HOST pointers unless a `tnad_opts.device_ptrs` flag says
 *     otherwise; the caller owns them; nothing is retained after return except
 *     inside an explicit `tnad_tape`;
 *   - the return value is TNAD_OK (0) or a negative TNAD_ERR_* code; the
 *     message is available from tnad_last_error(ctx); no entry point aborts;
 *   - one context per host thread; a context owns one CUDA stream, its device
 *     workspace and the tapes it hands out.
 *
 * Reference functions replaced (paths inside under-Peter/TensorNetworkAD.jl):
 *   model_tensor(::Ising,β)         src/exampletensors.jl:30-35
 *   trg(a,χ,niter;tol)              src/trg.jl:13-30   (+ Zygote adjoint)
 *   trg_svd                         src/trg.jl:33-44
 *   svd adjoint / svd_back          src/trg.jl:55-61, 72-106 (file lines 77-128)
 *   ctmrg(rt;tol,maxit)             src/ctmrg.jl:110-117 + src/fixedpoint.jl:11-41
 *   ctmrgstep                       src/ctmrg.jl:126-153
 *   indexperm_symmetrize            src/ipeps.jl:32-39
 *   energy(h,ipeps;χ,tol,maxit)     src/variationalipeps.jl:28-40 (+ Zygote adjoint)
 *   expectationvalue                src/variationalipeps.jl:49-56
 */
#ifndef TNAD_H
#define TNAD_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef struct tnad_ctx tnad_ctx;
typedef struct tnad_tape tnad_tape;

enum {
  TNAD_OK = 0,
  TNAD_ERR_ARG = -1,           /* bad argument (null pointer, negative size)      */
  TNAD_ERR_SHAPE = -2,         /* inconsistent tensor sizes (DimensionMismatch)    */
  TNAD_ERR_CUDA = -3,          /* CUDA runtime error                              */
  TNAD_ERR_NOT_CONVERGED = -4, /* an iterative kernel hit its sweep/iteration cap */
  TNAD_ERR_NONFINITE = -5,     /* NaN/Inf met in a norm or result                 */
  TNAD_ERR_NOMEM = -6,         /* device allocation failed                        */
  TNAD_ERR_STATE = -7,         /* tape used twice / wrong kind / no GPU build     */
  TNAD_ERR_TIMEOUT = -8        /* a bounded device-side wait gave up              */
};

/* Arithmetic of the dense contractions. */
enum {
  TNAD_PREC_FP64 = 0,   /* DFMA tiles: the plain FP64 path                           */
  TNAD_PREC_TF32X3 = 1, /* tcgen05 kind::tf32, 3 split products, FP32 accumulation    */
  TNAD_PREC_LADDER = 2  /* TF32X3 until the residual stalls, then FP64 polishing      */
};

/* Eigen/SVD solver used for the CTMRG projector. */
enum {
  TNAD_SOLVER_FULL_SVD = 0, /* full FP64 one-sided Jacobi SVD of the χd×χd corner   */
  TNAD_SOLVER_SUBSPACE = 1  /* warm-started subspace iteration + FP64 Jacobi on the
                               small Rayleigh-Ritz problem (top-χ only)              */
};

/* Gradient of the CTMRG fixed point. */
enum {
  TNAD_ADJOINT_UNROLLED = 0,   /* reverse through every step (reference semantics) */
  TNAD_ADJOINT_FIXEDPOINT = 1  /* implicit adjoint at the converged environment    */
};

typedef struct tnad_opts {
  int32_t prec;            /* TNAD_PREC_*                                         */
  int32_t solver;          /* TNAD_SOLVER_*                                       */
  int32_t adjoint;         /* TNAD_ADJOINT_*                                      */
  int32_t device_ptrs;     /* 1: every array argument is a device pointer         */
  int32_t warm_start;      /* 1: start CTMRG from the C,T passed in (learned net) */
  int32_t stop_rule;       /* 0: reference StopFunction on all χd values;
                              1: ‖Δ(top-χ values)‖₂ ≤ tol (subspace solver)       */
  int32_t fp_maxit;        /* fixed-point adjoint iteration cap                   */
  int32_t reserved0;
  double fp_tol;           /* fixed-point adjoint relative residual target        */
  double ladder_tol;       /* LADDER: residual where TF32X3 hands over to FP64   */
  int64_t tape_budget;     /* bytes of per-step tape kept on device; beyond it
                              steps are recomputed from (C,T) checkpoints         */
} tnad_opts;

/* -------- context -------- */
int tnad_ctx_create(tnad_ctx** out, int device);
void tnad_ctx_destroy(tnad_ctx* ctx);
const char* tnad_last_error(const tnad_ctx* ctx);
int tnad_version(void);
void tnad_opts_default(tnad_opts* o);
/* Bytes of device workspace the context holds now (diagnostics). */
int64_t tnad_ctx_workspace_bytes(const tnad_ctx* ctx);
/* Number of CUDA kernels the context has launched so far. */
int64_t tnad_ctx_kernel_launches(const tnad_ctx* ctx);
/* Kernel timer (measurement support, no reference counterpart): from now on
   bracket every launch of kernel family `name` ("jacobi_round", "gemm_tf32x3",
   "gemm_f64"; "" switches it off) with CUDA events on the context stream. */
int tnad_ctx_kernel_timer(tnad_ctx* ctx, const char* name);
/* Totals since the timer was set: launches, summed device time (ms) and the
   summed algorithmic work of those launches (FP64-equivalent flops).  Syncs. */
int tnad_ctx_kernel_timer_read(tnad_ctx* ctx, int64_t* launches, double* total_ms, double* work);
/* The context's CUDA stream (cudaStream_t), for callers that time around it. */
void* tnad_ctx_stream(tnad_ctx* ctx);
void tnad_tape_free(tnad_tape* tape);

/* -------- building blocks (the role OMEinsum plays in the reference) -------- */
/* Column-major C(M×N) = alpha·op(A)·op(B) + beta·C with op ∈ {'N','T'}; prec is
   TNAD_PREC_FP64 (DFMA) or TNAD_PREC_TF32X3 (tcgen05).  Host pointers. */
int tnad_gemm(tnad_ctx* ctx, int prec, char ta, char tb, int64_t M, int64_t N, int64_t K, double alpha,
              const double* A, int64_t lda, const double* B, int64_t ldb, double beta, double* C, int64_t ldc);
/* Pairwise contraction C[lc] = Σ A[la]·B[lb] (the pairwise form of ein"la,lb -> lc"
   used throughout src/ctmrg.jl, src/trg.jl, src/variationalipeps.jl).  Labels are
   single characters; dims_a/dims_b give the extents in label order.  Host pointers. */
int tnad_contract(tnad_ctx* ctx, int prec, const double* A, const char* la, const int64_t* dims_a,
                  const double* B, const char* lb, const int64_t* dims_b, double* C, const char* lc);

/* -------- example tensors (host arithmetic) -------- */
/* model_tensor(::Ising, β) and its β-derivative: both 2×2×2×2.
   Replaces src/exampletensors.jl:30-35.  da may be NULL. */
int tnad_model_tensor_ising(double beta, double* a, double* da);

/* -------- TRG -------- */
/* trg(a, χ, niter; tol): ln Z per site of the d×d×d×d tensor a.
   Replaces src/trg.jl:13-30.  If tape != NULL a tape for tnad_trg_backward is
   returned (free with tnad_tape_free). */
int tnad_trg(tnad_ctx* ctx, const double* a, int d, int chi, int niter, double tol,
             double* lnZ, tnad_tape** tape);
/* Pullback of trg: da = dlnZ · ∂lnZ/∂a  (Zygote adjoint of src/trg.jl:13-30 with
   the SVD adjoint of src/trg.jl:55-128). */
int tnad_trg_backward(tnad_ctx* ctx, tnad_tape* tape, double dlnZ, double* da);

/* trg_svd(t, χ, tol) of src/trg.jl:33-44 for t of size d1×d2×d3×d4.
   u: d1×d2×k, v: k×d3×d4 (buffers sized for k = min(χ, d1d2, d3d4)); *k_out = k. */
int tnad_trg_svd(tnad_ctx* ctx, const double* t, int d1, int d2, int d3, int d4, int chi,
                 double tol, double* u, double* v, int* k_out);

/* -------- FP64 decompositions and their adjoint -------- */
/* Thin SVD A = U·diag(S)·Vᵀ of an m×n matrix (m ≥ n) by one-sided Jacobi in FP64.
   U: m×n, S: n (descending), V: n×n.  Replaces LinearAlgebra.svd at
   src/trg.jl:36 and src/ctmrg.jl:136. */
int tnad_svd(tnad_ctx* ctx, const double* A, int m, int n, double* U, double* S, double* V);
/* Allocation-free FP64 Jacobi SVD (no counterpart in the reference): the same
   decomposition as tnad_svd for m×n matrices with n ≤ m ≤ 256, for callers that
   cannot allocate device memory (a host framework that owns all device memory
   through its own allocator, or a latency-critical loop where an allocation
   would synchronise the device).  Needs no context: A, U, S, V are DEVICE
   pointers supplied by the caller (m×n, n, n×n, column-major) and stream is a
   cudaStream_t (0: legacy default stream).  Its scratch is a fixed static device
   array (about 1.1 MB, held by every GPU that loads the library until exit),
   shared by all calls: calls that overlap on the GPU race.  The first call on a
   device resolves that array's address and should come before any stream
   capture.  Sizes beyond 256 return TNAD_ERR_SHAPE. */
int tnad_svd_noalloc(const double* A, int m, int n, double* U, double* S, double* V, void* stream);
/* svd_back(U,S,V,dU,dS,dV; η) of src/trg.jl:94-128 (real).  dU/dS/dV may be NULL. */
int tnad_svd_back(tnad_ctx* ctx, const double* U, const double* S, const double* V,
                  int m, int n, const double* dU, const double* dS, const double* dV,
                  double eta, double* dA);

/* -------- CTMRG -------- */
/* One ctmrgstep (src/ctmrg.jl:126-153): bulk d×d×d×d, C χ×χ, T χ×d×χ → C', T',
   vals (χd, s./s[1]). */
int tnad_ctmrgstep(tnad_ctx* ctx, const double* bulk, int d, int chi, const double* C,
                   const double* T, double* Cn, double* Tn, double* vals);
/* Pullback of one ctmrgstep: (dCn, dTn) → (dbulk, dC, dT). */
int tnad_ctmrgstep_backward(tnad_ctx* ctx, const double* bulk, int d, int chi,
                            const double* C, const double* T, const double* dCn,
                            const double* dTn, double* dbulk, double* dC, double* dT);
/* _initializect_square(bulk, Val(:raw), χ)  src/ctmrg.jl:74-86. */
int tnad_init_raw(tnad_ctx* ctx, const double* bulk, int d, int chi, double* C, double* T);
/* ctmrg(rt; tol, maxit) from (C0,T0): src/ctmrg.jl:110-117 with the StopFunction
   semantics of src/fixedpoint.jl:17-41.  opts may be NULL (FP64, full SVD,
   reference stop rule).  With tape != NULL, tnad_ctmrg_backward gives the
   bulk gradient (the initial environment carries none: src/autodiff.jl:4-5). */
int tnad_ctmrg(tnad_ctx* ctx, const double* bulk, int d, int chi, const double* C0,
               const double* T0, double tol, int maxit, const tnad_opts* opts, double* C,
               double* T, int* steps, tnad_tape** tape);
int tnad_ctmrg_backward(tnad_ctx* ctx, tnad_tape* tape, const double* dC, const double* dT,
                        double* dbulk);

/* -------- iPEPS energy -------- */
/* indexperm_symmetrize (src/ipeps.jl:32-39) of a D×D×D×D×s tensor. */
int tnad_symmetrize(tnad_ctx* ctx, const double* A, int D, int s, double* out);
/* expectationvalue(h, ap, rt) (src/variationalipeps.jl:49-56): ap is
   D²×D²×D²×D²×s×s, h s×s×s×s, C χ×χ, T χ×D²×χ. */
int tnad_expectationvalue(tnad_ctx* ctx, const double* h, const double* ap, int d, int s,
                          int chi, const double* C, const double* T, double* E);
/* energy(h, ipeps; χ, tol, maxit)  src/variationalipeps.jl:28-40.
   A: D×D×D×D×s (unsymmetrised, as passed to energy), h: s×s×s×s.
   C_init/T_init: warm-start environment when opts->warm_start (else NULL).
   steps/C_out/T_out may be NULL. */
int tnad_energy(tnad_ctx* ctx, const double* h, const double* A, int D, int s, int chi,
                double tol, int maxit, const tnad_opts* opts, const double* C_init,
                const double* T_init, double* E, int* steps, double* C_out, double* T_out,
                tnad_tape** tape);
/* dA = dE · ∂energy/∂A (Zygote.gradient of energy, src/variationalipeps.jl:71-73). */
int tnad_energy_backward(tnad_ctx* ctx, tnad_tape* tape, double dE, double* dA);
/* Diagnostics of an energy tape (any pointer may be NULL): CTMRG steps, FP64
   polishing steps of the mixed solver, step of the TF32X3→FP64 hand-over,
   fixed-point adjoint iterations (after tnad_energy_backward), last stop-rule
   residual and last fixed-point relative residual.  No reference counterpart
   (the reference reports none of these). */
int tnad_energy_stats(const tnad_tape* tape, int* steps, int* fp64_steps, int* switch_step, int* fp_iters,
                      double* last_diff, double* fp_residual);

#ifdef __cplusplus
}
#endif
#endif /* TNAD_H */
