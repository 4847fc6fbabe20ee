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
 *   svd adjoint / svd_back          src/trg.jl:55-61, 72-105
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
typedef struct tnad_mlp tnad_mlp;

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
  TNAD_PREC_LADDER = 2, /* TF32X3 until the residual stalls, then FP64 polishing      */
  TNAD_PREC_FP64_TC = 3 /* tnad_gemm only: FP64-accurate products from six BF16 slices
                           per operand on the tcgen05 tensor cores (about 2^-47 of
                           the row/column scales; no reference counterpart)           */
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

/* Initial CTMRG environment of tnad_energy. */
enum {
  TNAD_WARM_NONE = 0,    /* :raw initialisation (src/ctmrg.jl:66-86)                    */
  TNAD_WARM_GIVEN = 1,   /* the C_init, T_init passed in                               */
  TNAD_WARM_LEARNED = 2  /* predicted by the network attached with tnad_ctx_set_warm_start,
                            judged by the CTMRG residual, :raw restart if it does not fall */
};

typedef struct tnad_opts {
  int32_t prec;            /* TNAD_PREC_*                                         */
  int32_t solver;          /* TNAD_SOLVER_*                                       */
  int32_t adjoint;         /* TNAD_ADJOINT_*                                      */
  int32_t device_ptrs;     /* 1: every array argument is a device pointer         */
  int32_t warm_start;      /* TNAD_WARM_*: where the CTMRG environment starts      */
  int32_t stop_rule;       /* 0: reference StopFunction on all χd values;
                              1: ‖Δ(top-χ values)‖₂ ≤ tol (subspace solver)       */
  int32_t fp_maxit;        /* fixed-point adjoint iteration cap                   */
  int32_t fp64_tc;         /* 1: the FP64 products of this call (the FP64 phase of
                              the ladder, the fixed-point adjoint's FP64 operator)
                              run as tensor-core FP64 emulation (TNAD_PREC_FP64_TC)
                              instead of DFMA tiles; 0 (default): DFMA             */
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
   TNAD_PREC_FP64 (DFMA), TNAD_PREC_TF32X3 or TNAD_PREC_FP64_TC (tcgen05).  Host
   pointers. */
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
   the SVD adjoint of src/trg.jl:55-61, 72-105). */
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
/* SVD A = U·diag(S)·Vᵀ of a symmetric n×n matrix (the symmetrised enlarged
   corner cpmat of src/ctmrg.jl:134-136, decomposed there by LinearAlgebra.svd),
   through its eigendecomposition: S = |λ| descending, V the eigenvectors,
   U = V·sign(λ).  For n ≥ 256 FP32 Jacobi sweeps are polished to FP64 accuracy
   by a refinement made of matrix products (FP64 Jacobi sweeps where that does
   not converge); prec = TNAD_PREC_FP64 runs those products as DFMA tiles,
   TNAD_PREC_FP64_TC on the tensor cores (TNAD_ERR_STATE without tcgen05).
   Host pointers. */
int tnad_svd_sym(tnad_ctx* ctx, int prec, const double* A, int n, double* U, double* S, double* V);
/* Diagnostics of the symmetric SVDs run on this context (no reference
   counterpart): how many took the product refinement and how many fell back
   to FP64 Jacobi sweeps.  Either pointer may be NULL. */
int tnad_ctx_solver_stats(const tnad_ctx* ctx, int64_t* eig_refined, int64_t* eig_fallback);
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
/* ComplexF64 versions (arrays interleaved (re, im), exactly as a Julia
   Array{ComplexF64} is laid out; host pointers).  tnad_svd_z: thin SVD of the
   m×n A (any m, n; K = min(m, n)): U m×K, S K (real, descending), V n×K with
   A = U·diag(S)·Vᴴ, by one-sided Jacobi with complex plane rotations; columns
   with a zero singular value come back as zero vectors.  Replaces
   LinearAlgebra.svd on complex input (test/svd.jl).  tnad_svd_back_z: svd_back
   of src/trg.jl:72-105 for complex U, V, including the imaginary-diagonal term
   of :85; dU m×K, dS K (real), dV n×K may be NULL. */
int tnad_svd_z(tnad_ctx* ctx, const double* A, int m, int n, double* U, double* S, double* V);
int tnad_svd_back_z(tnad_ctx* ctx, const double* U, const double* S, const double* V, int m, int n,
                    const double* dU, const double* dS, const double* dV, double eta, double* dA);
/* svd_back(U,S,V,dU,dS,dV; η) of src/trg.jl:72-105 (real).  dU/dS/dV may be NULL. */
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
/* optimiseipeps(ipeps, h; χ, tol, maxit, optimargs, optimmethod = LBFGS(m)) of
   src/variationalipeps.jl:67-75, run inside the library: L-BFGS with m correction
   pairs on the site tensor A (D×D×D×D×s, in: the start, out: the minimiser),
   every evaluation the energy and gradient of tnad_energy/tnad_energy_backward
   under opts (CTMRG from :raw each time, as the reference does).  The iterate,
   gradient and pairs stay on the device; each line-search trial returns only its
   energy to the host.  Stops after `iterations`, when |ΔE| ≤ f_tol·|E|, when
   max|∂E/∂A| ≤ g_tol, or when the backtracking line search finds no decrease.
   E_out, iters_out, evals_out may be NULL.  With opts->device_ptrs, h and A are
   device pointers. */
int tnad_optimiseipeps(tnad_ctx* ctx, const double* h, double* A, int D, int s, int chi, double tol, int maxit,
                       const tnad_opts* opts, int m, int iterations, double f_tol, double g_tol, double* E_out,
                       int* iters_out, int* evals_out);
/* dA = dE · ∂energy/∂A (Zygote.gradient of energy, src/variationalipeps.jl:71-73). */
int tnad_energy_backward(tnad_ctx* ctx, tnad_tape* tape, double dE, double* dA);
/* Diagnostics of an energy tape (any pointer may be NULL): CTMRG steps, FP64
   polishing steps of the mixed solver, step of the TF32X3→FP64 hand-over,
   fixed-point adjoint iterations (after tnad_energy_backward), last stop-rule
   residual and last fixed-point relative residual.  No reference counterpart
   (the reference reports none of these). */
int tnad_energy_stats(const tnad_tape* tape, int* steps, int* fp64_steps, int* switch_step, int* fp_iters,
                      double* last_diff, double* fp_residual);
/* After a fixed-point tnad_energy_backward: ‖f(x*) − x*‖/‖x*‖ of the gauge-aligned
   CTMRG step at the converged environment.  The implicit adjoint assumes x* is
   a fixed point; a residual well above the stop tolerance (the aligned gauge
   did not lock) flags a gradient that should not be trusted.  No reference
   counterpart. */
int tnad_energy_fixed_point_residual(const tnad_tape* tape, double* residual);

/* -------- learned warm start (no reference counterpart) --------
   A 3-layer perceptron n_in → width → width → n_out (ReLU between layers) that
   maps the symmetrised site tensor to a gauge-fixed CTMRG environment.  Its
   products run as BF16 tcgen05 GEMMs with FP32 accumulation; parameters are an
   FP32 array  W1 (width×n_in) | b1 | W2 (width×width) | b2 | W3 (n_out×width) | b3
   (column-major matrices), trained with AdamW.  Activations and data are
   column-major feature × sample, FP32.  With device_ptrs = 1 the X, Y, grad
   arrays are device pointers. */
int tnad_mlp_create(tnad_ctx* ctx, int n_in, int width, int n_out, uint64_t seed, tnad_mlp** out);
/* The network's product on its own (host arrays, FP32 column-major):
   C = alpha·op(A)·op(B) + beta·C with op(A), op(B) rounded to BF16, FP32
   accumulation on the tensor cores, chunks of 512 K values summed in FP64. */
int tnad_gemm_bf16(tnad_ctx* ctx, char ta, char tb, int64_t M, int64_t N, int64_t K, float alpha, const float* A,
                   int64_t lda, const float* B, int64_t ldb, float beta, float* C, int64_t ldc);
void tnad_mlp_free(tnad_mlp* net);
int64_t tnad_mlp_param_count(const tnad_mlp* net);
int tnad_mlp_get_params(tnad_ctx* ctx, const tnad_mlp* net, float* params);
/* Sets the parameters and resets the AdamW state. */
int tnad_mlp_set_params(tnad_ctx* ctx, tnad_mlp* net, const float* params);
/* Y (n_out×batch) = net(X (n_in×batch)). */
int tnad_mlp_forward(tnad_ctx* ctx, tnad_mlp* net, const float* X, int batch, float* Y, int device_ptrs);
/* loss = mean((net(X) − Y)²) and its gradient (param_count floats; may be NULL). */
int tnad_mlp_gradient(tnad_ctx* ctx, tnad_mlp* net, const float* X, const float* Y, int batch, float* loss,
                      float* grad, int device_ptrs);
/* Copies a training set (X n_in×n_samples, Y n_out×n_samples, host arrays) to
   device memory owned by the network (n_samples = 0 releases it). */
int tnad_mlp_set_data(tnad_ctx* ctx, tnad_mlp* net, const float* X, const float* Y, int64_t n_samples);
/* One AdamW step (β = 0.9, 0.999, ε = 1e-8; decoupled weight decay on the
   weight matrices) on the mini-batch idx[0..batch) (host array) of the
   n_samples columns of X (n_in×n_samples) and Y (n_out×n_samples); X = Y =
   NULL selects the set loaded by tnad_mlp_set_data.  loss may be NULL (then
   the call does not wait for the GPU). */
int tnad_mlp_train_step(tnad_ctx* ctx, tnad_mlp* net, const float* X, const float* Y, int64_t n_samples,
                        const int32_t* idx, int batch, float lr, float weight_decay, float* loss, int device_ptrs);
/* Gauge fixing of a symmetric CTMRG environment (the network's targets):
   C = W·diag(λ)·Wᵀ with |λ| descending, Tg = Wᵀ·T·W on both χ legs, then the
   column signs s_a (s_0 = +1) chosen so that for each a ≥ 1 the largest
   |Tg[a,i,b]| over i and b < a is positive after Tg[a,i,b] ← s_a s_b Tg[a,i,b].
   C χ×χ, T χ×d×χ in; lam χ and Tg χ×d×χ out (host arrays). */
int tnad_env_gauge_fix(tnad_ctx* ctx, const double* C, const double* T, int chi, int d, double* lam, double* Tg);
/* Attaches (net != NULL) or detaches the network used by TNAD_WARM_LEARNED for
   site tensors D×D×D×D×s at bond dimension χ; n_in = D⁴·s, n_out = χ + χ·D²·χ.
   The context does not own the network. */
int tnad_ctx_set_warm_start(tnad_ctx* ctx, tnad_mlp* net, int D, int s, int chi);
/* Network input of a site tensor A (D×D×D×D×s): indexperm_symmetrize(A)
   (normalised) times the sign of its largest-|·| entry, as n_in floats. */
int tnad_warm_start_features(tnad_ctx* ctx, const double* A, int D, int s, float* x);
/* The predicted environment for site tensor A: C = diag(λ̂)/‖λ̂‖ and T the
   χ-leg-symmetrised prediction /‖·‖ (host arrays χ×χ and χ×D²×χ). */
int tnad_warm_start_env(tnad_ctx* ctx, const double* A, int D, int s, int chi, double* C, double* T);
/* Outcome of the last TNAD_WARM_LEARNED energy call: 1 prediction kept,
   -1 rejected by the residual judge (restarted from :raw), 0 not used. */
int tnad_ctx_warm_start_status(const tnad_ctx* ctx);

#ifdef __cplusplus
}
#endif
#endif /* TNAD_H */
