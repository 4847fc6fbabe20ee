// Internal declarations of libtnad: context, device workspace, tensors and the
// kernel entry points shared between translation units.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include <string>
#include <vector>

#include "tnad.h"

namespace tnad {

struct Error {
  int code;
  std::string msg;
};

[[noreturn]] void fail(int code, const std::string& msg);

#define TNAD_CK(x)                                                                  \
  do {                                                                              \
    cudaError_t e_ = (x);                                                           \
    if (e_ != cudaSuccess)                                                          \
      ::tnad::fail(TNAD_ERR_CUDA, std::string(#x) + ": " + cudaGetErrorString(e_)); \
  } while (0)

#define TNAD_REQUIRE(cond, code, msg) \
  do {                                \
    if (!(cond)) ::tnad::fail(code, msg); \
  } while (0)

// Stack-ordered device workspace over persistent chunks.  alloc() bumps, and
// a Mark restores the stack (chunks are kept for reuse until ctx destruction).
class Arena {
 public:
  struct Mark {
    size_t chunk;
    size_t used;
  };
  void* alloc(size_t bytes);
  Mark mark() const;
  void reset(const Mark& m);
  void release_all();
  int64_t bytes_held() const;

 private:
  struct Chunk {
    char* base;
    size_t cap;
    size_t used;
  };
  std::vector<Chunk> chunks_;
  size_t cur_ = 0;
};

// A column-major FP64 tensor view on the device.
struct Ten {
  double* p = nullptr;
  int nd = 0;
  int64_t dim[10] = {0, 0, 0, 0, 0, 0, 0, 0, 0, 0};
  int64_t numel() const {
    int64_t n = 1;
    for (int i = 0; i < nd; ++i) n *= dim[i];
    return n;
  }
};
Ten make_ten(double* p, std::initializer_list<int64_t> dims);

}  // namespace tnad

struct tnad_ctx {
  int device = 0;
  int sm_count = 0;
  cudaStream_t stream = nullptr;
  tnad::Arena ws;
  std::string err;
  int64_t launches = 0;
  double* d_red = nullptr;  // small device scratch for reductions (4096 doubles)
  double* h_pin = nullptr;  // pinned host mirror (64 doubles)
  int* d_flag = nullptr;    // device flags / counters (64 ints)
  int* h_flag = nullptr;    // pinned host mirror of the flags
  bool tc_ok = false;       // tcgen05 GEMM path available (sm_100 family)
  // One-shot fault injection for the failure-path tests, set from the
  // environment variable TNAD_TEST_FAULT when the context is created:
  //   kFaultTcWithhold — the next tensor-core GEMM launch does not issue the TMA
  //     loads of its first K slice and waits at most 20 ms on an mbarrier, so
  //     the bounded wait runs out (TNAD_ERR_TIMEOUT) with no copy in flight;
  //   kFaultJacobiCap — the next Jacobi SVD is capped at one FP64 sweep
  //     (TNAD_ERR_NOT_CONVERGED).
  // Each is cleared when used; later calls on the context run normally.
  int fault_once = 0;
  // FP64 products (TNAD_PREC_FP64) of the current call run as gemm_fp64tc on
  // the tensor cores instead of DFMA tiles (tnad_opts.fp64_tc; Fp64TcScope)
  bool fp64_tc = false;
  // Symmetric SVDs of n ≥ 256 polish their FP32 Jacobi result by the GEMM
  // refinement of eig_refine.cu (false: FP64 Jacobi sweeps, set by
  // TNAD_EIG_POLISH=jacobi in the environment when the context is created),
  // and how often that refinement was taken / fell back to the sweeps
  bool eig_refine = true;
  int64_t eig_refined = 0, eig_fallback = 0;
  // size n whose last refinement fell back, and how many more SVDs of that
  // size go straight to the FP64 sweeps (jacobi.cu, kEigSkip)
  int64_t eig_skip_n = 0;
  int eig_skip_left = 0;
  // FP32 Jacobi sweeps of the symmetric SVD as block rounds (k_jacobi_block;
  // false: one launch per element round, set by TNAD_JACOBI_BLOCKS=0)
  bool jacobi_blocks = true;
  // kernel timer (tnad_ctx_kernel_timer): events around every launch of one
  // kernel family, with the algorithmic work (flops or bytes) of each launch
  std::string ktimer;
  std::vector<std::pair<cudaEvent_t, cudaEvent_t>> kt_ev;
  double kt_work = 0.0;
  int64_t kt_launches = 0;  // kernel launches inside the timed brackets
  // learned warm start (tnad_ctx_set_warm_start): network, the (D, s, χ) it
  // was trained for, and the outcome of the last energy call that used it
  tnad_mlp* warm_net = nullptr;
  int warm_D = 0, warm_s = 0, warm_chi = 0;
  int warm_status = 0;
};

namespace tnad {

enum { kFaultNone = 0, kFaultTcWithhold = 1, kFaultJacobiCap = 2 };

// Phase timer: with TNAD_TRACE set in the environment, CUDA events bracket
// named phases on the context stream and a per-phase summary goes to stderr
// when the tracer is destroyed.  Without TNAD_TRACE it does nothing.
class PhaseTrace {
 public:
  PhaseTrace(tnad_ctx* c, const char* name);
  ~PhaseTrace();
  void mark(const char* phase);  // closes the previous phase, opens `phase`
  bool on() const { return on_; }

 private:
  tnad_ctx* c_;
  const char* name_;
  bool on_;
  std::vector<std::pair<const char*, cudaEvent_t>> ev_;
};

// Brackets one launch (or a graph of `launches` launches) of kernel family
// `name` with CUDA events when the context's kernel timer is set to that family.
struct KernelTimer {
  tnad_ctx* c;
  cudaEvent_t e1 = nullptr;
  KernelTimer(tnad_ctx* ctx, const char* name, double work, int64_t launches = 1) : c(ctx) {
    if (c->ktimer.empty() || c->ktimer != name) return;
    cudaEvent_t e0;
    if (cudaEventCreate(&e0) != cudaSuccess || cudaEventCreate(&e1) != cudaSuccess) return;
    cudaEventRecord(e0, c->stream);
    c->kt_ev.push_back({e0, e1});
    c->kt_work += work;
    c->kt_launches += launches;
  }
  ~KernelTimer() {
    if (e1) cudaEventRecord(e1, c->stream);
  }
};

// Sets the context's FP64-product route for one call and restores it after.
struct Fp64TcScope {
  tnad_ctx* c;
  bool prev;
  Fp64TcScope(tnad_ctx* ctx, bool on) : c(ctx), prev(ctx->fp64_tc) { c->fp64_tc = on && c->tc_ok; }
  ~Fp64TcScope() { c->fp64_tc = prev; }
};

// RAII scope over the context's workspace stack.
struct WsScope {
  tnad_ctx* c;
  Arena::Mark m;
  explicit WsScope(tnad_ctx* ctx) : c(ctx), m(ctx->ws.mark()) {}
  ~WsScope() { c->ws.reset(m); }
};
inline double* ws_d(tnad_ctx* c, int64_t n) { return (double*)c->ws.alloc((size_t)n * 8); }
inline float* ws_f(tnad_ctx* c, int64_t n) { return (float*)c->ws.alloc((size_t)n * 4); }

inline void count_launch(tnad_ctx* c, int n = 1) { c->launches += n; }
void check_launch(tnad_ctx* c, const char* what);

// ---------------- elementwise / reductions (elementwise.cu) ----------------
void fill(tnad_ctx* c, double* x, int64_t n, double v);
void copy_d2d(tnad_ctx* c, double* dst, const double* src, int64_t n);
// y = a*x + b*y
void axpby(tnad_ctx* c, int64_t n, double a, const double* x, double b, double* y);
void scale(tnad_ctx* c, int64_t n, double a, double* x);
// out = x + xᵀ for an n×n matrix (out may alias nothing)
void add_transpose(tnad_ctx* c, int64_t n, const double* x, double* out);
// Generic permutation of a column-major tensor: out has dims in.dim[perm[k]].
// out = alpha*permute(in) + beta*out
void permute(tnad_ctx* c, const Ten& in, const int* perm, double* out, double alpha = 1.0,
             double beta = 0.0);
// Deterministic sum of squares into dev_out[0] (device).
void sumsq_dev(tnad_ctx* c, const double* x, int64_t n, double* dev_out);
// Σ x∘y into dev_out[0].
void dot_dev(tnad_ctx* c, const double* x, const double* y, int64_t n, double* dev_out);
// Blocking helpers returning host values.
double norm_host(tnad_ctx* c, const double* x, int64_t n);
double dot_host(tnad_ctx* c, const double* x, const double* y, int64_t n);
// max |x| and its first index: dev_out[0] = max, dev_out[1] = index (as double)
void maxabs_dev(tnad_ctx* c, const double* x, int64_t n, double* dev_out);
// x /= dev_s[0]
void div_by_dev(tnad_ctx* c, double* x, int64_t n, const double* dev_s);
// x = x * dev_s[0] ... generic scalar ops on device scalars
void normalize_inplace(tnad_ctx* c, double* x, int64_t n, double* dev_norm_out);

// ---------------- GEMM (gemm_f64.cu, gemm_tc.cu) ----------------
// Column-major C(M×N) = alpha·op(A)·op(B) + beta·C ; ta/tb in {'N','T'}.
void gemm_f64(tnad_ctx* c, char ta, char tb, int64_t M, int64_t N, int64_t K, double alpha,
              const double* A, int64_t lda, const double* B, int64_t ldb, double beta, double* C,
              int64_t ldc);
// Same contract, 3xTF32 on tcgen05 tensor cores with FP32 accumulation.
void gemm_tf32x3(tnad_ctx* c, char ta, char tb, int64_t M, int64_t N, int64_t K, double alpha,
                 const double* A, int64_t lda, const double* B, int64_t ldb, double beta,
                 double* C, int64_t ldc);
// FP32 C(M×N) = alpha·op(A)·op(B) + beta·C with operands rounded to BF16 and FP32
// accumulation on tcgen05 tensor cores (chunks of 512 K values summed in FP64).
void gemm_bf16(tnad_ctx* c, char ta, char tb, int64_t M, int64_t N, int64_t K, float alpha, const float* A,
               int64_t lda, const float* B, int64_t ldb, float beta, float* C, int64_t ldc);
// Same contract, FP64-accurate (about 2^−47 of the row/column scales) from BF16
// slices on the tcgen05 tensor cores (gemm_oz.cu); unless `always`, products
// below a few million multiply-adds go to gemm_f64 (as fast there).
void gemm_fp64tc(tnad_ctx* c, char ta, char tb, int64_t M, int64_t N, int64_t K, double alpha,
                 const double* A, int64_t lda, const double* B, int64_t ldb, double beta,
                 double* C, int64_t ldc, bool always = false);
// Raises TNAD_ERR_TIMEOUT if a tensor-core GEMM gave up on a bounded wait (syncs).
void check_tc_errors(tnad_ctx* c);
void gemm(tnad_ctx* c, int prec, char ta, char tb, int64_t M, int64_t N, int64_t K, double alpha,
          const double* A, int64_t lda, const double* B, int64_t ldb, double beta, double* C,
          int64_t ldc);

// ---------------- pairwise contraction (contract.cpp) ----------------
// C[lc] = alpha · Σ A[la]·B[lb] + beta·C[lc]; labels are single characters.
// C.p must hold numel(C); its dims are filled in from A and B.
void contract(tnad_ctx* c, int prec, const Ten& A, const char* la, const Ten& B, const char* lb,
              Ten& C, const char* lc, double alpha = 1.0, double beta = 0.0);
// Output dims of a contraction (without computing).
Ten contract_shape(const Ten& A, const char* la, const Ten& B, const char* lb, const char* lc);

// ---------------- FP64 Jacobi SVD (jacobi.cu) ----------------
// Thin SVD of m×n (m ≥ n) A: U m×n, S n (descending), V n×n.  A is not modified.
// symmetric=true: A is symmetric, null-space columns of U are completed from V.
// rel_sweeps: sweeps with the purely relative stop rule before the rounding
// floor ε·‖A‖_F applies (relative accuracy of small triplets, needed where
// √s of them is differentiated, as in TRG; 0 gives LAPACK-level accuracy).
void svd_jacobi(tnad_ctx* c, const double* A, int64_t m, int64_t n, double* U, double* S,
                double* V, bool symmetric, int rel_sweeps = 20);
// Refines X (n×n, nearly orthonormal approximate eigenvectors of the symmetric
// A, n ≤ 2048) to FP64 accuracy by matrix products; lam gets the eigenvalues
// (column order of X).  fro2: ‖A‖²_F on the device.  false: no convergence
// (X is then unusable and the caller falls back to Jacobi sweeps).
bool eig_refine(tnad_ctx* c, const double* A, int64_t n, double* X, double* lam, const double* fro2);
// FP64-accurate eigendecomposition of a small symmetric p×p matrix (p ≤ 256):
// one-CTA FP32 Jacobi, then eig_refine; W, lam sorted by |λ| descending.
// false: the refinement did not converge (W, lam untouched).
bool eigh_fp32_refined(tnad_ctx* c, const double* H, int64_t p, double* W, double* lam);
// Symmetric eigendecomposition of a small p×p matrix (p ≤ 256) by cyclic Jacobi in
// one CTA: A = W·diag(lam)·Wᵀ, sorted by |lam| descending.
void eigh_small(tnad_ctx* c, const double* A, int64_t p, double* W, double* lam);
// The same with the sweep precision (fp32: FP32 rotations, FP64 in/out), a sweep
// cap, the sweep count in dev_info[0] (may be null), and the order: |λ|
// descending, or λ descending when by_value.
void eigh_small_prec(tnad_ctx* c, bool fp32, const double* A, int64_t p, double* W, double* lam, int max_sweeps,
                     int* dev_info, bool by_value = false);

// ---------------- SVD adjoint (svd_back.cu) ----------------
// Square thin SVD (n×n) with dU non-zero only in its first k columns (dUk n×k).
// kept_sym: Uᵀ·dU is symmetric on the kept k×k block (a gauge-invariant use of
// U[:, 1:k]), whose terms are then exactly 0 and skipped.
void svd_back_cols(tnad_ctx* c, int prec, const double* U, const double* S, const double* V, int64_t n, int64_t k,
                   const double* dUk, double eta, double* dA, bool kept_sym = false);
// svd_back for thin SVD (U m×n, S n, V n×n), dU m×n or null, dS n or null, dV n×n or null.
void svd_back(tnad_ctx* c, int prec, const double* U, const double* S, const double* V, int64_t m,
              int64_t n, const double* dU, const double* dS, const double* dV, double eta,
              double* dA);

}  // namespace tnad
