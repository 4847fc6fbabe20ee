// FP64 one-sided (Hestenes) Jacobi SVD: the decomposition of src/ctmrg.jl:136
// and src/trg.jl:36 (LinearAlgebra.svd).  GB300 has a narrow FP64 pipe, so the
// schedule spreads every round over all SMs: a round of the circle-method
// tournament pairs all columns at once, one warp per column pair (three dot
// products by warp shuffle, one plane rotation of W and V).  A sweep is n−1
// rounds; sweeps repeat until no pair needed a rotation (relative
// orthogonality ≤ m·ε), capped at kMaxSweeps (→ TNAD_ERR_NOT_CONVERGED).
// Singular values are the column norms, sorted descending by a rank kernel
// (ties by index, so the result is deterministic).
#include <algorithm>
#include <atomic>
#include <cfloat>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <mutex>

#include "tc_common.cuh"
#include "tnad_internal.h"

namespace tnad {

static const int kMaxSweeps = 100;
static const int kRelSweeps = 20;  // relative-rule sweeps of the general (non-symmetric) SVD
static const int kMaxSweeps32 = 30;  // FP32 preconditioning sweeps (symmetric A)
static const int64_t kPrecondMinN = 256;  // smaller matrices skip the FP32 preconditioning
static const int kEigSkip = 8;  // symmetric SVDs of a size that skip the refinement after it fell back

__device__ __forceinline__ double wsum(double v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}

__device__ __forceinline__ void pair_of(int r, int k, int NP, int* p, int* q) {
  // circle method over NP (even) players; round r in [0, NP-1), pair k in [0, NP/2)
  if (k == 0) {
    *p = NP - 1;
    *q = r;
  } else {
    *p = (r + k) % (NP - 1);
    *q = (r - k + (NP - 1)) % (NP - 1);
  }
}

__global__ void k_jacobi_round(double* __restrict__ W, double* __restrict__ V, int64_t m, int64_t n, int r, int NP,
                               double tol, double abs_eps, const double* __restrict__ fro2, int* __restrict__ rotated) {
  int warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  int lane = threadIdx.x & 31;
  if (warp >= NP / 2) return;
  int p, q;
  pair_of(r, warp, NP, &p, &q);
  if (p >= n || q >= n) return;  // bye
  if (p > q) {
    int t = p;
    p = q;
    q = t;
  }
  double* wp = W + (int64_t)p * m;
  double* wq = W + (int64_t)q * m;
  double a = 0.0, b = 0.0, g = 0.0;
  for (int64_t i = lane; i < m; i += 32) {
    double x = wp[i], y = wq[i];
    a = fma(x, x, a);
    b = fma(y, y, b);
    g = fma(x, y, g);
  }
  a = wsum(a);
  b = wsum(b);
  g = wsum(g);
  if (g == 0.0 || a == 0.0 || b == 0.0) return;
  // Stop rule: relative orthogonality m·ε, plus the rounding floor.  Every
  // rotation against a large column leaves noise of size ~ε·‖A‖ in a small one,
  // so |γ| cannot drop below ~ε·‖A‖_F·(‖w_p‖+‖w_q‖); rotating below that only
  // reshuffles noise (and never terminates on graded spectra such as TRG's).
  if (fabs(g) <= tol * sqrt(a) * sqrt(b) + abs_eps * sqrt(fro2[0]) * (sqrt(a) + sqrt(b))) return;
  double zeta = (b - a) / (2.0 * g);
  double t;
  if (fabs(zeta) > 1e150)
    t = 0.5 / zeta;
  else
    t = copysign(1.0, zeta) / (fabs(zeta) + sqrt(1.0 + zeta * zeta));
  double cs = 1.0 / sqrt(1.0 + t * t);
  double sn = cs * t;
  for (int64_t i = lane; i < m; i += 32) {
    double x = wp[i], y = wq[i];
    wp[i] = cs * x - sn * y;
    wq[i] = sn * x + cs * y;
  }
  double* vp = V + (int64_t)p * n;
  double* vq = V + (int64_t)q * n;
  for (int64_t i = lane; i < n; i += 32) {
    double x = vp[i], y = vq[i];
    vp[i] = cs * x - sn * y;
    vq[i] = sn * x + cs * y;
  }
  if (lane == 0) atomicAdd(rotated, 1);
}

// Same round with one 128-thread CTA per column pair: each thread keeps R rows
// of both columns in registers (one read and one write of W per round), the
// three dot products reduce through warp shuffles and shared memory.  T is
// double for the decomposition itself and float for the preconditioning sweeps
// (rotation angles are always formed in FP64).
template <typename T>
__device__ __forceinline__ T wsum_t(T v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}

// EIG = true (symmetric A, m = n, W = A·V): the rotation diagonalises the 2×2
// block of VᵀAV instead of the Gram matrix of W, from a = v_p·w_p, b = v_q·w_q
// and g = (v_p·w_q + v_q·w_p)/2 (the two-sided Jacobi method for eigenvalues,
// in the one-sided storage).  Columns for eigenvalues ±λ are then never mixed,
// as they are in the SVD form, where both have the singular value |λ|.  Its
// stop rule is absolute: |g| ≤ tol·√|ab| + abs_eps·‖A‖_F.
template <int R, typename T, bool EIG = false>
__global__ void __launch_bounds__(128) k_jacobi_round_cta(T* __restrict__ W, T* __restrict__ V, int64_t m,
                                                          int64_t n, int r, int NP, double tol, double abs_eps,
                                                          const double* __restrict__ fro2, int* __restrict__ rotated) {
  __shared__ T red[3][4];
  __shared__ T rot[2];
  int p, q;
  pair_of(r, blockIdx.x, NP, &p, &q);
  if (p >= n || q >= n) return;  // bye (uniform across the CTA)
  if (p > q) {
    int t = p;
    p = q;
    q = t;
  }
  T* wp = W + (int64_t)p * m;
  T* wq = W + (int64_t)q * m;
  T* vp = V + (int64_t)p * n;
  T* vq = V + (int64_t)q * n;
  T x[R], y[R], vx[R], vy[R];
  T a = 0, b = 0, g = 0;
  // V's columns are loaded up front with W's (n ≤ m here): their latency
  // overlaps the reduction instead of following the rotation decision
#pragma unroll
  for (int k = 0; k < R; ++k) {
    const int64_t i = threadIdx.x + (int64_t)k * 128;
    x[k] = i < m ? wp[i] : (T)0;
    y[k] = i < m ? wq[i] : (T)0;
    vx[k] = i < n ? vp[i] : (T)0;
    vy[k] = i < n ? vq[i] : (T)0;
  }
#pragma unroll
  for (int k = 0; k < R; ++k) {
    if (EIG) {
      a = fma(vx[k], x[k], a);
      b = fma(vy[k], y[k], b);
      g = fma(vx[k], y[k], g);
      g = fma(vy[k], x[k], g);
    } else {
      a = fma(x[k], x[k], a);
      b = fma(y[k], y[k], b);
      g = fma(x[k], y[k], g);
    }
  }
  if (EIG) g *= (T)0.5;
  a = wsum_t(a);
  b = wsum_t(b);
  g = wsum_t(g);
  const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
  if (lane == 0) {
    red[0][w] = a;
    red[1][w] = b;
    red[2][w] = g;
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    // The stop test and the rotation angle are formed in the sweep's own
    // precision: on GB300 the FP64 square roots and divisions of this single
    // thread sit on the round's critical path.
    const T A = red[0][0] + red[0][1] + red[0][2] + red[0][3];
    const T B = red[1][0] + red[1][1] + red[1][2] + red[1][3];
    const T G = red[2][0] + red[2][1] + red[2][2] + red[2][3];
    T cs = 1, sn = 0;
    bool do_rot;
    if (EIG) {
      do_rot = G != (T)0 && fabs(G) > (T)tol * sqrt(fabs(A * B)) + (T)abs_eps * sqrt((T)fro2[0]);
    } else {
      const T sa = sqrt(A), sb = sqrt(B);
      do_rot = G != (T)0 && A != (T)0 && B != (T)0 &&
               fabs(G) > (T)tol * sa * sb + (T)abs_eps * sqrt((T)fro2[0]) * (sa + sb);
    }
    if (do_rot) {
      const T zeta = (B - A) / ((T)2 * G);
      const T big = sizeof(T) == 8 ? (T)1e150 : (T)1e18;
      const T t = fabs(zeta) > big ? (T)0.5 / zeta : copysign((T)1, zeta) / (fabs(zeta) + sqrt((T)1 + zeta * zeta));
      cs = (T)1 / sqrt((T)1 + t * t);
      sn = cs * t;
      atomicAdd(rotated, 1);
    }
    rot[0] = cs;
    rot[1] = sn;
  }
  __syncthreads();
  const T cs = rot[0], sn = rot[1];
  if (sn == (T)0) return;
#pragma unroll
  for (int k = 0; k < R; ++k) {
    const int64_t i = threadIdx.x + (int64_t)k * 128;
    if (i < m) {
      wp[i] = cs * x[k] - sn * y[k];
      wq[i] = sn * x[k] + cs * y[k];
    }
  }
#pragma unroll
  for (int k = 0; k < R; ++k) {
    const int64_t i = threadIdx.x + (int64_t)k * 128;
    if (i < n) {
      vp[i] = cs * vx[k] - sn * vy[k];
      vq[i] = sn * vx[k] + cs * vy[k];
    }
  }
}

// one round over all column pairs (T = double or float)
template <typename T, bool EIG = false>
void jacobi_round_launch(tnad_ctx* c, T* W, T* V, int64_t m, int64_t n, int r, int NP, double tol, double ae,
                         const double* fro2, int* flag) {
  const unsigned np2 = (unsigned)(NP / 2);
  if (m <= 256)
    k_jacobi_round_cta<2, T, EIG><<<np2, 128, 0, c->stream>>>(W, V, m, n, r, NP, tol, ae, fro2, flag);
  else if (m <= 512)
    k_jacobi_round_cta<4, T, EIG><<<np2, 128, 0, c->stream>>>(W, V, m, n, r, NP, tol, ae, fro2, flag);
  else if (m <= 1024)
    k_jacobi_round_cta<8, T, EIG><<<np2, 128, 0, c->stream>>>(W, V, m, n, r, NP, tol, ae, fro2, flag);
  else
    k_jacobi_round_cta<16, T, EIG><<<np2, 128, 0, c->stream>>>(W, V, m, n, r, NP, tol, ae, fro2, flag);
}

// Block variant of the FP32 round.  The columns are grouped in blocks of 4
// (the last one may be short) and the circle-method tournament runs over the
// NB blocks (NB even; with an odd count of real blocks, block NB − 1 is a bye
// whose columns lie beyond n and count as absent).  CTA k takes the block pair
// (P, Q) of round r and holds their 8 columns of W (m rows) and V (n rows) in
// shared memory.  It applies the same plane rotation as k_jacobi_round_cta to
// every cross pair (column of P, column of Q): 4 inner rounds of 4 disjoint
// pairs, TP threads per pair, each thread with 16 rows of the pair's columns in
// registers (independent loads), the dot products reduced by shuffles and a
// fixed-order sum of the pair's warp partials (every thread of the pair forms
// the same angle).  In the first round of a sweep (intra = 1) the pairs inside
// P and inside Q are rotated first (3 inner rounds), so that the NB − 1
// launches of a sweep visit every column pair once, as the n − 1 launches of
// the element rounds do, with a quarter of their launches and global passes.
constexpr int kJB = 4;          // columns per block
constexpr int kJBRows = 16;     // rows per thread
//
// With `bulk` (m and n multiples of 4, W and V 16-byte aligned) the columns
// move between global and shared memory as one-dimensional bulk copies
// (cp.async.bulk): thread 0 issues the 16 loads against one mbarrier and,
// at the end, the 16 stores; the wait on the mbarrier is bounded (2 s of
// %globaltimer), after which the CTA sets *err, waits once more (bounded) for
// its copies in flight and returns without rotating.
template <bool EIG, int TP>
__global__ void __launch_bounds__(kJB * TP) k_jacobi_block(float* __restrict__ W, float* __restrict__ V, int m, int n,
                                                           int NB, int r, int intra, double tol, double abs_eps,
                                                           const double* __restrict__ fro2,
                                                           int* __restrict__ rotated, int bulk, int* __restrict__ err) {
  extern __shared__ __align__(16) unsigned char smraw[];
  float* Ws = reinterpret_cast<float*>(smraw);  // 8 columns × m
  float* Vs = Ws + (size_t)2 * kJB * m;         // 8 columns × n
  __shared__ float red[kJB][TP / 32][3];
  __shared__ __align__(8) uint64_t bar;
  int P, Q;
  pair_of(r, blockIdx.x, NB, &P, &Q);
  const int tid = threadIdx.x, nt = blockDim.x;
  auto gcol = [&](int c) { return c < kJB ? P * kJB + c : Q * kJB + (c - kJB); };
  if (bulk) {
    const uint32_t b = tc::su32(&bar);
    if (tid == 0) {
      tc::mbar_init(b, 1);
      asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    __syncthreads();
    if (tid == 0) {
      uint32_t bytes = 0;
      for (int c = 0; c < 2 * kJB; ++c)
        if (gcol(c) < n) bytes += (uint32_t)(m + n) * 4u;
      tc::mbar_expect_tx(b, bytes);
      for (int c = 0; c < 2 * kJB; ++c) {
        const int g = gcol(c);
        if (g >= n) continue;
        asm volatile(
            "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
                tc::su32(Ws + (size_t)c * m)),
            "l"(W + (int64_t)g * m), "r"(m * 4), "r"(b)
            : "memory");
        asm volatile(
            "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
                tc::su32(Vs + (size_t)c * n)),
            "l"(V + (int64_t)g * n), "r"(n * 4), "r"(b)
            : "memory");
      }
    }
    const bool ok = tc::mbar_wait(b, 0, err, 1, 2000000000ull);
    if (__syncthreads_or(ok ? 0 : 1)) {
      tc::mbar_wait(b, 0, err, 1, 2000000000ull);  // the copies still in flight, bounded
      return;
    }
  } else {
    for (int c = 0; c < 2 * kJB; ++c) {
      const int g = gcol(c);
      if (g >= n) continue;
      const float* wsrc = W + (int64_t)g * m;
      const float* vsrc = V + (int64_t)g * n;
      for (int i = tid; i < m; i += nt) Ws[(size_t)c * m + i] = wsrc[i];
      for (int i = tid; i < n; i += nt) Vs[(size_t)c * n + i] = vsrc[i];
    }
    __syncthreads();
  }
  const float thr_abs = (float)abs_eps * sqrtf((float)fro2[0]);
  const int slot = tid / TP, lt = tid % TP, wip = lt >> 5, lane = tid & 31;
  int nrot = 0;
  // one inner-round step for local columns (a, c) of this thread's pair; every
  // thread of the CTA calls it once per inner round (the barrier inside)
  auto process = [&](int a, int c) {
    int ga = gcol(a), gc = gcol(c);
    const bool present = ga < n && gc < n;
    if (ga > gc) {
      const int t = a;
      a = c;
      c = t;
    }
    float x[kJBRows], y[kJBRows], vx[kJBRows], vy[kJBRows];
    float A = 0.f, B = 0.f, G = 0.f, G2 = 0.f;
    if (present) {
#pragma unroll
      for (int e = 0; e < kJBRows; ++e) {
        const int i = lt + TP * e;
        x[e] = i < m ? Ws[(size_t)a * m + i] : 0.f;
        y[e] = i < m ? Ws[(size_t)c * m + i] : 0.f;
        vx[e] = i < n ? Vs[(size_t)a * n + i] : 0.f;
        vy[e] = i < n ? Vs[(size_t)c * n + i] : 0.f;
      }
#pragma unroll
      for (int e = 0; e < kJBRows; ++e) {
        if (EIG) {
          A = fmaf(vx[e], x[e], A);
          B = fmaf(vy[e], y[e], B);
          G = fmaf(vx[e], y[e], G);
          G2 = fmaf(vy[e], x[e], G2);
        } else {
          A = fmaf(x[e], x[e], A);
          B = fmaf(y[e], y[e], B);
          G = fmaf(x[e], y[e], G);
        }
      }
      if (EIG) G = 0.5f * (G + G2);
      A = wsum_t(A);
      B = wsum_t(B);
      G = wsum_t(G);
      if (lane == 0) {
        red[slot][wip][0] = A;
        red[slot][wip][1] = B;
        red[slot][wip][2] = G;
      }
    }
    __syncthreads();
    bool do_rot = false;
    float cs = 1.f, sn = 0.f;
    if (present) {
      A = B = G = 0.f;
#pragma unroll
      for (int w = 0; w < TP / 32; ++w) {
        A += red[slot][w][0];
        B += red[slot][w][1];
        G += red[slot][w][2];
      }
      if (EIG) {
        do_rot = G != 0.f && fabsf(G) > (float)tol * sqrtf(fabsf(A * B)) + thr_abs;
      } else {
        const float sa = sqrtf(A), sb = sqrtf(B);
        do_rot = G != 0.f && A != 0.f && B != 0.f && fabsf(G) > (float)tol * sa * sb + thr_abs * (sa + sb);
      }
      if (do_rot) {
        const float zeta = (B - A) / (2.f * G);
        const float t =
            fabsf(zeta) > 1e18f ? 0.5f / zeta : copysignf(1.f, zeta) / (fabsf(zeta) + sqrtf(1.f + zeta * zeta));
        cs = 1.f / sqrtf(1.f + t * t);
        sn = cs * t;
#pragma unroll
        for (int e = 0; e < kJBRows; ++e) {
          const int i = lt + TP * e;
          if (i < m) {
            Ws[(size_t)a * m + i] = cs * x[e] - sn * y[e];
            Ws[(size_t)c * m + i] = sn * x[e] + cs * y[e];
          }
          if (i < n) {
            Vs[(size_t)a * n + i] = cs * vx[e] - sn * vy[e];
            Vs[(size_t)c * n + i] = sn * vx[e] + cs * vy[e];
          }
        }
        if (lt == 0) ++nrot;
      }
    }
    __syncthreads();
  };
  if (intra) {
    // pairs inside P (slots 0, 1) and inside Q (slots 2, 3): 3 inner rounds
    for (int ir = 0; ir < kJB - 1; ++ir) {
      int a, c;
      pair_of(ir, slot & 1, kJB, &a, &c);
      if (slot >= 2) {
        a += kJB;
        c += kJB;
      }
      process(a, c);
    }
  }
  // cross pairs: in inner round ir, slot k pairs P's column k with Q's column (k + ir) mod 4
  for (int ir = 0; ir < kJB; ++ir) process(slot, kJB + ((slot + ir) & (kJB - 1)));
  if (bulk) {
    // the rotations wrote shared memory through the generic proxy: fence it
    // towards the async proxy before the bulk stores read it
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
    __syncthreads();
    if (tid == 0) {
      for (int c = 0; c < 2 * kJB; ++c) {
        const int g = gcol(c);
        if (g >= n) continue;
        asm volatile("cp.async.bulk.global.shared::cta.bulk_group [%0], [%1], %2;" ::"l"(W + (int64_t)g * m),
                     "r"(tc::su32(Ws + (size_t)c * m)), "r"(m * 4)
                     : "memory");
        asm volatile("cp.async.bulk.global.shared::cta.bulk_group [%0], [%1], %2;" ::"l"(V + (int64_t)g * n),
                     "r"(tc::su32(Vs + (size_t)c * n)), "r"(n * 4)
                     : "memory");
      }
      asm volatile("cp.async.bulk.commit_group;" ::: "memory");
      asm volatile("cp.async.bulk.wait_group 0;" ::: "memory");
    }
  } else {
    for (int c = 0; c < 2 * kJB; ++c) {
      const int g = gcol(c);
      if (g >= n) continue;
      float* wdst = W + (int64_t)g * m;
      float* vdst = V + (int64_t)g * n;
      for (int i = tid; i < m; i += nt) wdst[i] = Ws[(size_t)c * m + i];
      for (int i = tid; i < n; i += nt) vdst[i] = Vs[(size_t)c * n + i];
    }
  }
  if (lt == 0 && nrot) atomicAdd(rotated, nrot);
}

// Threads per pair of the FP32 block rounds (16 rows each, 64 threads): 0 when
// the block rounds do not apply (m beyond 1024 rows, or n > m).  Taller
// matrices keep the element rounds: with 128 threads per pair the block rounds
// were measured no faster at n = 1600, and their FP32 start needed more
// refinement iterations there.
inline int jacobi_block_tp(int64_t m, int64_t n) {
  if (n > m || m > 64 * kJBRows) return 0;
  return 64;
}

template <bool EIG>
void jacobi_block_launch(tnad_ctx* c, float* W, float* V, int64_t m, int64_t n, int tp, int NB, int r, double tol,
                         double ae, const double* fro2, int* flag) {
  static std::atomic<bool> attr{false};
  if (!attr) {
    TNAD_CK(cudaFuncSetAttribute(k_jacobi_block<EIG, 64>, cudaFuncAttributeMaxDynamicSharedMemorySize, 96 * 1024));
    attr = true;
  }
  (void)tp;  // 64 threads per pair (jacobi_block_tp)
  const size_t sm = (size_t)2 * kJB * (m + n) * sizeof(float);
  // bulk copies need 16-byte aligned columns: m, n multiples of 4 and aligned bases
  const int bulk = (m % 4 == 0 && n % 4 == 0 && ((uintptr_t)W & 15) == 0 && ((uintptr_t)V & 15) == 0) ? 1 : 0;
  k_jacobi_block<EIG, 64><<<(unsigned)(NB / 2), kJB * 64, sm, c->stream>>>(W, V, (int)m, (int)n, NB, r,
                                                                           r == 0 ? 1 : 0, tol, ae, fro2, flag, bulk,
                                                                           flag + 2);
}

// One Jacobi sweep (flag reset + the NP−1 rounds) recorded once as a CUDA
// graph and replayed for every sweep: the rounds are short kernels whose
// launch cost is comparable to their run time.  Very small matrices are
// launched directly.
template <typename T, bool EIG = false>
struct SweepGraph {
  cudaGraphExec_t exec = nullptr;
  double ae_ = -1.0;
  int tp = 0;  // > 0 (FP32 only): block rounds (k_jacobi_block, tp threads per pair), NB − 1 launches a sweep
  ~SweepGraph() {
    if (exec) cudaGraphExecDestroy(exec);
  }
  void run(tnad_ctx* c, const char* family, T* W, T* V, int64_t m, int64_t n, int NP, double tol, double ae,
           const double* fro2, int* flag, double round_flops) {
    if constexpr (sizeof(T) == 4) {
      if (tp > 0) {
        run_blocks(c, family, W, V, m, n, tol, ae, fro2, flag, round_flops * (double)(NP - 1));
        return;
      }
    }
    if (NP < 64) {
      TNAD_CK(cudaMemsetAsync(flag, 0, sizeof(int), c->stream));
      for (int r = 0; r < NP - 1; ++r) {
        KernelTimer kt(c, family, round_flops);
        jacobi_round_launch<T, EIG>(c, W, V, m, n, r, NP, tol, ae, fro2, flag);
      }
    } else {
      if (exec && ae != ae_) {
        TNAD_CK(cudaGraphExecDestroy(exec));
        exec = nullptr;
      }
      if (!exec) {
        cudaGraph_t g = nullptr;
        TNAD_CK(cudaStreamBeginCapture(c->stream, cudaStreamCaptureModeThreadLocal));
        cudaError_t e = cudaMemsetAsync(flag, 0, sizeof(int), c->stream);
        for (int r = 0; r < NP - 1 && e == cudaSuccess; ++r) {
          jacobi_round_launch<T, EIG>(c, W, V, m, n, r, NP, tol, ae, fro2, flag);
          e = cudaGetLastError();
        }
        const cudaError_t e2 = cudaStreamEndCapture(c->stream, &g);
        if (e == cudaSuccess) e = e2;
        if (e == cudaSuccess) e = cudaGraphInstantiate(&exec, g, 0);
        if (g) cudaGraphDestroy(g);
        if (e != cudaSuccess) fail(TNAD_ERR_CUDA, std::string("jacobi sweep graph: ") + cudaGetErrorString(e));
        ae_ = ae;
      }
      // timed as one bracket around the replayed sweep (events cannot go inside
      // the graph): the average launch duration includes the graph's own gaps
      KernelTimer kt(c, family, round_flops * (NP - 1), NP - 1);
      TNAD_CK(cudaGraphLaunch(exec, c->stream));
    }
    count_launch(c, NP - 1);
    check_launch(c, family);
  }
  // one sweep of block rounds (NB − 1 launches of k_jacobi_block), captured
  // once as a graph and replayed; sweep_flops: the sweep's algorithmic work
  void run_blocks(tnad_ctx* c, const char* family, T* W, T* V, int64_t m, int64_t n, double tol, double ae,
                  const double* fro2, int* flag, double sweep_flops) {
    const int nreal = (int)((n + kJB - 1) / kJB);
    const int NB = nreal + (nreal & 1);
    if (exec && ae != ae_) {
      TNAD_CK(cudaGraphExecDestroy(exec));
      exec = nullptr;
    }
    if (!exec) {
      cudaGraph_t g = nullptr;
      TNAD_CK(cudaStreamBeginCapture(c->stream, cudaStreamCaptureModeThreadLocal));
      cudaError_t e = cudaMemsetAsync(flag, 0, sizeof(int), c->stream);
      for (int r = 0; r < NB - 1 && e == cudaSuccess; ++r) {
        jacobi_block_launch<EIG>(c, W, V, m, n, tp, NB, r, tol, ae, fro2, flag);
        e = cudaGetLastError();
      }
      const cudaError_t e2 = cudaStreamEndCapture(c->stream, &g);
      if (e == cudaSuccess) e = e2;
      if (e == cudaSuccess) e = cudaGraphInstantiate(&exec, g, 0);
      if (g) cudaGraphDestroy(g);
      if (e != cudaSuccess) fail(TNAD_ERR_CUDA, std::string("jacobi block sweep graph: ") + cudaGetErrorString(e));
      ae_ = ae;
    }
    KernelTimer kt(c, family, sweep_flops, NB - 1);
    TNAD_CK(cudaGraphLaunch(exec, c->stream));
    count_launch(c, NB - 1);
    check_launch(c, family);
  }
};

__global__ void k_to_float(const double* __restrict__ x, int64_t n, float* __restrict__ y) {
  for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < n; e += (int64_t)gridDim.x * blockDim.x)
    y[e] = (float)x[e];
}

__global__ void k_to_double(const float* __restrict__ x, int64_t n, double* __restrict__ y) {
  for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < n; e += (int64_t)gridDim.x * blockDim.x)
    y[e] = (double)x[e];
}

__global__ void k_eye_f(float* V, int64_t n) {
  for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < n * n; e += (int64_t)gridDim.x * blockDim.x)
    V[e] = (e % n == e / n) ? 1.f : 0.f;
}

__global__ void k_eye(double* V, int64_t n) {
  int64_t nn = n * n;
  for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < nn; e += (int64_t)gridDim.x * blockDim.x)
    V[e] = (e % n == e / n) ? 1.0 : 0.0;
}

// s_j = ‖W_j‖ ; sg_j = sign(V_j·W_j) (used for the null/weak columns of a symmetric A)
__global__ void k_colnorms(const double* __restrict__ W, const double* __restrict__ Vw, int64_t m, int64_t n,
                           double* __restrict__ s, double* __restrict__ sg) {
  int warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  int lane = threadIdx.x & 31;
  if (warp >= n) return;
  const double* w = W + (int64_t)warp * m;
  const double* v = Vw + (int64_t)warp * n;
  double a = 0.0, g = 0.0;
  for (int64_t i = lane; i < m; i += 32) {
    a = fma(w[i], w[i], a);
    if (i < n) g = fma(v[i], w[i], g);
  }
  a = wsum(a);
  g = wsum(g);
  if (lane == 0) {
    s[warp] = sqrt(a);
    sg[warp] = g < 0.0 ? -1.0 : 1.0;
  }
}

// rank[j] = #{i : s_i > s_j or (s_i == s_j and i < j)}  → descending order
__global__ void k_rank(const double* __restrict__ s, int64_t n, int* __restrict__ rank) {
  int64_t j = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (j >= n) return;
  double sj = s[j];
  int r = 0;
  for (int64_t i = 0; i < n; ++i) {
    double si = s[i];
    r += (si > sj || (si == sj && i < j)) ? 1 : 0;
  }
  rank[j] = r;
}

// Scatter sorted: S[rank j] = ‖W_j‖, V_out[:, rank j] = V_j and
//  - symmetric A: U[:, rank j] = sign(V_j·W_j)·V_j — the left vectors of a
//    symmetric matrix are its signed right vectors when V_j is an eigenvector,
//    and V (a product of plane rotations) is orthogonal to working precision,
//    including null columns.  A column whose singular value is shared (to
//    1e-8 relative) with another one, e.g. a pair of eigenvalues ±λ, is only
//    determined up to a rotation inside that singular subspace, and there V_j
//    need not be an eigenvector: such a column (above the weak threshold) takes
//    U[:, rank j] = W_j/‖W_j‖ = A·V_j/σ_j, so that U, S, V stay an SVD;
//  - general A: U[:, rank j] = W_j/‖W_j‖; columns below weak_rel·‖A‖_F (whose
//    direction carries the ε·‖A‖ rounding noise) are counted and afterwards
//    re-orthonormalised against all larger ones by k_complete_col.
__global__ void k_scatter(const double* __restrict__ W, const double* __restrict__ Vw, const double* __restrict__ s,
                          const double* __restrict__ sg, const int* __restrict__ rank, int64_t m, int64_t n,
                          int symmetric, double weak_rel, const double* __restrict__ fro2, double* __restrict__ U,
                          double* __restrict__ S, double* __restrict__ Vout, int* __restrict__ nweak) {
  int64_t j = blockIdx.y;
  int r = rank[j];
  double sj = s[j];
  bool weak = !(sj > weak_rel * sqrt(fro2[0])) || !(sj > 1e-300);
  // shared singular value (symmetric A): does another column have σ within 1e-8·σ_j?
  int shared = 0;
  if (symmetric && !weak)
    for (int64_t i = threadIdx.x; i < n; i += blockDim.x)
      shared |= (i != j && fabs(s[i] - sj) <= 1e-8 * sj) ? 1 : 0;
  shared = __syncthreads_or(shared);
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < m; i += (int64_t)gridDim.x * blockDim.x) {
    double u;
    if (symmetric && !shared)
      u = i < n ? sg[j] * Vw[i + j * n] : 0.0;
    else
      u = sj > 1e-300 ? W[i + j * m] / sj : 0.0;
    U[i + (int64_t)r * m] = u;
  }
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
    Vout[i + (int64_t)r * n] = Vw[i + j * n];
  if (blockIdx.x == 0 && threadIdx.x == 0) {
    S[r] = sj > 1e-300 ? sj : 0.0;
    if (weak && !symmetric) atomicAdd(nweak, 1);
  }
}

// Re-orthonormalisation of a weak column k of U (general matrices): start from
// the column itself (or e_pick, the unit vector least covered by columns
// 0..k-1, when it is zero); two rounds of classical Gram-Schmidt against
// columns 0..k-1; normalise.  One CTA per column, columns in order.
__global__ void k_complete_col(double* __restrict__ U, int64_t m, int64_t k, double* __restrict__ coef) {
  extern __shared__ double sh[];
  double* x = sh;  // m
  __shared__ double red[32];
  __shared__ int pick;
  // choose the unit vector e_i with the smallest projection onto span(U[:,0:k])
  if (threadIdx.x == 0) pick = -1;
  __syncthreads();
  double best = 2.0;
  int bi = 0;
  for (int64_t i = threadIdx.x; i < m; i += blockDim.x) {
    double p = 0.0;
    for (int64_t c = 0; c < k; ++c) p += U[i + c * m] * U[i + c * m];
    if (p < best) { best = p; bi = (int)i; }
  }
  // block argmin (first index on ties)
  __shared__ double bv[1024];
  __shared__ int bix[1024];
  bv[threadIdx.x] = best;
  bix[threadIdx.x] = bi;
  __syncthreads();
  for (int s = blockDim.x / 2; s > 0; s >>= 1) {
    if (threadIdx.x < s) {
      if (bv[threadIdx.x + s] < bv[threadIdx.x] ||
          (bv[threadIdx.x + s] == bv[threadIdx.x] && bix[threadIdx.x + s] < bix[threadIdx.x])) {
        bv[threadIdx.x] = bv[threadIdx.x + s];
        bix[threadIdx.x] = bix[threadIdx.x + s];
      }
    }
    __syncthreads();
  }
  if (threadIdx.x == 0) pick = bix[0];
  __syncthreads();
  // start from the current (noisy) column when it is non-zero, else from e_pick
  __shared__ double nz;
  if (threadIdx.x == 0) nz = 0.0;
  __syncthreads();
  double part = 0.0;
  for (int64_t i = threadIdx.x; i < m; i += blockDim.x) part += fabs(U[i + k * m]);
  part = wsum(part);
  if ((threadIdx.x & 31) == 0) atomicAdd(&nz, part);
  __syncthreads();
  for (int64_t i = threadIdx.x; i < m; i += blockDim.x) x[i] = nz > 0.0 ? U[i + k * m] : ((i == pick) ? 1.0 : 0.0);
  __syncthreads();
  for (int pass = 0; pass < 2; ++pass) {
    // coef[c] = U[:,c]·x
    for (int64_t c = threadIdx.x >> 5; c < k; c += blockDim.x >> 5) {
      double a = 0.0;
      for (int64_t i = threadIdx.x & 31; i < m; i += 32) a += U[i + c * m] * x[i];
      a = wsum(a);
      if ((threadIdx.x & 31) == 0) coef[c] = a;
    }
    __syncthreads();
    for (int64_t i = threadIdx.x; i < m; i += blockDim.x) {
      double a = x[i];
      for (int64_t c = 0; c < k; ++c) a -= U[i + c * m] * coef[c];
      x[i] = a;
    }
    __syncthreads();
  }
  double a = 0.0;
  for (int64_t i = threadIdx.x; i < m; i += blockDim.x) a += x[i] * x[i];
  a = wsum(a);
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = a;
  __syncthreads();
  if (threadIdx.x == 0) {
    double t = 0.0;
    for (int w = 0; w < (int)(blockDim.x >> 5); ++w) t += red[w];
    red[0] = sqrt(t);
  }
  __syncthreads();
  double nrm = red[0];
  for (int64_t i = threadIdx.x; i < m; i += blockDim.x) U[i + k * m] = x[i] / nrm;
}

// rank[j] = #{i : |λ_i| > |λ_j| or (= and i < j)}: descending |λ|
__global__ void k_eig_rank(const double* __restrict__ lam, int64_t n, int* __restrict__ rank) {
  const int64_t j = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (j >= n) return;
  const double a = fabs(lam[j]);
  int r = 0;
  for (int64_t i = 0; i < n; ++i) {
    const double b = fabs(lam[i]);
    r += (b > a || (b == a && i < j)) ? 1 : 0;
  }
  rank[j] = r;
}

// SVD of a symmetric A from its eigendecomposition A = X·diag(λ)·Xᵀ:
// S[r] = |λ_j|, V[:, r] = X[:, j], U[:, r] = sign(λ_j)·X[:, j] with r = rank[j]
__global__ void k_scatter_eig(const double* __restrict__ X, const double* __restrict__ lam,
                              const int* __restrict__ rank, int64_t n, double* __restrict__ U, double* __restrict__ S,
                              double* __restrict__ V) {
  const int64_t j = blockIdx.y;
  const int64_t r = rank[j];
  const double l = lam[j];
  const double sg = l < 0.0 ? -1.0 : 1.0;
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    const double x = X[i + j * n];
    V[i + r * n] = x;
    U[i + r * n] = sg * x;
  }
  if (blockIdx.x == 0 && threadIdx.x == 0) S[r] = fabs(l);
}

void svd_jacobi(tnad_ctx* c, const double* A, int64_t m, int64_t n, double* U, double* S, double* V,
                bool symmetric, int rel_sweeps) {
  TNAD_REQUIRE(m >= n && n >= 1, TNAD_ERR_SHAPE, "svd_jacobi: needs m >= n >= 1");
  WsScope scope(c);
  double* W = ws_d(c, m * n);
  double* Vw = ws_d(c, n * n);
  double* s = ws_d(c, n);
  double* sg = ws_d(c, n);
  double* fro2 = ws_d(c, 1);
  int* rank = (int*)c->ws.alloc(n * sizeof(int));
  copy_d2d(c, W, A, m * n);
  sumsq_dev(c, A, m * n, fro2);
  k_eye<<<(int)std::min<int64_t>((n * n + 255) / 256, 4096), 256, 0, c->stream>>>(Vw, n);
  count_launch(c);
  const int NP = (int)(n + (n & 1));
  // Relative orthogonality target.  After a rotation the computed |γ|/√(αβ)
  // is only as small as the rounding of an m-term dot product (~√m·ε on
  // average, up to m·ε); a √m·ε target therefore keeps re-rotating noise-level
  // columns forever.  m·ε still leaves U, V orthogonal far below 1e-10.
  const double tol = (double)std::max<int64_t>(m, 16) * DBL_EPSILON;
  const double abs_eps = 2.0 * DBL_EPSILON;
  // General A: columns with s_j ≤ 1e-8·‖A‖_F carry rounding noise in their
  // direction; they are re-orthonormalised so that U stays orthogonal.  The SVD
  // adjoint only needs those columns to span the complement of the larger ones
  // (its F-matrix is ≈ 1/s_p² across that gap), and callers that differentiate
  // through √s of such a column (trg_svd's +1 quirk) zero its value first.
  const double weak_rel = 1e-8;
  int* flag = c->d_flag;
  bool converged = (n == 1);
  const bool trace = std::getenv("TNAD_TRACE") != nullptr;  // per-sweep rotation counts to stderr
  const int threads = 256;
  const int blocks = (NP / 2 * 32 + threads - 1) / threads;
  const int64_t nb_nn = std::min<int64_t>((n * n + 255) / 256, 4096);
  if (symmetric && n >= kPrecondMinN && m <= 2048 && !converged) {
    // FP32 preconditioning: Jacobi sweeps on a float copy (the FP32 pipe is
    // much wider than the FP64 one) until rotations stop at FP32 accuracy; the
    // accumulated V32 is re-orthogonalised in FP64 (Newton–Schulz).  Then
    // either the GEMM refinement of eig_refine.cu brings V to FP64 accuracy
    // (the sweeps then use the eigenvalue rule, so that ±λ pairs come out as
    // eigenvectors), or the FP64 sweeps below start from W = A·V, whose
    // columns are then orthogonal to ~1e-5: a few sweeps instead of ~20.
    //
    // A size whose last refinement did not converge (a graded spectrum; the
    // plain path decomposes similar corners every step) skips the next
    // kEigSkip attempts: those take the SVD-rule FP32 start, whose relative
    // orthogonality suits the FP64 sweeps, and count as fallbacks.
    bool refine = c->eig_refine && m == n && n <= 2048;
    if (refine && c->eig_skip_n == n && c->eig_skip_left > 0) {
      --c->eig_skip_left;
      ++c->eig_fallback;
      refine = false;
    }
    float* W32 = ws_f(c, m * n);
    float* V32 = ws_f(c, n * n);
    k_to_float<<<(int)std::min<int64_t>((m * n + 255) / 256, 4096), 256, 0, c->stream>>>(A, m * n, W32);
    k_eye_f<<<(int)nb_nn, 256, 0, c->stream>>>(V32, n);
    count_launch(c, 2);
    // eigenvalue rule: rotate while |v_pᵀAv_q| > 2ε₃₂‖A‖_F (the FP32 floor);
    // SVD rule: relative orthogonality 4√m·ε₃₂ of the columns of W
    const double tol32 = refine ? 0.0 : 4.0 * std::sqrt((double)m) * FLT_EPSILON, ae32 = 2.0 * FLT_EPSILON;
    // block rounds (b columns per block): 1/b of the launches and global passes
    SweepGraph<float> sweep32;
    SweepGraph<float, true> sweep32e;
    if (c->jacobi_blocks) sweep32.tp = sweep32e.tp = jacobi_block_tp(m, n);
    const double round_flops = (double)(n / 2) * (12.0 * (double)m + 6.0 * (double)n);
    for (int sweep = 0; sweep < kMaxSweeps32; ++sweep) {
      if (refine)
        sweep32e.run(c, "jacobi_round_f32", W32, V32, m, n, NP, tol32, ae32, fro2, flag, round_flops);
      else
        sweep32.run(c, "jacobi_round_f32", W32, V32, m, n, NP, tol32, ae32, fro2, flag, round_flops);
      // rotation count, and the error slot of the block rounds' bounded waits
      TNAD_CK(cudaMemcpyAsync(c->h_flag, flag, 3 * sizeof(int), cudaMemcpyDeviceToHost, c->stream));
      TNAD_CK(cudaStreamSynchronize(c->stream));
      if (c->h_flag[2] != 0) {
        TNAD_CK(cudaMemsetAsync(flag + 2, 0, sizeof(int), c->stream));
        fail(TNAD_ERR_TIMEOUT, "jacobi block round: bounded mbarrier wait expired");
      }
      if (trace) std::fprintf(stderr, "[tnad trace] svd n=%lld fp32 sweep %d rotations %d\n", (long long)n, sweep, c->h_flag[0]);
      // The FP64 polish re-converges the small-σ columns anyway (V32's absolute
      // FP32 error is large relative to them), so the FP32 phase stops once
      // fewer than 16n pairs (~3% of them) still rotate.
      if (c->h_flag[0] <= 16 * (int)n) break;
    }
    k_to_double<<<(int)nb_nn, 256, 0, c->stream>>>(V32, n * n, Vw);
    count_launch(c);
    // V ← V·(3I − VᵀV)/2, three times: orthogonal to FP64 rounding.  The first
    // step (from ‖VᵀV − I‖ ~ 1e-5) runs its products on the tensor cores
    // (3xTF32, error ~1e-7); the two FP64 steps after it square the error away.
    double* G = ws_d(c, n * n);
    double* V2 = ws_d(c, n * n);
    for (int it = 0; it < 3; ++it) {
      const int pr = (it == 0 && c->tc_ok) ? TNAD_PREC_TF32X3 : TNAD_PREC_FP64;
      gemm(c, pr, 'T', 'N', n, n, n, 1.0, Vw, n, Vw, n, 0.0, G, n);
      copy_d2d(c, V2, Vw, n * n);
      gemm(c, pr, 'N', 'N', n, n, n, -0.5, Vw, n, G, n, 1.5, V2, n);
      copy_d2d(c, Vw, V2, n * n);
    }
    if (refine) {
      // V2 becomes the refined eigenvectors; Vw stays as the sweeps' start
      double* lam = ws_d(c, n);
      copy_d2d(c, V2, Vw, n * n);
      if (eig_refine(c, A, n, V2, lam, fro2)) {
        ++c->eig_refined;
        if (c->eig_skip_n == n) c->eig_skip_n = 0;
        k_eig_rank<<<(int)((n + 255) / 256), 256, 0, c->stream>>>(lam, n, rank);
        dim3 g((unsigned)std::min<int64_t>((n + 255) / 256, 16), (unsigned)n);
        k_scatter_eig<<<g, 256, 0, c->stream>>>(V2, lam, rank, n, U, S, V);
        count_launch(c, 2);
        check_launch(c, "svd_scatter_eig");
        return;
      }
      ++c->eig_fallback;
      c->eig_skip_n = n;
      c->eig_skip_left = kEigSkip;
    }
    gemm_f64(c, 'N', 'N', m, n, n, 1.0, A, m, Vw, n, 0.0, W, m);
  }
  SweepGraph<double> sweep64;
  int prev_rot = 0;
  int max_sweeps = kMaxSweeps;
  if (c->fault_once == kFaultJacobiCap) {  // failure-path test: one sweep only
    max_sweeps = 1;
    c->fault_once = kFaultNone;
  }
  for (int sweep = 0; sweep < max_sweeps && !converged; ++sweep) {
    // Purely relative sweeps first (rel_sweeps of them): they drive null and
    // noise-level columns to exact orthogonality (the triplets trg_svd's √s
    // pullback relies on).  Afterwards, or from the start for rel_sweeps = 0,
    // the rounding floor applies: every triplet is then accurate to ε·‖A‖_F
    // (the accuracy of LAPACK's SVD), and noise-level columns stop rotating.
    const double ae = sweep < rel_sweeps ? 0.0 : abs_eps;
    // algorithmic FP64 work of one round: per pair 3 dot products (6m flops)
    // and one plane rotation of W (6m) and V (6n)
    const double round_flops = (double)(n / 2) * (12.0 * (double)m + 6.0 * (double)n);
    if (m <= 2048) {
      // timer family: the large decompositions (the adjoint's χd×χd corner) apart
      // from the p×p Rayleigh–Ritz ones
      sweep64.run(c, n >= kPrecondMinN ? "jacobi_round" : "jacobi_round_small", W, Vw, m, n, NP, tol, ae, fro2,
                  flag, round_flops);
    } else {
      TNAD_CK(cudaMemsetAsync(flag, 0, sizeof(int), c->stream));
      for (int r = 0; r < NP - 1; ++r) {
        KernelTimer kt(c, "jacobi_round", round_flops);
        k_jacobi_round<<<blocks, threads, 0, c->stream>>>(W, Vw, m, n, r, NP, tol, ae, fro2, flag);
      }
      count_launch(c, NP - 1);
      check_launch(c, "jacobi_round");
    }
    TNAD_CK(cudaMemcpyAsync(c->h_flag, flag, sizeof(int), cudaMemcpyDeviceToHost, c->stream));
    TNAD_CK(cudaStreamSynchronize(c->stream));
    if (trace) std::fprintf(stderr, "[tnad trace] svd n=%lld fp64 sweep %d rotations %d\n", (long long)n, sweep, c->h_flag[0]);
    const int rot = c->h_flag[0];
    // symmetric, LAPACK-level rule: a sweep that only rotated a few pairs, far
    // fewer than the sweep before (quadratic regime), applied only tiny angles
    // and needs no further check sweep
    if (rot == 0 || (symmetric && rel_sweeps == 0 && sweep > 0 && rot <= n / 8 && 8 * rot <= prev_rot))
      converged = true;
    prev_rot = rot;
  }
  TNAD_REQUIRE(converged, TNAD_ERR_NOT_CONVERGED, "svd_jacobi: no convergence within the sweep cap");
  k_colnorms<<<(int)((n * 32 + 255) / 256), 256, 0, c->stream>>>(W, Vw, m, n, s, sg);
  k_rank<<<(int)((n + 255) / 256), 256, 0, c->stream>>>(s, n, rank);
  TNAD_CK(cudaMemsetAsync(flag + 1, 0, sizeof(int), c->stream));
  dim3 g((unsigned)std::min<int64_t>((std::max(m, n) + 255) / 256, 16), (unsigned)n);
  k_scatter<<<g, 256, 0, c->stream>>>(W, Vw, s, sg, rank, m, n, symmetric ? 1 : 0, weak_rel, fro2, U, S, V,
                                      flag + 1);
  count_launch(c, 3);
  check_launch(c, "svd_scatter");
  if (!symmetric) {
    TNAD_CK(cudaMemcpyAsync(c->h_flag + 1, flag + 1, sizeof(int), cudaMemcpyDeviceToHost, c->stream));
    TNAD_CK(cudaStreamSynchronize(c->stream));
    int nnull = c->h_flag[1];
    if (nnull > 0) {
      TNAD_REQUIRE(m <= 4096, TNAD_ERR_SHAPE, "svd_jacobi: weak-column completion limited to m <= 4096");
      double* coef = ws_d(c, n);
      for (int64_t k = n - nnull; k < n; ++k) {
        k_complete_col<<<1, 1024, m * sizeof(double), c->stream>>>(U, m, k, coef);
        count_launch(c);
      }
      check_launch(c, "svd_complete");
    }
  }
}

// ---------------------------------------------------------------------------
// Allocation-free variant of the FP64 Jacobi SVD (tnad_svd_noalloc).
//
// Its scratch lives in one file-scope device array of fixed size, sized for
// matrices up to kNoAllocMax × kNoAllocMax.  Every GPU that loads this library
// holds that array (about 1.1 MB) until the process exits.  All calls on a
// device share it, and it keeps the previous call's contents: the entry point
// initialises everything it reads, and calls that overlap on the GPU (two
// streams, or two host threads) race on it.
// ---------------------------------------------------------------------------
static const int kNoAllocMax = 256;
static const int64_t kNoAllocDoubles = 2 * (int64_t)kNoAllocMax * kNoAllocMax  // W, V working copies
                                       + 4 * kNoAllocMax                      // s, sign, coef, rank (as ints)
                                       + 64;                                   // ‖A‖²_F and counters
static __device__ __align__(256) double g_noalloc_scratch[kNoAllocDoubles];

// single-block Σ A² into out[0] (the scratch's ‖A‖²_F slot)
__global__ void k_sumsq_one_block(const double* __restrict__ A, int64_t n, double* __restrict__ out) {
  __shared__ double sh[256];
  double s = 0.0;
  for (int64_t i = threadIdx.x; i < n; i += blockDim.x) s = fma(A[i], A[i], s);
  sh[threadIdx.x] = s;
  __syncthreads();
  for (int k = blockDim.x / 2; k > 0; k >>= 1) {
    if ((int)threadIdx.x < k) sh[threadIdx.x] += sh[threadIdx.x + k];
    __syncthreads();
  }
  if (threadIdx.x == 0) out[0] = sh[0];
}

__global__ void k_copy_eye(const double* __restrict__ A, int64_t mn, double* __restrict__ W, double* __restrict__ V,
                           int64_t n) {
  for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < mn + n * n; e += (int64_t)gridDim.x * blockDim.x) {
    if (e < mn)
      W[e] = A[e];
    else {
      const int64_t f = e - mn;
      V[f] = (f % n == f / n) ? 1.0 : 0.0;
    }
  }
}

}  // namespace tnad

// Scratch address of g_noalloc_scratch per device, resolved once per device
// (with that device current) by cudaGetSymbolAddress: in host code the
// array's name is only a host-side shadow, never a device address.
static double* noalloc_scratch_addr(int dev) {
  static double* addr[64] = {nullptr};
  static std::mutex mu;
  if (dev < 0 || dev >= 64) return nullptr;
  std::lock_guard<std::mutex> lock(mu);
  if (!addr[dev]) {
    void* p = nullptr;
    if (cudaGetSymbolAddress(&p, tnad::g_noalloc_scratch) != cudaSuccess) {
      (void)cudaGetLastError();
      return nullptr;
    }
    addr[dev] = (double*)p;
  }
  return addr[dev];
}

// Thin SVD A = U·diag(S)·Vᵀ (m ≥ n, n ≤ m ≤ 256) by the same one-sided Jacobi
// kernels as tnad_svd, without any device allocation: for callers that cannot
// call cudaMalloc (a host framework that owns all device memory through its own
// allocator, or a latency-critical loop where an allocation would synchronise
// the device).  A, U, S, V are DEVICE pointers (m×n, n, n×n, column-major);
// stream may be 0.  The call waits for its stream once per Jacobi sweep (it
// reads the sweep's rotation count on the host).  The first call on a device
// resolves the scratch address for that device and should therefore happen
// before any stream capture; the cached address is not re-resolved after a
// cudaDeviceReset.  A launch error that earlier, unrelated work left pending
// is cleared on entry, so that only this call's own launches are reported.
// Returns TNAD_ERR_SHAPE for m or n beyond 256 (the static scratch's limit),
// TNAD_ERR_ARG for null pointers or m < n, TNAD_ERR_NOT_CONVERGED /
// TNAD_ERR_CUDA as tnad_svd does.
extern "C" int tnad_svd_noalloc(const double* A, int m, int n, double* U, double* S, double* V, void* stream) {
  using namespace tnad;
  if (!A || !U || !S || !V || n < 1 || m < n) return TNAD_ERR_ARG;
  if (m > kNoAllocMax || n > kNoAllocMax) return TNAD_ERR_SHAPE;
  (void)cudaGetLastError();
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) return TNAD_ERR_CUDA;
  double* base = noalloc_scratch_addr(dev);
  if (!base) return TNAD_ERR_CUDA;
  cudaStream_t st = (cudaStream_t)stream;
  const int64_t mm = kNoAllocMax;
  double* W = base;
  double* Vw = W + mm * mm;
  double* s = Vw + mm * mm;
  double* sg = s + mm;
  double* coef = sg + mm;
  int* rank = (int*)(coef + mm);
  double* fro2 = coef + 2 * mm;
  int* flag = (int*)(fro2 + 8);
  const int64_t mn = (int64_t)m * n;
  k_copy_eye<<<(int)std::min<int64_t>((mn + (int64_t)n * n + 255) / 256, 1024), 256, 0, st>>>(A, mn, W, Vw, n);
  k_sumsq_one_block<<<1, 256, 0, st>>>(A, mn, fro2);
  const int NP = n + (n & 1);
  const double tol = (double)std::max(m, 16) * DBL_EPSILON;
  const double abs_eps = 2.0 * DBL_EPSILON;
  bool converged = (n == 1);
  int hflag = 0;
  for (int sweep = 0; sweep < kMaxSweeps && !converged; ++sweep) {
    if (cudaMemsetAsync(flag, 0, sizeof(int), st) != cudaSuccess) return TNAD_ERR_CUDA;
    const double ae = sweep < kRelSweeps ? 0.0 : abs_eps;
    for (int r = 0; r < NP - 1; ++r)
      k_jacobi_round_cta<2, double><<<(unsigned)(NP / 2), 128, 0, st>>>(W, Vw, m, n, r, NP, tol, ae, fro2, flag);
    if (cudaGetLastError() != cudaSuccess) return TNAD_ERR_CUDA;
    if (cudaMemcpyAsync(&hflag, flag, sizeof(int), cudaMemcpyDeviceToHost, st) != cudaSuccess ||
        cudaStreamSynchronize(st) != cudaSuccess)
      return TNAD_ERR_CUDA;
    if (hflag == 0) converged = true;
  }
  if (!converged) return TNAD_ERR_NOT_CONVERGED;
  k_colnorms<<<(n * 32 + 255) / 256, 256, 0, st>>>(W, Vw, m, n, s, sg);
  k_rank<<<(n + 255) / 256, 256, 0, st>>>(s, n, rank);
  if (cudaMemsetAsync(flag + 1, 0, sizeof(int), st) != cudaSuccess) return TNAD_ERR_CUDA;
  dim3 g(1, (unsigned)n);
  k_scatter<<<g, 256, 0, st>>>(W, Vw, s, sg, rank, m, n, 0, 1e-8, fro2, U, S, V, flag + 1);
  int nweak = 0;
  if (cudaMemcpyAsync(&nweak, flag + 1, sizeof(int), cudaMemcpyDeviceToHost, st) != cudaSuccess ||
      cudaStreamSynchronize(st) != cudaSuccess)
    return TNAD_ERR_CUDA;
  for (int k = n - nweak; k < n; ++k) k_complete_col<<<1, 1024, m * sizeof(double), st>>>(U, m, k, coef);
  if (cudaGetLastError() != cudaSuccess || cudaStreamSynchronize(st) != cudaSuccess) return TNAD_ERR_CUDA;
  return TNAD_OK;
}
