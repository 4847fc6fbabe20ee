// FP64 (DFMA) GEMM of the plain path.  Column-major, op(A)/op(B) ∈ {N,T}.
// GB300 issues FP64 at a small fraction of its FP32/tensor rate, so this kernel
// is bound by the DFMA pipe: register-tiled TM×TN micro-tiles over a BM×BN×16
// shared-memory tile, deterministic split-K (fixed-order partial sums) when the
// output has too few tiles to fill the 152 SMs.
#include <algorithm>

#include "tnad_internal.h"

namespace tnad {

template <int BM, int BN, int TM, int TN>
__global__ void __launch_bounds__((BM / TM) * (BN / TN))
    k_gemm_f64(int ta, int tb, int64_t M, int64_t N, int64_t K, int64_t kchunk, double alpha,
               const double* __restrict__ A, int64_t lda, const double* __restrict__ B, int64_t ldb,
               double beta, double* __restrict__ C, int64_t ldc, double* __restrict__ Cpart) {
  constexpr int BK = 16;
  constexpr int NT = (BM / TM) * (BN / TN);
  __shared__ double As[BK][BM + 1];
  __shared__ double Bs[BK][BN + 1];
  const int tid = threadIdx.x;
  const int64_t m0 = (int64_t)blockIdx.x * BM, n0 = (int64_t)blockIdx.y * BN;
  const int64_t kbeg = (int64_t)blockIdx.z * kchunk;
  const int64_t kend = min(K, kbeg + kchunk);
  const int tr = (tid % (BM / TM)) * TM;
  const int tc = (tid / (BM / TM)) * TN;
  double acc[TM][TN];
#pragma unroll
  for (int i = 0; i < TM; ++i)
#pragma unroll
    for (int j = 0; j < TN; ++j) acc[i][j] = 0.0;

  for (int64_t k0 = kbeg; k0 < kend; k0 += BK) {
    // A tile: op(A)(i,k), i in [m0,m0+BM), k in [k0,k0+BK)
    for (int e = tid; e < BM * BK; e += NT) {
      int i, k;
      if (!ta) { i = e % BM; k = e / BM; } else { k = e % BK; i = e / BK; }
      int64_t gi = m0 + i, gk = k0 + k;
      double v = 0.0;
      if (gi < M && gk < kend) v = !ta ? A[gi + gk * lda] : A[gk + gi * lda];
      As[k][i] = v;
    }
    for (int e = tid; e < BN * BK; e += NT) {
      int j, k;
      if (!tb) { k = e % BK; j = e / BK; } else { j = e % BN; k = e / BN; }
      int64_t gj = n0 + j, gk = k0 + k;
      double v = 0.0;
      if (gj < N && gk < kend) v = !tb ? B[gk + gj * ldb] : B[gj + gk * ldb];
      Bs[k][j] = v;
    }
    __syncthreads();
#pragma unroll
    for (int k = 0; k < BK; ++k) {
      double a[TM], b[TN];
#pragma unroll
      for (int i = 0; i < TM; ++i) a[i] = As[k][tr + i];
#pragma unroll
      for (int j = 0; j < TN; ++j) b[j] = Bs[k][tc + j];
#pragma unroll
      for (int i = 0; i < TM; ++i)
#pragma unroll
        for (int j = 0; j < TN; ++j) acc[i][j] = fma(a[i], b[j], acc[i][j]);
    }
    __syncthreads();
  }
  if (Cpart) {
    double* P = Cpart + (int64_t)blockIdx.z * M * N;
#pragma unroll
    for (int i = 0; i < TM; ++i)
#pragma unroll
      for (int j = 0; j < TN; ++j) {
        int64_t gi = m0 + tr + i, gj = n0 + tc + j;
        if (gi < M && gj < N) P[gi + gj * M] = acc[i][j];
      }
  } else {
#pragma unroll
    for (int i = 0; i < TM; ++i)
#pragma unroll
      for (int j = 0; j < TN; ++j) {
        int64_t gi = m0 + tr + i, gj = n0 + tc + j;
        if (gi < M && gj < N) {
          double v = alpha * acc[i][j];
          C[gi + gj * ldc] = beta == 0.0 ? v : v + beta * C[gi + gj * ldc];
        }
      }
  }
}

__global__ void k_splitk_reduce(int64_t M, int64_t N, int ks, const double* __restrict__ P, double alpha,
                                double beta, double* __restrict__ C, int64_t ldc) {
  int64_t MN = M * N;
  for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < MN; e += (int64_t)gridDim.x * blockDim.x) {
    double s = 0.0;
    for (int z = 0; z < ks; ++z) s += P[e + z * MN];
    int64_t i = e % M, j = e / M;
    double v = alpha * s;
    C[i + j * ldc] = beta == 0.0 ? v : v + beta * C[i + j * ldc];
  }
}

// Matrix-vector products (N = 1), the Gram–Schmidt steps of GMRES: a tiled
// GEMM would compute whole 32×32 tiles for one useful column.
// y(M) = alpha·A·x + beta·y with A M×K (lda), x K values (stride incx), K small:
// one thread per row, coalesced over the rows of A.
__global__ void k_gemv_n(int64_t M, int64_t K, double alpha, const double* __restrict__ A, int64_t lda,
                         const double* __restrict__ x, int64_t incx, double beta, double* __restrict__ y) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < M; i += (int64_t)gridDim.x * blockDim.x) {
    double s = 0.0;
    for (int64_t k = 0; k < K; ++k) s = fma(A[i + k * lda], x[k * incx], s);
    const double v = alpha * s;
    y[i] = beta == 0.0 ? v : v + beta * y[i];
  }
}

// part[chunk, i] = Σ_{k in chunk} A[k + i·lda]·x[k] for the M ≤ 32 columns of
// A (K×M, lda): y = Aᵀx split over K chunks, threads strided over k (coalesced),
// a fixed-order block reduction per column.
constexpr int kGemvMaxM = 32;
__global__ void __launch_bounds__(256) k_gemv_t_part(int64_t M, int64_t K, int64_t kchunk,
                                                     const double* __restrict__ A, int64_t lda,
                                                     const double* __restrict__ x, int64_t incx,
                                                     double* __restrict__ part) {
  __shared__ double red[8][kGemvMaxM];
  const int64_t k0 = (int64_t)blockIdx.x * kchunk, k1 = min(K, k0 + kchunk);
  double acc[kGemvMaxM];
#pragma unroll
  for (int i = 0; i < kGemvMaxM; ++i) acc[i] = 0.0;
  for (int64_t k = k0 + threadIdx.x; k < k1; k += blockDim.x) {
    const double xv = x[k * incx];
#pragma unroll
    for (int i = 0; i < kGemvMaxM; ++i)
      if (i < M) acc[i] = fma(A[k + i * lda], xv, acc[i]);
  }
  const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
#pragma unroll
  for (int i = 0; i < kGemvMaxM; ++i) {
    double v = acc[i];
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    if (lane == 0) red[w][i] = v;
  }
  __syncthreads();
  if (threadIdx.x < M) {
    double s = 0.0;
    for (int ww = 0; ww < 8; ++ww) s += red[ww][threadIdx.x];
    part[blockIdx.x * M + threadIdx.x] = s;
  }
}

// y[i] = alpha·Σ_chunk part[chunk, i] + beta·y[i] (fixed order)
__global__ void k_gemv_t_sum(int64_t M, int nchunk, const double* __restrict__ part, double alpha, double beta,
                             double* __restrict__ y) {
  const int64_t i = threadIdx.x;
  if (i >= M) return;
  double s = 0.0;
  for (int z = 0; z < nchunk; ++z) s += part[z * M + i];
  const double v = alpha * s;
  y[i] = beta == 0.0 ? v : v + beta * y[i];
}

void gemm_f64(tnad_ctx* c, char ta, char tb, int64_t M, int64_t N, int64_t K, double alpha, const double* A,
              int64_t lda, const double* B, int64_t ldb, double beta, double* C, int64_t ldc) {
  if (M <= 0 || N <= 0) return;
  if (K <= 0) {
    if (beta == 0.0) {
      for (int64_t j = 0; j < N; ++j) fill(c, C + j * ldc, M, 0.0);
    } else if (beta != 1.0) {
      for (int64_t j = 0; j < N; ++j) scale(c, M, beta, C + j * ldc);
    }
    return;
  }
  int ita = (ta == 'T' || ta == 't'), itb = (tb == 'T' || tb == 't');
  if (N == 1 && (!ita || M <= kGemvMaxM)) {
    // matrix-vector product: x = op(B) is a K-vector with stride ldb when tb = T
    const int64_t incx = itb ? ldb : 1;
    KernelTimer kt(c, "gemm_f64", 2.0 * (double)M * (double)K);
    if (!ita) {
      k_gemv_n<<<(int)std::min<int64_t>((M + 255) / 256, 4096), 256, 0, c->stream>>>(M, K, alpha, A, lda, B, incx,
                                                                                     beta, C);
      count_launch(c);
    } else {
      // K chunks of at least 512 values, at most 2 CTAs per SM: the FP64 pipe
      // of every SM takes part (34 chunks of 2048 at K = 69632 left the
      // product DFMA-bound on 34 SMs)
      const int64_t nch = std::max<int64_t>(1, std::min<int64_t>((K + 511) / 512, 2 * c->sm_count));
      const int64_t kchunk = (K + nch - 1) / nch;
      WsScope scope(c);
      double* part = ws_d(c, nch * M);
      k_gemv_t_part<<<(unsigned)nch, 256, 0, c->stream>>>(M, K, kchunk, A, lda, B, incx, part);
      k_gemv_t_sum<<<1, kGemvMaxM, 0, c->stream>>>(M, (int)nch, part, alpha, beta, C);
      count_launch(c, 2);
    }
    check_launch(c, "gemv_f64");
    return;
  }
  // 64×64 tiles when they alone give half the SMs work, 32×32 otherwise
  const int64_t tiles64 = ((M + 63) / 64) * ((N + 63) / 64);
  const bool big = (M >= 64 && N >= 64 && tiles64 >= c->sm_count / 2);
  const int BM = big ? 64 : 32, BN = big ? 64 : 32;
  int64_t tiles = ((M + BM - 1) / BM) * ((N + BN - 1) / BN);
  // Each SM retires only ~2 DFMA per clock, so a GEMM whose output has fewer
  // tiles than SMs is split along K until about two CTAs per SM are busy
  // (chunks of at least 16 K values; partial sums reduced in fixed order).
  int ks = 1;
  if (tiles < 2 * c->sm_count && K >= 32) {
    int64_t want = (2 * c->sm_count + tiles - 1) / tiles;
    int64_t cap = K / 16;
    ks = (int)std::max<int64_t>(1, std::min<int64_t>({want, cap, 128}));
  }
  int64_t kchunk = (K + ks - 1) / ks;
  kchunk = (kchunk + 15) / 16 * 16;
  ks = (int)((K + kchunk - 1) / kchunk);
  WsScope scope(c);
  double* part = nullptr;
  if (ks > 1) part = ws_d(c, (int64_t)ks * M * N);
  dim3 grid((unsigned)((M + BM - 1) / BM), (unsigned)((N + BN - 1) / BN), (unsigned)ks);
  KernelTimer kt(c, "gemm_f64", 2.0 * (double)M * (double)N * (double)K);
  if (big)
    k_gemm_f64<64, 64, 4, 4><<<grid, 256, 0, c->stream>>>(ita, itb, M, N, K, kchunk, alpha, A, lda, B, ldb, beta, C,
                                                          ldc, part);
  else
    k_gemm_f64<32, 32, 2, 2><<<grid, 256, 0, c->stream>>>(ita, itb, M, N, K, kchunk, alpha, A, lda, B, ldb, beta, C,
                                                          ldc, part);
  count_launch(c);
  check_launch(c, "gemm_f64");
  if (ks > 1) {
    int64_t MN = M * N;
    int nb = (int)std::min<int64_t>((MN + 255) / 256, 4096);
    k_splitk_reduce<<<nb, 256, 0, c->stream>>>(M, N, ks, part, alpha, beta, C, ldc);
    count_launch(c);
    check_launch(c, "splitk_reduce");
  }
}

void gemm(tnad_ctx* c, int prec, char ta, char tb, int64_t M, int64_t N, int64_t K, double alpha, const double* A,
          int64_t lda, const double* B, int64_t ldb, double beta, double* C, int64_t ldc) {
  if (prec == TNAD_PREC_TF32X3) {
    TNAD_REQUIRE(c->tc_ok, TNAD_ERR_STATE, "TF32X3 contractions need an sm_100-family GPU (tcgen05)");
    gemm_tf32x3(c, ta, tb, M, N, K, alpha, A, lda, B, ldb, beta, C, ldc);
  } else if (prec == TNAD_PREC_FP64_TC) {
    gemm_fp64tc(c, ta, tb, M, N, K, alpha, A, lda, B, ldb, beta, C, ldc, true);
  } else if (prec == TNAD_PREC_FP64 && c->fp64_tc) {
    gemm_fp64tc(c, ta, tb, M, N, K, alpha, A, lda, B, ldb, beta, C, ldc);
  } else {
    gemm_f64(c, ta, tb, M, N, K, alpha, A, lda, B, ldb, beta, C, ldc);
  }
}

}  // namespace tnad
