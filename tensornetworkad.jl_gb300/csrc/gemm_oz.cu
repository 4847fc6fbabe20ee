// FP64-accurate GEMM on the tcgen05 tensor cores from error-free BF16 slices
// (the splitting idea of Ozaki et al., "Error-free transformations of matrix
// multiplication by using fast routines of matrix multiplication and its
// applications", Numer. Algorithms 59 (2012), applied to BF16 products with
// FP32 accumulation).
//
// C(M×N) = alpha·op(A)·op(B) + beta·C for FP64 column-major operands:
//
//  1. every row i of op(A) gets a power-of-two scale 2^eA_i ≥ max_k |A_ik| (and
//     every column j of op(B) one, 2^eB_j);
//  2. the scaled entry x = A_ik·2^(55−eA_i) is rounded to an integer Y (|Y| <
//     2^55; the error is below 2^−55 of the row's largest entry) and written in
//     balanced base 256: Y = Σ_s q_s·2^(48−8s), |q_s| ≤ 128, s = 0..5.  Slice
//     plane s holds q_s·2^(−8s), exact in BF16 (8 significant bits);
//  3. with a_s, b_t the slices, A_ik·B_kj ≈ 2^(eA_i+eB_j−14)·Σ_{s,t} a_s·b_t.
//     The pairs with s + t ≤ 6 (26 of 36) are kept; the rest lie below 2^−56 of
//     the scale.  (Level 6 is needed: the balanced low digits are larger than
//     the top digit of a typical entry, and dropping level 6 costs ~2^−45 of
//     |A|·|B| on N(0,1) data.)  Pairs are summed by level L = s + t into six
//     TMEM accumulators: levels 0..4 one each, levels 5 and 6 together.  Within
//     a K chunk of 128 a level-L sum (L ≤ 4) is an integer times 2^(−8L) below
//     2^24 in magnitude, so the FP32 tensor-core accumulation of levels 0..4 is
//     exact whatever its rounding; the tensor cores truncate every product to
//     the accumulator's precision, so an inexact accumulator is only affordable
//     for the levels at 2^−40 and below;
//  4. after each chunk the accumulators are drained to registers: levels 0..4
//     combined exactly into one int64 running sum per element (units of 2^−32),
//     levels 5..6 into an FP32 sum; at the end the two are combined once in FP64
//     and scaled by 2^(eA_i+eB_j−14).
//
// The result is accurate to about 2^−47 of (max_k|A_ik|)·(max_k|B_kj|) per
// product term, measured 6.5e-15 of (|A|·|B|)_ij on N(0,1) data (a DFMA GEMM:
// ~1e-16), on the BF16 tensor pipe instead of GB300's narrow FP64 pipe.
//
// Kernel layout: one 128×64 output tile per CTA, 10 warps.  Warp 8 lane 0 streams
// 32-wide K slices of the six A planes and six B planes with one 3D TMA load
// each (64-byte swizzled rows) into a 3-stage ring; warp 9 allocates TMEM (six
// accumulators × 64 columns) and issues the 26·2 tcgen05.mma kind::f16 per
// slice; warps 0..7 drain each finished chunk (warp w: TMEM lanes
// 32·(w mod 4), columns 32·(w div 4)) and release the accumulators to the next
// chunk before doing their integer arithmetic.  Every wait is bounded (2 s of
// %globaltimer → TNAD_ERR_TIMEOUT through check_tc_errors).  Split-K over CTAs
// writes FP64 partials that a reduction sums in a fixed order.
#include <cuda_bf16.h>

#include <algorithm>
#include <atomic>
#include <cstring>
#include <mutex>

#include "tc_common.cuh"
#include "tnad_internal.h"

namespace tnad {

namespace {

using namespace tc;

constexpr int OZ_S = 6;                          // slices per operand
constexpr int OZ_BM = 128, OZ_BN = 64;           // output tile
constexpr int OZ_KS = 32;                        // K per smem slice (64-byte BF16 rows)
constexpr int OZ_CHUNK = 4;                      // slices per exact accumulation chunk (128 K)
constexpr int OZ_STAGES = 3;
constexpr int OZ_PLANE_A = OZ_BM * 64;           // 8 KiB
constexpr int OZ_PLANE_B = OZ_BN * 64;           // 4 KiB
constexpr int OZ_STAGE = OZ_S * (OZ_PLANE_A + OZ_PLANE_B);  // 72 KiB
constexpr int OZ_SMEM = OZ_STAGES * OZ_STAGE + 1024 + 256;
constexpr int OZ_THREADS = 320;
constexpr int OZ_MAX_SLICES_PER_CTA = 1024;      // 32768 K per CTA: the int64 sum stays below 2^62
constexpr int kExpZero = -(1 << 30);             // row/column of zeros (memset 0x80 is below it)
constexpr int kExpNonFinite = 1 << 29;           // row/column holding Inf or NaN

__device__ __forceinline__ int exp_bound(double x) {
  // smallest E with |x| < 2^E (kExpNonFinite for Inf/NaN, very negative for 0)
  const uint64_t b = (uint64_t)__double_as_longlong(x);
  const int ex = (int)((b >> 52) & 0x7ff);
  const uint64_t mant = b & ((1ull << 52) - 1);
  if (ex == 0x7ff) return kExpNonFinite;
  if (ex == 0) return mant == 0 ? (int)0x80808080 : 64 - __clzll((long long)mant) - 1074;
  return ex - 1022;
}

// e[r] = max over the row r of op(X) of exp_bound (atomicMax per 32×32 tile row)
__global__ void k_oz_exp(const double* __restrict__ X, int64_t ld, int tr, int64_t rows, int64_t K,
                         int* __restrict__ e) {
  __shared__ double tile[32][33];
  const int64_t r0 = (int64_t)blockIdx.y * 32, k0 = (int64_t)blockIdx.x * 32;
  const int tx = threadIdx.x, ty = threadIdx.y;  // 32 × 8
  for (int j = ty; j < 32; j += 8) {
    int64_t r, k;
    if (!tr) { r = r0 + tx; k = k0 + j; } else { k = k0 + tx; r = r0 + j; }
    double v = 0.0;
    if (r < rows && k < K) v = !tr ? X[r + k * ld] : X[k + r * ld];
    if (!tr) tile[tx][j] = v; else tile[j][tx] = v;
  }
  __syncthreads();
  for (int j = ty; j < 32; j += 8) {
    int m = exp_bound(tile[j][tx]);
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) m = max(m, __shfl_xor_sync(0xffffffffu, m, o));
    if (tx == 0 && r0 + j < rows) atomicMax(e + r0 + j, m);
  }
}

// six BF16 slice planes (K-major, rows_pad × k_pad each) of op(X)
__global__ void k_oz_slice(const double* __restrict__ X, int64_t ld, int tr, int64_t rows, int64_t K,
                           int64_t rows_pad, int64_t k_pad, const int* __restrict__ e,
                           __nv_bfloat16* __restrict__ out) {
  __shared__ double tile[32][33];
  const int64_t r0 = (int64_t)blockIdx.y * 32, k0 = (int64_t)blockIdx.x * 32;
  const int tx = threadIdx.x, ty = threadIdx.y;
  for (int j = ty; j < 32; j += 8) {
    int64_t r, k;
    if (!tr) { r = r0 + tx; k = k0 + j; } else { k = k0 + tx; r = r0 + j; }
    double v = 0.0;
    if (r < rows && k < K) v = !tr ? X[r + k * ld] : X[k + r * ld];
    if (!tr) tile[tx][j] = v; else tile[j][tx] = v;
  }
  __syncthreads();
  const int64_t plane = rows_pad * k_pad;
  for (int j = ty; j < 32; j += 8) {
    const int64_t r = r0 + j, k = k0 + tx;
    if (r >= rows_pad || k >= k_pad) continue;
    const int er = r < rows ? e[r] : kExpZero - 1;
    int64_t Y = 0;
    if (er > kExpZero && er < kExpNonFinite) {
      // Y = round(x·2^(55−er)) from the bits of x (integer arithmetic only)
      const uint64_t b = (uint64_t)__double_as_longlong(tile[j][tx]);
      const int ex = (int)((b >> 52) & 0x7ff);
      uint64_t mant = b & ((1ull << 52) - 1);
      int sh;
      if (ex == 0) {
        sh = 1 - 1075 + 55 - er;
      } else {
        mant |= 1ull << 52;
        sh = ex - 1075 + 55 - er;
      }
      uint64_t u;
      if (sh >= 0)
        u = mant << sh;  // sh ≤ 2: |x| < 2^er
      else if (sh > -60)
        u = (mant + (1ull << (-sh - 1))) >> (-sh);
      else
        u = 0;
      Y = (b >> 63) ? -(int64_t)u : (int64_t)u;
    }
#pragma unroll
    for (int s = 0; s < OZ_S; ++s) {
      const int bsh = 48 - 8 * s;
      const int64_t q = (Y + (1ll << (bsh - 1))) >> bsh;  // balanced digit, |q| ≤ 128
      Y -= q << bsh;
      out[s * plane + r * k_pad + k] = __float2bfloat16_rn((float)q * __int_as_float((127 - 8 * s) << 23));
    }
  }
}

__global__ void __launch_bounds__(OZ_THREADS, 1)
    k_gemm_oz(const __grid_constant__ CUtensorMap tA, const __grid_constant__ CUtensorMap tB, int M, int N,
              int kslices_total, int kps, const int* __restrict__ eA, const int* __restrict__ eB, double alpha,
              double beta, double* __restrict__ C, int64_t ldc, double* __restrict__ P, int* err, uint64_t wait_ns) {
  const int kbeg = blockIdx.z * kps;
  const int kblocks = min(kps, kslices_total - kbeg);
  const int nchunks = (kblocks + OZ_CHUNK - 1) / OZ_CHUNK;
  extern __shared__ uint8_t smem_raw[];
  uint8_t* smem = (uint8_t*)(((uintptr_t)smem_raw + 1023) & ~(uintptr_t)1023);
  uint64_t* bars = (uint64_t*)(smem + OZ_STAGES * OZ_STAGE);
  uint32_t* tmem_slot = (uint32_t*)(bars + 2 * OZ_STAGES + 3);
  const uint32_t full0 = su32(bars), empty0 = su32(bars + OZ_STAGES);
  const uint32_t tfull = su32(bars + 2 * OZ_STAGES), tempty = su32(bars + 2 * OZ_STAGES + 1);
  const uint32_t done = su32(bars + 2 * OZ_STAGES + 2);
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int m0 = blockIdx.x * OZ_BM, n0 = blockIdx.y * OZ_BN;

  if (threadIdx.x == 0) {
    for (int s = 0; s < OZ_STAGES; ++s) {
      mbar_init(full0 + 8 * s, 1);
      mbar_init(empty0 + 8 * s, 1);
    }
    mbar_init(tfull, 1);
    mbar_init(tempty, 8);
    mbar_init(done, 1);
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  if (warp == 9) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(su32(tmem_slot)),
                 "r"(512u)
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
  }
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
  const uint32_t tmem = *tmem_slot;

  if (warp == 8) {
    if (lane == 0) {
      // ---------------- TMA producer ----------------
      int issued = 0;
      for (int kb = 0; kb < kblocks; ++kb) {
        const int s = kb % OZ_STAGES;
        const uint32_t ph = (uint32_t)(kb / OZ_STAGES) & 1u;
        if (kb >= OZ_STAGES && !mbar_wait(empty0 + 8 * s, ph ^ 1u, err, 11, wait_ns)) break;
        uint8_t* st = smem + s * OZ_STAGE;
        const uint32_t fb = full0 + 8 * s;
        mbar_expect_tx(fb, (uint32_t)OZ_STAGE);
        const int kx = (kbeg + kb) * OZ_KS;
        tma_load_3d(su32(st), &tA, kx, m0, 0, fb);
        tma_load_3d(su32(st + OZ_S * OZ_PLANE_A), &tB, kx, n0, 0, fb);
        issued = kb + 1;
      }
      for (int kb = (issued > OZ_STAGES ? issued - OZ_STAGES : 0); kb < issued; ++kb)
        mbar_wait(full0 + 8 * (kb % OZ_STAGES), (uint32_t)(kb / OZ_STAGES) & 1u, err, 12, wait_ns);
    }
  } else if (warp == 9) {
    if (lane == 0) {
      // ---------------- MMA issuer ----------------
      // D = F32, A = B = BF16, both K-major, N = 64, M = 128
      const uint32_t idesc = (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(OZ_BN >> 3) << 17) |
                             ((uint32_t)(OZ_BM >> 4) << 24);
      bool ok = true;
      int kb = 0;
      for (int ch = 0; ch < nchunks && ok; ++ch) {
        // the accumulators are free once the drain warps have read chunk ch − 1
        if (ch >= 1 && !mbar_wait(tempty, (uint32_t)(ch - 1) & 1u, err, 13, wait_ns)) {
          ok = false;
          break;
        }
        asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
        bool first[6] = {true, true, true, true, true, true};
        const int kend = min(kblocks, (ch + 1) * OZ_CHUNK);
        for (; kb < kend; ++kb) {
          const int s = kb % OZ_STAGES;
          if (!mbar_wait(full0 + 8 * s, (uint32_t)(kb / OZ_STAGES) & 1u, err, 14, wait_ns)) {
            ok = false;
            break;
          }
          asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
          const uint32_t st = su32(smem + s * OZ_STAGE);
#pragma unroll
          for (int k = 0; k < 2; ++k) {  // two 16-wide K steps per 32-wide slice (32 bytes each)
            // slice pairs (sa, sb) with sa + sb = L ≤ 6 into accumulator min(L, 5)
#pragma unroll
            for (int L = 0; L <= 6; ++L) {
              const int acc = L < 5 ? L : 5;
#pragma unroll
              for (int sa = (L > 5 ? L - 5 : 0); sa <= (L < 5 ? L : 5); ++sa) {
                const int sb = L - sa;
                const uint64_t ad = smem_desc(st + sa * OZ_PLANE_A + k * 32, 512, 4);
                const uint64_t bd = smem_desc(st + OZ_S * OZ_PLANE_A + sb * OZ_PLANE_B + k * 32, 512, 4);
                mma_bf16(tmem + (uint32_t)(acc * 64), ad, bd, idesc, first[acc] ? 0u : 1u);
                first[acc] = false;
              }
            }
          }
          mma_commit(empty0 + 8 * s);  // slot free once these MMAs have read it
        }
        if (ok) mma_commit(tfull);
      }
      mma_commit(done);  // every MMA of this CTA has completed once `done` fires
      mbar_wait(done, 0u, err, 15, wait_ns);
    }
  } else {
    // ---------------- drain warps 0..7 ----------------
    const int q = warp & 3, h = warp >> 2;
    long long Z[32];  // levels 0..4, exact, in units of 2^−32 of the slice scale
    float F5[32];     // levels 5 and 6
#pragma unroll
    for (int j = 0; j < 32; ++j) {
      Z[j] = 0;
      F5[j] = 0.f;
    }
    bool ok = true;
    for (int ch = 0; ch < nchunks && ok; ++ch) {
      if (!mbar_wait(tfull, (uint32_t)ch & 1u, err, 16, wait_ns)) {
        ok = false;
        break;
      }
      asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
      uint32_t v[32];
#pragma unroll
      for (int L = 0; L < 6; ++L) {
        const uint32_t ta = tmem + ((uint32_t)(q * 32) << 16) + (uint32_t)(L * 64 + h * 32);
        asm volatile(
            "tcgen05.ld.sync.aligned.32x32b.x32.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15,"
            "%16,%17,%18,%19,%20,%21,%22,%23,%24,%25,%26,%27,%28,%29,%30,%31}, [%32];"
            : "=r"(v[0]), "=r"(v[1]), "=r"(v[2]), "=r"(v[3]), "=r"(v[4]), "=r"(v[5]), "=r"(v[6]), "=r"(v[7]),
              "=r"(v[8]), "=r"(v[9]), "=r"(v[10]), "=r"(v[11]), "=r"(v[12]), "=r"(v[13]), "=r"(v[14]),
              "=r"(v[15]), "=r"(v[16]), "=r"(v[17]), "=r"(v[18]), "=r"(v[19]), "=r"(v[20]), "=r"(v[21]),
              "=r"(v[22]), "=r"(v[23]), "=r"(v[24]), "=r"(v[25]), "=r"(v[26]), "=r"(v[27]), "=r"(v[28]),
              "=r"(v[29]), "=r"(v[30]), "=r"(v[31])
            : "r"(ta)
            : "memory");
        asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
        if (L == 5) {  // last read of this chunk: hand the accumulators back to the MMA warp
          asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
          __syncwarp();
          if (lane == 0) mbar_arrive(tempty);
        }
#pragma unroll
        for (int j = 0; j < 32; ++j) {
          const float f = __uint_as_float(v[j]);
          // level L ≤ 4 holds an exact integer times 2^(−8L), |·| < 2^24 before scaling
          if (L < 5) Z[j] += (long long)__float2int_rn(f * __int_as_float((127 + 8 * L) << 23)) << (32 - 8 * L);
          else F5[j] += f;
        }
      }
    }
    // ---------------- epilogue ----------------
    const int row = m0 + q * 32 + lane;
    const bool err_set = (*(volatile int*)err) != 0;
    if (ok && !err_set && row < M) {
      const int ea = eA[row];
#pragma unroll
      for (int j = 0; j < 32; ++j) {
        const int col = n0 + h * 32 + j;
        if (col >= N) continue;
        const int eb = eB[col];
        double v;
        if (ea >= kExpNonFinite || eb >= kExpNonFinite)
          v = __longlong_as_double(0x7ff8000000000000ll);  // NaN in, NaN out
        else if (ea <= kExpZero || eb <= kExpZero)
          v = 0.0;
        else
          v = ldexp(ldexp((double)Z[j], -32) + (double)F5[j], ea + eb - 14);
        if (P) {
          P[(int64_t)blockIdx.z * M * N + (int64_t)row + (int64_t)col * M] = v;
        } else {
          double* p = C + (int64_t)row + (int64_t)col * ldc;
          *p = beta == 0.0 ? alpha * v : alpha * v + beta * (*p);
        }
      }
    }
  }
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  if (warp == 9) {
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(512u) : "memory");
  }
}

// C = alpha·Σ_z P[z] + beta·C (fixed order: deterministic)
__global__ void k_oz_reduce(int64_t M, int64_t N, int splits, const double* __restrict__ P, double alpha,
                            double beta, double* __restrict__ C, int64_t ldc) {
  const int64_t MN = M * N;
  for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < MN; e += (int64_t)gridDim.x * blockDim.x) {
    double s = 0.0;
    for (int z = 0; z < splits; ++z) s += P[e + z * MN];
    const int64_t i = e % M, j = e / M;
    C[i + j * ldc] = beta == 0.0 ? alpha * s : alpha * s + beta * C[i + j * ldc];
  }
}

// 3D map over the six slice planes: {k_pad, rows_pad, 6}, box {32, box_rows, 6}
CUtensorMap make_plane_map(void* base, int64_t k_pad, int64_t rows_pad, int box_rows) {
  CUtensorMap m;
  std::memset(&m, 0, sizeof(m));
  EncodeTiledFn fn = tensor_map_encoder();
  TNAD_REQUIRE(fn, TNAD_ERR_CUDA, "cuTensorMapEncodeTiled unavailable");
  cuuint64_t dims[3] = {(cuuint64_t)k_pad, (cuuint64_t)rows_pad, (cuuint64_t)OZ_S};
  cuuint64_t strides[2] = {(cuuint64_t)(k_pad * 2), (cuuint64_t)(rows_pad * k_pad * 2)};
  cuuint32_t box[3] = {(cuuint32_t)OZ_KS, (cuuint32_t)box_rows, (cuuint32_t)OZ_S};
  cuuint32_t es[3] = {1, 1, 1};
  CUresult r = fn(&m, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 3, base, dims, strides, box, es, CU_TENSOR_MAP_INTERLEAVE_NONE,
                  CU_TENSOR_MAP_SWIZZLE_64B, CU_TENSOR_MAP_L2_PROMOTION_L2_256B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
  TNAD_REQUIRE(r == CUDA_SUCCESS, TNAD_ERR_CUDA, "cuTensorMapEncodeTiled (slice planes) failed (" +
                                                     std::to_string((int)r) + ")");
  return m;
}

void oz_prepare(tnad_ctx* c) {
  static std::atomic<bool> done{false};
  static std::mutex mu;
  if (done) return;
  std::lock_guard<std::mutex> lock(mu);
  if (done) return;
  TNAD_CK(cudaFuncSetAttribute(k_gemm_oz, cudaFuncAttributeMaxDynamicSharedMemorySize, OZ_SMEM));
  done = true;
}

}  // namespace

// below this many multiply-adds the DFMA GEMM is as fast (launch-bound)
static const double kOzMinWork = 4.0e6;

void gemm_fp64tc(tnad_ctx* c, char ta, char tb, int64_t M, int64_t N, int64_t K, double alpha, const double* A,
                 int64_t lda, const double* B, int64_t ldb, double beta, double* Cm, int64_t ldc, bool always) {
  if (M <= 0 || N <= 0) return;
  TNAD_REQUIRE(c->tc_ok || !always, TNAD_ERR_STATE, "FP64 tensor-core products need an sm_100-family GPU (tcgen05)");
  if (!c->tc_ok || K <= 0 || (!always && (double)M * (double)N * (double)K < kOzMinWork)) {
    gemm_f64(c, ta, tb, M, N, K, alpha, A, lda, B, ldb, beta, Cm, ldc);
    return;
  }
  TNAD_REQUIRE(M < (1ll << 31) && N < (1ll << 31) && K < (1ll << 31), TNAD_ERR_ARG, "gemm_fp64tc: size");
  oz_prepare(c);
  const int64_t Mp = (M + OZ_BM - 1) / OZ_BM * OZ_BM, Np = (N + OZ_BN - 1) / OZ_BN * OZ_BN;
  const int64_t Kp = (K + OZ_KS - 1) / OZ_KS * OZ_KS;
  WsScope scope(c);
  int* eA = (int*)c->ws.alloc((size_t)Mp * sizeof(int));
  int* eB = (int*)c->ws.alloc((size_t)Np * sizeof(int));
  __nv_bfloat16* pa = (__nv_bfloat16*)c->ws.alloc((size_t)OZ_S * Mp * Kp * 2);
  __nv_bfloat16* pb = (__nv_bfloat16*)c->ws.alloc((size_t)OZ_S * Np * Kp * 2);
  TNAD_CK(cudaMemsetAsync(eA, 0x80, (size_t)Mp * sizeof(int), c->stream));
  TNAD_CK(cudaMemsetAsync(eB, 0x80, (size_t)Np * sizeof(int), c->stream));
  const int ita = (ta == 'T' || ta == 't'), itb = (tb == 'T' || tb == 't');
  // op(B)ᵀ (N rows, K contiguous) is read as B untransposed with tr = !itb
  {
    dim3 g((unsigned)(Kp / 32), (unsigned)((M + 31) / 32)), b(32, 8);
    k_oz_exp<<<g, b, 0, c->stream>>>(A, lda, ita, M, K, eA);
    dim3 g2((unsigned)(Kp / 32), (unsigned)((N + 31) / 32));
    k_oz_exp<<<g2, b, 0, c->stream>>>(B, ldb, itb ? 0 : 1, N, K, eB);
    dim3 g3((unsigned)(Kp / 32), (unsigned)(Mp / 32));
    k_oz_slice<<<g3, b, 0, c->stream>>>(A, lda, ita, M, K, Mp, Kp, eA, pa);
    dim3 g4((unsigned)(Kp / 32), (unsigned)(Np / 32));
    k_oz_slice<<<g4, b, 0, c->stream>>>(B, ldb, itb ? 0 : 1, N, K, Np, Kp, eB, pb);
  }
  count_launch(c, 4);
  check_launch(c, "oz_slice");
  const CUtensorMap tA = make_plane_map(pa, Kp, Mp, OZ_BM);
  const CUtensorMap tB = make_plane_map(pb, Kp, Np, OZ_BN);
  // split K over CTAs: about one wave of the GPU, at least one chunk per split,
  // at most 32768 K values per CTA (int32 running sums)
  const int kst = (int)(Kp / OZ_KS);
  const int64_t tiles = (Mp / OZ_BM) * (Np / OZ_BN);
  int splits = (int)std::max<int64_t>(1, std::min<int64_t>((c->sm_count + tiles - 1) / tiles,
                                                           (kst + OZ_CHUNK - 1) / OZ_CHUNK));
  splits = std::max(splits, (kst + OZ_MAX_SLICES_PER_CTA - 1) / OZ_MAX_SLICES_PER_CTA);
  int kps = (kst + splits - 1) / splits;
  kps = (kps + OZ_CHUNK - 1) / OZ_CHUNK * OZ_CHUNK;
  splits = (kst + kps - 1) / kps;
  double* Pp = splits > 1 ? ws_d(c, (int64_t)splits * M * N) : nullptr;
  KernelTimer kt(c, "gemm_fp64tc", 2.0 * (double)M * (double)N * (double)K);  // logical FP64 flops
  dim3 grid((unsigned)(Mp / OZ_BM), (unsigned)(Np / OZ_BN), (unsigned)splits);
  k_gemm_oz<<<grid, OZ_THREADS, OZ_SMEM, c->stream>>>(tA, tB, (int)M, (int)N, kst, kps, eA, eB, alpha, beta, Cm, ldc,
                                                       Pp, c->d_flag + 8, 2000000000ull);
  count_launch(c);
  check_launch(c, "gemm_fp64tc");
  if (Pp) {
    const int64_t MN = M * N;
    k_oz_reduce<<<(int)std::min<int64_t>((MN + 255) / 256, 4096), 256, 0, c->stream>>>(M, N, splits, Pp, alpha, beta,
                                                                                      Cm, ldc);
    count_launch(c);
    check_launch(c, "oz_reduce");
  }
}

}  // namespace tnad
