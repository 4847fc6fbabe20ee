// 3xTF32 GEMM on the 5th-generation tensor cores (tcgen05, sm_103a).
//
// C(M×N) = alpha·op(A)·op(B) + beta·C for FP64 column-major operands, computed
// as  A_hi·B_hi + A_hi·B_lo + A_lo·B_hi  with x = x_hi + x_lo split into TF32
// pieces (x_hi = rn_tf32(x), x_lo = rn_tf32(x − x_hi)) and FP32 accumulation in
// TMEM: about FP32 accuracy from the TF32 tensor pipe.
//
//   pack kernel : FP64 (any transpose) → K-major FP32 hi/lo planes, zero padded
//                 to the tile grid (rows padded to 128 / BN, K to 32);
//   GEMM kernel : one 128×BN output tile per CTA, 4 warps.  Warp 0 lane 0
//                 streams 128B-swizzled 32-wide K slices of the four planes with
//                 TMA (cp.async.bulk.tensor) into a 3-stage ring guarded by
//                 mbarriers; warp 1 lane 0 issues 3 tcgen05.mma (kind::tf32) per
//                 8-wide K step into a TMEM accumulator and frees ring slots with
//                 tcgen05.commit; then all four warps drain TMEM (tcgen05.ld
//                 32x32b, warp w owns lanes 32w..32w+31), apply alpha/beta and
//                 store FP64 with coalesced column writes.
// The same kernel, instantiated with SPLIT = false, is the BF16 GEMM of the
// learned warm-start network: FP32 operands packed to one BF16 plane each,
// one tcgen05.mma kind::f16 per 16-wide K step, FP32 accumulation and output.
// Every mbarrier wait is bounded (~2 s of %globaltimer); on timeout the CTA
// records an error, drains its own TMA loads (bounded), frees TMEM and exits,
// and the host reports TNAD_ERR_TIMEOUT.
#include <atomic>
#include <cuda.h>
#include <cuda_bf16.h>

#include <cstring>
#include <mutex>

#include "tc_common.cuh"
#include "tnad_internal.h"

namespace tnad {

namespace {

constexpr int BM = 128, BK = 32, STAGES = 3;  // BK: FP32 elements per 128-byte K slice
constexpr int TILE_A = BM * 128;              // 16 KiB per plane (128 rows × 128 B)

template <int BN, bool SPLIT>
struct Cfg {
  static constexpr int TILE_B = BN * 128;
  static constexpr int PLANES = SPLIT ? 2 : 1;  // hi/lo planes per operand
  static constexpr int STAGE = PLANES * (TILE_A + TILE_B);
  static constexpr int SMEM = STAGES * STAGE + 1024 + 256;
  static constexpr int KSLICE = SPLIT ? 32 : 64;  // elements per 128-byte K slice (TF32 / BF16)
};

using namespace tc;

// UMMA descriptor of a K-major tile with 128-byte swizzled rows (8-row groups 1024 B apart)
__device__ __forceinline__ uint64_t smem_desc(uint32_t addr) { return tc::smem_desc(addr, 1024, 2); }

__device__ __forceinline__ float tf32_rn(float x) {
  uint32_t r;
  asm("cvt.rna.tf32.f32 %0, %1;" : "=r"(r) : "f"(x));
  return __uint_as_float(r);
}

template <int BN, bool SPLIT, typename OutT>
__global__ void __launch_bounds__(128, 1)
    k_gemm_tc(const __grid_constant__ CUtensorMap tAh, const __grid_constant__ CUtensorMap tAl,
              const __grid_constant__ CUtensorMap tBh, const __grid_constant__ CUtensorMap tBl, int M, int N,
              int kblocks_total, int kps, double alpha, double beta, OutT* __restrict__ C, int64_t ldc,
              double* __restrict__ P, int* err, uint64_t wait_ns, int withhold_first) {
  using CF = Cfg<BN, SPLIT>;
  // split-K: CTA z owns K slices [kbeg, kbeg + kblocks); with P != null it
  // writes its raw FP32 sum as an FP64 partial, reduced in FP64 afterwards
  const int kbeg = blockIdx.z * kps;
  const int kblocks = min(kps, kblocks_total - kbeg);
  extern __shared__ uint8_t smem_raw[];
  uint8_t* smem = (uint8_t*)(((uintptr_t)smem_raw + 1023) & ~(uintptr_t)1023);
  uint64_t* bars = (uint64_t*)(smem + STAGES * CF::STAGE);
  uint32_t* tmem_slot = (uint32_t*)(bars + 2 * STAGES + 1);
  const uint32_t full0 = su32(bars), empty0 = su32(bars + STAGES), done = su32(bars + 2 * STAGES);
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int m0 = blockIdx.x * BM, n0 = blockIdx.y * BN;

  if (threadIdx.x == 0) {
    for (int s = 0; s < STAGES; ++s) {
      mbar_init(full0 + 8 * s, 1);
      mbar_init(empty0 + 8 * s, 1);
    }
    mbar_init(done, 1);
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  if (warp == 1) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(su32(tmem_slot)),
                 "r"((uint32_t)BN)
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
  }
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
  const uint32_t tmem = *tmem_slot;

  if (warp == 0 && lane == 0) {
    // ---------------- TMA producer ----------------
    int issued = 0;
    for (int kb = 0; kb < kblocks; ++kb) {
      const int s = kb % STAGES;
      const uint32_t ph = (uint32_t)(kb / STAGES) & 1u;
      if (kb >= STAGES && !mbar_wait(empty0 + 8 * s, ph ^ 1u, err, 1, wait_ns)) break;
      uint8_t* st = smem + s * CF::STAGE;
      const uint32_t fb = full0 + 8 * s;
      mbar_expect_tx(fb, (uint32_t)CF::STAGE);
      const int kx = (kbeg + kb) * CF::KSLICE;
      if (withhold_first && kb == 0) {
        // failure-path test: the slice's bytes are expected but never loaded,
        // so every wait on this stage runs out; no copy is in flight for it
      } else if (SPLIT) {
        tma_load_2d(su32(st), &tAh, kx, m0, fb);
        tma_load_2d(su32(st + TILE_A), &tAl, kx, m0, fb);
        tma_load_2d(su32(st + 2 * TILE_A), &tBh, kx, n0, fb);
        tma_load_2d(su32(st + 2 * TILE_A + CF::TILE_B), &tBl, kx, n0, fb);
      } else {
        tma_load_2d(su32(st), &tAh, kx, m0, fb);
        tma_load_2d(su32(st + TILE_A), &tBh, kx, n0, fb);
      }
      issued = kb + 1;
    }
    // make sure none of this CTA's copies is still in flight when it exits
    for (int kb = (issued > STAGES ? issued - STAGES : 0); kb < issued; ++kb)
      mbar_wait(full0 + 8 * (kb % STAGES), (uint32_t)(kb / STAGES) & 1u, err, 2, wait_ns);
  } else if (warp == 1 && lane == 0) {
    // ---------------- MMA issuer ----------------
    // instruction descriptor: D = F32; A, B = TF32 (kind::tf32) or BF16 (kind::f16); both K-major
    const uint32_t fmt = SPLIT ? 2u : 1u;
    const uint32_t idesc = (1u << 4) | (fmt << 7) | (fmt << 10) | ((uint32_t)(BN >> 3) << 17) |
                           ((uint32_t)(BM >> 4) << 24);
    bool ok = true;
    for (int kb = 0; kb < kblocks && ok; ++kb) {
      const int s = kb % STAGES;
      const uint32_t ph = (uint32_t)(kb / STAGES) & 1u;
      if (!mbar_wait(full0 + 8 * s, ph, err, 3, wait_ns)) {
        ok = false;
        break;
      }
      asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
      const uint32_t st = su32(smem + s * CF::STAGE);
      if (SPLIT) {
        const uint64_t ah = smem_desc(st), al = smem_desc(st + TILE_A);
        const uint64_t bh = smem_desc(st + 2 * TILE_A), bl = smem_desc(st + 2 * TILE_A + CF::TILE_B);
#pragma unroll
        for (int k = 0; k < 4; ++k) {
          const uint64_t off = (uint64_t)((k * 32) >> 4);  // 32 bytes per 8-wide TF32 step
          mma_tf32(tmem, ah + off, bh + off, idesc, (kb > 0 || k > 0) ? 1u : 0u);
          mma_tf32(tmem, ah + off, bl + off, idesc, 1u);
          mma_tf32(tmem, al + off, bh + off, idesc, 1u);
        }
      } else {
        const uint64_t ah = smem_desc(st), bh = smem_desc(st + TILE_A);
#pragma unroll
        for (int k = 0; k < 4; ++k) {
          const uint64_t off = (uint64_t)((k * 32) >> 4);  // 32 bytes per 16-wide BF16 step
          mma_bf16(tmem, ah + off, bh + off, idesc, (kb > 0 || k > 0) ? 1u : 0u);
        }
      }
      mma_commit(empty0 + 8 * s);  // slot free once these MMAs have read it
    }
    mma_commit(done);
  }
  __syncwarp();

  // ---------------- epilogue: TMEM → registers → FP64 global ----------------
  const bool okd = mbar_wait(done, 0u, err, 4, wait_ns);
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
  const int row = m0 + warp * 32 + lane;
  const bool err_set = (*(volatile int*)err) != 0;
#pragma unroll 1
  for (int c0 = 0; c0 < BN; c0 += 16) {
    uint32_t v[16];
    const uint32_t ta = tmem + ((uint32_t)(warp * 32) << 16) + (uint32_t)c0;
    asm volatile(
        "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, [%16];"
        : "=r"(v[0]), "=r"(v[1]), "=r"(v[2]), "=r"(v[3]), "=r"(v[4]), "=r"(v[5]), "=r"(v[6]), "=r"(v[7]),
          "=r"(v[8]), "=r"(v[9]), "=r"(v[10]), "=r"(v[11]), "=r"(v[12]), "=r"(v[13]), "=r"(v[14]), "=r"(v[15])
        : "r"(ta)
        : "memory");
    asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
    if (okd && !err_set && row < M) {
      if (P) {
        double* Pz = P + (int64_t)blockIdx.z * M * N;
#pragma unroll
        for (int j = 0; j < 16; ++j) {
          const int col = n0 + c0 + j;
          if (col < N) Pz[(int64_t)row + (int64_t)col * M] = (double)__uint_as_float(v[j]);
        }
      } else {
#pragma unroll
        for (int j = 0; j < 16; ++j) {
          const int col = n0 + c0 + j;
          if (col < N) {
            double r = alpha * (double)__uint_as_float(v[j]);
            OutT* p = C + (int64_t)row + (int64_t)col * ldc;
            *p = (OutT)(beta == 0.0 ? r : r + beta * (double)(*p));
          }
        }
      }
    }
  }
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  if (warp == 1) {
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"((uint32_t)BN) : "memory");
  }
}

// op(X) (rows × K, from FP64 column-major with leading dim ld, transposed when
// tr) → K-major hi/lo FP32 planes of size rows_pad × k_pad.
__global__ void k_pack_split(const double* __restrict__ X, int64_t ld, int tr, int64_t rows, int64_t K,
                             int64_t rows_pad, int64_t k_pad, float* __restrict__ hi, float* __restrict__ lo) {
  // 32×32 tiles through shared memory: reads coalesced in the source's fast
  // index, writes coalesced along K.
  __shared__ double tile[32][33];
  const int64_t r0 = (int64_t)blockIdx.y * 32, k0 = (int64_t)blockIdx.x * 32;
  const int tx = threadIdx.x, ty = threadIdx.y;  // 32 × 8
  for (int j = ty; j < 32; j += 8) {
    // tile[rr][kk] = op(X)(r0+rr, k0+kk)
    int64_t r, k;
    if (!tr) { r = r0 + tx; k = k0 + j; } else { k = k0 + tx; r = r0 + j; }
    double v = 0.0;
    if (r < rows && k < K) v = !tr ? X[r + k * ld] : X[k + r * ld];
    if (!tr) tile[tx][j] = v; else tile[j][tx] = v;
  }
  __syncthreads();
  for (int j = ty; j < 32; j += 8) {
    const int64_t r = r0 + j, k = k0 + tx;
    if (r < rows_pad && k < k_pad) {
      const double x = tile[j][tx];
      const float h = tf32_rn((float)x);
      const float l = tf32_rn((float)(x - (double)h));
      hi[r * k_pad + k] = h;
      lo[r * k_pad + k] = l;
    }
  }
}

// op(X) (rows × K, FP32 column-major) → one K-major BF16 plane, zero padded
__global__ void k_pack_bf16(const float* __restrict__ X, int64_t ld, int tr, int64_t rows, int64_t K,
                            int64_t rows_pad, int64_t k_pad, __nv_bfloat16* __restrict__ out) {
  __shared__ float tile[32][33];
  const int64_t r0 = (int64_t)blockIdx.y * 32, k0 = (int64_t)blockIdx.x * 32;
  const int tx = threadIdx.x, ty = threadIdx.y;  // 32 × 8
  for (int j = ty; j < 32; j += 8) {
    int64_t r, k;
    if (!tr) { r = r0 + tx; k = k0 + j; } else { k = k0 + tx; r = r0 + j; }
    float v = 0.f;
    if (r < rows && k < K) v = !tr ? X[r + k * ld] : X[k + r * ld];
    if (!tr) tile[tx][j] = v; else tile[j][tx] = v;
  }
  __syncthreads();
  for (int j = ty; j < 32; j += 8) {
    const int64_t r = r0 + j, k = k0 + tx;
    if (r < rows_pad && k < k_pad) out[r * k_pad + k] = __float2bfloat16_rn(tile[j][tx]);
  }
}

constexpr int kChunkBlocks = 4;  // 4 × 32 = 128 K values per FP32 tensor-core accumulation

// C = alpha·Σ_z P[z] + beta·C   (fixed order: deterministic)
template <typename OutT>
__global__ void k_splitk_sum(int64_t M, int64_t N, int splits, const double* __restrict__ P, double alpha,
                             double beta, OutT* __restrict__ C, int64_t ldc) {
  const int64_t MN = M * N;
  for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < MN; e += (int64_t)gridDim.x * blockDim.x) {
    double s = 0.0;
    for (int z = 0; z < splits; ++z) s += P[e + z * MN];
    const int64_t i = e % M, j = e / M;
    const double r = alpha * s;
    C[i + j * ldc] = (OutT)(beta == 0.0 ? r : r + beta * (double)C[i + j * ldc]);
  }
}

EncodeTiledFn encode_fn() { return tensor_map_encoder(); }

CUtensorMap make_map(void* base, int64_t k_pad, int64_t rows_pad, int box_rows, bool bf16) {
  CUtensorMap m;
  std::memset(&m, 0, sizeof(m));
  EncodeTiledFn fn = encode_fn();
  TNAD_REQUIRE(fn, TNAD_ERR_CUDA, "cuTensorMapEncodeTiled unavailable");
  cuuint64_t dims[2] = {(cuuint64_t)k_pad, (cuuint64_t)rows_pad};
  const int esz = bf16 ? 2 : 4;
  cuuint64_t strides[1] = {(cuuint64_t)(k_pad * esz)};
  cuuint32_t box[2] = {(cuuint32_t)(128 / esz), (cuuint32_t)box_rows};  // one 128-byte K slice
  cuuint32_t es[2] = {1, 1};
  CUresult r = fn(&m, bf16 ? CU_TENSOR_MAP_DATA_TYPE_BFLOAT16 : CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 2, base, dims,
                  strides, box, es,
                  CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_128B, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
                  CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
  TNAD_REQUIRE(r == CUDA_SUCCESS, TNAD_ERR_CUDA, "cuTensorMapEncodeTiled failed (" + std::to_string((int)r) + ")");
  return m;
}

template <int BN, bool SPLIT, typename OutT>
void launch_tc(tnad_ctx* c, int64_t M, int64_t N, int64_t K, double alpha, void* Ah, void* Al, void* Bh, void* Bl,
               int64_t Mp, int64_t Np, int64_t Kp, double beta, OutT* Cm, int64_t ldc, const char* timer_name) {
  using CF = Cfg<BN, SPLIT>;
  static std::atomic<bool> attr{false};
  if (!attr) {
    TNAD_CK(cudaFuncSetAttribute(k_gemm_tc<BN, SPLIT, OutT>, cudaFuncAttributeMaxDynamicSharedMemorySize, CF::SMEM));
    attr = true;
  }
  CUtensorMap tAh = make_map(Ah, Kp, Mp, BM, !SPLIT);
  CUtensorMap tBh = make_map(Bh, Kp, Np, BN, !SPLIT);
  CUtensorMap tAl = SPLIT ? make_map(Al, Kp, Mp, BM, false) : tAh;
  CUtensorMap tBl = SPLIT ? make_map(Bl, Kp, Np, BN, false) : tBh;
  // K is cut into chunks of ≤ kChunkBlocks slices; the tensor cores accumulate
  // each chunk in FP32 (error growing with the chunk length) and the chunks are
  // summed in FP64.  Chunks also multiply the CTA count of these short-K GEMMs.
  const int kbt = (int)(Kp / CF::KSLICE);
  const int chunk = SPLIT ? kChunkBlocks : 2 * kChunkBlocks;
  const int splits = (kbt + chunk - 1) / chunk;
  const int kps = (kbt + splits - 1) / splits;
  dim3 grid((unsigned)(Mp / BM), (unsigned)(Np / BN), (unsigned)splits);
  int* err = c->d_flag + 8;
  WsScope scope(c);
  double* P = splits > 1 ? ws_d(c, (int64_t)splits * M * N) : nullptr;
  int withhold = 0;
  uint64_t wait_ns = 2000000000ull;
  if (c->fault_once == kFaultTcWithhold) {
    withhold = 1;
    wait_ns = 20000000ull;
    c->fault_once = kFaultNone;
  }
  KernelTimer kt(c, timer_name, 2.0 * (double)M * (double)N * (double)K);  // logical flops
  k_gemm_tc<BN, SPLIT, OutT><<<grid, 128, CF::SMEM, c->stream>>>(tAh, tAl, tBh, tBl, (int)M, (int)N, kbt, kps, alpha,
                                                                 beta, Cm, ldc, P, err, wait_ns, withhold);
  count_launch(c);
  check_launch(c, timer_name);
  if (P) {
    const int64_t MN = M * N;
    k_splitk_sum<OutT><<<(int)std::min<int64_t>((MN + 255) / 256, 4096), 256, 0, c->stream>>>(M, N, splits, P,
                                                                                            alpha, beta, Cm, ldc);
    count_launch(c);
    check_launch(c, "splitk_sum");
  }
}

}  // namespace

// below this many multiply-adds the FP64 DFMA tile is as fast and more accurate
static const double kTcMinWork = 4.0e6;

void gemm_tf32x3(tnad_ctx* c, char ta, char tb, int64_t M, int64_t N, int64_t K, double alpha, const double* A,
                 int64_t lda, const double* B, int64_t ldb, double beta, double* Cm, int64_t ldc) {
  if (M <= 0 || N <= 0) return;
  if (K <= 0 || (double)M * (double)N * (double)K < kTcMinWork || M < 64 || N < 16) {
    gemm_f64(c, ta, tb, M, N, K, alpha, A, lda, B, ldb, beta, Cm, ldc);
    return;
  }
  TNAD_REQUIRE(M < (1ll << 31) && N < (1ll << 31) && K < (1ll << 31), TNAD_ERR_ARG, "gemm_tf32x3: size");
  const int BN = N > 64 ? 128 : 64;
  const int64_t Mp = (M + BM - 1) / BM * BM, Np = (N + BN - 1) / BN * BN, Kp = (K + BK - 1) / BK * BK;
  WsScope scope(c);
  float* Ah = ws_f(c, Mp * Kp);
  float* Al = ws_f(c, Mp * Kp);
  float* Bh = ws_f(c, Np * Kp);
  float* Bl = ws_f(c, Np * Kp);
  const int ita = (ta == 'T' || ta == 't'), itb = (tb == 'T' || tb == 't');
  {
    dim3 g((unsigned)(Kp / 32), (unsigned)(Mp / 32)), b(32, 8);
    k_pack_split<<<g, b, 0, c->stream>>>(A, lda, ita, M, K, Mp, Kp, Ah, Al);
  }
  {
    // op(B) is K×N; the packed operand is op(B)ᵀ (N rows, K contiguous): rows of
    // op(B)ᵀ are columns of op(B), i.e. (B, not transposed) read with tr = !itb.
    dim3 g((unsigned)(Kp / 32), (unsigned)(Np / 32)), b(32, 8);
    k_pack_split<<<g, b, 0, c->stream>>>(B, ldb, itb ? 0 : 1, N, K, Np, Kp, Bh, Bl);
  }
  count_launch(c, 2);
  check_launch(c, "pack_split");
  if (BN == 128)
    launch_tc<128, true, double>(c, M, N, K, alpha, Ah, Al, Bh, Bl, Mp, Np, Kp, beta, Cm, ldc, "gemm_tf32x3");
  else
    launch_tc<64, true, double>(c, M, N, K, alpha, Ah, Al, Bh, Bl, Mp, Np, Kp, beta, Cm, ldc, "gemm_tf32x3");
}

void gemm_bf16(tnad_ctx* c, char ta, char tb, int64_t M, int64_t N, int64_t K, float alpha, const float* A,
               int64_t lda, const float* B, int64_t ldb, float beta, float* Cm, int64_t ldc) {
  if (M <= 0 || N <= 0) return;
  TNAD_REQUIRE(c->tc_ok, TNAD_ERR_STATE, "BF16 GEMM needs an sm_100-family GPU (tcgen05)");
  TNAD_REQUIRE(K > 0 && M < (1ll << 31) && N < (1ll << 31) && K < (1ll << 31), TNAD_ERR_ARG, "gemm_bf16: size");
  const int BN = N > 64 ? 128 : 64;
  const int64_t Mp = (M + BM - 1) / BM * BM, Np = (N + BN - 1) / BN * BN, Kp = (K + 63) / 64 * 64;
  WsScope scope(c);
  __nv_bfloat16* Ab = (__nv_bfloat16*)c->ws.alloc((size_t)Mp * Kp * 2);
  __nv_bfloat16* Bb = (__nv_bfloat16*)c->ws.alloc((size_t)Np * Kp * 2);
  const int ita = (ta == 'T' || ta == 't'), itb = (tb == 'T' || tb == 't');
  {
    dim3 g((unsigned)(Kp / 32), (unsigned)(Mp / 32)), b(32, 8);
    k_pack_bf16<<<g, b, 0, c->stream>>>(A, lda, ita, M, K, Mp, Kp, Ab);
  }
  {
    dim3 g((unsigned)(Kp / 32), (unsigned)(Np / 32)), b(32, 8);
    k_pack_bf16<<<g, b, 0, c->stream>>>(B, ldb, itb ? 0 : 1, N, K, Np, Kp, Bb);
  }
  count_launch(c, 2);
  check_launch(c, "pack_bf16");
  if (BN == 128)
    launch_tc<128, false, float>(c, M, N, K, alpha, Ab, nullptr, Bb, nullptr, Mp, Np, Kp, beta, Cm, ldc, "gemm_bf16");
  else
    launch_tc<64, false, float>(c, M, N, K, alpha, Ab, nullptr, Bb, nullptr, Mp, Np, Kp, beta, Cm, ldc, "gemm_bf16");
}

EncodeTiledFn tensor_map_encoder() {
  static EncodeTiledFn fn = nullptr;
  static std::once_flag once;
  std::call_once(once, [] {
    void* p = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPoint("cuTensorMapEncodeTiled", &p, cudaEnableDefault, &q) == cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      fn = (EncodeTiledFn)p;
  });
  return fn;
}

// Host check of the bounded-wait error flag (TNAD_ERR_TIMEOUT when a tensor-core
// GEMM gave up on one of its barriers).
void check_tc_errors(tnad_ctx* c) {
  int h = 0;
  TNAD_CK(cudaMemcpyAsync(&h, c->d_flag + 8, sizeof(int), cudaMemcpyDeviceToHost, c->stream));
  TNAD_CK(cudaStreamSynchronize(c->stream));
  if (h != 0) {
    TNAD_CK(cudaMemsetAsync(c->d_flag + 8, 0, sizeof(int), c->stream));
    fail(TNAD_ERR_TIMEOUT, "tcgen05 GEMM: bounded mbarrier wait expired (stage " + std::to_string(h) + ")");
  }
}

}  // namespace tnad
