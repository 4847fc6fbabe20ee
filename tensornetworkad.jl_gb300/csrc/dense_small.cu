// Small dense kernels of the subspace eigensolver, each in one CTA:
//  - Cholesky of a p×p Gram matrix and the inverse of its triangular factor
//    (CholeskyQR of the n×p block: Q = Y·R⁻¹);
//  - cyclic parallel Jacobi eigendecomposition of a symmetric p×p matrix held
//    in shared memory (circle-method rounds of p/2 disjoint rotations), in
//    FP32 while the contractions run at 3xTF32 accuracy and in FP64 for the
//    polishing steps; eigenvectors accumulate in global memory;
//  - a counter-based Gaussian generator for deterministic start blocks.
#include <cfloat>
#include <atomic>
#include <cmath>

#include "tnad_internal.h"

namespace tnad {

// ---------------------------------------------------------------- Cholesky
// G (p×p, column-major, symmetric positive semi-definite) → R (p×p, upper
// triangular, zeros below) with G + E = RᵀR and E ≥ 0 diagonal: a pivot below
// kPivotFloor·max_k G_kk (a column numerically inside the span of the previous
// ones, e.g. when the subspace is wider than the rank of the matrix it
// iterates on) is raised to that floor, so the factor stays finite and the
// column maps to a vector of norm ≲ 1.  *fail = 1 when G has no positive
// finite diagonal.  One CTA, right-looking, the matrix in shared memory.
constexpr double kPivotFloor = 1e-14;

template <typename T>
__global__ void __launch_bounds__(512) k_chol_factor(const double* __restrict__ G, int p, double floor_rel,
                                                     double* __restrict__ Rg, int* __restrict__ fail) {
  extern __shared__ unsigned char sm_raw[];
  T* A = reinterpret_cast<T*>(sm_raw);  // working copy of G (upper triangle), p × ld
  const int ld = p + 1;                 // padded leading dimension
  __shared__ T piv[2];                  // 1/d_k, sqrt(d_k) of the current step
  __shared__ int bad;
  __shared__ T floor_;
  for (int e = threadIdx.x; e < p * p; e += blockDim.x) A[(e % p) + (e / p) * ld] = (T)G[e];
  __syncthreads();
  if (threadIdx.x == 0) {
    T mx = 0;
    for (int k = 0; k < p; ++k) mx = fmax(mx, A[k + k * ld]);
    bad = (mx > (T)0 && isfinite(mx)) ? 0 : 1;
    floor_ = bad ? (T)1e-30 : (T)floor_rel * mx;
  }
  const int w = threadIdx.x >> 5, lane = threadIdx.x & 31, nw = blockDim.x >> 5;
  // zeros below the diagonal of the output factor
  for (int j = w; j < p; j += nw)
    for (int i = j + 1 + lane; i < p; i += 32) Rg[i + (int64_t)j * p] = 0.0;
  __syncthreads();
  // right-looking, one barrier pair per pivot; warp w owns columns j ≡ w (mod nw)
  // and its lanes the rows of each column:  R[k, j] = A[k, j]/√d_k and
  // A[i, j] −= A[k, i]·A[k, j]/d_k for k < i ≤ j
  for (int k = 0; k < p; ++k) {
    if (threadIdx.x == 0) {
      T d = A[k + k * ld];
      if (!(d > floor_)) d = floor_;
      piv[0] = (T)1 / d;
      piv[1] = sqrt(d);
    }
    __syncthreads();
    const T inv_d = piv[0], rkk = piv[1], inv_r = inv_d * rkk;  // 1/√d
    for (int j = k + ((w - k) % nw + nw) % nw; j < p; j += nw) {
      const T akj = A[k + j * ld];
      if (lane == 0) Rg[k + (int64_t)j * p] = (double)(j == k ? rkk : akj * inv_r);
      if (j == k) continue;
      const T f = akj * inv_d;
      for (int i = k + 1 + lane; i <= j; i += 32) A[i + j * ld] -= A[k + i * ld] * f;
    }
    __syncthreads();
  }
  if (threadIdx.x == 0 && bad) *fail = 1;
}

// Rinv = R⁻¹ for upper-triangular R (p×p): one warp per column j solves
// R·x = e_j by back substitution (lanes split each row's dot product), R in
// shared memory with leading dimension p+1; 8 columns per CTA.
template <typename T>
__global__ void k_tri_inv(const double* __restrict__ Rg, int p, double* __restrict__ Rinv) {
  extern __shared__ unsigned char sm_raw[];
  T* R = reinterpret_cast<T*>(sm_raw);  // p × ld
  const int ld = p + 1;
  T* rd = R + p * ld;  // 1/R[i,i]
  T* X = rd + p;       // 8 × p solution columns
  for (int e = threadIdx.x; e < p * p; e += blockDim.x) {
    const int i = e % p, j = e / p;
    R[i + j * ld] = (T)Rg[e];
  }
  for (int i = threadIdx.x; i < p; i += blockDim.x) rd[i] = (T)1 / (T)Rg[i + (int64_t)i * p];
  __syncthreads();
  const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int j = blockIdx.x * 8 + w;
  if (j >= p) return;
  T* x = X + w * p;
  for (int i = j; i >= 0; --i) {
    T s = 0;
    for (int l = i + 1 + lane; l <= j; l += 32) s += R[i + l * ld] * x[l];
    for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
    if (lane == 0) x[i] = ((i == j ? (T)1 : (T)0) - s) * rd[i];
    __syncwarp();
  }
  for (int i = lane; i < p; i += 32) Rinv[i + (int64_t)j * p] = i <= j ? (double)x[i] : 0.0;
}

template <typename T>
void chol_inv_t(tnad_ctx* c, const double* G, int64_t p, double floor_rel, double* Rinv, int* dev_fail) {
  static std::atomic<bool> attr{false};
  const size_t es = sizeof(T);
  if (!attr) {
    TNAD_CK(cudaFuncSetAttribute(k_chol_factor<T>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)(160 * 161 * es)));
    TNAD_CK(cudaFuncSetAttribute(k_tri_inv<T>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                 (int)((160 * 161 + 9 * 160) * es)));
    attr = true;
  }
  WsScope scope(c);
  double* R = ws_d(c, p * p);
  KernelTimer kt(c, "chol", (double)p * p * p / 3.0);
  k_chol_factor<T><<<1, 512, (size_t)p * (p + 1) * es, c->stream>>>(G, (int)p, floor_rel, R, dev_fail);
  k_tri_inv<T><<<(unsigned)((p + 7) / 8), 256, (size_t)(p * (p + 1) + 9 * p) * es, c->stream>>>(R, (int)p, Rinv);
  count_launch(c, 2);
  check_launch(c, "chol_inv");
}

void chol_inv_upper(tnad_ctx* c, const double* G, int64_t p, double* Rinv, int* dev_fail) {
  TNAD_REQUIRE(p >= 1 && p <= 160, TNAD_ERR_SHAPE, "chol_inv_upper: p must be in [1,160]");
  chol_inv_t<double>(c, G, p, kPivotFloor, Rinv, dev_fail);
}

// FP32 factorisation (relative pivot floor 1e-7) for Gram matrices that are
// already close to I: the second CholeskyQR pass while the contractions run
// at TF32X3 accuracy.
void chol_inv_upper_f32(tnad_ctx* c, const double* G, int64_t p, double* Rinv, int* dev_fail) {
  TNAD_REQUIRE(p >= 1 && p <= 160, TNAD_ERR_SHAPE, "chol_inv_upper_f32: p must be in [1,160]");
  chol_inv_t<float>(c, G, p, 1e-7, Rinv, dev_fail);
}

// ---------------------------------------------------------------- Jacobi eigh
__device__ __forceinline__ void circle_pair(int r, int k, int NP, int* p, int* q) {
  if (k == 0) {
    *p = NP - 1;
    *q = r;
  } else {
    *p = (r + k) % (NP - 1);
    *q = (r - k + (NP - 1)) % (NP - 1);
  }
}

// A (p×p symmetric, FP64 in global) → lam (p, sorted by |λ| descending, or by λ
// descending when by_value), W (p×p eigenvectors as columns, same order).
// Z: p×p scratch for the unsorted vectors.  Sweeps until no rotation is needed
// (or max_sweeps; the sweep count goes to info[0]).
template <typename T>
__global__ void k_eigh_jacobi(const double* __restrict__ A, int p, int max_sweeps, double* __restrict__ lam,
                              double* __restrict__ W, T* __restrict__ Z, int* __restrict__ info, int by_value) {
  extern __shared__ unsigned char smraw[];
  T* H = reinterpret_cast<T*>(smraw);  // p×p, leading dimension ld = p+1 (bank-conflict free)
  const int ld = p + 1;
  __shared__ T cs_[128], sn_[128];
  __shared__ int pp_[128], qq_[128];
  __shared__ int rotated;
  __shared__ double fro_part[32];
  const int NP = p + (p & 1);
  const double eps_t = sizeof(T) == 8 ? DBL_EPSILON : FLT_EPSILON;
  const T tol = (T)(4.0 * eps_t * sqrt((double)p));
  double ss = 0.0;
  for (int e = threadIdx.x; e < p * p; e += blockDim.x) {
    const double v = A[e];
    ss += v * v;
    H[(e % p) + (e / p) * ld] = (T)v;
    Z[e] = (e % p == e / p) ? (T)1 : (T)0;
  }
  for (int o = 16; o > 0; o >>= 1) ss += __shfl_xor_sync(0xffffffffu, ss, o);
  if ((threadIdx.x & 31) == 0) fro_part[threadIdx.x >> 5] = ss;
  __syncthreads();
  // Rounding floor of the stop rule: every rotation leaves noise of size
  // ~ε·‖H‖ in the off-diagonal entries of small eigenvalues, which a purely
  // relative rule would keep rotating until the sweep cap.
  double fro2 = 0.0;
  for (int w = 0; w < (int)(blockDim.x >> 5); ++w) fro2 += fro_part[w];
  const T absfl = (T)(2.0 * eps_t * sqrt((double)p) * sqrt(fro2));
  int sweep = 0;
  for (; sweep < max_sweeps; ++sweep) {
    if (threadIdx.x == 0) rotated = 0;
    __syncthreads();
    for (int r = 0; r < NP - 1; ++r) {
      // rotation parameters for the NP/2 disjoint pairs of this round
      for (int k = threadIdx.x; k < NP / 2; k += blockDim.x) {
        int a, b;
        circle_pair(r, k, NP, &a, &b);
        T c = 1, s = 0;
        if (a < p && b < p) {
          if (a > b) {
            int t = a;
            a = b;
            b = t;
          }
          const T apq = H[a + b * ld], app = H[a + a * ld], aqq = H[b + b * ld];
          // stop rule in the kernel's own precision (an FP64 test in the FP32
          // kernel would run on GB300's narrow FP64 pipe)
          if (apq != (T)0 && fabs(apq) > tol * sqrt(fabs(app)) * sqrt(fabs(aqq)) && fabs(apq) > absfl) {
            const T tau = (aqq - app) / ((T)2 * apq);
            const T t = (tau >= (T)0 ? (T)1 : (T)-1) / (fabs(tau) + sqrt((T)1 + tau * tau));
            c = (T)1 / sqrt((T)1 + t * t);
            s = t * c;
            rotated = 1;
          }
        } else {
          a = b = -1;
        }
        pp_[k] = a;
        qq_[k] = b;
        cs_[k] = c;
        sn_[k] = s;
      }
      __syncthreads();
      // warp w takes pairs k ≡ w (mod warps), its lanes the matrix index (no
      // integer division in the inner loops)
      const int wid = threadIdx.x >> 5, lane = threadIdx.x & 31, nwarp = blockDim.x >> 5;
      // rows: (row a, row b) ← (c·row a − s·row b, s·row a + c·row b)
      for (int k = wid; k < NP / 2; k += nwarp) {
        const int a = pp_[k], b = qq_[k];
        if (a < 0 || sn_[k] == (T)0) continue;
        const T c = cs_[k], s = sn_[k];
        for (int col = lane; col < p; col += 32) {
          const T x = H[a + col * ld], y = H[b + col * ld];
          H[a + col * ld] = c * x - s * y;
          H[b + col * ld] = s * x + c * y;
        }
      }
      __syncthreads();
      // columns of H and of Z; then the rotated pair's off-diagonal entry is 0
      for (int k = wid; k < NP / 2; k += nwarp) {
        const int a = pp_[k], b = qq_[k];
        if (a < 0 || sn_[k] == (T)0) continue;
        const T c = cs_[k], s = sn_[k];
        for (int row = lane; row < p; row += 32) {
          const T x = H[row + a * ld], y = H[row + b * ld];
          H[row + a * ld] = c * x - s * y;
          H[row + b * ld] = s * x + c * y;
          const T zx = Z[row + a * p], zy = Z[row + b * p];
          Z[row + a * p] = c * zx - s * zy;
          Z[row + b * p] = s * zx + c * zy;
        }
        __syncwarp();
        if (lane == 0) {
          H[a + b * ld] = (T)0;
          H[b + a * ld] = (T)0;
        }
      }
      __syncthreads();
    }
    const int done = (rotated == 0);
    __syncthreads();
    if (done) break;
  }
  // sort by key descending (ties by index): rank_j = #{i: k_i > k_j or (= and i<j)},
  // key |λ|, or λ itself when by_value
  for (int j = threadIdx.x; j < p; j += blockDim.x) {
    const double lj = (double)H[j + j * ld];
    const double kj = by_value ? lj : fabs(lj);
    int rk = 0;
    for (int i = 0; i < p; ++i) {
      const double li = (double)H[i + i * ld];
      const double ki = by_value ? li : fabs(li);
      rk += (ki > kj || (ki == kj && i < j)) ? 1 : 0;
    }
    lam[rk] = lj;
    for (int i = 0; i < p; ++i) W[i + (int64_t)rk * p] = (double)Z[i + (int64_t)j * p];
  }
  if (threadIdx.x == 0 && info) info[0] = sweep;
}

void eigh_small_prec(tnad_ctx* c, bool fp32, const double* A, int64_t p, double* W, double* lam, int max_sweeps,
                     int* dev_info, bool by_value) {
  TNAD_REQUIRE(p >= 1 && p <= 256, TNAD_ERR_SHAPE, "eigh_small: p must be in [1,256]");
  WsScope scope(c);
  const size_t sm = (size_t)(p + 1) * p * (fp32 ? 4 : 8);
  const size_t kMaxSm = 200 * 1024;
  TNAD_REQUIRE(sm <= kMaxSm, TNAD_ERR_SHAPE, "eigh_small: matrix does not fit in shared memory");
  static std::atomic<bool> attr32{false}, attr64{false};
  // eigenvectors accumulate in global memory (L1-cached); H lives in shared memory
  KernelTimer kt(c, fp32 ? "eigh_f32" : "eigh_f64", 0.0);
  if (fp32) {
    if (!attr32) {
      TNAD_CK(cudaFuncSetAttribute(k_eigh_jacobi<float>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kMaxSm));
      attr32 = true;
    }
    float* Z = ws_f(c, p * p);
    k_eigh_jacobi<float><<<1, 512, sm, c->stream>>>(A, (int)p, max_sweeps, lam, W, Z, dev_info, by_value ? 1 : 0);
  } else {
    if (!attr64) {
      TNAD_CK(cudaFuncSetAttribute(k_eigh_jacobi<double>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kMaxSm));
      attr64 = true;
    }
    double* Z = ws_d(c, p * p);
    k_eigh_jacobi<double><<<1, 512, sm, c->stream>>>(A, (int)p, max_sweeps, lam, W, Z, dev_info, by_value ? 1 : 0);
  }
  count_launch(c);
  check_launch(c, "eigh_small");
}

void eigh_small(tnad_ctx* c, const double* A, int64_t p, double* W, double* lam) {
  eigh_small_prec(c, false, A, p, W, lam, 40, nullptr);
}

// ---------------------------------------------------------------- polar factor
// O = polar(X) for a χ×χ X (χ ≤ 128) by Newton–Schulz, O ← O·(3I − OᵀO)/2,
// in FP32 in one CTA (the caller polishes in FP64); larger χ take polar_ns_gemm.  info[0] = 1 when the
// result is orthogonal to 1e-4 (else the caller falls back to sign alignment).
__global__ void k_polar_ns(const double* __restrict__ X, int m, int iters, double* __restrict__ O,
                           int* __restrict__ info) {
  extern __shared__ float psm[];
  const int ld = m + 1;         // padded leading dimension (bank-conflict free)
  float* A = psm;               // m×m current iterate
  float* G = psm + m * ld;      // AᵀA
  float* B = psm + 2 * m * ld;  // next iterate
  __shared__ float red[32];
  __shared__ int done;
  const int mm = m * m;
  // scale by 1/‖X‖_F·√m so that all singular values are ≤ 1 < √3
  float s = 0.f;
  for (int e = threadIdx.x; e < mm; e += blockDim.x) s += (float)(X[e] * X[e]);
  for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = s;
  __syncthreads();
  if (threadIdx.x == 0) {
    float t = 0.f;
    for (int w = 0; w < (int)(blockDim.x >> 5); ++w) t += red[w];
    red[0] = t > 0.f ? sqrtf((float)m / t) : 1.f;
  }
  __syncthreads();
  const float sc = fminf(red[0], 1.0f) * 0.999f;
  for (int e = threadIdx.x; e < mm; e += blockDim.x) A[(e % m) + (e / m) * ld] = (float)X[e] * (red[0] > 1.f ? sc : 1.0f);
  __syncthreads();
  float worst = 0.f;
  for (int it = 0; it <= iters; ++it) {
    // G = AᵀA, and how far it is from I; each thread owns a 2×2 block of G
    // (half the shared-memory loads per multiply-add of one element per thread)
    float dev = 0.f;
    const int mh = (m + 1) >> 1;
    for (int e = threadIdx.x; e < mh * mh; e += blockDim.x) {
      const int i0 = 2 * (e % mh), j0 = 2 * (e / mh);
      const int i1 = min(i0 + 1, m - 1), j1 = min(j0 + 1, m - 1);
      float g00 = 0.f, g01 = 0.f, g10 = 0.f, g11 = 0.f;
      for (int k = 0; k < m; ++k) {
        const float a0 = A[k + i0 * ld], a1 = A[k + i1 * ld], b0 = A[k + j0 * ld], b1 = A[k + j1 * ld];
        g00 += a0 * b0;
        g01 += a0 * b1;
        g10 += a1 * b0;
        g11 += a1 * b1;
      }
      G[i0 + j0 * ld] = g00;
      G[i0 + j1 * ld] = g01;
      G[i1 + j0 * ld] = g10;
      G[i1 + j1 * ld] = g11;
      dev = fmaxf(dev, fabsf(g00 - (i0 == j0 ? 1.f : 0.f)));
      dev = fmaxf(dev, fabsf(g01 - (i0 == j1 ? 1.f : 0.f)));
      dev = fmaxf(dev, fabsf(g10 - (i1 == j0 ? 1.f : 0.f)));
      dev = fmaxf(dev, fabsf(g11 - (i1 == j1 ? 1.f : 0.f)));
    }
    for (int o = 16; o > 0; o >>= 1) dev = fmaxf(dev, __shfl_xor_sync(0xffffffffu, dev, o));
    __syncthreads();
    if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = dev;
    __syncthreads();
    if (threadIdx.x == 0) {
      float t = 0.f;
      for (int w = 0; w < (int)(blockDim.x >> 5); ++w) t = fmaxf(t, red[w]);
      red[0] = t;
      // all iterations run: stopping once AᵀA is at FP32 rounding (and polishing
      // in FP64) changed the converged gauge enough to make the fixed-point
      // adjoint's GMRES several times slower
      done = it == iters ? 1 : 0;
    }
    __syncthreads();
    worst = red[0];
    if (done) break;
    // B = A·(1.5 I − 0.5 G), 2×2 blocks per thread
    for (int e = threadIdx.x; e < mh * mh; e += blockDim.x) {
      const int i0 = 2 * (e % mh), j0 = 2 * (e / mh);
      const int i1 = min(i0 + 1, m - 1), j1 = min(j0 + 1, m - 1);
      float b00 = 0.f, b01 = 0.f, b10 = 0.f, b11 = 0.f;
      for (int k = 0; k < m; ++k) {
        const float a0 = A[i0 + k * ld], a1 = A[i1 + k * ld], g0 = G[k + j0 * ld], g1 = G[k + j1 * ld];
        b00 += a0 * g0;
        b01 += a0 * g1;
        b10 += a1 * g0;
        b11 += a1 * g1;
      }
      B[i0 + j0 * ld] = 1.5f * A[i0 + j0 * ld] - 0.5f * b00;
      B[i0 + j1 * ld] = 1.5f * A[i0 + j1 * ld] - 0.5f * b01;
      B[i1 + j0 * ld] = 1.5f * A[i1 + j0 * ld] - 0.5f * b10;
      B[i1 + j1 * ld] = 1.5f * A[i1 + j1 * ld] - 0.5f * b11;
    }
    __syncthreads();
    float* t = A;
    A = B;
    B = t;
  }
  for (int e = threadIdx.x; e < mm; e += blockDim.x) O[e] = (double)A[(e % m) + (e / m) * ld];
  if (threadIdx.x == 0) info[0] = worst < 1e-4f ? 1 : 0;
}

// info[0] = 1 when max |G − I| < 1e-4 for the m×m matrix G = OᵀO (one CTA)
__global__ void k_orth_info(const double* __restrict__ G, int64_t m, int* __restrict__ info) {
  __shared__ double red[32];
  double dev = 0.0;
  for (int64_t e = threadIdx.x; e < m * m; e += blockDim.x)
    dev = fmax(dev, fabs(G[e] - ((e % m) == (e / m) ? 1.0 : 0.0)));
  for (int o = 16; o > 0; o >>= 1) dev = fmax(dev, __shfl_xor_sync(0xffffffffu, dev, o));
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = dev;
  __syncthreads();
  if (threadIdx.x == 0) {
    double t = 0.0;
    for (int w = 0; w < (int)(blockDim.x >> 5); ++w) t = fmax(t, red[w]);
    info[0] = t < 1e-4 ? 1 : 0;
  }
}

// Polar factor for m > 128 (beyond one CTA's shared memory): the same
// Newton–Schulz iteration O ← O·(3I − OᵀO)/2 from O = 0.999·X (X is a product of
// two orthonormal bases, so its singular values are ≤ 1), with its products on
// the multi-CTA GEMMs (TF32X3 where the tensor cores are available; the caller
// polishes in FP64), and the same orthogonality flag.
static void polar_ns_gemm(tnad_ctx* c, const double* X, int64_t m, int iters, double* O, int* dev_info) {
  WsScope scope(c);
  double* G = ws_d(c, m * m);
  double* O2 = ws_d(c, m * m);
  const int pr = c->tc_ok ? TNAD_PREC_TF32X3 : TNAD_PREC_FP64;
  copy_d2d(c, O, X, m * m);
  scale(c, m * m, 0.999, O);
  for (int it = 0; it < iters; ++it) {
    gemm(c, pr, 'T', 'N', m, m, m, 1.0, O, m, O, m, 0.0, G, m);
    copy_d2d(c, O2, O, m * m);
    gemm(c, pr, 'N', 'N', m, m, m, -0.5, O, m, G, m, 1.5, O2, m);
    copy_d2d(c, O, O2, m * m);
  }
  gemm(c, pr, 'T', 'N', m, m, m, 1.0, O, m, O, m, 0.0, G, m);
  k_orth_info<<<1, 1024, 0, c->stream>>>(G, m, dev_info);
  count_launch(c);
  check_launch(c, "polar_ns_gemm");
}

void polar_ns(tnad_ctx* c, const double* X, int64_t m, int iters, double* O, int* dev_info) {
  TNAD_REQUIRE(m >= 1, TNAD_ERR_SHAPE, "polar_ns: m must be >= 1");
  if (m > 128) {
    polar_ns_gemm(c, X, m, iters, O, dev_info);
    return;
  }
  static std::atomic<bool> attr{false};
  if (!attr) {
    TNAD_CK(cudaFuncSetAttribute(k_polar_ns, cudaFuncAttributeMaxDynamicSharedMemorySize, 3 * 129 * 128 * 4));
    attr = true;
  }
  KernelTimer kt(c, "polar_ns", 0.0);
  k_polar_ns<<<1, 1024, (size_t)3 * (m + 1) * m * 4, c->stream>>>(X, (int)m, iters, O, dev_info);
  count_launch(c);
  check_launch(c, "polar_ns");
}

// ---------------------------------------------------------------- Gaussian fill
__device__ __forceinline__ uint64_t mix64(uint64_t x) {
  x ^= x >> 30;
  x *= 0xbf58476d1ce4e5b9ull;
  x ^= x >> 27;
  x *= 0x94d049bb133111ebull;
  x ^= x >> 31;
  return x;
}

// x[i] = scale·N(0,1) sample from a counter-based hash (SplitMix64 finaliser + Box–Muller)
// With sumsq != null the scale is relative to the RMS of the existing entries
// (scale·√(Σx²/n)), read on the device so that no host synchronisation is needed.
__global__ void k_randn(double* __restrict__ x, int64_t n, uint64_t seed, double scale, int accumulate,
                        const double* __restrict__ sumsq) {
  if (sumsq) {
    const double ms = sumsq[0] / (double)n;
    scale *= ms > 0.0 ? sqrt(ms) : 1.0;
  }
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    const uint64_t h1 = mix64(seed * 0x9e3779b97f4a7c15ull + 2 * (uint64_t)i + 1);
    const uint64_t h2 = mix64(h1 ^ 0xd6e8feb86659fd93ull);
    const double u1 = ((double)(h1 >> 11) + 0.5) * (1.0 / 9007199254740992.0);
    const double u2 = (double)(h2 >> 11) * (1.0 / 9007199254740992.0);
    const double g = sqrt(-2.0 * log(u1)) * cospi(2.0 * u2);
    x[i] = accumulate ? x[i] + scale * g : scale * g;
  }
}

void randn(tnad_ctx* c, double* x, int64_t n, uint64_t seed, double scale, bool accumulate,
           const double* dev_sumsq) {
  int nb = (int)std::min<int64_t>((n + 255) / 256, 4096);
  k_randn<<<nb, 256, 0, c->stream>>>(x, n, seed, scale, accumulate ? 1 : 0, dev_sumsq);
  count_launch(c);
  check_launch(c, "randn");
}

}  // namespace tnad
