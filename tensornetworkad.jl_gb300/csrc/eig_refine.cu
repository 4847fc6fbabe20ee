// FP64 refinement of an approximate symmetric eigendecomposition A·X = X·Λ by
// matrix products: the iteration of Ogita and Aishima ("Iterative refinement
// for symmetric eigenvalue decomposition", Japan J. Indust. Appl. Math. 35,
// 2018), with near-degenerate groups resolved by Rayleigh–Ritz and a
// Newton–Schulz re-orthogonalisation after every update.  It replaces the FP64
// Jacobi sweeps that polish the FP32 Jacobi result of the symmetric SVD
// (src/ctmrg.jl:136 on the symmetrised enlarged corner): every O(n³) step is a
// GEMM (on the tensor cores when the context routes FP64 products there), and
// GB300's narrow FP64 pipe only sees O(n²) elementwise work.
//
// One iteration, X (n×n) nearly orthonormal:
//   S = Xᵀ·(A·X),  G = Xᵀ·X,  R = I − G,  λ_j = S_jj / G_jj
//   group: i ~ j when the first-order correction of the pair is not small,
//          |S_ij + λ_j R_ij| > η |λ_j − λ_i| (either order); groups are the
//          intervals of the |λ|-sorted order spanned by such pairs
//   Rayleigh–Ritz inside every group of size ≥ 2 whose largest |λ| is above
//          the noise level max(4nε‖A‖_F, 8·max|S_ij|) (eigh of S on the group,
//          one CTA per group, FP64 Jacobi in shared memory; S and G follow the
//          rotation).  Eigenvalues below that level cannot yet be told apart
//          from zero; a null space stays one unsolved group, and small
//          eigenvalues are solved once the error has dropped below them
//   E_ij = (S_ij + λ_j R_ij)/(λ_j − λ_i) between groups, R_ij/2 inside one
//          (and on the diagonal): X ← X·(I + E), then X ← X·(3I − XᵀX)/2
// until max|S_ij|/‖A‖_F ≤ 1e-10 and max|R_ij| ≤ 1e-8 with no group to solve
// (that update and its re-orthogonalisation are the last), then λ_j = x_jᵀAx_j.
// A group larger than kMaxGroup, or no convergence within kMaxIt iterations,
// returns false and the caller polishes with FP64 Jacobi sweeps instead (graded
// spectra, whose small eigenvalues FP32 cannot separate).
#include <algorithm>
#include <atomic>
#include <cfloat>
#include <cmath>
#include <cstdio>
#include <cstdlib>

#include "tnad_internal.h"

namespace tnad {

namespace {

constexpr int kMaxIt = 8;
constexpr int kMaxGroup = 64;
constexpr double kEta = 0.05;
constexpr int kMaxN = 2048;  // one CTA of 1024 threads scans the sorted order
constexpr double kMaxStartOff = 1e-4;  // max|S_ij|/‖A‖_F of a usable start (FP32 Jacobi: ~1e-6)

__device__ __forceinline__ double warp_max(double v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v = fmax(v, __shfl_xor_sync(0xffffffffu, v, o));
  return v;
}

__device__ __forceinline__ int warp_min_i(int v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v = min(v, __shfl_xor_sync(0xffffffffu, v, o));
  return v;
}

__device__ __forceinline__ int warp_max_i(int v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v = max(v, __shfl_xor_sync(0xffffffffu, v, o));
  return v;
}

// One warp per column j: λ_j = S_jj/G_jj, |λ_j|, max_{i≠j}|S_ij|, max_i|δ_ij − G_ij|.
__global__ void k_ref_colstats(const double* __restrict__ S, const double* __restrict__ G, int n,
                               double* __restrict__ lam, double* __restrict__ absl, double* __restrict__ cmo,
                               double* __restrict__ cmr) {
  const int j = (blockIdx.x * blockDim.x + threadIdx.x) >> 5, lane = threadIdx.x & 31;
  if (j >= n) return;
  const double* s = S + (int64_t)j * n;
  const double* g = G + (int64_t)j * n;
  double mo = 0.0, mr = 0.0;
  bool bad = false;
  for (int i = lane; i < n; i += 32) {
    const double si = s[i], gi = g[i];
    bad |= !isfinite(si) || !isfinite(gi);
    mr = fmax(mr, fabs((i == j ? 1.0 : 0.0) - gi));
    if (i != j) mo = fmax(mo, fabs(si));
  }
  // fmax drops NaN operands: a non-finite entry is reported as an infinite maximum
  if (__any_sync(0xffffffffu, bad)) mo = mr = INFINITY;
  mo = warp_max(mo);
  mr = warp_max(mr);
  if (lane == 0) {
    const double l = s[j] / g[j];
    lam[j] = l;
    absl[j] = fabs(l);
    cmo[j] = mo;
    cmr[j] = mr;
  }
}

// λ_j = S_jj/G_jj and |λ_j| (after a Rayleigh–Ritz rotation)
__global__ void k_ref_lam(const double* __restrict__ S, const double* __restrict__ G, int n, double* __restrict__ lam) {
  const int j = blockIdx.x * blockDim.x + threadIdx.x;
  if (j < n) lam[j] = S[j + (int64_t)j * n] / G[j + (int64_t)j * n];
}

// pos_j = #{i : |λ_i| > |λ_j| or (= and i < j)} (descending |λ|), perm[pos_j] = j
__global__ void k_ref_rank(const double* __restrict__ absl, int n, int* __restrict__ pos, int* __restrict__ perm) {
  const int j = blockIdx.x * blockDim.x + threadIdx.x;
  if (j >= n) return;
  const double a = absl[j];
  int r = 0;
  for (int i = 0; i < n; ++i) {
    const double b = absl[i];
    r += (b > a || (b == a && i < j)) ? 1 : 0;
  }
  pos[j] = r;
  perm[r] = j;
}

// One warp per column i: the sorted positions spanned by i and its strongly
// coupled partners k (|S_ki − λ_i G_ki| or |S_ki − λ_k G_ki| above η|λ_i − λ_k|;
// R_ki = −G_ki off the diagonal) mark the interval [lo, hi) of the sorted
// order as linked: cover[lo] += 1, cover[hi] −= 1.
__global__ void k_ref_strong(const double* __restrict__ S, const double* __restrict__ G, const double* __restrict__ lam,
                             const int* __restrict__ pos, int n, double eta, int* __restrict__ cover) {
  const int i = (blockIdx.x * blockDim.x + threadIdx.x) >> 5, lane = threadIdx.x & 31;
  if (i >= n) return;
  const double li = lam[i];
  const double* s = S + (int64_t)i * n;
  const double* g = G + (int64_t)i * n;
  const int pi = pos[i];
  int lo = pi, hi = pi;
  for (int k = lane; k < n; k += 32) {
    if (k == i) continue;
    const double lk = lam[k];
    const double den = eta * fabs(li - lk);
    const double n1 = fabs(s[k] - li * g[k]), n2 = fabs(s[k] - lk * g[k]);
    if (n1 > den || n2 > den) {
      const int pk = pos[k];
      lo = min(lo, pk);
      hi = max(hi, pk);
    }
  }
  lo = warp_min_i(lo);
  hi = warp_max_i(hi);
  if (lane == 0 && hi > lo) {
    atomicAdd(&cover[lo], 1);
    atomicAdd(&cover[hi], -1);
  }
}

// inclusive scan over the 1024 threads of the block (one value per thread)
__device__ int block_scan_incl(int v, int* sh) {
  const int t = threadIdx.x;
  sh[t] = v;
  __syncthreads();
  for (int off = 1; off < 1024; off <<= 1) {
    const int add = t >= off ? sh[t - off] : 0;
    __syncthreads();
    sh[t] += add;
    __syncthreads();
  }
  const int r = sh[t];
  __syncthreads();
  return r;
}

// Groups from the linked intervals (one CTA of 1024 threads, n ≤ 2048, two
// sorted positions per thread).  Writes gid[j] for every column and the list
// of groups to solve (size ≥ 2, largest |λ| above the noise level): their start in
// the sorted order, size and offset of their k×k block in the Q buffer.
// Stats: si[0] = groups to solve, si[1] = largest such group, si[2] = columns
// in them; sd[0] = max|S_ij|/‖A‖_F, sd[1] = max|R_ij|.
__global__ void __launch_bounds__(1024) k_ref_groups(const int* __restrict__ cover, const int* __restrict__ perm,
                                                     const double* __restrict__ absl, const double* __restrict__ cmo,
                                                     const double* __restrict__ cmr, int n,
                                                     const double* __restrict__ fro2, int* __restrict__ gid,
                                                     int* __restrict__ g_start, int* __restrict__ g_size,
                                                     int* __restrict__ g_qoff, int* __restrict__ si,
                                                     double* __restrict__ sd) {
  __shared__ int sh[1024];
  __shared__ int run_at[1024];
  __shared__ int headflag[kMaxN];
  __shared__ double redo[32], redr[32];
  __shared__ int wmx[32], wcols[32];
  __shared__ double noise_sh;
  const int t = threadIdx.x, w = t >> 5, lane = t & 31;
  const int r0 = 2 * t, r1 = 2 * t + 1;
  const double fro = sqrt(fro2[0]);
  // largest off-diagonal |S_ij| and |R_ij| (columns r0, r1 of this thread)
  double mo = 0.0, mr = 0.0;
  if (r0 < n) {
    mo = fmax(mo, cmo[r0]);
    mr = fmax(mr, cmr[r0]);
  }
  if (r1 < n) {
    mo = fmax(mo, cmo[r1]);
    mr = fmax(mr, cmr[r1]);
  }
  mo = warp_max(mo);
  mr = warp_max(mr);
  if (lane == 0) {
    redo[w] = mo;
    redr[w] = mr;
  }
  __syncthreads();
  if (t == 0) {
    double MO = 0.0, MR = 0.0;
    for (int k = 0; k < 32; ++k) {
      MO = fmax(MO, redo[k]);
      MR = fmax(MR, redr[k]);
    }
    sd[0] = fro > 0.0 ? MO / fro : 0.0;
    sd[1] = MR;
    // eigenvalues below the current off-diagonal error (or the rounding floor)
    // are not yet told apart from zero: their groups are not solved
    noise_sh = fmax(4.0 * (double)n * DBL_EPSILON * fro, 8.0 * MO);
  }
  // cover prefix: sorted position r is linked to r+1 when Σ_{u ≤ r} cover[u] > 0
  const int c0 = r0 < n ? cover[r0] : 0, c1 = r1 < n ? cover[r1] : 0;
  const int incl = block_scan_incl(c0 + c1, sh);  // running sum at r1
  const int run0 = incl - c1;                     // running sum at r0
  run_at[t] = incl;
  __syncthreads();
  const double noise = noise_sh;
  // heads: position r starts a group when r = 0 or r−1 is not linked to r
  const int h0 = (r0 < n) ? ((r0 == 0) ? 1 : (run_at[t - 1] > 0 ? 0 : 1)) : 0;
  const int h1 = (r1 < n) ? (run0 > 0 ? 0 : 1) : 0;
  const int hid = block_scan_incl(h0 + h1, sh);  // heads at positions ≤ r1
  const int id0 = hid - h1 - 1, id1 = hid - 1;
  if (r0 < n) gid[perm[r0]] = id0;
  if (r1 < n) gid[perm[r1]] = id1;
  if (r0 < n) headflag[r0] = h0;
  if (r1 < n) headflag[r1] = h1;
  __syncthreads();
  // group sizes from the heads (scan forward to the next head); a group is
  // solved when it has two members or more and its largest |λ| (its head, the
  // order being descending) is above the noise level
  int solve0 = 0, solve1 = 0, size0 = 0, size1 = 0;
  if (r0 < n && h0) {
    int e = r0 + 1;
    while (e < n && !headflag[e]) ++e;
    size0 = e - r0;
    solve0 = (size0 >= 2 && absl[perm[r0]] > noise) ? 1 : 0;
  }
  if (r1 < n && h1) {
    int e = r1 + 1;
    while (e < n && !headflag[e]) ++e;
    size1 = e - r1;
    solve1 = (size1 >= 2 && absl[perm[r1]] > noise) ? 1 : 0;
  }
  // compact the groups to solve, in sorted order, with Q offsets Σ size²
  const int nsol = block_scan_incl(solve0 + solve1, sh);
  const int q0 = solve0 ? size0 * size0 : 0, q1 = solve1 ? size1 * size1 : 0;
  const int qsum = block_scan_incl(q0 + q1, sh);
  if (solve0) {
    const int k = nsol - solve1 - 1;
    g_start[k] = r0;
    g_size[k] = size0;
    g_qoff[k] = qsum - q1 - q0;
  }
  if (solve1) {
    const int k = nsol - 1;
    g_start[k] = r1;
    g_size[k] = size1;
    g_qoff[k] = qsum - q1;
  }
  int mx = max(solve0 ? size0 : 0, solve1 ? size1 : 0);
  int cols = (solve0 ? size0 : 0) + (solve1 ? size1 : 0);
  mx = warp_max_i(mx);
  for (int o = 16; o > 0; o >>= 1) cols += __shfl_xor_sync(0xffffffffu, cols, o);
  if (lane == 0) {
    wmx[w] = mx;
    wcols[w] = cols;
  }
  __syncthreads();
  if (t == 0) {
    int M = 0, Cc = 0;
    for (int k = 0; k < 32; ++k) {
      M = max(M, wmx[k]);
      Cc += wcols[k];
    }
    si[1] = M;
    si[2] = Cc;
  }
  if (t == 1023) si[0] = nsol;
}

// Rayleigh–Ritz of one group per CTA: H = S restricted to the group's columns
// (k ≤ kMaxGroup, symmetrised), cyclic Jacobi in FP64 in shared memory, the
// eigenvectors (unsorted) to Q at the group's offset.
__global__ void __launch_bounds__(256) k_ref_rr(const double* __restrict__ S, int n, const int* __restrict__ perm,
                                                const int* __restrict__ g_start, const int* __restrict__ g_size,
                                                const int* __restrict__ g_qoff, double* __restrict__ Qbuf) {
  extern __shared__ double smr[];
  const int k = g_size[blockIdx.x];
  const int ld = k + 1;
  double* H = smr;           // k × ld
  double* Z = H + k * ld;    // k × k
  __shared__ int mem[kMaxGroup];
  __shared__ double cs_[kMaxGroup / 2], sn_[kMaxGroup / 2];
  __shared__ int pp_[kMaxGroup / 2], qq_[kMaxGroup / 2];
  __shared__ int rotated;
  __shared__ double fro_part[8];
  const int st = g_start[blockIdx.x];
  for (int i = threadIdx.x; i < k; i += blockDim.x) mem[i] = perm[st + i];
  __syncthreads();
  double ss = 0.0;
  for (int e = threadIdx.x; e < k * k; e += blockDim.x) {
    const int i = e % k, j = e / k;
    const double v = 0.5 * (S[mem[i] + (int64_t)mem[j] * n] + S[mem[j] + (int64_t)mem[i] * n]);
    H[i + j * ld] = v;
    Z[e] = (i == j) ? 1.0 : 0.0;
    ss += v * v;
  }
  for (int o = 16; o > 0; o >>= 1) ss += __shfl_xor_sync(0xffffffffu, ss, o);
  if ((threadIdx.x & 31) == 0) fro_part[threadIdx.x >> 5] = ss;
  __syncthreads();
  double f2 = 0.0;
  for (int w = 0; w < 8; ++w) f2 += fro_part[w];
  const double tol = 4.0 * DBL_EPSILON * sqrt((double)k);
  const double absfl = 2.0 * DBL_EPSILON * sqrt((double)k) * sqrt(f2);
  const int NP = k + (k & 1);
  const int wid = threadIdx.x >> 5, lane = threadIdx.x & 31, nwarp = blockDim.x >> 5;
  for (int sweep = 0; sweep < 40; ++sweep) {
    if (threadIdx.x == 0) rotated = 0;
    __syncthreads();
    for (int r = 0; r < NP - 1; ++r) {
      for (int q = threadIdx.x; q < NP / 2; q += blockDim.x) {
        int a, b;
        if (q == 0) {
          a = NP - 1;
          b = r;
        } else {
          a = (r + q) % (NP - 1);
          b = (r - q + (NP - 1)) % (NP - 1);
        }
        double c = 1.0, s = 0.0;
        if (a < k && b < k) {
          if (a > b) {
            const int tt = a;
            a = b;
            b = tt;
          }
          const double apq = H[a + b * ld], app = H[a + a * ld], aqq = H[b + b * ld];
          if (apq != 0.0 && fabs(apq) > tol * sqrt(fabs(app)) * sqrt(fabs(aqq)) && fabs(apq) > absfl) {
            const double tau = (aqq - app) / (2.0 * apq);
            const double tt = (tau >= 0.0 ? 1.0 : -1.0) / (fabs(tau) + sqrt(1.0 + tau * tau));
            c = 1.0 / sqrt(1.0 + tt * tt);
            s = tt * c;
            rotated = 1;
          }
        } else {
          a = b = -1;
        }
        pp_[q] = a;
        qq_[q] = b;
        cs_[q] = c;
        sn_[q] = s;
      }
      __syncthreads();
      for (int q = wid; q < NP / 2; q += nwarp) {
        const int a = pp_[q], b = qq_[q];
        if (a < 0 || sn_[q] == 0.0) continue;
        const double c = cs_[q], s = sn_[q];
        for (int col = lane; col < k; col += 32) {
          const double x = H[a + col * ld], y = H[b + col * ld];
          H[a + col * ld] = c * x - s * y;
          H[b + col * ld] = s * x + c * y;
        }
      }
      __syncthreads();
      for (int q = wid; q < NP / 2; q += nwarp) {
        const int a = pp_[q], b = qq_[q];
        if (a < 0 || sn_[q] == 0.0) continue;
        const double c = cs_[q], s = sn_[q];
        for (int row = lane; row < k; row += 32) {
          const double x = H[row + a * ld], y = H[row + b * ld];
          H[row + a * ld] = c * x - s * y;
          H[row + b * ld] = s * x + c * y;
          const double zx = Z[row + a * k], zy = Z[row + b * k];
          Z[row + a * k] = c * zx - s * zy;
          Z[row + b * k] = s * zx + c * zy;
        }
        __syncwarp();
        if (lane == 0) {
          H[a + b * ld] = 0.0;
          H[b + a * ld] = 0.0;
        }
      }
      __syncthreads();
    }
    const int done = (rotated == 0);
    __syncthreads();
    if (done) break;
  }
  double* Q = Qbuf + g_qoff[blockIdx.x];
  for (int e = threadIdx.x; e < k * k; e += blockDim.x) Q[e] = Z[e];
}

// M[r, m_j] ← Σ_i M[r, m_i]·Q[i, j] for the members m of group blockIdx.x and
// the 128 rows r of blockIdx.y (a column rotation of M restricted to the group)
__global__ void __launch_bounds__(128) k_ref_rot_cols(double* __restrict__ M, int ldm, int nrows,
                                                      const int* __restrict__ perm, const int* __restrict__ g_start,
                                                      const int* __restrict__ g_size, const int* __restrict__ g_qoff,
                                                      const double* __restrict__ Qbuf) {
  extern __shared__ double smc[];
  const int k = g_size[blockIdx.x];
  double* Q = smc;           // k×k
  double* tile = Q + k * k;  // 128 × k (row-major per thread: tile[t*k + i])
  __shared__ int mem[kMaxGroup];
  const int st = g_start[blockIdx.x];
  for (int i = threadIdx.x; i < k; i += blockDim.x) mem[i] = perm[st + i];
  const double* Qg = Qbuf + g_qoff[blockIdx.x];
  for (int e = threadIdx.x; e < k * k; e += blockDim.x) Q[e] = Qg[e];
  __syncthreads();
  const int r = blockIdx.y * 128 + threadIdx.x;
  if (r >= nrows) return;
  double* tr = tile + threadIdx.x * k;
  for (int i = 0; i < k; ++i) tr[i] = M[r + (int64_t)mem[i] * ldm];
  for (int j = 0; j < k; ++j) {
    double acc = 0.0;
    for (int i = 0; i < k; ++i) acc = fma(tr[i], Q[i + j * k], acc);
    M[r + (int64_t)mem[j] * ldm] = acc;
  }
}

// M[m_j, col] ← Σ_i Q[i, j]·M[m_i, col] (a row rotation restricted to the group)
__global__ void __launch_bounds__(128) k_ref_rot_rows(double* __restrict__ M, int ldm, int ncols,
                                                      const int* __restrict__ perm, const int* __restrict__ g_start,
                                                      const int* __restrict__ g_size, const int* __restrict__ g_qoff,
                                                      const double* __restrict__ Qbuf) {
  extern __shared__ double smc[];
  const int k = g_size[blockIdx.x];
  double* Q = smc;
  double* tile = Q + k * k;
  __shared__ int mem[kMaxGroup];
  const int st = g_start[blockIdx.x];
  for (int i = threadIdx.x; i < k; i += blockDim.x) mem[i] = perm[st + i];
  const double* Qg = Qbuf + g_qoff[blockIdx.x];
  for (int e = threadIdx.x; e < k * k; e += blockDim.x) Q[e] = Qg[e];
  __syncthreads();
  const int col = blockIdx.y * 128 + threadIdx.x;
  if (col >= ncols) return;
  double* tr = tile + threadIdx.x * k;
  for (int i = 0; i < k; ++i) tr[i] = M[mem[i] + (int64_t)col * ldm];
  for (int j = 0; j < k; ++j) {
    double acc = 0.0;
    for (int i = 0; i < k; ++i) acc = fma(Q[i + j * k], tr[i], acc);
    M[mem[j] + (int64_t)col * ldm] = acc;
  }
}

// E_ij = (S_ij + λ_j R_ij)/(λ_j − λ_i) between groups; R_ij/2 inside a group
// and on the diagonal (R = I − G)
__global__ void k_ref_E(const double* __restrict__ S, const double* __restrict__ G, const double* __restrict__ lam,
                        const int* __restrict__ gid, int n, double* __restrict__ E) {
  const int64_t nn = (int64_t)n * n;
  for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < nn; e += (int64_t)gridDim.x * blockDim.x) {
    const int i = (int)(e % n), j = (int)(e / n);
    const double r = (i == j ? 1.0 : 0.0) - G[e];
    double v;
    if (i == j || gid[i] == gid[j]) {
      v = 0.5 * r;
    } else {
      const double den = lam[j] - lam[i];
      v = den != 0.0 ? (S[e] + lam[j] * r) / den : 0.5 * r;
    }
    E[e] = v;
  }
}

// lam_j = Σ_i X_ij·Y_ij (one warp per column)
__global__ void k_ref_coldots(const double* __restrict__ X, const double* __restrict__ Y, int n,
                              double* __restrict__ lam) {
  const int j = (blockIdx.x * blockDim.x + threadIdx.x) >> 5, lane = threadIdx.x & 31;
  if (j >= n) return;
  double s = 0.0;
  for (int i = lane; i < n; i += 32) s = fma(X[i + (int64_t)j * n], Y[i + (int64_t)j * n], s);
  for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
  if (lane == 0) lam[j] = s;
}

int nblk(int64_t n, int t = 256) { return (int)std::min<int64_t>((n + t - 1) / t, 4096); }

// W[:, r] = X[:, j], lam_out[r] = lam[j] with r the rank of |λ_j| (descending,
// ties by index); one CTA of 256 threads per column j
__global__ void __launch_bounds__(256) k_ref_sort_abs(const double* __restrict__ X, const double* __restrict__ lam,
                                                      int n, double* __restrict__ W, double* __restrict__ lam_out) {
  const int j = blockIdx.x;
  __shared__ int part[8];
  __shared__ int rank_sh;
  const double a = fabs(lam[j]);
  int r = 0;
  for (int i = threadIdx.x; i < n; i += blockDim.x) {
    const double b = fabs(lam[i]);
    r += (b > a || (b == a && i < j)) ? 1 : 0;
  }
  for (int o = 16; o > 0; o >>= 1) r += __shfl_xor_sync(0xffffffffu, r, o);
  if ((threadIdx.x & 31) == 0) part[threadIdx.x >> 5] = r;
  __syncthreads();
  if (threadIdx.x == 0) {
    int t = 0;
    for (int w = 0; w < 8; ++w) t += part[w];
    rank_sh = t;
    lam_out[t] = lam[j];
  }
  __syncthreads();
  const int64_t rr = rank_sh;
  for (int i = threadIdx.x; i < n; i += blockDim.x) W[i + rr * n] = X[i + (int64_t)j * n];
}

}  // namespace

bool eig_refine(tnad_ctx* c, const double* A, int64_t n64, double* X, double* lam, const double* fro2) {
  if (n64 < 2 || n64 > kMaxN) return false;
  const int n = (int)n64;
  static std::atomic<bool> attr{false};
  if (!attr) {
    const int rr_sm = (kMaxGroup * (kMaxGroup + 1) + kMaxGroup * kMaxGroup) * 8;
    const int rot_sm = (kMaxGroup * kMaxGroup + 128 * kMaxGroup) * 8;
    TNAD_CK(cudaFuncSetAttribute(k_ref_rr, cudaFuncAttributeMaxDynamicSharedMemorySize, rr_sm));
    TNAD_CK(cudaFuncSetAttribute(k_ref_rot_cols, cudaFuncAttributeMaxDynamicSharedMemorySize, rot_sm));
    TNAD_CK(cudaFuncSetAttribute(k_ref_rot_rows, cudaFuncAttributeMaxDynamicSharedMemorySize, rot_sm));
    attr = true;
  }
  WsScope scope(c);
  const int64_t nn = (int64_t)n * n;
  double* AX = ws_d(c, nn);
  double* S = ws_d(c, nn);
  double* G = ws_d(c, nn);
  double* E = ws_d(c, nn);
  double* Xn = ws_d(c, nn);
  double* absl = ws_d(c, n);
  double* cmo = ws_d(c, n);
  double* cmr = ws_d(c, n);
  double* Qbuf = ws_d(c, (int64_t)n * kMaxGroup);
  double* sd = ws_d(c, 4);
  int* ibuf = (int*)c->ws.alloc(sizeof(int) * (size_t)(7 * n + 8));
  int* pos = ibuf;
  int* perm = pos + n;
  int* cover = perm + n;  // n + 1
  int* gid = cover + n + 1;
  int* g_start = gid + n;
  int* g_size = g_start + n;
  int* g_qoff = g_size + n;
  int* si = g_qoff + n;  // 4 ints
  const int64_t col_threads = (int64_t)n * 32;
  bool done = false;
  double prev_off = 0.0;
  for (int it = 0; it < kMaxIt && !done; ++it) {
    KernelTimer kt(c, "eig_refine", 6.0 * 2.0 * (double)nn * n);
    gemm(c, TNAD_PREC_FP64, 'N', 'N', n, n, n, 1.0, A, n, X, n, 0.0, AX, n);
    gemm(c, TNAD_PREC_FP64, 'T', 'N', n, n, n, 1.0, X, n, AX, n, 0.0, S, n);
    gemm(c, TNAD_PREC_FP64, 'T', 'N', n, n, n, 1.0, X, n, X, n, 0.0, G, n);
    k_ref_colstats<<<nblk(col_threads), 256, 0, c->stream>>>(S, G, n, lam, absl, cmo, cmr);
    k_ref_rank<<<nblk(n), 256, 0, c->stream>>>(absl, n, pos, perm);
    TNAD_CK(cudaMemsetAsync(cover, 0, sizeof(int) * (size_t)(n + 1), c->stream));
    k_ref_strong<<<nblk(col_threads), 256, 0, c->stream>>>(S, G, lam, pos, n, kEta, cover);
    k_ref_groups<<<1, 1024, 0, c->stream>>>(cover, perm, absl, cmo, cmr, n, fro2, gid, g_start, g_size, g_qoff, si,
                                            sd);
    count_launch(c, 5);
    check_launch(c, "eig_refine_groups");
    int hs[4];
    double hd[2];
    TNAD_CK(cudaMemcpyAsync(hs, si, sizeof(int) * 3, cudaMemcpyDeviceToHost, c->stream));
    TNAD_CK(cudaMemcpyAsync(hd, sd, sizeof(double) * 2, cudaMemcpyDeviceToHost, c->stream));
    TNAD_CK(cudaStreamSynchronize(c->stream));
    const int ngroups = hs[0], maxgroup = hs[1];
    if (std::getenv("TNAD_TRACE"))
      std::fprintf(stderr, "[tnad trace] eig_refine n=%d it %d off %.2e orth %.2e groups %d (max %d, cols %d)\n", n, it,
                   hd[0], hd[1], ngroups, maxgroup, hs[2]);
    // not an approximate eigendecomposition (the first measurement), growing
    // errors, non-finite entries or a group too large for one CTA: give up
    if (!std::isfinite(hd[0]) || !std::isfinite(hd[1]) || maxgroup > kMaxGroup) return false;
    if ((it == 0 && hd[0] > kMaxStartOff) || (it > 0 && hd[0] > 4.0 * prev_off)) return false;
    prev_off = hd[0];
    done = it >= 1 && hd[0] <= 1e-10 && hd[1] <= 1e-8 && ngroups == 0;
    if (ngroups > 0) {
      // Rayleigh–Ritz inside the groups; S, G and X follow the block rotation
      const size_t rr_sm = (size_t)(maxgroup * (maxgroup + 1) + maxgroup * maxgroup) * 8;
      const size_t rot_sm = (size_t)(maxgroup * maxgroup + 128 * maxgroup) * 8;
      k_ref_rr<<<ngroups, 256, rr_sm, c->stream>>>(S, n, perm, g_start, g_size, g_qoff, Qbuf);
      const dim3 gr((unsigned)ngroups, (unsigned)((n + 127) / 128));
      k_ref_rot_cols<<<gr, 128, rot_sm, c->stream>>>(S, n, n, perm, g_start, g_size, g_qoff, Qbuf);
      k_ref_rot_rows<<<gr, 128, rot_sm, c->stream>>>(S, n, n, perm, g_start, g_size, g_qoff, Qbuf);
      k_ref_rot_cols<<<gr, 128, rot_sm, c->stream>>>(G, n, n, perm, g_start, g_size, g_qoff, Qbuf);
      k_ref_rot_rows<<<gr, 128, rot_sm, c->stream>>>(G, n, n, perm, g_start, g_size, g_qoff, Qbuf);
      k_ref_rot_cols<<<gr, 128, rot_sm, c->stream>>>(X, n, n, perm, g_start, g_size, g_qoff, Qbuf);
      k_ref_lam<<<nblk(n), 256, 0, c->stream>>>(S, G, n, lam);
      count_launch(c, 7);
      check_launch(c, "eig_refine_rr");
    }
    k_ref_E<<<nblk(nn), 256, 0, c->stream>>>(S, G, lam, gid, n, E);
    count_launch(c);
    check_launch(c, "eig_refine_E");
    // X ← X·(I + E), then one Newton–Schulz step X ← X·(3I − XᵀX)/2
    copy_d2d(c, Xn, X, nn);
    gemm(c, TNAD_PREC_FP64, 'N', 'N', n, n, n, 1.0, X, n, E, n, 1.0, Xn, n);
    gemm(c, TNAD_PREC_FP64, 'T', 'N', n, n, n, 1.0, Xn, n, Xn, n, 0.0, G, n);
    copy_d2d(c, X, Xn, nn);
    gemm(c, TNAD_PREC_FP64, 'N', 'N', n, n, n, -0.5, Xn, n, G, n, 1.5, X, n);
  }
  if (!done) return false;
  gemm(c, TNAD_PREC_FP64, 'N', 'N', n, n, n, 1.0, A, n, X, n, 0.0, AX, n);
  k_ref_coldots<<<nblk(col_threads), 256, 0, c->stream>>>(X, AX, n, lam);
  count_launch(c);
  check_launch(c, "eig_refine_lam");
  return true;
}

// Eigendecomposition H = W·diag(lam)·Wᵀ of a small symmetric p×p matrix
// (p ≤ 256) to FP64 accuracy: the one-CTA FP32 Jacobi solve (eigenvalue rule,
// so ±λ pairs stay apart) polished by the product refinement above, sorted by
// |λ| descending.  false: the refinement did not converge (W, lam untouched).
bool eigh_fp32_refined(tnad_ctx* c, const double* H, int64_t p, double* W, double* lam) {
  if (!c->eig_refine || p < 2 || p > 256) return false;
  WsScope scope(c);
  double* X = ws_d(c, p * p);
  double* l = ws_d(c, p);
  double* fro2 = ws_d(c, 1);
  eigh_small_prec(c, true, H, p, X, l, 40, nullptr);
  sumsq_dev(c, H, p * p, fro2);
  if (!eig_refine(c, H, p, X, l, fro2)) {
    ++c->eig_fallback;
    return false;
  }
  ++c->eig_refined;
  k_ref_sort_abs<<<(unsigned)p, 256, 0, c->stream>>>(X, l, (int)p, W, lam);
  count_launch(c);
  check_launch(c, "eigh_fp32_refined");
  return true;
}

}  // namespace tnad
