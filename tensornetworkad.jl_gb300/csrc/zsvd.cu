// ComplexF64 SVD and its adjoint: LinearAlgebra.svd on complex matrices and
// svd_back of src/trg.jl:72-105 with its complex term (the imaginary part of
// diag(Uᴴ·dU) at :85), as exercised by the reference's test/svd.jl.
//
// Complex arrays cross the C ABI interleaved (re, im), as a Julia
// Array{ComplexF64} is laid out; on the device they are split into real and
// imaginary planes so that every product runs on the real GEMMs of this
// library (op(A)·op(B) = four real products).
//
// The decomposition is one-sided Jacobi with complex plane rotations: for the
// column pair (p, q) with α = ‖w_p‖², β = ‖w_q‖², γ = w_pᴴw_q = |γ|e^{iφ}, the
// column w_q is first multiplied by e^{−iφ}, after which the Gram matrix of the
// pair is the real [[α, |γ|], [|γ|, β]] and the real Jacobi rotation
// orthogonalises it.  Singular values are the column norms, sorted descending.
#include <algorithm>
#include <cfloat>
#include <cmath>
#include <cstring>
#include <vector>

#include "tnad_api.h"

namespace tnad {

namespace {

__device__ __forceinline__ double wsum_z(double v) {
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}

__device__ __forceinline__ void pair_of_z(int r, int k, int NP, int* p, int* q) {
  if (k == 0) {
    *p = NP - 1;
    *q = r;
  } else {
    *p = (r + k) % (NP - 1);
    *q = (r - k + (NP - 1)) % (NP - 1);
  }
}

// one round of the circle-method tournament, one warp per column pair
__global__ void k_zjacobi_round(double* __restrict__ Wr, double* __restrict__ Wi, double* __restrict__ Vr,
                                double* __restrict__ Vi, int64_t m, int64_t n, int r, int NP, double tol,
                                int* __restrict__ rotated) {
  const int warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5, lane = threadIdx.x & 31;
  if (warp >= NP / 2) return;
  int p, q;
  pair_of_z(r, warp, NP, &p, &q);
  if (p >= n || q >= n) return;
  if (p > q) {
    const int t = p;
    p = q;
    q = t;
  }
  double* pr = Wr + (int64_t)p * m;
  double* pi = Wi + (int64_t)p * m;
  double* qr = Wr + (int64_t)q * m;
  double* qi = Wi + (int64_t)q * m;
  double a = 0.0, b = 0.0, gr = 0.0, gi = 0.0;
  for (int64_t i = lane; i < m; i += 32) {
    a += pr[i] * pr[i] + pi[i] * pi[i];
    b += qr[i] * qr[i] + qi[i] * qi[i];
    gr += pr[i] * qr[i] + pi[i] * qi[i];  // conj(w_p)·w_q
    gi += pr[i] * qi[i] - pi[i] * qr[i];
  }
  a = wsum_z(a);
  b = wsum_z(b);
  gr = wsum_z(gr);
  gi = wsum_z(gi);
  const double g = hypot(gr, gi);
  if (g == 0.0 || a == 0.0 || b == 0.0 || g <= tol * sqrt(a) * sqrt(b)) return;
  const double er = gr / g, ei = -gi / g;  // e^{−iφ}
  const double zeta = (b - a) / (2.0 * g);
  const double t = (zeta >= 0.0 ? 1.0 : -1.0) / (fabs(zeta) + sqrt(1.0 + zeta * zeta));
  const double cs = 1.0 / sqrt(1.0 + t * t), sn = cs * t;
  for (int64_t i = lane; i < m; i += 32) {
    const double xr = pr[i], xi = pi[i];
    const double yr = er * qr[i] - ei * qi[i], yi = er * qi[i] + ei * qr[i];
    pr[i] = cs * xr - sn * yr;
    pi[i] = cs * xi - sn * yi;
    qr[i] = sn * xr + cs * yr;
    qi[i] = sn * xi + cs * yi;
  }
  double* vpr = Vr + (int64_t)p * n;
  double* vpi = Vi + (int64_t)p * n;
  double* vqr = Vr + (int64_t)q * n;
  double* vqi = Vi + (int64_t)q * n;
  for (int64_t i = lane; i < n; i += 32) {
    const double xr = vpr[i], xi = vpi[i];
    const double yr = er * vqr[i] - ei * vqi[i], yi = er * vqi[i] + ei * vqr[i];
    vpr[i] = cs * xr - sn * yr;
    vpi[i] = cs * xi - sn * yi;
    vqr[i] = sn * xr + cs * yr;
    vqi[i] = sn * xi + cs * yi;
  }
  if (lane == 0) atomicAdd(rotated, 1);
}

// S sorted descending; U[:, r] = w_j/σ_j, V[:, r] = v_j (planar outputs)
__global__ void k_zscatter(const double* __restrict__ Wr, const double* __restrict__ Wi, const double* __restrict__ Vr,
                           const double* __restrict__ Vi, int64_t m, int64_t n, double* __restrict__ Ur,
                           double* __restrict__ Ui, double* __restrict__ S, double* __restrict__ Vor,
                           double* __restrict__ Voi) {
  const int64_t j = blockIdx.x;
  __shared__ double nrm[2];
  __shared__ int rank_s;
  double a = 0.0;
  for (int64_t i = threadIdx.x; i < m; i += blockDim.x) a += Wr[i + j * m] * Wr[i + j * m] + Wi[i + j * m] * Wi[i + j * m];
  a = wsum_z(a);
  if (threadIdx.x == 0) {
    nrm[0] = 0.0;
    rank_s = 0;
  }
  __syncthreads();
  if ((threadIdx.x & 31) == 0) atomicAdd(&nrm[0], a);  // one warp per block: exact order
  __syncthreads();
  const double sj = sqrt(nrm[0]);
  // rank: columns with a larger norm (ties by index); norms recomputed per column k
  int r = 0;
  for (int64_t k = 0; k < n; ++k) {
    if (k == j) continue;
    double b = 0.0;
    for (int64_t i = threadIdx.x; i < m; i += blockDim.x) b += Wr[i + k * m] * Wr[i + k * m] + Wi[i + k * m] * Wi[i + k * m];
    b = wsum_z(b);
    const double sk = sqrt(b);
    r += (sk > sj || (sk == sj && k < j)) ? 1 : 0;
  }
  const int64_t rk = r;
  for (int64_t i = threadIdx.x; i < m; i += blockDim.x) {
    Ur[i + rk * m] = sj > 1e-300 ? Wr[i + j * m] / sj : 0.0;
    Ui[i + rk * m] = sj > 1e-300 ? Wi[i + j * m] / sj : 0.0;
  }
  for (int64_t i = threadIdx.x; i < n; i += blockDim.x) {
    Vor[i + rk * n] = Vr[i + j * n];
    Voi[i + rk * n] = Vi[i + j * n];
  }
  if (threadIdx.x == 0) S[rk] = sj;
}

__global__ void k_split(const double* __restrict__ z, int64_t n, double* __restrict__ re, double* __restrict__ im) {
  for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < n; e += (int64_t)gridDim.x * blockDim.x) {
    re[e] = z[2 * e];
    im[e] = z[2 * e + 1];
  }
}

__global__ void k_join(const double* __restrict__ re, const double* __restrict__ im, int64_t n, double* __restrict__ z) {
  for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < n; e += (int64_t)gridDim.x * blockDim.x) {
    z[2 * e] = re[e];
    z[2 * e + 1] = im[e];
  }
}

// (re, im) of the m×n matrix → its conjugate transpose (n×m)
__global__ void k_ctranspose(const double* __restrict__ re, const double* __restrict__ im, int64_t m, int64_t n,
                             double* __restrict__ tre, double* __restrict__ tim) {
  for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < m * n; e += (int64_t)gridDim.x * blockDim.x) {
    const int64_t i = e % m, j = e / m;
    tre[j + i * n] = re[e];
    tim[j + i * n] = -im[e];
  }
}

__global__ void k_eye2(double* re, double* im, int64_t n) {
  for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < n * n; e += (int64_t)gridDim.x * blockDim.x) {
    re[e] = (e % n == e / n) ? 1.0 : 0.0;
    im[e] = 0.0;
  }
}

// res (K×K, planar) of svd_back, src/trg.jl:76-93:
//   F_ij = (s_j² − s_i²)/((s_j² − s_i²)² + η), Sinv = s/(s² + η)
//   res = (J + Jᴴ)·diag(S) + diag(i·imag(diag(UᴴdU))·Sinv)   [J = F∘(UᴴdU)]
//       + diag(S)·(K + Kᴴ)                                   [K = F∘(VᴴdV)]
//       + diag(dS)
__global__ void k_zsvdback_res(int64_t K, const double* __restrict__ S, const double* __restrict__ Xr,
                               const double* __restrict__ Xi, const double* __restrict__ Yr,
                               const double* __restrict__ Yi, const double* __restrict__ dS, double eta,
                               double* __restrict__ Rr, double* __restrict__ Ri) {
  for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < K * K; e += (int64_t)gridDim.x * blockDim.x) {
    const int64_t i = e % K, j = e / K;
    const double si = S[i], sj = S[j];
    const double d = __dsub_rn(__dmul_rn(sj, sj), __dmul_rn(si, si));
    const double f = __ddiv_rn(d, __dadd_rn(__dmul_rn(d, d), eta));  // F_ij; F_ji = −f
    const int64_t t = j + i * K;                                     // (j, i)
    double rr = 0.0, ri = 0.0;
    if (Xr) {
      // (J + Jᴴ)_ij = F_ij X_ij + conj(F_ji X_ji) = f·(X_ij − conj(X_ji)), times s_j
      rr += f * (Xr[e] - Xr[t]) * sj;
      ri += f * (Xi[e] + Xi[t]) * sj;
      if (i == j) ri += Xi[e] * si / (si * si + eta);
    }
    if (Yr) {
      rr += si * f * (Yr[e] - Yr[t]);
      ri += si * f * (Yi[e] + Yi[t]);
    }
    if (dS && i == j) rr += dS[i];
    Rr[e] = rr;
    Ri[e] = ri;
  }
}

// P ← P·diag(Sinv) on the K columns of a planar (rows × K) matrix
__global__ void k_zscale_cols(int64_t rows, int64_t K, double* __restrict__ Pr, double* __restrict__ Pi,
                              const double* __restrict__ S, double eta) {
  for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < rows * K; e += (int64_t)gridDim.x * blockDim.x) {
    const double s = S[e / rows], f = s / (s * s + eta);
    Pr[e] *= f;
    Pi[e] *= f;
  }
}

int nbz(int64_t n) { return (int)std::min<int64_t>((n + 255) / 256, 4096); }

struct ZMat {
  double* re;
  double* im;
};

ZMat zalloc(tnad_ctx* c, int64_t n) { return ZMat{ws_d(c, n), ws_d(c, n)}; }

// C = alpha·op(A)·op(B) + beta·C, op ∈ {'N', 'C'} (conjugate transpose), planar
// complex; four real FP64 products
void zgemm(tnad_ctx* c, char ta, char tb, int64_t M, int64_t N, int64_t K, double alpha, ZMat A, int64_t lda, ZMat B,
           int64_t ldb, double beta, ZMat Cm, int64_t ldc) {
  const char ra = ta == 'C' ? 'T' : 'N', rb = tb == 'C' ? 'T' : 'N';
  const double sa = ta == 'C' ? -1.0 : 1.0, sb = tb == 'C' ? -1.0 : 1.0;  // sign of the imaginary part of op(·)
  // Cr = Ar·Br − (sa·Ai)(sb·Bi);  Ci = Ar·(sb·Bi) + (sa·Ai)·Br
  gemm_f64(c, ra, rb, M, N, K, alpha, A.re, lda, B.re, ldb, beta, Cm.re, ldc);
  gemm_f64(c, ra, rb, M, N, K, -alpha * sa * sb, A.im, lda, B.im, ldb, 1.0, Cm.re, ldc);
  gemm_f64(c, ra, rb, M, N, K, alpha * sb, A.re, lda, B.im, ldb, beta, Cm.im, ldc);
  gemm_f64(c, ra, rb, M, N, K, alpha * sa, A.im, lda, B.re, ldb, 1.0, Cm.im, ldc);
}

// thin SVD of the planar m×n A with m ≥ n: U m×n, S n, V n×n
void zsvd_tall(tnad_ctx* c, ZMat A, int64_t m, int64_t n, ZMat U, double* S, ZMat V) {
  WsScope scope(c);
  ZMat W = zalloc(c, m * n), Vw = zalloc(c, n * n);
  copy_d2d(c, W.re, A.re, m * n);
  copy_d2d(c, W.im, A.im, m * n);
  k_eye2<<<nbz(n * n), 256, 0, c->stream>>>(Vw.re, Vw.im, n);
  count_launch(c);
  const int NP = (int)(n + (n & 1));
  const double tol = (double)std::max<int64_t>(m, 16) * DBL_EPSILON;
  int* flag = c->d_flag;
  bool converged = n == 1;
  const int blocks = (NP / 2 * 32 + 255) / 256;
  for (int sweep = 0; sweep < 100 && !converged; ++sweep) {
    TNAD_CK(cudaMemsetAsync(flag, 0, sizeof(int), c->stream));
    for (int r = 0; r < NP - 1; ++r)
      k_zjacobi_round<<<blocks, 256, 0, c->stream>>>(W.re, W.im, Vw.re, Vw.im, m, n, r, NP, tol, flag);
    count_launch(c, NP - 1);
    check_launch(c, "zjacobi_round");
    TNAD_CK(cudaMemcpyAsync(c->h_flag, flag, sizeof(int), cudaMemcpyDeviceToHost, c->stream));
    TNAD_CK(cudaStreamSynchronize(c->stream));
    converged = c->h_flag[0] == 0;
  }
  TNAD_REQUIRE(converged, TNAD_ERR_NOT_CONVERGED, "complex svd: no convergence within the sweep cap");
  k_zscatter<<<(unsigned)n, 32, 0, c->stream>>>(W.re, W.im, Vw.re, Vw.im, m, n, U.re, U.im, S, V.re, V.im);
  count_launch(c);
  check_launch(c, "zscatter");
}

}  // namespace

}  // namespace tnad

using namespace tnad;

extern "C" int tnad_svd_z(tnad_ctx* c, const double* A, int m, int n, double* U, double* S, double* V) {
  API_BEGIN(c)
  TNAD_REQUIRE(A && U && S && V && m >= 1 && n >= 1, TNAD_ERR_ARG, "tnad_svd_z: bad arguments");
  WsScope scope(c);
  const int64_t mm = m, nn = n, K = std::min(mm, nn);
  double* dz = ws_d(c, 2 * mm * nn);
  TNAD_CK(cudaMemcpyAsync(dz, A, (size_t)2 * mm * nn * 8, cudaMemcpyHostToDevice, c->stream));
  ZMat Ad = zalloc(c, mm * nn);
  k_split<<<nbz(mm * nn), 256, 0, c->stream>>>(dz, mm * nn, Ad.re, Ad.im);
  count_launch(c);
  ZMat Uo = zalloc(c, mm * K), Vo = zalloc(c, nn * K);
  double* So = ws_d(c, K);
  if (m >= n) {
    zsvd_tall(c, Ad, mm, nn, Uo, So, Vo);
  } else {
    // Aᴴ = Ũ·S·Ṽᴴ (Aᴴ is n×m, tall): A = Ṽ·S·Ũᴴ, so U = Ṽ and V = Ũ
    ZMat At = zalloc(c, mm * nn);
    k_ctranspose<<<nbz(mm * nn), 256, 0, c->stream>>>(Ad.re, Ad.im, mm, nn, At.re, At.im);
    count_launch(c);
    zsvd_tall(c, At, nn, mm, Vo, So, Uo);
  }
  double* zu = ws_d(c, 2 * mm * K);
  double* zv = ws_d(c, 2 * nn * K);
  k_join<<<nbz(mm * K), 256, 0, c->stream>>>(Uo.re, Uo.im, mm * K, zu);
  k_join<<<nbz(nn * K), 256, 0, c->stream>>>(Vo.re, Vo.im, nn * K, zv);
  count_launch(c, 2);
  TNAD_CK(cudaMemcpyAsync(U, zu, (size_t)2 * mm * K * 8, cudaMemcpyDeviceToHost, c->stream));
  TNAD_CK(cudaMemcpyAsync(V, zv, (size_t)2 * nn * K * 8, cudaMemcpyDeviceToHost, c->stream));
  TNAD_CK(cudaMemcpyAsync(S, So, (size_t)K * 8, cudaMemcpyDeviceToHost, c->stream));
  TNAD_CK(cudaStreamSynchronize(c->stream));
  TNAD_CK(cudaGetLastError());
  API_END(c)
}

extern "C" int tnad_svd_back_z(tnad_ctx* c, const double* U, const double* S, const double* V, int m, int n,
                               const double* dU, const double* dS, const double* dV, double eta, double* dA) {
  API_BEGIN(c)
  TNAD_REQUIRE(U && S && V && dA && m >= 1 && n >= 1, TNAD_ERR_ARG, "tnad_svd_back_z: bad arguments");
  WsScope scope(c);
  const int64_t mm = m, nn = n, K = std::min(mm, nn);
  auto load = [&](const double* h, int64_t cnt) {
    double* dz = ws_d(c, 2 * cnt);
    TNAD_CK(cudaMemcpyAsync(dz, h, (size_t)2 * cnt * 8, cudaMemcpyHostToDevice, c->stream));
    ZMat z = zalloc(c, cnt);
    k_split<<<nbz(cnt), 256, 0, c->stream>>>(dz, cnt, z.re, z.im);
    count_launch(c);
    return z;
  };
  ZMat Ud = load(U, mm * K), Vd = load(V, nn * K);
  double* Sd = ws_d(c, K);
  TNAD_CK(cudaMemcpyAsync(Sd, S, (size_t)K * 8, cudaMemcpyHostToDevice, c->stream));
  double* dSd = nullptr;
  if (dS) {
    dSd = ws_d(c, K);
    TNAD_CK(cudaMemcpyAsync(dSd, dS, (size_t)K * 8, cudaMemcpyHostToDevice, c->stream));
  }
  ZMat X{nullptr, nullptr}, Y{nullptr, nullptr}, dUd{nullptr, nullptr}, dVd{nullptr, nullptr};
  if (dU) {
    dUd = load(dU, mm * K);
    X = zalloc(c, K * K);
    zgemm(c, 'C', 'N', K, K, mm, 1.0, Ud, mm, dUd, mm, 0.0, X, K);  // Uᴴ·dU
  }
  if (dV) {
    dVd = load(dV, nn * K);
    Y = zalloc(c, K * K);
    zgemm(c, 'C', 'N', K, K, nn, 1.0, Vd, nn, dVd, nn, 0.0, Y, K);  // Vᴴ·dV
  }
  ZMat R = zalloc(c, K * K);
  k_zsvdback_res<<<nbz(K * K), 256, 0, c->stream>>>(K, Sd, X.re, X.im, Y.re, Y.im, dSd, eta, R.re, R.im);
  count_launch(c);
  // dA = U·res·Vᴴ (src/trg.jl:96)
  ZMat T1 = zalloc(c, mm * K), G = zalloc(c, mm * nn);
  zgemm(c, 'N', 'N', mm, K, K, 1.0, Ud, mm, R, K, 0.0, T1, mm);
  zgemm(c, 'N', 'C', mm, nn, K, 1.0, T1, mm, Vd, nn, 0.0, G, mm);
  if (dU && mm != K) {
    // (dU − U·(Uᴴ·dU))·diag(Sinv)·Vᴴ   (src/trg.jl:98-99)
    ZMat P = zalloc(c, mm * K);
    copy_d2d(c, P.re, dUd.re, mm * K);
    copy_d2d(c, P.im, dUd.im, mm * K);
    zgemm(c, 'N', 'N', mm, K, K, -1.0, Ud, mm, X, K, 1.0, P, mm);
    k_zscale_cols<<<nbz(mm * K), 256, 0, c->stream>>>(mm, K, P.re, P.im, Sd, eta);
    count_launch(c);
    zgemm(c, 'N', 'C', mm, nn, K, 1.0, P, mm, Vd, nn, 1.0, G, mm);
  }
  if (dV && nn != K) {
    // U·diag(Sinv)·(dVᴴ − (dVᴴ·V)·Vᴴ)   (src/trg.jl:102-103), as U·diag(Sinv)·Qᴴ with Q = dV − V·(Vᴴ·dV)
    ZMat Q = zalloc(c, nn * K), Us = zalloc(c, mm * K);
    copy_d2d(c, Q.re, dVd.re, nn * K);
    copy_d2d(c, Q.im, dVd.im, nn * K);
    zgemm(c, 'N', 'N', nn, K, K, -1.0, Vd, nn, Y, K, 1.0, Q, nn);
    copy_d2d(c, Us.re, Ud.re, mm * K);
    copy_d2d(c, Us.im, Ud.im, mm * K);
    k_zscale_cols<<<nbz(mm * K), 256, 0, c->stream>>>(mm, K, Us.re, Us.im, Sd, eta);
    count_launch(c);
    zgemm(c, 'N', 'C', mm, nn, K, 1.0, Us, mm, Q, nn, 1.0, G, mm);
  }
  double* dz = ws_d(c, 2 * mm * nn);
  k_join<<<nbz(mm * nn), 256, 0, c->stream>>>(G.re, G.im, mm * nn, dz);
  count_launch(c);
  TNAD_CK(cudaMemcpyAsync(dA, dz, (size_t)2 * mm * nn * 8, cudaMemcpyDeviceToHost, c->stream));
  TNAD_CK(cudaStreamSynchronize(c->stream));
  TNAD_CK(cudaGetLastError());
  API_END(c)
}
