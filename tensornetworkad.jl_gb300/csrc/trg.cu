// TRG on the device: trg (src/trg.jl:13-30), trg_svd (src/trg.jl:33-44) and the
// reverse pass (Zygote adjoint of the same loop with svd_back, src/trg.jl:55-61, 72-105).
// The bond dimension follows the reference exactly, including its
// searchsortedfirst quirk: k = min(#(s > tol) + 1, χ, length(s)).
#include <cmath>

#include "tnad_trg.h"

namespace tnad {

static int nb(int64_t n) { return (int)std::min<int64_t>((n + 255) / 256, 4096); }

// u[:, j] = U[:, j]·√S_j (j < k) ; v[j, c] = √S_j·V[c, j]
__global__ void k_trg_split(const double* __restrict__ U, const double* __restrict__ S, const double* __restrict__ V,
                            int64_t m, int64_t n, int64_t k, double* __restrict__ u, double* __restrict__ v) {
  int64_t tot = m * k + k * n;
  for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < tot; e += (int64_t)gridDim.x * blockDim.x) {
    if (e < m * k) {
      int64_t j = e / m;
      u[e] = U[e] * sqrt(S[j]);
    } else {
      int64_t f = e - m * k;
      int64_t j = f % k, cc = f / k;
      v[f] = sqrt(S[j]) * V[cc + j * n];
    }
  }
}

// Pullback of k_trg_split into (dU m×ns, dV n×ns, dS ns); zero beyond k.
// √S at S = 0 has no derivative: a kept zero singular value gets dS = 0.
__global__ void k_trg_split_bwd(const double* __restrict__ U, const double* __restrict__ S,
                                const double* __restrict__ V, int64_t m, int64_t n, int64_t ns, int64_t k,
                                const double* __restrict__ du, const double* __restrict__ dv, double* __restrict__ dU,
                                double* __restrict__ dV, double* __restrict__ dS) {
  int64_t tot = m * ns + n * ns + ns;
  for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < tot; e += (int64_t)gridDim.x * blockDim.x) {
    if (e < m * ns) {
      int64_t j = e / m;
      dU[e] = j < k ? du[e] * sqrt(S[j]) : 0.0;
    } else if (e < m * ns + n * ns) {
      int64_t f = e - m * ns;
      int64_t cc = f % n, j = f / n;
      dV[f] = j < k ? dv[j + k * cc] * sqrt(S[j]) : 0.0;
    } else {
      int64_t j = e - m * ns - n * ns;
      double r = 0.0;
      if (j < k && S[j] > 0.0) {
        double acc = 0.0;
        for (int64_t i = 0; i < m; ++i) acc += du[i + j * m] * U[i + j * m];
        for (int64_t cc = 0; cc < n; ++cc) acc += dv[j + k * cc] * V[cc + j * n];
        r = acc / (2.0 * sqrt(S[j]));
      }
      dS[j] = r;
    }
  }
}

__global__ void k_trace_ijij(const double* __restrict__ a, int64_t d0, int64_t d1, double* out) {
  if (threadIdx.x == 0 && blockIdx.x == 0) {
    double t = 0.0;
    for (int64_t j = 0; j < d1; ++j)
      for (int64_t i = 0; i < d0; ++i) t += a[i + d0 * (j + d1 * (i + d0 * j))];
    out[0] = t;
  }
}

__global__ void k_trace_bwd(double* __restrict__ da, int64_t d0, int64_t d1, double g) {
  int64_t n = d0 * d1;
  for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < n; e += (int64_t)gridDim.x * blockDim.x) {
    int64_t i = e % d0, j = e / d0;
    da[i + d0 * (j + d1 * (i + d0 * j))] += g;
  }
}

// da_raw = da_norm/mv ; da_raw[idx] += g·sign(a_raw[idx]) where g is on the host
__global__ void k_maxnorm_bwd(int64_t n, const double* __restrict__ dan, double mv, const double* __restrict__ araw,
                              int64_t idx, const double* __restrict__ dotdev, double extra, double* __restrict__ out) {
  double g = -dotdev[0] / (mv * mv) + extra;
  for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < n; e += (int64_t)gridDim.x * blockDim.x) {
    double v = dan[e] / mv;
    if (e == idx) v += g * (araw[e] >= 0.0 ? 1.0 : -1.0);
    out[e] = v;
  }
}

static void svd_any(tnad_ctx* c, const double* A, int64_t m, int64_t n, double* U, double* S, double* V) {
  // thin SVD for any shape; U m×ns, V n×ns, ns = min(m,n)
  if (m >= n) {
    svd_jacobi(c, A, m, n, U, S, V, false);
  } else {
    WsScope scope(c);
    double* At = ws_d(c, m * n);
    Ten t = make_ten(const_cast<double*>(A), {m, n});
    int perm[2] = {1, 0};
    permute(c, t, perm, At);
    svd_jacobi(c, At, n, m, V, S, U, false);  // Aᵀ = V S Uᵀ
  }
}

static void svd_back_any(tnad_ctx* c, const double* U, const double* S, const double* V, int64_t m, int64_t n,
                         const double* dU, const double* dS, const double* dV, double* dA) {
  if (m >= n) {
    svd_back(c, TNAD_PREC_FP64, U, S, V, m, n, dU, dS, dV, 1e-40, dA);
  } else {
    WsScope scope(c);
    double* t = ws_d(c, m * n);
    svd_back(c, TNAD_PREC_FP64, V, S, U, n, m, dV, dS, dU, 1e-40, t);  // (Aᵀ)̄
    Ten tt = make_ten(t, {n, m});
    int perm[2] = {1, 0};
    permute(c, tt, perm, dA);
  }
}

void trg_svd_fwd(tnad_ctx* c, const double* t, const int64_t dd[4], int chi, double tol, TrgSvd& s, DevPool* pool) {
  s.m = dd[0] * dd[1];
  s.n = dd[2] * dd[3];
  s.ns = std::min(s.m, s.n);
  for (int q = 0; q < 4; ++q) s.dims[q] = dd[q];
  s.U = pool->d(s.m * s.ns);
  s.S = pool->d(s.ns);
  s.V = pool->d(s.n * s.ns);
  svd_any(c, t, s.m, s.n, s.U, s.S, s.V);
  std::vector<double> hs(s.ns);
  TNAD_CK(cudaMemcpyAsync(hs.data(), s.S, s.ns * 8, cudaMemcpyDeviceToHost, c->stream));
  TNAD_CK(cudaStreamSynchronize(c->stream));
  int64_t cnt = 0;
  for (double x : hs) cnt += (x > tol) ? 1 : 0;
  s.k = std::min<int64_t>(std::min<int64_t>(cnt + 1, chi), s.ns);
  // Values at the rounding floor (at or below tol, or below 64ε·s₁ where the
  // solver's absolute accuracy ends) carry noise vectors; LAPACK reports them as
  // ~1e-17..1e-15 with its own noise.  They are set to exactly 0: a kept noise
  // column (the +1 quirk) then contributes u = v = 0 and no noise-amplified √s
  // pullback (d√s/ds = 1/(2√s)); lnZ moves by less than the floor itself.
  const double floor_s = std::max(tol, 64.0 * 2.220446049250313e-16 * (hs.empty() ? 0.0 : hs[0]));
  bool any = false;
  for (double& x : hs)
    if (x <= floor_s && x != 0.0) {
      x = 0.0;
      any = true;
    }
  if (any) TNAD_CK(cudaMemcpyAsync(s.S, hs.data(), s.ns * 8, cudaMemcpyHostToDevice, c->stream));
  s.u = pool->d(s.m * s.k);
  s.v = pool->d(s.k * s.n);
  k_trg_split<<<nb(s.m * s.k + s.k * s.n), 256, 0, c->stream>>>(s.U, s.S, s.V, s.m, s.n, s.k, s.u, s.v);
  count_launch(c);
  check_launch(c, "trg_split");
}

void trg_svd_bwd(tnad_ctx* c, const TrgSvd& s, const double* du, const double* dv, double* dt) {
  WsScope scope(c);
  double* dU = ws_d(c, s.m * s.ns);
  double* dV = ws_d(c, s.n * s.ns);
  double* dS = ws_d(c, s.ns);
  k_trg_split_bwd<<<nb(s.m * s.ns + s.n * s.ns + s.ns), 256, 0, c->stream>>>(s.U, s.S, s.V, s.m, s.n, s.ns, s.k, du,
                                                                              dv, dU, dV, dS);
  count_launch(c);
  svd_back_any(c, s.U, s.S, s.V, s.m, s.n, dU, dS, dV, dt);
}

void trg_fwd(tnad_ctx* c, TrgTape& tp, const double* a0, int d, int chi, int niter, double tol) {
  DevPool& P = tp.pool;
  tp.niter = niter;
  tp.chi = chi;
  int64_t dims[4] = {d, d, d, d};
  int64_t na = (int64_t)d * d * d * d;
  double* a = P.d(na);
  copy_d2d(c, a, a0, na);
  double lnZ = 0.0;
  for (int it = 1; it <= niter; ++it) {
    TrgIter I;
    for (int q = 0; q < 4; ++q) I.dims[q] = dims[q];
    I.araw = a;
    na = dims[0] * dims[1] * dims[2] * dims[3];
    // maxval = maximum(abs.(a)); a /= maxval; lnZ += 2^(1-n) log(maxval)   (src/trg.jl:16-18)
    maxabs_dev(c, a, na, c->d_red);
    TNAD_CK(cudaMemcpyAsync(c->h_pin, c->d_red, 16, cudaMemcpyDeviceToHost, c->stream));
    TNAD_CK(cudaStreamSynchronize(c->stream));
    I.mv = c->h_pin[0];
    I.idx = (int64_t)c->h_pin[1];
    TNAD_REQUIRE(std::isfinite(I.mv) && I.mv > 0.0, TNAD_ERR_NONFINITE, "trg: max |a| is zero or non-finite");
    double* an = P.d(na);
    copy_d2d(c, an, a, na);
    scale(c, na, 1.0 / I.mv, an);
    lnZ += std::pow(2.0, 1 - it) * std::log(I.mv);
    Ten at = make_ten(an, {dims[0], dims[1], dims[2], dims[3]});
    // dr_ul = ein"urdl -> drul"(a); ld_ru = ein"urdl -> ldru"(a)   (:20-21)
    const int p1[4] = {2, 1, 0, 3}, p2[4] = {3, 2, 1, 0};
    double* drul = P.d(na);
    double* ldru = P.d(na);
    permute(c, at, p1, drul);
    permute(c, at, p2, ldru);
    int64_t d1[4] = {dims[2], dims[1], dims[0], dims[3]};
    int64_t d2[4] = {dims[3], dims[2], dims[1], dims[0]};
    trg_svd_fwd(c, drul, d1, chi, tol, I.s1, &P);  // dr, ul
    trg_svd_fwd(c, ldru, d2, chi, tol, I.s2, &P);  // ld, ru
    // a = ein"npu,por,dom,lmn -> urdl"(dr, ld, ul, ru)   (:25)
    Ten dr = make_ten(I.s1.u, {d1[0], d1[1], I.s1.k});
    Ten ul = make_ten(I.s1.v, {I.s1.k, d1[2], d1[3]});
    Ten ld = make_ten(I.s2.u, {d2[0], d2[1], I.s2.k});
    Ten ru = make_ten(I.s2.v, {I.s2.k, d2[2], d2[3]});
    I.x = make_ten(P.d(dr.dim[0] * dr.dim[2] * ld.dim[1] * ld.dim[2]), {});
    contract(c, TNAD_PREC_FP64, dr, "npu", ld, "por", I.x, "nuor");
    I.y = make_ten(P.d(ul.dim[0] * ul.dim[1] * ru.dim[0] * ru.dim[2]), {});
    contract(c, TNAD_PREC_FP64, ul, "dom", ru, "lmn", I.y, "doln");
    Ten an2 = make_ten(P.d(I.s1.k * I.s2.k * I.s1.k * I.s2.k), {});
    contract(c, TNAD_PREC_FP64, I.x, "nuor", I.y, "doln", an2, "urdl");
    for (int q = 0; q < 4; ++q) dims[q] = an2.dim[q];
    a = an2.p;
    tp.it.push_back(I);
  }
  // trace = ein"ijij -> "(a)[]; lnZ += log(trace)/2^niter   (:27-28)
  TNAD_REQUIRE(dims[0] == dims[2] && dims[1] == dims[3], TNAD_ERR_SHAPE, "trg: final tensor is not ijij-traceable");
  k_trace_ijij<<<1, 32, 0, c->stream>>>(a, dims[0], dims[1], c->d_red);
  count_launch(c);
  TNAD_CK(cudaMemcpyAsync(c->h_pin, c->d_red, 8, cudaMemcpyDeviceToHost, c->stream));
  TNAD_CK(cudaStreamSynchronize(c->stream));
  tp.trace = c->h_pin[0];
  lnZ += std::log(tp.trace) / std::pow(2.0, niter);
  tp.afin = a;
  for (int q = 0; q < 4; ++q) tp.fdims[q] = dims[q];
  tp.lnZ = lnZ;
  TNAD_REQUIRE(std::isfinite(lnZ), TNAD_ERR_NONFINITE, "trg: non-finite lnZ");
}

void trg_bwd(tnad_ctx* c, TrgTape& tp, double dlnZ, double* da_out) {
  WsScope scope(c);
  int64_t nfin = tp.fdims[0] * tp.fdims[1] * tp.fdims[2] * tp.fdims[3];
  double* ga = ws_d(c, nfin);
  fill(c, ga, nfin, 0.0);
  k_trace_bwd<<<nb(tp.fdims[0] * tp.fdims[1]), 256, 0, c->stream>>>(ga, tp.fdims[0], tp.fdims[1],
                                                                     dlnZ / (std::pow(2.0, tp.niter) * tp.trace));
  count_launch(c);
  for (int it = tp.niter; it >= 1; --it) {
    TrgIter& I = tp.it[it - 1];
    const int64_t* dm = I.dims;
    int64_t na = dm[0] * dm[1] * dm[2] * dm[3];
    Ten dr = make_ten(I.s1.u, {I.s1.dims[0], I.s1.dims[1], I.s1.k});
    Ten ul = make_ten(I.s1.v, {I.s1.k, I.s1.dims[2], I.s1.dims[3]});
    Ten ld = make_ten(I.s2.u, {I.s2.dims[0], I.s2.dims[1], I.s2.k});
    Ten ru = make_ten(I.s2.v, {I.s2.k, I.s2.dims[2], I.s2.dims[3]});
    Ten gA = make_ten(ga, {I.s1.k, I.s2.k, I.s1.k, I.s2.k});
    Ten gx = make_ten(ws_d(c, I.x.numel()), {});
    Ten gy = make_ten(ws_d(c, I.y.numel()), {});
    contract(c, TNAD_PREC_FP64, gA, "urdl", I.y, "doln", gx, "nuor");
    contract(c, TNAD_PREC_FP64, I.x, "nuor", gA, "urdl", gy, "doln");
    Ten gdr = make_ten(ws_d(c, dr.numel()), {});
    Ten gld = make_ten(ws_d(c, ld.numel()), {});
    Ten gul = make_ten(ws_d(c, ul.numel()), {});
    Ten gru = make_ten(ws_d(c, ru.numel()), {});
    contract(c, TNAD_PREC_FP64, gx, "nuor", ld, "por", gdr, "npu");
    contract(c, TNAD_PREC_FP64, dr, "npu", gx, "nuor", gld, "por");
    contract(c, TNAD_PREC_FP64, gy, "doln", ru, "lmn", gul, "dom");
    contract(c, TNAD_PREC_FP64, ul, "dom", gy, "doln", gru, "lmn");
    double* gdrul = ws_d(c, na);
    double* gldru = ws_d(c, na);
    trg_svd_bwd(c, I.s1, gdr.p, gul.p, gdrul);
    trg_svd_bwd(c, I.s2, gld.p, gru.p, gldru);
    // back through the two permutations (both are involutions)
    double* gan = ws_d(c, na);
    const int p1[4] = {2, 1, 0, 3}, p2[4] = {3, 2, 1, 0};
    Ten t1 = make_ten(gdrul, {I.s1.dims[0], I.s1.dims[1], I.s1.dims[2], I.s1.dims[3]});
    Ten t2 = make_ten(gldru, {I.s2.dims[0], I.s2.dims[1], I.s2.dims[2], I.s2.dims[3]});
    permute(c, t1, p1, gan);
    permute(c, t2, p2, gan, 1.0, 1.0);
    // back through a /= maxval ; lnZ += 2^(1-n) log(maxval) (gradient of maximum goes to the first argmax)
    double* dot = ws_d(c, 1);
    dot_dev(c, gan, I.araw, na, dot);
    double extra = dlnZ * std::pow(2.0, 1 - it) / I.mv;
    double* graw = ws_d(c, na);
    k_maxnorm_bwd<<<nb(na), 256, 0, c->stream>>>(na, gan, I.mv, I.araw, I.idx, dot, extra, graw);
    count_launch(c);
    ga = graw;
  }
  copy_d2d(c, da_out, ga, tp.it.empty() ? nfin : tp.it[0].dims[0] * tp.it[0].dims[1] * tp.it[0].dims[2] * tp.it[0].dims[3]);
}

}  // namespace tnad
