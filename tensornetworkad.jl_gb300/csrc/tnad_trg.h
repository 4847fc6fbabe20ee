// TRG driver state shared by trg.cu and the C ABI.
#pragma once

#include "tnad_drivers.h"

namespace tnad {

struct TrgSvd {
  int64_t dims[4] = {0, 0, 0, 0};  // t: d1×d2×d3×d4
  int64_t m = 0, n = 0, ns = 0, k = 0;
  double *U = nullptr, *S = nullptr, *V = nullptr;  // thin SVD of reshape(t, d1d2, d3d4)
  double *u = nullptr, *v = nullptr;                // u: d1×d2×k, v: k×d3×d4
};

struct TrgIter {
  int64_t dims[4] = {0, 0, 0, 0};  // dims of the incoming tensor
  double* araw = nullptr;          // incoming tensor before max-normalisation
  double mv = 1.0;                 // maximum(abs.(a))
  int64_t idx = 0;                 // first argmax
  TrgSvd s1, s2;                   // splits of drul and ldru
  Ten x, y;                        // pairwise intermediates of the contraction
};

struct TrgTape {
  int niter = 0, chi = 0;
  DevPool pool;
  std::vector<TrgIter> it;
  double* afin = nullptr;
  int64_t fdims[4] = {0, 0, 0, 0};
  double trace = 0.0, lnZ = 0.0;
};

void trg_svd_fwd(tnad_ctx* c, const double* t, const int64_t dd[4], int chi, double tol, TrgSvd& s, DevPool* pool);
void trg_svd_bwd(tnad_ctx* c, const TrgSvd& s, const double* du, const double* dv, double* dt);
void trg_fwd(tnad_ctx* c, TrgTape& tp, const double* a0, int d, int chi, int niter, double tol);
void trg_bwd(tnad_ctx* c, TrgTape& tp, double dlnZ, double* da);

}  // namespace tnad
