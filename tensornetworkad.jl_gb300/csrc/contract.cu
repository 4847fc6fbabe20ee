// Pairwise tensor contraction on the device: the role OMEinsum's ein"..." plays
// in the reference (e.g. src/ctmrg.jl:130-140, src/variationalipeps.jl:52).
// A contraction is mapped to one GEMM: free labels of A become the rows, free
// labels of B the columns, shared labels the inner dimension.  Operands whose
// memory order already matches a (transposed) matrix view are used in place;
// otherwise one permutation kernel packs them.  The output is permuted only
// when the requested label order interleaves A's and B's free labels.
#include <cstring>
#include <string>

#include "tnad_internal.h"

namespace tnad {

static int find_label(const char* s, char ch) {
  for (int i = 0; s[i]; ++i)
    if (s[i] == ch) return i;
  return -1;
}

Ten contract_shape(const Ten& A, const char* la, const Ten& B, const char* lb, const char* lc) {
  Ten C;
  C.nd = (int)strlen(lc);
  for (int k = 0; k < C.nd; ++k) {
    int ia = find_label(la, lc[k]);
    int ib = find_label(lb, lc[k]);
    TNAD_REQUIRE(ia >= 0 || ib >= 0, TNAD_ERR_ARG, std::string("contract: output label not in inputs: ") + lc);
    C.dim[k] = ia >= 0 ? A.dim[ia] : B.dim[ib];
  }
  return C;
}

// Is `have` (labels in memory order) equal to the concatenation x+y ?
static bool is_concat(const std::string& have, const std::string& x, const std::string& y) { return have == x + y; }

static void perm_to(tnad_ctx* c, const Ten& T, const std::string& have, const std::string& want, double* out) {
  int perm[10];
  for (size_t k = 0; k < want.size(); ++k) perm[k] = (int)have.find(want[k]);
  permute(c, T, perm, out);
}

void contract(tnad_ctx* c, int prec, const Ten& A0, const char* la0, const Ten& B0, const char* lb0, Ten& C,
              const char* lc0, double alpha, double beta) {
  TNAD_REQUIRE((int)strlen(la0) == A0.nd && (int)strlen(lb0) == B0.nd, TNAD_ERR_ARG,
               std::string("contract: label/rank mismatch ") + la0 + "," + lb0);
  std::string la = la0, lb = lb0, lc = lc0;
  // shape check of shared labels
  for (size_t i = 0; i < la.size(); ++i) {
    int j = find_label(lb0, la[i]);
    if (j >= 0)
      TNAD_REQUIRE(A0.dim[i] == B0.dim[j], TNAD_ERR_SHAPE,
                   std::string("contract: dimension mismatch on label ") + la[i] + " in " + la0 + "," + lb0);
  }
  Ten shp = contract_shape(A0, la0, B0, lb0, lc0);
  C.nd = shp.nd;
  for (int k = 0; k < C.nd; ++k) C.dim[k] = shp.dim[k];
  for (char ch : la)
    TNAD_REQUIRE(lb.find(ch) != std::string::npos || lc.find(ch) != std::string::npos, TNAD_ERR_ARG,
                 "contract: summed-out label only in A (use a reduction)");
  for (char ch : lb)
    TNAD_REQUIRE(la.find(ch) != std::string::npos || lc.find(ch) != std::string::npos, TNAD_ERR_ARG,
                 "contract: summed-out label only in B (use a reduction)");
  for (char ch : lc)
    TNAD_REQUIRE(!(la.find(ch) != std::string::npos && lb.find(ch) != std::string::npos), TNAD_ERR_ARG,
                 "contract: batch labels are not supported");

  // Put the operand owning the first output label first.
  const Ten* A = &A0;
  const Ten* B = &B0;
  if (!lc.empty() && la.find(lc[0]) == std::string::npos) {
    std::swap(A, B);
    std::swap(la, lb);
  }
  std::string Ml, Nl, Kl;
  for (char ch : lc) (la.find(ch) != std::string::npos ? Ml : Nl) += ch;
  const Ten* big = A->numel() >= B->numel() ? A : B;
  const std::string& lbig = (big == A) ? la : lb;
  for (char ch : lbig)
    if (la.find(ch) != std::string::npos && lb.find(ch) != std::string::npos) Kl += ch;

  auto dims_of = [&](const Ten* T, const std::string& lab, const std::string& sel) {
    int64_t p = 1;
    for (char ch : sel) p *= T->dim[lab.find(ch)];
    return p;
  };
  int64_t M = dims_of(A, la, Ml), N = dims_of(B, lb, Nl), K = dims_of(A, la, Kl);

  WsScope scope(c);
  const double* Ap = A->p;
  char ta = 'N';
  int64_t lda = M > 0 ? M : 1;
  if (is_concat(la, Ml, Kl)) {
    ta = 'N';
    lda = M;
  } else if (is_concat(la, Kl, Ml)) {
    ta = 'T';
    lda = K;
  } else {
    double* t = ws_d(c, A->numel());
    perm_to(c, *A, la, Ml + Kl, t);
    Ap = t;
  }
  const double* Bp = B->p;
  char tb = 'N';
  int64_t ldb = K;
  if (is_concat(lb, Kl, Nl)) {
    tb = 'N';
    ldb = K;
  } else if (is_concat(lb, Nl, Kl)) {
    tb = 'T';
    ldb = N;
  } else {
    double* t = ws_d(c, B->numel());
    perm_to(c, *B, lb, Kl + Nl, t);
    Bp = t;
  }
  if (lda < 1) lda = 1;
  if (ldb < 1) ldb = 1;
  if (lc == Ml + Nl) {
    gemm(c, prec, ta, tb, M, N, K, alpha, Ap, lda, Bp, ldb, beta, C.p, M > 0 ? M : 1);
  } else {
    double* t = ws_d(c, M * N);
    gemm(c, prec, ta, tb, M, N, K, 1.0, Ap, lda, Bp, ldb, 0.0, t, M > 0 ? M : 1);
    Ten T;
    T.p = t;
    std::string have = Ml + Nl;
    T.nd = (int)have.size();
    for (int k = 0; k < T.nd; ++k) {
      char ch = have[k];
      size_t ia = la.find(ch);
      T.dim[k] = ia != std::string::npos ? A->dim[ia] : B->dim[lb.find(ch)];
    }
    int perm[10];
    for (size_t k = 0; k < lc.size(); ++k) perm[k] = (int)have.find(lc[k]);
    permute(c, T, perm, C.p, alpha, beta);
  }
}

}  // namespace tnad
