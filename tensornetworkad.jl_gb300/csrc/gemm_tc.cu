// placeholder: replaced by the tcgen05 kernel
#include "tnad_internal.h"
namespace tnad {
void gemm_tf32x3(tnad_ctx* c, char ta, char tb, int64_t M, int64_t N, int64_t K, double alpha, const double* A,
                 int64_t lda, const double* B, int64_t ldb, double beta, double* C, int64_t ldc) {
  fail(TNAD_ERR_STATE, "tf32x3 GEMM not built");
}
}  // namespace tnad
