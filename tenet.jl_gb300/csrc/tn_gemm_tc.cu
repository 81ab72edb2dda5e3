// K2 (mixed) — split-precision complex GEMM for ComplexF64 data.
//
// Placeholder translation unit: the tcgen05/TMEM kernel is added here.  Until then the
// mixed-precision GEMM entry point reports that it is not available, so nothing silently
// changes precision.
#include "tn_internal.cuh"

tn_status_t gemm_mixed_c64(tn_ctx* ctx, char opa, char opb, int64_t m, int64_t n, int64_t k, cxd alpha, const cxd* A,
                           int64_t lda, int64_t sA, const cxd* B, int64_t ldb, int64_t sB, cxd beta, cxd* C,
                           int64_t ldc, int64_t sC, int64_t batch) {
  (void)opa; (void)opb; (void)m; (void)n; (void)k; (void)alpha; (void)A; (void)lda; (void)sA; (void)B; (void)ldb;
  (void)sB; (void)beta; (void)C; (void)ldc; (void)sC; (void)batch;
  return tn_set_error(ctx, TN_EUNSUPPORTED, "mixed-precision GEMM is not built yet");
}
