// GEMM dispatch for the transform and the integrand.
#include "gc_tc_gemm.cuh"

namespace gc {

int tc_two_sided(gc_context *ctx, int precision, int n, int cnt, const double *M, int nX,
                 const double *CX, int nY, const double *CY, double *T1, double *out,
                 long long ostride) {
  if (precision == GC_PREC_FP64)
    return fp64_two_sided(ctx, n, cnt, M, nX, CX, nY, CY, T1, out, ostride);
  return set_error(ctx, GC_EUNSUPPORTED, "two_sided: precision %d not built", precision);
}

int tc_gemm_nt(gc_context *ctx, int precision, int m, int n, int k, const double *A, int lda,
               const double *B, int ldb, double *C, int ldc) {
  if (precision == GC_PREC_FP64) {
    const double one = 1.0, zero = 0.0;
    GC_CUBLAS(ctx, cublasDgemm(ctx->cublas, CUBLAS_OP_N, CUBLAS_OP_T, m, n, k, &one, A, lda, B, ldb,
                               &zero, C, ldc));
    return GC_OK;
  }
  return set_error(ctx, GC_EUNSUPPORTED, "gemm_nt: precision %d not built", precision);
}

}  // namespace gc
