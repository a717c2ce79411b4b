// complex64 GEMM dispatch for the mixed-precision path.
#include "bemgpu_internal.h"

int bem_cgemm(bemgpu_ctx_s *ctx, int kind, char opA, int m, int n, int k, const float alpha[2], const float *A,
              int64_t lda, const float *B, int64_t ldb, const float beta[2], float *C, int64_t ldc,
              cudaStream_t stream) {
  return bem_cgemm_fma(ctx, kind, opA, m, n, k, alpha, A, lda, B, ldb, beta, C, ldc, stream);
}
