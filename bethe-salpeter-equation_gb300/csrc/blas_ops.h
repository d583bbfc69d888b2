// cuBLAS BLAS-3 calls on complex64 / complex128 data, overloaded on the element type so the
// eigensolver templates call one name for both precisions.
#pragma once

#include <cublas_v2.h>
#include <cuda_runtime.h>

namespace bse {

inline cublasStatus_t xhemm(cublasHandle_t h, int m, int n, const float2* al, const float2* A, int lda, const float2* B,
                            int ldb, const float2* be, float2* C, int ldc) {
    return cublasChemm(h, CUBLAS_SIDE_LEFT, CUBLAS_FILL_MODE_LOWER, m, n, al, A, lda, B, ldb, be, C, ldc);
}
inline cublasStatus_t xhemm(cublasHandle_t h, int m, int n, const double2* al, const double2* A, int lda,
                            const double2* B, int ldb, const double2* be, double2* C, int ldc) {
    return cublasZhemm(h, CUBLAS_SIDE_LEFT, CUBLAS_FILL_MODE_LOWER, m, n, al, A, lda, B, ldb, be, C, ldc);
}
inline cublasStatus_t xtrmm(cublasHandle_t h, cublasSideMode_t side, cublasOperation_t op, int m, int n,
                            const float2* al, const float2* T, int ldt, const float2* B, int ldb, float2* C, int ldc) {
    return cublasCtrmm(h, side, CUBLAS_FILL_MODE_UPPER, op, CUBLAS_DIAG_NON_UNIT, m, n, al, T, ldt, B, ldb, C, ldc);
}
inline cublasStatus_t xtrmm(cublasHandle_t h, cublasSideMode_t side, cublasOperation_t op, int m, int n,
                            const double2* al, const double2* T, int ldt, const double2* B, int ldb, double2* C,
                            int ldc) {
    return cublasZtrmm(h, side, CUBLAS_FILL_MODE_UPPER, op, CUBLAS_DIAG_NON_UNIT, m, n, al, T, ldt, B, ldb, C, ldc);
}
inline cublasStatus_t xgemm(cublasHandle_t h, cublasOperation_t ta, cublasOperation_t tb, int m, int n, int k,
                            const float2* al, const float2* A, int lda, const float2* B, int ldb, const float2* be,
                            float2* C, int ldc) {
    return cublasCgemm(h, ta, tb, m, n, k, al, A, lda, B, ldb, be, C, ldc);
}
inline cublasStatus_t xgemm(cublasHandle_t h, cublasOperation_t ta, cublasOperation_t tb, int m, int n, int k,
                            const double2* al, const double2* A, int lda, const double2* B, int ldb,
                            const double2* be, double2* C, int ldc) {
    return cublasZgemm(h, ta, tb, m, n, k, al, A, lda, B, ldb, be, C, ldc);
}
inline cublasStatus_t xher2k(cublasHandle_t h, int n, int k, const float2* al, const float2* A, int lda,
                             const float2* B, int ldb, const float* be, float2* C, int ldc) {
    return cublasCher2k(h, CUBLAS_FILL_MODE_LOWER, CUBLAS_OP_N, n, k, al, A, lda, B, ldb, be, C, ldc);
}
inline cublasStatus_t xher2k(cublasHandle_t h, int n, int k, const double2* al, const double2* A, int lda,
                             const double2* B, int ldb, const double* be, double2* C, int ldc) {
    return cublasZher2k(h, CUBLAS_FILL_MODE_LOWER, CUBLAS_OP_N, n, k, al, A, lda, B, ldb, be, C, ldc);
}

// B <- U^{-1} B, U upper triangular (left side, no transpose, non-unit diagonal)
inline cublasStatus_t xtrsm_lu(cublasHandle_t h, int m, int n, const float2* U, int ldu, float2* B, int ldb) {
    const float2 one = make_float2(1.f, 0.f);
    return cublasCtrsm(h, CUBLAS_SIDE_LEFT, CUBLAS_FILL_MODE_UPPER, CUBLAS_OP_N, CUBLAS_DIAG_NON_UNIT, m, n, &one, U, ldu, B, ldb);
}
inline cublasStatus_t xtrsm_lu(cublasHandle_t h, int m, int n, const double2* U, int ldu, double2* B, int ldb) {
    const double2 one = make_double2(1.0, 0.0);
    return cublasZtrsm(h, CUBLAS_SIDE_LEFT, CUBLAS_FILL_MODE_UPPER, CUBLAS_OP_N, CUBLAS_DIAG_NON_UNIT, m, n, &one, U, ldu, B, ldb);
}
inline cublasStatus_t xherk(cublasHandle_t h, int n, int k, const float2* A, int lda, float2* C, int ldc) {
    const float one = 1.0f, zero = 0.0f;
    return cublasCherk(h, CUBLAS_FILL_MODE_UPPER, CUBLAS_OP_C, n, k, &one, A, lda, &zero, C, ldc);
}
inline cublasStatus_t xherk(cublasHandle_t h, int n, int k, const double2* A, int lda, double2* C, int ldc) {
    const double one = 1.0, zero = 0.0;
    return cublasZherk(h, CUBLAS_FILL_MODE_UPPER, CUBLAS_OP_C, n, k, &one, A, lda, &zero, C, ldc);
}

}  // namespace bse
