// GEMM building blocks of the transform and the integrand, dispatched on
// gc_precision: FP64 uses cuBLAS DGEMM; BF16X3 / BF16X6 run the split-precision
// tcgen05 kernel of gc_tc_gemm.cu.
#pragma once
#include "gc_internal.cuh"

namespace gc {

// Reads and clears the context's device flag (a bounded wait of a tensor-core
// GEMM expired): GC_ETIMEOUT if it was set. Synchronises the context's stream.
// The GEMM wrappers below do not synchronise; their callers read the flag at
// their next synchronisation point.
int check_flag(gc_context *ctx);

// out_k (nX x nY, column-major, stride ostride) = CX^T M_k CY for cnt
// column-major n x n matrices M_k; T1 is scratch of cnt*n*max(nX) doubles.
int tc_two_sided(gc_context *ctx, int precision, int n, int cnt, const double *M, int nX,
                 const double *CX, int nY, const double *CY, double *T1, double *out,
                 long long ostride);

// C (m x n, column-major, ldc) = A (m x k, lda) . B (n x k, ldb)^T.
int tc_gemm_nt(gc_context *ctx, int precision, int m, int n, int k, const double *A, int lda,
               const double *B, int ldb, double *C, int ldc);

// result = sum_{i,nu} (Ksym Y)[i,nu] * Y[i,nu] for a symmetric N x N Ksym and
// an N x N Y (both column-major), with the product on tensor cores.
int tc_dot_gemm(gc_context *ctx, int precision, int N, const double *Ksym, const double *Y,
                double *result);

// C[m + n*ldc] = sum_k A(m,k) B(n,k) with A(m,k) = A[m*sam + k*sak] and
// B(n,k) = B[n*sbn + k*sbk], on the sliced FP64-accurate tensor-core path.
int tc_gemm_strided(gc_context *ctx, int precision, int M, int N, int K, const double *A,
                    long long sam, long long sak, const double *B, long long sbn, long long sbk,
                    double *C, long long ldc);

// As tc_gemm_strided, computing only the tiles of C that reach the lower triangle
// (diagonal included) of each `period`-wide column block; the rest of C is not
// written (for products known to be symmetric in each block).
int tc_gemm_strided_lower(gc_context *ctx, int precision, int M, int N, int K, const double *A,
                          long long sam, long long sak, const double *B, long long sbn,
                          long long sbk, double *C, long long ldc, int period);

// C[m + n*ldc] -= sum_k P(m,k) P(n,k) for m >= n (the lower triangle of an M x M
// C, diagonal included) with P(m,k) = P[m*sm + k*sk], on the sliced path; the
// strict upper triangle of C is not touched. nbatch products, P and C of batch b at
// b*sb from the base pointers.
int tc_syrk_sub_lower(gc_context *ctx, int precision, int M, int K, const double *P, long long sm,
                      long long sk, double *C, long long ldc, int nbatch = 1, long long sb = 0);

int fp64_two_sided(gc_context *ctx, int n, int cnt, const double *M, int nX, const double *CX,
                   int nY, const double *CY, double *T1, double *out, long long ostride);

}  // namespace gc
