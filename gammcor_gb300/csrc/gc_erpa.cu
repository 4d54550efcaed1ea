// ERPA eigenproblem A+ A- Y = omega^2 Y.
//
// GC_ERPA_SYMM1 follows ERPASYMM1 (interpa.f:1652-1781): symmetrise A+-,
// A+^1/2 = V diag(sqrt|e|) V^T from eig(A+), eig(A+^1/2 A- A+^1/2) -> omega^2, Z,
// Y = A+^1/2 Z, normalise 2/omega Y^T A- Y = 1 for omega^2 > 1e-6.
//
// GC_ERPA_CHOLESKY factors A+ = L L^T instead of taking its square root:
// L^T A- L is similar to A+^1/2 A- A+^1/2 (same omega^2), and Y = L u / sqrt(2 omega)
// satisfies the same eigen-equation and normalisation, so W(lambda), which depends
// on Y only through Y Y^T over kept modes, is unchanged. One eigensolve instead of two.
#include "gc_internal.cuh"
#include "gc_tc_gemm.cuh"

namespace {

const double kSmall = 1e-6;  // interpa.f:1664

__global__ void k_symmetrize(int N, double *__restrict__ a) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  int j = blockIdx.y * blockDim.y + threadIdx.y;
  if (i >= N || j >= N || j <= i) return;
  size_t u = i + (size_t)j * N, l = j + (size_t)i * N;
  double v = 0.5 * (a[u] + a[l]);
  a[u] = v;
  a[l] = v;
}

// Copy the upper triangle onto the lower one.
__global__ void k_mirror_upper(int N, double *__restrict__ a) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  int j = blockIdx.y * blockDim.y + threadIdx.y;
  if (i >= N || j >= N || j <= i) return;
  a[j + (size_t)i * N] = a[i + (size_t)j * N];
}

__global__ void k_zero_upper(int N, double *__restrict__ a) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  int j = blockIdx.y * blockDim.y + threadIdx.y;
  if (i >= N || j >= N || j <= i) return;
  a[i + (size_t)j * N] = 0.0;
}

// out(:, k) = V(:, k) * sqrt(|e_k|)
__global__ void k_scale_cols_sqrt_abs(int N, const double *__restrict__ V,
                                      const double *__restrict__ e, double *__restrict__ out) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  int k = blockIdx.y;
  if (i >= N) return;
  out[i + (size_t)k * N] = V[i + (size_t)k * N] * sqrt(fabs(e[k]));
}

// ERPASYMM1 normalisation: for omega^2 > Small, omega = sqrt, s = 2/omega y^T (A- y),
// y *= 1/sqrt(s) (0 if s <= 0). T = A- Y. One block per column.
__global__ void k_norm_symm1(int N, double *__restrict__ Y, const double *__restrict__ T,
                             double *__restrict__ eig) {
  int nu = blockIdx.x;
  __shared__ double red[256];
  double w2 = eig[nu];
  if (!(w2 > kSmall)) return;  // uniform per block
  double s = 0.0;
  const double *y = Y + (size_t)nu * N, *t = T + (size_t)nu * N;
  for (int i = threadIdx.x; i < N; i += blockDim.x) s += y[i] * t[i];
  red[threadIdx.x] = s;
  __syncthreads();
  for (int w = blockDim.x / 2; w > 0; w >>= 1) {
    if (threadIdx.x < w) red[threadIdx.x] += red[threadIdx.x + w];
    __syncthreads();
  }
  double om = sqrt(w2);
  double sum = 2.0 / om * red[0];
  double f = sum > 0.0 ? 1.0 / sqrt(sum) : 0.0;
  for (int i = threadIdx.x; i < N; i += blockDim.x) Y[(size_t)nu * N + i] *= f;
  __syncthreads();
  if (threadIdx.x == 0) eig[nu] = om;
}

// Cholesky form: y_nu = L u_nu / sqrt(2 omega) for omega^2 > Small.
__global__ void k_norm_chol(int N, double *__restrict__ Y, double *__restrict__ eig) {
  int nu = blockIdx.y;
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  double w2 = eig[nu];
  if (!(w2 > kSmall)) return;
  double om = sqrt(w2);
  if (i < N) Y[(size_t)nu * N + i] *= 1.0 / sqrt(2.0 * om);
}

__global__ void k_sqrt_eig(int N, double *__restrict__ eig) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < N && eig[i] > kSmall) eig[i] = sqrt(eig[i]);
}

int syevd(gc_context *ctx, int N, double *A, double *w) {
  int lwork = 0;
  GC_CUSOLVER(ctx, cusolverDnDsyevd_bufferSize(ctx->cusolver, CUSOLVER_EIG_MODE_VECTOR,
                                               CUBLAS_FILL_MODE_LOWER, N, A, N, w, &lwork));
  gc::DevBuf<double> work;
  GC_TRY(work.alloc(ctx, std::max(lwork, 1)));
  GC_CUSOLVER(ctx, cusolverDnDsyevd(ctx->cusolver, CUSOLVER_EIG_MODE_VECTOR, CUBLAS_FILL_MODE_LOWER,
                                    N, A, N, w, work.p, lwork, ctx->dev_info));
  int info = 0;
  GC_CUDA(ctx, cudaMemcpyAsync(&info, ctx->dev_info, sizeof(int), cudaMemcpyDeviceToHost,
                               ctx->stream));
  GC_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
  if (info != 0) return gc::set_error(ctx, GC_ECUSOLVER, "dsyevd info=%d (N=%d)", info, N);
  return GC_OK;
}

}  // namespace

namespace gc {

int erpa_solve(gc_context *ctx, int N, double *abplus, double *abmin, double *Y, double *eig,
               int mode, int gemm_precision) {
  if (N <= 0 || !abplus || !abmin || !Y || !eig)
    return set_error(ctx, GC_EINVAL, "erpa: bad arguments N=%d", N);
  dim3 b2(32, 8), g2(ceil_div(N, 32), ceil_div(N, 8));
  k_symmetrize<<<g2, b2, 0, ctx->stream>>>(N, abplus);
  GC_LAUNCHED(ctx);
  k_symmetrize<<<g2, b2, 0, ctx->stream>>>(N, abmin);
  GC_LAUNCHED(ctx);
  const double one = 1.0, zero = 0.0;
  const size_t NN = (size_t)N * N;
  if (mode == GC_ERPA_SYMM1) {
    DevBuf<double> V, P, H;
    GC_TRY(V.alloc(ctx, NN));
    GC_TRY(P.alloc(ctx, NN));
    GC_TRY(H.alloc(ctx, NN));
    GC_CUDA(ctx, cudaMemcpyAsync(V.p, abplus, NN * sizeof(double), cudaMemcpyDeviceToDevice,
                                 ctx->stream));
    GC_TRY(syevd(ctx, N, V.p, eig));
    k_scale_cols_sqrt_abs<<<dim3(ceil_div(N, 256), N), 256, 0, ctx->stream>>>(N, V.p, eig, H.p);
    GC_LAUNCHED(ctx);
    // P = (V diag(sqrt|e|)) V^T, made exactly symmetric from its upper triangle
    GC_CUBLAS(ctx, cublasDgemm(ctx->cublas, CUBLAS_OP_N, CUBLAS_OP_T, N, N, N, &one, H.p, N, V.p, N,
                               &zero, P.p, N));
    k_mirror_upper<<<g2, b2, 0, ctx->stream>>>(N, P.p);
    GC_LAUNCHED(ctx);
    // H = A- P ; V = P H
    GC_CUBLAS(ctx, cublasDgemm(ctx->cublas, CUBLAS_OP_N, CUBLAS_OP_N, N, N, N, &one, abmin, N, P.p,
                               N, &zero, H.p, N));
    GC_CUBLAS(ctx, cublasDgemm(ctx->cublas, CUBLAS_OP_N, CUBLAS_OP_N, N, N, N, &one, P.p, N, H.p, N,
                               &zero, V.p, N));
    GC_TRY(syevd(ctx, N, V.p, eig));
    // Y = P Z ; T = A- Y
    GC_CUBLAS(ctx, cublasDgemm(ctx->cublas, CUBLAS_OP_N, CUBLAS_OP_N, N, N, N, &one, P.p, N, V.p, N,
                               &zero, Y, N));
    GC_CUBLAS(ctx, cublasDgemm(ctx->cublas, CUBLAS_OP_N, CUBLAS_OP_N, N, N, N, &one, abmin, N, Y, N,
                               &zero, H.p, N));
    k_norm_symm1<<<N, 256, 0, ctx->stream>>>(N, Y, H.p, eig);
    GC_LAUNCHED(ctx);
    return GC_OK;
  }
  if (mode == GC_ERPA_CHOLESKY) {
    DevBuf<double> L, M;
    GC_TRY(L.alloc(ctx, NN));
    GC_TRY(M.alloc(ctx, NN));
    GC_CUDA(ctx, cudaMemcpyAsync(L.p, abplus, NN * sizeof(double), cudaMemcpyDeviceToDevice,
                                 ctx->stream));
    int lwork = 0;
    GC_CUSOLVER(ctx, cusolverDnDpotrf_bufferSize(ctx->cusolver, CUBLAS_FILL_MODE_LOWER, N, L.p, N,
                                                 &lwork));
    {
      DevBuf<double> work;
      GC_TRY(work.alloc(ctx, std::max(lwork, 1)));
      GC_CUSOLVER(ctx, cusolverDnDpotrf(ctx->cusolver, CUBLAS_FILL_MODE_LOWER, N, L.p, N, work.p,
                                        lwork, ctx->dev_info));
      int info = 0;
      GC_CUDA(ctx, cudaMemcpyAsync(&info, ctx->dev_info, sizeof(int), cudaMemcpyDeviceToHost,
                                   ctx->stream));
      GC_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
      if (info > 0)
        return set_error(ctx, GC_ENOTPD, "A+B is not positive definite (potrf minor %d)", info);
      if (info < 0) return set_error(ctx, GC_ECUSOLVER, "potrf info=%d", info);
    }
    k_zero_upper<<<g2, b2, 0, ctx->stream>>>(N, L.p);
    GC_LAUNCHED(ctx);
    const bool tc = gemm_precision == GC_PREC_FP64TC5 || gemm_precision == GC_PREC_FP64TC6;
    if (tc) {
      // T = A- L (into Y as scratch); M = L^T T; after the eigensolve Y = L U.
      // Products of the FP64-accurate sliced tensor-core GEMM (L has a zero upper triangle).
      GC_TRY(tc_gemm_strided(ctx, gemm_precision, N, N, N, abmin, 1, N, L.p, N, 1, Y, N));
      GC_TRY(tc_gemm_strided(ctx, gemm_precision, N, N, N, L.p, N, 1, Y, N, 1, M.p, N));
      k_symmetrize<<<g2, b2, 0, ctx->stream>>>(N, M.p);
      GC_LAUNCHED(ctx);
      GC_TRY(syevd(ctx, N, M.p, eig));
      GC_TRY(tc_gemm_strided(ctx, gemm_precision, N, N, N, L.p, 1, N, M.p, N, 1, Y, N));
    } else {
      // M = A- L (into Y as scratch), then M = L^T (A- L)
      GC_CUBLAS(ctx, cublasDtrmm(ctx->cublas, CUBLAS_SIDE_RIGHT, CUBLAS_FILL_MODE_LOWER, CUBLAS_OP_N,
                                 CUBLAS_DIAG_NON_UNIT, N, N, &one, L.p, N, abmin, N, Y, N));
      GC_CUBLAS(ctx, cublasDtrmm(ctx->cublas, CUBLAS_SIDE_LEFT, CUBLAS_FILL_MODE_LOWER, CUBLAS_OP_T,
                                 CUBLAS_DIAG_NON_UNIT, N, N, &one, L.p, N, Y, N, M.p, N));
      GC_TRY(syevd(ctx, N, M.p, eig));
      // Y = L U
      GC_CUBLAS(ctx, cublasDtrmm(ctx->cublas, CUBLAS_SIDE_LEFT, CUBLAS_FILL_MODE_LOWER, CUBLAS_OP_N,
                                 CUBLAS_DIAG_NON_UNIT, N, N, &one, L.p, N, M.p, N, Y, N));
    }
    k_norm_chol<<<dim3(ceil_div(N, 256), N), 256, 0, ctx->stream>>>(N, Y, eig);
    GC_LAUNCHED(ctx);
    k_sqrt_eig<<<ceil_div(N, 256), 256, 0, ctx->stream>>>(N, eig);
    GC_LAUNCHED(ctx);
    return GC_OK;
  }
  return set_error(ctx, GC_EINVAL, "erpa: unknown mode %d", mode);
}

}  // namespace gc

extern "C" int gc_erpa(gc_context *ctx, int ndimx, double *abplus, double *abmin, double *eigvec,
                       double *eig, int mode) {
  if (!ctx) return GC_EINVAL;
  return gc::erpa_solve(ctx, ndimx, abplus, abmin, eigvec, eig, mode, GC_PREC_FP64);
}
