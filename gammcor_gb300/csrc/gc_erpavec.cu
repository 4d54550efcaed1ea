// ERPAVEC (interpa.f:962-1070): the ERPA solver of state-averaged (NoSt > 1)
// references, which ACEInteg_FOFO calls instead of ERPASYMM1 (abfofo.f90:3777).
//
// It diagonalises the non-symmetric product A+ A- directly (DGEEV), so it also
// handles an A+B that is not positive definite:
//   1. symmetrise A+-, H = A+ A-, right eigenvectors and eigenvalues of H;
//   2. runs of eigenvalues (in the solver's order) within 1e-8 of the first of
//      the run are degenerate groups (CREATE_SPACE, interpa.f:1119-1150), and each
//      group is orthonormalised by V <- V S^-1/2, S = V^T V (ORTHO_DEGVEC,
//      interpa.f:1153-1205);
//   3. a mode with |Im| > 1e-12 gets omega = 0 and a zero vector;
//   4. for omega^2 > 1e-6: omega = sqrt, s = 2/omega y^T A- y; s < 0 marks a
//      de-excitation (omega -> -omega); y *= 1/sqrt|s|. Any other nonzero
//      eigenvalue gets omega = 0, and a zero eigenvalue keeps 0; both vectors are
//      zeroed.
// Here the eigensolve is cuSOLVER's general FP64 eigensolver (cusolverDnXgeev);
// the product, the group orthonormalisation and the normalisation sums run on
// the device.
#include <cmath>
#include <complex>
#include <vector>

#include "gc_internal.cuh"

namespace {

const double kSmall = 1e-6;        // interpa.f:968
const double kThrDeg = 1e-8;       // CREATE_SPACE, interpa.f:1126
const double kThrImag = 1e-12;     // interpa.f:1006

__global__ void k_sym_avg_vec(int N, double *__restrict__ a) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  int j = blockIdx.y * blockDim.y + threadIdx.y;
  if (i >= N || j >= N || j <= i) return;
  const size_t u = i + (size_t)j * N, l = j + (size_t)i * N;
  const double v = 0.5 * (a[u] + a[l]);
  a[u] = v;
  a[l] = v;
}

// sum[nu] = sum_i Y[i, nu] T[i, nu] (one block per column)
__global__ void k_col_dots(int N, const double *__restrict__ Y, const double *__restrict__ T,
                           double *__restrict__ sum) {
  __shared__ double red[256];
  const double *y = Y + (size_t)blockIdx.x * N, *t = T + (size_t)blockIdx.x * N;
  double s = 0.0;
  for (int i = threadIdx.x; i < N; i += blockDim.x) s += y[i] * t[i];
  red[threadIdx.x] = s;
  __syncthreads();
  for (int w = blockDim.x / 2; w > 0; w >>= 1) {
    if (threadIdx.x < w) red[threadIdx.x] += red[threadIdx.x + w];
    __syncthreads();
  }
  if (threadIdx.x == 0) sum[blockIdx.x] = red[0];
}

// Y[:, nu] *= f[nu]
__global__ void k_scale_cols(int N, double *__restrict__ Y, const double *__restrict__ f) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x, nu = blockIdx.y;
  if (i < N) Y[(size_t)i + (size_t)nu * N] *= f[nu];
}

}  // namespace

namespace gc {

int erpavec(gc_context *ctx, int N, double *abplus, double *abmin, double *Y, double *eig) {
  const size_t NN = (size_t)N * N;
  const dim3 b2(32, 8), g2(ceil_div(N, 32), ceil_div(N, 8));
  k_sym_avg_vec<<<g2, b2, 0, ctx->stream>>>(N, abplus);
  GC_LAUNCHED(ctx);
  k_sym_avg_vec<<<g2, b2, 0, ctx->stream>>>(N, abmin);
  GC_LAUNCHED(ctx);
  DevBuf<double> H, W;
  GC_TRY(H.alloc(ctx, NN));
  GC_TRY(W.alloc(ctx, 2 * (size_t)N));  // complex eigenvalues (re, im)
  const double one = 1.0, zero = 0.0;
  GC_CUBLAS(ctx, cublasDgemm(ctx->cublas, CUBLAS_OP_N, CUBLAS_OP_N, N, N, N, &one, abplus, N,
                             abmin, N, &zero, H.p, N));
  // right eigenvectors of H (Y holds them, LAPACK layout of complex pairs)
  cusolverDnParams_t params = nullptr;
  GC_CUSOLVER(ctx, cusolverDnCreateParams(&params));
  size_t dws = 0, hws = 0;
  cusolverStatus_t st = cusolverDnXgeev_bufferSize(
      ctx->cusolver, params, CUSOLVER_EIG_MODE_NOVECTOR, CUSOLVER_EIG_MODE_VECTOR, N, CUDA_R_64F,
      H.p, N, CUDA_C_64F, W.p, CUDA_R_64F, nullptr, N, CUDA_R_64F, Y, N, CUDA_R_64F, &dws, &hws);
  if (st != CUSOLVER_STATUS_SUCCESS) {
    cusolverDnDestroyParams(params);
    return set_error(ctx, GC_ECUSOLVER, "erpavec: geev buffer size: status %d", (int)st);
  }
  DevBuf<unsigned char> dwork;
  std::vector<unsigned char> hwork(std::max<size_t>(hws, 1));
  int r = dwork.alloc(ctx, std::max<size_t>(dws, 1));
  if (r != GC_OK) {
    cusolverDnDestroyParams(params);
    return r;
  }
  GC_CUDA(ctx, cudaEventRecord(ctx->eig_ev[0], ctx->stream));
  st = cusolverDnXgeev(ctx->cusolver, params, CUSOLVER_EIG_MODE_NOVECTOR, CUSOLVER_EIG_MODE_VECTOR,
                       N, CUDA_R_64F, H.p, N, CUDA_C_64F, W.p, CUDA_R_64F, nullptr, N, CUDA_R_64F,
                       Y, N, CUDA_R_64F, dwork.p, dws, hwork.data(), hws, ctx->dev_info);
  cusolverDnDestroyParams(params);
  GC_CUSOLVER(ctx, st);
  GC_CUDA(ctx, cudaEventRecord(ctx->eig_ev[1], ctx->stream));
  std::vector<double> w(2 * (size_t)N);
  int info = 0;
  GC_CUDA(ctx, cudaMemcpyAsync(w.data(), W.p, w.size() * sizeof(double), cudaMemcpyDeviceToHost,
                               ctx->stream));
  GC_CUDA(ctx, cudaMemcpyAsync(&info, ctx->dev_info, sizeof(int), cudaMemcpyDeviceToHost,
                               ctx->stream));
  GC_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
  {
    float ms = 0.f;
    GC_CUDA(ctx, cudaEventElapsedTime(&ms, ctx->eig_ev[0], ctx->eig_ev[1]));
    ctx->eig_ms += ms;
    ctx->eig_calls++;
  }
  if (info != 0) return set_error(ctx, GC_ECUSOLVER, "erpavec: geev info=%d (N=%d)", info, N);
  H.release();
  std::vector<double> er(N), ei(N);
  for (int k = 0; k < N; ++k) {
    er[k] = w[2 * k];
    ei[k] = w[2 * k + 1];
  }
  // degenerate groups in the solver's order, orthonormalised by S^-1/2
  int start = 0;
  for (int k = 1; k <= N; ++k) {
    if (k < N && std::fabs(er[k] - er[start]) <= kThrDeg) continue;
    const int m = k - start;
    if (m > 1) {
      DevBuf<double> S, Sw, V2, work;
      GC_TRY(S.alloc(ctx, (size_t)m * m));
      GC_TRY(Sw.alloc(ctx, m));
      GC_TRY(V2.alloc(ctx, (size_t)N * m));
      double *Vg = Y + (size_t)start * N;
      GC_CUBLAS(ctx, cublasDgemm(ctx->cublas, CUBLAS_OP_T, CUBLAS_OP_N, m, m, N, &one, Vg, N, Vg,
                                 N, &zero, S.p, m));
      int lw = 0;
      GC_CUSOLVER(ctx, cusolverDnDsyevd_bufferSize(ctx->cusolver, CUSOLVER_EIG_MODE_VECTOR,
                                                   CUBLAS_FILL_MODE_UPPER, m, S.p, m, Sw.p, &lw));
      GC_TRY(work.alloc(ctx, std::max(lw, 1)));
      GC_CUSOLVER(ctx, cusolverDnDsyevd(ctx->cusolver, CUSOLVER_EIG_MODE_VECTOR,
                                        CUBLAS_FILL_MODE_UPPER, m, S.p, m, Sw.p, work.p, lw,
                                        ctx->dev_info));
      std::vector<double> hv((size_t)m * m), hs(m);
      GC_CUDA(ctx, cudaMemcpyAsync(hv.data(), S.p, hv.size() * sizeof(double),
                                   cudaMemcpyDeviceToHost, ctx->stream));
      GC_CUDA(ctx, cudaMemcpyAsync(hs.data(), Sw.p, m * sizeof(double), cudaMemcpyDeviceToHost,
                                   ctx->stream));
      GC_CUDA(ctx, cudaMemcpyAsync(&info, ctx->dev_info, sizeof(int), cudaMemcpyDeviceToHost,
                                   ctx->stream));
      GC_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
      if (info != 0) return set_error(ctx, GC_ECUSOLVER, "erpavec: group Gram eigensolve info=%d", info);
      // S^-1/2 = V diag(1/sqrt s) V^T (m x m, host: at most a few degenerate vectors)
      std::vector<double> smh((size_t)m * m, 0.0);
      for (int a = 0; a < m; ++a)
        for (int b = 0; b < m; ++b) {
          double v = 0.0;
          for (int c = 0; c < m; ++c) v += hv[a + (size_t)c * m] * hv[b + (size_t)c * m] / std::sqrt(hs[c]);
          smh[a + (size_t)b * m] = v;
        }
      GC_CUDA(ctx, cudaMemcpyAsync(S.p, smh.data(), smh.size() * sizeof(double),
                                   cudaMemcpyHostToDevice, ctx->stream));
      GC_CUBLAS(ctx, cublasDgemm(ctx->cublas, CUBLAS_OP_N, CUBLAS_OP_N, N, m, m, &one, Vg, N, S.p, m,
                                 &zero, V2.p, N));
      GC_CUDA(ctx, cudaMemcpyAsync(Vg, V2.p, (size_t)N * m * sizeof(double),
                                   cudaMemcpyDeviceToDevice, ctx->stream));
      GC_CUDA(ctx, cudaStreamSynchronize(ctx->stream));  // smh is host memory
    }
    start = k;
  }
  // complex modes, then the 2/omega y^T A- y normalisation with its sign
  DevBuf<double> T, sums, f;
  GC_TRY(T.alloc(ctx, NN));
  GC_TRY(sums.alloc(ctx, N));
  GC_TRY(f.alloc(ctx, N));
  GC_CUBLAS(ctx, cublasDgemm(ctx->cublas, CUBLAS_OP_N, CUBLAS_OP_N, N, N, N, &one, abmin, N, Y, N,
                             &zero, T.p, N));
  k_col_dots<<<N, 256, 0, ctx->stream>>>(N, Y, T.p, sums.p);
  GC_LAUNCHED(ctx);
  std::vector<double> hsum(N), hf(N), hom(N);
  GC_CUDA(ctx, cudaMemcpyAsync(hsum.data(), sums.p, N * sizeof(double), cudaMemcpyDeviceToHost,
                               ctx->stream));
  GC_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
  for (int k = 0; k < N; ++k) {
    double e = std::fabs(ei[k]) > kThrImag ? 0.0 : er[k];
    double s = 0.0;
    if (e > kSmall) {
      e = std::sqrt(e);
      const double sn = 2.0 / e * hsum[k];
      if (sn < 0.0) e = -e;  // de-excitation
      s = 1.0 / std::sqrt(std::fabs(sn));
    } else if (e != 0.0) {
      e = 0.0;
    }
    hom[k] = e;
    hf[k] = s;
  }
  GC_CUDA(ctx, cudaMemcpyAsync(f.p, hf.data(), N * sizeof(double), cudaMemcpyHostToDevice,
                               ctx->stream));
  GC_CUDA(ctx, cudaMemcpyAsync(eig, hom.data(), N * sizeof(double), cudaMemcpyHostToDevice,
                               ctx->stream));
  k_scale_cols<<<dim3(ceil_div(N, 256), N), 256, 0, ctx->stream>>>(N, Y, f.p);
  GC_LAUNCHED(ctx);
  GC_CUDA(ctx, cudaStreamSynchronize(ctx->stream));  // hf and hom are host memory
  return GC_OK;
}

}  // namespace gc
