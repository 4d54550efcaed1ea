// Frequency-integration AC (ACFREQ): WIter_FOFO (ac_fofo.f90:1-181).
//
// The reference expands C(lambda, omega) = 1/2 (A(lambda) + omega^2)^-1 A+(lambda),
// A(lambda) = A+(lambda) A-(lambda), to third order in lambda at every point of a
// 25-point frequency grid, inverting A0 + omega^2 by LU at every point and
// spending about nine N^3 products per point on the series.
//
// Here the series is carried in the eigenbasis of the lambda = 0 problem. With
// A+0 = L L^T and L^T A-0 L = U W U^T (one Cholesky and one eigensolve), B = L U
// gives A0 = B W B^-1, and every coefficient of the series keeps the form
// C_n = B X_n B^T:
//   X0 = D/2,  X1 = D P/2 - D A1t X0,
//   Xn = -n D A1t X(n-1) - n (n-1) D A2t X(n-2)   (n >= 2),
// with D = diag(1 / (w_i + omega^2)), P = B^-1 A+1 B^-T = U^T L^-1 A+1 L^-T U,
// K = B^T A-1 B, A1t = B^-1 A1 B = K + P W and A2t = B^-1 A2 B = P K (A1, A2 the
// reference's lambda and lambda^2 coefficients of A(lambda)). The frequency sum
// S = sum_omega 4/pi w_omega sum_n X_n / (n! (n + 1)) is accumulated in the
// eigenbasis and COM = B S B^T is formed once. Per frequency that is two GEMMs
// per order above the first (Max_Cn = 3: three GEMMs) and element-wise passes; no
// LU. The GEMMs run in the chosen precision (FP64, or the FP64-accurate sliced
// tensor-core GEMM); the Cholesky, the eigensolve (dsyevd, or FP32 refined to
// FP64 accuracy) and the triangular solves stay FP64.
#include <cmath>
#include <vector>

#include "gc_internal.cuh"
#include "gc_tc_gemm.cuh"

namespace {

// C (m x n) = op(A) op(B), column-major, in the given precision.
int gemm(gc_context *ctx, int prec, bool ta, bool tb, int m, int n, int k, const double *A, int lda,
         const double *B, int ldb, double *C, int ldc) {
  if (gc::is_sliced(prec))
    // A(m, k) = A[m * sam + k * sak]; B(n, k) = B[n * sbn + k * sbk]
    return gc::tc_gemm_strided(ctx, prec, m, n, k, A, ta ? lda : 1, ta ? 1 : lda, B, tb ? 1 : ldb,
                               tb ? ldb : 1, C, ldc);
  const double one = 1.0, zero = 0.0;
  GC_CUBLAS(ctx, cublasDgemm(ctx->cublas, ta ? CUBLAS_OP_T : CUBLAS_OP_N,
                             tb ? CUBLAS_OP_T : CUBLAS_OP_N, m, n, k, &one, A, lda, B, ldb, &zero,
                             C, ldc));
  return GC_OK;
}

// out[i, j] = a * x[i, j] + b * y[i, j] * w[j]   (w may be NULL: 1)
__global__ void k_axpy_colscale(size_t NN, int N, double a, const double *__restrict__ x, double b,
                                const double *__restrict__ y, const double *__restrict__ w,
                                double *__restrict__ out) {
  for (size_t e = blockIdx.x * (size_t)blockDim.x + threadIdx.x; e < NN;
       e += (size_t)gridDim.x * blockDim.x) {
    const int j = (int)(e / N);
    out[e] = a * x[e] + b * y[e] * (w ? w[j] : 1.0);
  }
}

// X1[i, j] = d_i P[i, j] / 2 - d_i A1t[i, j] d_j / 2, d = 1 / (w + om2); S += c1 X1 + c0 D/2
__global__ void k_freq_x1(size_t NN, int N, double om2, const double *__restrict__ w,
                          const double *__restrict__ P, const double *__restrict__ A1t, double c0,
                          double c1, double *__restrict__ X1, double *__restrict__ S) {
  for (size_t e = blockIdx.x * (size_t)blockDim.x + threadIdx.x; e < NN;
       e += (size_t)gridDim.x * blockDim.x) {
    const int j = (int)(e / N), i = (int)(e - (size_t)j * N);
    const double di = 1.0 / (w[i] + om2), dj = 1.0 / (w[j] + om2);
    const double x = 0.5 * di * P[e] - 0.5 * di * A1t[e] * dj;
    X1[e] = x;
    S[e] += c1 * x + (i == j ? c0 * 0.5 * di : 0.0);
  }
}

// Xn[i, j] = -n d_i T1[i, j] - n (n - 1) d_i T2[i, j]; with T2 = NULL the second term is
// -n (n - 1) d_i A2t[i, j] d_j / 2 (A2t X0 with X0 = D/2). S += cn Xn.
__global__ void k_freq_xn(size_t NN, int N, double om2, int nord, const double *__restrict__ w,
                          const double *__restrict__ T1, const double *__restrict__ T2,
                          const double *__restrict__ A2t, double cn, double *__restrict__ Xn,
                          double *__restrict__ S) {
  for (size_t e = blockIdx.x * (size_t)blockDim.x + threadIdx.x; e < NN;
       e += (size_t)gridDim.x * blockDim.x) {
    const int j = (int)(e / N), i = (int)(e - (size_t)j * N);
    const double di = 1.0 / (w[i] + om2);
    const double t2 = T2 ? T2[e] : 0.5 * A2t[e] / (w[j] + om2);
    const double x = -(double)nord * di * T1[e] - (double)nord * (nord - 1) * di * t2;
    Xn[e] = x;
    S[e] += cn * x;
  }
}

// out = x + d I
__global__ void k_add_diag(size_t NN, int N, const double *__restrict__ x, double d,
                           double *__restrict__ out) {
  for (size_t e = blockIdx.x * (size_t)blockDim.x + threadIdx.x; e < NN;
       e += (size_t)gridDim.x * blockDim.x) {
    const int j = (int)(e / N), i = (int)(e - (size_t)j * N);
    out[e] = x[e] + (i == j ? d : 0.0);
  }
}

// out = a x + b y (element-wise)
__global__ void k_lincomb(size_t NN, double a, const double *__restrict__ x, double b,
                          const double *__restrict__ y, double *__restrict__ out) {
  for (size_t e = blockIdx.x * (size_t)blockDim.x + threadIdx.x; e < NN;
       e += (size_t)gridDim.x * blockDim.x)
    out[e] = a * x[e] + (y ? b * y[e] : 0.0);
}

// ECorr partials: sum over pairs i = (p, q), j = (r, s) not in one group of
// [(C_p + C_q)(C_r + C_s) COM[i, j] - delta_ij (n_p (1 - n_q) + n_q (1 - n_p))] (rs|pq)
// (ac_fofo.f90:127-181). One partial per CTA.
__global__ void k_freq_energy(int n, int nocc, int N, const double *__restrict__ com,
                              const int *__restrict__ pp, const int *__restrict__ pq,
                              const double *__restrict__ cpl, const double *__restrict__ dnq,
                              const int *__restrict__ grp, const double *__restrict__ fofo,
                              double *__restrict__ part) {
  __shared__ double red[256];
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  double e = 0.0;
  if (i < N) {
    const int p = pp[i], q = pq[i];
    const double cpq = cpl[i];  // C_p + C_q
    const size_t ld = (size_t)n * nocc;
    for (int j = blockIdx.y; j < N; j += gridDim.y) {
      const int r = pp[j], s = pq[j];
      if (grp[p] == grp[q] && grp[q] == grp[r] && grp[r] == grp[s]) continue;
      double a = cpq * cpl[j] * com[(size_t)i + (size_t)j * N];
      if (i == j) a -= dnq[i];
      e += a * fofo[((size_t)r + (size_t)s * n) * ld + p + (size_t)q * n];  // (rs|pq)
    }
  }
  red[threadIdx.x] = e;
  __syncthreads();
  for (int wdt = blockDim.x / 2; wdt > 0; wdt >>= 1) {
    if (threadIdx.x < wdt) red[threadIdx.x] += red[threadIdx.x + wdt];
    __syncthreads();
  }
  if (threadIdx.x == 0) part[blockIdx.x + (size_t)gridDim.x * blockIdx.y] = red[0];
}

__global__ void k_sum_parts(size_t cnt, const double *__restrict__ part, double *__restrict__ out) {
  __shared__ double red[1024];
  double s = 0.0;
  for (size_t i = threadIdx.x; i < cnt; i += blockDim.x) s += part[i];
  red[threadIdx.x] = s;
  __syncthreads();
  for (int w = blockDim.x / 2; w > 0; w >>= 1) {
    if (threadIdx.x < w) red[threadIdx.x] += red[threadIdx.x + w];
    __syncthreads();
  }
  if (threadIdx.x == 0) out[0] = red[0];
}

// COM of WIter_FOFO in the reference's own form (ac_fofo.f90:55-119): the inverse of
// A0 + omega^2 by LU at every frequency (dgetrf, dgetrs on the identity) and the series
// with FP64 products. The path when A+B(0) is not positive definite, where the
// eigenbasis form has no Cholesky factor.
int freq_com_lu(gc_context *ctx, int N, const double *a0p, const double *a0m, const double *a1p,
                const double *a1m, int nfreq, int max_cn, double *com) {
  const size_t NN = (size_t)N * N;
  gc::DevBuf<double> A0, A1, A2, Wm, inv, C0, C1, C2, w0, w1, work;
  for (auto *b : {&A0, &A1, &A2, &Wm, &inv, &C0, &C1, &C2, &w0, &w1}) GC_TRY(b->alloc(ctx, NN));
  gc::DevBuf<int> ipiv;
  GC_TRY(ipiv.alloc(ctx, N));
  const double one = 1.0, zero = 0.0;
  auto mm = [&](const double *A, const double *B, double *C, double alpha, double beta) {
    return cublasDgemm(ctx->cublas, CUBLAS_OP_N, CUBLAS_OP_N, N, N, N, &alpha, A, N, B, N, &beta, C,
                       N);
  };
  GC_CUBLAS(ctx, mm(a0p, a0m, A0.p, one, zero));   // A0 = A+0 A-0
  GC_CUBLAS(ctx, mm(a0p, a1m, A1.p, one, zero));   // A1 = A+0 A-1 + A+1 A-0
  GC_CUBLAS(ctx, mm(a1p, a0m, A1.p, one, one));
  GC_CUBLAS(ctx, mm(a1p, a1m, A2.p, one, zero));   // A2 = A+1 A-1
  int lw = 0;
  GC_CUSOLVER(ctx, cusolverDnDgetrf_bufferSize(ctx->cusolver, N, N, Wm.p, N, &lw));
  GC_TRY(work.alloc(ctx, std::max(lw, 1)));
  std::vector<double> xf(nfreq), wf(nfreq);
  GC_TRY(gc_freq_grid(nfreq, xf.data(), wf.data()));
  const double pi = 4.0 * std::atan(1.0);
  const unsigned ew = std::min<unsigned>(gc::ceil_div(NN, 256), 152u * 16u);
  GC_CUDA(ctx, cudaMemsetAsync(com, 0, NN * sizeof(double), ctx->stream));
  std::vector<int> infos;
  gc::DevBuf<int> dinfo;
  GC_TRY(dinfo.alloc(ctx, nfreq));
  for (int k = 0; k < nfreq; ++k) {
    k_add_diag<<<ew, 256, 0, ctx->stream>>>(NN, N, A0.p, xf[k] * xf[k], Wm.p);
    GC_LAUNCHED(ctx);
    GC_CUSOLVER(ctx, cusolverDnDgetrf(ctx->cusolver, N, N, Wm.p, N, work.p, ipiv.p, dinfo.p + k));
    GC_CUDA(ctx, cudaMemsetAsync(inv.p, 0, NN * sizeof(double), ctx->stream));
    k_add_diag<<<ew, 256, 0, ctx->stream>>>(NN, N, inv.p, 1.0, inv.p);  // identity
    GC_LAUNCHED(ctx);
    GC_CUSOLVER(ctx, cusolverDnDgetrs(ctx->cusolver, CUBLAS_OP_N, N, N, Wm.p, N, ipiv.p, inv.p, N,
                                      dinfo.p + k));
    const double wfact = 4.0 / pi * wf[k];
    GC_CUBLAS(ctx, mm(inv.p, a0p, C0.p, 0.5, zero));       // C0 = inv A+0 / 2
    GC_CUBLAS(ctx, mm(inv.p, A1.p, w0.p, one, zero));      // inv A1
    GC_CUBLAS(ctx, mm(w0.p, C0.p, C1.p, one, zero));       // C1 = inv A+1 / 2 - inv A1 C0
    GC_CUBLAS(ctx, mm(inv.p, a1p, C1.p, 0.5, -1.0));
    GC_CUBLAS(ctx, mm(inv.p, A2.p, w1.p, one, zero));      // inv A2
    k_lincomb<<<ew, 256, 0, ctx->stream>>>(NN, wfact, C0.p, 0.5 * wfact, C1.p, C2.p);
    GC_LAUNCHED(ctx);
    k_lincomb<<<ew, 256, 0, ctx->stream>>>(NN, 1.0, com, 1.0, C2.p, com);
    GC_LAUNCHED(ctx);
    double fact = 1.0;
    double *c0 = C0.p, *c1 = C1.p, *c2 = C2.p;
    for (int nord = 2; nord <= max_cn; ++nord) {
      fact *= nord;
      GC_CUBLAS(ctx, mm(w0.p, c1, c2, one, zero));
      GC_CUBLAS(ctx, mm(w1.p, c0, c2, -(double)nord * (nord - 1), -(double)nord));
      k_lincomb<<<ew, 256, 0, ctx->stream>>>(NN, 1.0, com, wfact / fact / (nord + 1), c2, com);
      GC_LAUNCHED(ctx);
      double *t = c0;
      c0 = c1;
      c1 = c2;
      c2 = t;
    }
  }
  infos.resize(nfreq);
  GC_CUDA(ctx, cudaMemcpyAsync(infos.data(), dinfo.p, nfreq * sizeof(int), cudaMemcpyDeviceToHost,
                               ctx->stream));
  GC_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
  for (int k = 0; k < nfreq; ++k)
    if (infos[k] != 0)
      return gc::set_error(ctx, GC_ECUSOLVER, "ac_freq_fofo: A0 + omega^2 singular at point %d "
                           "(getrf info %d)", k + 1, infos[k]);
  return GC_OK;
}

}  // namespace

namespace {
int freq_energy(gc_context *ctx, const gc::SysDev &sd, int N, const double *com,
                const double *fofo, int precision, double *ecorr);
}  // namespace

extern "C" int gc_freq_grid(int nfreq, double *x, double *w) {
  // FreqGrid, ac_iter.f:414-429: Gauss-Legendre on [-1, 1] mapped to [0, inf), x0 = 1/2
  if (nfreq <= 0 || !x || !w) return GC_EINVAL;
  GC_TRY(gc_gauleg(-1.0, 1.0, x, w, nfreq));
  const double x0 = 0.5;
  for (int i = 0; i < nfreq; ++i) {
    w[i] = 2.0 * x0 * w[i] / ((1.0 - x[i]) * (1.0 - x[i]));
    x[i] = x0 * (1.0 + x[i]) / (1.0 - x[i]);
  }
  return GC_OK;
}

extern "C" int gc_ac_freq_fofo(gc_context *ctx, int nbas, int ninact, int nact, int ndimx,
                               const double *occ, const double *ure, const double *xone,
                               const int *indn, const double *rdm2act, const double *ffoo,
                               const double *fofo, int nfreq, int max_cn, int precision,
                               int erpa_mode, double *ecorr, double *etot) {
  if (!ctx) return GC_EINVAL;
  if (!ecorr || !ffoo || !fofo || nfreq <= 0 || nfreq > 1000 || max_cn < 1 || max_cn > 12 ||
      (precision != GC_PREC_FP64 && !gc::is_sliced(precision)) ||
      (erpa_mode != GC_ERPA_CHOLESKY && erpa_mode != GC_ERPA_CHOLESKY_REFINED))
    return gc::set_error(ctx, GC_EINVAL, "ac_freq_fofo: bad arguments");
  const int N = ndimx;
  gc::SysDev sd;
  GC_TRY(gc::sys_upload(ctx, sd, nbas, ninact, nact, N, occ, xone, indn, rdm2act));
  if (ure) GC_TRY(gc::rotate_h(ctx, sd, ure));
  const size_t NN = (size_t)N * N;
  gc::DevBuf<double> a0p, a0m, a1p, a1m, L, U, w;
  for (auto *b : {&a0p, &a0m, &a1p, &a1m, &L, &U}) GC_TRY(b->alloc(ctx, NN));
  GC_TRY(w.alloc(ctx, N));
  // A+-B at lambda = 0 and 1; the slope A+-1 = A+-B(1) - A+-B(0) (ac_fofo.f90:41-52)
  GC_TRY(gc::assemble_ab(ctx, sd, ffoo, fofo, 0.0, a0p.p, a0m.p, etot));
  GC_TRY(gc::assemble_ab(ctx, sd, ffoo, fofo, 1.0, a1p.p, a1m.p, nullptr));
  GC_TRY(gc::axpby_into(ctx, NN, 1.0, a1p.p, -1.0, a0p.p, a1p.p));
  GC_TRY(gc::axpby_into(ctx, NN, 1.0, a1m.p, -1.0, a0m.p, a1m.p));
  // A+0 = L L^T, L^T A-0 L = U W U^T; without a Cholesky factor (A+B(0) not positive
  // definite) the reference's LU form at every frequency
  const int rc = gc::chol_eig(ctx, N, a0p.p, a0m.p, L.p, U.p, w.p, erpa_mode, precision);
  if (rc == GC_ENOTPD) {
    L.release();
    U.release();
    gc::DevBuf<double> com;
    GC_TRY(com.alloc(ctx, NN));
    GC_TRY(freq_com_lu(ctx, N, a0p.p, a0m.p, a1p.p, a1m.p, nfreq, max_cn, com.p));
    return freq_energy(ctx, sd, N, com.p, fofo, precision, ecorr);
  }
  GC_TRY(rc);
  a0p.release();
  a0m.release();
  gc::DevBuf<double> B, P, K, A1t, A2t, T1;
  for (auto *b : {&B, &P, &K, &A1t, &A2t, &T1}) GC_TRY(b->alloc(ctx, NN));
  const int p = precision;
  GC_TRY(gemm(ctx, p, false, false, N, N, N, L.p, N, U.p, N, B.p, N));  // B = L U
  // P = U^T (L^-1 A+1 L^-T) U with FP64 triangular solves
  const double one = 1.0;
  GC_CUDA(ctx, cudaMemcpyAsync(T1.p, a1p.p, NN * sizeof(double), cudaMemcpyDeviceToDevice,
                               ctx->stream));
  GC_CUBLAS(ctx, cublasDtrsm(ctx->cublas, CUBLAS_SIDE_LEFT, CUBLAS_FILL_MODE_LOWER, CUBLAS_OP_N,
                             CUBLAS_DIAG_NON_UNIT, N, N, &one, L.p, N, T1.p, N));
  GC_CUBLAS(ctx, cublasDtrsm(ctx->cublas, CUBLAS_SIDE_RIGHT, CUBLAS_FILL_MODE_LOWER, CUBLAS_OP_T,
                             CUBLAS_DIAG_NON_UNIT, N, N, &one, L.p, N, T1.p, N));
  GC_TRY(gemm(ctx, p, false, false, N, N, N, T1.p, N, U.p, N, A2t.p, N));   // (.) U
  GC_TRY(gemm(ctx, p, true, false, N, N, N, U.p, N, A2t.p, N, P.p, N));     // U^T (.)
  // K = B^T A-1 B
  GC_TRY(gemm(ctx, p, false, false, N, N, N, a1m.p, N, B.p, N, T1.p, N));
  GC_TRY(gemm(ctx, p, true, false, N, N, N, B.p, N, T1.p, N, K.p, N));
  a1p.release();
  a1m.release();
  L.release();
  U.release();
  // A1t = K + P W, A2t = P K
  const unsigned ew = std::min<unsigned>(gc::ceil_div(NN, 256), 152u * 16u);
  k_axpy_colscale<<<ew, 256, 0, ctx->stream>>>(NN, N, 1.0, K.p, 1.0, P.p, w.p, A1t.p);
  GC_LAUNCHED(ctx);
  GC_TRY(gemm(ctx, p, false, false, N, N, N, P.p, N, K.p, N, A2t.p, N));
  // frequency sum in the eigenbasis
  std::vector<double> xf(nfreq), wf(nfreq);
  GC_TRY(gc_freq_grid(nfreq, xf.data(), wf.data()));
  gc::DevBuf<double> S, Xa, Xb, Xc, T2;
  for (auto *b : {&S, &Xa, &Xb, &Xc, &T2}) GC_TRY(b->alloc(ctx, NN));
  GC_CUDA(ctx, cudaMemsetAsync(S.p, 0, NN * sizeof(double), ctx->stream));
  const double pi = 4.0 * std::atan(1.0);
  for (int k = 0; k < nfreq; ++k) {
    const double om2 = xf[k] * xf[k], wfact = 4.0 / pi * wf[k];
    // X(n-2), X(n-1), X(n) rotate through Xa, Xb, Xc; X0 = D/2 is never stored
    double *xm2 = nullptr, *xm1 = Xa.p, *xn = Xb.p, *spare = Xc.p;
    k_freq_x1<<<ew, 256, 0, ctx->stream>>>(NN, N, om2, w.p, P.p, A1t.p, wfact, wfact * 0.5, xm1,
                                           S.p);
    GC_LAUNCHED(ctx);
    double fact = 1.0;
    for (int nord = 2; nord <= max_cn; ++nord) {
      fact *= nord;
      GC_TRY(gemm(ctx, p, false, false, N, N, N, A1t.p, N, xm1, N, T1.p, N));   // A1t X(n-1)
      if (xm2) GC_TRY(gemm(ctx, p, false, false, N, N, N, A2t.p, N, xm2, N, T2.p, N));
      k_freq_xn<<<ew, 256, 0, ctx->stream>>>(NN, N, om2, nord, w.p, T1.p, xm2 ? T2.p : nullptr,
                                             A2t.p, wfact / fact / (nord + 1), xn, S.p);
      GC_LAUNCHED(ctx);
      double *old = xm2 ? xm2 : spare;
      xm2 = xm1;
      xm1 = xn;
      xn = old;
    }
  }
  // COM = B S B^T
  GC_TRY(gemm(ctx, p, false, true, N, N, N, S.p, N, B.p, N, T1.p, N));
  GC_TRY(gemm(ctx, p, false, false, N, N, N, B.p, N, T1.p, N, T2.p, N));
  return freq_energy(ctx, sd, N, T2.p, fofo, precision, ecorr);
}

namespace {

// ECorr of WIter_FOFO from COM (ac_fofo.f90:127-181).
int freq_energy(gc_context *ctx, const gc::SysDev &sd, int N, const double *com,
                const double *fofo, int precision, double *ecorr) {
  const unsigned gy = (unsigned)std::min(N, 1024);
  const size_t npart = (size_t)gc::ceil_div(N, 256) * gy;
  gc::DevBuf<double> part, res;
  GC_TRY(part.alloc(ctx, npart));
  GC_TRY(res.alloc(ctx, 1));
  k_freq_energy<<<dim3(gc::ceil_div(N, 256), gy), 256, 0, ctx->stream>>>(
      sd.n, sd.nocc, N, com, sd.pair_p.p, sd.pair_q.p, sd.cpl.p, sd.dnq.p, sd.grp.p, fofo, part.p);
  GC_LAUNCHED(ctx);
  k_sum_parts<<<1, 1024, 0, ctx->stream>>>(npart, part.p, res.p);
  GC_LAUNCHED(ctx);
  GC_CUDA(ctx, cudaMemcpyAsync(ecorr, res.p, sizeof(double), cudaMemcpyDeviceToHost, ctx->stream));
  if (precision != GC_PREC_FP64) GC_TRY(gc::check_flag(ctx));
  GC_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
  if (!std::isfinite(*ecorr))
    return gc::set_error(ctx, GC_ENONFINITE, "ac_freq_fofo: the energy is not finite");
  return GC_OK;
}

}  // namespace
