// AC integrand W(lambda), ACEneERPA_FOFO (abfofo.f90:3791-3927).
//
// The reference takes, for every pair of pairs (rs, pq) not lying in one
// orbital group, ddot(tVec(:,pq), tVec(:,rs)) over kept eigenvectors and
// weights it with 2 (C_r+C_s)(C_p+C_q) (rs|pq). Written as a matrix product:
//   Kt[pq, rs] = mask * (C_p+C_q)(C_r+C_s) (rs|pq)       (lambda independent)
//   W = 2 sum_{i,nu} Yk[i,nu] (Kt Yk)[i,nu] - sum_pq mask (n_p(1-n_q)+n_q(1-n_p)) (pq|pq)
// with Yk = Y restricted to 1e-3 < omega < 1e8. One GEMM and one reduction
// replace N^2 dot products of length N. On the tensor-core path the diagonal of
// Kt is taken out of the product and its term 2 Kt_ii (Yk Yk^T)_ii, which
// nearly cancels the diagonal correction, is summed in FP64.
#include <cmath>

#include "gc_internal.cuh"
#include "gc_tc_gemm.cuh"

namespace {

const double kSmallE = 1e-3, kBigE = 1e8;  // abfofo.f90:3808

// Kt[i, j] = mask (C_p + C_q)(C_r + C_s) (rs|pq) with the per-pair sums cpl; the
// pair-of-pairs mask and the FOFO address are integer work, so the element costs
// two FP64 products (GB300's FP64 pipe, not HBM, bounds this kernel otherwise).
__global__ void k_kt(int n, int nocc, int N, const int *__restrict__ pp, const int *__restrict__ pq,
                     const double *__restrict__ cpl, const double *__restrict__ dnq,
                     const int *__restrict__ grp, const double *__restrict__ fofo, int split_diag,
                     double *__restrict__ kt, double *__restrict__ diag,
                     double *__restrict__ kdiag) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  int j = blockIdx.y * blockDim.y + threadIdx.y;
  if (i >= N || j >= N) return;
  int p = pp[i], q = pq[i], r = pp[j], s = pq[j];
  bool same = grp[p] == grp[q] && grp[q] == grp[r] && grp[r] == grp[s];
  size_t ld = (size_t)n * nocc;
  double f = fofo[(size_t)(r + (size_t)s * n) * ld + p + (size_t)q * n];  // (rs|pq)
  double kv = same ? 0.0 : (cpl[i] * cpl[j]) * f;
  kt[i + (size_t)j * N] = (split_diag && i == j) ? 0.0 : kv;
  if (i == j) {
    diag[i] = same ? 0.0 : -dnq[i] * f;
    kdiag[i] = kv;
  }
}

// diag[i] += 2 Kt_ii sum_nu Yk[i,nu]^2  (FP64)
__global__ void k_diag_term(int N, const double *__restrict__ Yk, const double *__restrict__ kdiag,
                            double *__restrict__ diag) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= N) return;
  double s = 0.0;
  for (int nu = 0; nu < N; ++nu) {
    double y = Yk[i + (size_t)nu * N];
    s += y * y;
  }
  diag[i] += 2.0 * kdiag[i] * s;
}

__global__ void k_mask_cols(int N, const double *__restrict__ Y, const double *__restrict__ eig,
                            double *__restrict__ Yk) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  int nu = blockIdx.y;
  if (i >= N) return;
  double e = eig[nu];
  bool keep = e > kSmallE && e < kBigE;
  Yk[i + (size_t)nu * N] = keep ? Y[i + (size_t)nu * N] : 0.0;
}

// partial[b] = sum over a grid-stride slice of 2 * Yk * T  (+ diag on block 0)
__global__ void k_contract(size_t total, int N, const double *__restrict__ Yk,
                           const double *__restrict__ T, const double *__restrict__ diag,
                           double *__restrict__ part) {
  __shared__ double red[256];
  double s = 0.0;
  for (size_t t = blockIdx.x * (size_t)blockDim.x + threadIdx.x; t < total;
       t += (size_t)gridDim.x * blockDim.x)
    s += Yk[t] * T[t];
  s *= 2.0;
  if (blockIdx.x == 0)
    for (int i = threadIdx.x; i < N; i += blockDim.x) s += diag[i];
  red[threadIdx.x] = s;
  __syncthreads();
  for (int w = blockDim.x / 2; w > 0; w >>= 1) {
    if (threadIdx.x < w) red[threadIdx.x] += red[threadIdx.x + w];
    __syncthreads();
  }
  if (threadIdx.x == 0) part[blockIdx.x] = red[0];
}

}  // namespace

namespace gc {

int integrand(gc_context *ctx, const SysDev &sd, const double *Y, const double *eig,
              const double *fofo, int precision, double *w_host) {
  PhaseScope ph(ctx, GC_PHASE_INTEGRAND);
  const int N = sd.ndimx;
  const size_t NN = (size_t)N * N;
  DevBuf<double> kt, yk, t, diag, kdiag, part;
  GC_TRY(kt.alloc(ctx, NN));
  GC_TRY(yk.alloc(ctx, NN));
  if (precision == GC_PREC_FP64) GC_TRY(t.alloc(ctx, NN));
  GC_TRY(diag.alloc(ctx, N));
  GC_TRY(kdiag.alloc(ctx, N));
  const int split = precision != GC_PREC_FP64;
  const int nb = 304;
  GC_TRY(part.alloc(ctx, nb));
  dim3 b2(32, 8), g2(ceil_div(N, 32), ceil_div(N, 8));
  k_kt<<<g2, b2, 0, ctx->stream>>>(sd.n, sd.nocc, N, sd.pair_p.p, sd.pair_q.p, sd.cpl.p,
                                   sd.dnq.p, sd.grp.p, fofo, split, kt.p, diag.p, kdiag.p);
  GC_LAUNCHED(ctx);
  k_mask_cols<<<dim3(ceil_div(N, 256), N), 256, 0, ctx->stream>>>(N, Y, eig, yk.p);
  GC_LAUNCHED(ctx);
  if (precision == GC_PREC_FP64) {
    // T = Kt Yk, then W = 2 sum Yk .* T + sum diag
    const double one = 1.0, zero = 0.0;
    GC_CUBLAS(ctx, cublasDgemm(ctx->cublas, CUBLAS_OP_N, CUBLAS_OP_N, N, N, N, &one, kt.p, N, yk.p,
                               N, &zero, t.p, N));
  } else {
    // off-diagonal Kt Yk on tensor cores with the dot product against Yk fused
    // into the epilogue; the diagonal term in FP64
    k_diag_term<<<ceil_div(N, 128), 128, 0, ctx->stream>>>(N, yk.p, kdiag.p, diag.p);
    GC_LAUNCHED(ctx);
    double dot = 0.0;
    GC_TRY(tc_dot_gemm(ctx, precision, N, kt.p, yk.p, &dot));
    std::vector<double> hd(N);
    GC_CUDA(ctx, cudaMemcpyAsync(hd.data(), diag.p, N * sizeof(double), cudaMemcpyDeviceToHost,
                                 ctx->stream));
    GC_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    double dsum = 0.0;
    for (double v : hd) dsum += v;
    *w_host = 2.0 * dot + dsum;
    if (!std::isfinite(*w_host))
      return set_error(ctx, GC_ENONFINITE, "integrand: W is not finite (non-finite integrals?)");
    return GC_OK;
  }
  k_contract<<<nb, 256, 0, ctx->stream>>>(NN, N, yk.p, t.p, diag.p, part.p);
  GC_LAUNCHED(ctx);
  double hp[nb];
  GC_CUDA(ctx, cudaMemcpyAsync(hp, part.p, sizeof hp, cudaMemcpyDeviceToHost, ctx->stream));
  GC_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
  double w = 0.0;
  for (int b = 0; b < nb; ++b) w += hp[b];
  *w_host = w;
  if (!std::isfinite(w))
    return set_error(ctx, GC_ENONFINITE, "integrand: W is not finite (non-finite integrals?)");
  return GC_OK;
}

}  // namespace gc

extern "C" int gc_ace_ne_erpa_fofo(gc_context *ctx, int nbas, int ninact, int nact, int ndimx,
                                   const double *occ, const int *indn, const double *eigvec,
                                   const double *eig, const double *fofo, int precision,
                                   double *w_host) {
  if (!ctx) return GC_EINVAL;
  if (!eigvec || !eig || !fofo || !w_host)
    return gc::set_error(ctx, GC_EINVAL, "ace_ne_erpa_fofo: null pointer");
  gc::SysDev sd;
  // no one-electron integrals or 2-RDM needed here
  std::vector<double> dummy_rdm((size_t)nact * nact * (nact * nact + 1) / 2 + 1, 0.0);
  GC_TRY(gc::sys_upload(ctx, sd, nbas, ninact, nact, ndimx, occ, nullptr, indn, dummy_rdm.data()));
  return gc::integrand(ctx, sd, eigvec, eig, fofo, precision, w_host);
}
