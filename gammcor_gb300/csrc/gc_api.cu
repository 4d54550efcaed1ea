// Context management, host-side helpers of the path (GauLeg, prepare_nums,
// pair builder) and the lambda-quadrature driver ACECORR.
#include <cmath>

#include "gc_internal.cuh"

namespace {

__global__ void k_axpby(size_t count, double a, const double *__restrict__ x, double b,
                        const double *__restrict__ y, double *__restrict__ out) {
  for (size_t t = blockIdx.x * (size_t)blockDim.x + threadIdx.x; t < count;
       t += (size_t)gridDim.x * blockDim.x)
    out[t] = a * x[t] + b * y[t];
}

}  // namespace

namespace gc {

namespace {
cudaEvent_t phase_event(gc_context *ctx) {
  if (!ctx->phase_pool.empty()) {
    cudaEvent_t e = ctx->phase_pool.back();
    ctx->phase_pool.pop_back();
    return e;
  }
  cudaEvent_t e = nullptr;
  return cudaEventCreate(&e) == cudaSuccess ? e : nullptr;
}
}  // namespace

PhaseScope::PhaseScope(gc_context *ctx, int phase) : ctx_(ctx), phase_(phase) {
  if (!ctx_ || !ctx_->phase_on) return;
  a_ = phase_event(ctx_);
  if (a_ && cudaEventRecord(a_, ctx_->stream) != cudaSuccess) {
    ctx_->phase_pool.push_back(a_);
    a_ = nullptr;
  }
}

PhaseScope::~PhaseScope() {
  if (!a_) return;
  cudaEvent_t b = phase_event(ctx_);
  if (!b || cudaEventRecord(b, ctx_->stream) != cudaSuccess) {
    ctx_->phase_pool.push_back(a_);
    if (b) ctx_->phase_pool.push_back(b);
    return;
  }
  ctx_->phase_pending.push_back({phase_, a_, b});
  phase_collect(ctx_, false);
}

void phase_collect(gc_context *ctx, bool wait) {
  std::vector<gc_phase_rec> keep;
  for (const gc_phase_rec &r : ctx->phase_pending) {
    cudaError_t q = wait ? cudaEventSynchronize(r.b) : cudaEventQuery(r.b);
    if (q == cudaErrorNotReady) {
      keep.push_back(r);
      continue;
    }
    float ms = 0.f;
    if (q == cudaSuccess && cudaEventElapsedTime(&ms, r.a, r.b) == cudaSuccess) {
      ctx->phase_ms[r.phase] += ms;
      ctx->phase_calls[r.phase]++;
    }
    ctx->phase_pool.push_back(r.a);
    ctx->phase_pool.push_back(r.b);
  }
  ctx->phase_pending.swap(keep);
}


int axpby_into(gc_context *ctx, size_t count, double a, const double *x, double b, const double *y,
               double *out) {
  unsigned grid = std::min<unsigned>(ceil_div(count, 256), 152u * 16u);
  k_axpby<<<grid, 256, 0, ctx->stream>>>(count, a, x, b, y, out);
  GC_LAUNCHED(ctx);
  return GC_OK;
}

}  // namespace gc

extern "C" {

int gc_create(gc_context **out, int device, void *stream) {
  if (!out) return GC_EINVAL;
  *out = nullptr;
  gc_context *ctx = new gc_context();
  ctx->device = device;
  cudaError_t e = cudaSetDevice(device);
  if (e != cudaSuccess) {
    delete ctx;
    return GC_ECUDA;
  }
  // The caller's stream is used as given (NULL is the legacy default stream),
  // so that work is ordered with whatever produced the inputs on that stream.
  ctx->stream = (cudaStream_t)stream;
  if (cublasCreate(&ctx->cublas) != CUBLAS_STATUS_SUCCESS ||
      cublasSetStream(ctx->cublas, ctx->stream) != CUBLAS_STATUS_SUCCESS ||
      cublasSetMathMode(ctx->cublas, CUBLAS_PEDANTIC_MATH) != CUBLAS_STATUS_SUCCESS) {
    gc_destroy(ctx);
    return GC_ECUBLAS;
  }
  if (cusolverDnCreate(&ctx->cusolver) != CUSOLVER_STATUS_SUCCESS ||
      cusolverDnSetStream(ctx->cusolver, ctx->stream) != CUSOLVER_STATUS_SUCCESS) {
    gc_destroy(ctx);
    return GC_ECUSOLVER;
  }
  if (cudaMalloc(&ctx->dev_info, sizeof(int)) != cudaSuccess ||
      cudaMalloc(&ctx->dev_flag, sizeof(int)) != cudaSuccess ||
      cudaMemset(ctx->dev_flag, 0, sizeof(int)) != cudaSuccess ||
      cudaMalloc(&ctx->dev_nonfinite, sizeof(int)) != cudaSuccess ||
      cudaEventCreate(&ctx->eig_ev[0]) != cudaSuccess ||
      cudaEventCreate(&ctx->eig_ev[1]) != cudaSuccess) {
    gc_destroy(ctx);
    return GC_ENOMEM;
  }
  *out = ctx;
  return GC_OK;
}

int gc_destroy(gc_context *ctx) {
  if (!ctx) return GC_OK;
  if (ctx->stream) cudaStreamSynchronize(ctx->stream);
  if (ctx->cusolver) cusolverDnDestroy(ctx->cusolver);
  if (ctx->cublas) cublasDestroy(ctx->cublas);
  if (ctx->dev_info) cudaFree(ctx->dev_info);
  if (ctx->dev_flag) cudaFree(ctx->dev_flag);
  if (ctx->dev_nonfinite) cudaFree(ctx->dev_nonfinite);
  for (cudaEvent_t e : ctx->eig_ev)
    if (e) cudaEventDestroy(e);
  for (const gc_phase_rec &r : ctx->phase_pending) {
    cudaEventDestroy(r.a);
    cudaEventDestroy(r.b);
  }
  for (cudaEvent_t e : ctx->phase_pool) cudaEventDestroy(e);
  delete ctx;
  return GC_OK;
}

const char *gc_last_error(const gc_context *ctx) { return ctx ? ctx->err.c_str() : "null context"; }

int gc_synchronize(gc_context *ctx) {
  if (!ctx) return GC_EINVAL;
  GC_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
  return GC_OK;
}

long long gc_kernel_launches(const gc_context *ctx) { return ctx ? ctx->launches : 0; }

int gc_eig_time(const gc_context *ctx, double *ms, long long *calls) {
  if (!ctx) return GC_EINVAL;
  if (ms) *ms = ctx->eig_ms;
  if (calls) *calls = ctx->eig_calls;
  return GC_OK;
}

int gc_set_phase_timing(gc_context *ctx, int on) {
  if (!ctx) return GC_EINVAL;
  ctx->phase_on = on ? 1 : 0;
  return GC_OK;
}

int gc_phase_time(gc_context *ctx, int phase, double *ms, long long *calls) {
  if (!ctx) return GC_EINVAL;
  if (phase < 0 || phase >= GC_PHASE_COUNT)
    return gc::set_error(ctx, GC_EINVAL, "phase %d outside 0..%d", phase, GC_PHASE_COUNT - 1);
  gc::phase_collect(ctx, true);
  if (ms) *ms = ctx->phase_ms[phase];
  if (calls) *calls = ctx->phase_calls[phase];
  return GC_OK;
}

int gc_set_eig_emulation(gc_context *ctx, int on) {
  if (!ctx) return GC_EINVAL;
  GC_CUSOLVER(ctx, cusolverDnSetEmulationStrategy(
                       ctx->cusolver, on ? CUDA_EMULATION_STRATEGY_EAGER : CUDA_EMULATION_STRATEGY_DEFAULT));
  ctx->eig_emulation = on ? 1 : 0;
  return GC_OK;
}

// misc.f:828-865 (Numerical Recipes gauleg, EPS = 3e-14)
int gc_gauleg(double x1, double x2, double *x, double *w, int n) {
  if (n <= 0 || !x || !w) return GC_EINVAL;
  const double eps = 3e-14;
  int m = (n + 1) / 2;
  double xm = 0.5 * (x2 + x1), xl = 0.5 * (x2 - x1);
  for (int i = 1; i <= m; ++i) {
    double z = std::cos(3.141592654 * (i - 0.25) / (n + 0.5)), z1, pp;
    int guard = 0;
    do {
      double p1 = 1.0, p2 = 0.0, p3;
      for (int j = 1; j <= n; ++j) {
        p3 = p2;
        p2 = p1;
        p1 = ((2.0 * j - 1.0) * z * p2 - (j - 1.0) * p3) / j;
      }
      pp = n * (z * p1 - p2) / (z * z - 1.0);
      z1 = z;
      z = z1 - p1 / pp;
    } while (std::fabs(z - z1) > eps && ++guard < 100);
    x[i - 1] = xm - xl * z;
    x[n - i] = xm + xl * z;
    w[i - 1] = 2.0 * xl / ((1.0 - z * z) * pp * pp);
    w[n - i] = w[i - 1];
  }
  return GC_OK;
}

// IndAux of ACCAS (accas.f:30-44) and prepare_nums (initia.f:2996-3035).
static void ind_aux(int nbas, const double *occ, int nele, std::vector<int> &aux) {
  aux.assign(nbas, 0);
  for (int i = 0; i < nbas; ++i) {
    aux[i] = (i + 1 <= nele) ? 0 : 2;
    if (occ[i] < 1.0 && occ[i] != 0.0) aux[i] = 1;
  }
}

int gc_prepare_nums(int nbas, const double *occ, int nele, int *num0, int *num1) {
  if (nbas <= 0 || !occ || !num0 || !num1) return GC_EINVAL;
  std::vector<int> aux;
  ind_aux(nbas, occ, nele, aux);
  int n0 = 0, n2 = 0;
  for (int i = 0; i < nbas && aux[i] == 0; ++i) n0++;
  for (int i = nbas - 1; i >= 0 && aux[i] == 2; --i) n2++;
  *num0 = n0;
  *num1 = nbas - n0 - n2;
  return GC_OK;
}

int gc_pair_space(int nbas, const double *occ, int nele, int ifl_core, double thr_sel_act,
                  double thr_qvirt, int *indn, int *ndimx) {
  if (nbas <= 0 || !occ || !indn || !ndimx) return GC_EINVAL;
  std::vector<int> aux;
  ind_aux(nbas, occ, nele, aux);
  int ind = 0;
  for (int I = 1; I <= nbas; ++I)
    for (int J = 1; J < I; ++J) {
      int a = aux[I - 1] + aux[J - 1];
      if (a == 0 || a == 4) continue;
      double oi = occ[I - 1], oj = occ[J - 1];
      if (aux[I - 1] == 1 && aux[J - 1] == 1 && std::fabs(oi - oj) / oi < thr_sel_act) continue;
      if (ifl_core == 1 || (oi != 1.0 && oj != 1.0)) {
        if (std::fabs(oi + oj - 2.0) > 1e-10 && std::fabs(oi + oj) > thr_qvirt) {
          indn[2 * ind] = I;
          indn[2 * ind + 1] = J;
          ind++;
        }
      }
    }
  *ndimx = ind;
  return GC_OK;
}

int gc_acecorr(gc_context *ctx, int nbas, int ninact, int nact, int ndimx, const double *occ,
               const double *xone, const int *indn, const double *rdm2act, const double *ffoo,
               const double *fofo, int ngrid, int erpa_mode, int precision, double *ecorr,
               double *ecas, double *w_out) {
  if (!ctx) return GC_EINVAL;
  if (ngrid <= 0 || ngrid > 100 || !xone || !ffoo || !fofo || !ecorr || !ecas)
    return gc::set_error(ctx, GC_EINVAL, "acecorr: bad arguments (ngrid=%d)", ngrid);
  if (!indn) return gc::set_error(ctx, GC_EINVAL, "acecorr: null IndN");
  gc::SysDev sd;
  // pairs in the coalescing order (the energies do not depend on the pair order)
  const std::vector<int> ind = gc::coalesced_pair_order(indn, ndimx);
  GC_TRY(gc::sys_upload(ctx, sd, nbas, ninact, nact, ndimx, occ, xone, ind.data(), rdm2act));
  std::vector<double> x(ngrid), w(ngrid);
  gc_gauleg(0.0, 1.0, x.data(), w.data(), ngrid);
  const size_t NN = (size_t)ndimx * ndimx;
  gc::DevBuf<double> ap, am, a0p, a0m, a1p, a1m, Y, eig;
  GC_TRY(ap.alloc(ctx, NN));
  GC_TRY(am.alloc(ctx, NN));
  GC_TRY(Y.alloc(ctx, NN));
  GC_TRY(eig.alloc(ctx, ndimx));
  const bool affine = erpa_mode == GC_ERPA_CHOLESKY || erpa_mode == GC_ERPA_CHOLESKY_REFINED;
  double e0 = 0.0;
  if (affine) {
    GC_TRY(a0p.alloc(ctx, NN));
    GC_TRY(a0m.alloc(ctx, NN));
    GC_TRY(a1p.alloc(ctx, NN));
    GC_TRY(a1m.alloc(ctx, NN));
    GC_TRY(gc::assemble_ab(ctx, sd, ffoo, fofo, 0.0, a0p.p, a0m.p, &e0));
    GC_TRY(gc::assemble_ab(ctx, sd, ffoo, fofo, 1.0, a1p.p, a1m.p, nullptr));
  }
  double acc = 0.0;
  for (int i = 0; i < ngrid; ++i) {
    double lam = x[i];
    if (affine) {
      GC_TRY(gc::axpby_into(ctx, NN, 1.0 - lam, a0p.p, lam, a1p.p, ap.p));
      GC_TRY(gc::axpby_into(ctx, NN, 1.0 - lam, a0m.p, lam, a1m.p, am.p));
      *ecas = e0;
    } else {
      GC_TRY(gc::assemble_ab(ctx, sd, ffoo, fofo, lam, ap.p, am.p, ecas));
    }
    GC_TRY(gc::erpa_solve(ctx, ndimx, ap.p, am.p, Y.p, eig.p, erpa_mode, precision));
    double wi = 0.0;
    GC_TRY(gc::integrand(ctx, sd, Y.p, eig.p, fofo, precision, &wi));
    if (w_out) w_out[i] = wi;
    acc += w[i] * wi;
  }
  *ecorr = acc;
  return GC_OK;
}

}  // extern "C"
