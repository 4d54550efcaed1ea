// Batched AC-CAS energies over many systems of uneven size.
//
// The reference computes one system per process (ACECORR, acfd.f:117-209).
// Here a batch of independent systems is spread over worker streams: each
// worker owns a context (stream, cuBLAS and cuSOLVER handles) and takes the
// largest remaining system first. Per system it runs the factored transform
// (FFOO, FOFO), the A+-B assembly at lambda = 0 and 1 (A+-B is affine in
// lambda), and for every requested lambda point the ERPA solve and the
// integrand. The batch is ordered after the caller's stream and the caller's
// stream waits for every worker before the call returns.
#include <algorithm>
#include <atomic>
#include <mutex>
#include <numeric>
#include <thread>

#include "gc_internal.cuh"

namespace {

struct Worker {
  gc_context *ctx = nullptr;
  cudaStream_t stream = nullptr;
  cudaEvent_t done = nullptr;
};

void omega_stats(const std::vector<double> &e, double *st) {
  std::vector<double> k;
  for (double v : e)
    if (v > 1e-3 && v < 1e8) k.push_back(v);
  for (int i = 0; i < GC_OMEGA_STATS; ++i) st[i] = 0.0;
  if (k.empty()) return;
  std::sort(k.begin(), k.end());
  double s = 0, si = 0;
  for (double v : k) s += v, si += 1.0 / v;
  st[0] = (double)k.size() / (double)e.size();
  st[1] = k.front();
  st[2] = k.back();
  st[3] = s / k.size();
  st[4] = si / k.size();
  st[5] = k[k.size() / 2];
}

int run_system(gc_context *ctx, const gc_system &s, const gc_ac_params &par, double *ecorr,
               double *ecas, double *w_out, double *stats_out) {
  const int n = s.nbas, nocc = s.ninact + s.nact, N = s.ndimx;
  const size_t NN = (size_t)N * N;
  gc::DevBuf<double> ffoo, fofo, co;
  GC_TRY(ffoo.alloc(ctx, (size_t)nocc * nocc * n * n));
  GC_TRY(fofo.alloc(ctx, (size_t)n * nocc * n * nocc));
  // occupied block of C: the first nocc columns of the column-major AO x MO matrix
  const double *C = s.cmo_dev;
  GC_TRY(gc_tran4_factored(ctx, n, s.rank, s.lfac_dev, n, C, nocc, C, n, C, nocc, C, fofo.p,
                           par.precision));
  GC_TRY(gc_tran4_factored(ctx, n, s.rank, s.lfac_dev, nocc, C, nocc, C, n, C, n, C, ffoo.p,
                           par.precision));
  gc::SysDev sd;
  GC_TRY(gc::sys_upload(ctx, sd, n, s.ninact, s.nact, N, s.occ, s.xone, s.indn, s.rdm2act));
  std::vector<double> x(par.ngrid), w(par.ngrid, 0.0);
  if (par.lambda) {
    for (int i = 0; i < par.ngrid; ++i) {
      x[i] = par.lambda[i];
      w[i] = par.weight ? par.weight[i] : 0.0;
    }
  } else {
    gc_gauleg(0.0, 1.0, x.data(), w.data(), par.ngrid);
  }
  gc::DevBuf<double> ap, am, Y, eig, a0p, a0m, a1p, a1m;
  GC_TRY(ap.alloc(ctx, NN));
  GC_TRY(am.alloc(ctx, NN));
  GC_TRY(Y.alloc(ctx, NN));
  GC_TRY(eig.alloc(ctx, N));
  double e0 = 0.0;
  if (par.affine) {
    GC_TRY(a0p.alloc(ctx, NN));
    GC_TRY(a0m.alloc(ctx, NN));
    GC_TRY(a1p.alloc(ctx, NN));
    GC_TRY(a1m.alloc(ctx, NN));
    GC_TRY(gc::assemble_ab(ctx, sd, ffoo.p, fofo.p, 0.0, a0p.p, a0m.p, &e0));
    GC_TRY(gc::assemble_ab(ctx, sd, ffoo.p, fofo.p, 1.0, a1p.p, a1m.p, nullptr));
  }
  double acc = 0.0;
  for (int i = 0; i < par.ngrid; ++i) {
    double lam = x[i];
    if (par.affine) {
      GC_TRY(gc::axpby_into(ctx, NN, 1.0 - lam, a0p.p, lam, a1p.p, ap.p));
      GC_TRY(gc::axpby_into(ctx, NN, 1.0 - lam, a0m.p, lam, a1m.p, am.p));
    } else {
      GC_TRY(gc::assemble_ab(ctx, sd, ffoo.p, fofo.p, lam, ap.p, am.p, &e0));
    }
    GC_TRY(gc::erpa_solve(ctx, N, ap.p, am.p, Y.p, eig.p, par.erpa_mode, par.precision));
    double wi = 0.0;
    GC_TRY(gc::integrand(ctx, sd, Y.p, eig.p, fofo.p, par.precision, &wi));
    if (w_out) w_out[i] = wi;
    if (stats_out) {
      std::vector<double> he(N);
      GC_CUDA(ctx, cudaMemcpyAsync(he.data(), eig.p, N * sizeof(double), cudaMemcpyDeviceToHost,
                                   ctx->stream));
      GC_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
      omega_stats(he, stats_out + (size_t)i * GC_OMEGA_STATS);
    }
    acc += w[i] * wi;
  }
  *ecorr = acc;
  *ecas = e0;
  return GC_OK;
}

}  // namespace

extern "C" int gc_ac_energy_batched(gc_context *ctx, int nsys, const gc_system *sys,
                                    const gc_ac_params *par, double *ecorr, double *ecas,
                                    double *w_lambda, double *omega_st, int *status) {
  if (!ctx) return GC_EINVAL;
  if (nsys <= 0 || !sys || !par || !ecorr || !ecas || par->ngrid <= 0 || par->ngrid > 100)
    return gc::set_error(ctx, GC_EINVAL, "ac_energy_batched: bad arguments");
  for (int i = 0; i < nsys; ++i)
    if (!sys[i].cmo_dev || !sys[i].lfac_dev || !sys[i].occ || !sys[i].xone || !sys[i].indn ||
        sys[i].nbas <= 0 || sys[i].ndimx <= 0 || sys[i].rank <= 0)
      return gc::set_error(ctx, GC_EINVAL, "ac_energy_batched: system %d incomplete", i);
  const int nw = std::max(1, std::min(par->nstreams, nsys));
  // largest systems first
  std::vector<int> order(nsys);
  std::iota(order.begin(), order.end(), 0);
  std::stable_sort(order.begin(), order.end(),
                   [&](int a, int b) { return sys[a].ndimx > sys[b].ndimx; });
  cudaEvent_t start;
  GC_CUDA(ctx, cudaEventCreateWithFlags(&start, cudaEventDisableTiming));
  GC_CUDA(ctx, cudaEventRecord(start, ctx->stream));
  std::vector<Worker> ws(nw);
  for (auto &w : ws) {
    GC_CUDA(ctx, cudaStreamCreateWithFlags(&w.stream, cudaStreamNonBlocking));
    GC_CUDA(ctx, cudaEventCreateWithFlags(&w.done, cudaEventDisableTiming));
    int r = gc_create(&w.ctx, ctx->device, w.stream);
    if (r != GC_OK) return gc::set_error(ctx, r, "ac_energy_batched: worker context");
    if (par->eig_emulation && (r = gc_set_eig_emulation(w.ctx, 1)) != GC_OK)
      return gc::set_error(ctx, r, "ac_energy_batched: %s", w.ctx->err.c_str());
    GC_CUDA(ctx, cudaStreamWaitEvent(w.stream, start, 0));
  }
  std::atomic<int> next{0};
  std::atomic<int> first_err{GC_OK};
  std::mutex err_mu;
  std::string err_msg;
  auto body = [&](Worker &w) {
    cudaSetDevice(ctx->device);
    for (;;) {
      int k = next.fetch_add(1);
      if (k >= nsys || first_err.load() != GC_OK) break;
      int i = order[k];
      int r = run_system(w.ctx, sys[i], *par, &ecorr[i], &ecas[i],
                         w_lambda ? w_lambda + (size_t)i * par->ngrid : nullptr,
                         omega_st ? omega_st + (size_t)i * par->ngrid * GC_OMEGA_STATS : nullptr);
      if (status) status[i] = r;
      if (r != GC_OK && !(status && r == GC_ENOTPD)) {
        int expected = GC_OK;
        if (first_err.compare_exchange_strong(expected, r)) {
          std::lock_guard<std::mutex> lk(err_mu);
          err_msg = "system " + std::to_string(i) + ": " + w.ctx->err;
        }
        break;
      }
    }
    cudaEventRecord(w.done, w.stream);
  };
  std::vector<std::thread> th;
  for (int t = 1; t < nw; ++t) th.emplace_back(body, std::ref(ws[t]));
  body(ws[0]);
  for (auto &t : th) t.join();
  for (auto &w : ws) {
    cudaStreamWaitEvent(ctx->stream, w.done, 0);
    ctx->launches += w.ctx->launches;
  }
  for (auto &w : ws) {
    gc_destroy(w.ctx);
    cudaStreamDestroy(w.stream);
    cudaEventDestroy(w.done);
  }
  cudaEventDestroy(start);
  if (first_err.load() != GC_OK)
    return gc::set_error(ctx, first_err.load(), "%s", err_msg.c_str());
  return GC_OK;
}
