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
//
// gc_ac_energy_batched builds each system's state, evaluates its points and
// frees the state. A gc_ac_session keeps the workers and every system's state
// (integrals, A+-B at lambda = 0 and 1) on the device between calls, so that
// points can be added to some systems later (the integrand surrogate evaluates
// the two end nodes of all systems, then the interior nodes of the systems its
// error estimate rejects) without repeating the transform or the assembly.
#include <algorithm>
#include <atomic>
#include <functional>
#include <memory>
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

// Device state of one system: transformed integrals, system description and,
// in the affine form, A+-B at lambda = 0 and 1.
struct SysState {
  gc::DevBuf<double> ffoo, fofo, a0p, a0m, a1p, a1m;
  gc::SysDev sd;
  double e0 = 0.0;     // E_CAS of the assembly
  int built = 0;       // 1 once the state is complete
  int status = GC_OK;  // status of the build
  cudaEvent_t ready = nullptr;
  ~SysState() {
    if (ready) cudaEventDestroy(ready);
  }
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

int build_state(gc_context *ctx, const gc_system &s, const gc_ac_params &par, SysState &st) {
  const int n = s.nbas, nocc = s.ninact + s.nact, N = s.ndimx;
  const size_t NN = (size_t)N * N;
  GC_TRY(st.ffoo.alloc(ctx, (size_t)nocc * nocc * n * n));
  GC_TRY(st.fofo.alloc(ctx, (size_t)n * nocc * n * nocc));
  // occupied block of C: the first nocc columns of the column-major AO x MO matrix
  const double *C = s.cmo_dev;
  GC_TRY(gc_tran4_factored(ctx, n, s.rank, s.lfac_dev, n, C, nocc, C, n, C, nocc, C, st.fofo.p,
                           par.precision));
  GC_TRY(gc_tran4_factored(ctx, n, s.rank, s.lfac_dev, nocc, C, nocc, C, n, C, n, C, st.ffoo.p,
                           par.precision));
  // pairs in the coalescing order (the energies do not depend on the pair order)
  const std::vector<int> ind = gc::coalesced_pair_order(s.indn, N);
  GC_TRY(gc::sys_upload(ctx, st.sd, n, s.ninact, s.nact, N, s.occ, s.xone, ind.data(), s.rdm2act));
  if (par.affine) {
    GC_TRY(st.a0p.alloc(ctx, NN));
    GC_TRY(st.a0m.alloc(ctx, NN));
    GC_TRY(st.a1p.alloc(ctx, NN));
    GC_TRY(st.a1m.alloc(ctx, NN));
    GC_TRY(gc::assemble_ab(ctx, st.sd, st.ffoo.p, st.fofo.p, 0.0, st.a0p.p, st.a0m.p, &st.e0));
    GC_TRY(gc::assemble_ab(ctx, st.sd, st.ffoo.p, st.fofo.p, 1.0, st.a1p.p, st.a1m.p, nullptr));
  }
  st.built = 1;
  return GC_OK;
}

// W(lambda) at np points x of a built state: w_out[i] (may be NULL), excitation
// statistics stats_out[i * GC_OMEGA_STATS] (may be NULL), sum_i wt[i] W_i in *acc
// when wt is given.
int eval_points(gc_context *ctx, const gc_system &s, const gc_ac_params &par, SysState &st,
                int np, const double *x, const double *wt, double *w_out, double *stats_out,
                double *acc) {
  const int N = s.ndimx;
  const size_t NN = (size_t)N * N;
  if (par.erpa_mode == GC_ERPA_CHOLESKY_REFINED && gc::is_sliced(par.precision) && np >= 2 &&
      ctx->eig_batch) {
    // all points' FP32 eigensolves in one batched call
    double sum = 0.0;
    auto fill = [&](int i, double *ap, double *am) -> int {
      const double lam = x[i];
      if (par.affine) {
        gc::PhaseScope ph(ctx, GC_PHASE_ASSEMBLY);
        GC_TRY(gc::axpby_into(ctx, NN, 1.0 - lam, st.a0p.p, lam, st.a1p.p, ap));
        GC_TRY(gc::axpby_into(ctx, NN, 1.0 - lam, st.a0m.p, lam, st.a1m.p, am));
        return GC_OK;
      }
      return gc::assemble_ab(ctx, st.sd, st.ffoo.p, st.fofo.p, lam, ap, am, &st.e0);
    };
    auto use = [&](int i, const double *Y, double *eig) -> int {
      double wi = 0.0;
      GC_TRY(gc::integrand(ctx, st.sd, Y, eig, st.fofo.p, par.precision, &wi));
      if (w_out) w_out[i] = wi;
      if (stats_out) {
        std::vector<double> he(N);
        GC_CUDA(ctx, cudaMemcpyAsync(he.data(), eig, N * sizeof(double), cudaMemcpyDeviceToHost,
                                     ctx->stream));
        GC_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
        omega_stats(he, stats_out + (size_t)i * GC_OMEGA_STATS);
      }
      if (wt) sum += wt[i] * wi;
      return GC_OK;
    };
    GC_TRY(gc::erpa_solve_points(ctx, N, np, par.precision, fill, use));
    if (acc) *acc = sum;
    return GC_OK;
  }
  gc::DevBuf<double> ap, am, Y, eig;
  GC_TRY(ap.alloc(ctx, NN));
  GC_TRY(am.alloc(ctx, NN));
  GC_TRY(Y.alloc(ctx, NN));
  GC_TRY(eig.alloc(ctx, N));
  double sum = 0.0;
  for (int i = 0; i < np; ++i) {
    const double lam = x[i];
    if (par.affine) {
      gc::PhaseScope ph(ctx, GC_PHASE_ASSEMBLY);
      GC_TRY(gc::axpby_into(ctx, NN, 1.0 - lam, st.a0p.p, lam, st.a1p.p, ap.p));
      GC_TRY(gc::axpby_into(ctx, NN, 1.0 - lam, st.a0m.p, lam, st.a1m.p, am.p));
    } else {
      GC_TRY(gc::assemble_ab(ctx, st.sd, st.ffoo.p, st.fofo.p, lam, ap.p, am.p, &st.e0));
    }
    GC_TRY(gc::erpa_solve(ctx, N, ap.p, am.p, Y.p, eig.p, par.erpa_mode, par.precision));
    double wi = 0.0;
    GC_TRY(gc::integrand(ctx, st.sd, Y.p, eig.p, st.fofo.p, par.precision, &wi));
    if (w_out) w_out[i] = wi;
    if (stats_out) {
      std::vector<double> he(N);
      GC_CUDA(ctx, cudaMemcpyAsync(he.data(), eig.p, N * sizeof(double), cudaMemcpyDeviceToHost,
                                   ctx->stream));
      GC_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
      omega_stats(he, stats_out + (size_t)i * GC_OMEGA_STATS);
    }
    if (wt) sum += wt[i] * wi;
  }
  if (acc) *acc = sum;
  return GC_OK;
}

int check_systems(gc_context *ctx, int nsys, const gc_system *sys, const char *who) {
  for (int i = 0; i < nsys; ++i)
    if (!sys[i].cmo_dev || !sys[i].lfac_dev || !sys[i].occ || !sys[i].xone || !sys[i].indn ||
        sys[i].nbas <= 0 || sys[i].ndimx <= 0 || sys[i].rank <= 0)
      return gc::set_error(ctx, GC_EINVAL, "%s: system %d incomplete", who, i);
  return GC_OK;
}

int make_workers(gc_context *ctx, const gc_ac_params &par, int nw, std::vector<Worker> &ws) {
  ws.resize(nw);
  for (auto &w : ws) {
    GC_CUDA(ctx, cudaStreamCreateWithFlags(&w.stream, cudaStreamNonBlocking));
    GC_CUDA(ctx, cudaEventCreateWithFlags(&w.done, cudaEventDisableTiming));
    int r = gc_create(&w.ctx, ctx->device, w.stream);
    if (r != GC_OK) return gc::set_error(ctx, r, "batch: worker context");
    if (par.eig_emulation && (r = gc_set_eig_emulation(w.ctx, 1)) != GC_OK)
      return gc::set_error(ctx, r, "batch: %s", w.ctx->err.c_str());
    if (par.eig_refine > 0 && (r = gc_set_eig_refinement(w.ctx, par.eig_refine)) != GC_OK)
      return gc::set_error(ctx, r, "batch: %s", w.ctx->err.c_str());
  }
  return GC_OK;
}

void free_workers(std::vector<Worker> &ws) {
  for (auto &w : ws) {
    if (w.ctx) gc_destroy(w.ctx);
    if (w.stream) cudaStreamDestroy(w.stream);
    if (w.done) cudaEventDestroy(w.done);
  }
  ws.clear();
}

// Runs task(worker, k) for k = 0..ntask-1 on the workers (one host thread each,
// dynamic scheduling in the order given), ordered after the caller's stream; the
// caller's stream waits for all of them. A task's nonzero return stops the
// batch unless accept(status) says the status is recorded per task.
int run_tasks(gc_context *ctx, std::vector<Worker> &ws, int ntask,
              const std::function<int(Worker &, int)> &task,
              const std::function<bool(int)> &accept) {
  cudaEvent_t start;
  GC_CUDA(ctx, cudaEventCreateWithFlags(&start, cudaEventDisableTiming));
  GC_CUDA(ctx, cudaEventRecord(start, ctx->stream));
  for (auto &w : ws) {
    GC_CUDA(ctx, cudaStreamWaitEvent(w.stream, start, 0));
    w.ctx->phase_on = ctx->phase_on;
    w.ctx->eig_batch = ctx->eig_batch;
  }
  std::atomic<int> next{0};
  std::atomic<int> first_err{GC_OK};
  std::mutex err_mu;
  std::string err_msg;
  auto body = [&](Worker &w) {
    cudaSetDevice(ctx->device);
    for (;;) {
      int k = next.fetch_add(1);
      if (k >= ntask || first_err.load() != GC_OK) break;
      int r = task(w, k);
      if (r != GC_OK && !accept(r)) {
        int expected = GC_OK;
        if (first_err.compare_exchange_strong(expected, r)) {
          std::lock_guard<std::mutex> lk(err_mu);
          err_msg = "task " + std::to_string(k) + ": " + w.ctx->err;
        }
        break;
      }
    }
    cudaEventRecord(w.done, w.stream);
  };
  const int nw = (int)ws.size();
  std::vector<std::thread> th;
  for (int t = 1; t < nw; ++t) th.emplace_back(body, std::ref(ws[t]));
  body(ws[0]);
  for (auto &t : th) t.join();
  for (auto &w : ws) {
    cudaStreamWaitEvent(ctx->stream, w.done, 0);
    ctx->launches += w.ctx->launches;
    ctx->refine_solves += w.ctx->refine_solves;
    ctx->refine_fallbacks += w.ctx->refine_fallbacks;
    ctx->refine_max_cluster = std::max(ctx->refine_max_cluster, w.ctx->refine_max_cluster);
    ctx->eig_ms += w.ctx->eig_ms;
    ctx->eig_calls += w.ctx->eig_calls;
    gc::phase_collect(w.ctx, true);
    for (int p = 0; p < GC_PHASE_COUNT; ++p) {
      ctx->phase_ms[p] += w.ctx->phase_ms[p];
      ctx->phase_calls[p] += w.ctx->phase_calls[p];
      w.ctx->phase_ms[p] = 0.0;
      w.ctx->phase_calls[p] = 0;
    }
    w.ctx->launches = w.ctx->refine_solves = w.ctx->refine_fallbacks = w.ctx->eig_calls = 0;
    w.ctx->eig_ms = 0.0;
  }
  cudaEventDestroy(start);
  if (first_err.load() != GC_OK)
    return gc::set_error(ctx, first_err.load(), "%s", err_msg.c_str());
  return GC_OK;
}

std::vector<int> largest_first(int count, const int *idx, const gc_system *sys) {
  std::vector<int> order(count);
  std::iota(order.begin(), order.end(), 0);
  std::stable_sort(order.begin(), order.end(), [&](int a, int b) {
    return sys[idx ? idx[a] : a].ndimx > sys[idx ? idx[b] : b].ndimx;
  });
  return order;
}

}  // namespace

struct gc_ac_session {
  gc_context *ctx = nullptr;
  std::vector<gc_system> sys;
  gc_ac_params par{};
  std::vector<Worker> ws;
  std::vector<std::unique_ptr<SysState>> st;
};

extern "C" int gc_ac_energy_batched(gc_context *ctx, int nsys, const gc_system *sys,
                                    const gc_ac_params *par, double *ecorr, double *ecas,
                                    double *w_lambda, double *omega_st, int *status) {
  if (!ctx) return GC_EINVAL;
  if (nsys <= 0 || !sys || !par || !ecorr || !ecas || par->ngrid <= 0 || par->ngrid > 100)
    return gc::set_error(ctx, GC_EINVAL, "ac_energy_batched: bad arguments");
  GC_TRY(check_systems(ctx, nsys, sys, "ac_energy_batched"));
  std::vector<double> x(par->ngrid), wt(par->ngrid, 0.0);
  if (par->lambda) {
    for (int i = 0; i < par->ngrid; ++i) {
      x[i] = par->lambda[i];
      wt[i] = par->weight ? par->weight[i] : 0.0;
    }
  } else {
    gc_gauleg(0.0, 1.0, x.data(), wt.data(), par->ngrid);
  }
  std::vector<Worker> ws;
  int r = make_workers(ctx, *par, std::max(1, std::min(par->nstreams, nsys)), ws);
  if (r != GC_OK) {
    free_workers(ws);
    return r;
  }
  const std::vector<int> order = largest_first(nsys, nullptr, sys);
  auto task = [&](Worker &w, int k) {
    const int i = order[k];
    SysState st;
    int rr = build_state(w.ctx, sys[i], *par, st);
    double acc = 0.0;
    if (rr == GC_OK)
      rr = eval_points(w.ctx, sys[i], *par, st, par->ngrid, x.data(), wt.data(),
                       w_lambda ? w_lambda + (size_t)i * par->ngrid : nullptr,
                       omega_st ? omega_st + (size_t)i * par->ngrid * GC_OMEGA_STATS : nullptr,
                       &acc);
    ecorr[i] = acc;
    ecas[i] = st.e0;
    if (status) status[i] = rr;
    return rr;
  };
  r = run_tasks(ctx, ws, nsys, task, [&](int rr) { return status && (rr == GC_ENOTPD || rr == GC_ENONFINITE); });
  free_workers(ws);
  return r;
}

extern "C" int gc_ac_session_create(gc_context *ctx, int nsys, const gc_system *sys,
                                    const gc_ac_params *par, gc_ac_session **out) {
  if (!ctx) return GC_EINVAL;
  if (!out || nsys <= 0 || !sys || !par)
    return gc::set_error(ctx, GC_EINVAL, "ac_session_create: bad arguments");
  if (!par->affine)
    return gc::set_error(ctx, GC_EINVAL, "ac_session_create: the session keeps the affine form");
  GC_TRY(check_systems(ctx, nsys, sys, "ac_session_create"));
  auto s = std::make_unique<gc_ac_session>();
  s->ctx = ctx;
  s->sys.assign(sys, sys + nsys);
  s->par = *par;
  s->par.lambda = s->par.weight = nullptr;
  s->st.resize(nsys);
  for (auto &p : s->st) p = std::make_unique<SysState>();
  int r = make_workers(ctx, s->par, std::max(1, std::min(par->nstreams, nsys)), s->ws);
  if (r != GC_OK) {
    free_workers(s->ws);
    return r;
  }
  *out = s.release();
  return GC_OK;
}

extern "C" int gc_ac_session_points(gc_ac_session *s, int nidx, const int *idx, int npoints,
                                    const double *lambda, double *w_out, double *omega_st,
                                    double *ecas, int *status) {
  if (!s) return GC_EINVAL;
  gc_context *ctx = s->ctx;
  const int nsys = (int)s->sys.size();
  if (nidx <= 0 || !idx || npoints <= 0 || npoints > 100 || !lambda || !w_out)
    return gc::set_error(ctx, GC_EINVAL, "ac_session_points: bad arguments");
  std::vector<char> seen(nsys, 0);
  for (int k = 0; k < nidx; ++k) {
    if (idx[k] < 0 || idx[k] >= nsys || seen[idx[k]])
      return gc::set_error(ctx, GC_EINVAL, "ac_session_points: index %d out of range or repeated",
                           idx[k]);
    seen[idx[k]] = 1;
  }
  std::vector<int> order = largest_first(nidx, idx, s->sys.data());
  auto task = [&](Worker &w, int k) {
    const int j = order[k];  // position in idx and in the outputs
    const int i = idx[j];
    SysState &st = *s->st[i];
    if (!st.built && st.status == GC_OK) {
      st.status = build_state(w.ctx, s->sys[i], s->par, st);
      if (st.status == GC_OK) {
        if (cudaEventCreateWithFlags(&st.ready, cudaEventDisableTiming) != cudaSuccess ||
            cudaEventRecord(st.ready, w.stream) != cudaSuccess)
          st.status = gc::set_error(w.ctx, GC_ECUDA, "ac_session_points: state event");
      }
    } else if (st.built && st.ready) {
      // built on another worker's stream in an earlier call
      if (cudaStreamWaitEvent(w.stream, st.ready, 0) != cudaSuccess)
        return gc::set_error(w.ctx, GC_ECUDA, "ac_session_points: state event wait");
    }
    int rr = st.status;
    if (rr == GC_OK)
      rr = eval_points(w.ctx, s->sys[i], s->par, st, npoints, lambda, nullptr,
                       w_out + (size_t)j * npoints,
                       omega_st ? omega_st + (size_t)j * npoints * GC_OMEGA_STATS : nullptr,
                       nullptr);
    if (ecas) ecas[j] = st.e0;
    if (status) status[j] = rr;
    return rr;
  };
  return run_tasks(ctx, s->ws, nidx, task, [&](int rr) { return status && (rr == GC_ENOTPD || rr == GC_ENONFINITE); });
}

extern "C" int gc_ac_session_destroy(gc_ac_session *s) {
  if (!s) return GC_EINVAL;
  for (auto &w : s->ws) cudaStreamSynchronize(w.stream);
  s->st.clear();  // stream-ordered frees on the workers' streams
  for (auto &w : s->ws) cudaStreamSynchronize(w.stream);
  free_workers(s->ws);
  delete s;
  return GC_OK;
}
