// Internal declarations shared by the translation units of libgammcor_gpu.
#pragma once

#include <cublas_v2.h>
#include <cuda_runtime.h>
#include <cusolverDn.h>

#include <cstdarg>
#include <functional>
#include <cstdint>
#include <cstdio>
#include <string>
#include <algorithm>
#include <numeric>
#include <vector>

#include "../../include/gammcor_gpu.h"

// One timed phase on a context's stream: events a (start) and b (end).
struct gc_phase_rec {
  int phase;
  cudaEvent_t a, b;
};

struct gc_context {
  int device = 0;
  cudaStream_t stream = nullptr;
  cublasHandle_t cublas = nullptr;
  cusolverDnHandle_t cusolver = nullptr;
  int *dev_info = nullptr;           // cuSOLVER info slot
  int *dev_flag = nullptr;           // device error flag for bounded waits
  int *dev_nonfinite = nullptr;      // count of non-finite matrix elements (ERPA input check)
  long long launches = 0;            // kernels of this library launched
  int eig_emulation = 0;             // cuSOLVER FP64 emulation strategy EAGER when 1
  int eig_refine = 2;                // refinement iterations of the FP32 eigensolve
  long long refine_solves = 0;       // GC_ERPA_CHOLESKY_REFINED solves
  long long refine_fallbacks = 0;    // of which fell back to dsyevd
  int refine_max_cluster = 0;        // largest cluster diagonalised in a block
  int chol_blocked = 1;              // blocked Cholesky with tensor-core trailing updates
  unsigned long long wait_ns = 1000000000ull;  // limit of the tensor-core GEMMs' pipeline waits
  int oz_tile = 0;  // column tile of the sliced GEMMs: 0 chosen per product, else 64/96/128
  int eig_batch = 1;  // batch the FP32 eigensolves of a system's points (gc_set_eig_batch)
  cudaEvent_t eig_ev[2] = {nullptr, nullptr};  // around each cuSOLVER eigensolve
  double eig_ms = 0.0;               // device time of the cuSOLVER eigensolves (dsyevd, ssyevd)
  long long eig_calls = 0;
  int phase_on = 0;                  // gc_set_phase_timing
  double phase_ms[GC_PHASE_COUNT] = {};
  long long phase_calls[GC_PHASE_COUNT] = {};
  std::vector<gc_phase_rec> phase_pending;  // recorded, not yet read
  std::vector<cudaEvent_t> phase_pool;      // timing events ready for reuse
  std::string err;
};

namespace gc {

// Phase timing: a scope records an event pair around a phase on the context's
// stream when timing is on; completed pairs are added to the phase totals
// without waiting (phase_collect(ctx, false)) or after the stream has passed them
// (phase_collect(ctx, true)).
void phase_collect(gc_context *ctx, bool wait);
class PhaseScope {
 public:
  PhaseScope(gc_context *ctx, int phase);
  ~PhaseScope();
  PhaseScope(const PhaseScope &) = delete;
  PhaseScope &operator=(const PhaseScope &) = delete;

 private:
  gc_context *ctx_;
  int phase_;
  cudaEvent_t a_ = nullptr;
};

// Status propagation --------------------------------------------------------
int set_error(gc_context *ctx, int code, const char *fmt, ...);

#define GC_CUDA(ctx, call)                                                        \
  do {                                                                            \
    cudaError_t e_ = (call);                                                      \
    if (e_ != cudaSuccess)                                                        \
      return gc::set_error((ctx), GC_ECUDA, "%s:%d %s: %s", __FILE__, __LINE__,  \
                           #call, cudaGetErrorString(e_));                        \
  } while (0)

#define GC_CUBLAS(ctx, call)                                                      \
  do {                                                                            \
    cublasStatus_t s_ = (call);                                                   \
    if (s_ != CUBLAS_STATUS_SUCCESS)                                              \
      return gc::set_error((ctx), GC_ECUBLAS, "%s:%d %s: status %d", __FILE__,   \
                           __LINE__, #call, (int)s_);                             \
  } while (0)

#define GC_CUSOLVER(ctx, call)                                                    \
  do {                                                                            \
    cusolverStatus_t s_ = (call);                                                 \
    if (s_ != CUSOLVER_STATUS_SUCCESS)                                            \
      return gc::set_error((ctx), GC_ECUSOLVER, "%s:%d %s: status %d", __FILE__, \
                           __LINE__, #call, (int)s_);                             \
  } while (0)

#define GC_TRY(call)                 \
  do {                               \
    int r_ = (call);                 \
    if (r_ != GC_OK) return r_;      \
  } while (0)

#define GC_LAUNCHED(ctx)                                                           \
  do {                                                                             \
    (ctx)->launches++;                                                             \
    cudaError_t e_ = cudaGetLastError();                                           \
    if (e_ != cudaSuccess)                                                         \
      return gc::set_error((ctx), GC_ECUDA, "%s:%d launch: %s", __FILE__, __LINE__, \
                           cudaGetErrorString(e_));                                \
  } while (0)

// Stream-ordered device buffer owned by a context call.
template <typename T>
struct DevBuf {
  T *p = nullptr;
  size_t n = 0;
  cudaStream_t s = nullptr;
  DevBuf() = default;
  DevBuf(const DevBuf &) = delete;
  DevBuf &operator=(const DevBuf &) = delete;
  ~DevBuf() { release(); }
  void release() {
    if (p) cudaFreeAsync(p, s);
    p = nullptr;
    n = 0;
  }
  int alloc(gc_context *ctx, size_t count) {
    release();
    s = ctx->stream;
    n = count;
    if (count == 0) return GC_OK;
    cudaError_t e = cudaMallocAsync((void **)&p, count * sizeof(T), ctx->stream);
    if (e != cudaSuccess) {
      p = nullptr;
      return set_error(ctx, GC_ENOMEM, "cudaMallocAsync(%zu bytes): %s", count * sizeof(T),
                       cudaGetErrorString(e));
    }
    return GC_OK;
  }
  int upload(gc_context *ctx, const T *host, size_t count) {
    GC_TRY(alloc(ctx, count));
    if (count)
      GC_CUDA(ctx, cudaMemcpyAsync(p, host, count * sizeof(T), cudaMemcpyHostToDevice, ctx->stream));
    return GC_OK;
  }
};

inline unsigned ceil_div(size_t a, size_t b) { return (unsigned)((a + b - 1) / b); }

// The FP64-accurate sliced tensor-core precisions (4, 5 or 6 integer BF16 slices).
inline bool is_sliced(int precision) {
  return precision == GC_PREC_FP64TC4 || precision == GC_PREC_FP64TC5 ||
         precision == GC_PREC_FP64TC6;
}

// Per-system description resident on the device ------------------------------
struct SysDev {
  int n = 0, nin = 0, nact = 0, nocc = 0, ndimx = 0;
  DevBuf<double> occ;      // (n)
  DevBuf<int> grp;         // (n) 0 inactive, 1 active, 2 virtual
  DevBuf<int> pair_p;      // (ndimx) 0-based p of pair (p > q)
  DevBuf<int> pair_q;      // (ndimx)
  DevBuf<double> h;        // (n, n) symmetrised one-electron MO matrix
  DevBuf<double> rv;       // RDM2val (nocc^4), RV[i + nocc*(j + nocc*(k + nocc*l))]
  // Per pair i = (p, q), with the CI coefficients C = sign(n - 1/2) sqrt(n) of
  // ACEneERPA_FOFO / AB_CAS_FOFO: C_p + C_q, C_p - C_q and their reciprocals (0 where
  // the sum or difference is 0), and n_p (1 - n_q) + n_q (1 - n_p). Computed once on
  // the host, so that the element kernels spend the narrow FP64 pipe on products only.
  DevBuf<double> cpl, cmi, rpl, rmi, dnq;  // (ndimx)
};

// IndN (2 x N, 1-based) reordered with q outer and p inner: consecutive pairs then
// address consecutive elements p + q n of a FOFO record, so the element kernels'
// gathers are coalesced. A+-B, the ERPA problem and W are invariant under a common
// permutation of the pairs, so paths that return only energies may use this order.
std::vector<int> coalesced_pair_order(const int *indn, int ndimx);

// Host-side setup of SysDev (pairs, groups, RDM2val).
int sys_upload(gc_context *ctx, SysDev &sd, int nbas, int ninact, int nact, int ndimx,
               const double *occ, const double *xone, const int *indn, const double *rdm2act);

// Assembly (gc_assembly.cu).
// ab1 = 1: the AB1 form of AB_CAS_FOFO (the lambda derivative, symmetrised).
int assemble_ab(gc_context *ctx, const SysDev &sd, const double *ffoo, const double *fofo,
                double alpha, double *abplus, double *abmin, double *etot_host, int ab1 = 0);
// One-electron matrix of sd rotated in place: h <- URe h URe^T, symmetrised.
int rotate_h(gc_context *ctx, SysDev &sd, const double *ure_host);

// ERPA (gc_erpa.cu).
// gemm_precision selects the arithmetic of the similarity and back-transform
// products of the Cholesky form (GC_PREC_FP64 or a sliced FP64-accurate mode).
// aplsqrt_out (GC_ERPA_SYMM1 only): A+^1/2 is written over abplus, as ERPASYMM1 does.
int erpa_solve(gc_context *ctx, int N, double *abplus, double *abmin, double *eigvec,
               double *eig, int mode, int gemm_precision, bool aplsqrt_out = false);

// A+ = L L^T (L lower, upper triangle zeroed) and the eigenpairs of L^T A- L: U (N x N,
// column k = eigenvector k), w (eigenvalues; ascending except in the refined mode).
// A+ and A- are read, symmetrised copies are used. mode: GC_ERPA_CHOLESKY (dsyevd) or
// GC_ERPA_CHOLESKY_REFINED; prec: arithmetic of the products (FP64 or FP64TC5/6).
int chol_eig(gc_context *ctx, int N, const double *abplus, const double *abmin, double *L,
             double *U, double *w, int mode, int prec);

// ERPAVEC (gc_erpavec.cu): A+- symmetrised in place, Y (N x N) and omega (N).
int erpavec(gc_context *ctx, int N, double *abplus, double *abmin, double *Y, double *eig);

// Integrand (gc_integrand.cu).
// ERPA solutions of np points in the refined Cholesky form with sliced products: the
// Cholesky factors of all points in one batched launch chain and their FP32 eigensolves
// in one batched call. fill(k, ap, am) writes A+B and A-B of point k into the two N x N
// buffers it is given, use(k, Y, eig) consumes that point's Y (N x N) and omega (N).
int erpa_solve_points(gc_context *ctx, int N, int np, int prec,
                      const std::function<int(int, double *, double *)> &fill,
                      const std::function<int(int, const double *, double *)> &use);

int integrand(gc_context *ctx, const SysDev &sd, const double *eigvec, const double *eig,
              const double *fofo, int precision, double *w_host);

// Elementwise helpers (gc_api.cu).
int axpby_into(gc_context *ctx, size_t count, double a, const double *x, double b,
               const double *y, double *out);

}  // namespace gc
