// W(lambda) of ACEneERPA_FOFO for callers that cannot allocate device memory.
//
// Some hosts of this library cannot call cudaMalloc at the point where they
// need the integrand: a Fortran program whose device memory is owned by its
// own pool, or a process that must not grow its device footprint after
// start-up. For them this file provides gc_ace_ne_erpa_fofo_noalloc, a variant
// of the integrand that works only in a fixed, file-scope device array and in
// the buffers the caller passes (eigenvectors, eigenvalues, FOFO integrals).
//
// The variant fuses what gc_ace_ne_erpa_fofo stages in N x N scratch
// matrices: each block builds tiles of S = Yk Yk^T from the eigenvectors
// (kept modes only), multiplies them with the masked, CI-weighted FOFO
// integrals gathered on the fly and leaves one partial sum; a one-block kernel
// adds the partials. The summand is symmetric in the two pairs, so only tiles
// on or above the diagonal are formed and the off-diagonal ones count twice:
// about N^3 FP64 multiply-adds per call (a few seconds at the NDimX limit).
// FP64 throughout.
#include <mutex>

#include "gc_internal.cuh"

namespace {

constexpr int kMaxPairs = 16384;  // NDimX limit of this entry point
constexpr int kMaxBasis = 2048;   // NBasis limit
constexpr int kBlocks = 1024;     // persistent blocks, one partial sum each
constexpr int kTile = 16;

// scratch layout (bytes): IndN (2*kMaxPairs ints) | Occ (kMaxBasis doubles) |
// partial sums (kBlocks doubles) | result (1 double)
constexpr size_t kOffIndn = 0;
constexpr size_t kOffOcc = kOffIndn + sizeof(int) * 2 * kMaxPairs;
constexpr size_t kOffPart = kOffOcc + sizeof(double) * kMaxBasis;
constexpr size_t kOffRes = kOffPart + sizeof(double) * kBlocks;
constexpr size_t kScratchBytes = kOffRes + 256;
static_assert(kScratchBytes == 155904, "the array size stated in include/gammcor_gpu.h");

// Shared by every call on a device; it keeps the last call's contents.
static __device__ __align__(256) unsigned char g_noalloc_scratch[kScratchBytes];

const double kSmallE = 1e-3, kBigE = 1e8;  // abfofo.f90:3808

__device__ __forceinline__ double cicoef(double o) { return o >= 0.5 ? sqrt(o) : -sqrt(o); }
__device__ __forceinline__ int group(int i, int nin, int nocc) {
  return i < nin ? 0 : (i < nocc ? 1 : 2);
}

__global__ void k_integrand_tiles(int n, int nin, int nocc, int N, const double *__restrict__ Y,
                                  const double *__restrict__ eig,
                                  const double *__restrict__ fofo, unsigned char *scratch) {
  const int *indn = (const int *)(scratch + kOffIndn);
  const double *occ = (const double *)(scratch + kOffOcc);
  double *part = (double *)(scratch + kOffPart);
  __shared__ double yi[kTile][kTile + 1], yj[kTile][kTile + 1];
  __shared__ double red[kTile * kTile];
  const int tx = threadIdx.x % kTile, ty = threadIdx.x / kTile;
  const long long tiles = (N + kTile - 1) / kTile;
  const long long ntiles = tiles * (tiles + 1) / 2;  // tiles (ti, tj) with ti <= tj
  const size_t ld = (size_t)n * nocc;
  double acc = 0.0;
  for (long long t = blockIdx.x; t < ntiles; t += gridDim.x) {
    // t = tj (tj + 1) / 2 + ti, 0 <= ti <= tj
    long long tj = (long long)((sqrt(8.0 * (double)t + 1.0) - 1.0) * 0.5);
    while (tj * (tj + 1) / 2 > t) --tj;
    while ((tj + 1) * (tj + 2) / 2 <= t) ++tj;
    const long long ti = t - tj * (tj + 1) / 2;
    const int i0 = (int)ti * kTile, j0 = (int)tj * kTile;
    const double wt = ti == tj ? 1.0 : 2.0;  // off-diagonal tiles stand for their mirror too
    const int i = i0 + tx, j = j0 + ty;
    double s = 0.0;
    for (int v0 = 0; v0 < N; v0 += kTile) {
      // yi[r][c] = Yk[i0 + r, v0 + c], yj likewise; dropped modes read as 0.
      // Consecutive threads (tx) read consecutive rows of the column-major Y.
      int v = v0 + ty;
      double e = v < N ? eig[v] : 0.0;
      bool keep = v < N && e > kSmallE && e < kBigE;
      int ri = i0 + tx, rj = j0 + tx;
      yi[tx][ty] = (keep && ri < N) ? Y[ri + (size_t)v * N] : 0.0;
      yj[tx][ty] = (keep && rj < N) ? Y[rj + (size_t)v * N] : 0.0;
      __syncthreads();
#pragma unroll
      for (int c = 0; c < kTile; ++c) s += yi[tx][c] * yj[ty][c];
      __syncthreads();
    }
    if (i < N && j < N) {
      int p = indn[2 * i] - 1, q = indn[2 * i + 1] - 1;
      int r = indn[2 * j] - 1, u = indn[2 * j + 1] - 1;
      int gp = group(p, nin, nocc), gq = group(q, nin, nocc), gr = group(r, nin, nocc),
          gu = group(u, nin, nocc);
      if (!(gp == gq && gq == gr && gr == gu)) {
        double f = fofo[(size_t)(r + (size_t)u * n) * ld + p + (size_t)q * n];  // (rs|pq)
        double c = (cicoef(occ[p]) + cicoef(occ[q])) * (cicoef(occ[r]) + cicoef(occ[u]));
        double a = 2.0 * c * s;
        if (i == j) a -= occ[p] * (1.0 - occ[q]) + occ[q] * (1.0 - occ[p]);
        acc += wt * a * f;
      }
    }
  }
  red[threadIdx.x] = acc;
  __syncthreads();
  for (int w = kTile * kTile / 2; w > 0; w >>= 1) {
    if (threadIdx.x < w) red[threadIdx.x] += red[threadIdx.x + w];
    __syncthreads();
  }
  if (threadIdx.x == 0) part[blockIdx.x] = red[0];
}

__global__ void k_sum_partials(int nb, unsigned char *scratch) {
  const double *part = (const double *)(scratch + kOffPart);
  __shared__ double red[256];
  double s = 0.0;
  for (int b = threadIdx.x; b < nb; b += blockDim.x) s += part[b];
  red[threadIdx.x] = s;
  __syncthreads();
  for (int w = 128; w > 0; w >>= 1) {
    if (threadIdx.x < w) red[threadIdx.x] += red[threadIdx.x + w];
    __syncthreads();
  }
  if (threadIdx.x == 0) *(double *)(scratch + kOffRes) = red[0];
}

// Device address of the scratch array, looked up once per device.
std::mutex g_mu;
unsigned char *g_addr[64] = {};

int scratch_address(gc_context *ctx, unsigned char **out) {
  if (ctx->device < 0 || ctx->device >= 64)
    return gc::set_error(ctx, GC_EINVAL, "noalloc: device %d out of range", ctx->device);
  std::lock_guard<std::mutex> lk(g_mu);
  if (!g_addr[ctx->device]) {
    int cur = 0;
    GC_CUDA(ctx, cudaGetDevice(&cur));
    GC_CUDA(ctx, cudaSetDevice(ctx->device));
    void *p = nullptr;
    cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
    cudaSetDevice(cur);
    if (e != cudaSuccess)
      return gc::set_error(ctx, GC_ECUDA, "noalloc: cudaGetSymbolAddress: %s", cudaGetErrorString(e));
    g_addr[ctx->device] = (unsigned char *)p;
  }
  *out = g_addr[ctx->device];
  return GC_OK;
}

}  // namespace

extern "C" int gc_ace_ne_erpa_fofo_noalloc(gc_context *ctx, int nbas, int ninact, int nact,
                                           int ndimx, const double *occ_host,
                                           const int *indn_host, const double *eigvec_dev,
                                           const double *eig_dev, const double *fofo_dev,
                                           double *w_host) {
  if (!ctx) return GC_EINVAL;
  if (!occ_host || !indn_host || !eigvec_dev || !eig_dev || !fofo_dev || !w_host)
    return gc::set_error(ctx, GC_EINVAL, "noalloc integrand: null pointer");
  if (nbas <= 0 || nbas > kMaxBasis || ndimx <= 0 || ndimx > kMaxPairs || ninact < 0 || nact < 0 ||
      ninact + nact > nbas)
    return gc::set_error(ctx, GC_EINVAL,
                         "noalloc integrand: nbas=%d ndimx=%d outside the limits of the fixed "
                         "scratch (nbas <= %d, ndimx <= %d)",
                         nbas, ndimx, kMaxBasis, kMaxPairs);
  const int nocc = ninact + nact;
  for (int i = 0; i < ndimx; ++i) {
    int a = indn_host[2 * i] - 1, b = indn_host[2 * i + 1] - 1;
    if (a < 0 || b < 0 || a >= nbas || b >= nocc || a <= b)
      return gc::set_error(ctx, GC_EINVAL, "noalloc integrand: pair %d = (%d,%d) is not valid",
                           i + 1, a + 1, b + 1);
  }
  // The array's address is per device: the call runs on the context's device only.
  int cur = -1;
  GC_CUDA(ctx, cudaGetDevice(&cur));
  if (cur != ctx->device)
    return gc::set_error(ctx, GC_EINVAL,
                         "noalloc integrand: current device %d is not the context's device %d", cur,
                         ctx->device);
  unsigned char *scr = nullptr;
  GC_TRY(scratch_address(ctx, &scr));
  GC_CUDA(ctx, cudaMemcpyAsync(scr + kOffIndn, indn_host, sizeof(int) * 2 * ndimx,
                               cudaMemcpyHostToDevice, ctx->stream));
  GC_CUDA(ctx, cudaMemcpyAsync(scr + kOffOcc, occ_host, sizeof(double) * nbas,
                               cudaMemcpyHostToDevice, ctx->stream));
  const long long tn = (ndimx + kTile - 1) / kTile;
  const int nb = (int)std::min<long long>(kBlocks, tn * (tn + 1) / 2);
  k_integrand_tiles<<<nb, kTile * kTile, 0, ctx->stream>>>(nbas, ninact, nocc, ndimx, eigvec_dev,
                                                            eig_dev, fofo_dev, scr);
  GC_LAUNCHED(ctx);
  k_sum_partials<<<1, 256, 0, ctx->stream>>>(nb, scr);
  GC_LAUNCHED(ctx);
  GC_CUDA(ctx, cudaMemcpyAsync(w_host, scr + kOffRes, sizeof(double), cudaMemcpyDeviceToHost,
                               ctx->stream));
  GC_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
  return GC_OK;
}
