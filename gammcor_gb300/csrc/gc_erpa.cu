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
#include <functional>

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

// Copy the lower triangle onto the upper one.
__global__ void k_mirror_lower(int N, double *__restrict__ a) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  int j = blockIdx.y * blockDim.y + threadIdx.y;
  if (i >= N || j >= N || j <= i) return;
  a[i + (size_t)j * N] = a[j + (size_t)i * N];
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
  __shared__ double sc;  // the column's factor, once per block
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  const int k = blockIdx.y;
  if (threadIdx.x == 0) sc = sqrt(fabs(e[k]));
  __syncthreads();
  if (i >= N) return;
  out[i + (size_t)k * N] = V[i + (size_t)k * N] * sc;
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
  // the column's factor is formed once per block (two FP64 square roots and a division
  // are many instructions of GB300's narrow FP64 pipe)
  __shared__ double sc;
  const int nu = blockIdx.y;
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  const double w2 = eig[nu];
  if (!(w2 > kSmall)) return;
  if (threadIdx.x == 0) sc = 1.0 / sqrt(2.0 * sqrt(w2));
  __syncthreads();
  if (i < N) Y[(size_t)nu * N + i] *= sc;
}

// *count += number of non-finite elements of a and b (n elements each).
__global__ void k_count_nonfinite(size_t n, const double *__restrict__ a,
                                  const double *__restrict__ b, int *count) {
  int c = 0;
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n;
       i += (size_t)gridDim.x * blockDim.x)
    c += !isfinite(a[i]) + !isfinite(b[i]);
  for (int off = 16; off > 0; off >>= 1) c += __shfl_down_sync(0xffffffffu, c, off);
  if ((threadIdx.x & 31) == 0 && c) atomicAdd(count, c);
}

__global__ void k_sqrt_eig(int N, double *__restrict__ eig) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < N && eig[i] > kSmall) eig[i] = sqrt(eig[i]);
}

// Adds the device time between the context's two eigensolve events (recorded around
// the cuSOLVER call, already complete: the caller synchronised).
int add_eig_time(gc_context *ctx) {
  float ms = 0.f;
  GC_CUDA(ctx, cudaEventElapsedTime(&ms, ctx->eig_ev[0], ctx->eig_ev[1]));
  ctx->eig_ms += ms;
  ctx->eig_calls++;
  return GC_OK;
}

int syevd(gc_context *ctx, int N, double *A, double *w) {
  int lwork = 0;
  GC_CUSOLVER(ctx, cusolverDnDsyevd_bufferSize(ctx->cusolver, CUSOLVER_EIG_MODE_VECTOR,
                                               CUBLAS_FILL_MODE_LOWER, N, A, N, w, &lwork));
  gc::DevBuf<double> work;
  GC_TRY(work.alloc(ctx, std::max(lwork, 1)));
  GC_CUDA(ctx, cudaEventRecord(ctx->eig_ev[0], ctx->stream));
  GC_CUSOLVER(ctx, cusolverDnDsyevd(ctx->cusolver, CUSOLVER_EIG_MODE_VECTOR, CUBLAS_FILL_MODE_LOWER,
                                    N, A, N, w, work.p, lwork, ctx->dev_info));
  GC_CUDA(ctx, cudaEventRecord(ctx->eig_ev[1], ctx->stream));
  int info = 0;
  GC_CUDA(ctx, cudaMemcpyAsync(&info, ctx->dev_info, sizeof(int), cudaMemcpyDeviceToHost,
                               ctx->stream));
  GC_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
  GC_TRY(add_eig_time(ctx));
  if (info != 0) return gc::set_error(ctx, GC_ECUSOLVER, "dsyevd info=%d (N=%d)", info, N);
  return GC_OK;
}


// ---- FP32 eigensolve refined to FP64 accuracy --------------------------------
//
// M = L^T A- L is diagonalised in FP32 (ssyevd on M rounded to FP32); the FP32
// eigenvectors X are then refined against the FP64 M. One iteration forms
//   G = X^T X,  S = X^T (M X),  lambda_i = S_ii / G_ii,
// groups indices into clusters (maximal runs of neighbours k, k+1 whose Rayleigh
// quotients differ by at most max(c_k, c_k+1) / kTau, c_j the largest coupling
// |S_ij - (lambda_i + lambda_j) / 2 G_ij| of column j),
// diagonalises each cluster block exactly in FP64 (Cholesky of G_CC, cyclic Jacobi,
// back-substitution: V_C^T G_CC V_C = I, V_C^T S_CC V_C diagonal), rotates G and S
// by the block-diagonal V, and updates
//   X <- X V (I + E),  E_ij = (S'_ij - lambda'_j G'_ij) / (lambda'_j - lambda'_i)
// across clusters and E = (I - G') / 2 inside them (first order in the residual,
// so every cross-cluster |E_ij| <= kTau), with the second-order term -E E^T / 2
// added to I + E so that the update keeps X orthonormal to third order. This is
// the iterative refinement of Ogita and Aishima (Japan J. Indust. Appl. Math. 35,
// 2018) with the clustered eigenvalues treated as exact small blocks. The
// eigenvalues returned are the Rayleigh quotients of the updated vectors to second
// order in E (an O(N^2) reduction; the quotients before the update inherit the
// FP32 vectors' error squared, ~1e-6 relative on cuSOLVER's ssyevd output).
// W(lambda) depends on the eigenvectors only through sum_nu f(omega_nu) y_nu y_nu^T,
// so rotations inside a cluster of (near-)equal eigenvalues do not matter; the
// block solve only has to be exact.
constexpr int kMaxCluster = 64;
constexpr double kTau = 0.05;

__global__ void k_d2f(size_t n, const double *__restrict__ a, float *__restrict__ b) {
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n;
       i += (size_t)gridDim.x * blockDim.x)
    b[i] = (float)a[i];
}

__global__ void k_f2d(size_t n, const float *__restrict__ a, double *__restrict__ b) {
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n;
       i += (size_t)gridDim.x * blockDim.x)
    b[i] = (double)a[i];
}

// lam_i = S_ii / G_ii; the diagonals themselves into dS, dG when given.
__global__ void k_rayleigh(int N, const double *__restrict__ G, const double *__restrict__ S,
                           double *__restrict__ lam, double *__restrict__ dS,
                           double *__restrict__ dG) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= N) return;
  const double s = S[i + (size_t)i * N], g = G[i + (size_t)i * N];
  lam[i] = s / g;
  if (dS) {
    dS[i] = s;
    dG[i] = g;
  }
}

// Rayleigh quotient of the updated column x'_j = X t_j (t_j = e_j + E e_j in the
// rotated basis) to second order in E: x'^T M x' = t^T S t and x'^T x' = t^T G t with
// the terms E_ij E_kj S_ik (i != k, third order) dropped; the -E E^T / 2 term of the
// update changes the quotient only at third order. One block per column j.
__global__ void k_eig_update(int N, const double *__restrict__ G, const double *__restrict__ S,
                             const double *__restrict__ T, const double *__restrict__ dS,
                             const double *__restrict__ dG, double *__restrict__ lam) {
  __shared__ double rn[256], rd[256];
  const int j = blockIdx.x;
  const size_t c = (size_t)j * N;
  double num = 0.0, den = 0.0;
  for (int i = threadIdx.x; i < N; i += blockDim.x) {
    if (i == j) continue;
    const double e = T[c + i];
    num += e * (2.0 * S[c + i] + e * dS[i]);
    den += e * (2.0 * G[c + i] + e * dG[i]);
  }
  rn[threadIdx.x] = num;
  rd[threadIdx.x] = den;
  __syncthreads();
  for (int w = blockDim.x / 2; w > 0; w >>= 1) {
    if (threadIdx.x < w) {
      rn[threadIdx.x] += rn[threadIdx.x + w];
      rd[threadIdx.x] += rd[threadIdx.x + w];
    }
    __syncthreads();
  }
  if (threadIdx.x == 0) {
    const double ejj = T[c + j];
    lam[j] = (dS[j] * (1.0 + 2.0 * ejj) + rn[0]) / (dG[j] * (1.0 + 2.0 * ejj) + rd[0]);
  }
}

// colm[j] = max over i != j of |S_ij - (lam_i + lam_j) / 2 G_ij|, the largest
// first-order coupling of column j (symmetric in i, j). One block per column.
__global__ void k_col_coupling(int N, const double *__restrict__ G, const double *__restrict__ S,
                               const double *__restrict__ lam, double *__restrict__ colm) {
  __shared__ double red[256];
  const int j = blockIdx.x;
  const size_t c = (size_t)j * N;
  const double lj = lam[j];
  double m = 0.0;
  for (int i = threadIdx.x; i < N; i += blockDim.x)
    if (i != j) m = fmax(m, fabs(S[c + i] - 0.5 * (lam[i] + lj) * G[c + i]));
  red[threadIdx.x] = m;
  __syncthreads();
  for (int w = blockDim.x / 2; w > 0; w >>= 1) {
    if (threadIdx.x < w) red[threadIdx.x] = fmax(red[threadIdx.x], red[threadIdx.x + w]);
    __syncthreads();
  }
  if (threadIdx.x == 0) colm[j] = red[0];
}

// Neighbours k, k+1 belong to one cluster when their Rayleigh quotients differ by
// at most max(colm_k, colm_k+1) / kTau (the first-order update of that pair would
// exceed kTau). cstart[k], csize[k]: the run around k. A run longer than
// kMaxCluster sets bit 1 of *flag (the solve then falls back to dsyevd).
__device__ __forceinline__ bool joined(const double *lam, const double *colm, int k) {
  return fabs(lam[k + 1] - lam[k]) <= fmax(colm[k], colm[k + 1]) / kTau;
}

__global__ void k_clusters(int N, const double *__restrict__ lam, const double *__restrict__ colm,
                           int *__restrict__ cstart, int *__restrict__ csize, int *flag) {
  int k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= N) return;
  int s = k;
  while (s > 0 && k - s < kMaxCluster - 1 && joined(lam, colm, s - 1)) --s;
  bool too_long = s > 0 && k - s == kMaxCluster - 1 && joined(lam, colm, s - 1);
  int e = k + 1;
  while (e < N && e - s < kMaxCluster && joined(lam, colm, e - 1)) ++e;
  too_long = too_long || (e < N && e - s == kMaxCluster && joined(lam, colm, e - 1));
  if (too_long) atomicOr(flag, 1);
  cstart[k] = s;
  csize[k] = e - s;
}

constexpr int kLd = kMaxCluster + 1;  // padded row of the shared blocks
constexpr size_t kClusterSmem = 3 * (size_t)kMaxCluster * kLd * sizeof(double);
constexpr size_t kBlkSmem = 2 * (size_t)kMaxCluster * kLd * sizeof(double);

// One block of kMaxCluster threads per cluster of size >= 2 (block k where
// cstart[k] == k): V_C with V_C^T G_CC V_C = I and V_C^T S_CC V_C diagonal, stored
// as rows k..k+m-1 of Vbuf (N x kMaxCluster, row-major). Failures set bit 2 of *flag.
__global__ void __launch_bounds__(kMaxCluster) k_cluster_eig(
    int N, const double *__restrict__ G, const double *__restrict__ S, const int *__restrict__ cstart,
    const int *__restrict__ csize, double *__restrict__ Vbuf, int *flag, int *maxc) {
  const int k = blockIdx.x;
  const int m = csize[k];
  if (cstart[k] != k || m < 2) return;
  extern __shared__ double sm[];
  double *A = sm, *C = sm + kMaxCluster * kLd, *V = sm + 2 * kMaxCluster * kLd;
  __shared__ double red[2][kMaxCluster];
  const int l = threadIdx.x;
  if (l < m)
    for (int b = 0; b < m; ++b) {
      size_t e = (size_t)(k + l) + (size_t)(k + b) * N;
      A[l * kLd + b] = S[e];
      C[l * kLd + b] = G[e];
      V[l * kLd + b] = l == b ? 1.0 : 0.0;
    }
  __syncthreads();
  // G_CC = C C^T (lower, left-looking)
  for (int j = 0; j < m; ++j) {
    if (l == 0) {
      double d = C[j * kLd + j];
      for (int q = 0; q < j; ++q) d -= C[j * kLd + q] * C[j * kLd + q];
      C[j * kLd + j] = d > 0.0 ? sqrt(d) : -1.0;
    }
    __syncthreads();
    const double cjj = C[j * kLd + j];
    if (!(cjj > 0.0)) {
      if (l == 0) atomicOr(flag, 2);
      return;  // uniform: every thread read the same cjj
    }
    if (l > j && l < m) {
      double v = C[l * kLd + j];
      for (int q = 0; q < j; ++q) v -= C[l * kLd + q] * C[j * kLd + q];
      C[l * kLd + j] = v / cjj;
    }
    __syncthreads();
  }
  // A <- C^-1 A (thread = column), then A <- A C^-T (thread = row), symmetrise
  if (l < m)
    for (int i = 0; i < m; ++i) {
      double v = A[i * kLd + l];
      for (int q = 0; q < i; ++q) v -= C[i * kLd + q] * A[q * kLd + l];
      A[i * kLd + l] = v / C[i * kLd + i];
    }
  __syncthreads();
  if (l < m)
    for (int b = 0; b < m; ++b) {
      double v = A[l * kLd + b];
      for (int q = 0; q < b; ++q) v -= A[l * kLd + q] * C[b * kLd + q];
      A[l * kLd + b] = v / C[b * kLd + b];
    }
  __syncthreads();
  if (l < m)
    for (int b = l + 1; b < m; ++b) {
      double v = 0.5 * (A[l * kLd + b] + A[b * kLd + l]);
      A[l * kLd + b] = v;
      A[b * kLd + l] = v;
    }
  __syncthreads();
  // cyclic Jacobi (Golub and Van Loan, Alg. 8.5.3), at most 40 sweeps
  bool converged = false;
  for (int sweep = 0; sweep < 40; ++sweep) {
    double off = 0.0, tot = 0.0;
    if (l < m)
      for (int b = 0; b < m; ++b) {
        double v = A[l * kLd + b] * A[l * kLd + b];
        tot += v;
        if (b != l) off += v;
      }
    red[0][l] = off;
    red[1][l] = tot;
    __syncthreads();
    for (int w = kMaxCluster / 2; w > 0; w >>= 1) {
      if (l < w) {
        red[0][l] += red[0][l + w];
        red[1][l] += red[1][l + w];
      }
      __syncthreads();
    }
    converged = red[0][0] <= 1e-30 * red[1][0];
    __syncthreads();
    if (converged) break;
    for (int p = 0; p < m - 1; ++p)
      for (int q = p + 1; q < m; ++q) {
        const double apq = A[p * kLd + q];
        if (apq == 0.0) continue;  // uniform: all threads read the same value
        const double theta = (A[q * kLd + q] - A[p * kLd + p]) / (2.0 * apq);
        const double t = (theta >= 0.0 ? 1.0 : -1.0) / (fabs(theta) + sqrt(theta * theta + 1.0));
        const double c = 1.0 / sqrt(t * t + 1.0), sn = t * c;
        __syncthreads();
        if (l < m) {
          double aip = A[l * kLd + p], aiq = A[l * kLd + q];
          A[l * kLd + p] = c * aip - sn * aiq;
          A[l * kLd + q] = sn * aip + c * aiq;
        }
        __syncthreads();
        if (l < m) {
          double api = A[p * kLd + l], aqi = A[q * kLd + l];
          A[p * kLd + l] = c * api - sn * aqi;
          A[q * kLd + l] = sn * api + c * aqi;
          double vip = V[l * kLd + p], viq = V[l * kLd + q];
          V[l * kLd + p] = c * vip - sn * viq;
          V[l * kLd + q] = sn * vip + c * viq;
        }
        __syncthreads();
      }
  }
  if (!converged) {
    if (l == 0) atomicOr(flag, 2);
    return;
  }
  // Order the block's eigenpairs by eigenvalue (Jacobi leaves them unordered): the
  // next iteration groups clusters from neighbouring indices, which must then hold
  // neighbouring eigenvalues.
  __shared__ int perm[kMaxCluster];
  if (l == 0) {
    for (int b = 0; b < m; ++b) perm[b] = b;
    for (int b = 1; b < m; ++b) {  // insertion sort on the diagonal of A
      const int pb = perm[b];
      const double v = A[pb * kLd + pb];
      int q = b - 1;
      while (q >= 0 && A[perm[q] * kLd + perm[q]] > v) {
        perm[q + 1] = perm[q];
        --q;
      }
      perm[q + 1] = pb;
    }
  }
  __syncthreads();
  if (l < m)
    for (int b = 0; b < m; ++b) A[l * kLd + b] = V[l * kLd + perm[b]];
  __syncthreads();
  if (l < m)
    for (int b = 0; b < m; ++b) V[l * kLd + b] = A[l * kLd + b];
  __syncthreads();
  // V_C = C^-T V (thread = column, backward substitution)
  if (l < m)
    for (int i = m - 1; i >= 0; --i) {
      double v = V[i * kLd + l];
      for (int q = i + 1; q < m; ++q) v -= C[q * kLd + i] * V[q * kLd + l];
      V[i * kLd + l] = v / C[i * kLd + i];
    }
  __syncthreads();
  if (l < m)
    for (int b = 0; b < m; ++b) Vbuf[(size_t)(k + l) * kMaxCluster + b] = V[l * kLd + b];
  if (l == 0) atomicMax(maxc, m);
}

// X[:, C] <- X[:, C] V_C for every cluster C, rows 0..nrows-1 (kMaxCluster rows
// per block; the block of X and V_C staged in shared memory).
__global__ void __launch_bounds__(kMaxCluster) k_blk_right(
    int nrows, double *__restrict__ X, long long ld, const int *__restrict__ cstart,
    const int *__restrict__ csize, const double *__restrict__ Vbuf) {
  const int k = blockIdx.y;
  const int m = csize[k];
  if (cstart[k] != k || m < 2) return;
  extern __shared__ double sm[];
  double *Vs = sm, *Xs = sm + kMaxCluster * kLd;
  const int t = threadIdx.x;
  for (int b = 0; b < m; ++b)
    if (t < m) Vs[b * kLd + t] = Vbuf[(size_t)(k + b) * kMaxCluster + t];
  const int i = blockIdx.x * kMaxCluster + t;
  if (i < nrows)
    for (int b = 0; b < m; ++b) Xs[t * kLd + b] = X[i + (size_t)(k + b) * ld];
  __syncthreads();
  if (i >= nrows) return;
  for (int j = 0; j < m; ++j) {
    double v = 0.0;
    for (int b = 0; b < m; ++b) v += Xs[t * kLd + b] * Vs[b * kLd + j];
    X[i + (size_t)(k + j) * ld] = v;
  }
}

// X[C, :] <- V_C^T X[C, :] (trans = 1) or V_C X[C, :] (trans = 0), columns 0..ncols-1.
__global__ void __launch_bounds__(kMaxCluster) k_blk_left(
    int ncols, double *__restrict__ X, long long ld, int trans, const int *__restrict__ cstart,
    const int *__restrict__ csize, const double *__restrict__ Vbuf) {
  const int k = blockIdx.y;
  const int m = csize[k];
  if (cstart[k] != k || m < 2) return;
  extern __shared__ double sm[];
  double *Vs = sm, *Xs = sm + kMaxCluster * kLd;
  const int t = threadIdx.x;
  // Vs[a][b] = (trans ? V^T : V)[a][b]
  for (int a = 0; a < m; ++a)
    if (t < m)
      Vs[a * kLd + t] = trans ? Vbuf[(size_t)(k + t) * kMaxCluster + a]
                              : Vbuf[(size_t)(k + a) * kMaxCluster + t];
  const int c = blockIdx.x * kMaxCluster + t;
  if (c < ncols)
    for (int b = 0; b < m; ++b) Xs[t * kLd + b] = X[(size_t)(k + b) + (size_t)c * ld];
  __syncthreads();
  if (c >= ncols) return;
  for (int a = 0; a < m; ++a) {
    double v = 0.0;
    for (int b = 0; b < m; ++b) v += Vs[a * kLd + b] * Xs[t * kLd + b];
    X[(size_t)(k + a) + (size_t)c * ld] = v;
  }
}

// E from the rotated G, S and their Rayleigh quotients. Below the diagonal
// E_ij = (S_ij - lam_j G_ij) / (lam_j - lam_i); above it E_ij = -G_ij - E_ji, so that
// (I + E)^T G (I + E) = I holds to first order whatever rounding made S slightly
// unsymmetric (for nearly equal lam that rounding, divided by the gap, then turns
// the pair instead of tilting it). Inside a cluster E = (I - G) / 2. A cross-cluster
// |E| above 1/2 (first order no longer valid) sets bit 4 of *flag.
__global__ void k_form_update(int N, const double *__restrict__ G, const double *__restrict__ S,
                              const double *__restrict__ lam, const int *__restrict__ cstart,
                              double *__restrict__ E, int *flag) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  const int j = blockIdx.y;
  if (i >= N) return;
  const size_t e = i + (size_t)j * N;
  double t;
  if (cstart[i] == cstart[j]) {
    t = 0.5 * ((i == j ? 1.0 : 0.0) - G[e]);
  } else {
    const int r = i > j ? i : j, c = i > j ? j : i;  // lower-triangle element (r, c)
    const size_t el = r + (size_t)c * N;
    const double elow = (S[el] - lam[c] * G[el]) / (lam[c] - lam[r]);
    if (!(fabs(elow) <= 0.5)) atomicOr(flag, 4);
    t = i > j ? elow : -G[e] - elow;
    if (!(fabs(t) <= 1.0)) t = 0.0;
  }
  E[e] = t;
}

// T = I + E - D / 2 with D = E E^T: the second-order term that keeps X (I + E)
// orthonormal to third order (E is antisymmetric to first order, so E E^T stands
// in for E^T E). In place over E.
__global__ void k_second_order(size_t NN, int N, double *__restrict__ E,
                               const double *__restrict__ D) {
  for (size_t e = blockIdx.x * (size_t)blockDim.x + threadIdx.x; e < NN;
       e += (size_t)gridDim.x * blockDim.x) {
    const size_t j = e / N, i = e - j * N;
    E[e] = (i == j ? 1.0 : 0.0) + E[e] - 0.5 * D[e];
  }
}

// Normalise every column of X to unit length (one block per column).
__global__ void k_colnorm(int N, double *__restrict__ X) {
  __shared__ double red[256];
  double *x = X + (size_t)blockIdx.x * N;
  double s = 0.0;
  for (int i = threadIdx.x; i < N; i += blockDim.x) s += x[i] * x[i];
  red[threadIdx.x] = s;
  __syncthreads();
  for (int w = blockDim.x / 2; w > 0; w >>= 1) {
    if (threadIdx.x < w) red[threadIdx.x] += red[threadIdx.x + w];
    __syncthreads();
  }
  const double f = red[0] > 0.0 ? 1.0 / sqrt(red[0]) : 0.0;
  for (int i = threadIdx.x; i < N; i += blockDim.x) x[i] *= f;
}

// C (m x n, ldc = m) = op(A) B with op(A) = A (transA = 0, A m x k) or A^T (A k x m),
// B k x n, all leading dimensions equal to the row count N of the square case.
int product(gc_context *ctx, int prec, bool transA, int m, int n, int k, const double *A,
            int lda, const double *B, int ldb, double *C, int ldc) {
  if (gc::is_sliced(prec))
    return gc::tc_gemm_strided(ctx, prec, m, n, k, A, transA ? lda : 1, transA ? 1 : lda, B, ldb,
                               1, C, ldc);
  const double one = 1.0, zero = 0.0;
  GC_CUBLAS(ctx, cublasDgemm(ctx->cublas, transA ? CUBLAS_OP_T : CUBLAS_OP_N, CUBLAS_OP_N, m, n, k,
                             &one, A, lda, B, ldb, &zero, C, ldc));
  return GC_OK;
}

// FP32 eigensolve of M plus ctx->eig_refine refinement iterations. On success
// Xout (N x N) holds the eigenvectors, lam (N) the eigenvalues (the second-order
// Rayleigh quotients of the updated vectors), *fallback = false.
// *fallback = true when the FP32 solver failed or a cluster could not be handled.
int refine_from_fp32(gc_context *ctx, int N, int prec, const double *M, const float *m32,
                     double *Xout, double *lam, bool *fallback);

int refined_eig(gc_context *ctx, int N, int prec, const double *M, double *Xout, double *lam,
                bool *fallback) {
  *fallback = false;
  const size_t NN = (size_t)N * N;
  gc::DevBuf<float> m32, w32, work;
  GC_TRY(m32.alloc(ctx, NN));
  GC_TRY(w32.alloc(ctx, N));
  const unsigned ew = std::min<size_t>(gc::ceil_div(NN, 256), 152 * 16);
  k_d2f<<<ew, 256, 0, ctx->stream>>>(NN, M, m32.p);
  GC_LAUNCHED(ctx);
  {
    int lwork = 0;
    GC_CUSOLVER(ctx, cusolverDnSsyevd_bufferSize(ctx->cusolver, CUSOLVER_EIG_MODE_VECTOR,
                                                 CUBLAS_FILL_MODE_LOWER, N, m32.p, N, w32.p, &lwork));
    GC_TRY(work.alloc(ctx, std::max(lwork, 1)));
    if (ctx->eig_emulation)
      GC_CUSOLVER(ctx, cusolverDnSetMathMode(ctx->cusolver, CUSOLVER_FP32_EMULATED_BF16X9_MATH));
    GC_CUDA(ctx, cudaEventRecord(ctx->eig_ev[0], ctx->stream));
    cusolverStatus_t st = cusolverDnSsyevd(ctx->cusolver, CUSOLVER_EIG_MODE_VECTOR,
                                           CUBLAS_FILL_MODE_LOWER, N, m32.p, N, w32.p, work.p, lwork,
                                           ctx->dev_info);
    GC_CUDA(ctx, cudaEventRecord(ctx->eig_ev[1], ctx->stream));
    if (ctx->eig_emulation)
      GC_CUSOLVER(ctx, cusolverDnSetMathMode(ctx->cusolver, CUSOLVER_DEFAULT_MATH));
    GC_CUSOLVER(ctx, st);
    work.release();
    int info = 0;
    GC_CUDA(ctx, cudaMemcpyAsync(&info, ctx->dev_info, sizeof(int), cudaMemcpyDeviceToHost,
                                 ctx->stream));
    GC_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    GC_TRY(add_eig_time(ctx));
    if (info != 0) {
      *fallback = true;
      return GC_OK;
    }
  }
  w32.release();
  return refine_from_fp32(ctx, N, prec, M, m32.p, Xout, lam, fallback);
}

// The refinement of an FP32 start: m32 holds FP32 eigenvectors of M (column-major,
// eigenvalues ascending). Same outputs as refined_eig.
int refine_from_fp32(gc_context *ctx, int N, int prec, const double *M, const float *m32,
                     double *Xout, double *lam, bool *fallback) {
  *fallback = false;
  const size_t NN = (size_t)N * N;
  gc::DevBuf<double> U0, U1, vbuf, dS, dG;
  gc::DevBuf<int> cst, csz, flag;
  gc::DevBuf<double> colm;
  GC_TRY(U0.alloc(ctx, 2 * NN));
  GC_TRY(U1.alloc(ctx, 2 * NN));
  GC_TRY(vbuf.alloc(ctx, (size_t)N * kMaxCluster));
  GC_TRY(dS.alloc(ctx, N));
  GC_TRY(dG.alloc(ctx, N));
  GC_TRY(cst.alloc(ctx, N));
  GC_TRY(csz.alloc(ctx, N));
  GC_TRY(flag.alloc(ctx, 2));
  GC_TRY(colm.alloc(ctx, N));
  GC_CUDA(ctx, cudaFuncSetAttribute(k_cluster_eig, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                    (int)kClusterSmem));
  GC_CUDA(ctx, cudaFuncSetAttribute(k_blk_right, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                    (int)kBlkSmem));
  GC_CUDA(ctx, cudaFuncSetAttribute(k_blk_left, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                    (int)kBlkSmem));
  GC_CUDA(ctx, cudaMemsetAsync(flag.p, 0, 2 * sizeof(int), ctx->stream));
  const unsigned ew = std::min<size_t>(gc::ceil_div(NN, 256), 152 * 16);
  k_f2d<<<ew, 256, 0, ctx->stream>>>(NN, m32, U0.p);
  GC_LAUNCHED(ctx);
  double *cur = U0.p, *nxt = U1.p;
  const int iters = std::max(1, std::min(4, ctx->eig_refine));
  const unsigned gN = gc::ceil_div(N, 256);
  const dim3 b2(32, 8), g2(gc::ceil_div(N, 32), gc::ceil_div(N, 8));
  for (int it = 0; it < iters; ++it) {
    double *X = cur, *P = cur + NN, *G = nxt, *S = nxt + NN;
    GC_TRY(product(ctx, prec, false, N, N, N, M, N, X, N, P, N));        // P = M X
    // [G S] = X^T [X P]; both blocks are symmetric, so on the tensor-core path only
    // their lower triangles are computed and mirrored
    if (gc::is_sliced(prec)) {
      GC_TRY(gc::tc_gemm_strided_lower(ctx, prec, N, 2 * N, N, X, N, 1, X, N, 1, G, N, N));
      k_mirror_lower<<<g2, b2, 0, ctx->stream>>>(N, G);
      GC_LAUNCHED(ctx);
      k_mirror_lower<<<g2, b2, 0, ctx->stream>>>(N, S);
      GC_LAUNCHED(ctx);
    } else {
      GC_TRY(product(ctx, prec, true, N, 2 * N, N, X, N, X, N, G, N));
      k_symmetrize<<<g2, b2, 0, ctx->stream>>>(N, G);
      GC_LAUNCHED(ctx);
      k_symmetrize<<<g2, b2, 0, ctx->stream>>>(N, S);
      GC_LAUNCHED(ctx);
    }
    k_rayleigh<<<gN, 256, 0, ctx->stream>>>(N, G, S, lam, nullptr, nullptr);
    GC_LAUNCHED(ctx);
    k_col_coupling<<<N, 256, 0, ctx->stream>>>(N, G, S, lam, colm.p);
    GC_LAUNCHED(ctx);
    k_clusters<<<gN, 256, 0, ctx->stream>>>(N, lam, colm.p, cst.p, csz.p, flag.p);
    GC_LAUNCHED(ctx);
    k_cluster_eig<<<N, kMaxCluster, kClusterSmem, ctx->stream>>>(N, G, S, cst.p, csz.p, vbuf.p,
                                                                 flag.p, flag.p + 1);
    GC_LAUNCHED(ctx);
    const dim3 gr(gc::ceil_div(N, kMaxCluster), N), gl2(gc::ceil_div(2 * (size_t)N, kMaxCluster), N);
    k_blk_right<<<gr, kMaxCluster, kBlkSmem, ctx->stream>>>(N, G, N, cst.p, csz.p, vbuf.p);
    GC_LAUNCHED(ctx);
    k_blk_right<<<gr, kMaxCluster, kBlkSmem, ctx->stream>>>(N, S, N, cst.p, csz.p, vbuf.p);
    GC_LAUNCHED(ctx);
    k_blk_left<<<gl2, kMaxCluster, kBlkSmem, ctx->stream>>>(2 * N, G, N, 1, cst.p, csz.p, vbuf.p);
    GC_LAUNCHED(ctx);
    k_rayleigh<<<gN, 256, 0, ctx->stream>>>(N, G, S, lam, dS.p, dG.p);
    GC_LAUNCHED(ctx);
    k_form_update<<<dim3(gN, N), 256, 0, ctx->stream>>>(N, G, S, lam, cst.p, P, flag.p);
    GC_LAUNCHED(ctx);
    k_eig_update<<<N, 256, 0, ctx->stream>>>(N, G, S, P, dS.p, dG.p, lam);
    GC_LAUNCHED(ctx);
    // D = E E^T into the S slot (S is no longer needed); low relative accuracy suffices
    if (gc::is_sliced(prec)) {
      GC_TRY(gc::tc_gemm_nt(ctx, GC_PREC_BF16X6, N, N, N, P, N, P, N, S, N));
    } else {
      const double one = 1.0, zero = 0.0;
      GC_CUBLAS(ctx, cublasDgemm(ctx->cublas, CUBLAS_OP_N, CUBLAS_OP_T, N, N, N, &one, P, N, P, N,
                                 &zero, S, N));
    }
    k_second_order<<<ew, 256, 0, ctx->stream>>>(NN, N, P, S);
    GC_LAUNCHED(ctx);
    k_blk_left<<<gr, kMaxCluster, kBlkSmem, ctx->stream>>>(N, P, N, 0, cst.p, csz.p, vbuf.p);
    GC_LAUNCHED(ctx);
    GC_TRY(product(ctx, prec, false, N, N, N, X, N, P, N, G, N));        // X' = X (V (I + E))
    std::swap(cur, nxt);
  }
  int hflag[2] = {0, 0};
  GC_CUDA(ctx, cudaMemcpyAsync(hflag, flag.p, 2 * sizeof(int), cudaMemcpyDeviceToHost, ctx->stream));
  GC_TRY(gc::check_flag(ctx));  // synchronises; a refinement GEMM whose wait expired fails here
  ctx->refine_max_cluster = std::max(ctx->refine_max_cluster, hflag[1]);
  if (hflag[0] != 0) {
    *fallback = true;
    return GC_OK;
  }
  k_colnorm<<<N, 256, 0, ctx->stream>>>(N, cur);
  GC_LAUNCHED(ctx);
  GC_CUDA(ctx, cudaMemcpyAsync(Xout, cur, NN * sizeof(double), cudaMemcpyDeviceToDevice,
                               ctx->stream));
  return GC_OK;
}

// One dpotrf over the lower triangle of A; *minor as in chol_blocked.
int chol_plain(gc_context *ctx, int N, double *A, int *minor) {
  *minor = 0;
  int lwork = 0;
  GC_CUSOLVER(ctx, cusolverDnDpotrf_bufferSize(ctx->cusolver, CUBLAS_FILL_MODE_LOWER, N, A, N,
                                               &lwork));
  gc::DevBuf<double> work;
  GC_TRY(work.alloc(ctx, std::max(lwork, 1)));
  GC_CUSOLVER(ctx, cusolverDnDpotrf(ctx->cusolver, CUBLAS_FILL_MODE_LOWER, N, A, N, work.p, lwork,
                                    ctx->dev_info));
  int info = 0;
  GC_CUDA(ctx, cudaMemcpyAsync(&info, ctx->dev_info, sizeof(int), cudaMemcpyDeviceToHost,
                               ctx->stream));
  GC_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
  if (info < 0) return gc::set_error(ctx, GC_ECUSOLVER, "potrf info=%d", info);
  *minor = info;
  return GC_OK;
}

// Blocked Cholesky of the tensor-core path. GB300's FP64 pipe is narrow (about two
// FP64 FMAs per cycle per SM), so the FP64 CUDA-core work is kept to what every SM
// can share: 64-wide diagonal blocks are factored in shared memory by one CTA
// (64^3/6 FMAs), the panel below is solved one row per thread on all SMs, and the
// trailing update A22 -= P P^T (all but N^2 * 64 / 2 of the N^3/3 FMAs) runs on the
// sliced FP64-accurate tensor-core GEMM, which subtracts into A22's lower triangle
// in its epilogue.
constexpr int kCholNb = 64;
constexpr int kCholLd = kCholNb + 1;  // padded column stride of the shared block

// Right-looking Cholesky of the kb x kb (kb <= 64) diagonal block A (leading
// dimension lda) in shared memory; L's lower triangle is written back. The update of
// step k uses the unscaled column k and the pivot's reciprocal, a_ij -= a_ik a_jk / d_k,
// and the columns are scaled by 1/sqrt(d_k) at the end, so a step needs one barrier.
// Thread 0 updates the next diagonal element and forms that pivot's factors (one FP64
// square root and one division) while warps 1-7 update the rest of the trailing
// triangle: the pivot's latency, not the FP64 work of one SM, set the time of a step.
// A pivot that is not positive (or not finite) records its global order k0 + k + 1 in
// *info, unless an earlier block already did, and is replaced by 1 so that the rest
// stays finite.
__global__ void __launch_bounds__(256) k_potrf_block(int kb, double *__restrict__ A, long long lda,
                                                     int k0, int *__restrict__ info,
                                                     long long sb) {
  // one CTA per matrix of a batch (A and info of matrix b at b * sb and b)
  A += blockIdx.x * sb;
  info += blockIdx.x;
  __shared__ double s[kCholNb * kCholLd];
  __shared__ double rk[kCholNb], sq[kCholNb], isq[kCholNb];  // 1/d, sqrt(d), 1/sqrt(d)
  __shared__ int bad;
  const int t = threadIdx.x, lane = t & 31, warp = t >> 5;
  for (int e = t; e < kb * kb; e += blockDim.x) {
    const int i = e % kb, j = e / kb;
    s[i + j * kCholLd] = i >= j ? A[i + j * lda] : 0.0;
  }
  auto pivot = [&](int k) {
    double d = s[k + k * kCholLd];
    if (!(d > 0.0)) {
      if (!bad) bad = k + 1;
      d = 1.0;
    }
    const double is = 1.0 / sqrt(d);
    isq[k] = is;
    sq[k] = d * is;
    rk[k] = is * is;
  };
  __syncthreads();
  if (t == 0) {
    bad = 0;
    pivot(0);
  }
  __syncthreads();
  for (int k = 0; k + 1 < kb; ++k) {
    const double r = rk[k];
    if (t == 0) {  // the next diagonal element, then its pivot
      const double akk = s[(k + 1) + k * kCholLd];
      s[(k + 1) + (k + 1) * kCholLd] -= akk * (akk * r);
      pivot(k + 1);
    } else if (warp > 0) {
      // the rest of the trailing lower triangle: warps 1-7 over columns j, lanes along them
      for (int j = k + warp; j < kb; j += 7) {
        const double tj = s[j + k * kCholLd] * r;
        for (int i = j + lane; i < kb; i += 32)
          if (i != k + 1) s[i + j * kCholLd] -= s[i + k * kCholLd] * tj;
      }
    }
    __syncthreads();
  }
  for (int e = t; e < kb * kb; e += blockDim.x) {
    const int i = e % kb, j = e / kb;
    if (i > j)
      A[i + j * lda] = s[i + j * kCholLd] * isq[j];
    else if (i == j)
      A[i + j * lda] = sq[j];
  }
  if (t == 0 && bad && *info == 0) *info = k0 + bad;
}

// Panel solve X L11^T = P for the m x 64 panel P below a factored 64-wide diagonal
// block L11 (both in the matrix, leading dimension lda), X overwriting P. Four lanes
// share a row, each holding the columns j = q (mod 4) of it in registers; column j is
// finished by its owner lane, broadcast to the other three by a shuffle and eliminated
// from their later columns (right-looking). A warp then holds 8 rows, so the FP64 work
// of a panel is spread over four times as many warps as with one row per thread (GB300's
// FP64 pipe is narrow and shared by the warps of an SM). L11 sits in shared memory with
// a padded row stride, read by the four lanes of a row from four banks.
constexpr int kTrsmRowsPerWarp = 8;
constexpr int kTrsmWarps = 4;
__global__ void __launch_bounds__(32 * kTrsmWarps) k_trsm_rows(int m, const double *__restrict__ L11,
                                                              long long lda,
                                                              double *__restrict__ P,
                                                              long long sb) {
  L11 += blockIdx.y * sb;  // matrix blockIdx.y of a batch
  P += blockIdx.y * sb;
  __shared__ double Ls[kCholNb * kCholLd];  // Ls[i * kCholLd + j] = L(i, j), j <= i
  __shared__ double rd[kCholNb];
  for (int e = threadIdx.x; e < kCholNb * kCholNb; e += blockDim.x) {
    const int j = e / kCholNb, i = e % kCholNb;  // coalesced along the column of L11
    Ls[i * kCholLd + j] = j <= i ? L11[i + j * lda] : 0.0;
  }
  for (int j = threadIdx.x; j < kCholNb; j += blockDim.x) rd[j] = 1.0 / L11[j + j * lda];
  __syncthreads();
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, q = lane & 3;
  const long long r = ((long long)blockIdx.x * kTrsmWarps + warp) * kTrsmRowsPerWarp + (lane >> 2);
  const bool live = r < m;
  double acc[kCholNb / 4];
#pragma unroll
  for (int t = 0; t < kCholNb / 4; ++t) acc[t] = live ? P[r + (4 * t + q) * lda] : 0.0;
#pragma unroll
  for (int j = 0; j < kCholNb; ++j) {
    const int t0 = j >> 2, q0 = j & 3;
    double xj = acc[t0] * rd[j];  // the owner lane's value is the one broadcast
    xj = __shfl_sync(0xffffffffu, xj, (lane & ~3) | q0);
    if (q == q0) acc[t0] = xj;
#pragma unroll
    for (int t = t0; t < kCholNb / 4; ++t) {
      const int i = 4 * t + q;
      if (i > j) acc[t] = fma(-xj, Ls[i * kCholLd + j], acc[t]);
    }
  }
  if (live)
#pragma unroll
    for (int t = 0; t < kCholNb / 4; ++t) P[r + (4 * t + q) * lda] = acc[t];
}

// Cholesky A = L L^T of the lower triangles of nmat N x N matrices (column-major, matrix
// b at A + b*sb) in place, by the kernels above and FP64-accurate products of precision
// prec (L L^T equals A to that product's ~2^-35 relative error; the diagonal blocks and
// panels are FP64). The matrices of a batch go through the 64-wide steps together: one
// launch per kernel and step for all of them. The strict upper triangles are left as they
// were. minor[b] = 0 on success, else the order of the first leading minor of matrix b
// that is not positive definite.
int chol_blocked_batch(gc_context *ctx, int N, int nmat, double *A, long long sb, int prec,
                       int *minor) {
  const long long lda = N;
  gc::DevBuf<int> info;
  GC_TRY(info.alloc(ctx, nmat));
  GC_CUDA(ctx, cudaMemsetAsync(info.p, 0, nmat * sizeof(int), ctx->stream));
  for (int k0 = 0; k0 < N; k0 += kCholNb) {
    const int kb = std::min(kCholNb, N - k0), m = N - k0 - kb;
    double *A11 = A + k0 + (size_t)k0 * lda;
    k_potrf_block<<<nmat, 256, 0, ctx->stream>>>(kb, A11, lda, k0, info.p, sb);
    GC_LAUNCHED(ctx);
    if (m == 0) break;
    double *P = A11 + kb;  // rows k0+kb.., columns k0..k0+kb
    k_trsm_rows<<<dim3(gc::ceil_div(m, kTrsmWarps * kTrsmRowsPerWarp), nmat), 32 * kTrsmWarps, 0,
                  ctx->stream>>>(m, A11, lda, P, sb);
    GC_LAUNCHED(ctx);
    GC_TRY(gc::tc_syrk_sub_lower(ctx, prec, m, kb, P, 1, lda, P + (size_t)kb * lda, lda, nmat, sb));
  }
  GC_CUDA(ctx, cudaMemcpyAsync(minor, info.p, nmat * sizeof(int), cudaMemcpyDeviceToHost,
                               ctx->stream));
  GC_TRY(gc::check_flag(ctx));  // synchronises; covers the trailing-update GEMMs
  return GC_OK;
}

// One matrix: *minor as minor[0] above.
int chol_blocked(gc_context *ctx, int N, double *A, int prec, int *minor) {
  return chol_blocked_batch(ctx, N, 1, A, 0, prec, minor);
}

// Eigenpairs of the symmetric M in place (vectors overwrite M, values in w):
// dsyevd, or the refined FP32 solve with dsyevd as its fallback.
int eigen(gc_context *ctx, int N, double *M, double *w, int mode, int prec) {
  if (mode != GC_ERPA_CHOLESKY_REFINED) return syevd(ctx, N, M, w);
  ctx->refine_solves++;
  bool fallback = N > 65535;
  if (!fallback) GC_TRY(refined_eig(ctx, N, prec, M, M, w, &fallback));
  if (fallback) {
    ctx->refine_fallbacks++;
    return syevd(ctx, N, M, w);
  }
  return GC_OK;
}

// bad[k] = 1 when the FP32 eigenvalues of matrix k are not finite and ascending (the
// refinement's cluster rule pairs neighbouring columns).
__global__ void k_ascending(int N, int np, const float *__restrict__ w, int *__restrict__ bad) {
  const int k = blockIdx.y;
  const float *wk = w + (size_t)k * N;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < N; i += gridDim.x * blockDim.x)
    if (!isfinite(wk[i]) || (i + 1 < N && !(wk[i] <= wk[i + 1]))) bad[k] = 1;
}

// The batched FP32 start of eigen_refined_batch: m32 (np x N x N) receives the FP32
// eigenvectors of the M[k], h (2 np) the solver status of each matrix and then whether its
// eigenvalues are not finite and ascending.
int fp32_batch_start(gc_context *ctx, int N, int np, double *const *M, gc::DevBuf<float> &m32,
                     std::vector<int> &h) {
  const size_t NN = (size_t)N * N;
  gc::DevBuf<float> w32;
  gc::DevBuf<int> info;
  GC_TRY(m32.alloc(ctx, NN * np));
  GC_TRY(w32.alloc(ctx, (size_t)N * np));
  GC_TRY(info.alloc(ctx, 2 * (size_t)np));
  const unsigned ew = std::min<size_t>(gc::ceil_div(NN, 256), 152 * 16);
  for (int k = 0; k < np; ++k) {
    k_d2f<<<ew, 256, 0, ctx->stream>>>(NN, M[k], m32.p + k * NN);
    GC_LAUNCHED(ctx);
  }
  GC_CUDA(ctx, cudaMemsetAsync(info.p, 0, 2 * (size_t)np * sizeof(int), ctx->stream));
  cusolverDnParams_t params = nullptr;
  GC_CUSOLVER(ctx, cusolverDnCreateParams(&params));
  struct ParamsGuard {
    cusolverDnParams_t p;
    ~ParamsGuard() { cusolverDnDestroyParams(p); }
  } guard{params};
  size_t wd = 0, wh = 0;
  GC_CUSOLVER(ctx, cusolverDnXsyevBatched_bufferSize(
                       ctx->cusolver, params, CUSOLVER_EIG_MODE_VECTOR, CUBLAS_FILL_MODE_LOWER, N,
                       CUDA_R_32F, m32.p, N, CUDA_R_32F, w32.p, CUDA_R_32F, &wd, &wh, np));
  gc::DevBuf<char> work;
  GC_TRY(work.alloc(ctx, std::max<size_t>(wd, 1)));
  std::vector<char> hwork(std::max<size_t>(wh, 1));
  GC_CUDA(ctx, cudaEventRecord(ctx->eig_ev[0], ctx->stream));
  GC_CUSOLVER(ctx, cusolverDnXsyevBatched(ctx->cusolver, params, CUSOLVER_EIG_MODE_VECTOR,
                                          CUBLAS_FILL_MODE_LOWER, N, CUDA_R_32F, m32.p, N,
                                          CUDA_R_32F, w32.p, CUDA_R_32F, work.p, wd, hwork.data(),
                                          wh, info.p, np));
  GC_CUDA(ctx, cudaEventRecord(ctx->eig_ev[1], ctx->stream));
  k_ascending<<<dim3(gc::ceil_div(N, 256), np), 256, 0, ctx->stream>>>(N, np, w32.p, info.p + np);
  GC_LAUNCHED(ctx);
  h.assign(2 * (size_t)np, 0);
  GC_CUDA(ctx, cudaMemcpyAsync(h.data(), info.p, 2 * (size_t)np * sizeof(int),
                               cudaMemcpyDeviceToHost, ctx->stream));
  GC_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
  float ms = 0.f;
  GC_CUDA(ctx, cudaEventElapsedTime(&ms, ctx->eig_ev[0], ctx->eig_ev[1]));
  ctx->eig_ms += ms;
  ctx->eig_calls += np;
  return GC_OK;
}

// Eigenpairs of np symmetric N x N matrices M[k] in place (vectors overwrite M[k], values
// in w[k]) in the refined form: one batched FP32 eigensolve (cusolverDnXsyevBatched) for
// all of them, then the refinement of each. Concurrent FP32 eigensolves of one order
// overlap poorly on separate streams; the batched solver runs them 2-4x faster. A
// matrix whose FP32 solve failed, or whose refinement cannot proceed, is solved alone
// (ssyevd start, then dsyevd), as eigen() does; so are all of them when the batched
// solver refuses the order or its workspace does not fit.
int eigen_refined_batch(gc_context *ctx, int N, int np, double *const *M, double *const *w,
                        int prec) {
  auto one_by_one = [&]() -> int {
    for (int k = 0; k < np; ++k) GC_TRY(eigen(ctx, N, M[k], w[k], GC_ERPA_CHOLESKY_REFINED, prec));
    return GC_OK;
  };
  if (np == 1 || N > 65535) return one_by_one();
  const size_t NN = (size_t)N * N;
  gc::DevBuf<float> m32;
  std::vector<int> h;
  const int r = fp32_batch_start(ctx, N, np, M, m32, h);
  if (r == GC_ECUSOLVER || r == GC_ENOMEM) {
    // the batched solver refused this order or batch, or its workspace does not fit:
    // the points are solved one at a time
    m32.release();
    return one_by_one();
  }
  GC_TRY(r);
  for (int k = 0; k < np; ++k) {
    if (h[k] != 0 || h[np + k] != 0) {  // solved alone: the ssyevd start, then dsyevd
      GC_TRY(eigen(ctx, N, M[k], w[k], GC_ERPA_CHOLESKY_REFINED, prec));
      continue;
    }
    ctx->refine_solves++;
    bool fallback = false;
    GC_TRY(refine_from_fp32(ctx, N, prec, M[k], m32.p + k * NN, M[k], w[k], &fallback));
    if (fallback) {
      ctx->refine_fallbacks++;
      GC_TRY(syevd(ctx, N, M[k], w[k]));
    }
  }
  return GC_OK;
}

}  // namespace

namespace gc {

// Checks A+-B for non-finite elements and symmetrises both in place.
int erpa_prepare(gc_context *ctx, int N, double *abplus, double *abmin) {
  const size_t NN = (size_t)N * N;
  // No eigensolver is handed a matrix with a NaN or an infinity.
  GC_CUDA(ctx, cudaMemsetAsync(ctx->dev_nonfinite, 0, sizeof(int), ctx->stream));
  const unsigned grid = std::min<size_t>(ceil_div(NN, 256), 152 * 8);
  k_count_nonfinite<<<grid, 256, 0, ctx->stream>>>(NN, abplus, abmin, ctx->dev_nonfinite);
  GC_LAUNCHED(ctx);
  int bad = 0;
  GC_CUDA(ctx, cudaMemcpyAsync(&bad, ctx->dev_nonfinite, sizeof(int), cudaMemcpyDeviceToHost,
                               ctx->stream));
  GC_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
  if (bad) return set_error(ctx, GC_ENONFINITE, "erpa: %d non-finite elements in A+B / A-B", bad);
  dim3 b2(32, 8), g2(ceil_div(N, 32), ceil_div(N, 8));
  k_symmetrize<<<g2, b2, 0, ctx->stream>>>(N, abplus);
  GC_LAUNCHED(ctx);
  k_symmetrize<<<g2, b2, 0, ctx->stream>>>(N, abmin);
  GC_LAUNCHED(ctx);
  return GC_OK;
}

// Cholesky form, first half: A+B = L L^T (L lower, zero upper triangle) and the
// symmetric M = L^T (A-B) L, from the symmetrised A+-B. T (N x N) is scratch.
int chol_form(gc_context *ctx, int N, const double *abplus, const double *abmin, double *L,
              double *M, double *T, int mode, int prec) {
  const size_t NN = (size_t)N * N;
  const dim3 b2(32, 8), g2(ceil_div(N, 32), ceil_div(N, 8));
  const double one = 1.0;
  GC_CUDA(ctx, cudaMemcpyAsync(L, abplus, NN * sizeof(double), cudaMemcpyDeviceToDevice,
                               ctx->stream));
  const bool tc = gc::is_sliced(prec);
  {
    PhaseScope ph(ctx, GC_PHASE_CHOLESKY);
    int minor = 0;
    if (tc && ctx->chol_blocked)
      GC_TRY(chol_blocked(ctx, N, L, prec, &minor));
    else
      GC_TRY(chol_plain(ctx, N, L, &minor));
    if (minor > 0)
      return set_error(ctx, GC_ENOTPD, "A+B is not positive definite (potrf minor %d)", minor);
    k_zero_upper<<<g2, b2, 0, ctx->stream>>>(N, L);
    GC_LAUNCHED(ctx);
  }
  PhaseScope ph(ctx, GC_PHASE_PRODUCTS);
  if (tc) {
    // T = A- L; M = L^T T: products of the FP64-accurate sliced tensor-core GEMM (L has a
    // zero upper triangle)
    GC_TRY(tc_gemm_strided(ctx, prec, N, N, N, abmin, 1, N, L, N, 1, T, N));
    GC_TRY(tc_gemm_strided(ctx, prec, N, N, N, L, N, 1, T, N, 1, M, N));
    k_symmetrize<<<g2, b2, 0, ctx->stream>>>(N, M);
    GC_LAUNCHED(ctx);
  } else {
    // T = A- L, then M = L^T T
    GC_CUBLAS(ctx, cublasDtrmm(ctx->cublas, CUBLAS_SIDE_RIGHT, CUBLAS_FILL_MODE_LOWER, CUBLAS_OP_N,
                               CUBLAS_DIAG_NON_UNIT, N, N, &one, L, N, abmin, N, T, N));
    GC_CUBLAS(ctx, cublasDtrmm(ctx->cublas, CUBLAS_SIDE_LEFT, CUBLAS_FILL_MODE_LOWER, CUBLAS_OP_T,
                               CUBLAS_DIAG_NON_UNIT, N, N, &one, L, N, T, N, M, N));
    if (mode == GC_ERPA_CHOLESKY_REFINED) {
      k_symmetrize<<<g2, b2, 0, ctx->stream>>>(N, M);
      GC_LAUNCHED(ctx);
    }
  }
  return GC_OK;
}

// Cholesky form, second half: Y = L U for the eigenvectors U of M (eigenvalues omega^2
// in eig), normalised as ERPASYMM1 normalises, and eig <- omega.
int chol_finish(gc_context *ctx, int N, const double *L, const double *U, double *Y, double *eig,
                int prec) {
  PhaseScope ph(ctx, GC_PHASE_PRODUCTS);
  if (gc::is_sliced(prec)) {
    GC_TRY(tc_gemm_strided(ctx, prec, N, N, N, L, 1, N, U, N, 1, Y, N));
  } else {
    const double one = 1.0;
    GC_CUBLAS(ctx, cublasDtrmm(ctx->cublas, CUBLAS_SIDE_LEFT, CUBLAS_FILL_MODE_LOWER, CUBLAS_OP_N,
                               CUBLAS_DIAG_NON_UNIT, N, N, &one, L, N, U, N, Y, N));
  }
  k_norm_chol<<<dim3(ceil_div(N, 256), N), 256, 0, ctx->stream>>>(N, Y, eig);
  GC_LAUNCHED(ctx);
  k_sqrt_eig<<<ceil_div(N, 256), 256, 0, ctx->stream>>>(N, eig);
  GC_LAUNCHED(ctx);
  return GC_OK;
}

int erpa_solve(gc_context *ctx, int N, double *abplus, double *abmin, double *Y, double *eig,
               int mode, int gemm_precision, bool aplsqrt_out) {
  if (N <= 0 || !abplus || !abmin || !Y || !eig)
    return set_error(ctx, GC_EINVAL, "erpa: bad arguments N=%d", N);
  const size_t NN = (size_t)N * N;
  if (mode == GC_ERPA_VEC) {
    // ERPAVEC reads A+-B as given (the non-finite check still applies)
    GC_CUDA(ctx, cudaMemsetAsync(ctx->dev_nonfinite, 0, sizeof(int), ctx->stream));
    const unsigned grid = std::min<size_t>(ceil_div(NN, 256), 152 * 8);
    k_count_nonfinite<<<grid, 256, 0, ctx->stream>>>(NN, abplus, abmin, ctx->dev_nonfinite);
    GC_LAUNCHED(ctx);
    int bad = 0;
    GC_CUDA(ctx, cudaMemcpyAsync(&bad, ctx->dev_nonfinite, sizeof(int), cudaMemcpyDeviceToHost,
                                 ctx->stream));
    GC_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    if (bad)
      return set_error(ctx, GC_ENONFINITE, "erpa: %d non-finite elements in A+B / A-B", bad);
    PhaseScope ph(ctx, GC_PHASE_EIGEN);
    return erpavec(ctx, N, abplus, abmin, Y, eig);
  }
  GC_TRY(erpa_prepare(ctx, N, abplus, abmin));
  const dim3 b2(32, 8), g2(ceil_div(N, 32), ceil_div(N, 8));
  const double one = 1.0, zero = 0.0;
  if (mode == GC_ERPA_SYMM1) {
    DevBuf<double> V, P, H;
    GC_TRY(V.alloc(ctx, NN));
    GC_TRY(P.alloc(ctx, NN));
    GC_TRY(H.alloc(ctx, NN));
    GC_CUDA(ctx, cudaMemcpyAsync(V.p, abplus, NN * sizeof(double), cudaMemcpyDeviceToDevice,
                                 ctx->stream));
    {
      PhaseScope ph(ctx, GC_PHASE_EIGEN);
      GC_TRY(syevd(ctx, N, V.p, eig));
    }
    PhaseScope ph(ctx, GC_PHASE_PRODUCTS);
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
    {
      PhaseScope phe(ctx, GC_PHASE_EIGEN);
      GC_TRY(syevd(ctx, N, V.p, eig));
    }
    // Y = P Z ; T = A- Y
    GC_CUBLAS(ctx, cublasDgemm(ctx->cublas, CUBLAS_OP_N, CUBLAS_OP_N, N, N, N, &one, P.p, N, V.p, N,
                               &zero, Y, N));
    GC_CUBLAS(ctx, cublasDgemm(ctx->cublas, CUBLAS_OP_N, CUBLAS_OP_N, N, N, N, &one, abmin, N, Y, N,
                               &zero, H.p, N));
    k_norm_symm1<<<N, 256, 0, ctx->stream>>>(N, Y, H.p, eig);
    GC_LAUNCHED(ctx);
    if (aplsqrt_out)  // ERPASYMM1 leaves A+^1/2 in its A+ argument (interpa.f:1652-1716)
      GC_CUDA(ctx, cudaMemcpyAsync(abplus, P.p, NN * sizeof(double), cudaMemcpyDeviceToDevice,
                                   ctx->stream));
    return GC_OK;
  }
  if (mode == GC_ERPA_CHOLESKY || mode == GC_ERPA_CHOLESKY_REFINED) {
    DevBuf<double> L, M;
    GC_TRY(L.alloc(ctx, NN));
    GC_TRY(M.alloc(ctx, NN));
    GC_TRY(chol_form(ctx, N, abplus, abmin, L.p, M.p, Y, mode, gemm_precision));
    {
      PhaseScope ph(ctx, GC_PHASE_EIGEN);
      GC_TRY(eigen(ctx, N, M.p, eig, mode, gemm_precision));
    }
    return chol_finish(ctx, N, L.p, M.p, Y, eig, gemm_precision);
  }
  return set_error(ctx, GC_EINVAL, "erpa: unknown mode %d", mode);
}

int erpa_solve_points(gc_context *ctx, int N, int np, int prec,
                      const std::function<int(int, double *, double *)> &fill,
                      const std::function<int(int, const double *, double *)> &use) {
  if (N <= 0 || np <= 0) return set_error(ctx, GC_EINVAL, "erpa points: N=%d np=%d", N, np);
  const size_t NN = (size_t)N * N;
  DevBuf<double> ap, am, T, LM, ev;
  GC_TRY(ap.alloc(ctx, NN));
  GC_TRY(am.alloc(ctx, NN));
  GC_TRY(T.alloc(ctx, NN));
  GC_TRY(LM.alloc(ctx, 2 * (size_t)np * NN));
  GC_TRY(ev.alloc(ctx, (size_t)np * N));
  std::vector<double *> Ls(np), Ms(np), ws(np);
  // A+-B of every point: A+B into the L slot, A-B into the M slot
  for (int k = 0; k < np; ++k) {
    Ls[k] = LM.p + 2 * (size_t)k * NN;
    Ms[k] = Ls[k] + NN;
    ws[k] = ev.p + (size_t)k * N;
    GC_TRY(fill(k, ap.p, am.p));
    GC_TRY(erpa_prepare(ctx, N, ap.p, am.p));
    GC_CUDA(ctx, cudaMemcpyAsync(Ls[k], ap.p, NN * sizeof(double), cudaMemcpyDeviceToDevice,
                                 ctx->stream));
    GC_CUDA(ctx, cudaMemcpyAsync(Ms[k], am.p, NN * sizeof(double), cudaMemcpyDeviceToDevice,
                                 ctx->stream));
  }
  ap.release();
  am.release();
  const dim3 b2(32, 8), g2(ceil_div(N, 32), ceil_div(N, 8));
  {
    // the Cholesky factors of all points, the 64-wide steps batched over the points
    PhaseScope ph(ctx, GC_PHASE_CHOLESKY);
    std::vector<int> minor(np, 0);
    if (gc::is_sliced(prec) && ctx->chol_blocked)
      GC_TRY(chol_blocked_batch(ctx, N, np, LM.p, 2 * (long long)NN, prec, minor.data()));
    else
      for (int k = 0; k < np; ++k) GC_TRY(chol_plain(ctx, N, Ls[k], &minor[k]));
    for (int k = 0; k < np; ++k)
      if (minor[k] > 0)
        return set_error(ctx, GC_ENOTPD, "A+B is not positive definite (potrf minor %d)",
                         minor[k]);
    for (int k = 0; k < np; ++k) {
      k_zero_upper<<<g2, b2, 0, ctx->stream>>>(N, Ls[k]);
      GC_LAUNCHED(ctx);
    }
  }
  for (int k = 0; k < np; ++k) {
    // M = L^T (A- L): T = A- L, then M (which held A-) = L^T T
    PhaseScope ph(ctx, GC_PHASE_PRODUCTS);
    GC_TRY(product(ctx, prec, false, N, N, N, Ms[k], N, Ls[k], N, T.p, N));
    GC_TRY(product(ctx, prec, true, N, N, N, Ls[k], N, T.p, N, Ms[k], N));
    k_symmetrize<<<g2, b2, 0, ctx->stream>>>(N, Ms[k]);
    GC_LAUNCHED(ctx);
  }
  {
    PhaseScope ph(ctx, GC_PHASE_EIGEN);
    GC_TRY(eigen_refined_batch(ctx, N, np, Ms.data(), ws.data(), prec));
  }
  for (int k = 0; k < np; ++k) {
    GC_TRY(chol_finish(ctx, N, Ls[k], Ms[k], T.p, ws[k], prec));
    GC_TRY(use(k, T.p, ws[k]));
  }
  return GC_OK;
}

}  // namespace gc

namespace gc {

int chol_eig(gc_context *ctx, int N, const double *abplus, const double *abmin, double *L,
             double *U, double *w, int mode, int prec) {
  if (N <= 0) return set_error(ctx, GC_EINVAL, "chol_eig: N=%d", N);
  const size_t NN = (size_t)N * N;
  const dim3 b2(32, 8), g2(ceil_div(N, 32), ceil_div(N, 8));
  DevBuf<double> am;
  GC_TRY(am.alloc(ctx, NN));
  GC_CUDA(ctx, cudaMemcpyAsync(L, abplus, NN * sizeof(double), cudaMemcpyDeviceToDevice, ctx->stream));
  GC_CUDA(ctx, cudaMemcpyAsync(am.p, abmin, NN * sizeof(double), cudaMemcpyDeviceToDevice,
                               ctx->stream));
  k_symmetrize<<<g2, b2, 0, ctx->stream>>>(N, L);
  GC_LAUNCHED(ctx);
  k_symmetrize<<<g2, b2, 0, ctx->stream>>>(N, am.p);
  GC_LAUNCHED(ctx);
  const bool tc = gc::is_sliced(prec);
  int minor = 0;
  if (tc && ctx->chol_blocked)
    GC_TRY(chol_blocked(ctx, N, L, prec, &minor));
  else
    GC_TRY(chol_plain(ctx, N, L, &minor));
  if (minor > 0)
    return set_error(ctx, GC_ENOTPD, "A+B is not positive definite (potrf minor %d)", minor);
  k_zero_upper<<<g2, b2, 0, ctx->stream>>>(N, L);
  GC_LAUNCHED(ctx);
  // U <- L^T A- L (the eigenvectors overwrite it)
  DevBuf<double> T;
  GC_TRY(T.alloc(ctx, NN));
  GC_TRY(product(ctx, prec, false, N, N, N, am.p, N, L, N, T.p, N));
  GC_TRY(product(ctx, prec, true, N, N, N, L, N, T.p, N, U, N));
  k_symmetrize<<<g2, b2, 0, ctx->stream>>>(N, U);
  GC_LAUNCHED(ctx);
  return eigen(ctx, N, U, w, mode == GC_ERPA_CHOLESKY_REFINED ? mode : GC_ERPA_CHOLESKY, prec);
}

}  // namespace gc

extern "C" int gc_erpa(gc_context *ctx, int ndimx, double *abplus, double *abmin, double *eigvec,
                       double *eig, int mode) {
  if (!ctx) return GC_EINVAL;
  GC_TRY(gc::erpa_solve(ctx, ndimx, abplus, abmin, eigvec, eig, mode, GC_PREC_FP64));
  return gc::check_flag(ctx);  // the refined form's BF16 product of E E^T runs on tensor cores
}

extern "C" int gc_erpa_ex(gc_context *ctx, int ndimx, double *abplus, double *abmin,
                          double *eigvec, double *eig, int mode, int precision) {
  if (!ctx) return GC_EINVAL;
  if (precision != GC_PREC_FP64 && !gc::is_sliced(precision))
    return gc::set_error(ctx, GC_EINVAL, "gc_erpa_ex: precision %d is not FP64-accurate", precision);
  GC_TRY(gc::erpa_solve(ctx, ndimx, abplus, abmin, eigvec, eig, mode, precision));
  return gc::check_flag(ctx);
}

extern "C" int gc_erpasymm1(gc_context *ctx, int ndimx, double *abplus, double *abmin,
                            double *eigvec, double *eig) {
  if (!ctx) return GC_EINVAL;
  GC_TRY(gc::erpa_solve(ctx, ndimx, abplus, abmin, eigvec, eig, GC_ERPA_SYMM1, GC_PREC_FP64, true));
  return gc::check_flag(ctx);
}

extern "C" int gc_set_pipeline_wait(gc_context *ctx, unsigned long long ns) {
  if (!ctx) return GC_EINVAL;
  if (ns > 1000000000ull)
    return gc::set_error(ctx, GC_EINVAL, "pipeline wait limit %llu ns above 1 s", ns);
  ctx->wait_ns = ns ? ns : 1000000000ull;
  return GC_OK;
}

extern "C" int gc_set_eig_batch(gc_context *ctx, int on) {
  if (!ctx) return GC_EINVAL;
  ctx->eig_batch = on ? 1 : 0;
  return GC_OK;
}

extern "C" int gc_set_gemm_tile(gc_context *ctx, int width) {
  if (!ctx) return GC_EINVAL;
  if (width != 0 && width != 64 && width != 96 && width != 128)
    return gc::set_error(ctx, GC_EINVAL, "GEMM tile width %d not one of 0, 64, 96, 128", width);
  ctx->oz_tile = width;
  return GC_OK;
}

extern "C" int gc_set_eig_refinement(gc_context *ctx, int iterations) {
  if (!ctx) return GC_EINVAL;
  if (iterations < 1 || iterations > 4)
    return gc::set_error(ctx, GC_EINVAL, "refinement iterations %d outside 1..4", iterations);
  ctx->eig_refine = iterations;
  return GC_OK;
}

extern "C" int gc_set_chol_blocked(gc_context *ctx, int on) {
  if (!ctx) return GC_EINVAL;
  ctx->chol_blocked = on ? 1 : 0;
  return GC_OK;
}

extern "C" int gc_eig_refine_stats(const gc_context *ctx, long long *solves, long long *fallbacks,
                                   int *max_cluster) {
  if (!ctx) return GC_EINVAL;
  if (solves) *solves = ctx->refine_solves;
  if (fallbacks) *fallbacks = ctx->refine_fallbacks;
  if (max_cluster) *max_cluster = ctx->refine_max_cluster;
  return GC_OK;
}
