// AC0-CAS correlation energy, AC0CAS_FOFO (abfofo.f90:1485-1750).
//
// At lambda = 0 the ERPA matrices are block diagonal once the pairs are grouped
// (create_AC0_blocks_1/2, abfofo.f90:1374-1484): the active-active pairs, the
// (active, q) pairs of every inactive q, the (p, active) pairs of every virtual
// p, and the (virtual, inactive) pairs, whose block is diagonal. The AC0
// energy is first order in lambda:
//   C = Y [2 (X^T A+' X - Y^T A-' Y)_ij / (omega_i + omega_j)] Y^T,
//   ECorr = sum_{pq, rs not in one group} (C_p + C_q)(C_r + C_s) C[pq, rs] (rs|pq),
// with Y, X, omega the block-diagonal zeroth-order ERPA solution (ERPASYMM0,
// interpa.f:1496-1650, per block) and A+-' the AB1 matrices (the lambda
// derivative of A+-B, AB_CAS_FOFO with AB1 = .true.).
//
// Here the pair list is put in block order before the assembly, so that A+-B(0)
// and A+-' come out in block order directly (as ABPM0_FOFO assembles them) and
// every block is a contiguous square. Then:
//   k_ac0_block_erpa  one CTA per block: ERPASYMM0 in FP64 shared memory (two
//                     cyclic-Jacobi eigensolves), Y, X and omega of the block;
//   k_ac0_iv          the (virtual, inactive) pairs: omega = A+(ii,ii), Y = X = 1/sqrt 2;
//   k_ac0_right       T+ = A+' Xbd, T- = A-' Ybd (block-diagonal right products);
//   k_ac0_work        work = 2 (Xbd^T T+ - Ybd^T T-) / (omega_i + omega_j);
//   k_ac0_back_right  U = work Ybd^T;
//   k_ac0_energy      C = Ybd U contracted with the masked, CI-weighted FOFO
//                     integrals on the fly, one partial sum per CTA.
// Every pass is O(N^2 m) for blocks of size m (at most nact(nact-1)/2): there is
// no O(N^3) step, unlike the ERPA solves of the lambda quadrature.
#include <algorithm>
#include <cmath>
#include <vector>

#include "gc_internal.cuh"

namespace {

constexpr int kMaxBlock = 64;  // largest block (threads per block-solve CTA)
constexpr int kRow = kMaxBlock;  // row stride of the block-diagonal factors Yrow / Xrow
const double kSmall = 1e-6;     // interpa.f:1511

// Cyclic Jacobi (Golub and Van Loan, Alg. 8.5.3) on the symmetric m x m matrix A
// (row stride ld) in shared memory, one thread per row; V <- eigenvectors (columns),
// the eigenvalues are left on the diagonal of A. Returns false if 40 sweeps did not
// bring the off-diagonal norm below 1e-30 of the total (uniform across the block).
__device__ bool block_jacobi(double *A, double *V, int m, int ld, double *red) {
  const int l = threadIdx.x;
  if (l < m)
    for (int b = 0; b < m; ++b) V[l * ld + b] = l == b ? 1.0 : 0.0;
  __syncthreads();
  for (int sweep = 0; sweep < 40; ++sweep) {
    double off = 0.0, tot = 0.0;
    if (l < m)
      for (int b = 0; b < m; ++b) {
        const double v = A[l * ld + b] * A[l * ld + b];
        tot += v;
        if (b != l) off += v;
      }
    red[l] = off;
    red[kMaxBlock + l] = tot;
    __syncthreads();
    for (int w = kMaxBlock / 2; w > 0; w >>= 1) {
      if (l < w) {
        red[l] += red[l + w];
        red[kMaxBlock + l] += red[kMaxBlock + l + w];
      }
      __syncthreads();
    }
    const bool done = red[0] <= 1e-30 * red[kMaxBlock];
    __syncthreads();
    if (done) return true;
    for (int p = 0; p < m - 1; ++p)
      for (int q = p + 1; q < m; ++q) {
        const double apq = A[p * ld + q];
        if (apq == 0.0) continue;  // uniform: every thread reads the same value
        const double theta = (A[q * ld + q] - A[p * ld + p]) / (2.0 * apq);
        const double t = (theta >= 0.0 ? 1.0 : -1.0) / (fabs(theta) + sqrt(theta * theta + 1.0));
        const double c = 1.0 / sqrt(t * t + 1.0), sn = t * c;
        __syncthreads();
        if (l < m) {
          const double aip = A[l * ld + p], aiq = A[l * ld + q];
          A[l * ld + p] = c * aip - sn * aiq;
          A[l * ld + q] = sn * aip + c * aiq;
        }
        __syncthreads();
        if (l < m) {
          const double api = A[p * ld + l], aqi = A[q * ld + l];
          A[p * ld + l] = c * api - sn * aqi;
          A[q * ld + l] = sn * api + c * aqi;
          const double vip = V[l * ld + p], viq = V[l * ld + q];
          V[l * ld + p] = c * vip - sn * viq;
          V[l * ld + q] = sn * vip + c * viq;
        }
        __syncthreads();
      }
  }
  return false;
}

// ERPASYMM0 of every block (one CTA of kMaxBlock threads each): block b covers the
// block-order positions bstart[b] .. bstart[b] + bsize[b] - 1 of the column-major
// N x N matrices ap, am (A+-B at lambda = 0). Writes Yrow/Xrow[(s + i) * kRow + c] =
// Y/X(i, c) of the block and eig[s + c]; a Jacobi that does not converge sets *flag.
__global__ void __launch_bounds__(kMaxBlock) k_ac0_block_erpa(
    int N, const double *__restrict__ ap, const double *__restrict__ am,
    const int *__restrict__ bstart, const int *__restrict__ bsize, int ld, double *__restrict__ Yrow,
    double *__restrict__ Xrow, double *__restrict__ eig, int *flag) {
  extern __shared__ double sm[];
  const int s = bstart[blockIdx.x], m = bsize[blockIdx.x];
  double *A = sm, *B = A + kMaxBlock * ld, *P = B + kMaxBlock * ld, *H = P + kMaxBlock * ld,
         *V = H + kMaxBlock * ld;
  __shared__ double red[2 * kMaxBlock];
  __shared__ double w2[kMaxBlock], sq[kMaxBlock];
  const int l = threadIdx.x;
  // symmetrised blocks (interpa.f:1532-1540)
  if (l < m)
    for (int j = 0; j < m; ++j) {
      const size_t e = (size_t)(s + l) + (size_t)(s + j) * N, t = (size_t)(s + j) + (size_t)(s + l) * N;
      A[l * ld + j] = 0.5 * (ap[e] + ap[t]);
      B[l * ld + j] = 0.5 * (am[e] + am[t]);
    }
  __syncthreads();
  if (!block_jacobi(A, V, m, ld, red)) {
    if (l == 0) atomicOr(flag, 1);
    return;  // uniform
  }
  if (l < m) sq[l] = sqrt(fabs(A[l * ld + l]));
  __syncthreads();
  // P = V diag(sqrt|e|) V^T = A+^1/2 (interpa.f:1546-1568)
  if (l < m)
    for (int j = 0; j < m; ++j) {
      double v = 0.0;
      for (int k = 0; k < m; ++k) v += V[l * ld + k] * sq[k] * V[j * ld + k];
      P[l * ld + j] = v;
    }
  __syncthreads();
  // H = A- P, then A <- P H (the symmetrised problem, interpa.f:1578-1581)
  if (l < m)
    for (int j = 0; j < m; ++j) {
      double v = 0.0;
      for (int k = 0; k < m; ++k) v += B[l * ld + k] * P[k * ld + j];
      H[l * ld + j] = v;
    }
  __syncthreads();
  if (l < m)
    for (int j = 0; j < m; ++j) {
      double v = 0.0;
      for (int k = 0; k < m; ++k) v += P[l * ld + k] * H[k * ld + j];
      A[l * ld + j] = v;
    }
  __syncthreads();
  if (l < m)  // the lower triangle, as the eigensolver reads it
    for (int j = l + 1; j < m; ++j) A[l * ld + j] = A[j * ld + l];
  __syncthreads();
  if (!block_jacobi(A, V, m, ld, red)) {
    if (l == 0) atomicOr(flag, 1);
    return;
  }
  if (l < m) w2[l] = A[l * ld + l];
  __syncthreads();
  // Y = P Z into H
  if (l < m)
    for (int j = 0; j < m; ++j) {
      double v = 0.0;
      for (int k = 0; k < m; ++k) v += P[l * ld + k] * V[k * ld + j];
      H[l * ld + j] = v;
    }
  __syncthreads();
  // thread = mode nu: normalise 2/omega y^T A- y = 1, X = A- y / omega (interpa.f:1598-1648)
  if (l < m) {
    const int nu = l;
    double om = w2[nu];
    if (om > kSmall) {
      om = sqrt(om);
      double sum = 0.0;
      for (int i = 0; i < m; ++i) {
        double bi = 0.0;
        for (int j = 0; j < m; ++j) bi += B[i * ld + j] * H[j * ld + nu];
        sum += H[i * ld + nu] * bi;
      }
      sum *= 2.0 / om;
      const double f = sum > 0.0 ? 1.0 / sqrt(sum) : 0.0;
      for (int i = 0; i < m; ++i) H[i * ld + nu] *= f;
      for (int i = 0; i < m; ++i) {
        double bi = 0.0;
        for (int j = 0; j < m; ++j) bi += B[i * ld + j] * H[j * ld + nu];
        Xrow[(size_t)(s + i) * kRow + nu] = bi / om;
        Yrow[(size_t)(s + i) * kRow + nu] = H[i * ld + nu];
      }
    } else {
      for (int i = 0; i < m; ++i) {
        Xrow[(size_t)(s + i) * kRow + nu] = 0.0;
        Yrow[(size_t)(s + i) * kRow + nu] = 0.0;
      }
    }
    eig[s + nu] = om;  // omega, or omega^2 where omega^2 <= Small
  }
}

// (virtual, inactive) pairs, positions iv0..N-1: omega = A+(ii,ii), Y = X = 1/sqrt 2
// (AC0CAS_FOFO, abfofo.f90:1600-1614; the 1/sqrt 2 factor of abpm_tran, tran.f90:634).
__global__ void k_ac0_iv(int N, int iv0, const double *__restrict__ ap, double *__restrict__ Yrow,
                         double *__restrict__ Xrow, double *__restrict__ eig) {
  const int i = iv0 + blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= N) return;
  const double fac = 1.0 / sqrt(2.0);
  eig[i] = ap[(size_t)i + (size_t)i * N];
  Yrow[(size_t)i * kRow] = fac;
  Xrow[(size_t)i * kRow] = fac;
}

// T+[r, c] = sum_k A+'[r, k] Xbd[k, c], T-[r, c] = sum_k A-'[r, k] Ybd[k, c], the sum over
// k in the block of c (bs[c] .. bs[c] + bz[c] - 1). Threads along r: coalesced columns.
__global__ void k_ac0_right(int N, const double *__restrict__ a1p, const double *__restrict__ a1m,
                            const int *__restrict__ bs, const int *__restrict__ bz,
                            const double *__restrict__ Xrow, const double *__restrict__ Yrow,
                            double *__restrict__ tp, double *__restrict__ tm) {
  const int r = blockIdx.x * blockDim.x + threadIdx.x, c = blockIdx.y;
  if (r >= N) return;
  const int s = bs[c], m = bz[c], cc = c - s;
  double vp = 0.0, vm = 0.0;
  for (int b = 0; b < m; ++b) {
    const size_t e = (size_t)r + (size_t)(s + b) * N;
    vp += a1p[e] * Xrow[(size_t)(s + b) * kRow + cc];
    vm += a1m[e] * Yrow[(size_t)(s + b) * kRow + cc];
  }
  tp[(size_t)r + (size_t)c * N] = vp;
  tm[(size_t)r + (size_t)c * N] = vm;
}

// work[r, c] = 2 ((Xbd^T T+)[r, c] - (Ybd^T T-)[r, c]) / (omega_r + omega_c) where both
// omegas are nonzero, else 0 (AC0CAS_FOFO, abfofo.f90:1625-1633).
__global__ void k_ac0_work(int N, const double *__restrict__ tp, const double *__restrict__ tm,
                           const int *__restrict__ bs, const int *__restrict__ bz,
                           const double *__restrict__ Xrow, const double *__restrict__ Yrow,
                           const double *__restrict__ eig, double *__restrict__ work) {
  const int r = blockIdx.x * blockDim.x + threadIdx.x, c = blockIdx.y;
  if (r >= N) return;
  const double er = eig[r], ec = eig[c];
  double v = 0.0;
  if (er != 0.0 && ec != 0.0) {
    const int s = bs[r], m = bz[r], rr = r - s;
    double xp = 0.0, ym = 0.0;
    for (int b = 0; b < m; ++b) {
      const size_t e = (size_t)(s + b) + (size_t)c * N;
      xp += Xrow[(size_t)(s + b) * kRow + rr] * tp[e];
      ym += Yrow[(size_t)(s + b) * kRow + rr] * tm[e];
    }
    v = 2.0 * (xp - ym) / (er + ec);
  }
  work[(size_t)r + (size_t)c * N] = v;
}

// U[r, c] = sum_k work[r, k] Ybd[c, k], k in the block of c (ABPM_BACKTRAN, right factor).
__global__ void k_ac0_back_right(int N, const double *__restrict__ work, const int *__restrict__ bs,
                                 const int *__restrict__ bz, const double *__restrict__ Yrow,
                                 double *__restrict__ u) {
  const int r = blockIdx.x * blockDim.x + threadIdx.x, c = blockIdx.y;
  if (r >= N) return;
  const int s = bs[c], m = bz[c];
  double v = 0.0;
  for (int b = 0; b < m; ++b)
    v += work[(size_t)r + (size_t)(s + b) * N] * Yrow[(size_t)c * kRow + b];
  u[(size_t)r + (size_t)c * N] = v;
}

// C[r, c] = sum_k Ybd[r, k] U[k, c] (k in the block of r), contracted on the fly with
// (C_p + C_q)(C_r' + C_s') (r's'|pq) for pairs r = (p, q), c = (r', s') not in one orbital
// group (the energy loop of AC0CAS_FOFO, abfofo.f90:1676-1720); one partial per CTA.
__global__ void k_ac0_energy(int n, int nocc, int N, const double *__restrict__ u,
                             const int *__restrict__ bs, const int *__restrict__ bz,
                             const double *__restrict__ Yrow, const int *__restrict__ pp,
                             const int *__restrict__ pq, const double *__restrict__ cpl,
                             const int *__restrict__ grp, const double *__restrict__ fofo,
                             double *__restrict__ part) {
  __shared__ double red[256];
  const int r = blockIdx.x * blockDim.x + threadIdx.x;
  double e = 0.0;
  if (r < N) {
    const int p = pp[r], q = pq[r], s = bs[r], m = bz[r];
    const double cpq = cpl[r];  // C_p + C_q
    const size_t ld = (size_t)n * nocc;
    for (int c = blockIdx.y; c < N; c += gridDim.y) {
      const int rr = pp[c], ss = pq[c];
      if (grp[p] == grp[q] && grp[q] == grp[rr] && grp[rr] == grp[ss]) continue;
      double cv = 0.0;
      for (int b = 0; b < m; ++b)
        cv += Yrow[(size_t)r * kRow + b] * u[(size_t)(s + b) + (size_t)c * N];
      const double f = fofo[((size_t)rr + (size_t)ss * n) * ld + p + (size_t)q * n];  // (r's'|pq)
      e += cpq * cpl[c] * cv * f;
    }
  }
  red[threadIdx.x] = e;
  __syncthreads();
  for (int w = blockDim.x / 2; w > 0; w >>= 1) {
    if (threadIdx.x < w) red[threadIdx.x] += red[threadIdx.x + w];
    __syncthreads();
  }
  if (threadIdx.x == 0) part[blockIdx.x + (size_t)gridDim.x * blockIdx.y] = red[0];
}

// out[0] = sum of part[0 .. cnt) (one block, fixed order).
__global__ void k_sum(size_t cnt, const double *__restrict__ part, double *__restrict__ out) {
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

}  // namespace

extern "C" int gc_ac0cas_fofo(gc_context *ctx, int nbas, int ninact, int nact, int ndimx,
                              const double *occ, const double *ure, const double *xone,
                              const int *indn, const double *rdm2act, const double *ffoo,
                              const double *fofo, double *ecorr, double *etot) {
  if (!ctx) return GC_EINVAL;
  if (!occ || !xone || !indn || !ffoo || !fofo || !ecorr || ndimx <= 0 || nbas <= 0 ||
      ninact < 0 || nact < 0 || ninact + nact > nbas)
    return gc::set_error(ctx, GC_EINVAL, "ac0cas_fofo: bad arguments");
  const int n = nbas, nocc = ninact + nact, N = ndimx;
  // Block order of the pairs (create_AC0_blocks_1/2): AA, AI for q = 1..nin, AV for
  // p = nocc+1..n, then the (virtual, inactive) pairs.
  auto grp = [&](int i) { return i < ninact ? 0 : (i < nocc ? 1 : 2); };
  std::vector<int> aa, iv;
  std::vector<std::vector<int>> ai(ninact), av(n > nocc ? n - nocc : 0);
  for (int i = 0; i < N; ++i) {
    const int p = indn[2 * i] - 1, q = indn[2 * i + 1] - 1;
    if (p <= q || p >= n || q < 0 || q >= nocc)
      return gc::set_error(ctx, GC_EINVAL, "ac0cas_fofo: pair %d = (%d,%d) is not valid", i + 1,
                           p + 1, q + 1);
    const int gp = grp(p), gq = grp(q);
    if (gp == 1 && gq == 1) aa.push_back(i);
    else if (gp == 1 && gq == 0) ai[q].push_back(i);
    else if (gp == 2 && gq == 1) av[p - nocc].push_back(i);
    else if (gp == 2 && gq == 0) iv.push_back(i);
    else
      return gc::set_error(ctx, GC_EINVAL, "ac0cas_fofo: pair (%d,%d) in no AC0 block", p + 1, q + 1);
  }
  std::vector<int> order, bstart, bsize, pos_s(N), pos_m(N);
  auto add_block = [&](const std::vector<int> &b) {
    if (b.empty()) return;
    bstart.push_back((int)order.size());
    bsize.push_back((int)b.size());
    for (int i : b) order.push_back(i);
  };
  add_block(aa);
  for (auto &b : ai) add_block(b);
  for (auto &b : av) add_block(b);
  const int iv0 = (int)order.size();
  for (int i : iv) order.push_back(i);
  int mmax = 1;
  for (size_t b = 0; b < bstart.size(); ++b) {
    mmax = std::max(mmax, bsize[b]);
    for (int k = 0; k < bsize[b]; ++k) {
      pos_s[bstart[b] + k] = bstart[b];
      pos_m[bstart[b] + k] = bsize[b];
    }
  }
  for (int k = iv0; k < N; ++k) {
    pos_s[k] = k;
    pos_m[k] = 1;
  }
  if (mmax > kMaxBlock)
    return gc::set_error(ctx, GC_EUNSUPPORTED, "ac0cas_fofo: an AC0 block of %d pairs (limit %d)",
                         mmax, kMaxBlock);
  std::vector<int> indn_blk(2 * (size_t)N);
  for (int k = 0; k < N; ++k) {
    indn_blk[2 * k] = indn[2 * order[k]];
    indn_blk[2 * k + 1] = indn[2 * order[k] + 1];
  }
  // A+-B(0) and the AB1 matrices, assembled in block order
  gc::SysDev sd;
  GC_TRY(gc::sys_upload(ctx, sd, n, ninact, nact, N, occ, xone, indn_blk.data(), rdm2act));
  if (ure) GC_TRY(gc::rotate_h(ctx, sd, ure));
  const size_t NN = (size_t)N * N;
  gc::DevBuf<double> a0p, a0m, a1p, a1m, Yrow, Xrow, eig;
  GC_TRY(a0p.alloc(ctx, NN));
  GC_TRY(a0m.alloc(ctx, NN));
  GC_TRY(a1p.alloc(ctx, NN));
  GC_TRY(a1m.alloc(ctx, NN));
  GC_TRY(gc::assemble_ab(ctx, sd, ffoo, fofo, 0.0, a0p.p, a0m.p, etot, 0));
  GC_TRY(gc::assemble_ab(ctx, sd, ffoo, fofo, 1.0, a1p.p, a1m.p, nullptr, 1));
  GC_TRY(Yrow.alloc(ctx, (size_t)N * kRow));
  GC_TRY(Xrow.alloc(ctx, (size_t)N * kRow));
  GC_TRY(eig.alloc(ctx, N));
  GC_CUDA(ctx, cudaMemsetAsync(Yrow.p, 0, (size_t)N * kRow * sizeof(double), ctx->stream));
  GC_CUDA(ctx, cudaMemsetAsync(Xrow.p, 0, (size_t)N * kRow * sizeof(double), ctx->stream));
  gc::DevBuf<int> dbs, dbz, pbs, pbz, flag;
  const int nblk = (int)bstart.size();
  if (nblk > 0) {
    GC_TRY(dbs.upload(ctx, bstart.data(), nblk));
    GC_TRY(dbz.upload(ctx, bsize.data(), nblk));
  }
  GC_TRY(pbs.upload(ctx, pos_s.data(), N));
  GC_TRY(pbz.upload(ctx, pos_m.data(), N));
  GC_TRY(flag.alloc(ctx, 1));
  GC_CUDA(ctx, cudaMemsetAsync(flag.p, 0, sizeof(int), ctx->stream));
  if (nblk > 0) {
    const int ld = mmax + 1;
    const size_t smem = 5 * (size_t)kMaxBlock * ld * sizeof(double);
    GC_CUDA(ctx, cudaFuncSetAttribute(k_ac0_block_erpa, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                      (int)smem));
    k_ac0_block_erpa<<<nblk, kMaxBlock, smem, ctx->stream>>>(N, a0p.p, a0m.p, dbs.p, dbz.p, ld,
                                                              Yrow.p, Xrow.p, eig.p, flag.p);
    GC_LAUNCHED(ctx);
  }
  if (iv0 < N) {
    k_ac0_iv<<<gc::ceil_div(N - iv0, 256), 256, 0, ctx->stream>>>(N, iv0, a0p.p, Yrow.p, Xrow.p,
                                                                 eig.p);
    GC_LAUNCHED(ctx);
  }
  // Products with the block-diagonal factors. Buffers are reused in stream order:
  // T+ -> a0p, T- -> a0m, work -> a1p, U -> a0p.
  const dim3 blk(256), grid(gc::ceil_div(N, 256), N);
  k_ac0_right<<<grid, blk, 0, ctx->stream>>>(N, a1p.p, a1m.p, pbs.p, pbz.p, Xrow.p, Yrow.p, a0p.p,
                                             a0m.p);
  GC_LAUNCHED(ctx);
  k_ac0_work<<<grid, blk, 0, ctx->stream>>>(N, a0p.p, a0m.p, pbs.p, pbz.p, Xrow.p, Yrow.p, eig.p,
                                            a1p.p);
  GC_LAUNCHED(ctx);
  k_ac0_back_right<<<grid, blk, 0, ctx->stream>>>(N, a1p.p, pbs.p, pbz.p, Yrow.p, a0p.p);
  GC_LAUNCHED(ctx);
  const unsigned gy = (unsigned)std::min(N, 1024);
  const size_t npart = (size_t)gc::ceil_div(N, 256) * gy;
  gc::DevBuf<double> part, res;
  GC_TRY(part.alloc(ctx, npart));
  GC_TRY(res.alloc(ctx, 1));
  k_ac0_energy<<<dim3(gc::ceil_div(N, 256), gy), 256, 0, ctx->stream>>>(
      n, nocc, N, a0p.p, pbs.p, pbz.p, Yrow.p, sd.pair_p.p, sd.pair_q.p, sd.cpl.p, sd.grp.p, fofo,
      part.p);
  GC_LAUNCHED(ctx);
  k_sum<<<1, 1024, 0, ctx->stream>>>(npart, part.p, res.p);
  GC_LAUNCHED(ctx);
  int hflag = 0;
  GC_CUDA(ctx, cudaMemcpyAsync(ecorr, res.p, sizeof(double), cudaMemcpyDeviceToHost, ctx->stream));
  GC_CUDA(ctx, cudaMemcpyAsync(&hflag, flag.p, sizeof(int), cudaMemcpyDeviceToHost, ctx->stream));
  GC_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
  if (hflag)
    return gc::set_error(ctx, GC_ECUSOLVER, "ac0cas_fofo: a block eigensolve did not converge");
  if (!std::isfinite(*ecorr))
    return gc::set_error(ctx, GC_ENONFINITE, "ac0cas_fofo: the energy is not finite");
  return GC_OK;
}
