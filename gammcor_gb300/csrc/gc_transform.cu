// AO -> MO four-index transform into the FFOO / FOFO record layout.
//
// gc_tran4_gen follows tran4_gen (tran.f90:313-423): phase 1 contracts every
// AO pair record rs with CA^T . M . CB, phase 2 contracts every (ab| column
// over the unpacked rs index with CC^T . M . CD. Out-of-core files become
// HBM buffers: the AOTWOSORT tensor, the half-transformed TMPMO intermediate
// (ntr x nA*nB) and the output all stay resident. Packed triangles are
// expanded by the unpack kernels below (triang_to_sq, tran.f90:1221-1247).
//
// gc_tran4_factored produces the same records from the ERI factor L:
// B_P = CA^T L_P CB for every P, then (ab|cd) = sum_P B_P(ab) B'_P(cd).
#include "gc_internal.cuh"
#include "gc_tc_gemm.cuh"

namespace {

__host__ __device__ inline long long tri_pack(int p, int q) {  // p <= q, 0-based
  return (long long)p + (long long)q * (q + 1) / 2;
}

// Expand records [rs0, rs0+cnt) of the packed tensor G (ntr x ntr, record-major)
// into cnt column-major n x n matrices.
__global__ void unpack_records(const double *__restrict__ G, long long ntr, int n, long long rs0,
                               int cnt, double *__restrict__ M) {
  long long total = (long long)cnt * n * n;
  for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x; t < total;
       t += (long long)gridDim.x * blockDim.x) {
    int p = (int)(t % n);
    long long r = t / n;
    int q = (int)(r % n);
    long long k = r / n;
    long long pq = p <= q ? tri_pack(p, q) : tri_pack(q, p);
    M[t] = G[(rs0 + k) * ntr + pq];
  }
}

// Expand columns [c0, c0+cnt) of H (ntr x ncol, row index = packed rs, column
// fastest) into cnt column-major n x n matrices. Tiled through shared memory so
// that both the H reads (along columns) and the M writes (along packed rs,
// i.e. along r for fixed s) are contiguous.
__global__ void unpack_columns(const double *__restrict__ H, long long ntr, long long ncol, int n,
                               long long c0, int cnt, double *__restrict__ M) {
  __shared__ double tile[32][33];
  long long rs_base = (long long)blockIdx.x * 32;
  long long c_base = (long long)blockIdx.y * 32;
  int tx = threadIdx.x, ty = threadIdx.y;  // 32 x 8
  for (int i = ty; i < 32; i += 8) {
    long long rs = rs_base + i;
    long long c = c_base + tx;
    tile[i][tx] = (rs < ntr && c < cnt) ? H[rs * ncol + c0 + c] : 0.0;
  }
  __syncthreads();
  for (int j = ty; j < 32; j += 8) {
    long long c = c_base + j;
    long long rs = rs_base + tx;
    if (c >= cnt || rs >= ntr) continue;
    // invert rs = r + s(s+1)/2, r <= s
    int s = (int)((sqrt(8.0 * (double)rs + 1.0) - 1.0) * 0.5);
    while ((long long)s * (s + 1) / 2 > rs) s--;
    while ((long long)(s + 1) * (s + 2) / 2 <= rs) s++;
    int r = (int)(rs - (long long)s * (s + 1) / 2);
    double v = tile[tx][j];
    double *Mc = M + c * (long long)n * n;
    Mc[r + (long long)s * n] = v;
    Mc[s + (long long)r * n] = v;
  }
}

// L (ntr x rank, column-major) -> rank column-major n x n matrices.
__global__ void unpack_factor(const double *__restrict__ L, long long ntr, int n, int P0, int cnt,
                              double *__restrict__ M) {
  long long total = (long long)cnt * n * n;
  for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x; t < total;
       t += (long long)gridDim.x * blockDim.x) {
    int p = (int)(t % n);
    long long r = t / n;
    int q = (int)(r % n);
    long long P = r / n;
    long long pq = p <= q ? tri_pack(p, q) : tri_pack(q, p);
    M[t] = L[(P0 + P) * ntr + pq];
  }
}

// Two-sided transform of cnt column-major n x n matrices M_k:
// out_k (nX x nY, column-major, stride ostride) = CX^T M_k CY.
int two_sided(gc_context *ctx, int n, int cnt, const double *M, int nX, const double *CX, int nY,
              const double *CY, double *T1, double *out, long long ostride) {
  const double one = 1.0, zero = 0.0;
  // T1 (nX x n*cnt) = CX^T . [M_0 | M_1 | ...]
  GC_CUBLAS(ctx, cublasDgemm(ctx->cublas, CUBLAS_OP_T, CUBLAS_OP_N, nX, n * cnt, n, &one, CX, n, M,
                             n, &zero, T1, nX));
  // out_k = T1_k . CY
  GC_CUBLAS(ctx, cublasDgemmStridedBatched(ctx->cublas, CUBLAS_OP_N, CUBLAS_OP_N, nX, nY, n, &one,
                                           T1, nX, (long long)nX * n, CY, n, 0, &zero, out, nX,
                                           ostride, cnt));
  return GC_OK;
}

int check_dims(gc_context *ctx, int nbas, int nA, int nB, int nC, int nD) {
  if (nbas <= 0 || nA <= 0 || nB <= 0 || nC <= 0 || nD <= 0 || nA > nbas || nB > nbas ||
      nC > nbas || nD > nbas)
    return gc::set_error(ctx, GC_EINVAL, "tran4: bad dimensions nbas=%d nA=%d nB=%d nC=%d nD=%d",
                         nbas, nA, nB, nC, nD);
  return GC_OK;
}

const size_t kChunkBytes = size_t(1) << 30;  // unpacked-matrix staging per chunk

}  // namespace

extern "C" int gc_tran4_gen(gc_context *ctx, int nbas, int nA, const double *CA, int nB,
                            const double *CB, int nC, const double *CC, int nD, const double *CD,
                            const double *G, double *out, int precision) {
  if (!ctx) return GC_EINVAL;
  gc::PhaseScope ph(ctx, GC_PHASE_TRANSFORM);
  GC_TRY(check_dims(ctx, nbas, nA, nB, nC, nD));
  if (precision < GC_PREC_FP64 || precision > GC_PREC_FP64TC4)
    return gc::set_error(ctx, GC_EINVAL, "tran4_gen: unknown precision %d", precision);
  const int n = nbas;
  const long long ntr = (long long)n * (n + 1) / 2;
  const long long nAB = (long long)nA * nB, nCD = (long long)nC * nD;
  const long long n2 = (long long)n * n;
  gc::DevBuf<double> H, M, T1;
  GC_TRY(H.alloc(ctx, ntr * nAB));
  int cs = (int)std::max<long long>(1, std::min<long long>(ntr, kChunkBytes / (8 * n2)));
  GC_TRY(M.alloc(ctx, (size_t)cs * n2));
  int tmax = std::max(nA, nC);
  GC_TRY(T1.alloc(ctx, (size_t)cs * n * tmax));
  // phase 1: (ab| for every rs
  for (long long rs0 = 0; rs0 < ntr; rs0 += cs) {
    int cnt = (int)std::min<long long>(cs, ntr - rs0);
    unsigned grid = std::min<unsigned>(gc::ceil_div((size_t)cnt * n2, 256), 152u * 32u);
    unpack_records<<<grid, 256, 0, ctx->stream>>>(G, ntr, n, rs0, cnt, M.p);
    GC_LAUNCHED(ctx);
    GC_TRY(gc::tc_two_sided(ctx, precision, n, cnt, M.p, nA, CA, nB, CB, T1.p, H.p + rs0 * nAB, nAB));
  }
  // phase 2: |cd) for every ab
  for (long long c0 = 0; c0 < nAB; c0 += cs) {
    int cnt = (int)std::min<long long>(cs, nAB - c0);
    dim3 grid(gc::ceil_div(ntr, 32), gc::ceil_div(cnt, 32));
    unpack_columns<<<grid, dim3(32, 8), 0, ctx->stream>>>(H.p, ntr, nAB, n, c0, cnt, M.p);
    GC_LAUNCHED(ctx);
    GC_TRY(gc::tc_two_sided(ctx, precision, n, cnt, M.p, nC, CC, nD, CD, T1.p, out + c0 * nCD, nCD));
  }
  return precision == GC_PREC_FP64 ? GC_OK : gc::check_flag(ctx);
}

extern "C" int gc_tran4_factored(gc_context *ctx, int nbas, int rank, const double *L, int nA,
                                 const double *CA, int nB, const double *CB, int nC,
                                 const double *CC, int nD, const double *CD, double *out,
                                 int precision) {
  if (!ctx) return GC_EINVAL;
  gc::PhaseScope ph(ctx, GC_PHASE_TRANSFORM);
  GC_TRY(check_dims(ctx, nbas, nA, nB, nC, nD));
  if (rank <= 0) return gc::set_error(ctx, GC_EINVAL, "tran4_factored: rank=%d", rank);
  const int n = nbas;
  const long long ntr = (long long)n * (n + 1) / 2;
  const long long nAB = (long long)nA * nB, nCD = (long long)nC * nD;
  const long long n2 = (long long)n * n;
  const bool same = (CA == CC && CB == CD && nA == nC && nB == nD);
  gc::DevBuf<double> Y, Z, M, T1;
  GC_TRY(Y.alloc(ctx, nAB * rank));
  if (!same) GC_TRY(Z.alloc(ctx, nCD * rank));
  int cs = (int)std::max<long long>(1, std::min<long long>(rank, kChunkBytes / (8 * n2)));
  GC_TRY(M.alloc(ctx, (size_t)cs * n2));
  GC_TRY(T1.alloc(ctx, (size_t)cs * n * std::max(nA, nC)));
  for (int P0 = 0; P0 < rank; P0 += cs) {
    int cnt = std::min(cs, rank - P0);
    unsigned grid = std::min<unsigned>(gc::ceil_div((size_t)cnt * n2, 256), 152u * 32u);
    unpack_factor<<<grid, 256, 0, ctx->stream>>>(L, ntr, n, P0, cnt, M.p);
    GC_LAUNCHED(ctx);
    GC_TRY(gc::tc_two_sided(ctx, precision, n, cnt, M.p, nA, CA, nB, CB, T1.p, Y.p + P0 * nAB, nAB));
    if (!same)
      GC_TRY(gc::tc_two_sided(ctx, precision, n, cnt, M.p, nC, CC, nD, CD, T1.p, Z.p + P0 * nCD, nCD));
  }
  // out (nCD x nAB, column-major == record-major) = Z . Y^T
  const double *Zp = same ? Y.p : Z.p;
  GC_TRY(gc::tc_gemm_nt(ctx, precision, (int)nCD, (int)nAB, rank, Zp, (int)nCD, Y.p, (int)nAB, out,
                        (int)nCD));
  return precision == GC_PREC_FP64 ? GC_OK : gc::check_flag(ctx);
}

namespace gc {

// FP64 fallback of the two building blocks; the tensor-core versions live in
// gc_tc_gemm.cu and are selected by precision.
int fp64_two_sided(gc_context *ctx, int n, int cnt, const double *M, int nX, const double *CX,
                   int nY, const double *CY, double *T1, double *out, long long ostride) {
  return two_sided(ctx, n, cnt, M, nX, CX, nY, CY, T1, out, ostride);
}

}  // namespace gc
