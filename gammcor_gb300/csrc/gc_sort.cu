// AO two-electron integrals into the AOTWOSORT layout that tran4_gen reads.
//
// readtwoint (sorter.f90:31-395) reads the AO integral file of the quantum-
// chemistry program, sorts every integral into the bucket of its rs pair index
// (add_to_Sorter, sorter.f90:456-472) and writes record rs = all pq values
// (get_from_Sorter, sorter.f90:517-539, which starts every record at zero and
// lets a later integral overwrite an earlier one for the same slot). Packed
// pair indices are pq = p + q(q-1)/2 for 1-based p <= q.
//
// gc_sort_twoint does the same on the device for one chunk of integrals (values
// and labels in device memory), in the label formats the reference decodes:
//   GC_TWOINT_DALTON8   one int per integral, p, q, r, s in bits 0-7, 8-15, 16-23,
//                       24-31 (Dalton, nibuf = 1, sorter.f90:84-104);
//   GC_TWOINT_DALTON16  two ints per integral, (r | s << 16) and (p | q << 16)
//                       (Dalton, nibuf = 2, sorter.f90:106-125);
//   GC_TWOINT_PQRS      four ints p, q, r, s per integral, any order within each
//                       pair (the value/label stream, sorter.f90:303-318);
//   GC_TWOINT_TRIANGLE  no labels: the ntr(ntr+1)/2 values with pq >= rs in the
//                       order p = 1..n, q = 1..p, r = 1..n, s = 1..r (sorter.f90:324-345).
// Every integral lands in record rs at pq and, by each format's rule, in record
// pq at rs. Within a chunk a slot written by several integrals keeps the value of
// the last one in input order: the slots first receive the largest input position
// aimed at them (atomicMax on the 64-bit slot), every integral then records
// whether it is its slot's winner, and only the winners write their values, so
// the result does not depend on thread scheduling. Chunks are applied in call
// order on the context's stream, so a later chunk overwrites an earlier one as in
// the reference.
#include <cstdint>

#include "gc_internal.cuh"
#include "gc_tc_gemm.cuh"

namespace {

__device__ __forceinline__ long long tri1(long long p, long long q) {  // 1-based, p <= q
  return p + q * (q - 1) / 2;
}

// The one or two placements of integral t: (record, element) 1-based; n placements.
__device__ __forceinline__ int placements(int format, long long t, const int *__restrict__ lab,
                                          long long *rec, long long *el) {
  long long pq, rs;
  bool both;
  if (format == GC_TWOINT_DALTON8) {
    const unsigned x = (unsigned)lab[t];
    const long long p = x & 255u, q = (x >> 8) & 255u, r = (x >> 16) & 255u, s = (x >> 24) & 255u;
    pq = p + q * (q - 1) / 2;
    rs = r + s * (s - 1) / 2;
    both = pq < rs;
  } else if (format == GC_TWOINT_DALTON16) {
    const unsigned a = (unsigned)lab[2 * t], b = (unsigned)lab[2 * t + 1];
    const long long r = a & 65535u, s = a >> 16, p = b & 65535u, q = b >> 16;
    pq = p + q * (q - 1) / 2;
    rs = r + s * (s - 1) / 2;
    both = pq < rs;
  } else if (format == GC_TWOINT_PQRS) {
    const long long p = lab[4 * t], q = lab[4 * t + 1], r = lab[4 * t + 2], s = lab[4 * t + 3];
    pq = p <= q ? tri1(p, q) : tri1(q, p);
    rs = r <= s ? tri1(r, s) : tri1(s, r);
    both = true;
  } else {  // GC_TWOINT_TRIANGLE: t = pq (pq - 1) / 2 + rs - 1 with rs <= pq
    long long a = (long long)((sqrt(8.0 * (double)t + 1.0) + 1.0) * 0.5);
    while (a * (a - 1) / 2 > t) --a;
    while ((a + 1) * a / 2 <= t) ++a;
    pq = a;
    rs = t - a * (a - 1) / 2 + 1;
    both = true;
  }
  rec[0] = rs;
  el[0] = pq;
  if (both) {
    rec[1] = pq;
    el[1] = rs;
    return 2;
  }
  return 1;
}

__device__ __forceinline__ bool in_range(long long rec, long long el, long long ntr) {
  return rec >= 1 && rec <= ntr && el >= 1 && el <= ntr;
}

// phase 0: zero the slots of this chunk; *bad counts labels outside 1..n
__global__ void k_sort_clear(int format, long long nints, const int *__restrict__ lab,
                             long long ntr, unsigned long long *__restrict__ out, int *bad) {
  for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x; t < nints;
       t += (long long)gridDim.x * blockDim.x) {
    long long rec[2], el[2];
    const int k = placements(format, t, lab, rec, el);
    for (int i = 0; i < k; ++i) {
      if (!in_range(rec[i], el[i], ntr)) {
        atomicAdd(bad, 1);
        continue;
      }
      out[(rec[i] - 1) * ntr + (el[i] - 1)] = 0ull;
    }
  }
}

// phase 1: every slot gets the largest (input position + 1) aimed at it
__global__ void k_sort_claim(int format, long long nints, const int *__restrict__ lab,
                             long long ntr, unsigned long long *__restrict__ out) {
  for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x; t < nints;
       t += (long long)gridDim.x * blockDim.x) {
    long long rec[2], el[2];
    const int k = placements(format, t, lab, rec, el);
    for (int i = 0; i < k; ++i)
      if (in_range(rec[i], el[i], ntr))
        atomicMax(out + (rec[i] - 1) * ntr + (el[i] - 1), (unsigned long long)(t + 1));
  }
}

// phase 2: win[t] bit i = placement i of integral t won its slot
__global__ void k_sort_winners(int format, long long nints, const int *__restrict__ lab,
                               long long ntr, const unsigned long long *__restrict__ out,
                               unsigned char *__restrict__ win) {
  for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x; t < nints;
       t += (long long)gridDim.x * blockDim.x) {
    long long rec[2], el[2];
    const int k = placements(format, t, lab, rec, el);
    unsigned char w = 0;
    for (int i = 0; i < k; ++i)
      if (in_range(rec[i], el[i], ntr) &&
          out[(rec[i] - 1) * ntr + (el[i] - 1)] == (unsigned long long)(t + 1))
        w |= (unsigned char)(1u << i);
    win[t] = w;
  }
}

// phase 3: the winners write their values
__global__ void k_sort_write(int format, long long nints, const int *__restrict__ lab,
                             const double *__restrict__ val, long long ntr,
                             const unsigned char *__restrict__ win, double *__restrict__ out) {
  for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x; t < nints;
       t += (long long)gridDim.x * blockDim.x) {
    const unsigned char w = win[t];
    if (!w) continue;
    long long rec[2], el[2];
    const int k = placements(format, t, lab, rec, el);
    for (int i = 0; i < k; ++i)
      if (w & (1u << i)) out[(rec[i] - 1) * ntr + (el[i] - 1)] = val[t];
  }
}

// The dense triangle has no duplicates: one pass writes both placements.
__global__ void k_sort_triangle(long long nints, const double *__restrict__ val, long long ntr,
                                double *__restrict__ out) {
  for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x; t < nints;
       t += (long long)gridDim.x * blockDim.x) {
    long long rec[2], el[2];
    placements(GC_TWOINT_TRIANGLE, t, nullptr, rec, el);
    const double v = val[t];
    out[(rec[0] - 1) * ntr + (el[0] - 1)] = v;
    out[(rec[1] - 1) * ntr + (el[1] - 1)] = v;
  }
}

}  // namespace

extern "C" int gc_sort_twoint(gc_context *ctx, int nbas, long long nints, const double *val_dev,
                              const int *labels_dev, int format, int init, double *ao_sorted_dev) {
  if (!ctx) return GC_EINVAL;
  const long long ntr = (long long)nbas * (nbas + 1) / 2;
  if (nbas <= 0 || nints < 0 || !val_dev || !ao_sorted_dev ||
      (format != GC_TWOINT_TRIANGLE && !labels_dev) || format < GC_TWOINT_DALTON8 ||
      format > GC_TWOINT_TRIANGLE || (format == GC_TWOINT_DALTON8 && nbas > 255) ||
      (format == GC_TWOINT_DALTON16 && nbas > 65535) ||
      (format == GC_TWOINT_TRIANGLE && nints != ntr * (ntr + 1) / 2))
    return gc::set_error(ctx, GC_EINVAL, "sort_twoint: bad arguments (nbas=%d nints=%lld format=%d)",
                         nbas, nints, format);
  if (init)
    GC_CUDA(ctx, cudaMemsetAsync(ao_sorted_dev, 0, (size_t)ntr * ntr * sizeof(double), ctx->stream));
  if (nints == 0) return GC_OK;
  const unsigned grid = (unsigned)std::min<long long>((nints + 255) / 256, 152ll * 32);
  if (format == GC_TWOINT_TRIANGLE) {
    k_sort_triangle<<<grid, 256, 0, ctx->stream>>>(nints, val_dev, ntr, ao_sorted_dev);
    GC_LAUNCHED(ctx);
    return GC_OK;
  }
  auto *out = reinterpret_cast<unsigned long long *>(ao_sorted_dev);
  gc::DevBuf<unsigned char> win;
  gc::DevBuf<int> bad;
  GC_TRY(win.alloc(ctx, (size_t)nints));
  GC_TRY(bad.alloc(ctx, 1));
  GC_CUDA(ctx, cudaMemsetAsync(bad.p, 0, sizeof(int), ctx->stream));
  k_sort_clear<<<grid, 256, 0, ctx->stream>>>(format, nints, labels_dev, ntr, out, bad.p);
  GC_LAUNCHED(ctx);
  k_sort_claim<<<grid, 256, 0, ctx->stream>>>(format, nints, labels_dev, ntr, out);
  GC_LAUNCHED(ctx);
  k_sort_winners<<<grid, 256, 0, ctx->stream>>>(format, nints, labels_dev, ntr, out, win.p);
  GC_LAUNCHED(ctx);
  k_sort_write<<<grid, 256, 0, ctx->stream>>>(format, nints, labels_dev, val_dev, ntr, win.p,
                                              ao_sorted_dev);
  GC_LAUNCHED(ctx);
  int hbad = 0;
  GC_CUDA(ctx, cudaMemcpyAsync(&hbad, bad.p, sizeof(int), cudaMemcpyDeviceToHost, ctx->stream));
  GC_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
  if (hbad)
    return gc::set_error(ctx, GC_EINVAL, "sort_twoint: %d labels outside 1..%d (skipped)", hbad,
                         nbas);
  return GC_OK;
}

extern "C" int gc_ao_eri_factored(gc_context *ctx, int nbas, int rank, const double *lfac_dev,
                                  double *ao_sorted_dev, int precision) {
  // (pq|rs) = sum_P L(pq, P) L(rs, P): the AOTWOSORT tensor as L L^T (ntr x ntr)
  if (!ctx) return GC_EINVAL;
  const long long ntr = (long long)nbas * (nbas + 1) / 2;
  if (nbas <= 0 || rank <= 0 || !lfac_dev || !ao_sorted_dev || ntr > 2147483647ll)
    return gc::set_error(ctx, GC_EINVAL, "ao_eri_factored: bad arguments");
  GC_TRY(gc::tc_gemm_nt(ctx, precision, (int)ntr, (int)ntr, rank, lfac_dev, (int)ntr, lfac_dev,
                        (int)ntr, ao_sorted_dev, (int)ntr));
  return precision == GC_PREC_FP64 ? GC_OK : gc::check_flag(ctx);
}
