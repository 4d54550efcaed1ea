// Split-precision tensor-core GEMM on tcgen05 (sm_103a).
//
//   C[m, n] = sum_pass sum_k A_pa(pass)[m, k] * B_pb(pass)[n, k]
//
// FP64 operands are split into BF16 planes x = x0 + x1 (+ x2) by pack_planes;
// a pass list selects the plane products that are kept (3 passes for
// hi*hi + hi*lo + lo*hi, 6 passes with a third plane, which brings the
// product error to the FP32 level). All passes accumulate into one FP32
// accumulator in tensor memory.
//
// Kernel structure (one CTA per 128 x BN output tile, 192 threads):
//   warp 0  TMA producer: 64-wide K slices of A and B into a STAGES-deep
//           shared-memory ring (128B swizzle), completion on mbarriers;
//   warp 1  allocates TMEM, one elected thread issues tcgen05.mma
//           (M=128, N=BN, K=16) and tcgen05.commit to release ring slots;
//   warps 2-5 epilogue: tcgen05.ld of the accumulator, then either a FP64
//           store or a fused dot product with an FP64 matrix (integrand).
// Every mbarrier wait is bounded; on expiry the CTA records an error in a
// device flag, drains its own copies and frees TMEM before returning.
#include <cuda.h>
#include <cuda_bf16.h>

#include <mutex>

#include "gc_tc_gemm.cuh"

namespace {

constexpr int BM = 128;
constexpr int BK = 64;  // bf16 elements per K slice = one 128-byte swizzle row
constexpr int STAGES = 4;
constexpr int MAXPASS = 8;
constexpr unsigned long long kWaitNs = 1000000000ull;  // a wait longer than 1 s is an error

struct PassList {
  int n;
  int pa[MAXPASS];
  int pb[MAXPASS];
};

struct Epi {
  int mode;             // 0: store C (FP64); 1: partial[cta] = sum C .* R
  double *c;            // mode 0 output
  long long ldn;        // element (m, n) at c[b*sb + m + n*ldn]
  long long sb;
  const double *r;      // mode 1 matrix, same indexing
  double *partial;      // mode 1: one double per CTA
};

// ---------------------------------------------------------------- PTX helpers
__device__ __forceinline__ uint32_t smem_u32(const void *p) {
  return (uint32_t)__cvta_generic_to_shared(p);
}

__device__ __forceinline__ void mbar_init(uint64_t *bar, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count));
}

__device__ __forceinline__ void mbar_expect_tx(uint64_t *bar, uint32_t bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)),
               "r"(bytes)
               : "memory");
}

__device__ __forceinline__ unsigned long long globaltimer() {
  unsigned long long t;
  asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
  return t;
}

// Bounded parity wait: returns false if the phase did not complete within kWaitNs.
__device__ __forceinline__ bool mbar_wait(uint64_t *bar, uint32_t parity) {
  uint32_t addr = smem_u32(bar);
  unsigned long long t0 = 0;
  for (unsigned it = 0;; ++it) {
    uint32_t ok;
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
        "selp.u32 %0, 1, 0, p;\n\t}"
        : "=r"(ok)
        : "r"(addr), "r"(parity)
        : "memory");
    if (ok) return true;
    if ((it & 255) == 0) {
      unsigned long long t = globaltimer();
      if (t0 == 0) t0 = t;
      else if (t - t0 > kWaitNs) return false;
    }
  }
}

__device__ __forceinline__ void tma_load_4d(void *dst, const CUtensorMap *map, uint64_t *bar, int c0,
                                            int c1, int c2, int c3) {
  asm volatile(
      "cp.async.bulk.tensor.4d.shared::cluster.global.tile.mbarrier::complete_tx::bytes"
      " [%0], [%1, {%3, %4, %5, %6}], [%2];" ::"r"(smem_u32(dst)),
      "l"((uint64_t)map), "r"(smem_u32(bar)), "r"(c0), "r"(c1), "r"(c2), "r"(c3)
      : "memory");
}

// Shared-memory matrix descriptor: K-major tile, 128-byte swizzle, 8-row groups
// 1024 bytes apart (SBO), version 1 (bits 46-47), layout SWIZZLE_128B (bits 61-63 = 2).
__device__ __forceinline__ uint64_t smem_desc(uint32_t saddr) {
  uint64_t d = 0;
  d |= (uint64_t)((saddr & 0x3FFFF) >> 4);
  d |= (uint64_t)1 << 16;            // LBO (unused for swizzled K-major)
  d |= (uint64_t)(1024 >> 4) << 32;  // SBO
  d |= (uint64_t)1 << 46;            // descriptor version
  d |= (uint64_t)2 << 61;            // SWIZZLE_128B
  return d;
}

// Instruction descriptor, kind::f16: D=F32, A=B=BF16, both K-major, M=128, N=bn.
__host__ __device__ constexpr uint32_t instr_desc(int bn) {
  return (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(bn >> 3) << 17) |
         ((uint32_t)(BM >> 4) << 24);
}

__device__ __forceinline__ void mma_bf16(uint32_t tmem, uint64_t ad, uint64_t bd, uint32_t idesc,
                                         uint32_t accumulate) {
  asm volatile(
      "{\n\t.reg .pred p;\n\t"
      "setp.ne.b32 p, %4, 0;\n\t"
      "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}" ::"r"(tmem),
      "l"(ad), "l"(bd), "r"(idesc), "r"(accumulate));
}

__device__ __forceinline__ void mma_commit(uint64_t *bar) {
  asm volatile(
      "tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(
          smem_u32(bar))
      : "memory");
}

__device__ __forceinline__ void tmem_ld16(uint32_t taddr, float *v) {
  uint32_t r[16];
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, "
      "%12, %13, %14, %15}, [%16];"
      : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]),
        "=r"(r[7]), "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]),
        "=r"(r[14]), "=r"(r[15])
      : "r"(taddr));
  asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
  for (int i = 0; i < 16; ++i) v[i] = __uint_as_float(r[i]);
}

// ------------------------------------------------------------------- kernel
template <int BN>
__global__ void __launch_bounds__(192, 1)
    k_tc_gemm(const __grid_constant__ CUtensorMap mapA, const __grid_constant__ CUtensorMap mapB,
              int M, int N, int kblocks, int a_batched, int b_batched, PassList passes, Epi epi,
              int *err_flag) {
  extern __shared__ __align__(1024) uint8_t smem_raw[];
  uint8_t *smem = (uint8_t *)(((uintptr_t)smem_raw + 1023) & ~(uintptr_t)1023);
  constexpr uint32_t A_BYTES = BM * BK * 2, B_BYTES = BN * BK * 2;
  uint8_t *sA = smem;
  uint8_t *sB = smem + STAGES * A_BYTES;
  uint64_t *full = (uint64_t *)(sB + STAGES * B_BYTES);
  uint64_t *empty = full + STAGES;
  uint64_t *accf = empty + STAGES;
  uint32_t *tmem_slot = (uint32_t *)(accf + 1);
  __shared__ int abort_flag;
  __shared__ double red[4];

  const int warp = threadIdx.x / 32, lane = threadIdx.x % 32;
  const int m0 = blockIdx.x * BM, n0 = blockIdx.y * BN, b = blockIdx.z;
  const int total = passes.n * kblocks;

  if (threadIdx.x == 0) {
    for (int s = 0; s < STAGES; ++s) {
      mbar_init(&full[s], 1);
      mbar_init(&empty[s], 1);
    }
    mbar_init(accf, 1);
    abort_flag = 0;
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  if (warp == 1) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(
                     smem_u32(tmem_slot)),
                 "r"((uint32_t)BN));
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
  }
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
  const uint32_t tmem = *tmem_slot;

  if (warp == 0 && lane == 0) {
    // ---------------- TMA producer
    int issued = 0;
    for (int it = 0; it < total; ++it) {
      int s = it % STAGES;
      uint32_t ph = (it / STAGES) & 1;
      if (!mbar_wait(&empty[s], ph ^ 1)) {
        atomicExch(&abort_flag, 1);
        break;
      }
      if (abort_flag) break;
      int pass = it / kblocks, kb = it % kblocks;
      mbar_expect_tx(&full[s], A_BYTES + B_BYTES);
      tma_load_4d(sA + s * A_BYTES, &mapA, &full[s], kb * BK, m0, a_batched ? b : 0,
                  passes.pa[pass]);
      tma_load_4d(sB + s * B_BYTES, &mapB, &full[s], kb * BK, n0, b_batched ? b : 0,
                  passes.pb[pass]);
      issued = it + 1;
    }
    if (abort_flag) {
      // drain copies already issued into the ring before the CTA exits
      for (int it = (issued > STAGES ? issued - STAGES : 0); it < issued; ++it)
        mbar_wait(&full[it % STAGES], (it / STAGES) & 1);
    }
  } else if (warp == 1 && lane == 0) {
    // ---------------- MMA issuer
    constexpr uint32_t idesc = instr_desc(BN);
    bool ok = true;
    for (int it = 0; it < total && ok; ++it) {
      int s = it % STAGES;
      uint32_t ph = (it / STAGES) & 1;
      if (!mbar_wait(&full[s], ph) || abort_flag) {
        atomicExch(&abort_flag, 1);
        ok = false;
        break;
      }
      asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
      uint32_t a_addr = smem_u32(sA + s * A_BYTES), b_addr = smem_u32(sB + s * B_BYTES);
#pragma unroll
      for (int kk = 0; kk < BK / 16; ++kk) {
        uint64_t ad = smem_desc(a_addr + kk * 32), bd = smem_desc(b_addr + kk * 32);
        mma_bf16(tmem, ad, bd, idesc, (it > 0 || kk > 0) ? 1u : 0u);
      }
      mma_commit(&empty[s]);
    }
    mma_commit(accf);  // arrives once all issued MMAs have completed
  } else if (warp >= 2) {
    // ---------------- epilogue
    const int q = warp & 3;  // TMEM lane quarter this warp may access
    const int m = m0 + q * 32 + lane;
    bool ok = mbar_wait(accf, 0);
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    double acc = 0.0;
    if (ok && !abort_flag) {
      for (int c0 = 0; c0 < BN; c0 += 16) {
        float v[16];
        tmem_ld16(tmem + ((uint32_t)(q * 32) << 16) + (uint32_t)c0, v);
        if (m < M) {
#pragma unroll
          for (int j = 0; j < 16; ++j) {
            int n = n0 + c0 + j;
            if (n < N) {
              long long o = (long long)b * epi.sb + m + (long long)n * epi.ldn;
              if (epi.mode == 0)
                epi.c[o] = (double)v[j];
              else
                acc += (double)v[j] * epi.r[o];
            }
          }
        }
      }
    } else {
      atomicExch(&abort_flag, 1);
    }
    if (epi.mode == 1) {
      for (int off = 16; off > 0; off >>= 1) acc += __shfl_down_sync(0xffffffffu, acc, off);
      if (lane == 0) red[warp - 2] = acc;
    }
  }
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  if (epi.mode == 1 && threadIdx.x == 0) {
    long long cta = blockIdx.x + (long long)gridDim.x * (blockIdx.y + (long long)gridDim.y * blockIdx.z);
    epi.partial[cta] = red[0] + red[1] + red[2] + red[3];
  }
  if (threadIdx.x == 0 && abort_flag) atomicExch(err_flag, 1);
  if (warp == 1) {
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem),
                 "r"((uint32_t)BN));
  }
}

// ------------------------------------------------------------ operand packing
// planes[s][b][r][kp] (bf16) from x[b*sb + r*sr + k*sk] (FP64): x = x0 + x1 + x2 + ...
__global__ void k_pack_planes(const double *__restrict__ x, int rows, int K, int Kp, int nb,
                              long long sr, long long sk, long long sb, int S,
                              __nv_bfloat16 *__restrict__ planes) {
  long long plane = (long long)nb * rows * Kp;
  long long total = plane;
  for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x; t < total;
       t += (long long)gridDim.x * blockDim.x) {
    int k = (int)(t % Kp);
    long long rr = t / Kp;
    int r = (int)(rr % rows);
    long long bb = rr / rows;
    double v = k < K ? x[bb * sb + r * sr + (long long)k * sk] : 0.0;
    for (int s = 0; s < S; ++s) {
      __nv_bfloat16 h = __double2bfloat16(v);
      planes[s * plane + t] = h;
      v -= (double)__bfloat162float(h);
    }
  }
}

// Same, for operands whose K index is the slow one (sk >> sr): a 32 x 32 tile
// is staged in shared memory so that reads run along rows and writes along K.
__global__ void k_pack_planes_t(const double *__restrict__ x, int rows, int K, int Kp, int nb,
                                long long sr, long long sk, long long sb, int S,
                                __nv_bfloat16 *__restrict__ planes) {
  __shared__ double tile[32][33];
  int r0 = blockIdx.x * 32, k0 = blockIdx.y * 32, bb = blockIdx.z;
  int tx = threadIdx.x, ty = threadIdx.y;  // 32 x 8
  for (int i = ty; i < 32; i += 8) {
    int k = k0 + i, r = r0 + tx;
    tile[i][tx] = (k < K && r < rows) ? x[bb * sb + (long long)r * sr + (long long)k * sk] : 0.0;
  }
  __syncthreads();
  long long plane = (long long)nb * rows * Kp;
  for (int i = ty; i < 32; i += 8) {
    int r = r0 + i, k = k0 + tx;
    if (r >= rows || k >= Kp) continue;
    double v = tile[tx][i];
    long long o = ((long long)bb * rows + r) * Kp + k;
    for (int s = 0; s < S; ++s) {
      __nv_bfloat16 h = __double2bfloat16(v);
      planes[s * plane + o] = h;
      v -= (double)__bfloat162float(h);
    }
  }
}

// ----------------------------------------------------------------- host side
typedef CUresult (*EncodeTiledFn)(CUtensorMap *, CUtensorMapDataType, cuuint32_t, void *,
                                  const cuuint64_t *, const cuuint64_t *, const cuuint32_t *,
                                  const cuuint32_t *, CUtensorMapInterleave, CUtensorMapSwizzle,
                                  CUtensorMapL2promotion, CUtensorMapFloatOOBfill);

EncodeTiledFn encode_fn() {
  static EncodeTiledFn fn = nullptr;
  static std::once_flag once;
  std::call_once(once, [] {
    void *p = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault,
                                         &q) == cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      fn = (EncodeTiledFn)p;
  });
  return fn;
}

// Operand planes [S][nb][rows][Kp] bf16 and their 4-D tensor map.
struct Operand {
  gc::DevBuf<__nv_bfloat16> buf;
  CUtensorMap map;
  int rows = 0, Kp = 0, nb = 1, S = 0;
};

int make_operand(gc_context *ctx, Operand &op, const double *x, int rows, int K, int nb,
                 long long sr, long long sk, long long sb, int S, int box_rows) {
  op.rows = rows;
  op.Kp = (K + BK - 1) / BK * BK;
  op.nb = nb;
  op.S = S;
  size_t plane = (size_t)nb * rows * op.Kp;
  GC_TRY(op.buf.alloc(ctx, plane * S));
  if (sk == 1) {
    unsigned grid = std::min<unsigned>(gc::ceil_div(plane, 256), 152u * 32u);
    k_pack_planes<<<grid, 256, 0, ctx->stream>>>(x, rows, K, op.Kp, nb, sr, sk, sb, S, op.buf.p);
  } else {
    dim3 grid(gc::ceil_div(rows, 32), gc::ceil_div(op.Kp, 32), nb);
    k_pack_planes_t<<<grid, dim3(32, 8), 0, ctx->stream>>>(x, rows, K, op.Kp, nb, sr, sk, sb, S,
                                                           op.buf.p);
  }
  GC_LAUNCHED(ctx);
  EncodeTiledFn enc = encode_fn();
  if (!enc) return gc::set_error(ctx, GC_ECUDA, "cuTensorMapEncodeTiled entry point unavailable");
  cuuint64_t dims[4] = {(cuuint64_t)op.Kp, (cuuint64_t)rows, (cuuint64_t)nb, (cuuint64_t)S};
  cuuint64_t strides[3] = {(cuuint64_t)op.Kp * 2, (cuuint64_t)rows * op.Kp * 2,
                           (cuuint64_t)nb * rows * op.Kp * 2};
  cuuint32_t box[4] = {(cuuint32_t)BK, (cuuint32_t)box_rows, 1, 1};
  cuuint32_t estr[4] = {1, 1, 1, 1};
  CUresult r = enc(&op.map, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 4, op.buf.p, dims, strides, box, estr,
                   CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_128B,
                   CU_TENSOR_MAP_L2_PROMOTION_L2_256B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
  if (r != CUDA_SUCCESS) return gc::set_error(ctx, GC_ECUDA, "cuTensorMapEncodeTiled failed (%d)", (int)r);
  return GC_OK;
}

PassList pass_list(int precision, int *S) {
  PassList p{};
  if (precision == GC_PREC_BF16X3) {
    *S = 2;
    p.n = 3;
    int a[3] = {1, 0, 0}, b[3] = {0, 1, 0};
    for (int i = 0; i < 3; ++i) p.pa[i] = a[i], p.pb[i] = b[i];
  } else {  // six passes over three planes: every product x_i y_j with i + j <= 2
    *S = 3;
    p.n = 6;
    int a[6] = {2, 1, 0, 1, 0, 0}, b[6] = {0, 1, 2, 0, 1, 0};
    for (int i = 0; i < 6; ++i) p.pa[i] = a[i], p.pb[i] = b[i];
  }
  return p;
}

constexpr int BN_T = 128;

size_t smem_bytes(int bn) {
  return 1024 + STAGES * (size_t)(BM * BK * 2 + bn * BK * 2) + (2 * STAGES + 1) * 8 + 16;
}

// C = A . B^T over prepared operands; A may be shared across the batch.
int run_gemm(gc_context *ctx, const Operand &A, const Operand &B, int M, int N, int nbatch,
             const PassList &pl, const Epi &epi) {
  if (A.Kp != B.Kp) return gc::set_error(ctx, GC_EINVAL, "tc_gemm: K mismatch");
  static std::once_flag once;
  static cudaError_t cfg = cudaSuccess;
  std::call_once(once, [] {
    cfg = cudaFuncSetAttribute(k_tc_gemm<BN_T>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                               (int)smem_bytes(BN_T));
  });
  GC_CUDA(ctx, cfg);
  dim3 grid(gc::ceil_div(M, BM), gc::ceil_div(N, BN_T), nbatch);
  k_tc_gemm<BN_T><<<grid, 192, smem_bytes(BN_T), ctx->stream>>>(
      A.map, B.map, M, N, A.Kp / BK, A.nb > 1 ? 1 : 0, B.nb > 1 ? 1 : 0, pl, epi, ctx->dev_flag);
  GC_LAUNCHED(ctx);
  return GC_OK;
}

int check_flag(gc_context *ctx) {
  int flag = 0;
  GC_CUDA(ctx, cudaMemcpyAsync(&flag, ctx->dev_flag, sizeof(int), cudaMemcpyDeviceToHost, ctx->stream));
  GC_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
  if (flag) {
    cudaMemsetAsync(ctx->dev_flag, 0, sizeof(int), ctx->stream);
    return gc::set_error(ctx, GC_ETIMEOUT, "tc_gemm: a bounded mbarrier wait expired");
  }
  return GC_OK;
}

}  // namespace

namespace gc {

int tc_two_sided(gc_context *ctx, int precision, int n, int cnt, const double *M, int nX,
                 const double *CX, int nY, const double *CY, double *T1, double *out,
                 long long ostride) {
  if (precision == GC_PREC_FP64)
    return fp64_two_sided(ctx, n, cnt, M, nX, CX, nY, CY, T1, out, ostride);
  int S;
  PassList pl = pass_list(precision, &S);
  // step 1: T1[(k,q), x] = sum_p M_k[p, q] CX[p, x]   (T1 column-major, ld = n*cnt)
  {
    Operand A, B;
    GC_TRY(make_operand(ctx, A, M, n * cnt, n, 1, n, 1, 0, S, BM));
    GC_TRY(make_operand(ctx, B, CX, nX, n, 1, n, 1, 0, S, BN_T));
    Epi e{0, T1, (long long)n * cnt, 0, nullptr, nullptr};
    GC_TRY(run_gemm(ctx, A, B, n * cnt, nX, 1, pl, e));
  }
  // step 2: out_k[x, y] = sum_q T1[(k,q), x] CY[q, y]   (batched over k)
  {
    Operand A, B;
    // A rows x, K = q: T1[(k*n + q) + x*(n*cnt)]
    GC_TRY(make_operand(ctx, A, T1, nX, n, cnt, (long long)n * cnt, 1, n, S, BM));
    GC_TRY(make_operand(ctx, B, CY, nY, n, 1, n, 1, 0, S, BN_T));
    Epi e{0, out, nX, ostride, nullptr, nullptr};
    GC_TRY(run_gemm(ctx, A, B, nX, nY, cnt, pl, e));
  }
  return check_flag(ctx);
}

int tc_gemm_nt(gc_context *ctx, int precision, int m, int n, int k, const double *A, int lda,
               const double *B, int ldb, double *C, int ldc) {
  if (precision == GC_PREC_FP64) {
    const double one = 1.0, zero = 0.0;
    GC_CUBLAS(ctx, cublasDgemm(ctx->cublas, CUBLAS_OP_N, CUBLAS_OP_T, m, n, k, &one, A, lda, B, ldb,
                               &zero, C, ldc));
    return GC_OK;
  }
  int S;
  PassList pl = pass_list(precision, &S);
  Operand a, b;
  // A (m x k) column-major: row i, k stride lda
  GC_TRY(make_operand(ctx, a, A, m, k, 1, 1, lda, 0, S, BM));
  GC_TRY(make_operand(ctx, b, B, n, k, 1, 1, ldb, 0, S, BN_T));
  Epi e{0, C, ldc, 0, nullptr, nullptr};
  GC_TRY(run_gemm(ctx, a, b, m, n, 1, pl, e));
  return check_flag(ctx);
}

int tc_dot_gemm(gc_context *ctx, int precision, int N, const double *Ksym, const double *Y,
                double *result) {
  int S;
  PassList pl = pass_list(precision, &S);
  Operand a, b;
  // rows i of the symmetric Kt (= its columns), rows nu of Y^T (= columns of Y)
  GC_TRY(make_operand(ctx, a, Ksym, N, N, 1, N, 1, 0, S, BM));
  GC_TRY(make_operand(ctx, b, Y, N, N, 1, N, 1, 0, S, BN_T));
  size_t ncta = (size_t)ceil_div(N, BM) * ceil_div(N, BN_T);
  DevBuf<double> part;
  GC_TRY(part.alloc(ctx, ncta));
  Epi e{1, nullptr, N, 0, Y, part.p};
  GC_TRY(run_gemm(ctx, a, b, N, N, 1, pl, e));
  std::vector<double> h(ncta);
  GC_CUDA(ctx, cudaMemcpyAsync(h.data(), part.p, ncta * sizeof(double), cudaMemcpyDeviceToHost,
                               ctx->stream));
  GC_TRY(check_flag(ctx));
  double s = 0.0;
  for (double v : h) s += v;
  *result = s;
  return GC_OK;
}

}  // namespace gc

extern "C" int gc_tc_gemm_nt(gc_context *ctx, int precision, int m, int n, int k, const double *A,
                             int lda, const double *B, int ldb, double *C, int ldc) {
  if (!ctx) return GC_EINVAL;
  if (m <= 0 || n <= 0 || k <= 0 || lda < m || ldb < n || ldc < m || !A || !B || !C)
    return gc::set_error(ctx, GC_EINVAL, "tc_gemm_nt: bad arguments");
  return gc::tc_gemm_nt(ctx, precision, m, n, k, A, lda, B, ldb, C, ldc);
}

extern "C" int gc_tc_gemm_time(gc_context *ctx, int precision, int m, int n, int k, int reps,
                               double *ms_per_launch) {
  if (!ctx) return GC_EINVAL;
  if (m <= 0 || n <= 0 || k <= 0 || reps <= 0 || !ms_per_launch ||
      (precision != GC_PREC_BF16X3 && precision != GC_PREC_BF16X6))
    return gc::set_error(ctx, GC_EINVAL, "tc_gemm_time: bad arguments");
  int S;
  PassList pl = pass_list(precision, &S);
  gc::DevBuf<double> a, b, c;
  GC_TRY(a.alloc(ctx, (size_t)m * k));
  GC_TRY(b.alloc(ctx, (size_t)n * k));
  GC_TRY(c.alloc(ctx, (size_t)m * n));
  GC_CUDA(ctx, cudaMemsetAsync(a.p, 0, (size_t)m * k * 8, ctx->stream));
  GC_CUDA(ctx, cudaMemsetAsync(b.p, 0, (size_t)n * k * 8, ctx->stream));
  Operand A, B;
  GC_TRY(make_operand(ctx, A, a.p, m, k, 1, k, 1, 0, S, BM));
  GC_TRY(make_operand(ctx, B, b.p, n, k, 1, k, 1, 0, S, BN_T));
  Epi e{0, c.p, m, 0, nullptr, nullptr};
  GC_TRY(run_gemm(ctx, A, B, m, n, 1, pl, e));  // warm-up
  cudaEvent_t t0, t1;
  GC_CUDA(ctx, cudaEventCreate(&t0));
  GC_CUDA(ctx, cudaEventCreate(&t1));
  GC_CUDA(ctx, cudaEventRecord(t0, ctx->stream));
  for (int r = 0; r < reps; ++r) GC_TRY(run_gemm(ctx, A, B, m, n, 1, pl, e));
  GC_CUDA(ctx, cudaEventRecord(t1, ctx->stream));
  GC_CUDA(ctx, cudaEventSynchronize(t1));
  float ms = 0.f;
  GC_CUDA(ctx, cudaEventElapsedTime(&ms, t0, t1));
  cudaEventDestroy(t0);
  cudaEventDestroy(t1);
  *ms_per_launch = ms / reps;
  return check_flag(ctx);
}
