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
// Every pipeline wait is bounded by the context's limit (1 s unless a test
// shortens it). On expiry the CTA records an error in a device flag and stops
// issuing work; before it frees TMEM and exits, the producer waits for the TMA
// copies it issued and the MMA thread commits the MMAs it issued and waits for
// them, both under their own fixed 1 s limit.
#include <cuda.h>
#include <cuda_bf16.h>

#include <mutex>

#include "gc_tc_gemm.cuh"

namespace {

constexpr int BM = 128;
constexpr int BK = 64;  // bf16 elements per K slice = one 128-byte swizzle row
constexpr int STAGES = 4;
constexpr int MAXPASS = 8;
constexpr unsigned long long kDrainNs = 1000000000ull;  // limit of the waits of the abort path

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

__device__ __forceinline__ bool mbar_try(uint32_t addr, uint32_t parity) {
  uint32_t ok;
  asm volatile(
      "{\n\t.reg .pred p;\n\t"
      "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
      "selp.u32 %0, 1, 0, p;\n\t}"
      : "=r"(ok)
      : "r"(addr), "r"(parity)
      : "memory");
  return ok != 0;
}

// Bounded parity wait: returns false if the phase did not complete within limit_ns.
// try_wait itself suspends the thread for a while, so the timer is read once per
// unsuccessful attempt (never when the first attempt succeeds).
__device__ __forceinline__ bool mbar_wait(uint64_t *bar, uint32_t parity,
                                          unsigned long long limit_ns) {
  const uint32_t addr = smem_u32(bar);
  if (mbar_try(addr, parity)) return true;
  const unsigned long long t0 = globaltimer();
  for (;;) {
    if (mbar_try(addr, parity)) return true;
    if (globaltimer() - t0 > limit_ns) return false;
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

// As smem_desc for 64-byte rows (32 BF16 of K) in the 64-byte swizzle: 8-row groups
// 512 bytes apart, layout SWIZZLE_64B (bits 61-63 = 4).
__device__ __forceinline__ uint64_t smem_desc64(uint32_t saddr) {
  uint64_t d = 0;
  d |= (uint64_t)((saddr & 0x3FFFF) >> 4);
  d |= (uint64_t)1 << 16;           // LBO (unused for swizzled K-major)
  d |= (uint64_t)(512 >> 4) << 32;  // SBO
  d |= (uint64_t)1 << 46;           // descriptor version
  d |= (uint64_t)4 << 61;           // SWIZZLE_64B
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

// As mma_bf16, with a use of the A collector buffer: C = 1 reads A from shared memory
// and keeps it in the buffer, 2 reads the buffer, 3 reads it and releases it, 0
// discards it (the plain form). The same A descriptor is given with every use.
template <int C>
__device__ __forceinline__ void mma_bf16_ca(uint32_t tmem, uint64_t ad, uint64_t bd,
                                            uint32_t idesc, uint32_t accumulate) {
  if constexpr (C == 1)
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "setp.ne.b32 p, %4, 0;\n\t"
        "tcgen05.mma.cta_group::1.kind::f16.collector::a::fill [%0], %1, %2, %3, p;\n\t}" ::"r"(tmem),
        "l"(ad), "l"(bd), "r"(idesc), "r"(accumulate));
  else if constexpr (C == 2)
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "setp.ne.b32 p, %4, 0;\n\t"
        "tcgen05.mma.cta_group::1.kind::f16.collector::a::use [%0], %1, %2, %3, p;\n\t}" ::"r"(tmem),
        "l"(ad), "l"(bd), "r"(idesc), "r"(accumulate));
  else if constexpr (C == 3)
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "setp.ne.b32 p, %4, 0;\n\t"
        "tcgen05.mma.cta_group::1.kind::f16.collector::a::lastuse [%0], %1, %2, %3, p;\n\t}" ::"r"(tmem),
        "l"(ad), "l"(bd), "r"(idesc), "r"(accumulate));
  else
    mma_bf16(tmem, ad, bd, idesc, accumulate);
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

// 32 lanes x 8 columns of 32-bit TMEM words, issued without waiting (several loads
// can be in flight before one tmem_ld_wait()).
__device__ __forceinline__ void tmem_ld8_issue(uint32_t taddr, uint32_t *r) {
  asm volatile("tcgen05.ld.sync.aligned.32x32b.x8.b32 {%0, %1, %2, %3, %4, %5, %6, %7}, [%8];"
               : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]),
                 "=r"(r[6]), "=r"(r[7])
               : "r"(taddr));
}

__device__ __forceinline__ void tmem_ld_wait() {
  asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
}

// ------------------------------------------------------------------- kernel
template <int BN>
__global__ void __launch_bounds__(192, 1)
    k_tc_gemm(const __grid_constant__ CUtensorMap mapA, const __grid_constant__ CUtensorMap mapB,
              int M, int N, int kblocks, int a_batched, int b_batched, PassList passes, Epi epi,
              int *err_flag, unsigned long long wait_ns) {
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
  volatile int *abort_v = &abort_flag;
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
      if (!mbar_wait(&empty[s], ph ^ 1, wait_ns)) {
        atomicExch(&abort_flag, 1);
        break;
      }
      if (*abort_v) break;
      int pass = it / kblocks, kb = it % kblocks;
      mbar_expect_tx(&full[s], A_BYTES + B_BYTES);
      tma_load_4d(sA + s * A_BYTES, &mapA, &full[s], kb * BK, m0, a_batched ? b : 0,
                  passes.pa[pass]);
      tma_load_4d(sB + s * B_BYTES, &mapB, &full[s], kb * BK, n0, b_batched ? b : 0,
                  passes.pb[pass]);
      issued = it + 1;
    }
    if (*abort_v) {
      // Drain the copies already issued into the ring before the CTA exits. Loads older
      // than the last STAGES were consumed by the MMA thread (their slot was released
      // before it was reused), so only the last STAGES can still be in flight.
      for (int it = (issued > STAGES ? issued - STAGES : 0); it < issued; ++it)
        mbar_wait(&full[it % STAGES], (it / STAGES) & 1, kDrainNs);
    }
  } else if (warp == 1 && lane == 0) {
    // ---------------- MMA issuer
    constexpr uint32_t idesc = instr_desc(BN);
    bool ok = true;
    for (int it = 0; it < total && ok; ++it) {
      int s = it % STAGES;
      uint32_t ph = (it / STAGES) & 1;
      if (!mbar_wait(&full[s], ph, wait_ns) || *abort_v) {
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
    // TMEM is freed after the final barrier: wait here for every MMA this thread
    // issued, whatever the epilogue saw (on the abort path it may have given up).
    if (!mbar_wait(accf, 0, kDrainNs)) atomicExch(&abort_flag, 1);
  } else if (warp >= 2) {
    // ---------------- epilogue
    const int q = warp & 3;  // TMEM lane quarter this warp may access
    const int m = m0 + q * 32 + lane;
    bool ok = mbar_wait(accf, 0, wait_ns);
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    double acc = 0.0;
    if (ok && !*abort_v) {
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

// ------------------------------------------------ FP64-accurate (sliced) GEMM
// Each row r of A is scaled by 2^-e_r (e_r: exponent of its largest entry) and
// cut into S integer slices a = sum_t alpha_t 2^-7(t+1), |alpha_0| <= 128,
// |alpha_t>0| <= 64, every alpha exact in BF16; likewise the rows of B with f_c.
// C[r,c] = 2^(e_r+f_c) sum_{t+u<S} 2^-7(t+u+2) sum_k alpha_t[r,k] beta_u[c,k].
// The products of one weight d = t+u share a TMEM accumulator; K is cut into
// chunks short enough that every FP32 partial sum is an integer below 2^24, so
// each chunk is exact, and the epilogue adds the chunks in FP64 registers.
// Column tile (TBN rows of B): the S weight accumulators take S * TBN of the 512 TMEM
// columns, so TBN = 128 for S = 4, 96 for S = 5 and 64 for S = 6 at most. A wider
// tile reads fewer operand bytes per product (shared memory and L2); a narrower
// one gives more CTAs to a small product. oz_tile() picks one per GEMM; every
// width gives the same result bits (each element's integer sums are the same).
constexpr int OZ_BK = 32;      // K per stage: 32 BF16 = one 64-byte swizzled row
constexpr int OZ_STAGES = 3;   // each stage holds every slice of A and of B
constexpr int OZ_MAXS = 6;
// Row exponent of a row holding a NaN or an infinity: its slices are zero and
// every product element of the row comes out NaN, so non-finite inputs stay
// visible in the result (the integer slices cannot carry them).
constexpr int kBadExp = 0x7fffffff;

constexpr int OZ_GROUP_M = 8;  // row tiles per raster group
// Epilogue: four warps (one per TMEM lane quarter) per 32 columns of the tile.
__host__ __device__ constexpr int oz_epi_warps(int tbn) { return 4 * (tbn / 32); }
__host__ __device__ constexpr int oz_threads(int tbn) {  // TMA warp, MMA warp, epilogue
  return 64 + 32 * oz_epi_warps(tbn);
}
__host__ __device__ constexpr int oz_max_tile(int S) { return S <= 4 ? 128 : (S == 5 ? 96 : 64); }

struct OzPlan {
  int S;          // slices per operand
  int npass;      // S(S+1)/2
  int chunk_kb;   // OZ_BK-wide K blocks per exact chunk
  int pa[OZ_MAXS * (OZ_MAXS + 1) / 2], pb[OZ_MAXS * (OZ_MAXS + 1) / 2],
      pd[OZ_MAXS * (OZ_MAXS + 1) / 2];
};

struct OzEpi {
  int mode;              // 0 store, 1 dot with r, 2 subtract from the lower triangle of c
  double *c;
  long long ldn, sb;
  const double *r;
  double *partial;
  const int *ea;         // row exponents of A, [batch][rows] (batch stride 0 if shared)
  const int *eb;         // row exponents of B
  long long ea_sb, eb_sb;
  int tri_period;        // > 0: skip tiles wholly above the diagonal of each
                         // tri_period-wide column block (C lower-triangular per block)
};

template <int S, int TBN>
__global__ void __launch_bounds__(oz_threads(TBN), 1)
    k_tc_gemm_oz(const __grid_constant__ CUtensorMap mapA, const __grid_constant__ CUtensorMap mapB,
                 int M, int N, int kblocks, int a_batched, int b_batched, OzPlan plan, OzEpi epi,
                 int *err_flag, unsigned long long wait_ns) {
  // One stage = the K block [kb*32, kb*32+32) of all S slices of the A tile (128 rows)
  // and of the B tile (TBN rows): every slice product t+u < S of the block is
  // issued from it, so each slice tile crosses L2 -> shared memory once per block.
  static_assert(S * TBN <= 512 && TBN % 32 == 0, "S weight accumulators exceed TMEM");
  constexpr int EPI = oz_epi_warps(TBN);
  extern __shared__ __align__(1024) uint8_t smem_raw[];
  uint8_t *smem = (uint8_t *)(((uintptr_t)smem_raw + 1023) & ~(uintptr_t)1023);
  constexpr uint32_t A_BYTES = BM * OZ_BK * 2, B_BYTES = TBN * OZ_BK * 2;
  constexpr uint32_t STAGE_BYTES = S * (A_BYTES + B_BYTES);
  uint64_t *full = (uint64_t *)(smem + OZ_STAGES * STAGE_BYTES);
  uint64_t *empty = full + OZ_STAGES;
  uint64_t *accf = empty + OZ_STAGES;
  uint64_t *acce = accf + 1;
  uint64_t *drainb = acce + 1;  // abort path: completion of the MMAs already issued
  uint32_t *tmem_slot = (uint32_t *)(drainb + 1);
  __shared__ int abort_flag;
  volatile int *abort_v = &abort_flag;
  __shared__ double red[EPI];

  const int warp = threadIdx.x / 32, lane = threadIdx.x % 32;
  // Grouped raster: CTAs are scheduled roughly in linear order, so consecutive ones
  // take OZ_GROUP_M row tiles before moving to the next column tile. A wave of CTAs
  // then shares a few A and B panels in L2 instead of sweeping every A panel
  // (which does not fit in L2 at large M) once per column tile.
  int mt, nt;
  {
    const int ntm = gridDim.x, ntn = gridDim.y;
    const long long t = blockIdx.x + (long long)ntm * blockIdx.y;
    const long long per_group = (long long)OZ_GROUP_M * ntn;
    const int first_m = (int)(t / per_group) * OZ_GROUP_M;
    const int gm = min(ntm - first_m, OZ_GROUP_M);
    const int r = (int)(t % per_group);
    mt = first_m + r % gm;
    nt = r / gm;
  }
  const int m0 = mt * BM, n0 = nt * TBN, b = blockIdx.z;
  const int nchunks = (kblocks + plan.chunk_kb - 1) / plan.chunk_kb;
  if (epi.tri_period > 0) {  // whole CTA, before any barrier or TMEM is set up
    const int c0 = n0 % epi.tri_period;
    if (c0 + TBN <= epi.tri_period && c0 >= m0 + BM) return;
  }

  if (threadIdx.x == 0) {
    for (int s = 0; s < OZ_STAGES; ++s) {
      mbar_init(&full[s], 1);
      mbar_init(&empty[s], 1);
    }
    mbar_init(accf, 1);
    mbar_init(acce, EPI);
    mbar_init(drainb, 1);
    abort_flag = 0;
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  if (warp == 1) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(
                     smem_u32(tmem_slot)),
                 "r"(512u));
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
  }
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
  const uint32_t tmem = *tmem_slot;

  if (warp == 0 && lane == 0) {
    int issued = 0;
    for (int kb = 0; kb < kblocks && !*abort_v; ++kb) {
      const int s = kb % OZ_STAGES;
      if (!mbar_wait(&empty[s], ((kb / OZ_STAGES) & 1) ^ 1, wait_ns)) {
        atomicExch(&abort_flag, 1);
        break;
      }
      mbar_expect_tx(&full[s], STAGE_BYTES);
      uint8_t *st = smem + s * STAGE_BYTES;
#pragma unroll
      for (int t = 0; t < S; ++t)
        tma_load_4d(st + t * A_BYTES, &mapA, &full[s], kb * OZ_BK, m0, a_batched ? b : 0, t);
#pragma unroll
      for (int u = 0; u < S; ++u)
        tma_load_4d(st + S * A_BYTES + u * B_BYTES, &mapB, &full[s], kb * OZ_BK, n0,
                    b_batched ? b : 0, u);
      issued = kb + 1;
    }
    if (*abort_v)  // only the last OZ_STAGES loads can still be in flight
      for (int j = (issued > OZ_STAGES ? issued - OZ_STAGES : 0); j < issued; ++j)
        mbar_wait(&full[j % OZ_STAGES], (j / OZ_STAGES) & 1, kDrainNs);
  } else if (warp == 1 && lane == 0) {
    constexpr uint32_t idesc = instr_desc(TBN);
    bool ok = true;
    for (int g = 0; g < nchunks && ok; ++g) {
      if (g > 0 && !mbar_wait(acce, (g - 1) & 1, wait_ns)) {
        ok = false;
        break;
      }
      asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
      const int kb0 = g * plan.chunk_kb, kb1 = min(kblocks, kb0 + plan.chunk_kb);
      for (int kb = kb0; kb < kb1; ++kb) {
        const int s = kb % OZ_STAGES;
        if (!mbar_wait(&full[s], (kb / OZ_STAGES) & 1, wait_ns) || *abort_v) {
          ok = false;
          break;
        }
        asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
        const uint32_t a_base = smem_u32(smem + s * STAGE_BYTES);
        const uint32_t b_base = a_base + S * A_BYTES;
        // A slice t at K step kk meets the B slices u < S - t back to back, so it is
        // read from shared memory once and then from the collector buffer. The first
        // product into weight t+u in the chunk is (0, t+u) at kb0, kk 0.
#pragma unroll
        for (int t = 0; t < S; ++t)
#pragma unroll
          for (int kk = 0; kk < OZ_BK / 16; ++kk) {
            const uint64_t ad = smem_desc64(a_base + t * A_BYTES + kk * 32);
            const uint32_t acc_in = (kb == kb0 && t == 0 && kk == 0) ? 0u : 1u;
            if (t == S - 1) {
              mma_bf16_ca<0>(tmem + (uint32_t)(t * TBN), ad, smem_desc64(b_base + kk * 32), idesc,
                             acc_in);
              continue;
            }
            mma_bf16_ca<1>(tmem + (uint32_t)(t * TBN), ad, smem_desc64(b_base + kk * 32), idesc,
                           acc_in);
#pragma unroll
            for (int u = 1; u + t < S - 1; ++u)
              mma_bf16_ca<2>(tmem + (uint32_t)((t + u) * TBN), ad,
                             smem_desc64(b_base + u * B_BYTES + kk * 32), idesc, acc_in);
            mma_bf16_ca<3>(tmem + (uint32_t)((S - 1) * TBN), ad,
                           smem_desc64(b_base + (S - 1 - t) * B_BYTES + kk * 32), idesc, acc_in);
          }
        mma_commit(&empty[s]);
      }
      mma_commit(accf);
    }
    if (!ok) atomicExch(&abort_flag, 1);
    // TMEM is freed after the final barrier, and the epilogue may have given up on the
    // last chunk: commit every MMA issued so far (a chunk may be half issued) to a
    // barrier of its own and wait until they have completed.
    mma_commit(drainb);
    if (!mbar_wait(drainb, 0, kDrainNs)) atomicExch(&abort_flag, 1);
  } else if (warp >= 2) {
    // Every chunk's FP32 sums are integers below 2^24, so the weights fold into one
    // int64 per column by Horner in base 2^7: t = sum_d v_d 2^(7 (SI - 1 - d)) is exact
    // for the first SI = min(S, 5) weights (|t| < 2^52 per chunk); a sixth weight is
    // rounded to units of 2^7 first (2^-42 of the scaled product, below FP64 rounding
    // of the result). The int64 sum over chunks is converted to FP64 once, at the end:
    // the per-chunk work is integer, not FP64, arithmetic.
    // Four warps per 32 columns (one per TMEM lane quarter, q = warp % 4); warp group
    // h = (warp - 2) / 4 owns columns [32 h, 32 h + 32) of the tile.
    constexpr int SI = S < 5 ? S : 5;
    constexpr int NC = 32;
    const int q = warp & 3;
    const int h = (warp - 2) / 4;
    const int m = m0 + q * 32 + lane;
    long long acc[NC];
#pragma unroll
    for (int j = 0; j < NC; ++j) acc[j] = 0;
    bool ok = true;
    for (int g = 0; g < nchunks && ok; ++g) {
      if (!mbar_wait(accf, g & 1, wait_ns) || *abort_v) {
        ok = false;
        break;
      }
      asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
#pragma unroll
      for (int c0 = 0; c0 < NC; c0 += 8) {
        uint32_t r[S][8];
#pragma unroll
        for (int d = 0; d < S; ++d)
          tmem_ld8_issue(tmem + ((uint32_t)(q * 32) << 16) + (uint32_t)(d * TBN + h * NC + c0),
                         r[d]);
        tmem_ld_wait();
#pragma unroll
        for (int j = 0; j < 8; ++j) {
          long long t = 0;
#pragma unroll
          for (int d = 0; d < SI; ++d) t = t * 128 + (long long)__float2int_rn(__uint_as_float(r[d][j]));
#pragma unroll
          for (int d = SI; d < S; ++d)
            t += (long long)__float2int_rn(__uint_as_float(r[d][j]) * exp2f(-7.0f * (d - SI + 1)));
          acc[c0 + j] += t;
        }
      }
      asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
      __syncwarp();
      if (lane == 0) asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(smem_u32(acce)) : "memory");
    }
    if (!ok) atomicExch(&abort_flag, 1);
    double dot = 0.0;
    if (ok && m < M) {
      const int ea = epi.ea[(long long)b * epi.ea_sb + m];
      const int er = ea - 7 * (SI + 1);
#pragma unroll
      for (int j = 0; j < NC; ++j) {
        int n = n0 + h * NC + j;
        if (n < N) {
          const int eb = epi.eb[(long long)b * epi.eb_sb + n];
          double cv = (ea == kBadExp || eb == kBadExp) ? __longlong_as_double(0x7ff8000000000000ll)
                                                       : ldexp((double)acc[j], er + eb);
          long long o = (long long)b * epi.sb + m + (long long)n * epi.ldn;
          if (epi.mode == 0)
            epi.c[o] = cv;
          else if (epi.mode == 2) {
            if (m >= n) epi.c[o] -= cv;
          } else
            dot += cv * epi.r[o];
        }
      }
    }
    if (epi.mode == 1) {
      for (int off = 16; off > 0; off >>= 1) dot += __shfl_down_sync(0xffffffffu, dot, off);
      if (lane == 0) red[warp - 2] = dot;
    }
  }
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  if (epi.mode == 1 && threadIdx.x == 0) {
    long long cta = blockIdx.x + (long long)gridDim.x * (blockIdx.y + (long long)gridDim.y * blockIdx.z);
    double sum = 0.0;
    for (int w = 0; w < EPI; ++w) sum += red[w];
    epi.partial[cta] = sum;
  }
  if (threadIdx.x == 0 && abort_flag) atomicExch(err_flag, 1);
  if (warp == 1) {
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(512u));
  }
}

// |x| as its bit pattern without the sign: for finite values the unsigned integer order is
// the order of |x|, and a value with the exponent field all ones is an infinity or a NaN.
__device__ __forceinline__ unsigned long long abs_bits(double v) {
  return (unsigned long long)__double_as_longlong(v) & 0x7fffffffffffffffull;
}
// 1 + ilogb of the value whose |x| bits are m (m > 0, finite), from the bits.
__device__ __forceinline__ int exp_of_bits(unsigned long long m) {
  const int E = (int)(m >> 52);
  return E > 0 ? E - 1022 : -1010 - __clzll((long long)m);
}
constexpr unsigned long long kInfBits = 0x7ff0000000000000ull;

// Row exponents: e[b][r] = 1 + ilogb(max_k |x[b,r,k]|) (0 for a zero row, kBadExp for a
// row with a non-finite element), with integer operations on the bit patterns (no FP64
// pipe): one warp per row (rows whose K elements are contiguous, sk = 1) ...
__global__ void k_row_exponent(const double *__restrict__ x, int rows, int K, int nb, long long sr,
                               long long sk, long long sb, int *__restrict__ e) {
  long long total = (long long)nb * rows;
  long long wid = (blockIdx.x * (long long)blockDim.x + threadIdx.x) / 32;
  int lane = threadIdx.x % 32;
  for (long long t = wid; t < total; t += (long long)gridDim.x * blockDim.x / 32) {
    int r = (int)(t % rows);
    long long bb = t / rows;
    const double *row = x + bb * sb + (long long)r * sr;
    unsigned long long mx = 0;
    for (int k = lane; k < K; k += 32) mx = max(mx, abs_bits(row[(long long)k * sk]));
    for (int off = 16; off > 0; off >>= 1) mx = max(mx, __shfl_down_sync(0xffffffffu, mx, off));
    if (lane == 0) e[t] = mx >= kInfBits ? kBadExp : (mx ? exp_of_bits(mx) : 0);
  }
}

// ... or, for consecutive rows contiguous (sr = 1), 32 rows per block with the lanes along
// the rows (loads coalesced for every k) and 8 warps splitting K.
__global__ void k_row_exponent_cols(const double *__restrict__ x, int rows, int K,
                                    long long sk, long long sb, int *__restrict__ e) {
  __shared__ unsigned long long part[8][32];
  const int tx = threadIdx.x, ty = threadIdx.y;
  const int r = blockIdx.x * 32 + tx;
  const long long bb = blockIdx.y;
  unsigned long long mx = 0;
  if (r < rows) {
    const double *row = x + bb * sb + r;
    for (int k = ty; k < K; k += 8) mx = max(mx, abs_bits(row[(long long)k * sk]));
  }
  part[ty][tx] = mx;
  __syncthreads();
  if (ty == 0 && r < rows) {
    for (int w = 1; w < 8; ++w) mx = max(mx, part[w][tx]);
    e[bb * rows + r] = mx >= kInfBits ? kBadExp : (mx ? exp_of_bits(mx) : 0);
  }
}

// x 2^sh rounded to the nearest integer (ties to even), for |x 2^sh| < 2^62, from the bit
// pattern of x with integer operations only: the same value as __double2ll_rn(ldexp(x, sh))
// (the scaling is exact unless the result is below 0.5, which rounds to 0 either way),
// without the FP64 pipe, which is narrow on GB300.
__device__ __forceinline__ long long scaled_round(double x, int sh) {
  const unsigned long long b = (unsigned long long)__double_as_longlong(x);
  const int E = (int)((b >> 52) & 0x7ff);
  unsigned long long m = b & 0xfffffffffffffull;
  int q = -1074;  // x = +-m 2^q
  if (E != 0) {
    m |= 1ull << 52;
    q = E - 1075;
  }
  q += sh;
  unsigned long long n;
  if (m == 0 || q < -63) {
    n = 0;  // |x 2^sh| < 2^53 2^-64 < 1/2
  } else if (q >= 0) {
    n = m << q;
  } else {
    const int sft = -q;  // 1..63
    const unsigned long long whole = m >> sft, rem = m & ((1ull << sft) - 1),
                             half = 1ull << (sft - 1);
    n = whole + ((rem > half || (rem == half && (whole & 1))) ? 1 : 0);
  }
  return (b >> 63) ? -(long long)n : (long long)n;
}

// Balanced base-128 digits of n = rint(x 2^(7S - e)) (|n| < 2^(7S) since |x| < 2^e):
// n = sum_s a_s 128^(S-1-s), |a_0| <= 128, |a_s| <= 64 otherwise; plane s gets a_s. All
// in integer arithmetic.
__device__ __forceinline__ void store_digits(double x, int e, int S, long long plane, long long o,
                                             __nv_bfloat16 *__restrict__ planes) {
  long long n = e == kBadExp ? 0 : scaled_round(x, 7 * S - e);
  for (int s = S - 1; s > 0; --s) {
    const long long d = ((n + 64) & 127) - 64;
    planes[s * plane + o] = __float2bfloat16_rn((float)d);
    n = (n - d) >> 7;
  }
  planes[o] = __float2bfloat16_rn((float)n);
}

// Integer slices: planes[t][b][r][kp] = alpha_t of x[b,r,k] 2^-e[b][r].
// Rows (b, r) over blockIdx.y, K over the threads: no 64-bit division per element.
__global__ void k_slice_planes(const double *__restrict__ x, int rows, int K, int Kp, int nb,
                               long long sr, long long sk, long long sb, int S,
                               const int *__restrict__ e, __nv_bfloat16 *__restrict__ planes) {
  const long long plane = (long long)nb * rows * Kp, nrr = (long long)nb * rows;
  for (long long rr = blockIdx.y; rr < nrr; rr += gridDim.y) {
    const long long bb = rr / rows;
    const int r = (int)(rr - bb * rows);
    const int ex = e[rr];
    const double *__restrict__ xr = x + bb * sb + (long long)r * sr;
    for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < Kp; k += gridDim.x * blockDim.x) {
      const double xv = k < K ? xr[(long long)k * sk] : 0.0;
      store_digits(xv, ex, S, plane, rr * Kp + k, planes);
    }
  }
}

// Transposed-read variant (K is the slow index of x).
__global__ void k_slice_planes_t(const double *__restrict__ x, int rows, int K, int Kp, int nb,
                                 long long sr, long long sk, long long sb, int S,
                                 const int *__restrict__ e, __nv_bfloat16 *__restrict__ planes) {
  __shared__ double tile[32][33];
  int r0 = blockIdx.x * 32, k0 = blockIdx.y * 32, bb = blockIdx.z;
  int tx = threadIdx.x, ty = threadIdx.y;
  for (int i = ty; i < 32; i += 8) {
    int k = k0 + i, r = r0 + tx;
    tile[i][tx] = (k < K && r < rows) ? x[bb * sb + (long long)r * sr + (long long)k * sk] : 0.0;
  }
  __syncthreads();
  long long plane = (long long)nb * rows * Kp;
  for (int i = ty; i < 32; i += 8) {
    int r = r0 + i, k = k0 + tx;
    if (r >= rows || k >= Kp) continue;
    const long long o = ((long long)bb * rows + r) * Kp + k;
    store_digits(tile[tx][i], e[(long long)bb * rows + r], S, plane, o, planes);
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
      A.map, B.map, M, N, A.Kp / BK, A.nb > 1 ? 1 : 0, B.nb > 1 ? 1 : 0, pl, epi, ctx->dev_flag,
      ctx->wait_ns);
  GC_LAUNCHED(ctx);
  return GC_OK;
}



// ---- sliced (FP64-accurate) operands and launch
struct OzOperand {
  gc::DevBuf<__nv_bfloat16> buf;
  gc::DevBuf<int> exps;
  CUtensorMap map;
  int rows = 0, Kp = 0, nb = 1, S = 0, box_rows = 0;
  const __nv_bfloat16 *planes = nullptr;  // buf.p, or another operand's planes (alias)
  const int *ex = nullptr;                // exps.p, or another operand's exponents
};

bool is_oz(int precision) { return gc::is_sliced(precision); }

OzPlan oz_plan(int precision) {
  OzPlan p{};
  p.S = precision == GC_PREC_FP64TC6 ? 6 : (precision == GC_PREC_FP64TC4 ? 4 : 5);
  int n = 0;
  for (int d = 0; d < p.S; ++d)
    for (int t = 0; t <= d; ++t) {
      p.pa[n] = t;
      p.pb[n] = d - t;
      p.pd[n] = d;
      ++n;
    }
  p.npass = n;
  // exact FP32 partial sums: (S+2) 2^12 c < 2^24 and 2^14 c < 2^24
  int c = (4096 / (p.S + 2)) / OZ_BK * OZ_BK;
  if ((long long)(p.S + 2) * 4096 * c >= (1ll << 24)) c -= OZ_BK;
  p.chunk_kb = c / OZ_BK;
  return p;
}

// The 4-D TMA map [S][nb][rows][Kp] of an operand's slice planes, box OZ_BK x box_rows.
int encode_oz_map(gc_context *ctx, OzOperand &op) {
  EncodeTiledFn enc = encode_fn();
  if (!enc) return gc::set_error(ctx, GC_ECUDA, "cuTensorMapEncodeTiled entry point unavailable");
  cuuint64_t dims[4] = {(cuuint64_t)op.Kp, (cuuint64_t)op.rows, (cuuint64_t)op.nb,
                        (cuuint64_t)op.S};
  cuuint64_t strides[3] = {(cuuint64_t)op.Kp * 2, (cuuint64_t)op.rows * op.Kp * 2,
                           (cuuint64_t)op.nb * op.rows * op.Kp * 2};
  cuuint32_t box[4] = {(cuuint32_t)OZ_BK, (cuuint32_t)op.box_rows, 1, 1};
  cuuint32_t estr[4] = {1, 1, 1, 1};
  CUresult r = enc(&op.map, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 4, (void *)op.planes, dims, strides,
                   box, estr, CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_64B,
                   CU_TENSOR_MAP_L2_PROMOTION_L2_256B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
  if (r != CUDA_SUCCESS) return gc::set_error(ctx, GC_ECUDA, "cuTensorMapEncodeTiled failed (%d)", (int)r);
  return GC_OK;
}

int make_oz_operand(gc_context *ctx, OzOperand &op, const double *x, int rows, int K, int nb,
                    long long sr, long long sk, long long sb, int S, int box_rows) {
  op.rows = rows;
  op.box_rows = box_rows;
  op.Kp = (K + BK - 1) / BK * BK;
  op.nb = nb;
  op.S = S;
  size_t plane = (size_t)nb * rows * op.Kp;
  GC_TRY(op.exps.alloc(ctx, (size_t)nb * rows));
  GC_TRY(op.buf.alloc(ctx, plane * S));
  if (sr == 1 && sk != 1 && nb <= 65535) {
    k_row_exponent_cols<<<dim3(gc::ceil_div(rows, 32), nb), dim3(32, 8), 0, ctx->stream>>>(
        x, rows, K, sk, sb, op.exps.p);
    GC_LAUNCHED(ctx);
  } else {
    size_t warps = (size_t)nb * rows;
    unsigned grid = std::min<unsigned>(gc::ceil_div(warps * 32, 256), 152u * 64u);
    k_row_exponent<<<grid, 256, 0, ctx->stream>>>(x, rows, K, nb, sr, sk, sb, op.exps.p);
    GC_LAUNCHED(ctx);
  }
  if (sk == 1) {
    const dim3 grid(std::min(gc::ceil_div(op.Kp, 256), 4u),
                    (unsigned)std::min<long long>((long long)nb * rows, 65535));
    k_slice_planes<<<grid, 256, 0, ctx->stream>>>(x, rows, K, op.Kp, nb, sr, sk, sb, S, op.exps.p,
                                                   op.buf.p);
  } else {
    dim3 grid(gc::ceil_div(rows, 32), gc::ceil_div(op.Kp, 32), nb);
    k_slice_planes_t<<<grid, dim3(32, 8), 0, ctx->stream>>>(x, rows, K, op.Kp, nb, sr, sk, sb, S,
                                                             op.exps.p, op.buf.p);
  }
  GC_LAUNCHED(ctx);
  op.planes = op.buf.p;
  op.ex = op.exps.p;
  return encode_oz_map(ctx, op);
}

// A second view of src's slice planes with another TMA box height (src must outlive it).
int alias_oz_operand(gc_context *ctx, const OzOperand &src, OzOperand &op, int box_rows) {
  op.rows = src.rows;
  op.Kp = src.Kp;
  op.nb = src.nb;
  op.S = src.S;
  op.box_rows = box_rows;
  op.planes = src.planes;
  op.ex = src.ex;
  return encode_oz_map(ctx, op);
}

// alignment pad, stages, 2 * stages + 3 barriers, TMEM slot
constexpr size_t oz_smem_bytes(int S, int tbn) {
  return 1024 + OZ_STAGES * (size_t)S * (BM * OZ_BK * 2 + tbn * OZ_BK * 2) +
         (2 * OZ_STAGES + 3) * 8 + 16;
}
static_assert(oz_smem_bytes(4, 128) <= 232448 && oz_smem_bytes(5, 96) <= 232448 &&
                  oz_smem_bytes(6, 64) <= 232448,
              "sliced GEMM stages exceed the 227 KB of shared memory per CTA");

// Relative time per CTA of each tile width (one CTA per SM at a time), measured at
// 6290^3 on GB300 (ms per wave of 152 CTAs: FP64TC5 0.227 at 64 and 0.240 at 96;
// FP64TC4 0.171, 0.183 and 0.201 at 64, 96 and 128). A CTA's time is set by the
// operand bytes it moves, so a wider tile costs little more per CTA.
constexpr double kOzTileCost64 = 1.0, kOzTileCost96 = 1.06, kOzTileCost128 = 1.18;

// Tile width for an M x N x nbatch product: the narrowest width unless a wider one
// finishes its CTA waves (152 SMs, one CTA each) sooner by the costs above.
int oz_tile(const gc_context *ctx, int S, long long M, long long N, long long nbatch) {
  const int widest = oz_max_tile(S);
  if (ctx->oz_tile > 0) return std::min(ctx->oz_tile, widest);
  int best = 64;
  double best_cost = 0.0;
  for (int tbn = 64; tbn <= widest; tbn += 32) {
    const long long ctas = (M + BM - 1) / BM * ((N + tbn - 1) / tbn) * nbatch;
    const double cost = (double)((ctas + 151) / 152) *
                        (tbn == 64 ? kOzTileCost64 : (tbn == 96 ? kOzTileCost96 : kOzTileCost128));
    if (tbn == 64 || cost < best_cost) {
      best = tbn;
      best_cost = cost;
    }
  }
  return best;
}

template <int S, int TBN>
int launch_oz(gc_context *ctx, const OzOperand &A, const OzOperand &B, int M, int N, int nbatch,
              const OzPlan &pl, const OzEpi &epi) {
  static std::once_flag once;
  static cudaError_t cfg = cudaSuccess;
  std::call_once(once, [] {
    cfg = cudaFuncSetAttribute(k_tc_gemm_oz<S, TBN>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                               (int)oz_smem_bytes(S, TBN));
  });
  GC_CUDA(ctx, cfg);
  dim3 grid(gc::ceil_div(M, BM), gc::ceil_div(N, TBN), nbatch);
  k_tc_gemm_oz<S, TBN><<<grid, oz_threads(TBN), oz_smem_bytes(S, TBN), ctx->stream>>>(
      A.map, B.map, M, N, A.Kp / OZ_BK, A.nb > 1 ? 1 : 0, B.nb > 1 ? 1 : 0, pl, epi, ctx->dev_flag,
      ctx->wait_ns);
  GC_LAUNCHED(ctx);
  return GC_OK;
}

// The B operand's TMA box height is the column tile width of the launch.
int run_oz(gc_context *ctx, const OzOperand &A, const OzOperand &B, int M, int N, int nbatch,
           const OzPlan &pl, OzEpi epi) {
  if (A.Kp != B.Kp) return gc::set_error(ctx, GC_EINVAL, "oz_gemm: K mismatch");
  epi.ea = A.ex;
  epi.eb = B.ex;
  epi.ea_sb = A.nb > 1 ? A.rows : 0;
  epi.eb_sb = B.nb > 1 ? B.rows : 0;
  const int w = B.box_rows;
  if (pl.S == 6 && w == 64) return launch_oz<6, 64>(ctx, A, B, M, N, nbatch, pl, epi);
  if (pl.S == 5 && w == 64) return launch_oz<5, 64>(ctx, A, B, M, N, nbatch, pl, epi);
  if (pl.S == 5 && w == 96) return launch_oz<5, 96>(ctx, A, B, M, N, nbatch, pl, epi);
  if (pl.S == 4 && w == 64) return launch_oz<4, 64>(ctx, A, B, M, N, nbatch, pl, epi);
  if (pl.S == 4 && w == 96) return launch_oz<4, 96>(ctx, A, B, M, N, nbatch, pl, epi);
  if (pl.S == 4 && w == 128) return launch_oz<4, 128>(ctx, A, B, M, N, nbatch, pl, epi);
  return gc::set_error(ctx, GC_EINVAL, "oz_gemm: no kernel for %d slices and tile %d", pl.S, w);
}

}  // namespace

namespace gc {

int check_flag(gc_context *ctx) {
  int flag = 0;
  GC_CUDA(ctx, cudaMemcpyAsync(&flag, ctx->dev_flag, sizeof(int), cudaMemcpyDeviceToHost, ctx->stream));
  GC_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
  if (flag) {
    GC_CUDA(ctx, cudaMemsetAsync(ctx->dev_flag, 0, sizeof(int), ctx->stream));
    return gc::set_error(ctx, GC_ETIMEOUT, "tc_gemm: a bounded mbarrier wait expired");
  }
  return GC_OK;
}

int tc_two_sided(gc_context *ctx, int precision, int n, int cnt, const double *M, int nX,
                 const double *CX, int nY, const double *CY, double *T1, double *out,
                 long long ostride) {
  if (precision == GC_PREC_FP64)
    return fp64_two_sided(ctx, n, cnt, M, nX, CX, nY, CY, T1, out, ostride);
  if (is_oz(precision)) {
    OzPlan pl = oz_plan(precision);
    {
      OzOperand A, B;
      GC_TRY(make_oz_operand(ctx, A, M, n * cnt, n, 1, n, 1, 0, pl.S, BM));
      GC_TRY(make_oz_operand(ctx, B, CX, nX, n, 1, n, 1, 0, pl.S,
                             oz_tile(ctx, pl.S, (long long)n * cnt, nX, 1)));
      OzEpi e{0, T1, (long long)n * cnt, 0, nullptr, nullptr, nullptr, nullptr, 0, 0};
      GC_TRY(run_oz(ctx, A, B, n * cnt, nX, 1, pl, e));
    }
    {
      OzOperand A, B;
      GC_TRY(make_oz_operand(ctx, A, T1, nX, n, cnt, (long long)n * cnt, 1, n, pl.S, BM));
      GC_TRY(make_oz_operand(ctx, B, CY, nY, n, 1, n, 1, 0, pl.S, oz_tile(ctx, pl.S, nX, nY, cnt)));
      OzEpi e{0, out, nX, ostride, nullptr, nullptr, nullptr, nullptr, 0, 0};
      GC_TRY(run_oz(ctx, A, B, nX, nY, cnt, pl, e));
    }
    return GC_OK;  // the device flag is read at the caller's next sync point
  }
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
  return GC_OK;  // the device flag is read at the caller's next sync point
}

int tc_gemm_nt(gc_context *ctx, int precision, int m, int n, int k, const double *A, int lda,
               const double *B, int ldb, double *C, int ldc) {
  if (precision == GC_PREC_FP64) {
    const double one = 1.0, zero = 0.0;
    GC_CUBLAS(ctx, cublasDgemm(ctx->cublas, CUBLAS_OP_N, CUBLAS_OP_T, m, n, k, &one, A, lda, B, ldb,
                               &zero, C, ldc));
    return GC_OK;
  }
  if (is_oz(precision)) {
    OzPlan pl = oz_plan(precision);
    OzOperand a, b;
    GC_TRY(make_oz_operand(ctx, a, A, m, k, 1, 1, lda, 0, pl.S, BM));
    GC_TRY(make_oz_operand(ctx, b, B, n, k, 1, 1, ldb, 0, pl.S, oz_tile(ctx, pl.S, m, n, 1)));
    OzEpi e{0, C, ldc, 0, nullptr, nullptr, nullptr, nullptr, 0, 0};
    GC_TRY(run_oz(ctx, a, b, m, n, 1, pl, e));
    return GC_OK;  // the device flag is read at the caller's next sync point
  }
  int S;
  PassList pl = pass_list(precision, &S);
  Operand a, b;
  // A (m x k) column-major: row i, k stride lda
  GC_TRY(make_operand(ctx, a, A, m, k, 1, 1, lda, 0, S, BM));
  GC_TRY(make_operand(ctx, b, B, n, k, 1, 1, ldb, 0, S, BN_T));
  Epi e{0, C, ldc, 0, nullptr, nullptr};
  GC_TRY(run_gemm(ctx, a, b, m, n, 1, pl, e));
  return GC_OK;  // the device flag is read at the caller's next sync point
}

int tc_gemm_strided(gc_context *ctx, int precision, int M, int N, int K, const double *A,
                    long long sam, long long sak, const double *B, long long sbn, long long sbk,
                    double *C, long long ldc) {
  if (precision == GC_PREC_FP64 || !is_oz(precision))
    return set_error(ctx, GC_EINVAL, "gemm_strided: needs a sliced FP64-accurate precision");
  OzPlan pl = oz_plan(precision);
  OzOperand a, b;
  GC_TRY(make_oz_operand(ctx, a, A, M, K, 1, sam, sak, 0, pl.S, BM));
  GC_TRY(make_oz_operand(ctx, b, B, N, K, 1, sbn, sbk, 0, pl.S, oz_tile(ctx, pl.S, M, N, 1)));
  OzEpi e{0, C, ldc, 0, nullptr, nullptr, nullptr, nullptr, 0, 0};
  GC_TRY(run_oz(ctx, a, b, M, N, 1, pl, e));
  return GC_OK;  // the device flag is read at the caller's next sync point
}

int tc_gemm_strided_lower(gc_context *ctx, int precision, int M, int N, int K, const double *A,
                          long long sam, long long sak, const double *B, long long sbn,
                          long long sbk, double *C, long long ldc, int period) {
  if (!is_oz(precision))
    return set_error(ctx, GC_EINVAL, "gemm_strided_lower: needs a sliced FP64-accurate precision");
  OzPlan pl = oz_plan(precision);
  OzOperand a, b;
  GC_TRY(make_oz_operand(ctx, a, A, M, K, 1, sam, sak, 0, pl.S, BM));
  GC_TRY(make_oz_operand(ctx, b, B, N, K, 1, sbn, sbk, 0, pl.S, oz_tile(ctx, pl.S, M, N, 1)));
  OzEpi e{0, C, ldc, 0, nullptr, nullptr, nullptr, nullptr, 0, 0, period};
  GC_TRY(run_oz(ctx, a, b, M, N, 1, pl, e));
  return GC_OK;  // the device flag is read at the caller's next sync point
}

int tc_syrk_sub_lower(gc_context *ctx, int precision, int M, int K, const double *P, long long sm,
                      long long sk, double *C, long long ldc, int nbatch, long long sb) {
  if (!is_oz(precision))
    return set_error(ctx, GC_EINVAL, "syrk_sub_lower: needs a sliced FP64-accurate precision");
  OzPlan pl = oz_plan(precision);
  OzOperand a, b;
  GC_TRY(make_oz_operand(ctx, a, P, M, K, nbatch, sm, sk, sb, pl.S, BM));
  GC_TRY(alias_oz_operand(ctx, a, b, oz_tile(ctx, pl.S, M, M, nbatch)));
  OzEpi e{2, C, ldc, nbatch > 1 ? sb : 0, nullptr, nullptr, nullptr, nullptr, 0, 0, M};
  GC_TRY(run_oz(ctx, a, b, M, M, nbatch, pl, e));
  return GC_OK;  // the device flag is read at the caller's next sync point
}

int tc_dot_gemm(gc_context *ctx, int precision, int N, const double *Ksym, const double *Y,
                double *result) {
  if (is_oz(precision)) {
    OzPlan pl = oz_plan(precision);
    OzOperand a, b;
    GC_TRY(make_oz_operand(ctx, a, Ksym, N, N, 1, N, 1, 0, pl.S, BM));
    GC_TRY(make_oz_operand(ctx, b, Y, N, N, 1, N, 1, 0, pl.S, oz_tile(ctx, pl.S, N, N, 1)));
    size_t ncta = (size_t)ceil_div(N, BM) * ceil_div(N, b.box_rows);
    DevBuf<double> part;
    GC_TRY(part.alloc(ctx, ncta));
    OzEpi e{1, nullptr, N, 0, Y, part.p, nullptr, nullptr, 0, 0};
    GC_TRY(run_oz(ctx, a, b, N, N, 1, pl, e));
    std::vector<double> h(ncta);
    GC_CUDA(ctx, cudaMemcpyAsync(h.data(), part.p, ncta * sizeof(double), cudaMemcpyDeviceToHost,
                                 ctx->stream));
    GC_TRY(check_flag(ctx));
    double sum = 0.0;
    for (double v : h) sum += v;
    *result = sum;
    return GC_OK;
  }
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
  GC_TRY(gc::tc_gemm_nt(ctx, precision, m, n, k, A, lda, B, ldb, C, ldc));
  return gc::check_flag(ctx);
}

// Deterministic operands for gc_tc_gemm_time: x = u 2^-k with u uniform in
// [-1, 1) and k in 0..19 from a hash of the element index, so that every row
// mixes magnitudes over six decades (what the slicing sees on real operands).
__global__ void k_fill_mixed(size_t n, unsigned long long seed, double *__restrict__ x) {
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n;
       i += (size_t)gridDim.x * blockDim.x) {
    unsigned long long h = (i + 1) * 0x9E3779B97F4A7C15ull ^ seed;
    h ^= h >> 31;
    h *= 0xBF58476D1CE4E5B9ull;
    h ^= h >> 29;
    const double u = (double)(h >> 11) * 0x1.0p-53 * 2.0 - 1.0;
    x[i] = ldexp(u, -(int)((h >> 3) % 20));
  }
}

// CUDA event pair destroyed on every return path.
struct EventPair {
  cudaEvent_t a = nullptr, b = nullptr;
  ~EventPair() {
    if (a) cudaEventDestroy(a);
    if (b) cudaEventDestroy(b);
  }
};

extern "C" int gc_tc_gemm_time(gc_context *ctx, int precision, int m, int n, int k, int reps,
                               double *ms_per_launch) {
  if (!ctx) return GC_EINVAL;
  if (m <= 0 || n <= 0 || k <= 0 || reps <= 0 || !ms_per_launch ||
      (precision != GC_PREC_BF16X3 && precision != GC_PREC_BF16X6 && !is_oz(precision)))
    return gc::set_error(ctx, GC_EINVAL, "tc_gemm_time: bad arguments");
  gc::DevBuf<double> a, b, c;
  GC_TRY(a.alloc(ctx, (size_t)m * k));
  GC_TRY(b.alloc(ctx, (size_t)n * k));
  GC_TRY(c.alloc(ctx, (size_t)m * n));
  k_fill_mixed<<<152 * 8, 256, 0, ctx->stream>>>((size_t)m * k, 0x1234567ull, a.p);
  GC_LAUNCHED(ctx);
  k_fill_mixed<<<152 * 8, 256, 0, ctx->stream>>>((size_t)n * k, 0x7654321ull, b.p);
  GC_LAUNCHED(ctx);
  EventPair ev;
  GC_CUDA(ctx, cudaEventCreate(&ev.a));
  GC_CUDA(ctx, cudaEventCreate(&ev.b));
  float ms = 0.f;
  if (is_oz(precision)) {
    OzPlan pl = oz_plan(precision);
    OzOperand A, B;
    GC_TRY(make_oz_operand(ctx, A, a.p, m, k, 1, k, 1, 0, pl.S, BM));
    GC_TRY(make_oz_operand(ctx, B, b.p, n, k, 1, k, 1, 0, pl.S, oz_tile(ctx, pl.S, m, n, 1)));
    OzEpi e{0, c.p, m, 0, nullptr, nullptr, nullptr, nullptr, 0, 0};
    GC_TRY(run_oz(ctx, A, B, m, n, 1, pl, e));  // warm-up
    GC_CUDA(ctx, cudaEventRecord(ev.a, ctx->stream));
    for (int r = 0; r < reps; ++r) GC_TRY(run_oz(ctx, A, B, m, n, 1, pl, e));
    GC_CUDA(ctx, cudaEventRecord(ev.b, ctx->stream));
    GC_CUDA(ctx, cudaEventSynchronize(ev.b));
    GC_CUDA(ctx, cudaEventElapsedTime(&ms, ev.a, ev.b));
  } else {
    int S;
    PassList pl = pass_list(precision, &S);
    Operand A, B;
    GC_TRY(make_operand(ctx, A, a.p, m, k, 1, k, 1, 0, S, BM));
    GC_TRY(make_operand(ctx, B, b.p, n, k, 1, k, 1, 0, S, BN_T));
    Epi e{0, c.p, m, 0, nullptr, nullptr};
    GC_TRY(run_gemm(ctx, A, B, m, n, 1, pl, e));  // warm-up
    GC_CUDA(ctx, cudaEventRecord(ev.a, ctx->stream));
    for (int r = 0; r < reps; ++r) GC_TRY(run_gemm(ctx, A, B, m, n, 1, pl, e));
    GC_CUDA(ctx, cudaEventRecord(ev.b, ctx->stream));
    GC_CUDA(ctx, cudaEventSynchronize(ev.b));
    GC_CUDA(ctx, cudaEventElapsedTime(&ms, ev.a, ev.b));
  }
  *ms_per_launch = ms / reps;
  return gc::check_flag(ctx);
}
