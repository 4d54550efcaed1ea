/*
 * gammcor_gpu.h -- C ABI of the GB300 AC-CAS (FOFO) library.
 *
 * Conventions shared by every entry point
 *  - Matrices are column-major with Fortran meaning: A(i,j) at A[i + j*ld].
 *  - Orbital and pair indices passed in IndN are 1-based, as in the reference.
 *  - "dev" arguments are device pointers on the context's device; "host"
 *    arguments are host memory. Work is ordered on the context's stream.
 *  - Every function returns a gc_status; GC_OK is 0. gc_last_error() gives a
 *    one-line message for the last failure on a context.
 *  - A context is not re-entrant: use one context per host thread.
 */
#ifndef GAMMCOR_GPU_H
#define GAMMCOR_GPU_H

#ifdef __cplusplus
extern "C" {
#endif

typedef struct gc_context gc_context;

enum gc_status {
  GC_OK = 0,
  GC_EINVAL = 1,      /* bad argument */
  GC_ECUDA = 2,       /* CUDA runtime error */
  GC_ECUBLAS = 3,     /* cuBLAS error */
  GC_ECUSOLVER = 4,   /* cuSOLVER error (eigensolver did not converge, ...) */
  GC_ENOTPD = 5,      /* Cholesky found A+B not positive definite */
  GC_ETIMEOUT = 6,    /* a bounded device wait ran out */
  GC_ENOMEM = 7,      /* device allocation failed */
  GC_EUNSUPPORTED = 8, /* shape or mode the library does not handle */
  GC_ENONFINITE = 9   /* a NaN or infinity in the inputs (occupations, one-electron
                         integrals, 2-RDM), in A+-B before the eigensolve, or in W */
};

/* Arithmetic of the integral transform and of the integrand contraction. */
enum gc_precision {
  GC_PREC_FP64 = 0,    /* plain FP64 (cuBLAS DGEMM) */
  GC_PREC_BF16X3 = 1,  /* split-BF16 3-pass on tcgen05 tensor cores, FP32 accumulate */
  GC_PREC_BF16X6 = 2,  /* three BF16 planes, 6 passes (products x_i y_j, i+j<=2): FP32-level
                          product error, tcgen05 tensor cores, FP32 accumulate */
  GC_PREC_FP64TC5 = 3, /* FP64-accurate on tcgen05: rows scaled by powers of two and cut into
                          5 integer BF16 slices; products of equal weight accumulate exactly in
                          FP32 over K chunks short enough to stay below 2^24; chunks summed in
                          FP64. 15 passes, error ~2^-35 of |A||B|^T */
  GC_PREC_FP64TC6 = 4, /* as FP64TC5 with 6 slices: 21 passes, error ~2^-42 of |A||B|^T */
  GC_PREC_FP64TC4 = 5  /* as FP64TC5 with 4 slices: 10 passes, error ~2^-28 of |A||B|^T
                          (between FP32 and FP64) */
};

/* ERPA eigen-solver form. */
enum gc_erpa_mode {
  GC_ERPA_SYMM1 = 0,     /* ERPASYMM1: eig(A+), A+^1/2 A- A+^1/2, eig  (2 eigensolves) */
  GC_ERPA_CHOLESKY = 1,  /* A+ = L L^T, eig(L^T A- L), Y = L u / sqrt(2 w) (1 eigensolve) */
  GC_ERPA_CHOLESKY_REFINED = 2, /* as GC_ERPA_CHOLESKY, with the eigensolve of L^T A- L done in
                          FP32 (ssyevd) and refined to FP64 accuracy: per iteration the Rayleigh
                          matrices S = X^T M X and G = X^T X in the GEMM precision, clusters of
                          close eigenvalues diagonalised exactly in FP64, and the update
                          X <- X (I + E - E E^T / 2) with E first order in the residual for the
                          rest. Falls back to dsyevd when a cluster is wider than 64 or a block
                          is singular */
  GC_ERPA_VEC = 3        /* ERPAVEC (interpa.f:962-1070), the solver of state-averaged references
                          (NoSt > 1): right eigenvectors of A+ A- (general FP64 eigensolver),
                          degenerate groups orthonormalised, complex modes dropped, modes of
                          negative norm returned with -omega; A+B need not be positive definite */
};

/* Context ------------------------------------------------------------- */
/* cuda_stream is used as given; NULL selects the legacy default stream. */
int gc_create(gc_context **ctx, int device, void *cuda_stream);
int gc_destroy(gc_context *ctx);
const char *gc_last_error(const gc_context *ctx);
int gc_synchronize(gc_context *ctx);
/* Number of kernels of this library launched on the context so far. */
long long gc_kernel_launches(const gc_context *ctx);
/* Device time (CUDA events) of the cuSOLVER eigensolves run on the context so far
 * (dsyevd of ERPASYMM1 and of the Cholesky form, ssyevd of the refined form, and in
 * batched calls one cusolverDnXsyevBatched per system for all its points), and the
 * number of matrices solved; batched calls add their workers' eigensolves. No counterpart in
 * the reference. */
int gc_eig_time(const gc_context *ctx, double *ms, long long *calls);
/* Phases of the AC path whose device time gc_phase_time reports. */
enum gc_phase {
  GC_PHASE_TRANSFORM = 0, /* FOFO and FFOO (tran4_gen / tran4_factored) */
  GC_PHASE_ASSEMBLY = 1,  /* A+-B at a point (assembly or the affine combination) */
  GC_PHASE_CHOLESKY = 2,  /* Cholesky factor of A+B (in batched calls one per system) */
  GC_PHASE_PRODUCTS = 3,  /* the ERPA solve's products: L^T A- L, Y = L U (or A+^1/2) */
  GC_PHASE_EIGEN = 4,     /* eigenpairs: dsyevd, or the FP32 eigensolve plus the FP64
                             refinement (in batched calls one phase per system) */
  GC_PHASE_INTEGRAND = 5, /* ACEneERPA */
  GC_PHASE_COUNT = 6
};
/* on = 1 records CUDA events around every phase above on the context's stream
 * (batched calls: on every worker); 0 stops recording. Totals accumulate until
 * read. No counterpart in the reference (it reports CPU times per routine). */
int gc_set_phase_timing(gc_context *ctx, int on);
/* Device time of one phase so far, summed over its calls (concurrent workers'
 * times add up), and the number of calls. Waits for the context's stream. */
int gc_phase_time(gc_context *ctx, int phase, double *ms, long long *calls);
/* on = 1 lets cuSOLVER run the FP64 eigensolver's internal matrix products with
 * its fixed-point FP64 emulation on tensor cores (cusolverDnSetEmulationStrategy
 * EAGER), and the FP32 eigensolver of GC_ERPA_CHOLESKY_REFINED with BF16x9
 * emulated FP32 math (CUSOLVER_FP32_EMULATED_BF16X9_MATH); on = 0 restores the
 * defaults. */
int gc_set_eig_emulation(gc_context *ctx, int on);
/* Refinement iterations of GC_ERPA_CHOLESKY_REFINED (default 2, range 1..4). */
int gc_set_eig_refinement(gc_context *ctx, int iterations);
/* on = 1 (default): the Cholesky of A+B in the ERPA forms with sliced tensor-core
 * products is this library's blocked factorization (FP64 64-wide diagonal blocks
 * and row-wise panel solves on the CUDA cores, trailing updates on the sliced
 * GEMM); on = 0: one cuSOLVER FP64 dpotrf. The FP64 path always uses dpotrf. */
int gc_set_chol_blocked(gc_context *ctx, int on);
/* Limit, in nanoseconds, of every pipeline wait of the tensor-core GEMM kernels
 * launched on the context (default and maximum 1 s; 0 restores the default).
 * A wait that runs out makes the kernel stop issuing work, wait (1 s at most)
 * for the copies and products it already issued, free its tensor memory and
 * raise a device flag; the call then returns GC_ETIMEOUT and the context stays
 * usable. Shortening the limit is a fault-injection setting for tests; no
 * counterpart in the reference. */
int gc_set_pipeline_wait(gc_context *ctx, unsigned long long ns);
/* Column tile width of the FP64-accurate sliced GEMMs (GC_PREC_FP64TC4/5/6): 0
 * (the default) picks one per product from its shape, 64, 96 or 128 forces it
 * (capped at 128 for FP64TC4, 96 for FP64TC5, 64 for FP64TC6). Every width gives
 * the same result bits; only the speed differs. No counterpart in the reference. */
int gc_set_gemm_tile(gc_context *ctx, int width);
/* on = 1 (default): the batched AC calls (gc_ac_energy_batched, sessions) solve the FP32
 * eigenproblems of all lambda points of a system in one batched cuSOLVER call
 * (cusolverDnXsyevBatched) before refining each, in the GC_ERPA_CHOLESKY_REFINED form
 * with sliced products; on = 0 solves them one point at a time. Batch workers take the
 * setting of the context the batched call is given. No counterpart in the reference. */
int gc_set_eig_batch(gc_context *ctx, int on);
/* Counters of GC_ERPA_CHOLESKY_REFINED on a context: solves, solves that fell back to
 * dsyevd, and the largest cluster of close eigenvalues diagonalised in a block. */
int gc_eig_refine_stats(const gc_context *ctx, long long *solves, long long *fallbacks,
                        int *max_cluster);

/* Host-side helpers ----------------------------------------------------- */

/* GauLeg, misc.f:828-865: Gauss-Legendre abscissas x(n) and weights w(n) on [x1,x2]. */
int gc_gauleg(double x1, double x2, double *x, double *w, int n);

/* prepare_nums, initia.f:2996-3035: leading fully occupied (num0) and partially
 * occupied (num1) orbital counts from Occ(nbas) and NELE. */
int gc_prepare_nums(int nbas, const double *occ, int nele, int *num0, int *num1);

/* Pair builder, accas.f:30-106 (IndN/IndX/NDimX of ACCAS). indn: host int
 * array of capacity 2*nbas*(nbas-1)/2, filled as IndN(2,NDimX) 1-based. */
int gc_pair_space(int nbas, const double *occ, int nele, int ifl_core,
                  double thr_sel_act, double thr_qvirt, int *indn, int *ndimx);

/* Integral transform -------------------------------------------------- */

/* tran4_gen, tran.f90:313-423. ao_sorted_dev: the AOTWOSORT tensor as ntr
 * records of ntr doubles (record rs holds (pq|rs) for packed pq, p<=q,
 * pq = p + q(q-1)/2). CA..CD: AO x MO coefficient blocks (nbas x nX,
 * column-major, device). out_dev: nA*nB records of nC*nD doubles, record
 * ab = a + (b-1)*nA, element cd = c + (d-1)*nC (the FFOO/FOFO file layout). */
int gc_tran4_gen(gc_context *ctx, int nbas,
                 int nA, const double *CA_dev, int nB, const double *CB_dev,
                 int nC, const double *CC_dev, int nD, const double *CD_dev,
                 const double *ao_sorted_dev, double *out_dev, int precision);

/* Label formats of the AO integral files readtwoint decodes (sorter.f90:31-395). */
enum gc_twoint_format {
  GC_TWOINT_DALTON8 = 0,   /* one int per integral: p, q, r, s in bits 0-7, 8-15, 16-23, 24-31 */
  GC_TWOINT_DALTON16 = 1,  /* two ints per integral: (r | s << 16), (p | q << 16) */
  GC_TWOINT_PQRS = 2,      /* four ints per integral: p, q, r, s */
  GC_TWOINT_TRIANGLE = 3   /* no labels: all ntr(ntr+1)/2 values with pq >= rs, pq outer */
};

/* readtwoint, sorter.f90:31-395: one chunk of AO integrals (val_dev, labels_dev,
 * device memory) sorted into the AOTWOSORT tensor ao_sorted_dev (ntr records of
 * ntr doubles, record rs holds (pq|rs), pq = p + q(q-1)/2). Each integral goes to
 * record rs at pq and, by the format's rule, to record pq at rs; a slot written
 * twice keeps the later integral, within a chunk and across chunks (calls are
 * ordered on the context's stream). init = 1 zeroes the tensor first, as the
 * reference starts every record at zero. Labels outside 1..nbas are skipped and
 * reported with GC_EINVAL after the chunk. */
int gc_sort_twoint(gc_context *ctx, int nbas, long long nints, const double *val_dev,
                   const int *labels_dev, int format, int init, double *ao_sorted_dev);

/* The AOTWOSORT tensor from the ERI factor: (pq|rs) = sum_P L(pq,P) L(rs,P), i.e.
 * L L^T with lfac_dev (ntr x rank, column-major), in the given precision. No
 * counterpart routine in the reference: the on-device producer of the tensor
 * that gc_tran4_gen reads, for inputs given as a factor. */
int gc_ao_eri_factored(gc_context *ctx, int nbas, int rank, const double *lfac_dev,
                       double *ao_sorted_dev, int precision);

/* Same output as gc_tran4_gen from the ERI factor instead of the 4-index AO
 * tensor: (pq|rs) = sum_P L(pq,P) L(rs,P), lfac_dev = L as (ntr x rank)
 * column-major with the AOTWOSORT pair packing. No counterpart routine in the
 * reference: it is the on-device AO ERI producer folded into tran4_gen. */
int gc_tran4_factored(gc_context *ctx, int nbas, int rank, const double *lfac_dev,
                      int nA, const double *CA_dev, int nB, const double *CB_dev,
                      int nC, const double *CC_dev, int nD, const double *CD_dev,
                      double *out_dev, int precision);

/* A+B / A-B assembly ----------------------------------------------------- */

/* AB_CAS_FOFO, abfofo.f90:8-293 with JK_loop, abfofo.f90:4468-5053
 * (ICASSCF=1, AB1=.false., URe = identity as LdInteg leaves it).
 *   occ_host(nbas), xone_host(nbas(nbas+1)/2) one-electron MO integrals,
 *   indn_host IndN(2,ndimx) 1-based (IndX(i) = i), rdm2act_host active 2-RDM
 *   in the NAddrRDM packing of rdm2.dat (value/2 as AB_CAS_FOFO stores it),
 *   ffoo_dev/fofo_dev from gc_tran4_gen, alpha = ACAlpha.
 * Writes abplus_dev/abmin_dev (ndimx x ndimx) and *etot_host (E_CAS w/o ENuc). */
int gc_ab_cas_fofo(gc_context *ctx, int nbas, int ninact, int nact, int ndimx,
                   const double *occ_host, const double *xone_host,
                   const int *indn_host, const double *rdm2act_host,
                   const double *ffoo_dev, const double *fofo_dev, double alpha,
                   double *abplus_dev, double *abmin_dev, double *etot_host);

/* AB_CAS_FOFO with every argument of the reference routine (abfofo.f90:8-10):
 * ure_host (nbas x nbas, column-major) rotates the one-electron integrals,
 * HNO = URe h URe^T symmetrised (abfofo.f90:97-100); NULL is the identity, as
 * LdInteg leaves it. ab1 = 1 returns the AB1 matrices (abfofo.f90:109-171,
 * 260-263): the lambda derivative of A+-B (AuxCoeff 0 inside one orbital group,
 * HNO zeroed inside a group, HNOCoef -1), symmetrised; with alpha = 1 it is
 * A+-B(1) - A+-B(0), as the AC0 and frequency routines use it. */
int gc_ab_cas_fofo_ex(gc_context *ctx, int nbas, int ninact, int nact, int ndimx,
                      const double *occ_host, const double *ure_host, const double *xone_host,
                      const int *indn_host, const double *rdm2act_host,
                      const double *ffoo_dev, const double *fofo_dev, double alpha, int ab1,
                      double *abplus_dev, double *abmin_dev, double *etot_host);

/* ERPA ---------------------------------------------------------------------- */

/* ERPASYMM1(EigVecR,Eig,APLSQRT,ABMIN,NBasis,NDimX), interpa.f:1652-1781, with the
 * reference's argument semantics: abplus_dev holds A+ on entry and A+^1/2 on return
 * (the routine overwrites APLSQRT), abmin_dev is symmetrised in place, eigvec_dev
 * receives Y, eig_dev omega (omega^2 where omega^2 <= 1e-6), ascending. FP64. */
int gc_erpasymm1(gc_context *ctx, int ndimx, double *abplus_dev, double *abmin_dev,
                 double *eigvec_dev, double *eig_dev);

/* ERPASYMM1, interpa.f:1652-1781 (mode GC_ERPA_SYMM1), or the Cholesky form.
 * abplus_dev/abmin_dev are read (and symmetrised in place). eigvec_dev(N,N)
 * receives Y (column nu), eig_dev(N) omega (omega^2 where omega^2 <= 1e-6),
 * ascending. */
int gc_erpa(gc_context *ctx, int ndimx, double *abplus_dev, double *abmin_dev,
            double *eigvec_dev, double *eig_dev, int mode);
/* gc_erpa with the arithmetic of the Cholesky form's matrix products (and of the
 * refinement products of GC_ERPA_CHOLESKY_REFINED) chosen by precision: GC_PREC_FP64
 * (cuBLAS) or GC_PREC_FP64TC4 / 5 / 6 (sliced tensor-core GEMM). The
 * eigenvalues of the refined mode are not sorted. */
int gc_erpa_ex(gc_context *ctx, int ndimx, double *abplus_dev, double *abmin_dev,
               double *eigvec_dev, double *eig_dev, int mode, int precision);

/* Integrand ---------------------------------------------------------------- */

/* ACEneERPA_FOFO, abfofo.f90:3791-3927: *w_host = W(lambda) of the routine. */
int gc_ace_ne_erpa_fofo(gc_context *ctx, int nbas, int ninact, int nact, int ndimx,
                        const double *occ_host, const int *indn_host,
                        const double *eigvec_dev, const double *eig_dev,
                        const double *fofo_dev, int precision, double *w_host);

/* W(lambda) as gc_ace_ne_erpa_fofo computes it, for callers that cannot
 * allocate device memory: a host whose device memory belongs to its own pool,
 * or a process that must not grow its device footprint after start-up. It
 * allocates nothing: its working data lives in one fixed device array of this
 * library (155 904 bytes, held by every device that loads the library until
 * the process exits), which limits it to nbas <= 2048 and ndimx <= 16384;
 * larger sizes return GC_EINVAL. The call must be made with the context's
 * device current (GC_EINVAL otherwise). The first call on a device looks up
 * that array's device address, so make it before any stream capture. Every
 * call shares the array: calls that overlap on the GPU (other streams, other
 * contexts on the device) race. The call waits for its result on the
 * context's stream. FP64 throughout, about ndimx^3 multiply-adds; no
 * counterpart routine in the reference. */
int gc_ace_ne_erpa_fofo_noalloc(gc_context *ctx, int nbas, int ninact, int nact,
                                int ndimx, const double *occ_host,
                                const int *indn_host, const double *eigvec_dev,
                                const double *eig_dev, const double *fofo_dev,
                                double *w_host);

/* AC0 ------------------------------------------------------------------------ */

/* AC0CAS_FOFO, abfofo.f90:1485-1750 (dispatched at acfd.f:64-68): the AC0
 * correlation energy, first order in the adiabatic connection. A+-B at
 * lambda = 0 is block diagonal in the pair groups of create_AC0_blocks_1/2
 * (abfofo.f90:1374-1484); each block's ERPA problem (ERPASYMM0,
 * interpa.f:1496-1650) is solved on the device in FP64, the AB1 matrices are
 * taken to the zeroth-order modes and back (abpm_tran, ABPM_BACKTRAN) and
 * contracted with FOFO. Arguments as gc_ab_cas_fofo_ex (ure_host NULL = identity);
 * *ecorr_host = ECorr, *etot_host = E_CAS w/o ENuc (may be NULL). Blocks larger
 * than 64 pairs (nact > 11) return GC_EUNSUPPORTED. */
int gc_ac0cas_fofo(gc_context *ctx, int nbas, int ninact, int nact, int ndimx,
                   const double *occ_host, const double *ure_host, const double *xone_host,
                   const int *indn_host, const double *rdm2act_host, const double *ffoo_dev,
                   const double *fofo_dev, double *ecorr_host, double *etot_host);

/* ACFREQ ---------------------------------------------------------------------- */

/* FreqGrid, ac_iter.f:414-429: nfreq Gauss-Legendre points on [-1, 1] mapped to
 * frequencies x in [0, inf) with x0 = 1/2, and their weights w. */
int gc_freq_grid(int nfreq, double *x, double *w);

/* WIter_FOFO, ac_fofo.f90:1-181 (the ACFREQ job, ac_iter.f:44-48): the AC
 * correlation energy from the imaginary-frequency integral of the response,
 * expanded to order max_cn in lambda (the reference uses nfreq = 25,
 * max_cn = 3), contracted with FOFO as the integrand is. The series is carried
 * in the eigenbasis of the lambda = 0 ERPA problem (one Cholesky, one
 * eigensolve of mode GC_ERPA_CHOLESKY or GC_ERPA_CHOLESKY_REFINED), so each
 * frequency costs element-wise passes and 2 (max_cn - 2) + 1 GEMMs in the given
 * precision (GC_PREC_FP64 or a sliced GC_PREC_FP64TC4/5/6) instead of an LU
 * inverse. When A+B(0) is not positive definite (no Cholesky factor) the
 * reference's own form runs instead: the LU inverse of A0 + omega^2 at every
 * frequency (dgetrf/dgetrs) and FP64 products. Other arguments as
 * gc_ab_cas_fofo_ex; *etot_host = E_CAS w/o ENuc (may be NULL). */
int gc_ac_freq_fofo(gc_context *ctx, int nbas, int ninact, int nact, int ndimx,
                    const double *occ_host, const double *ure_host, const double *xone_host,
                    const int *indn_host, const double *rdm2act_host, const double *ffoo_dev,
                    const double *fofo_dev, int nfreq, int max_cn, int precision, int erpa_mode,
                    double *ecorr_host, double *etot_host);

/* Whole lambda quadrature ------------------------------------------------ */

/* ACECORR, acfd.f:117-209 with ACEInteg_FOFO, abfofo.f90:3664-3789: for each
 * Gauss-Legendre point lambda_i (ngrid points on [0,1]) assemble A+-B, solve
 * ERPA and contract; *ecorr_host = sum_i w_i W(lambda_i), *ecas_host = E_CAS,
 * w_out_host(ngrid) = W(lambda_i) (may be NULL).
 * erpa_mode: GC_ERPA_SYMM1 reassembles A+-B at every point as the reference
 * does; GC_ERPA_CHOLESKY assembles A+-B at lambda = 0 and 1 once and forms
 * each point as A0 + lambda (A1 - A0). */
int gc_acecorr(gc_context *ctx, int nbas, int ninact, int nact, int ndimx,
               const double *occ_host, const double *xone_host,
               const int *indn_host, const double *rdm2act_host,
               const double *ffoo_dev, const double *fofo_dev, int ngrid,
               int erpa_mode, int precision,
               double *ecorr_host, double *ecas_host, double *w_out_host);

/* Batch of systems -------------------------------------------------------- */

/* One AC-CAS instance: the arguments ACECORR receives (occupations, one-electron
 * MO integrals, IndN, active 2-RDM) plus what LdInteg hands to tran4_gen (MO
 * coefficients and the AO integrals, here as the ERI factor). */
typedef struct gc_system {
  int nbas, ninact, nact, ndimx, rank;
  const double *occ;       /* host, nbas */
  const double *xone;      /* host, nbas(nbas+1)/2 */
  const int *indn;         /* host, IndN(2, ndimx), 1-based */
  const double *rdm2act;   /* host, NAddrRDM-packed active 2-RDM */
  const double *cmo_dev;   /* device, nbas x nbas AO x MO, column-major */
  const double *lfac_dev;  /* device, ntr x rank ERI factor, column-major */
} gc_system;

typedef struct gc_ac_params {
  int ngrid;       /* Gauss-Legendre points on [0,1] (5 in ACECORR) */
  int precision;   /* gc_precision of the transform and the integrand */
  int erpa_mode;   /* gc_erpa_mode */
  int affine;      /* 1: assemble A+-B at lambda = 0 and 1 once, combine per point */
  int nstreams;    /* concurrent worker streams */
  int eig_emulation; /* 1: gc_set_eig_emulation on every worker context */
  int eig_refine;  /* refinement iterations of GC_ERPA_CHOLESKY_REFINED (0: default 2) */
  const double *lambda;  /* host, ngrid points; NULL: Gauss-Legendre points on [0,1] */
  const double *weight;  /* host, ngrid weights used with lambda (NULL: all zero) */
} gc_ac_params;

/* Per system and lambda point, statistics of the ERPA excitation energies kept by
 * the integrand (1e-3 < omega < 1e8): fraction kept, min, max, mean, mean of
 * 1/omega, median. */
#define GC_OMEGA_STATS 6

/* ACECORR for nsys independent systems (no counterpart in the reference, which
 * runs one system per process). ecorr/ecas (nsys), w_lambda (nsys*ngrid, may be
 * NULL), omega_stats (nsys*ngrid*GC_OMEGA_STATS, may be NULL). status (nsys, may
 * be NULL): per-system gc_status; when given, systems with A+B not positive
 * definite (GC_ENOTPD) or with non-finite inputs (GC_ENONFINITE) are reported
 * there instead of failing the call. */
int gc_ac_energy_batched(gc_context *ctx, int nsys, const gc_system *sys,
                         const gc_ac_params *par, double *ecorr, double *ecas,
                         double *w_lambda, double *omega_stats, int *status);

/* A batch whose per-system device state (FFOO, FOFO, A+-B at lambda = 0 and 1)
 * stays resident between calls, so that lambda points can be added to some of
 * its systems later without repeating the transform or the assembly (the
 * integrand surrogate evaluates the end nodes of every system first and the
 * interior nodes only where its error estimate rejects the prediction). The
 * state of a system is built on its first use. par->affine must be 1; ngrid,
 * lambda and weight of par are not used. sys and the host arrays it points to
 * must stay valid until gc_ac_session_destroy. */
typedef struct gc_ac_session gc_ac_session;
int gc_ac_session_create(gc_context *ctx, int nsys, const gc_system *sys,
                         const gc_ac_params *par, gc_ac_session **session);
/* W(lambda) at npoints points (host lambda) for the systems idx[0..nidx) (distinct
 * indices into the session's systems): w_out (nidx*npoints), omega_stats
 * (nidx*npoints*GC_OMEGA_STATS, may be NULL), ecas (nidx, may be NULL), status
 * (nidx, may be NULL; as in gc_ac_energy_batched). Outputs follow the order of idx. */
int gc_ac_session_points(gc_ac_session *session, int nidx, const int *idx, int npoints,
                         const double *lambda, double *w_out, double *omega_stats,
                         double *ecas, int *status);
int gc_ac_session_destroy(gc_ac_session *session);

/* Integrand surrogate (no counterpart in the reference) ---------------------
 * Multilayer perceptron in -> H -> H -> H -> out with GELU on the hidden layers,
 * BF16 weights in the forward pass, FP32 accumulation, FP32 master weights and
 * Adam moments for training. Parameters flattened as W1 (H x in), b1, W2 (H x H),
 * b2, W3 (H x H), b3, W4 (out x H), b4, row-major. x_dev (batch x in), targets
 * and outputs (batch x out) are row-major FP32 device arrays. */
typedef struct gc_mlp gc_mlp;
int gc_mlp_create(gc_context *ctx, int in_dim, int hidden, int out_dim,
                  unsigned long long seed, gc_mlp **mlp);
int gc_mlp_destroy(gc_mlp *mlp);
long long gc_mlp_num_params(const gc_mlp *mlp);
int gc_mlp_set_params(gc_context *ctx, gc_mlp *mlp, const float *params_dev);
int gc_mlp_get_params(gc_context *ctx, gc_mlp *mlp, float *params_dev);
int gc_mlp_forward(gc_context *ctx, gc_mlp *mlp, int batch, const float *x_dev, float *y_dev);
/* Mean-squared-error loss and its gradient w.r.t. the parameters (grad_dev may be NULL). */
int gc_mlp_gradients(gc_context *ctx, gc_mlp *mlp, int batch, const float *x_dev,
                     const float *t_dev, float *grad_dev, float *loss_host);
/* One Adam step (beta 0.9 / 0.999) on the MSE loss of the batch. */
int gc_mlp_train_step(gc_context *ctx, gc_mlp *mlp, int batch, const float *x_dev,
                      const float *t_dev, float lr, float *loss_host);

/* Building block ---------------------------------------------------------- */

/* C (m x n, ldc) = A (m x k, lda) . B (n x k, ldb)^T, all column-major FP64,
 * computed in the given precision (GC_PREC_BF16X3 / GC_PREC_BF16X6 on the
 * tcgen05 tensor cores, GC_PREC_FP64 with DGEMM). No counterpart routine in the
 * reference: it is the contraction engine under tran4_gen and the integrand,
 * exported so that it can be checked on its own. */
int gc_tc_gemm_nt(gc_context *ctx, int precision, int m, int n, int k,
                  const double *A_dev, int lda, const double *B_dev, int ldb,
                  double *C_dev, int ldc);

/* Average device time of one launch of the tensor-core GEMM kernel for an
 * m x n x k product: operands filled with deterministic pseudo-random values
 * that mix magnitudes over six decades in every row, prepared once, then one
 * untimed launch and reps launches timed with CUDA events on the context
 * stream. No counterpart in the reference. */
int gc_tc_gemm_time(gc_context *ctx, int precision, int m, int n, int k, int reps,
                    double *ms_per_launch);

#ifdef __cplusplus
}
#endif
#endif /* GAMMCOR_GPU_H */
