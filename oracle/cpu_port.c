/*
 * CPU FP64 port of the AC-CAS (FOFO) element kernels, for timing the CPU baseline.
 *
 * TEST AND BENCHMARK INFRASTRUCTURE ONLY: tests/ check it against the
 * line-faithful oracle (oracle/ac_cas_ref.py); bench.py times it as the CPU
 * baseline. The product path never loads it.
 *
 * What is here is the part of the path that has no BLAS form, written as
 * OpenMP loops over the host cores:
 *   - cpu_ab_cas_fofo: A+B and A-B of AB_CAS_FOFO (abfofo.f90:8-293) with the
 *     terms of JK_loop (abfofo.f90:4468-5053), in the gather form (each element
 *     (pq, rs) summed from its closed-form terms instead of scattered record
 *     by record), E_CAS included;
 *   - cpu_integrand_kt: the masked, CI-weighted FOFO matrix of ACEneERPA_FOFO
 *     (abfofo.f90:3791-3927), so that W = 2 sum(Yk .* (Kt Yk)) + sum(diag)
 *     is one GEMM (done by the caller with BLAS).
 * Layouts: FOFO record (k,l) = k + l*n of n*nocc elements (i,j) = i + j*n;
 * FFOO record (k,l) = k + l*nocc of n*n elements; matrices column-major.
 * Orbital groups: 0 inactive (i < nin), 1 active, 2 virtual.
 */
#include <math.h>
#include <stdlib.h>
#include <string.h>

typedef struct {
  int n, nin, nact, nocc;
} geo_t;

static inline double FO(const double *f, const geo_t *g, int a, int b, int c, int d) {
  /* (ab|cd), b, d < nocc */
  return f[((size_t)a + (size_t)b * g->n) * ((size_t)g->n * g->nocc) + (size_t)c + (size_t)d * g->n];
}
static inline double FF(const double *f, const geo_t *g, int a, int b, int c, int d) {
  /* (ab|cd), c, d < nocc */
  return f[((size_t)c + (size_t)d * g->nocc) * ((size_t)g->n * g->n) + (size_t)a + (size_t)b * g->n];
}
static inline int grp(const geo_t *g, int i) { return i < g->nin ? 0 : (i < g->nocc ? 1 : 2); }
/* AuxCoeff of AB_CAS_FOFO (abfofo.f90:109-156): 1 when the four groups agree, else lambda */
static inline double AC(int a, int b, int c, int d, double lam) {
  return (a == b && b == c && c == d) ? 1.0 : lam;
}
/* AuxInd (abfofo.f90:158-160): 1 for inactive/active pairs other than active-active, 2 for
 * active-active, 0 otherwise */
static inline int auxind(int a, int b) {
  if (a <= 1 && b <= 1) return (a == 1 && b == 1) ? 2 : 1;
  return 0;
}
static inline double cicoef(double o) { return o >= 0.5 ? sqrt(o) : -sqrt(o); }

/* RDM2val(i,j,k,l) = FRDM2(i,k,j,l) over occupied orbitals (abfofo.f90:84-92,
 * interpa.f:5244-5272); rdm2act holds the NAddrRDM-packed active block. */
static void build_rv(const geo_t *g, const double *occ, const double *rdm2act, double *rv) {
  const int nocc = g->nocc, nin = g->nin, nact = g->nact;
  for (int l = 0; l < nocc; ++l)
    for (int k = 0; k < nocc; ++k)
      for (int j = 0; j < nocc; ++j)
        for (int i = 0; i < nocc; ++i) {
          /* FRDM2(ip, iq, ir, is) with ip=i, iq=k, ir=j, is=l */
          const int ip = i, iq = k, ir = j, is = l;
          double r = 0.0;
          if (ip == ir && iq == is && (occ[ip] == 1.0 || occ[iq] == 1.0)) r += 2.0 * occ[ip] * occ[iq];
          if (ip == is && iq == ir && (occ[ip] == 1.0 || occ[iq] == 1.0)) r -= occ[ip] * occ[iq];
          if (ip >= nin && iq >= nin && ir >= nin && is >= nin) {
            long long i12 = (long long)(ip - nin) * nact + (iq - nin) + 1;
            long long i34 = (long long)(ir - nin) * nact + (is - nin) + 1;
            long long mx = i12 > i34 ? i12 : i34, mn = i12 > i34 ? i34 : i12;
            r = rdm2act[mx * (mx - 1) / 2 + mn - 1];
          }
          rv[i + (size_t)nocc * (j + (size_t)nocc * (k + (size_t)nocc * l))] = r;
        }
}

#define RVX(i, j, k, l) rv[(i) + (size_t)nocc * ((j) + (size_t)nocc * ((k) + (size_t)nocc * (l)))]

int cpu_ab_cas_fofo(int n, int nin, int nact, int N, const double *occ, const double *xone,
                    const int *pp, const int *pq, const double *rdm2act, const double *ffoo,
                    const double *fofo, double lam, double *abp, double *abm, double *etot) {
  const geo_t G = {n, nin, nact, nin + nact};
  const geo_t *g = &G;
  const int nocc = g->nocc, na = nact;
  const size_t nn = (size_t)n * n, na2 = (size_t)na * na;
  double *rv = malloc(sizeof(double) * (size_t)nocc * nocc * nocc * nocc);
  double *h = malloc(sizeof(double) * nn), *hno = malloc(sizeof(double) * nn);
  double *auxi = malloc(sizeof(double) * nn), *auxio = malloc(sizeof(double) * nn);
  double *wmat = calloc(nn, sizeof(double));
  const size_t s1 = (size_t)n * nocc * na2, s4 = nn * na2, s8 = (size_t)nocc * nocc * na2;
  double *z1 = calloc(s1 + 1, 8), *z4 = calloc(s4 + 1, 8), *z7 = calloc(s4 + 1, 8),
         *z5 = calloc(s1 + 1, 8), *z6 = calloc(s1 + 1, 8), *z8 = calloc(s8 + 1, 8),
         *z9 = calloc(s4 + 1, 8), *z10 = calloc(s8 + 1, 8), *z13 = calloc(s8 + 1, 8),
         *z11 = calloc(s1 + 1, 8), *z12 = calloc(s1 + 1, 8);
  if (!rv || !h || !hno || !auxi || !auxio || !wmat || !z1 || !z4 || !z7 || !z5 || !z6 || !z8 ||
      !z9 || !z10 || !z13 || !z11 || !z12)
    return 1;
  build_rv(g, occ, rdm2act, rv);
  /* one-electron matrix from the packed triangle (triang_to_sq, tran.f90:1221-1247) */
  {
    size_t t = 0;
    for (int q = 0; q < n; ++q)
      for (int p = 0; p <= q; ++p, ++t) h[p + (size_t)q * n] = h[q + (size_t)p * n] = xone[t];
  }
  /* E_CAS = 2 sum_i n_i h_ii + sum RDM2val(i,j,k,l) (ij|kl) (abfofo.f90:97-107, JK_loop FFOO pass) */
  if (etot) {
    double e1 = 0.0, e2 = 0.0;
    for (int i = 0; i < nocc; ++i) e1 += occ[i] * h[i + (size_t)i * n];
#pragma omp parallel for reduction(+ : e2) collapse(2)
    for (int l = 0; l < nocc; ++l)
      for (int k = 0; k < nocc; ++k)
        for (int j = 0; j < nocc; ++j)
          for (int i = 0; i < nocc; ++i) e2 += RVX(i, j, k, l) * FF(ffoo, g, i, j, k, l);
    *etot = 2.0 * e1 + e2;
  }
  /* HNO (lambda-scaled, with the (1-lambda) inactive/active Coulomb-exchange of the other
   * groups), AuxI and AuxIO (JK_loop) */
#pragma omp parallel for schedule(static)
  for (int j = 0; j < n; ++j)
    for (int i = 0; i < n; ++i) {
      const int gi = grp(g, i), gj = grp(g, j);
      double corr = 0.0, ai = 0.0, aio = 0.0;
      for (int k = 0; k < nocc; ++k) {
        const int gk = grp(g, k);
        const double ok = occ[k], jv = FF(ffoo, g, i, j, k, k), kv = FO(fofo, g, j, k, i, k);
        if (gi == gj && gk != gi) corr += ok * (2.0 * jv - kv);
        const double t = ok * (2.0 * AC(gi, gj, gk, gk, lam) * jv - AC(gi, gi, gj, gk, lam) * kv);
        ai += t;
        if (k < nin) aio += t;
      }
      const double hv = h[i + (size_t)j * n];
      hno[i + (size_t)j * n] = gi != gj ? lam * hv : hv + (1.0 - lam) * corr;
      auxi[i + (size_t)j * n] = ai;
      auxio[i + (size_t)j * n] = aio;
    }
  /* WMAT(k, r) = sum_{l,i,j} AuxCoeff (kl|ij) RDM2val(i,j,r,l), r occupied */
#pragma omp parallel for schedule(static)
  for (int r = 0; r < nocc; ++r)
    for (int k = 0; k < n; ++k) {
      double s = 0.0;
      const int gk = grp(g, k);
      for (int l = 0; l < nocc; ++l)
        for (int j = 0; j < nocc; ++j)
          for (int i = 0; i < nocc; ++i)
            s += AC(gk, grp(g, l), grp(g, i), grp(g, j), lam) * FO(fofo, g, k, l, i, j) *
                 RVX(i, j, r, l);
      wmat[k + (size_t)r * n] = s;
    }
  /* 2-RDM intermediates: sums over two active indices of an integral times RDM2val */
  if (na > 0) {
#pragma omp parallel for schedule(static) collapse(2)
    for (int d = 0; d < na; ++d)
      for (int c = 0; c < na; ++c)
        for (int b = 0; b < nocc; ++b)
          for (int a = 0; a < n; ++a) {
            double s = 0.0;
            for (int u = 0; u < na; ++u)
              for (int t = 0; t < na; ++t)
                s += FO(fofo, g, a, b, nin + t, nin + u) * RVX(nin + t, nin + u, nin + c, nin + d);
            z1[a + (size_t)n * (b + (size_t)nocc * (c + (size_t)na * d))] = s;
          }
#pragma omp parallel for schedule(static) collapse(2)
    for (int s_ = 0; s_ < na; ++s_)
      for (int q = 0; q < na; ++q)
        for (int p = 0; p < n; ++p)
          for (int r = 0; r < n; ++r) {
            double a4 = 0.0, a7 = 0.0;
            for (int u = 0; u < na; ++u)
              for (int t = 0; t < na; ++t) {
                const double f = FO(fofo, g, r, nin + u, p, nin + t);
                a4 += f * RVX(nin + t, nin + q, nin + s_, nin + u);
                a7 += f * RVX(nin + t, nin + q, nin + u, nin + s_);
              }
            const size_t o = p + (size_t)n * (r + (size_t)n * (q + (size_t)na * s_));
            z4[o] = a4;
            z7[o] = a7;
          }
#pragma omp parallel for schedule(static) collapse(2)
    for (int s_ = 0; s_ < na; ++s_)
      for (int p = 0; p < na; ++p)
        for (int q = 0; q < nocc; ++q)
          for (int r = 0; r < n; ++r) {
            double a5 = 0.0, a6 = 0.0;
            for (int u = 0; u < na; ++u)
              for (int t = 0; t < na; ++t) {
                const double f = FO(fofo, g, r, nin + u, nin + t, q);
                a5 += f * RVX(nin + t, nin + p, nin + s_, nin + u);
                a6 += f * RVX(nin + t, nin + p, nin + u, nin + s_);
              }
            const size_t o = r + (size_t)n * (q + (size_t)nocc * (p + (size_t)na * s_));
            z5[o] = a5;
            z6[o] = a6;
          }
#pragma omp parallel for schedule(static) collapse(2)
    for (int r = 0; r < na; ++r)
      for (int p = 0; p < na; ++p)
        for (int s_ = 0; s_ < nocc; ++s_)
          for (int q = 0; q < nocc; ++q) {
            double a8 = 0.0, a10 = 0.0, a13 = 0.0;
            for (int u = 0; u < na; ++u)
              for (int t = 0; t < na; ++t) {
                a8 += FF(ffoo, g, nin + t, nin + u, q, s_) * RVX(nin + t, nin + u, nin + p, nin + r);
                const double f = FF(ffoo, g, nin + t, q, s_, nin + u);
                a10 += f * RVX(nin + t, nin + p, nin + r, nin + u);
                a13 += f * RVX(nin + t, nin + p, nin + u, nin + r);
              }
            const size_t o = q + (size_t)nocc * (s_ + (size_t)nocc * (p + (size_t)na * r));
            z8[o] = a8;
            z10[o] = a10;
            z13[o] = a13;
          }
#pragma omp parallel for schedule(static) collapse(2)
    for (int s_ = 0; s_ < na; ++s_)
      for (int q = 0; q < na; ++q)
        for (int r = 0; r < n; ++r)
          for (int p = 0; p < n; ++p) {
            double a = 0.0;
            for (int l = 0; l < na; ++l)
              for (int k = 0; k < na; ++k)
                a += FF(ffoo, g, p, r, nin + k, nin + l) * RVX(nin + q, nin + s_, nin + k, nin + l);
            z9[p + (size_t)n * (r + (size_t)n * (q + (size_t)na * s_))] = a;
          }
#pragma omp parallel for schedule(static) collapse(2)
    for (int r = 0; r < na; ++r)
      for (int q = 0; q < na; ++q)
        for (int s_ = 0; s_ < nocc; ++s_)
          for (int p = 0; p < n; ++p) {
            double a11 = 0.0, a12 = 0.0;
            for (int u = 0; u < na; ++u)
              for (int t = 0; t < na; ++t) {
                const double f = FF(ffoo, g, nin + t, p, s_, nin + u);
                a11 += f * RVX(nin + t, nin + q, nin + r, nin + u);
                a12 += f * RVX(nin + t, nin + q, nin + u, nin + r);
              }
            const size_t o = p + (size_t)n * (s_ + (size_t)nocc * (q + (size_t)na * r));
            z11[o] = a11;
            z12[o] = a12;
          }
  }
  /* A+B and A-B, element (row pair i, column pair j) */
#pragma omp parallel for schedule(dynamic, 16)
  for (int j = 0; j < N; ++j)
    for (int i = 0; i < N; ++i) {
      const int p = pp[i], q = pq[i], r = pp[j], s = pq[j];
      const int gp = grp(g, p), gq = grp(g, q), gr = grp(g, r), gs = grp(g, s);
      const double op = occ[p], oq = occ[q], orr = occ[r], os = occ[s];
      double vp = 0.0, vm = 0.0, v;
      const double ac = AC(gp, gq, gr, gs, lam);
      const double X1 = (auxind(gp, gr) == 1 ? op * orr : 0.0) + (auxind(gq, gs) == 1 ? oq * os : 0.0) -
                        (auxind(gq, gr) == 1 ? oq * orr : 0.0) - (auxind(gp, gs) == 1 ? op * os : 0.0);
      if (r >= nin && p >= nin) {
        vm += 4.0 * ac * X1 * FO(fofo, g, r, s, p, q);
        v = ac * X1 * FO(fofo, g, p, s, r, q);
        vp += v;
        vm -= v;
        v = -ac * X1 * FF(ffoo, g, p, r, q, s);
        vp += v;
        vm += v;
      }
      const int pa = gp == 1, qa = gq == 1, ra = gr == 1, sa = gs == 1;
      const int pA = p - nin, qA = q - nin, rA = r - nin, sA = s - nin;
      if (p >= nin && ra && qa) {
        v = AC(gp, gs, 1, 1, lam) * z1[p + (size_t)n * (s + (size_t)nocc * (qA + (size_t)na * rA))];
        vp += v;
        vm -= v;
      }
      if (r >= nin && sa && pa) {
        v = AC(gq, gr, 1, 1, lam) * z1[r + (size_t)n * (q + (size_t)nocc * (pA + (size_t)na * sA))];
        vp += v;
        vm -= v;
      }
      if (r >= nin && sa) {
        if (qa && p >= nin) {
          const size_t o = p + (size_t)n * (r + (size_t)n * (qA + (size_t)na * sA));
          const double c = AC(gp, gr, 1, 1, lam);
          v = c * z4[o];
          vp += v;
          vm += v;
          v = -c * z7[o];
          vp += v;
          vm -= v;
        }
        if (pa) {
          const size_t o = r + (size_t)n * (q + (size_t)nocc * (pA + (size_t)na * sA));
          const double c = AC(gq, gr, 1, 1, lam);
          v = c * z5[o];
          vp += v;
          vm -= v;
          v = -c * z6[o];
          vp += v;
          vm += v;
        }
      }
      if (ra && pa) {
        const size_t o = q + (size_t)nocc * (s + (size_t)nocc * (pA + (size_t)na * rA));
        const double c = AC(gq, gs, 1, 1, lam);
        v = c * z8[o];
        vp += v;
        vm += v;
        v = c * z10[o];
        vp += v;
        vm += v;
        v = -c * z13[o];
        vp += v;
        vm -= v;
      }
      if (sa && r >= nin && qa && p >= nin) {
        v = AC(gp, gr, 1, 1, lam) * z9[p + (size_t)n * (r + (size_t)n * (qA + (size_t)na * sA))];
        vp += v;
        vm += v;
      }
      if (ra && qa && p >= nin) {
        const size_t o = p + (size_t)n * (s + (size_t)nocc * (qA + (size_t)na * rA));
        const double c = AC(gp, gs, 1, 1, lam);
        v = c * z11[o];
        vp += v;
        vm -= v;
        v = -c * z12[o];
        vp += v;
        vm += v;
      }
      /* one-body part: the final loop of AB_CAS_FOFO (abfofo.f90:189-258) */
#define AUX(ga, gb, x, y) \
  (auxind(ga, gb) == 1 ? auxi[(x) + (size_t)(y) * n] : (auxind(ga, gb) == 2 ? auxio[(x) + (size_t)(y) * n] : 0.0))
      double v1 = 0.0, v2 = 0.0;
      if (p == r) v1 += (op - os) * hno[q + (size_t)s * n] - wmat[q + (size_t)s * n] + op * AUX(gp, gr, q, s);
      if (q == s) v1 += (oq - orr) * hno[p + (size_t)r * n] - wmat[p + (size_t)r * n] + oq * AUX(gq, gs, p, r);
      if (q == r) v2 += (oq - os) * hno[p + (size_t)s * n] - wmat[p + (size_t)s * n] + oq * AUX(gq, gr, p, s);
      if (p == s) v2 += (op - orr) * hno[q + (size_t)r * n] - wmat[q + (size_t)r * n] + op * AUX(gp, gs, q, r);
#undef AUX
      vp += v1 + v2;
      vm += v1 - v2;
      const double Cp = cicoef(op), Cq = cicoef(oq), Cr = cicoef(orr), Cs = cicoef(os);
      double d = (Cp + Cq) * (Cr + Cs);
      if (d != 0.0) vp /= d;
      d = (Cp - Cq) * (Cr - Cs);
      if (d != 0.0) vm /= d;
      abp[i + (size_t)j * N] = vp;
      abm[i + (size_t)j * N] = vm;
    }
  free(rv); free(h); free(hno); free(auxi); free(auxio); free(wmat);
  free(z1); free(z4); free(z7); free(z5); free(z6); free(z8); free(z9); free(z10); free(z13);
  free(z11); free(z12);
  return 0;
}

/* Kt[i, j] = mask (C_p + C_q)(C_r + C_s) (rs|pq) for pairs i = (p, q), j = (r, s), with
 * mask = not all four orbitals in one group (abfofo.f90:3823-3834,3889); diag[i] =
 * -mask (n_p (1 - n_q) + n_q (1 - n_p)) (pq|pq), the pq == rs correction. */
void cpu_integrand_kt(int n, int nin, int nact, int N, const double *occ, const int *pp,
                      const int *pq, const double *fofo, double *kt, double *diag) {
  const geo_t G = {n, nin, nact, nin + nact};
  const geo_t *g = &G;
#pragma omp parallel for schedule(static)
  for (int j = 0; j < N; ++j)
    for (int i = 0; i < N; ++i) {
      const int p = pp[i], q = pq[i], r = pp[j], s = pq[j];
      const int same = grp(g, p) == grp(g, q) && grp(g, q) == grp(g, r) && grp(g, r) == grp(g, s);
      const double f = FO(fofo, g, r, s, p, q);
      const double c = (cicoef(occ[p]) + cicoef(occ[q])) * (cicoef(occ[r]) + cicoef(occ[s]));
      kt[i + (size_t)j * N] = same ? 0.0 : c * f;
      if (i == j) diag[i] = same ? 0.0 : -(occ[p] * (1.0 - occ[q]) + occ[q] * (1.0 - occ[p])) * f;
    }
}
