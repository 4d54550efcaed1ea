// ERPA A+B / A-B assembly in gather form.
//
// AB_CAS_FOFO (abfofo.f90:8-293) streams FOFO and FFOO records through
// JK_loop (abfofo.f90:4468-5053) and scatters contributions into
// ABPLUS(ipq,irs). Here every output element (ipq, irs) is computed by one
// thread from closed forms of the same terms:
//   * integral terms read FOFO / FFOO elements directly,
//   * the 2-RDM terms T1..T6 read small intermediates Z (sums over two
//     active indices of an integral times RDM2val) built once per system,
//   * the one-body part reads HNO, AuxI, AuxIO and WMAT (n x n), which the
//     reference accumulates in the same loops.
// Every coefficient is 1, lambda or (1 - lambda), so A+-B is affine in lambda.
#include <cmath>

#include "gc_internal.cuh"

namespace {

struct Geo {
  int n, nin, nact, nocc;
  // AB1 = .false.: AuxCoeff = 1 for four equal groups, HNO kept inside a group with the
  // (1 - lambda) inactive/active correction. AB1 = .true. (the lambda derivative,
  // abfofo.f90:109-156 and HNOCoef, abfofo.f90:167-171, 4494-4500): AuxCoeff = 0 there,
  // HNO zeroed inside a group and the correction taken with coefficient -1.
  double same = 1.0;   // AuxCoeff of four equal groups
  int ab1 = 0;
};

__device__ __forceinline__ double Fofo(const double *__restrict__ f, const Geo &g, int a, int b,
                                       int c, int d) {  // (ab|cd), b, d < nocc
  size_t ld = (size_t)g.n * g.nocc;
  return f[(size_t)(a + (size_t)b * g.n) * ld + c + (size_t)d * g.n];
}
__device__ __forceinline__ double Ffoo(const double *__restrict__ f, const Geo &g, int a, int b,
                                       int c, int d) {  // (ab|cd), c, d < nocc
  size_t ld = (size_t)g.n * g.n;
  return f[(size_t)(c + (size_t)d * g.nocc) * ld + a + (size_t)b * g.n];
}
__device__ __forceinline__ double RV(const double *__restrict__ rv, int nocc, int i, int j, int k,
                                     int l) {
  return rv[i + (size_t)nocc * (j + (size_t)nocc * (k + (size_t)nocc * l))];
}
// AuxCoeff(g1,g2,g3,g4): g.same if the four orbital groups are equal, else lambda.
__device__ __forceinline__ double AC(const Geo &g, int a, int b, int c, int d, double lam) {
  return (a == b && b == c && c == d) ? g.same : lam;
}
// AuxInd(g1,g2) of AB_CAS_FOFO: 1 for inactive/active combinations other than
// active-active, 2 for active-active, 0 otherwise.
__device__ __forceinline__ int AuxInd(int a, int b) {
  if (a <= 1 && b <= 1) return (a == 1 && b == 1) ? 2 : 1;
  return 0;
}

// ---------------------------------------------------------------------------
// One-body matrices (lambda dependent): HNO, AuxI, AuxIO; column-major n x n.
__global__ void k_onebody(Geo g, const double *__restrict__ h, const double *__restrict__ occ,
                          const int *__restrict__ grp, const double *__restrict__ fofo,
                          const double *__restrict__ ffoo, double lam, double *__restrict__ hno,
                          double *__restrict__ auxi, double *__restrict__ auxio) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  int j = blockIdx.y * blockDim.y + threadIdx.y;
  if (i >= g.n || j >= g.n) return;
  int gi = grp[i], gj = grp[j];
  double hv = h[i + (size_t)j * g.n];
  double corr = 0.0, ai = 0.0, aio = 0.0;
  for (int k = 0; k < g.nocc; ++k) {
    int gk = grp[k];
    double ok = occ[k];
    double jv = Ffoo(ffoo, g, i, j, k, k);          // (ij|kk)
    double kv = Fofo(fofo, g, j, k, i, k);          // (jk|ik)
    if (gi == gj && gk != gi) corr += ok * (2.0 * jv - kv);
    double t = ok * (2.0 * AC(g, gi, gj, gk, gk, lam) * jv - AC(g, gi, gi, gj, gk, lam) * kv);
    ai += t;
    if (k < g.nin) aio += t;
  }
  size_t o = i + (size_t)j * g.n;
  hno[o] = (gi != gj) ? lam * hv : (g.ab1 ? -corr : hv + (1.0 - lam) * corr);
  auxi[o] = ai;
  auxio[o] = aio;
}

// WMAT(k, r) = sum_{l,i,j < nocc} AuxCoeff(k,l,i,j) (kl|ij) RDM2val(i,j,r,l); zero for r >= nocc.
// WMAT[k, r] = sum_{i,j,l < nocc} AC(k, l, i, j) (kl|ij) RDM2val(i, j, r, l) for r < nocc
// is a product Fw RV' with K = nocc^3 (kappa = i + nocc (j + nocc l)):
//   Fw[k + n kappa] = AC(groups of k, l, i, j) (ij|kl)     (n x K; consecutive k are
//                                                           consecutive FOFO elements)
//   RV'[kappa + K r] = RDM2val(i, j, r, l)                  (K x nocc)
// so it runs as one FP64 DGEMM instead of an nocc^3 loop per element on the CUDA cores.
__global__ void k_pack_wmat_f(Geo g, const int *__restrict__ grp, const double *__restrict__ fofo,
                              double lam, double *__restrict__ fw) {
  const int k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= g.n) return;
  const int K = g.nocc * g.nocc * g.nocc, gk = grp[k];
  for (int kappa = blockIdx.y; kappa < K; kappa += gridDim.y) {  // i + nocc (j + nocc l)
    const int i = kappa % g.nocc, j = (kappa / g.nocc) % g.nocc, l = kappa / (g.nocc * g.nocc);
    fw[k + (size_t)g.n * kappa] = AC(g, gk, grp[l], grp[i], grp[j], lam) * Fofo(fofo, g, i, j, k, l);
  }
}
__global__ void k_pack_wmat_rv(int nocc, const double *__restrict__ rv, double *__restrict__ rvp) {
  const size_t K = (size_t)nocc * nocc * nocc;
  const size_t total = K * nocc;
  for (size_t t = blockIdx.x * (size_t)blockDim.x + threadIdx.x; t < total;
       t += (size_t)gridDim.x * blockDim.x) {
    const size_t kappa = t % K;
    const int r = (int)(t / K);
    const int i = (int)(kappa % nocc), j = (int)((kappa / nocc) % nocc), l = (int)(kappa / ((size_t)nocc * nocc));
    rvp[t] = RV(rv, nocc, i, j, r, l);
  }
}

// E_CAS two-electron part: sum_{ijkl < nocc} RDM2val(i,j,k,l) (ij|kl); per-block partials.
__global__ void k_etwo(Geo g, const double *__restrict__ ffoo, const double *__restrict__ rv,
                       double *__restrict__ part) {
  __shared__ double red[256];
  size_t total = (size_t)g.nocc * g.nocc * g.nocc * g.nocc;
  double s = 0.0;
  for (size_t t = blockIdx.x * (size_t)blockDim.x + threadIdx.x; t < total;
       t += (size_t)gridDim.x * blockDim.x) {
    int i = t % g.nocc;
    size_t r = t / g.nocc;
    int j = r % g.nocc;
    r /= g.nocc;
    int k = r % g.nocc;
    int l = (int)(r / g.nocc);
    s += rv[t] * Ffoo(ffoo, g, i, j, k, l);
  }
  red[threadIdx.x] = s;
  __syncthreads();
  for (int w = blockDim.x / 2; w > 0; w >>= 1) {
    if (threadIdx.x < w) red[threadIdx.x] += red[threadIdx.x + w];
    __syncthreads();
  }
  if (threadIdx.x == 0) part[blockIdx.x] = red[0];
}

// ---------------------------------------------------------------------------
// 2-RDM intermediates (lambda independent). Capital letters are orbital
// indices T = nin + t of active orbitals; small letters index the active block.

// Z1[a,b,c,d] = sum_tu (ab|TU) RV[T,U,C,D]; a < n, b < nocc, c,d < nact.
__global__ void k_z1(Geo g, const double *__restrict__ fofo, const double *__restrict__ rv,
                     double *__restrict__ z) {
  size_t total = (size_t)g.n * g.nocc * g.nact * g.nact;
  for (size_t t = blockIdx.x * (size_t)blockDim.x + threadIdx.x; t < total;
       t += (size_t)gridDim.x * blockDim.x) {
    int a = t % g.n;
    size_t r = t / g.n;
    int b = r % g.nocc;
    r /= g.nocc;
    int c = r % g.nact, d = (int)(r / g.nact);
    double s = 0.0;
    for (int u = 0; u < g.nact; ++u)
      for (int tt = 0; tt < g.nact; ++tt)
        s += Fofo(fofo, g, g.nin + tt, g.nin + u, a, b) *  // (ab|TU) as (TU|ab): coalesced in a
             RV(rv, g.nocc, g.nin + tt, g.nin + u, g.nin + c, g.nin + d);
    z[t] = s;
  }
}

// Z4[p,r,q,s] = sum_tu (rU|pT) RV[T,Q,S,U];  Z7[p,r,q,s] = sum_tu (rU|pT) RV[T,Q,U,S]
// (p fastest, so that the element kernel reads them along consecutive p).
__global__ void k_z47(Geo g, const double *__restrict__ fofo, const double *__restrict__ rv,
                      double *__restrict__ z4, double *__restrict__ z7) {
  size_t total = (size_t)g.n * g.n * g.nact * g.nact;
  for (size_t t = blockIdx.x * (size_t)blockDim.x + threadIdx.x; t < total;
       t += (size_t)gridDim.x * blockDim.x) {
    int p = t % g.n;
    size_t r0 = t / g.n;
    int r = r0 % g.n;
    r0 /= g.n;
    int q = r0 % g.nact, s = (int)(r0 / g.nact);
    int Q = g.nin + q, S = g.nin + s;
    double a4 = 0.0, a7 = 0.0;
    for (int u = 0; u < g.nact; ++u)
      for (int tt = 0; tt < g.nact; ++tt) {
        double f = Fofo(fofo, g, r, g.nin + u, p, g.nin + tt);
        a4 += f * RV(rv, g.nocc, g.nin + tt, Q, S, g.nin + u);
        a7 += f * RV(rv, g.nocc, g.nin + tt, Q, g.nin + u, S);
      }
    size_t o = p + (size_t)g.n * (r + (size_t)g.n * (q + (size_t)g.nact * s));
    z4[o] = a4;
    z7[o] = a7;
  }
}

// Z5[r,q,p,s] = sum_tu (rU|Tq) RV[T,P,S,U];  Z6[r,q,p,s] = sum_tu (rU|Tq) RV[T,P,U,S].
__global__ void k_z56(Geo g, const double *__restrict__ fofo, const double *__restrict__ rv,
                      double *__restrict__ z5, double *__restrict__ z6) {
  size_t total = (size_t)g.n * g.nocc * g.nact * g.nact;
  for (size_t t = blockIdx.x * (size_t)blockDim.x + threadIdx.x; t < total;
       t += (size_t)gridDim.x * blockDim.x) {
    int r = t % g.n;
    size_t r0 = t / g.n;
    int q = r0 % g.nocc;
    r0 /= g.nocc;
    int p = r0 % g.nact, s = (int)(r0 / g.nact);
    int P = g.nin + p, S = g.nin + s;
    double a5 = 0.0, a6 = 0.0;
    for (int u = 0; u < g.nact; ++u)
      for (int tt = 0; tt < g.nact; ++tt) {
        double f = Fofo(fofo, g, g.nin + tt, q, r, g.nin + u);  // (rU|Tq) as (Tq|rU)
        a5 += f * RV(rv, g.nocc, g.nin + tt, P, S, g.nin + u);
        a6 += f * RV(rv, g.nocc, g.nin + tt, P, g.nin + u, S);
      }
    z5[t] = a5;
    z6[t] = a6;
  }
}

// Z8[q,s,p,r] = sum_tu (TU|qs) RV[T,U,P,R];  q,s < nocc (read from FOFO record (T,U)).
__global__ void k_z8(Geo g, const double *__restrict__ fofo, const double *__restrict__ rv,
                     double *__restrict__ z) {
  size_t total = (size_t)g.nocc * g.nocc * g.nact * g.nact;
  for (size_t t = blockIdx.x * (size_t)blockDim.x + threadIdx.x; t < total;
       t += (size_t)gridDim.x * blockDim.x) {
    int q = t % g.nocc;
    size_t r0 = t / g.nocc;
    int s = r0 % g.nocc;
    r0 /= g.nocc;
    int p = r0 % g.nact, r = (int)(r0 / g.nact);
    double a = 0.0;
    for (int u = 0; u < g.nact; ++u)
      for (int tt = 0; tt < g.nact; ++tt)
        a += Fofo(fofo, g, g.nin + tt, g.nin + u, q, s) *  // (TU|qs) from FOFO: coalesced in q
             RV(rv, g.nocc, g.nin + tt, g.nin + u, g.nin + p, g.nin + r);
    z[t] = a;
  }
}

// Z9[p,r,q,s] = sum_kl (pr|KL) RV[Q,S,K,L].
__global__ void k_z9(Geo g, const double *__restrict__ ffoo, const double *__restrict__ rv,
                     double *__restrict__ z) {
  size_t total = (size_t)g.n * g.n * g.nact * g.nact;
  for (size_t t = blockIdx.x * (size_t)blockDim.x + threadIdx.x; t < total;
       t += (size_t)gridDim.x * blockDim.x) {
    int p = t % g.n;
    size_t r0 = t / g.n;
    int r = r0 % g.n;
    r0 /= g.n;
    int q = r0 % g.nact, s = (int)(r0 / g.nact);
    double a = 0.0;
    for (int l = 0; l < g.nact; ++l)
      for (int k = 0; k < g.nact; ++k)
        a += Ffoo(ffoo, g, p, r, g.nin + k, g.nin + l) *
             RV(rv, g.nocc, g.nin + q, g.nin + s, g.nin + k, g.nin + l);
    z[t] = a;
  }
}

// Z10[q,s,p,r] = sum_tu (Tq|sU) RV[T,P,R,U];  Z13[q,s,p,r] = sum_tu (Tq|sU) RV[T,P,U,R].
__global__ void k_z1013(Geo g, const double *__restrict__ ffoo, const double *__restrict__ rv,
                        double *__restrict__ z10, double *__restrict__ z13) {
  size_t total = (size_t)g.nocc * g.nocc * g.nact * g.nact;
  for (size_t t = blockIdx.x * (size_t)blockDim.x + threadIdx.x; t < total;
       t += (size_t)gridDim.x * blockDim.x) {
    int q = t % g.nocc;
    size_t r0 = t / g.nocc;
    int s = r0 % g.nocc;
    r0 /= g.nocc;
    int p = r0 % g.nact, r = (int)(r0 / g.nact);
    int P = g.nin + p, R = g.nin + r;
    double a10 = 0.0, a13 = 0.0;
    for (int u = 0; u < g.nact; ++u)
      for (int tt = 0; tt < g.nact; ++tt) {
        double f = Ffoo(ffoo, g, q, g.nin + tt, s, g.nin + u);  // (Tq|sU) as (qT|sU)
        a10 += f * RV(rv, g.nocc, g.nin + tt, P, R, g.nin + u);
        a13 += f * RV(rv, g.nocc, g.nin + tt, P, g.nin + u, R);
      }
    z10[t] = a10;
    z13[t] = a13;
  }
}

// Z11[p,s,q,r] = sum_tu (Tp|sU) RV[T,Q,R,U];  Z12[p,s,q,r] = sum_tu (Tp|sU) RV[T,Q,U,R].
__global__ void k_z1112(Geo g, const double *__restrict__ ffoo, const double *__restrict__ rv,
                        double *__restrict__ z11, double *__restrict__ z12) {
  size_t total = (size_t)g.n * g.nocc * g.nact * g.nact;
  for (size_t t = blockIdx.x * (size_t)blockDim.x + threadIdx.x; t < total;
       t += (size_t)gridDim.x * blockDim.x) {
    int p = t % g.n;
    size_t r0 = t / g.n;
    int s = r0 % g.nocc;
    r0 /= g.nocc;
    int q = r0 % g.nact, r = (int)(r0 / g.nact);
    int Q = g.nin + q, R = g.nin + r;
    double a11 = 0.0, a12 = 0.0;
    for (int u = 0; u < g.nact; ++u)
      for (int tt = 0; tt < g.nact; ++tt) {
        double f = Ffoo(ffoo, g, p, g.nin + tt, s, g.nin + u);  // (Tp|sU) as (pT|sU)
        a11 += f * RV(rv, g.nocc, g.nin + tt, Q, R, g.nin + u);
        a12 += f * RV(rv, g.nocc, g.nin + tt, Q, g.nin + u, R);
      }
    z11[t] = a11;
    z12[t] = a12;
  }
}

struct Zs {
  const double *z1, *z4, *z7, *z5, *z6, *z8, *z9, *z10, *z13, *z11, *z12;
};

// ---------------------------------------------------------------------------
// A+B and A-B, element (row = pair i, column = pair j), column-major N x N.
__global__ void k_ab(Geo g, int N, const int *__restrict__ pp, const int *__restrict__ pq,
                     const double *__restrict__ occ, const int *__restrict__ grp,
                     const double *__restrict__ fofo, const double *__restrict__ ffoo, Zs Z,
                     const double *__restrict__ hno, const double *__restrict__ auxi,
                     const double *__restrict__ auxio, const double *__restrict__ wmat, double lam,
                     const double *__restrict__ rpl, const double *__restrict__ rmi,
                     double *__restrict__ abp, double *__restrict__ abm) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  int j = blockIdx.y * blockDim.y + threadIdx.y;
  if (i >= N || j >= N) return;
  const int n = g.n, nin = g.nin, nocc = g.nocc, na = g.nact;
  int p = pp[i], q = pq[i], r = pp[j], s = pq[j];
  int gp = grp[p], gq = grp[q], gr = grp[r], gs = grp[s];
  double op = occ[p], oq = occ[q], orr = occ[r], os = occ[s];
  // Every term enters A+B and A-B either with the same sign (sym, accumulated in S) or
  // with opposite signs (anti, in A); A+B = S + A, A-B = S - A (+ the Coulomb term, A-B
  // only). Each Z term is then one FP64 FMA with its coefficient (1, 0 or lambda):
  // GB300's FP64 pipe, not HBM, bounds this kernel.
  double S = 0.0, A = 0.0, Mo = 0.0;
  const double ac = AC(g, gp, gq, gr, gs, lam);
  auto ai = [](int a, int b) { return AuxInd(a, b) == 1; };
  const double X1 = (ai(gp, gr) ? op * orr : 0.0) + (ai(gq, gs) ? oq * os : 0.0) -
                    (ai(gq, gr) ? oq * orr : 0.0) - (ai(gp, gs) ? op * os : 0.0);
  if (r >= nin && p >= nin) {
    const double t = ac * X1;
    // FOFO Coulomb: A- += 4 AC X1 (rs|pq) (its two A+ parts cancel)
    Mo = 4.0 * t * Fofo(fofo, g, r, s, p, q);
    // FOFO exchange (anti): AC X1 (ps|rq), read as (rq|ps): record (r, q) is shared by a
    // warp of consecutive p and its elements p + s n are contiguous
    A = t * Fofo(fofo, g, r, q, p, s);
    // FFOO exchange (sym): -AC X1 (pr|qs)
    S = -t * Ffoo(ffoo, g, p, r, q, s);
  }
  const bool pa = gp == 1, qa = gq == 1, ra = gr == 1, sa = gs == 1;
  const int pA = p - nin, qA = q - nin, rA = r - nin, sA = s - nin;
  // FOFO T1 (p -> q), anti
  if (p >= nin && ra && qa)
    A = fma(AC(g, gp, gs, 1, 1, lam),
            Z.z1[p + (size_t)n * (s + (size_t)nocc * (qA + (size_t)na * rA))], A);
  // FOFO T3, anti
  if (r >= nin && sa && pa)
    A = fma(AC(g, gq, gr, 1, 1, lam),
            Z.z1[r + (size_t)n * (q + (size_t)nocc * (pA + (size_t)na * sA))], A);
  if (r >= nin && sa) {
    if (qa && p >= nin) {
      const size_t o = p + (size_t)n * (r + (size_t)n * (qA + (size_t)na * sA));
      const double c = AC(g, gp, gr, 1, 1, lam);
      S = fma(c, Z.z4[o], S);   // T4
      A = fma(-c, Z.z7[o], A);  // T6 (p -> q)
    }
    if (pa) {
      const size_t o = r + (size_t)n * (q + (size_t)nocc * (pA + (size_t)na * sA));
      const double c = AC(g, gq, gr, 1, 1, lam);
      A = fma(c, Z.z5[o], A);   // T4 (p -> q)
      S = fma(-c, Z.z6[o], S);  // T6
    }
  }
  if (ra && pa) {
    const size_t o = q + (size_t)nocc * (s + (size_t)nocc * (pA + (size_t)na * rA));
    const double c = AC(g, gq, gs, 1, 1, lam);
    S = fma(c, Z.z8[o] + Z.z10[o], S);  // FFOO T1 + T2
    A = fma(-c, Z.z13[o], A);           // T5 (p -> q)
  }
  if (sa && r >= nin && qa && p >= nin)  // FFOO T3, sym
    S = fma(AC(g, gp, gr, 1, 1, lam),
            Z.z9[p + (size_t)n * (r + (size_t)n * (qA + (size_t)na * sA))], S);
  if (ra && qa && p >= nin) {
    const size_t o = p + (size_t)n * (s + (size_t)nocc * (qA + (size_t)na * rA));
    const double c = AC(g, gp, gs, 1, 1, lam);
    A = fma(c, Z.z11[o], A);   // T2 (p -> q)
    S = fma(-c, Z.z12[o], S);  // T5
  }
  // one-body part (final loop of AB_CAS_FOFO): sym (p = r, q = s) and anti (q = r, p = s)
  auto aux = [&](int ga, int gb, int x, int y) -> double {
    int a = AuxInd(ga, gb);
    if (a == 1) return auxi[x + (size_t)y * n];
    if (a == 2) return auxio[x + (size_t)y * n];
    return 0.0;
  };
  if (p == r)
    S += (op - os) * hno[q + (size_t)s * n] - wmat[q + (size_t)s * n] + op * aux(gp, gr, q, s);
  if (q == s)
    S += (oq - orr) * hno[p + (size_t)r * n] - wmat[p + (size_t)r * n] + oq * aux(gq, gs, p, r);
  if (q == r)
    A += (oq - os) * hno[p + (size_t)s * n] - wmat[p + (size_t)s * n] + oq * aux(gq, gr, p, s);
  if (p == s)
    A += (op - orr) * hno[q + (size_t)r * n] - wmat[q + (size_t)r * n] + op * aux(gp, gs, q, r);
  double vp = S + A, vm = S - A + Mo;
  // divide by (C_p + C_q)(C_r + C_s) and (C_p - C_q)(C_r - C_s) where they are not 0,
  // as products of the pair reciprocals (no FP64 square root or division per element)
  const double ai_ = rpl[i], aj_ = rpl[j], bi_ = rmi[i], bj_ = rmi[j];
  if (ai_ != 0.0 && aj_ != 0.0) vp *= ai_ * aj_;
  if (bi_ != 0.0 && bj_ != 0.0) vm *= bi_ * bj_;
  size_t o = i + (size_t)j * N;
  abp[o] = vp;
  abm[o] = vm;
}

// sq_symmetrize (tran.f90:1303-1319): a(i,j) = a(j,i) = (a(i,j) + a(j,i)) / 2.
__global__ void k_sym_avg(int N, double *__restrict__ a) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  int j = blockIdx.y * blockDim.y + threadIdx.y;
  if (i >= N || j >= N || j <= i) return;
  const size_t u = i + (size_t)j * N, l = j + (size_t)i * N;
  const double v = 0.5 * (a[u] + a[l]);
  a[u] = v;
  a[l] = v;
}

}  // namespace

namespace gc {

std::vector<int> coalesced_pair_order(const int *indn, int ndimx) {
  if (!indn || ndimx <= 0) return {};
  std::vector<int> idx(ndimx);
  std::iota(idx.begin(), idx.end(), 0);
  std::stable_sort(idx.begin(), idx.end(), [&](int a, int b) {
    const int qa = indn[2 * a + 1], qb = indn[2 * b + 1];
    return qa != qb ? qa < qb : indn[2 * a] < indn[2 * b];
  });
  std::vector<int> out(2 * (size_t)ndimx);
  for (int k = 0; k < ndimx; ++k) {
    out[2 * k] = indn[2 * idx[k]];
    out[2 * k + 1] = indn[2 * idx[k] + 1];
  }
  return out;
}

int rotate_h(gc_context *ctx, SysDev &sd, const double *ure_host) {
  // HNO = URe . h . URe^T, then sq_symmetrize (abfofo.f90:97-100)
  const int n = sd.n;
  DevBuf<double> u, w;
  GC_TRY(u.upload(ctx, ure_host, (size_t)n * n));
  GC_TRY(w.alloc(ctx, (size_t)n * n));
  const double one = 1.0, zero = 0.0;
  GC_CUBLAS(ctx, cublasDgemm(ctx->cublas, CUBLAS_OP_N, CUBLAS_OP_N, n, n, n, &one, u.p, n, sd.h.p, n,
                             &zero, w.p, n));
  GC_CUBLAS(ctx, cublasDgemm(ctx->cublas, CUBLAS_OP_N, CUBLAS_OP_T, n, n, n, &one, w.p, n, u.p, n,
                             &zero, sd.h.p, n));
  dim3 bs(32, 8), gs(ceil_div(n, 32), ceil_div(n, 8));
  k_sym_avg<<<gs, bs, 0, ctx->stream>>>(n, sd.h.p);
  GC_LAUNCHED(ctx);
  return GC_OK;
}

int set_error(gc_context *ctx, int code, const char *fmt, ...) {
  if (ctx) {
    char buf[512];
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(buf, sizeof buf, fmt, ap);
    va_end(ap);
    ctx->err = buf;
  }
  return code;
}

int sys_upload(gc_context *ctx, SysDev &sd, int nbas, int ninact, int nact, int ndimx,
               const double *occ, const double *xone, const int *indn, const double *rdm2act) {
  if (nbas <= 0 || ninact < 0 || nact < 0 || ninact + nact > nbas || ndimx <= 0 || !occ ||
      !indn || (!rdm2act && nact > 0))
    return set_error(ctx, GC_EINVAL, "system: bad arguments nbas=%d ninact=%d nact=%d ndimx=%d",
                     nbas, ninact, nact, ndimx);
  const int n = nbas, nocc = ninact + nact;
  auto finite = [](const double *x, size_t cnt) {
    for (size_t i = 0; i < cnt; ++i)
      if (!std::isfinite(x[i])) return false;
    return true;
  };
  if (!finite(occ, n) || (xone && !finite(xone, (size_t)n * (n + 1) / 2)) ||
      (nact > 0 && !finite(rdm2act, (size_t)nact * nact * (nact * nact + 1) / 2)))
    return set_error(ctx, GC_ENONFINITE,
                     "system: non-finite value in the occupations, one-electron integrals or 2-RDM");
  sd.n = n;
  sd.nin = ninact;
  sd.nact = nact;
  sd.nocc = nocc;
  sd.ndimx = ndimx;
  std::vector<int> grp(n), pp(ndimx), pq(ndimx);
  for (int i = 0; i < n; ++i) grp[i] = i < ninact ? 0 : (i < nocc ? 1 : 2);
  for (int i = 0; i < ndimx; ++i) {
    int a = indn[2 * i] - 1, b = indn[2 * i + 1] - 1;
    if (a < 0 || b < 0 || a >= n || b >= n || a <= b || b >= nocc)
      return set_error(ctx, GC_EINVAL, "system: pair %d = (%d,%d) is not a p>q pair with q occupied",
                       i + 1, a + 1, b + 1);
    pp[i] = a;
    pq[i] = b;
  }
  GC_TRY(sd.occ.upload(ctx, occ, n));
  GC_TRY(sd.grp.upload(ctx, grp.data(), n));
  GC_TRY(sd.pair_p.upload(ctx, pp.data(), ndimx));
  GC_TRY(sd.pair_q.upload(ctx, pq.data(), ndimx));
  {
    auto cicoef = [](double o) { return o >= 0.5 ? std::sqrt(o) : -std::sqrt(o); };
    std::vector<double> cpl(ndimx), cmi(ndimx), rpl(ndimx), rmi(ndimx), dnq(ndimx);
    for (int i = 0; i < ndimx; ++i) {
      const double cp = cicoef(occ[pp[i]]), cq = cicoef(occ[pq[i]]);
      const double op = occ[pp[i]], oq = occ[pq[i]];
      cpl[i] = cp + cq;
      cmi[i] = cp - cq;
      rpl[i] = cpl[i] != 0.0 ? 1.0 / cpl[i] : 0.0;
      rmi[i] = cmi[i] != 0.0 ? 1.0 / cmi[i] : 0.0;
      dnq[i] = op * (1.0 - oq) + oq * (1.0 - op);
    }
    GC_TRY(sd.cpl.upload(ctx, cpl.data(), ndimx));
    GC_TRY(sd.cmi.upload(ctx, cmi.data(), ndimx));
    GC_TRY(sd.rpl.upload(ctx, rpl.data(), ndimx));
    GC_TRY(sd.rmi.upload(ctx, rmi.data(), ndimx));
    GC_TRY(sd.dnq.upload(ctx, dnq.data(), ndimx));
  }
  if (xone) {
    std::vector<double> h((size_t)n * n);
    size_t t = 0;
    for (int q = 0; q < n; ++q)
      for (int p = 0; p <= q; ++p, ++t) {
        h[p + (size_t)q * n] = xone[t];
        h[q + (size_t)p * n] = xone[t];
      }
    GC_TRY(sd.h.upload(ctx, h.data(), h.size()));
  }
  // RDM2val(i,j,k,l) = FRDM2(i,k,j,l) (abfofo.f90:84-92, interpa.f:5244-5272)
  std::vector<double> rv((size_t)nocc * nocc * nocc * nocc, 0.0);
  auto frdm2 = [&](int ip, int iq, int ir, int is) -> double {
    double r = 0.0;
    if (ip == ir && iq == is && (occ[ip] == 1.0 || occ[iq] == 1.0)) r += 2.0 * occ[ip] * occ[iq];
    if (ip == is && iq == ir && (occ[ip] == 1.0 || occ[iq] == 1.0)) r -= occ[ip] * occ[iq];
    if (ip >= ninact && iq >= ninact && ir >= ninact && is >= ninact) {
      long long i12 = (long long)(ip - ninact) * nact + (iq - ninact) + 1;
      long long i34 = (long long)(ir - ninact) * nact + (is - ninact) + 1;
      long long mx = i12 > i34 ? i12 : i34, mn = i12 > i34 ? i34 : i12;
      r = rdm2act[mx * (mx - 1) / 2 + mn - 1];
    }
    return r;
  };
  for (int l = 0; l < nocc; ++l)
    for (int k = 0; k < nocc; ++k)
      for (int j = 0; j < nocc; ++j)
        for (int i = 0; i < nocc; ++i)
          rv[i + (size_t)nocc * (j + (size_t)nocc * (k + (size_t)nocc * l))] = frdm2(i, k, j, l);
  GC_TRY(sd.rv.upload(ctx, rv.data(), rv.size()));
  return GC_OK;
}

// Intermediates that depend only on the system, cached per assembly call set.
struct ZBufs {
  DevBuf<double> z1, z4, z7, z5, z6, z8, z9, z10, z13, z11, z12;
};

static int build_z(gc_context *ctx, const SysDev &sd, const double *ffoo, const double *fofo,
                   ZBufs &Zb) {
  Geo g{sd.n, sd.nin, sd.nact, sd.nocc};
  size_t na2 = (size_t)sd.nact * sd.nact;
  size_t s1 = (size_t)sd.n * sd.nocc * na2, s4 = (size_t)sd.n * sd.n * na2,
         s8 = (size_t)sd.nocc * sd.nocc * na2;
  size_t one = 1;
  GC_TRY(Zb.z1.alloc(ctx, std::max(s1, one)));
  GC_TRY(Zb.z4.alloc(ctx, std::max(s4, one)));
  GC_TRY(Zb.z7.alloc(ctx, std::max(s4, one)));
  GC_TRY(Zb.z5.alloc(ctx, std::max(s1, one)));
  GC_TRY(Zb.z6.alloc(ctx, std::max(s1, one)));
  GC_TRY(Zb.z8.alloc(ctx, std::max(s8, one)));
  GC_TRY(Zb.z9.alloc(ctx, std::max(s4, one)));
  GC_TRY(Zb.z10.alloc(ctx, std::max(s8, one)));
  GC_TRY(Zb.z13.alloc(ctx, std::max(s8, one)));
  GC_TRY(Zb.z11.alloc(ctx, std::max(s1, one)));
  GC_TRY(Zb.z12.alloc(ctx, std::max(s1, one)));
  if (sd.nact == 0) return GC_OK;
  auto grid = [](size_t total) { return std::min<unsigned>(ceil_div(total, 256), 152u * 64u); };
  k_z1<<<grid(s1), 256, 0, ctx->stream>>>(g, fofo, sd.rv.p, Zb.z1.p);
  GC_LAUNCHED(ctx);
  k_z47<<<grid(s4), 256, 0, ctx->stream>>>(g, fofo, sd.rv.p, Zb.z4.p, Zb.z7.p);
  GC_LAUNCHED(ctx);
  k_z56<<<grid(s1), 256, 0, ctx->stream>>>(g, fofo, sd.rv.p, Zb.z5.p, Zb.z6.p);
  GC_LAUNCHED(ctx);
  k_z8<<<grid(s8), 256, 0, ctx->stream>>>(g, fofo, sd.rv.p, Zb.z8.p);
  GC_LAUNCHED(ctx);
  k_z9<<<grid(s4), 256, 0, ctx->stream>>>(g, ffoo, sd.rv.p, Zb.z9.p);
  GC_LAUNCHED(ctx);
  k_z1013<<<grid(s8), 256, 0, ctx->stream>>>(g, ffoo, sd.rv.p, Zb.z10.p, Zb.z13.p);
  GC_LAUNCHED(ctx);
  k_z1112<<<grid(s1), 256, 0, ctx->stream>>>(g, ffoo, sd.rv.p, Zb.z11.p, Zb.z12.p);
  GC_LAUNCHED(ctx);
  return GC_OK;
}

int assemble_ab(gc_context *ctx, const SysDev &sd, const double *ffoo, const double *fofo,
                double alpha, double *abplus, double *abmin, double *etot_host, int ab1) {
  PhaseScope ph(ctx, GC_PHASE_ASSEMBLY);
  Geo g{sd.n, sd.nin, sd.nact, sd.nocc, ab1 ? 0.0 : 1.0, ab1 ? 1 : 0};
  const int n = sd.n, N = sd.ndimx;
  ZBufs Zb;
  GC_TRY(build_z(ctx, sd, ffoo, fofo, Zb));
  DevBuf<double> hno, auxi, auxio, wmat;
  GC_TRY(hno.alloc(ctx, (size_t)n * n));
  GC_TRY(auxi.alloc(ctx, (size_t)n * n));
  GC_TRY(auxio.alloc(ctx, (size_t)n * n));
  GC_TRY(wmat.alloc(ctx, (size_t)n * n));
  dim3 b2(16, 16), g2(ceil_div(n, 16), ceil_div(n, 16));
  k_onebody<<<g2, b2, 0, ctx->stream>>>(g, sd.h.p, sd.occ.p, sd.grp.p, fofo, ffoo, alpha, hno.p,
                                        auxi.p, auxio.p);
  GC_LAUNCHED(ctx);
  GC_CUDA(ctx, cudaMemsetAsync(wmat.p, 0, (size_t)n * n * sizeof(double), ctx->stream));
  if (sd.nocc > 0) {
    const int nocc = sd.nocc, K = nocc * nocc * nocc;
    DevBuf<double> fw, rvp;
    GC_TRY(fw.alloc(ctx, (size_t)n * K));
    GC_TRY(rvp.alloc(ctx, (size_t)K * nocc));
    k_pack_wmat_f<<<dim3(ceil_div(n, 128), std::min(K, 65535)), 128, 0, ctx->stream>>>(
        g, sd.grp.p, fofo, alpha, fw.p);
    GC_LAUNCHED(ctx);
    k_pack_wmat_rv<<<std::min<unsigned>(ceil_div((size_t)K * nocc, 256), 152u * 8u), 256, 0,
                     ctx->stream>>>(nocc, sd.rv.p, rvp.p);
    GC_LAUNCHED(ctx);
    const double one = 1.0, zero = 0.0;
    GC_CUBLAS(ctx, cublasDgemm(ctx->cublas, CUBLAS_OP_N, CUBLAS_OP_N, n, nocc, K, &one, fw.p, n,
                               rvp.p, K, &zero, wmat.p, n));
  }
  Zs Z{Zb.z1.p, Zb.z4.p, Zb.z7.p, Zb.z5.p, Zb.z6.p, Zb.z8.p, Zb.z9.p, Zb.z10.p, Zb.z13.p,
       Zb.z11.p, Zb.z12.p};
  dim3 b3(32, 8), g3(ceil_div(N, 32), ceil_div(N, 8));
  k_ab<<<g3, b3, 0, ctx->stream>>>(g, N, sd.pair_p.p, sd.pair_q.p, sd.occ.p, sd.grp.p, fofo, ffoo,
                                   Z, hno.p, auxi.p, auxio.p, wmat.p, alpha, sd.rpl.p, sd.rmi.p,
                                   abplus, abmin);
  GC_LAUNCHED(ctx);
  if (ab1) {  // AB_CAS_FOFO symmetrises the AB1 matrices (sq_symmetrize, abfofo.f90:260-263)
    dim3 bs(32, 8), gs(ceil_div(N, 32), ceil_div(N, 8));
    k_sym_avg<<<gs, bs, 0, ctx->stream>>>(N, abplus);
    GC_LAUNCHED(ctx);
    k_sym_avg<<<gs, bs, 0, ctx->stream>>>(N, abmin);
    GC_LAUNCHED(ctx);
  }
  if (etot_host) {
    const int nb = 120;
    DevBuf<double> part;
    GC_TRY(part.alloc(ctx, nb));
    k_etwo<<<nb, 256, 0, ctx->stream>>>(g, ffoo, sd.rv.p, part.p);
    GC_LAUNCHED(ctx);
    double hpart[nb];
    std::vector<double> occ(n), h((size_t)n * n);
    GC_CUDA(ctx, cudaMemcpyAsync(hpart, part.p, sizeof hpart, cudaMemcpyDeviceToHost, ctx->stream));
    GC_CUDA(ctx, cudaMemcpyAsync(occ.data(), sd.occ.p, n * sizeof(double), cudaMemcpyDeviceToHost,
                                 ctx->stream));
    GC_CUDA(ctx, cudaMemcpyAsync(h.data(), sd.h.p, h.size() * sizeof(double),
                                 cudaMemcpyDeviceToHost, ctx->stream));
    GC_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    double e1 = 0.0, e2 = 0.0;
    for (int i = 0; i < sd.nocc; ++i) e1 += occ[i] * h[i + (size_t)i * n];
    for (int b = 0; b < nb; ++b) e2 += hpart[b];
    *etot_host = 2.0 * e1 + e2;
  }
  return GC_OK;
}

}  // namespace gc

extern "C" int gc_ab_cas_fofo_ex(gc_context *ctx, int nbas, int ninact, int nact, int ndimx,
                                 const double *occ, const double *ure, const double *xone,
                                 const int *indn, const double *rdm2act, const double *ffoo,
                                 const double *fofo, double alpha, int ab1, double *abplus,
                                 double *abmin, double *etot) {
  if (!ctx) return GC_EINVAL;
  if (!xone || !ffoo || !fofo || !abplus || !abmin)
    return gc::set_error(ctx, GC_EINVAL, "ab_cas_fofo: null pointer");
  if (ure)
    for (size_t i = 0; i < (size_t)nbas * nbas; ++i)
      if (!std::isfinite(ure[i]))
        return gc::set_error(ctx, GC_ENONFINITE, "ab_cas_fofo: non-finite value in URe");
  gc::SysDev sd;
  GC_TRY(gc::sys_upload(ctx, sd, nbas, ninact, nact, ndimx, occ, xone, indn, rdm2act));
  if (ure) GC_TRY(gc::rotate_h(ctx, sd, ure));
  GC_TRY(gc::assemble_ab(ctx, sd, ffoo, fofo, alpha, abplus, abmin, etot, ab1 ? 1 : 0));
  return GC_OK;
}

extern "C" int gc_ab_cas_fofo(gc_context *ctx, int nbas, int ninact, int nact, int ndimx,
                              const double *occ, const double *xone, const int *indn,
                              const double *rdm2act, const double *ffoo, const double *fofo,
                              double alpha, double *abplus, double *abmin, double *etot) {
  return gc_ab_cas_fofo_ex(ctx, nbas, ninact, nact, ndimx, occ, nullptr, xone, indn, rdm2act, ffoo,
                           fofo, alpha, 0, abplus, abmin, etot);
}
