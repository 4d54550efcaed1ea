"""Multi-threaded CPU FP64 port of the reference AC-CAS (FOFO) algorithm.

TEST AND BENCHMARK INFRASTRUCTURE ONLY. bench.py times it as the CPU baseline
(its `--impl reference` arm and the `cpu_baseline` field); tests/ check it
against the line-faithful oracle (oracle/ac_cas_ref.py). The product path
never calls it.

It computes what ACECORR (acfd.f:117-209) computes, with the reference's
algorithm at every lambda point -- A+-B reassembled (AB_CAS_FOFO,
abfofo.f90:8-293), ERPASYMM1 with two dsyevd calls (interpa.f:1652-1781) and
the integrand (ACEneERPA_FOFO, abfofo.f90:3791-3927) -- but with every part in
a multi-threaded form so that the host cores are used the way the reference's
MKL build uses them:

* the FOFO/FFOO transform from the ERI factor as BLAS-3 products (numpy);
* the A+-B elements and the masked integral matrix of the integrand as OpenMP
  loops in C (oracle/cpu_port.c, compiled here with gcc);
* the two dsyevd of ERPASYMM1 and its products through scipy/numpy (LAPACK and
  BLAS, threaded);
* the integrand's N^2 dot products of length N as one GEMM.

Every product goes through scipy's BLAS (scipy.linalg.blas.dgemm), the same
library as its LAPACK: numpy and scipy ship separate OpenBLAS builds, and two
thread pools taking turns on the same cores ran the products 5-10x slower.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess
from pathlib import Path

import numpy as np
import scipy.linalg
from scipy.linalg.blas import dgemm

from . import ac_cas_ref as R

HERE = Path(__file__).resolve().parent
SRC = HERE / "cpu_port.c"
LIB = HERE / "libcpu_port.so"
_lib = None


def build(force: bool = False) -> Path:
    """Compile oracle/cpu_port.c with gcc (OpenMP, -O3, portable flags)."""
    if force or not LIB.exists() or LIB.stat().st_mtime < SRC.stat().st_mtime:
        tmp = LIB.with_suffix(".so.tmp")
        subprocess.run(["gcc", "-O3", "-fopenmp", "-fPIC", "-shared", "-o", str(tmp), str(SRC),
                        "-lm"], check=True)
        os.replace(tmp, LIB)
    return LIB


def load():
    global _lib
    if _lib is None:
        build()
        lib = C.CDLL(str(LIB))
        dp, ip = C.POINTER(C.c_double), C.POINTER(C.c_int)
        lib.cpu_ab_cas_fofo.restype = C.c_int
        lib.cpu_ab_cas_fofo.argtypes = [C.c_int, C.c_int, C.c_int, C.c_int, dp, dp, ip, ip, dp,
                                        dp, dp, C.c_double, dp, dp, dp]
        lib.cpu_integrand_kt.restype = None
        lib.cpu_integrand_kt.argtypes = [C.c_int, C.c_int, C.c_int, C.c_int, dp, ip, ip, dp, dp,
                                         dp]
        _lib = lib
    return _lib


def _d(a):
    return a.ctypes.data_as(C.POINTER(C.c_double))


def _i(a):
    return a.ctypes.data_as(C.POINTER(C.c_int))


def transform_factored(cmo: np.ndarray, lfac: np.ndarray, nin: int, nact: int, chunk: int = 64):
    """FOFO and FFOO (tran4_gen's record layout, tran.f90:313-423) from the ERI factor:
    (pq|rs) = sum_P L[pq,P] L[rs,P], so each block is a product B^T B' of the
    factor's transformed columns. Returns (ffoo, fofo) as [record, element]."""
    from gammcor_gb300.synth import unpack_sym
    n = cmo.shape[0]
    nocc = nin + nact
    rank = lfac.shape[1]
    cf = np.asfortranarray(cmo)
    Bfo = np.empty((rank, n * nocc))
    Dff = np.empty((rank, n * n))
    Eoo = np.empty((rank, nocc * nocc))
    for p0 in range(0, rank, chunk):
        Lp = unpack_sym(np.ascontiguousarray(lfac[:, p0:p0 + chunk].T), n)  # (c, n, n)
        c = Lp.shape[0]
        X = dgemm(1.0, Lp.reshape(c * n, n), cf)                # X[(P, mu), b] = (L_P C)[mu, b]
        Xt = np.asfortranarray(X.reshape(c, n, n).transpose(1, 0, 2).reshape(n, c * n))
        F = dgemm(1.0, cf, Xt, trans_a=True)                    # F[a, (P, b)] = (C^T L_P C)[a, b]
        full = F.reshape(n, c, n).transpose(1, 2, 0)            # [P, b, a]
        Dff[p0:p0 + c] = full.reshape(c, -1)                    # element a + b n
        Bfo[p0:p0 + c] = full[:, :nocc, :].reshape(c, -1)       # a + b n, b < nocc
        Eoo[p0:p0 + c] = full[:, :nocc, :nocc].reshape(c, -1)
    fofo = dgemm(1.0, Bfo, Bfo, trans_a=True)   # [record (k,l), element (i,j)] = sum_P B_P(k,l) B_P(i,j)
    ffoo = dgemm(1.0, Eoo, Dff, trans_a=True)   # [record (k,l) occupied, element (i,j)]
    return np.ascontiguousarray(ffoo), np.ascontiguousarray(fofo)


def ab_cas_fofo(occ, xone, indn, nin, nact, ffoo, fofo, rdm2act, alpha):
    """AB_CAS_FOFO (abfofo.f90:8-293) through the OpenMP element port.
    Returns (ABPLUS, ABMIN, ETot) with ABPLUS[ipq, irs], as the oracle."""
    lib = load()
    n = occ.shape[0]
    N = indn.shape[0]
    pp = np.ascontiguousarray(indn[:, 0] - 1, dtype=np.int32)
    pq = np.ascontiguousarray(indn[:, 1] - 1, dtype=np.int32)
    abp = np.empty((N, N), order="F")
    abm = np.empty((N, N), order="F")
    et = np.zeros(1)
    rc = lib.cpu_ab_cas_fofo(n, nin, nact, N, _d(np.ascontiguousarray(occ, dtype=np.float64)),
                             _d(np.ascontiguousarray(xone, dtype=np.float64)), _i(pp), _i(pq),
                             _d(np.ascontiguousarray(rdm2act, dtype=np.float64)),
                             _d(np.ascontiguousarray(ffoo)), _d(np.ascontiguousarray(fofo)),
                             float(alpha), _d(abp), _d(abm), _d(et))
    if rc != 0:
        raise MemoryError("cpu_ab_cas_fofo: allocation failed")
    return abp, abm, float(et[0])


def integrand_matrix(occ, indn, nin, nact, fofo):
    """(Kt, diag): W = 2 sum(Yk * (Kt @ Yk)) + sum(diag) (ACEneERPA_FOFO, abfofo.f90:3791-3927)."""
    lib = load()
    n = occ.shape[0]
    N = indn.shape[0]
    pp = np.ascontiguousarray(indn[:, 0] - 1, dtype=np.int32)
    pq = np.ascontiguousarray(indn[:, 1] - 1, dtype=np.int32)
    kt = np.empty((N, N), order="F")
    diag = np.empty(N)
    lib.cpu_integrand_kt(n, nin, nact, N, _d(np.ascontiguousarray(occ, dtype=np.float64)),
                         _i(pp), _i(pq), _d(np.ascontiguousarray(fofo)), _d(kt), _d(diag))
    return kt, diag


def erpasymm1(abplus, abmin):
    """ERPASYMM1 (interpa.f:1652-1781): symmetrise A+-, A+^1/2 from dsyevd(A+),
    dsyevd(A+^1/2 A- A+^1/2), Y = A+^1/2 Z, normalise 2/omega Y^T A- Y = 1 for
    omega^2 > 1e-6; the normalisation sums of all columns from one product."""
    ap = np.asfortranarray(0.5 * (abplus + abplus.T))
    am = np.asfortranarray(0.5 * (abmin + abmin.T))
    e, V = scipy.linalg.eigh(ap, driver="evd", overwrite_a=True, check_finite=False)
    P = dgemm(1.0, V * np.sqrt(np.abs(e))[None, :], V, trans_b=True)
    P = np.asfortranarray(0.5 * (P + P.T))
    M = dgemm(1.0, P, dgemm(1.0, am, P))
    w2, Z = scipy.linalg.eigh(M, lower=True, driver="evd", overwrite_a=True, check_finite=False)
    Y = dgemm(1.0, P, Z)
    eig = w2.copy()
    pos = eig > R.SMALL_OMEGA2
    eig[pos] = np.sqrt(eig[pos])
    T = dgemm(1.0, am, Y)
    ssum = np.where(pos, 2.0 / np.where(pos, eig, 1.0) * np.einsum("ij,ij->j", Y, T), 0.0)
    f = np.where(ssum > 0, 1.0 / np.sqrt(np.where(ssum > 0, ssum, 1.0)), 0.0)
    Y[:, pos] *= f[pos][None, :]
    return Y, eig


def ac_ene_erpa_fofo(Y, eig, kt, diag):
    """W of ACEneERPA_FOFO from the kept eigenvectors (1e-3 < omega < 1e8, abfofo.f90:3808)."""
    keep = (eig > R.SMALL_E) & (eig < R.BIG_E)
    Yk = np.asfortranarray(Y[:, keep])
    return float(2.0 * np.einsum("ij,ij->", Yk, dgemm(1.0, kt, Yk)) + diag.sum())


def acecorr(occ, xone, indn, nin, nact, ffoo, fofo, rdm2act, ngrid=5, lambdas=None,
            weights=None):
    """ACECORR (acfd.f:117-209) with the reference's per-point algorithm: A+-B
    reassembled at every lambda, ERPASYMM1 (two dsyevd), the integrand. Returns
    (E_CAS, ECorr, [W_i])."""
    if lambdas is None:
        x, w = R.gauleg(0.0, 1.0, ngrid)
    else:
        x, w = np.asarray(lambdas), np.asarray(weights)
    kt, diag = integrand_matrix(occ, indn, nin, nact, fofo)
    ws, ecas = [], None
    for lam in x:
        abp, abm, ecas = ab_cas_fofo(occ, xone, indn, nin, nact, ffoo, fofo, rdm2act, lam)
        Y, eig = erpasymm1(abp, abm)
        ws.append(ac_ene_erpa_fofo(Y, eig, kt, diag))
    return ecas, float(np.dot(w, ws)), ws


def energy_of_system(s, ngrid=8):
    """AC-CAS energy of one synthetic system from its ERI factor and MO coefficients."""
    indn = R.pair_space(s.occ, s.nele)
    ffoo, fofo = transform_factored(s.cmo, s.lfac, s.nin, s.nact)
    return acecorr(s.occ, s.xone, indn, s.nin, s.nact, ffoo, fofo, s.rdm2act, ngrid=ngrid)
