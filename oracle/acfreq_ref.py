"""CPU FP64 restatement of GAMMCOR's frequency-integration AC (ACFREQ, FOFO).

TEST INFRASTRUCTURE ONLY (the oracle of gc_ac_freq_fofo): only tests/ import
it. Parity status as oracle/ac_cas_ref.py: unpinned against reference-produced
numbers.

WIter_FOFO (ac_fofo.f90:1-181, called by ACIter, ac_iter.f:44-48, for
ITwoEl = 3) integrates the lambda-dependent response over imaginary
frequency. A+-B(lambda) = A+-0 + lambda A+-1 (AB_CAS_FOFO at ACAlpha = 0 and 1,
the difference taken as the lambda slope) and, with
A0 = A+0 A-0, A1 = A+0 A-1 + A+1 A-0, A2 = A+1 A-1, the Taylor coefficients in
lambda of C(lambda, omega) = 1/2 (A(lambda) + omega^2)^-1 A+(lambda) are
    C0 = 1/2 inv A+0,  C1 = 1/2 inv A+1 - inv A1 C0,
    Cn = -n inv A1 C(n-1) - n (n-1) inv A2 C(n-2)      (n = 2 .. Max_Cn = 3)
with inv = (A0 + omega^2)^-1 (dgetrf/dgetri at every frequency). The lambda
integral of the series and the frequency quadrature (FreqGrid, ac_iter.f:414-429:
Gauss-Legendre on [-1, 1] mapped to [0, inf) with x0 = 1/2, NGrid = 25) give
    COM = sum_omega 4/pi w_omega [C0 + C1/2 + sum_n Cn / (n! (n + 1))],
and the energy is the integrand's contraction of COM with FOFO (ac_fofo.f90:127-181):
    ECorr = sum_{pq, rs not in one group} [(C_p + C_q)(C_r + C_s) COM[pq, rs]
            - delta_{pq,rs} (n_p (1 - n_q) + n_q (1 - n_p))] (rs|pq).
"""
from __future__ import annotations

import numpy as np

from .ac_cas_ref import ab_cas_fofo, gauleg


def freq_grid(nfreq: int):
    """FreqGrid (ac_iter.f:414-429)."""
    x, w = gauleg(-1.0, 1.0, nfreq)
    x0 = 0.5
    wf = 2.0 * x0 * w / (1.0 - x) ** 2
    xf = x0 * (1.0 + x) / (1.0 - x)
    return xf, wf


def com_matrix(abp0, abm0, abp1, abm1, ngrid=25, max_cn=3):
    """The frequency-integrated COM of WIter_FOFO (ac_fofo.f90:55-119)."""
    N = abp0.shape[0]
    A0 = abp0 @ abm0
    A1 = abp0 @ abm1 + abp1 @ abm0
    A2 = abp1 @ abm1
    xf, wf = freq_grid(ngrid)
    COM = np.zeros((N, N))
    for om, wt in zip(xf, wf):
        inv = np.linalg.inv(A0 + om ** 2 * np.eye(N))
        C0 = 0.5 * inv @ abp0
        work0 = inv @ A1                    # "LAMBDA*A1"
        C1 = 0.5 * inv @ abp1 - work0 @ C0
        work1 = inv @ A2                    # "LAMBDA*A2"
        wfact = 4.0 / np.pi * wt
        COM += wfact * (C0 + 0.5 * C1)
        fact = 1.0
        for n in range(2, max_cn + 1):
            fact *= n
            C2 = -n * (work0 @ C1) - n * (n - 1) * (work1 @ C0)
            COM += wfact / fact / (n + 1) * C2
            C0, C1 = C1, C2
    return COM


def witer_fofo(occ, xone, ure, indn, nin, nact, ffoo, fofo, rdm2act, ngrid=25, max_cn=3):
    """WIter_FOFO (ac_fofo.f90:1-181). Returns (ECorr, ECASSCF)."""
    n = occ.shape[0]
    nocc = nin + nact
    abp0, abm0, ecas = ab_cas_fofo(occ, xone, ure, indn, nin, nact, ffoo, fofo, rdm2act, 0.0)
    abp1, abm1, _ = ab_cas_fofo(occ, xone, ure, indn, nin, nact, ffoo, fofo, rdm2act, 1.0)
    COM = com_matrix(abp0, abm0, abp1 - abp0, abm1 - abm0, ngrid, max_cn)
    g = np.where(np.arange(n) < nin, 0, np.where(np.arange(n) < nocc, 1, 2))
    C = np.sign(occ - 0.5) * np.sqrt(occ)
    C[occ - 0.5 == 0] = np.sqrt(occ[occ - 0.5 == 0])
    p, q = indn[:, 0] - 1, indn[:, 1] - 1
    ints = fofo[(p + q * n)[None, :], (p + q * n)[:, None]]   # [ipq, irs] = (rs|pq)
    cc = (C[p] + C[q])[:, None] * (C[p] + C[q])[None, :]
    same = (g[p][:, None] == g[q][:, None]) & (g[q][:, None] == g[p][None, :]) & \
           (g[p][None, :] == g[q][None, :])
    aux = cc * COM
    aux[np.diag_indices_from(aux)] -= occ[p] * (1.0 - occ[q]) + occ[q] * (1.0 - occ[p])
    ecorr = float(np.sum(np.where(same, 0.0, aux * ints)))
    return ecorr, ecas
