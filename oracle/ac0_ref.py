"""CPU FP64 restatement of GAMMCOR's AC0-CAS (FOFO) energy.

TEST INFRASTRUCTURE ONLY (the oracle of gc_ac0cas_fofo): only tests/ import
it. Parity status as oracle/ac_cas_ref.py: unpinned against reference-produced
numbers (no Fortran compiler, no regression outputs); pinned by the tests
against the GPU path and by its own consistency checks.

AC0CAS_FOFO (abfofo.f90:1485-1750, dispatched at acfd.f:64-68 for ICASSCF=1,
ITwoEl=3) is the first-order (linearised) adiabatic connection:

1. A+-B at lambda = 0 (ABPM0_FOFO, abfofo.f90:1105-1320, equal to AB_CAS_FOFO at
   ACAlpha = 0) is block diagonal once the pairs are grouped
   (create_AC0_blocks_1/2, abfofo.f90:1374-1484): one block of active-active
   pairs, one per inactive orbital q for the (active, q) pairs, one per virtual
   orbital p for the (p, active) pairs, and the (virtual, inactive) pairs whose
   block is diagonal;
2. each block's ERPA problem is solved by ERPASYMM0 (interpa.f:1496-1650), which
   returns Y, X and omega (pack_Eblock, abfofo.f90:2119-2150); a
   (virtual, inactive) pair has omega = A+(ii,ii) and Y = X = 1/sqrt(2);
3. the AB1 matrices (AB_CAS_FOFO at ACAlpha = 1 with AB1 = .true., the lambda
   derivative) are transformed to the zeroth-order modes, A+ with X and A- with Y
   (abpm_tran, tran.f90:620-729);
4. C = 2 (X^T A+' X - Y^T A-' Y)_ij / (omega_i + omega_j), back-transformed with Y
   (ABPM_BACKTRAN, abfofo.f90:2152-2258);
5. ECorr = sum over pairs pq, rs not in one orbital group of
   (C_p + C_q)(C_r + C_s) C[pq, rs] (rs|pq), streaming FOFO (abfofo.f90:1676-1720).
"""
from __future__ import annotations

import numpy as np
import scipy.linalg

from .ac_cas_ref import SMALL_OMEGA2, ab_cas_fofo


def ac0_blocks(indn, nin, nact, n):
    """create_AC0_blocks_1/2 (abfofo.f90:1374-1484): the block order of the pairs.
    Returns (blocks, iv): blocks = list of arrays of 0-based pair indices (AA, then
    AI for q = 1..nin, then AV for p = nocc+1..n; empty blocks dropped), iv = the
    (virtual, inactive) pair indices."""
    nocc = nin + nact

    def grp(i):  # IGem - 1 for 0-based orbital i
        return 0 if i < nin else (1 if i < nocc else 2)

    aa, ai, av, iv = [], {q: [] for q in range(nin)}, {p: [] for p in range(nocc, n)}, []
    for i, (p1, q1) in enumerate(indn):
        p, q = p1 - 1, q1 - 1
        gp, gq = grp(p), grp(q)
        if gp == 1 and gq == 1:
            aa.append(i)
        elif gp == 1 and gq == 0:
            ai[q].append(i)
        elif gp == 2 and gq == 1:
            av[p].append(i)
        elif gp == 2 and gq == 0:
            iv.append(i)
    blocks = [np.array(aa)] if aa else []
    blocks += [np.array(ai[q]) for q in range(nin) if ai[q]]
    blocks += [np.array(av[p]) for p in range(nocc, n) if av[p]]
    return blocks, np.array(iv, dtype=np.int64)


def erpasymm0(abp, abm):
    """ERPASYMM0 (interpa.f:1496-1650): (Y, X, Eig) of one block; Y = X = 0 and
    Eig = omega^2 for omega^2 <= Small."""
    ap = 0.5 * (abp + abp.T)
    am = 0.5 * (abm + abm.T)
    e, V = scipy.linalg.eigh(ap, driver="evd")
    P = (V * np.sqrt(np.abs(e))[None, :]) @ V.T
    P = 0.5 * (P + P.T)
    w2, Z = scipy.linalg.eigh(P @ (am @ P), driver="evd")
    Y = P @ Z
    eig = w2.copy()
    X = np.zeros_like(Y)
    for nu in range(len(eig)):
        if eig[nu] > SMALL_OMEGA2:
            eig[nu] = np.sqrt(eig[nu])
            s = 2.0 / eig[nu] * (Y[:, nu] @ am @ Y[:, nu])
            Y[:, nu] *= 1.0 / np.sqrt(s) if s > 0 else 0.0
            X[:, nu] = am @ Y[:, nu] / eig[nu]
        else:
            Y[:, nu] = 0.0
    return Y, X, eig


def ac0cas_fofo(occ, xone, ure, indn, nin, nact, ffoo, fofo, rdm2act):
    """AC0CAS_FOFO (abfofo.f90:1485-1750). Returns (ECorr, ETot)."""
    n = occ.shape[0]
    nocc = nin + nact
    N = indn.shape[0]
    a0p, a0m, etot = ab_cas_fofo(occ, xone, ure, indn, nin, nact, ffoo, fofo, rdm2act, 0.0)
    a1p, a1m, _ = ab_cas_fofo(occ, xone, ure, indn, nin, nact, ffoo, fofo, rdm2act, 1.0, ab1=True)
    blocks, iv = ac0_blocks(indn, nin, nact, n)
    order = np.concatenate(blocks + [iv]).astype(np.int64)   # block position -> pair index
    assert sorted(order) == list(range(N))
    # block-diagonal Y and X in block order; omega per block position
    Ybd = np.zeros((N, N))
    Xbd = np.zeros((N, N))
    eig = np.zeros(N)
    pos = 0
    for b in blocks:
        m = len(b)
        Y, X, e = erpasymm0(a0p[np.ix_(b, b)], a0m[np.ix_(b, b)])
        Ybd[pos:pos + m, pos:pos + m] = Y
        Xbd[pos:pos + m, pos:pos + m] = X
        eig[pos:pos + m] = e
        pos += m
    fac = 1.0 / np.sqrt(2.0)
    for i in iv:
        Ybd[pos, pos] = Xbd[pos, pos] = fac
        eig[pos] = a0p[i, i]
        pos += 1
    # abpm_tran: A+' with X, A-' with Y, in block order (IV-IV entries carry fac^2 = 1/2)
    bp = Xbd.T @ a1p[np.ix_(order, order)] @ Xbd
    bm = Ybd.T @ a1m[np.ix_(order, order)] @ Ybd
    work = np.zeros((N, N))
    nz = eig != 0.0
    den = eig[:, None] + eig[None, :]
    m2 = nz[:, None] & nz[None, :]
    work[m2] = 2.0 * (bp[m2] - bm[m2]) / den[m2]
    # ABPM_BACKTRAN, then back to pair order
    cb = Ybd @ work @ Ybd.T
    cmat = np.zeros((N, N))
    cmat[np.ix_(order, order)] = cb
    # energy loop (abfofo.f90:1676-1720)
    g = np.where(np.arange(n) < nin, 0, np.where(np.arange(n) < nocc, 1, 2))
    C = np.sign(occ - 0.5) * np.sqrt(occ)
    C[occ - 0.5 == 0] = np.sqrt(occ[occ - 0.5 == 0])
    p, q = indn[:, 0] - 1, indn[:, 1] - 1
    ints = fofo[(p + q * n)[None, :], (p + q * n)[:, None]]   # [ipq, irs] = (rs|pq)
    cc = (C[p] + C[q])[:, None] * (C[p] + C[q])[None, :]
    same = (g[p][:, None] == g[q][:, None]) & (g[q][:, None] == g[p][None, :]) & \
           (g[p][None, :] == g[q][None, :])
    ecorr = float(np.sum(np.where(same, 0.0, cc * cmat * ints)))
    return ecorr, etot
