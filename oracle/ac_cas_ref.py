"""CPU FP64 restatement of GAMMCOR's AC-CAS (FOFO) path.

TEST INFRASTRUCTURE ONLY. This module is the oracle the CUDA path is checked
against: only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline and
reference legs may import it. The product path never calls it.

Parity status: UNPINNED against reference-produced numbers. The reference is
Fortran + MKL and cannot be compiled where this project is built (no Fortran
compiler), and its regression outputs (TESTS/AC/TEST1/gammcor.out) are not
distributed. The restatement is pinned instead by self-consistency checks in
tests/: E_CAS from the assembly equals the CI energy of the generator; A+-B is
affine in lambda; the ERPA residual and normalisation hold; FOFO/FFOO equal a
dense einsum transform; A+-B and W(lambda) equal an independent restatement of
the in-core formulas (oracle/incore_ref.py); Gauss-Legendre nodes equal
numpy's leggauss.

Each function follows the reference routine named in its docstring, keeping
the loop structure, pair order, masks, thresholds and the 2-RDM convention;
innermost loops are vectorised with numpy where that does not change what is
summed. Arrays use Fortran index meaning with 0-based offsets: A[i, j] is
A(i+1, j+1) of the reference.
"""
from __future__ import annotations

import numpy as np
import scipy.linalg

THR_SEL_ACT = 1e-8     # ThrSelAct default (systemdef.f90)
THR_QVIRT = 1e-7       # ThrQVirt default
SMALL_OMEGA2 = 1e-6    # interpa.f:1664 Small
SMALL_E, BIG_E = 1e-3, 1e8   # abfofo.f90:3808


# ----------------------------------------------------------------- helpers
def triang_to_sq(mat_tr: np.ndarray, n: int) -> np.ndarray:
    """tran.f90:1221-1247 for a batch (..., ntr) -> (..., n, n) [p, q]."""
    p, q = [], []
    for qq in range(n):
        for pp in range(qq + 1):
            p.append(pp)
            q.append(qq)
    out = np.zeros(mat_tr.shape[:-1] + (n, n))
    out[..., p, q] = mat_tr
    out[..., q, p] = mat_tr
    return out


def gauleg(x1: float, x2: float, n: int):
    """misc.f:828-865 (Numerical Recipes gauleg, EPS = 3e-14)."""
    x = np.zeros(n)
    w = np.zeros(n)
    m = (n + 1) // 2
    xm = 0.5 * (x2 + x1)
    xl = 0.5 * (x2 - x1)
    for i in range(1, m + 1):
        z = np.cos(3.141592654 * (i - 0.25) / (n + 0.5))
        while True:
            p1, p2 = 1.0, 0.0
            for j in range(1, n + 1):
                p3 = p2
                p2 = p1
                p1 = ((2.0 * j - 1.0) * z * p2 - (j - 1.0) * p3) / j
            pp = n * (z * p1 - p2) / (z * z - 1.0)
            z1 = z
            z = z1 - p1 / pp
            if not abs(z - z1) > 3e-14:
                break
        x[i - 1] = xm - xl * z
        x[n - i] = xm + xl * z
        w[i - 1] = 2.0 * xl / ((1.0 - z * z) * pp * pp)
        w[n - i] = w[i - 1]
    return x, w


def ind_aux(occ: np.ndarray, nele: int) -> np.ndarray:
    """IndAux of accas.f:30-44: 0 below NELE, 2 above, 1 for 0<Occ<1."""
    n = occ.shape[0]
    aux = np.where(np.arange(1, n + 1) <= nele, 0, 2)
    aux[(occ < 1.0) & (occ != 0.0)] = 1
    return aux


def prepare_nums(occ: np.ndarray, nele: int):
    """initia.f:2996-3035 -> (Num0, Num1)."""
    aux = ind_aux(occ, nele)
    n = occ.shape[0]
    num0 = 0
    for i in range(n):
        if aux[i] != 0:
            break
        num0 += 1
    num2 = 0
    for i in range(n - 1, -1, -1):
        if aux[i] != 2:
            break
        num2 += 1
    return num0, n - num0 - num2


def pair_space(occ: np.ndarray, nele: int, ifl_core: int = 1,
               thr_sel_act: float = THR_SEL_ACT, thr_qvirt: float = THR_QVIRT):
    """accas.f:54-99. Returns IndN as (NDimX, 2) 1-based, loop order I outer."""
    aux = ind_aux(occ, nele)
    n = occ.shape[0]
    pairs = []
    for I in range(1, n + 1):
        for J in range(1, I):
            a = aux[I - 1] + aux[J - 1]
            if a == 0 or a == 4:
                continue
            oi, oj = occ[I - 1], occ[J - 1]
            if aux[I - 1] == 1 and aux[J - 1] == 1 and abs(oi - oj) / oi < thr_sel_act:
                continue
            if ifl_core == 1 or (oi != 1.0 and oj != 1.0):
                if abs(oi + oj - 2.0) > 1e-10 and abs(oi + oj) > thr_qvirt:
                    pairs.append((I, J))
    return np.array(pairs, dtype=np.int64).reshape(-1, 2)


def naddr_rdm(i1, i2, i3, i4, nact):
    """interpa.f:4529-4541 (1-based)."""
    i12 = (i1 - 1) * nact + i2
    i34 = (i3 - 1) * nact + i4
    mx = max(i12, i34)
    mn = min(i12, i34)
    return mx * (mx - 1) // 2 + mn


def frdm2(ip, iq, ir, is_, rdm2act, occ, ind2, nact):
    """interpa.f:5244-5272 (1-based orbital indices)."""
    r = 0.0
    if ip == ir and iq == is_ and (occ[ip - 1] == 1.0 or occ[iq - 1] == 1.0):
        r += 2.0 * occ[ip - 1] * occ[iq - 1]
    if ip == is_ and iq == ir and (occ[ip - 1] == 1.0 or occ[iq - 1] == 1.0):
        r -= occ[ip - 1] * occ[iq - 1]
    if ind2[ip - 1] * ind2[iq - 1] * ind2[ir - 1] * ind2[is_ - 1] != 0:
        r = rdm2act[naddr_rdm(ind2[ip - 1], ind2[iq - 1], ind2[ir - 1], ind2[is_ - 1], nact) - 1]
    return r


def rdm2val(rdm2act, occ, nin, nact):
    """RDM2val(i,j,k,l) = FRDM2(i,k,j,l) over occupied orbitals (abfofo.f90:84-92)."""
    nocc = nin + nact
    ind2 = np.zeros(occ.shape[0], dtype=np.int64)
    ind2[nin:nocc] = np.arange(1, nact + 1)
    out = np.zeros((nocc,) * 4)
    for l in range(1, nocc + 1):
        for k in range(1, nocc + 1):
            for j in range(1, nocc + 1):
                for i in range(1, nocc + 1):
                    out[i - 1, j - 1, k - 1, l - 1] = frdm2(i, k, j, l, rdm2act, occ, ind2, nact)
    return out


# -------------------------------------------------------------- transform
def tran4_gen(nbas, CA, CB, CC, CD, ao_sorted):
    """tran.f90:313-423, in memory.

    ao_sorted: AOTWOSORT records, shape (ntr, ntr); record rs holds (pq|rs)
    for packed pq. CA..CD: AO x MO (nbas x nX). Returns the output file as an
    array (nA*nB, nC*nD): record ab = a + b*nA, element cd = c + d*nC.
    """
    nA, nB, nC, nD = CA.shape[1], CB.shape[1], CC.shape[1], CD.shape[1]
    ntr = nbas * (nbas + 1) // 2
    # phase 1: (ab| for each rs
    work3 = np.empty((ntr, nA * nB))
    for s in range(0, ntr, 512):              # cbuf blocks
        sq = triang_to_sq(ao_sorted[s:s + 512], nbas)     # [rs, p, q]
        w1 = np.matmul(CA.T[None], sq)                      # CA^T . M
        w2 = np.matmul(w1, CB[None])                        # . CB  -> (nA, nB)
        work3[s:s + 512] = w2.transpose(0, 2, 1).reshape(-1, nA * nB)  # column-major a fastest
    # phase 2: |cd) for each ab
    out = np.empty((nA * nB, nC * nD))
    for s in range(0, nA * nB, 256):
        sq = triang_to_sq(work3[:, s:s + 256].T, nbas)      # [ab, r, s]
        w1 = np.matmul(CC.T[None], sq)
        w2 = np.matmul(w1, CD[None])
        out[s:s + 256] = w2.transpose(0, 2, 1).reshape(-1, nC * nD)
    return out


def transform_fofo_ffoo(cmo, ao_sorted, num0, num1):
    """initia.f:1414-1425: FFOO (occ,occ,full,full) and FOFO (full,occ,full,occ)."""
    nbas = cmo.shape[0]
    nocc = num0 + num1
    co = cmo[:, :nocc]
    ffoo = tran4_gen(nbas, co, co, cmo, cmo, ao_sorted)
    fofo = tran4_gen(nbas, cmo, co, cmo, co, ao_sorted)
    return ffoo, fofo


# -------------------------------------------------------------- assembly
def _groups(nbas, nin, nocc):
    g = np.empty(nbas, dtype=np.int64)
    g[:nin] = 0
    g[nin:nocc] = 1
    g[nocc:] = 2
    return g


def ab_cas_fofo(occ, xone, ure, indn, nin, nact, ffoo, fofo, rdm2act, alpha, ab1=False):
    """AB_CAS_FOFO (abfofo.f90:8-293) + JK_loop (abfofo.f90:4468-5053).

    indn: (NDimX, 2) 1-based pairs (IndX(i) = i). ffoo/fofo: arrays in the
    tran4_gen output layout. Returns (ABPLUS, ABMIN, ETot), ABPLUS[ipq, irs].
    """
    nbas = occ.shape[0]
    nocc = nin + nact
    ndimx = indn.shape[0]
    IG = _groups(nbas, nin, nocc)            # IGem - 1
    RV = rdm2val(rdm2act, occ, nin, nact)
    ABP = np.zeros((ndimx, ndimx))
    ABM = np.zeros((ndimx, ndimx))

    work1 = triang_to_sq(xone, nbas)
    HNO = ure @ work1 @ ure.T
    HNO = 0.5 * (HNO + HNO.T)                 # sq_symmetrize
    etot = 2.0 * np.sum(occ[:nocc] * np.diag(HNO)[:nocc])

    same = IG[:, None] == IG[None, :]
    if ab1:
        HNO = np.where(same, 0.0, alpha * HNO)
    else:
        HNO = np.where(same, HNO, alpha * HNO)

    auxind = np.zeros((3, 3), dtype=np.int64)
    auxind[0:2, 0:2] = 1
    auxind[1, 1] = 2
    ac = np.full((3, 3, 3, 3), alpha)
    for g in range(3):
        ac[g, g, g, g] = 0.0 if ab1 else 1.0

    pos = np.zeros((nbas, nbas), dtype=np.int64)
    for i in range(ndimx):
        pos[indn[i, 0] - 1, indn[i, 1] - 1] = i + 1

    AuxI = np.zeros((nbas, nbas))
    AuxIO = np.zeros((nbas, nbas))
    WMAT = np.zeros((nbas, nbas))
    hnocoef = -1.0 if ab1 else 1.0 - alpha
    etot = _jk_loop(ABP, ABM, HNO, AuxI, AuxIO, WMAT, RV, occ, ac, IG, auxind, pos,
                    nin, nocc, nbas, ffoo, fofo, hnocoef, etot)

    C = np.sign(occ - 0.5) * np.sqrt(occ)
    C[occ - 0.5 == 0] = np.sqrt(occ[occ - 0.5 == 0])   # Fortran sign(a, 0) = +|a|

    def aux_pick(gx, gy, xi, yi):
        a = auxind[IG[gx], IG[gy]]
        if a == 1:
            return AuxI[xi, yi]
        if a == 2:
            return AuxIO[xi, yi]
        return 0.0

    for icol in range(ndimx):
        ir, is_ = indn[icol, 0] - 1, indn[icol, 1] - 1
        if ir == is_:
            continue
        for irow in range(ndimx):
            ip, iq = indn[irow, 0] - 1, indn[irow, 1] - 1
            val = 0.0
            if ip == ir:
                val += (occ[ip] - occ[is_]) * HNO[iq, is_] - WMAT[iq, is_]
                val += occ[ip] * aux_pick(ip, ir, iq, is_)
            if iq == is_:
                val += (occ[iq] - occ[ir]) * HNO[ip, ir] - WMAT[ip, ir]
                val += occ[iq] * aux_pick(iq, is_, ip, ir)
            ABP[irow, icol] += val
            ABM[irow, icol] += val
            val = 0.0
            if iq == ir:
                val += (occ[iq] - occ[is_]) * HNO[ip, is_] - WMAT[ip, is_]
                val += occ[iq] * aux_pick(iq, ir, ip, is_)
            if ip == is_:
                val += (occ[ip] - occ[ir]) * HNO[iq, ir] - WMAT[iq, ir]
                val += occ[ip] * aux_pick(ip, is_, iq, ir)
            ABP[irow, icol] += val
            ABM[irow, icol] -= val
            d = (C[ip] + C[iq]) * (C[ir] + C[is_])
            if d != 0.0:
                ABP[irow, icol] /= d
            d = (C[ip] - C[iq]) * (C[ir] - C[is_])
            if d != 0.0:
                ABM[irow, icol] /= d
    if ab1:
        ABP = 0.5 * (ABP + ABP.T)
        ABM = 0.5 * (ABM + ABM.T)
    return ABP, ABM, etot


def _jk_loop(ABP, ABM, HNO, AuxI, AuxIO, WMAT, RV, occ, ac, IG, auxind, pos,
             nin, nocc, nbas, ffoo, fofo, hnocoef, etot):
    """JK_loop (abfofo.f90:4468-5053). Index variables are 0-based here."""
    act = slice(nin, nocc)
    A1 = (auxind == 1)

    def ai(x, y):
        return A1[IG[x], IG[y]]

    def add(ipq, irs, vp, vm):
        ABP[ipq - 1, irs - 1] += vp
        ABM[ipq - 1, irs - 1] += vm

    # ---------------- exchange loop (FO|FO): records kl = kk + ll*nbas
    for ll in range(nocc):
        for kk in range(nbas):
            rec = fofo[kk + ll * nbas]
            ints = np.zeros((nbas, nbas))
            ints[:, :nocc] = rec.reshape(nocc, nbas).T
            k, l = kk, ll
            # one-electron part, exchange
            val = hnocoef * occ[l]
            if IG[l] == 0:
                if IG[k] == 1:
                    HNO[nin:nocc, k] -= val * ints[nin:nocc, l]
                elif IG[k] == 2:
                    HNO[nocc:, k] -= val * ints[nocc:, l]
            if IG[l] == 1:
                if IG[k] == 0:
                    HNO[:nin, k] -= val * ints[:nin, l]
                elif IG[k] == 2:
                    HNO[nocc:, k] -= val * ints[nocc:, l]
            coef = ac[IG, IG, IG[k], IG[l]] * occ[l]
            if l < nin:
                AuxIO[:, k] -= coef * ints[:, l]
            AuxI[:, k] -= coef * ints[:, l]
            # WMAT
            blk = ints[:nocc, :nocc]
            for ir in range(nocc):
                r = RV[:, :, ir, l]
                v = 0.0
                v += ac[IG[k], IG[l], 0, 0] * np.sum(blk[:nin, :nin] * r[:nin, :nin])
                v += ac[IG[k], IG[l], 1, 0] * np.sum(blk[nin:, :nin] * r[nin:, :nin])
                v += ac[IG[k], IG[l], 0, 1] * np.sum(blk[:nin, nin:] * r[:nin, nin:])
                v += ac[IG[k], IG[l], 1, 1] * np.sum(blk[nin:, nin:] * r[nin:, nin:])
                WMAT[k, ir] += v
            # Coulomb
            if k >= nin:
                ir, is_ = k, l
                irs = pos[ir, is_]
                if irs > 0:
                    for iq in range(nocc):
                        for ip in range(nin, nbas):
                            ipq = pos[ip, iq]
                            if ipq > 0:
                                av = ac[IG[ip], IG[iq], IG[ir], IG[is_]]
                                v = 0.0
                                if ai(ip, ir): v += occ[ip] * occ[ir]
                                if ai(iq, is_): v += occ[iq] * occ[is_]
                                if ai(iq, ir): v -= occ[iq] * occ[ir]
                                if ai(ip, is_): v -= occ[ip] * occ[is_]
                                v = 2 * av * v * ints[ip, iq]
                                add(ipq, irs, v, v)
                                v = 0.0
                                if ai(iq, ir): v += occ[iq] * occ[ir]
                                if ai(ip, is_): v += occ[ip] * occ[is_]
                                if ai(ip, ir): v -= occ[ip] * occ[ir]
                                if ai(iq, is_): v -= occ[iq] * occ[is_]
                                v = 2 * av * v * ints[ip, iq]
                                add(ipq, irs, v, -v)
            # exchange
            if k >= nin:
                ip, is_ = k, l
                for ir in range(nin, nbas):
                    irs = pos[ir, is_]
                    if irs > 0:
                        for iq in range(nocc):
                            ipq = pos[ip, iq]
                            if ipq > 0:
                                av = ac[IG[ip], IG[iq], IG[ir], IG[is_]]
                                v = 0.0
                                if ai(iq, ir): v += occ[iq] * occ[ir]
                                if ai(ip, is_): v += occ[ip] * occ[is_]
                                if ai(ip, ir): v -= occ[ip] * occ[ir]
                                if ai(iq, is_): v -= occ[iq] * occ[is_]
                                v = -av * v * ints[ir, iq]
                                add(ipq, irs, v, -v)
            # T1 p->q
            if k >= nin:
                ip, is_ = k, l
                for ir in range(nin, nocc):
                    irs = pos[ir, is_]
                    if irs > 0:
                        for iq in range(nin, nocc):
                            ipq = pos[ip, iq]
                            if ipq > 0:
                                v = ac[IG[ip], IG[is_], 1, 1] * np.sum(RV[act, act, iq, ir] * ints[act, act])
                                add(ipq, irs, v, -v)
            # T3
            if k >= nin:
                iq, ir = l, k
                for is_ in range(nin, nocc):
                    irs = pos[ir, is_]
                    if irs > 0:
                        for ip in range(nin, nocc):
                            ipq = pos[ip, iq]
                            if ipq > 0:
                                v = ac[IG[iq], IG[ir], 1, 1] * np.sum(RV[act, act, ip, is_] * ints[act, act])
                                add(ipq, irs, v, -v)
            # T4 + T6
            if k >= nin and nin <= l < nocc:
                ir, iu = k, l
                for is_ in range(nin, nocc):        # T4
                    irs = pos[ir, is_]
                    if irs > 0:
                        for iq in range(nin, nocc):
                            for ip in range(nin, nbas):
                                ipq = pos[ip, iq]
                                if ipq > 0:
                                    v = ac[IG[ip], IG[ir], IG[iu], 1] * np.sum(RV[act, iq, is_, iu] * ints[ip, act])
                                    add(ipq, irs, v, v)
                for is_ in range(nin, nocc):        # T4 p->q
                    irs = pos[ir, is_]
                    if irs > 0:
                        for iq in range(nocc):
                            for ip in range(nin, nocc):
                                ipq = pos[ip, iq]
                                if ipq > 0:
                                    v = ac[IG[iq], IG[ir], IG[iu], 1] * np.sum(RV[act, ip, is_, iu] * ints[act, iq])
                                    add(ipq, irs, v, -v)
                for is_ in range(nin, nocc):        # T6
                    irs = pos[ir, is_]
                    if irs > 0:
                        for iq in range(nocc):
                            for ip in range(nin, nocc):
                                ipq = pos[ip, iq]
                                if ipq > 0:
                                    v = -ac[IG[iq], IG[ir], IG[iu], 1] * np.sum(RV[act, ip, iu, is_] * ints[act, iq])
                                    add(ipq, irs, v, v)
                for is_ in range(nin, nocc):        # T6 p->q
                    irs = pos[ir, is_]
                    if irs > 0:
                        for iq in range(nin, nocc):
                            for ip in range(nin, nbas):
                                ipq = pos[ip, iq]
                                if ipq > 0:
                                    v = -ac[IG[ip], IG[ir], IG[iu], 1] * np.sum(RV[act, iq, iu, is_] * ints[ip, act])
                                    add(ipq, irs, v, -v)

    # ---------------- Coulomb loop (FF|OO): records kl = kk + ll*nocc
    for ll in range(nocc):
        for kk in range(nocc):
            ints = ffoo[kk + ll * nocc].reshape(nbas, nbas).T    # ints[i, j]
            k, l = kk, ll
            etot += np.sum(RV[:, :, k, l] * ints[:nocc, :nocc])
            if k == l:
                val = 2 * hnocoef * occ[k]
                if k >= nin:
                    HNO[:nin, :nin] += val * ints[:nin, :nin]
                if k < nin:
                    HNO[nin:nocc, nin:nocc] += val * ints[nin:nocc, nin:nocc]
                HNO[nocc:, nocc:] += val * ints[nocc:, nocc:]
                val = 2 * occ[k]
                if k < nin:
                    w = val * ints * ac[IG[:, None], IG[None, :], 0, 0]
                    AuxIO += w
                    AuxI += w
                if nin <= k < nocc:
                    AuxI += val * ints * ac[IG[:, None], IG[None, :], 1, 1]
            # exchange
            iq, is_ = k, l
            for ir in range(nin, nbas):
                irs = pos[ir, is_]
                if irs > 0:
                    for ip in range(nin, nbas):
                        ipq = pos[ip, iq]
                        if ipq > 0:
                            av = ac[IG[ip], IG[iq], IG[ir], IG[is_]]
                            v = 0.0
                            if ai(ip, ir): v += occ[ip] * occ[ir]
                            if ai(iq, is_): v += occ[iq] * occ[is_]
                            if ai(iq, ir): v -= occ[iq] * occ[ir]
                            if ai(ip, is_): v -= occ[ip] * occ[is_]
                            v = -av * v * ints[ip, ir]
                            add(ipq, irs, v, v)
            # T1
            for ir in range(nin, nocc):
                irs = pos[ir, is_]
                if irs > 0:
                    for ip in range(nin, nocc):
                        ipq = pos[ip, iq]
                        if ipq > 0:
                            v = ac[IG[iq], IG[is_], 1, 1] * np.sum(RV[act, act, ip, ir] * ints[act, act])
                            add(ipq, irs, v, v)
            # T3
            if IG[k] == 1 and IG[l] == 1:
                for is2 in range(nin, nocc):
                    for ir in range(nin, nbas):
                        irs = pos[ir, is2]
                        if irs > 0:
                            for iq2 in range(nin, nocc):
                                for ip in range(nin, nbas):
                                    ipq = pos[ip, iq2]
                                    if ipq > 0:
                                        v = ac[IG[ip], IG[ir], 1, 1] * RV[iq2, is2, k, l] * ints[ip, ir]
                                        add(ipq, irs, v, v)
            # T2 + T5
            if nin <= l < nocc:
                is2, iu = k, l
                for ir in range(nin, nocc):          # T2
                    irs = pos[ir, is2]
                    if irs > 0:
                        for iq2 in range(nocc):
                            for ip in range(nin, nocc):
                                ipq = pos[ip, iq2]
                                if ipq > 0:
                                    v = ac[IG[iq2], IG[is2], IG[iu], 1] * np.sum(RV[act, ip, ir, iu] * ints[act, iq2])
                                    add(ipq, irs, v, v)
                for ir in range(nin, nocc):          # T2 p->q
                    irs = pos[ir, is2]
                    if irs > 0:
                        for iq2 in range(nin, nocc):
                            for ip in range(nin, nbas):
                                ipq = pos[ip, iq2]
                                if ipq > 0:
                                    v = ac[IG[ip], IG[is2], IG[iu], 1] * np.sum(RV[act, iq2, ir, iu] * ints[act, ip])
                                    add(ipq, irs, v, -v)
                for ir in range(nin, nocc):          # T5
                    irs = pos[ir, is2]
                    if irs > 0:
                        for iq2 in range(nin, nocc):
                            for ip in range(nin, nbas):
                                ipq = pos[ip, iq2]
                                if ipq > 0:
                                    v = -ac[IG[ip], IG[is2], IG[iu], 1] * np.sum(RV[act, iq2, iu, ir] * ints[act, ip])
                                    add(ipq, irs, v, v)
                for ir in range(nin, nocc):          # T5 p->q
                    irs = pos[ir, is2]
                    if irs > 0:
                        for iq2 in range(nocc):
                            for ip in range(nin, nocc):
                                ipq = pos[ip, iq2]
                                if ipq > 0:
                                    v = -ac[IG[iq2], IG[is2], IG[iu], 1] * np.sum(RV[act, ip, iu, ir] * ints[act, iq2])
                                    add(ipq, irs, v, -v)
    return etot


# ------------------------------------------------------------------- ERPA
def erpasymm1(abplus, abmin):
    """ERPASYMM1 (interpa.f:1652-1781) with Diag8 (misc.f:541-616) = dsyevd.

    Returns (EigVecR, Eig, APLSQRT): EigVecR[:, nu] = Y_nu; Eig = omega for
    omega^2 > 1e-6 (else omega^2, unnormalised Y), ascending.
    """
    ap = abplus.copy()
    am = abmin.copy()
    iu = np.triu_indices(ap.shape[0], 1)
    ap[iu] = 0.5 * (ap[iu] + ap.T[iu])
    ap.T[iu] = ap[iu]
    am[iu] = 0.5 * (am[iu] + am.T[iu])
    am.T[iu] = am[iu]
    e, V = scipy.linalg.eigh(ap, driver='evd')
    P = (V * np.sqrt(np.abs(e))[None, :]) @ V.T
    P = 0.5 * (P + P.T)
    H = am @ P
    M = P @ H
    w2, Z = scipy.linalg.eigh(M, lower=True, driver='evd')
    Y = P @ Z
    eig = w2.copy()
    for nu in range(Y.shape[1]):
        if eig[nu] > SMALL_OMEGA2:
            eig[nu] = np.sqrt(eig[nu])
            s = 2.0 / eig[nu] * (Y[:, nu] @ am @ Y[:, nu])
            s = 1.0 / np.sqrt(s) if s > 0 else 0.0
            Y[:, nu] *= s
    return Y, eig, P


def ac_ene_erpa_fofo(evec, eval_, occ, nin, nact, indn, fofo):
    """ACEneERPA_FOFO (abfofo.f90:3791-3927). Returns W (ECorr of the routine)."""
    nbas = occ.shape[0]
    nocc = nin + nact
    ndimx = indn.shape[0]
    IG = _groups(nbas, nin, nocc)
    C = np.sign(occ - 0.5) * np.sqrt(occ)
    C[occ - 0.5 == 0] = np.sqrt(occ[occ - 0.5 == 0])
    pos = np.zeros((nbas, nbas), dtype=np.int64)
    for i in range(ndimx):
        pos[indn[i, 0] - 1, indn[i, 1] - 1] = i + 1
    cond = (eval_ > SMALL_E) & (eval_ < BIG_E)
    tvec = np.where(cond[:, None], evec.T, 0.0)        # tVec(kk, :) = EVec(:, kk)
    ecorr = 0.0
    # (p, q) list in the j-outer / i-inner order of the routine
    pq = [(j, i) for j in range(nbas) for i in range(j + 1) if pos[j, i] != 0]
    pj = np.array([a for a, _ in pq], dtype=np.int64)
    qi = np.array([b for _, b in pq], dtype=np.int64)
    ipq = pos[pj, qi] - 1
    for k in range(nocc):
        for l in range(nbas):
            if pos[l, k] == 0:
                continue
            irs = pos[l, k] - 1
            ir, is_ = l, k
            rec = fofo[l + k * nbas]
            ints = np.zeros((nbas, nbas))
            ints[:, :nocc] = rec.reshape(nocc, nbas).T
            crs = C[l] + C[k]
            cpq = C[pj] + C[qi]
            allsame = (IG[pj] == IG[qi]) & (IG[qi] == IG[ir]) & (IG[ir] == IG[is_])
            m = ~allsame
            sumy = tvec[:, ipq].T @ tvec[:, irs]
            aux = 2 * crs * cpq * sumy
            diag = (qi == is_) & (pj == ir)
            aux = np.where(diag, aux - occ[pj] * (1.0 - occ[is_]) - occ[is_] * (1.0 - occ[pj]), aux)
            ecorr += np.sum(np.where(m, aux * ints[pj, qi], 0.0))
    return ecorr


def ace_integ_fofo(occ, xone, indn, nin, nact, ffoo, fofo, rdm2act, alpha):
    """ACEInteg_FOFO (abfofo.f90:3664-3789), ICASSCF=1, NoSt=1, IFunSR=0."""
    nbas = occ.shape[0]
    abp, abm, ecas = ab_cas_fofo(occ, xone, np.eye(nbas), indn, nin, nact, ffoo, fofo,
                                 rdm2act, alpha)
    Y, eig, _ = erpasymm1(abp, abm)
    w = ac_ene_erpa_fofo(Y, eig, occ, nin, nact, indn, fofo)
    return w, ecas


def acecorr(occ, xone, indn, nin, nact, ffoo, fofo, rdm2act, ngrid=5):
    """ACECORR lambda loop (acfd.f:117-209). Returns (E_CAS, ECorr, [W_i], x, w)."""
    x, w = gauleg(0.0, 1.0, ngrid)
    ecorr = 0.0
    ws = []
    ecas = None
    for i in range(ngrid):
        wi, ecas = ace_integ_fofo(occ, xone, indn, nin, nact, ffoo, fofo, rdm2act, x[i])
        ws.append(wi)
        ecorr += w[i] * wi
    return ecas, ecorr, ws, x, w
