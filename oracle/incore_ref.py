"""Independent dense restatement of the in-core AC-CAS formulas.

TEST INFRASTRUCTURE ONLY (see oracle/ac_cas_ref.py). This is the second CPU
cross-check of the same quantities, written from the in-core routines rather
than the FOFO ones:

* AB_CAS   (interpa.f:3659-4106): A+B / A-B per (rs, pq) element from the
  full MO integral tensor (ITwoEl=1),
* ACEneERPA (acfd.f:4969-5043): W(lambda) from the same tensor.

The element formulas are evaluated over all orbital quadruples with numpy
einsum/masks and then gathered to pairs, so the summation order differs from
the FOFO restatement while the algebra is the reference's.
"""
from __future__ import annotations

import numpy as np

from .ac_cas_ref import SMALL_E, BIG_E


def _groups(n, nin, nocc):
    g = np.full(n, 2)
    g[:nin] = 0
    g[nin:nocc] = 1
    return g


def ab_cas_incore(V, occ, hno, g2act, nin, nact, indn, alpha):
    """AB_CAS. V[p,q,r,s] = (pq|rs) in the NO basis; hno full (n,n) one-electron
    matrix; g2act[t,u,v,w] = FRDM2 over active orbitals. Returns (ABPLUS,
    ABMIN, ETot) with ABPLUS[ipq, irs] (row = (p,q) pair, as AB_CAS_FOFO)."""
    n = occ.shape[0]
    nocc = nin + nact
    g = _groups(n, nin, nocc)
    o = occ
    one = o == 1.0
    act = slice(nin, nocc)
    # FRDM2 over all occupied orbitals
    G = np.zeros((nocc,) * 4)
    for p in range(nocc):
        for q in range(nocc):
            if one[p] or one[q]:
                G[p, q, p, q] += 2 * o[p] * o[q]
                G[p, q, q, p] -= o[p] * o[q]
    G[act, act, act, act] = g2act
    etot = 2 * np.sum(o * np.diag(hno)) + np.einsum('pqrs,prqs->', G, V[:nocc, :nocc, :nocc, :nocc])

    same4 = ((g[:, None, None, None] == g[None, :, None, None])
             & (g[None, :, None, None] == g[None, None, :, None])
             & (g[None, None, :, None] == g[None, None, None, :]))
    AC = np.where(same4, 1.0, alpha)
    # one-electron part of the alpha-Hamiltonian
    H = hno.copy()
    diffg = g[:, None] != g[None, :]
    tmask = (g[None, :] != g[:, None])                 # [i, t] : g_t != g_i
    J = np.einsum('ttij->tij', V)
    K = np.einsum('titj->tij', V)
    corr = np.einsum('it,t,tij->ij', tmask.astype(float), o, 2 * J - K)
    H = np.where(diffg, alpha * hno, hno + (1 - alpha) * corr)
    # AuxI, AuxIO
    actt = np.einsum('ttpq->tpq', AC)
    JK = 2 * np.einsum('pqtt->tpq', V) - np.einsum('ptqt->tpq', V)
    AuxI = np.einsum('t,tpq,tpq->pq', o[:nocc], actt[:nocc], JK[:nocc])
    AuxIO = np.einsum('t,tpq,tpq->pq', o[:nin], actt[:nin], JK[:nin])
    # WMAT(p, r), r occupied
    W = np.zeros((n, n))
    Vo = V[:nocc, :nocc, :, :nocc]                     # (t,w,p,u)
    ACo = AC[:nocc, :nocc, :, :nocc]
    W[:, :nocc] = (np.einsum('twpu,wutr,twpu->pr', Vo, G, ACo, optimize=True)
                   + np.einsum('tupw,wurt,twpu->pr', V[:nocc, :nocc, :, :nocc], G, ACo, optimize=True))

    # element A_rspq for all (r, s, p, q)
    Aux = AC * (2 * V - V.transpose(0, 2, 1, 3))         # AuxPQRS[p,q,r,s]
    e = np.eye(n)
    A = np.zeros((n, n, n, n))                            # [r, s, p, q]
    # one-electron
    A += np.einsum('pr,ps,qs->rspq', e, (o[:, None] - o[None, :]), H)
    A += np.einsum('qs,qr,pr->rspq', e, (o[:, None] - o[None, :]), H)
    ga = g2act
    aux_rs_pq = Aux.transpose(2, 3, 0, 1)                 # [r,s,p,q] = AuxPQRS[p,q,r,s]
    opo = o[:, None] * o[None, :]
    actm = (o != 0) & ~one
    # T1 + T2 on (p, r)
    nzpr = (opo != 0)
    onepr = one[:, None] | one[None, :]
    m_simple = (nzpr & onepr)                             # [p, r]
    A += np.einsum('pr,rspq->rspq', np.where(m_simple, opo, 0.0), aux_rs_pq)
    A += np.einsum('pr,p,qs->rspq', e * m_simple, o, AuxI)
    m_act = nzpr & ~onepr
    if nact:
        acsq = np.where((g[:, None] == 1) & (g[None, :] == 1), 1.0, alpha)    # [s, q]
        Va = V[:, :, act, act]                                               # (s,q,t,u)
        X = (np.einsum('sqtu,purt->sqpr', Va, ga, optimize=True)
             + np.einsum('sutq,putr->sqpr', V[:, act, act, :], ga, optimize=True))
        blk = np.zeros((n, n, n, n))
        blk[:, :, act, act] = X
        A += np.einsum('sq,sqpr,pr->rspq', acsq, blk, m_act.astype(float), optimize=True)
        A += np.einsum('pr,p,qs->rspq', e * m_act, o, AuxIO)
    # T3 + T4 on (q, s)
    A += np.einsum('qs,rspq->rspq', np.where(m_simple, opo, 0.0), aux_rs_pq)
    A += np.einsum('qs,q,pr->rspq', e * m_simple, o, AuxI)
    if nact:
        acpr = acsq
        X = (np.einsum('utpr,stqu->prsq', V[act, act, :, :], ga, optimize=True)
             + np.einsum('urpt,stuq->prsq', V[act, :, :, act], ga, optimize=True))
        blk = np.zeros((n, n, n, n))
        blk[:, :, act, act] = X
        A += np.einsum('pr,prsq,qs->rspq', acpr, blk, m_act.astype(float), optimize=True)
        A += np.einsum('qs,q,pr->rspq', e * m_act, o, AuxIO)
    # T5 on (r, q)
    A -= np.einsum('qr,rspq->rspq', np.where(m_simple, opo, 0.0), aux_rs_pq)
    if nact:
        acps = acsq
        X = np.einsum('ptsu,tuqr->psqr', V[:, act, :, act], ga, optimize=True)
        blk = np.zeros((n, n, n, n))
        blk[:, :, act, act] = X
        A -= np.einsum('ps,psqr,qr->rspq', acps, blk, m_act.astype(float), optimize=True)
    # T6 on (p, s)
    A -= np.einsum('ps,rspq->rspq', np.where(m_simple, opo, 0.0), aux_rs_pq)
    if nact:
        X = np.einsum('tqur,sput->qrsp', V[act, :, act, :], ga, optimize=True)
        blk = np.zeros((n, n, n, n))
        blk[:, :, act, act] = X
        A -= np.einsum('qr,qrsp,ps->rspq', acsq, blk, m_act.astype(float), optimize=True)
    # WMAT
    A -= 0.5 * np.einsum('sq,pr->rspq', e, W)
    A -= 0.5 * np.einsum('pr,qs->rspq', e, W)

    C = np.sqrt(o) * np.where(o < 0.5, -1.0, 1.0)
    r_, s_ = indn[:, 0] - 1, indn[:, 1] - 1
    Arow = A[r_, s_]                                     # [irs, p, q]
    Ap = Arow[:, r_, s_] + Arow[:, s_, r_]               # [irs, ipq]: (p,q)=(IPP,IQQ) and swapped
    Am = Arow[:, r_, s_] - Arow[:, s_, r_]
    dp = (C[r_] + C[s_])[:, None] * (C[r_] + C[s_])[None, :]
    dm = (C[r_] - C[s_])[:, None] * (C[r_] - C[s_])[None, :]
    Ap = np.where(dp != 0, Ap / np.where(dp != 0, dp, 1.0), Ap)
    Am = np.where(dm != 0, Am / np.where(dm != 0, dm, 1.0), Am)
    # AB_CAS stores ABPLUS(IRS, IPQ); transpose to the (pq, rs) row convention
    return Ap.T, Am.T, etot


def ac_ene_erpa_incore(V, evec, eval_, occ, nin, nact, indn):
    """ACEneERPA (acfd.f:4969-5043). W from the full MO tensor."""
    n = occ.shape[0]
    g = _groups(n, nin, nin + nact)
    C = np.sqrt(occ) * np.where(occ < 0.5, -1.0, 1.0)
    keep = (eval_ > SMALL_E) & (eval_ < BIG_E)
    Yk = evec[:, keep]
    S = Yk @ Yk.T                                        # SumY(I, J)
    p, r = indn[:, 0] - 1, indn[:, 1] - 1
    mask = ~((g[p][:, None] == g[r][:, None]) & (g[p][None, :] == g[r][None, :])
             & (g[p][:, None] == g[p][None, :]))
    cs = C[r]
    cp = C[p]
    # Aux = 2 (C_s + C_q)(C_p + C_r) SumY with I=(p,r), J=(q,s)
    aux = 2 * (cp + cs)[:, None] * (cp + cs)[None, :] * S
    d = -occ[p] * (1 - occ[r]) - occ[r] * (1 - occ[p])
    aux[np.arange(len(p)), np.arange(len(p))] += d
    ints = V[p[:, None], r[:, None], p[None, :], r[None, :]]   # (p r | q s)
    return float(np.sum(np.where(mask, aux * ints, 0.0)))
