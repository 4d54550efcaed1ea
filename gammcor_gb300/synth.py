"""Seeded synthetic AC-CAS systems.

GAMMCOR reads its inputs (AO integrals, MO coefficients, CAS 1- and 2-RDMs)
from Molpro/Dalton/ORCA dumps (initia.f:995-1580). This module builds the same
quantities from a seed so that every stage of the path can be run without an
external quantum-chemistry code:

* AO ERIs  (mn|ls) = sum_P L[mn,P] L[ls,P], L symmetric in mn,
  L ~ N(0,1) * exp(-|m-n|/8) * exp(-P/60); 8-fold symmetric and PSD.
* core Hamiltonian: symmetric, diagonal U(-20,5), off-diagonal N(0,0.1).
* MO coefficients: Q of a QR of a seeded Gaussian matrix (AO overlap = 1),
  columns ordered by the diagonal of a closed-shell Fock matrix built from the
  lowest NELE orbitals of a core-Hamiltonian ordering.
* RDMs: exact lowest Ms=0 eigenvector of the CAS(k,k) determinant CI in the
  field of the frozen inactive core (a CI solver written for this project;
  the reference receives RDMs from Molpro).
* orbital preparation as LdInteg does it (initia.f:1146-1398): active orbitals
  rotated to natural orbitals sorted by decreasing occupation (SortP), inactive
  and virtual blocks canonicalised by diagonalising the Fock matrix built from
  the CAS 1-RDM (initia.f:1255-1370).

Packed pair index convention (AOTWOSORT records, sorter.f90:95-100, and the
XOne triangle read by triang_to_sq, tran.f90:1221-1247): for 0-based p <= q,
pq = p + q*(q+1)/2.
"""
from __future__ import annotations

import itertools
import math
from dataclasses import dataclass, field

import numpy as np


def ntri(n: int) -> int:
    return n * (n + 1) // 2


def tri_index(n: int):
    """(p, q) 0-based arrays of the packed upper triangle, p <= q, q-major."""
    p, q = [], []
    for qq in range(n):
        for pp in range(qq + 1):
            p.append(pp)
            q.append(qq)
    return np.array(p), np.array(q)


def unpack_sym(packed: np.ndarray, n: int) -> np.ndarray:
    """Packed triangle (..., ntr) -> symmetric (..., n, n)."""
    p, q = tri_index(n)
    out = np.zeros(packed.shape[:-1] + (n, n), dtype=packed.dtype)
    out[..., p, q] = packed
    out[..., q, p] = packed
    return out


def pack_sym(full: np.ndarray) -> np.ndarray:
    n = full.shape[-1]
    p, q = tri_index(n)
    return full[..., p, q]


# Global factor on the ERI factor L. With L ~ N(0,1) exp(-|m-n|/8) exp(-P/60)
# unscaled, (mm|mm) is about 30 Eh against a core-Hamiltonian spread of 25 Eh:
# the closed-shell SCF does not converge and ERPA is unstable for every seed
# tried. With L scaled by 0.1 the SCF converges and A+B is positive definite
# at lambda = 0 and 1 for the seeds tried (hence on all of [0, 1], A+B being
# affine in lambda); A-B of a CAS-CI (not CASSCF) reference stays indefinite,
# which ERPASYMM1 tolerates by dropping omega^2 <= 1e-6.
ERI_SCALE = 0.1


@dataclass
class System:
    """One synthetic AC-CAS instance in the MO (natural-orbital) basis."""
    n: int                      # NBasis
    nin: int                    # inactive (doubly occupied) orbitals
    nact: int                   # active orbitals (CAS(nact, nact))
    rank: int                   # ERI factor rank
    seed: int
    lfac: np.ndarray            # (ntr, rank) packed-pair ERI factor, AO basis
    h_ao: np.ndarray            # (n, n) core Hamiltonian, AO basis
    cmo: np.ndarray             # (n, n) AO x MO coefficients (column a = MO a)
    occ: np.ndarray             # (n,) occupations in [0,1] (Occ of the reference)
    xone: np.ndarray            # (ntr,) packed one-electron integrals, MO basis
    rdm2act: np.ndarray         # (nact^2 (nact^2+1)/2,) packed active 2-RDM (NAddrRDM)
    e_cas: float                # CAS-CI electronic energy (no nuclear repulsion)
    nele: int                   # electron pairs (NELE)
    extra: dict = field(default_factory=dict)

    @property
    def nocc(self) -> int:
        return self.nin + self.nact

    def ao_eri_packed(self) -> np.ndarray:
        """AOTWOSORT-layout tensor G[rs, pq] = (pq|rs), shape (ntr, ntr)."""
        return self.lfac @ self.lfac.T


# ---------------------------------------------------------------- ERI factor
def make_lfac(n: int, rank: int, rng: np.random.Generator) -> np.ndarray:
    p, q = tri_index(n)
    dist = np.abs(p - q).astype(np.float64)
    g = rng.standard_normal((ntri(n), rank))
    g *= np.exp(-dist / 8.0)[:, None]
    g *= np.exp(-np.arange(rank, dtype=np.float64) / 60.0)[None, :]
    return g


def jk_from_factor(lfac: np.ndarray, n: int, dens: np.ndarray, chunk: int = 256,
                   cocc: np.ndarray | None = None):
    """J[m,n] = sum_ls (mn|ls) D[l,s],  K[m,n] = sum_ls (ml|ns) D[l,s].

    When cocc is given, D = cocc cocc^T and K is built as sum_P X_P X_P^T with
    X_P = L_P cocc, which costs rank*n^2*nocc instead of rank*n^3.
    """
    p, q = tri_index(n)
    w = dens[p, q] + dens[q, p]
    w[p == q] *= 0.5
    jvec = lfac.T @ w                         # (rank,)
    jpk = lfac @ jvec
    J = unpack_sym(jpk, n)
    K = np.zeros((n, n))
    rank = lfac.shape[1]
    for s in range(0, rank, chunk):
        lp = unpack_sym(lfac[:, s:s + chunk].T.copy(), n)   # (c, n, n)
        if cocc is not None:
            x = np.matmul(lp, cocc[None])                    # (c, n, nocc)
            K += np.einsum('pmi,pni->mn', x, x, optimize=True)
        else:
            K += np.matmul(np.matmul(lp, dens), lp).sum(axis=0)
    return J, K


def scf(lfac: np.ndarray, h: np.ndarray, guess: np.ndarray, nocc: int,
        max_iter: int = 60, tol: float = 1e-10):
    """Closed-shell SCF from guess orbitals: level shift + density damping,
    switching to Pulay DIIS once the commutator error is small.

    Returns (orbitals, orbital energies, energy, iterations); orbitals are the
    eigenvectors of the final Fock matrix, ascending.
    """
    n = h.shape[0]
    co = guess[:, :nocc]
    D = co @ co.T
    fs, es = [], []
    e_old = None
    it = 0
    for it in range(1, max_iter + 1):
        # K from a factorised density: D = X X^T with X from its eigenvectors
        w, v = np.linalg.eigh(D)
        keep = w > 1e-12
        X = v[:, keep] * np.sqrt(w[keep])[None, :]
        J, K = jk_from_factor(lfac, n, D, cocc=X)
        F = h + 2 * J - K
        e = float(np.sum(D * (h + F)))
        err = F @ D - D @ F
        emax = np.abs(err).max()
        if e_old is not None and abs(e - e_old) < tol and emax < 1e-8:
            break
        e_old = e
        if emax < 1e-2:
            fs.append(F)
            es.append(err)
            fs, es = fs[-8:], es[-8:]
            m = len(fs)
            B = -np.ones((m + 1, m + 1))
            B[m, m] = 0.0
            for i in range(m):
                for j in range(m):
                    B[i, j] = np.sum(es[i] * es[j])
            rhs = np.zeros(m + 1)
            rhs[m] = -1.0
            try:
                coef = np.linalg.solve(B, rhs)[:m]
                Fx = sum(ci * fi for ci, fi in zip(coef, fs))
            except np.linalg.LinAlgError:
                Fx = F
            _, c = np.linalg.eigh(Fx)
            D = c[:, :nocc] @ c[:, :nocc].T
        else:
            fs, es = [], []
            _, c = np.linalg.eigh(F + 2.0 * (np.eye(n) - D))
            D = 0.5 * D + 0.5 * (c[:, :nocc] @ c[:, :nocc].T)
    eps, c = np.linalg.eigh(F)
    return c, eps, e, it


def mo_eri_from_factor(lfac: np.ndarray, n: int, c1, c2, c3, c4):
    """(ab|cd) = sum_P (C1^T L_P C2)_ab (C3^T L_P C4)_cd, dense 4-index."""
    rank = lfac.shape[1]
    b12 = np.empty((rank, c1.shape[1], c2.shape[1]))
    b34 = np.empty((rank, c3.shape[1], c4.shape[1]))
    for s in range(0, rank, 256):
        lp = unpack_sym(lfac[:, s:s + 256].T.copy(), n)
        b12[s:s + 256] = np.matmul(np.matmul(c1.T[None], lp), c2[None])
        b34[s:s + 256] = np.matmul(np.matmul(c3.T[None], lp), c4[None])
    return np.einsum('Pab,Pcd->abcd', b12, b34, optimize=True)


# ------------------------------------------------------------------ CAS-CI
class _Strings:
    """Occupation strings of nel electrons in norb orbitals and E^sigma_pq."""

    def __init__(self, norb: int, nel: int):
        self.norb, self.nel = norb, nel
        strs = [sum(1 << i for i in c) for c in itertools.combinations(range(norb), nel)]
        self.strs = strs
        self.index = {s: i for i, s in enumerate(strs)}
        ns = len(strs)
        # E[p, q] as dense (ns, ns) matrices: <s'|a+_p a_q|s>
        E = np.zeros((norb, norb, ns, ns))
        for j, s in enumerate(strs):
            for q in range(norb):
                if not (s >> q) & 1:
                    continue
                sq = s & ~(1 << q)
                sgn_q = (-1) ** bin(s & ((1 << q) - 1)).count('1')
                for p in range(norb):
                    if (sq >> p) & 1:
                        continue
                    sp = sq | (1 << p)
                    sgn_p = (-1) ** bin(sq & ((1 << p) - 1)).count('1')
                    E[p, q, self.index[sp], j] = sgn_q * sgn_p
        self.E = E


def cas_ci(h_eff: np.ndarray, eri_act: np.ndarray, nel_act: int, e_core: float):
    """Lowest Ms=0 eigenpair of the CAS determinant Hamiltonian.

    Returns (energy, gamma1, gamma2) with gamma1[p,q] = <E_pq> (spin-summed)
    and gamma2[p,q,r,s] = FRDM2 convention (interpa.f:5244-5272):
    0.5 * (<E_pr E_qs> - delta_qr <E_ps>).
    """
    nact = h_eff.shape[0]
    na = nb = nel_act // 2
    sa = _Strings(nact, na)
    sb = sa if nb == na else _Strings(nact, nb)
    Ea, Eb = sa.E, sb.E
    nsa, nsb = len(sa.strs), len(sb.strs)
    k1 = h_eff - 0.5 * np.einsum('prrq->pq', eri_act)
    V = eri_act.reshape(nact * nact, nact * nact)

    def epq_all(cm):
        # D[p,q] = E_pq c  for c as (nsa, nsb, m)
        da = np.einsum('pqij,jbm->pqibm', Ea, cm, optimize=True)
        db = np.einsum('pqij,ajm->pqaim', Eb, cm, optimize=True)
        return da + db

    def sigma(cm):
        D = epq_all(cm)                               # (p,q,a,b,m)
        out = np.einsum('pq,pqabm->abm', k1, D, optimize=True)
        G = np.tensordot(V, D.reshape(nact * nact, -1), axes=(1, 0))
        G = G.reshape(nact, nact, nsa, nsb, -1)
        out += 0.5 * (np.einsum('pqij,pqjbm->ibm', Ea, G, optimize=True)
                      + np.einsum('pqij,pqajm->aim', Eb, G, optimize=True))
        return out

    # Singlet ground state: for Ms=0 and na == nb, states of even S have
    # coefficient matrices C[a,b] symmetric under the alpha<->beta swap, odd S
    # antisymmetric; the lowest even-S state is the singlet.
    def sym(cm):
        return 0.5 * (cm + cm.transpose(1, 0, 2))

    ndet = nsa * nsb
    if ndet <= 1200:
        eye = np.eye(ndet).reshape(nsa, nsb, ndet)
        H = sigma(sym(eye)).reshape(ndet, ndet)
        H = sym(H.reshape(nsa, nsb, ndet)).reshape(ndet, ndet)
        H = 0.5 * (H + H.T)
        w, v = np.linalg.eigh(H)
        cands = [i for i in range(ndet)
                 if np.abs(v[:, i].reshape(nsa, nsb) - v[:, i].reshape(nsa, nsb).T).max() < 1e-8
                 and np.linalg.norm(v[:, i]) > 0.5]
        c = v[:, cands[0]]
    else:
        from scipy.sparse.linalg import LinearOperator, eigsh
        op = LinearOperator((ndet, ndet),
                            matvec=lambda x: sym(sigma(sym(x.reshape(nsa, nsb, 1)))).ravel(),
                            dtype=np.float64)
        rng = np.random.default_rng(12345)
        v0 = sym(rng.standard_normal((nsa, nsb, 1))).ravel()
        w, v = eigsh(op, k=1, which='SA', tol=1e-13, v0=v0, maxiter=5000)
        c = v[:, 0]
    c = c / np.linalg.norm(c)
    cm = c.reshape(nsa, nsb, 1)
    D = epq_all(cm)[..., 0].reshape(nact, nact, ndet)
    g1 = np.einsum('pqx,x->pq', D, c)
    # <E_pr E_qs> = (E_rp c) . (E_qs c)
    EE = np.einsum('rpx,qsx->pqrs', D, D, optimize=True)
    g2 = EE - np.einsum('qr,ps->pqrs', np.eye(nact), g1)
    g2 = 0.5 * g2
    e_act = float(c @ sigma(cm).ravel())
    return e_act + e_core, g1, g2


def naddr_rdm(i1, i2, i3, i4, nact):
    """NAddrRDM (interpa.f:4529-4541), 1-based indices -> 1-based address."""
    i12 = (i1 - 1) * nact + i2
    i34 = (i3 - 1) * nact + i4
    mx = np.maximum(i12, i34)
    mn = np.minimum(i12, i34)
    return mx * (mx - 1) // 2 + mn


def pack_rdm2act(g2: np.ndarray) -> np.ndarray:
    nact = g2.shape[0]
    out = np.zeros(nact ** 2 * (nact ** 2 + 1) // 2)
    idx = np.arange(1, nact + 1)
    I, J, K, L = np.meshgrid(idx, idx, idx, idx, indexing='ij')
    addr = naddr_rdm(I, J, K, L, nact) - 1
    out[addr.ravel()] = g2.ravel()
    return out


def unpack_rdm2act(packed: np.ndarray, nact: int) -> np.ndarray:
    idx = np.arange(1, nact + 1)
    I, J, K, L = np.meshgrid(idx, idx, idx, idx, indexing='ij')
    return packed[naddr_rdm(I, J, K, L, nact) - 1]


# ------------------------------------------------------------- generator
def make_system(n: int, nin: int, nact: int, rank: int, seed: int, eri_scale: float = ERI_SCALE) -> System:
    rng = np.random.default_rng(seed)
    lfac = make_lfac(n, rank, rng) * eri_scale
    h = np.diag(rng.uniform(-20.0, 5.0, n))
    off = rng.normal(0.0, 0.1, (n, n))
    off = np.triu(off, 1)
    h = h + off + off.T
    q, r = np.linalg.qr(rng.standard_normal((n, n)))
    cmo = q * np.sign(np.diag(r))[None, :]
    nele = nin + nact // 2
    # The QR matrix is the initial guess of a closed-shell SCF; the converged
    # canonical orbitals are ordered by Fock diagonal (orbital energy).
    cmo, eps, e_scf, scf_iter = scf(lfac, h, cmo, nele)

    nocc = nin + nact
    # frozen-core CAS-CI
    ccore = cmo[:, :nin]
    dcore = ccore @ ccore.T
    Jc, Kc = jk_from_factor(lfac, n, dcore, cocc=ccore)
    fcore = h + 2 * Jc - Kc
    e_core = float(np.sum(dcore * (h + fcore)))
    cact = cmo[:, nin:nocc]
    h_eff = cact.T @ fcore @ cact
    eri_act = mo_eri_from_factor(lfac, n, cact, cact, cact, cact)
    e_cas, g1, g2 = cas_ci(h_eff, eri_act, nact, e_core)

    # natural orbitals, decreasing occupation (SortP)
    occ_act, u = np.linalg.eigh(0.5 * g1)
    order = np.argsort(-occ_act, kind='stable')
    occ_act, u = np.abs(occ_act[order]), u[:, order]
    cmo = cmo.copy()
    cmo[:, nin:nocc] = cact @ u
    g2no = np.einsum('pqrs,pa,qb,rc,sd->abcd', g2, u, u, u, u, optimize=True)

    occ = np.zeros(n)
    occ[:nin] = 1.0
    occ[nin:nocc] = occ_act
    # canonicalise inactive and virtual blocks with the CAS Fock matrix
    gam = np.zeros((n, n))
    gam[:nocc, :nocc] = np.diag(occ[:nocc])
    dens = cmo @ gam @ cmo.T
    J, K = jk_from_factor(lfac, n, dens, cocc=cmo[:, :nocc] * np.sqrt(occ[:nocc])[None, :])
    fmo = cmo.T @ (h + 2 * J - K) @ cmo
    if nin > 0:
        _, ui = np.linalg.eigh(fmo[:nin, :nin])
        cmo[:, :nin] = cmo[:, :nin] @ ui
    if n > nocc:
        _, uv = np.linalg.eigh(fmo[nocc:, nocc:])
        cmo[:, nocc:] = cmo[:, nocc:] @ uv
    xone = pack_sym(cmo.T @ h @ cmo)
    return System(n=n, nin=nin, nact=nact, rank=rank, seed=seed, lfac=lfac, h_ao=h,
                  cmo=cmo, occ=occ, xone=xone, rdm2act=pack_rdm2act(g2no),
                  e_cas=e_cas, nele=nele, extra=dict(e_scf=e_scf, scf_iter=scf_iter))


# Workload shapes named by the benchmark configurations.
CFG_SMALL = dict(n=64, nin=6, nact=4, rank=300)          # plain AC-CAS, 5 lambda points
CFG_PRECISION = dict(n=400, nin=40, nact=8, rank=2400)   # transform-scale precision study
CFG_LARGE = dict(n=500, nin=30, nact=8, rank=3000)       # large single system


def batched_shapes(count: int = 64, seed: int = 2024):
    """Uneven batch: n ~ U[50,250], inactive ~ U[5,25], CAS(2,2)..CAS(6,6), rank 6n."""
    rng = np.random.default_rng(seed)
    out = []
    for i in range(count):
        n = int(rng.integers(50, 251))
        nin = int(rng.integers(5, 26))
        nact = int(rng.choice([2, 4, 6]))
        out.append(dict(n=n, nin=nin, nact=nact, rank=6 * n, seed=seed * 1000 + i))
    return out


# ------------------------------------------------- device-side generation
def make_system_device(n: int, nin: int, nact: int, rank: int, seed: int,
                       eri_scale: float = ERI_SCALE, device: str = "cuda:0") -> System:
    """make_system with the factor-based J/K builds, the SCF and the
    canonicalisation run in FP64 torch on a GPU. The random draws are the
    same numpy draws as make_system; results agree with it to rounding."""
    import torch

    rng = np.random.default_rng(seed)
    lfac = make_lfac(n, rank, rng) * eri_scale
    h = np.diag(rng.uniform(-20.0, 5.0, n))
    off = rng.normal(0.0, 0.1, (n, n))
    off = np.triu(off, 1)
    h = h + off + off.T
    q, r = np.linalg.qr(rng.standard_normal((n, n)))
    guess = q * np.sign(np.diag(r))[None, :]
    nele = nin + nact // 2
    nocc = nin + nact

    dev = torch.device(device)
    p, qq = tri_index(n)
    pt, qt = torch.as_tensor(p, device=dev), torch.as_tensor(qq, device=dev)
    L = torch.as_tensor(lfac, device=dev)
    Lsq = torch.zeros((rank, n, n), dtype=torch.float64, device=dev)
    Lsq[:, pt, qt] = L.T
    Lsq[:, qt, pt] = L.T
    H = torch.as_tensor(h, device=dev)
    eye = torch.eye(n, dtype=torch.float64, device=dev)

    def jk(D, X):
        Jv = torch.einsum('pmn,mn->p', Lsq, D)
        J = torch.einsum('p,pmn->mn', Jv, Lsq)
        Y = torch.matmul(Lsq, X)                      # (rank, n, k)
        K = torch.einsum('pmi,pni->mn', Y, Y)
        return J, K

    # SCF (same scheme as scf()); J/K on the device, the n x n eigenproblems on the host
    def eigh_h(Mt):
        w, v = np.linalg.eigh(Mt.cpu().numpy())
        return torch.as_tensor(w, device=dev), torch.as_tensor(v, device=dev)

    c = torch.as_tensor(guess, device=dev)
    D = c[:, :nele] @ c[:, :nele].T
    fs, es = [], []
    e_old = None
    it = 0
    for it in range(1, 61):
        w, v = eigh_h(D)
        keep = w > 1e-12
        X = v[:, keep] * torch.sqrt(w[keep])[None, :]
        J, K = jk(D, X)
        F = H + 2 * J - K
        e = float(torch.sum(D * (H + F)))
        err = F @ D - D @ F
        emax = float(err.abs().max())
        if e_old is not None and abs(e - e_old) < 1e-10 and emax < 1e-8:
            break
        e_old = e
        if emax < 1e-2:
            fs.append(F)
            es.append(err)
            fs, es = fs[-8:], es[-8:]
            m = len(fs)
            B = -np.ones((m + 1, m + 1))
            B[m, m] = 0.0
            for i in range(m):
                for j in range(m):
                    B[i, j] = float(torch.sum(es[i] * es[j]))
            rhs = np.zeros(m + 1)
            rhs[m] = -1.0
            try:
                coef = np.linalg.solve(B, rhs)[:m]
                Fx = sum(float(ci) * fi for ci, fi in zip(coef, fs))
            except np.linalg.LinAlgError:
                Fx = F
            _, cc = eigh_h(Fx)
            D = cc[:, :nele] @ cc[:, :nele].T
        else:
            fs, es = [], []
            _, cc = eigh_h(F + 2.0 * (eye - D))
            D = 0.5 * D + 0.5 * (cc[:, :nele] @ cc[:, :nele].T)
    _, cmo_t = eigh_h(F)

    # frozen-core CAS-CI
    ccore = cmo_t[:, :nin]
    dcore = ccore @ ccore.T
    Jc, Kc = jk(dcore, ccore)
    fcore = H + 2 * Jc - Kc
    e_core = float(torch.sum(dcore * (H + fcore)))
    cact = cmo_t[:, nin:nocc]
    h_eff = (cact.T @ fcore @ cact).cpu().numpy()
    B = torch.matmul(torch.matmul(cact.T[None], Lsq), cact[None])        # (rank, nact, nact)
    eri_act = torch.einsum('Pab,Pcd->abcd', B, B).cpu().numpy()
    e_cas, g1, g2 = cas_ci(h_eff, eri_act, nact, e_core)

    occ_act, u = np.linalg.eigh(0.5 * g1)
    order = np.argsort(-occ_act, kind='stable')
    occ_act, u = np.abs(occ_act[order]), u[:, order]
    cmo = cmo_t.cpu().numpy().copy()
    cmo[:, nin:nocc] = cmo[:, nin:nocc] @ u
    g2no = np.einsum('pqrs,pa,qb,rc,sd->abcd', g2, u, u, u, u, optimize=True)
    occ = np.zeros(n)
    occ[:nin] = 1.0
    occ[nin:nocc] = occ_act
    cm = torch.as_tensor(cmo, device=dev)
    Xo = cm[:, :nocc] * torch.sqrt(torch.as_tensor(occ[:nocc], device=dev))[None, :]
    J, K = jk(Xo @ Xo.T, Xo)
    fmo = (cm.T @ (H + 2 * J - K) @ cm).cpu().numpy()
    if nin > 0:
        _, ui = np.linalg.eigh(fmo[:nin, :nin])
        cmo[:, :nin] = cmo[:, :nin] @ ui
    if n > nocc:
        _, uv = np.linalg.eigh(fmo[nocc:, nocc:])
        cmo[:, nocc:] = cmo[:, nocc:] @ uv
    xone = pack_sym(cmo.T @ h @ cmo)
    cmt = torch.as_tensor(cmo, device=dev)
    fdiag = torch.diagonal(cmt.T @ (H + 2 * J - K) @ cmt).cpu().numpy()  # CAS Fock diagonal
    del Lsq
    return System(n=n, nin=nin, nact=nact, rank=rank, seed=seed, lfac=lfac, h_ao=h,
                  cmo=cmo, occ=occ, xone=xone, rdm2act=pack_rdm2act(g2no),
                  e_cas=e_cas, nele=nele, extra=dict(e_scf=e, scf_iter=it, fock_diag=fdiag))
