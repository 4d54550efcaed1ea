"""CPU restatement of ERPAVEC, the ERPA solver of state-averaged references.

TEST INFRASTRUCTURE ONLY (the oracle of the GC_ERPA_VEC mode): only tests/
import it. Parity status as oracle/ac_cas_ref.py (unpinned against
reference-produced numbers); pinned in tests/ against ERPASYMM1 where both apply.

ERPAVEC (interpa.f:962-1070) takes the right eigenvectors of A+ A- from DGEEV
(numpy.linalg.eig is LAPACK's dgeev), orthonormalises runs of degenerate
eigenvalues (CREATE_SPACE, interpa.f:1119-1150; ORTHO_DEGVEC, interpa.f:1153-1205),
zeroes complex modes and normalises 2/omega y^T A- y to +-1, flipping the sign
of omega for modes of negative norm (de-excitations).
"""
from __future__ import annotations

import numpy as np

from .ac_cas_ref import SMALL_OMEGA2


def erpavec(abplus, abmin):
    """Returns (EigVecR, Eig) in DGEEV's order."""
    ap = 0.5 * (abplus + abplus.T)
    am = 0.5 * (abmin + abmin.T)
    w, V = np.linalg.eig(ap @ am)
    er, ei = w.real.copy(), w.imag.copy()
    # LAPACK stores a complex pair as the real and the imaginary part of one vector
    Y = np.zeros_like(ap)
    k = 0
    N = len(er)
    while k < N:
        if abs(ei[k]) > 0.0 and k + 1 < N:
            Y[:, k] = V[:, k].real
            Y[:, k + 1] = V[:, k].imag
            k += 2
        else:
            Y[:, k] = V[:, k].real
            k += 1
    # CREATE_SPACE + ORTHO_DEGVEC
    start = 0
    for k in range(1, N + 1):
        if k < N and abs(er[k] - er[start]) <= 1e-8:
            continue
        m = k - start
        if m > 1:
            Vg = Y[:, start:k]
            s, U = np.linalg.eigh(Vg.T @ Vg)
            Y[:, start:k] = Vg @ (U / np.sqrt(s)[None, :]) @ U.T
        start = k
    eig = np.zeros(N)
    for nu in range(N):
        e = 0.0 if abs(ei[nu]) > 1e-12 else er[nu]
        if abs(ei[nu]) > 1e-12:
            Y[:, nu] = 0.0
        f = 0.0
        if e > SMALL_OMEGA2:
            e = np.sqrt(e)
            sn = 2.0 / e * (Y[:, nu] @ am @ Y[:, nu])
            if sn < 0:
                e = -e
            f = 1.0 / np.sqrt(abs(sn))
        elif e != 0.0:
            e = 0.0
        eig[nu] = e
        Y[:, nu] *= f
    return Y, eig
