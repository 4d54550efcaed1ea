"""Generate tests/golden/ac_cas_n64.npz: a 64-basis AC-CAS case (6 inactive,
CAS(4,4), ERI factor rank 300, 5 Gauss-Legendre points) with its inputs and
the oracle's outputs. Run from the repository root:

    python tests/golden/make_golden.py
"""
import sys
import time
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parents[2]
sys.path.insert(0, str(ROOT))

from gammcor_gb300 import synth  # noqa: E402
from oracle import ac_cas_ref as R  # noqa: E402


def main(seed: int = 0):
    s = synth.make_system(**synth.CFG_SMALL, seed=seed)
    G = s.ao_eri_packed()
    num0, num1 = R.prepare_nums(s.occ, s.nele)
    assert (num0, num1) == (s.nin, s.nact)
    ffoo, fofo = R.transform_fofo_ffoo(s.cmo, G, num0, num1)
    indn = R.pair_space(s.occ, s.nele)
    t0 = time.time()
    ecas, ecorr, ws, x, w = R.acecorr(s.occ, s.xone, indn, s.nin, s.nact, ffoo, fofo, s.rdm2act,
                                      ngrid=5)
    print(f"seed {seed}: N={len(indn)} E_CAS={ecas:.12f} (CI {s.e_cas:.12f}) "
          f"ECorr={ecorr:.12f} W={ws} [{time.time() - t0:.0f}s]")
    # the 8-point rule of the batched configurations, for the measured form's tests
    _, ecorr8, ws8, x8, w8 = R.acecorr(s.occ, s.xone, indn, s.nin, s.nact, ffoo, fofo,
                                       s.rdm2act, ngrid=8)
    print(f"8 points: ECorr={ecorr8:.12f}")
    np.savez_compressed(
        Path(__file__).parent / "ac_cas_n64.npz", n=s.n, nin=s.nin, nact=s.nact, rank=s.rank,
        seed=seed, nele=s.nele, lfac=s.lfac, cmo=s.cmo, occ=s.occ, xone=s.xone,
        rdm2act=s.rdm2act, indn=indn, ngrid=5, x=x, w=w, ecas=ecas, ecorr=ecorr,
        w_lambda=np.array(ws), x8=x8, w8=w8, ecorr8=ecorr8, w_lambda8=np.array(ws8),
        e_ci=s.e_cas, fock_diag=np.asarray(s.extra.get("fock_diag", np.zeros(s.n))),
        ffoo_sum=ffoo.sum(), fofo_sum=fofo.sum())


if __name__ == "__main__":
    main(int(sys.argv[1]) if len(sys.argv) > 1 else 0)
