"""The multi-threaded CPU port (the CPU baseline the bench times) against the
line-faithful oracle, on small systems: A+-B and E_CAS at several lambda, the
FOFO/FFOO transform from the ERI factor, and the whole lambda quadrature."""
import numpy as np
import pytest

from gammcor_gb300 import synth
from oracle import ac_cas_ref as R
from oracle import cpu_port as P


@pytest.fixture(scope="module")
def case():
    s = synth.make_system(n=20, nin=3, nact=4, rank=70, seed=2)
    ffoo, fofo = R.transform_fofo_ffoo(s.cmo, s.ao_eri_packed(), s.nin, s.nact)
    return s, ffoo, fofo, R.pair_space(s.occ, s.nele)


def test_transform_from_factor(case):
    s, ffoo, fofo, _ = case
    ff, fo = P.transform_factored(s.cmo, s.lfac, s.nin, s.nact, chunk=16)
    assert np.abs(ff - ffoo).max() < 1e-12
    assert np.abs(fo - fofo).max() < 1e-12


@pytest.mark.parametrize("lam", [0.0, 0.37, 1.0])
def test_ab_cas_fofo(case, lam):
    s, ffoo, fofo, indn = case
    a, b, e = R.ab_cas_fofo(s.occ, s.xone, np.eye(s.n), indn, s.nin, s.nact, ffoo, fofo,
                            s.rdm2act, lam)
    a2, b2, e2 = P.ab_cas_fofo(s.occ, s.xone, indn, s.nin, s.nact, ffoo, fofo, s.rdm2act, lam)
    assert np.abs(a - a2).max() < 1e-12 * np.abs(a).max()
    assert np.abs(b - b2).max() < 1e-11 * np.abs(b).max()
    assert abs(e - e2) < 1e-10


def test_acecorr(case):
    s, ffoo, fofo, indn = case
    ecas, ecorr, ws, _, _ = R.acecorr(s.occ, s.xone, indn, s.nin, s.nact, ffoo, fofo, s.rdm2act,
                                      ngrid=5)
    ecas2, ecorr2, ws2 = P.acecorr(s.occ, s.xone, indn, s.nin, s.nact, ffoo, fofo, s.rdm2act,
                                   ngrid=5)
    assert abs(ecorr - ecorr2) < 1e-12
    assert abs(ecas - ecas2) < 1e-10
    np.testing.assert_allclose(ws2, ws, atol=1e-12)
