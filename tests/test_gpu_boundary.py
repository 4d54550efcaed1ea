"""Arguments of the reference routines that the plain entry points leave at
their LdInteg values, checked through the C ABI against the oracle:

* AB_CAS_FOFO's URe (HNO = URe h URe^T, abfofo.f90:97-100) with a random
  orthogonal rotation, and its AB1 form (abfofo.f90:109-171, 260-263);
* ERPASYMM1's APLSQRT output (A+ overwritten with A+^1/2, interpa.f:1652-1716).

Tolerances as in the parity tests: A+-B 1e-10 relative to the largest
element, E_CAS 1e-9 Eh; A+^1/2 1e-10 relative.
"""
import numpy as np
import pytest
import torch

from gammcor_gb300 import api
from oracle import ac_cas_ref as R

from .helpers import oracle_integrals, small_system

pytestmark = pytest.mark.gpu
DEV = "cuda:0"


def t(x):
    return torch.as_tensor(np.ascontiguousarray(x), dtype=torch.float64, device=DEV)


@pytest.fixture(scope="module")
def case(gpu_lib):
    s = small_system(n=24, nin=3, nact=4, rank=90, seed=3)
    G, ffoo, fofo = oracle_integrals(s)
    return s, ffoo, fofo, R.pair_space(s.occ, s.nele)


def rel(a, b):
    return np.abs(a - b).max() / np.abs(b).max()


@pytest.mark.parametrize("ab1,lam", [(False, 0.4), (True, 0.6), (True, 1.0)])
def test_ab_cas_fofo_ure_ab1(case, ab1, lam):
    s, ffoo, fofo, indn = case
    q, _ = np.linalg.qr(np.random.default_rng(7).standard_normal((s.n, s.n)))
    ure = np.eye(s.n) + 0.05 * (q - np.eye(s.n))   # a non-trivial, non-orthogonal rotation too
    abp, abm, e = R.ab_cas_fofo(s.occ, s.xone, ure, indn, s.nin, s.nact, ffoo, fofo, s.rdm2act,
                                lam, ab1=ab1)
    gp, gm, ge = api.ab_cas_fofo(s.occ, s.xone, indn, s.nact, s.nin, t(ffoo), t(fofo), s.rdm2act,
                                 lam, ure=ure, ab1=ab1)
    assert rel(gp.cpu().numpy(), abp) < 1e-10
    assert rel(gm.cpu().numpy(), abm) < 1e-10
    assert abs(ge - e) < 1e-9


def test_ab1_is_the_lambda_derivative(case):
    s, ffoo, fofo, indn = case
    a0p, a0m, _ = api.ab_cas_fofo(s.occ, s.xone, indn, s.nact, s.nin, t(ffoo), t(fofo),
                                  s.rdm2act, 0.0)
    a1p, a1m, _ = api.ab_cas_fofo(s.occ, s.xone, indn, s.nact, s.nin, t(ffoo), t(fofo),
                                  s.rdm2act, 1.0)
    dp, dm, _ = api.ab_cas_fofo(s.occ, s.xone, indn, s.nact, s.nin, t(ffoo), t(fofo), s.rdm2act,
                                1.0, ab1=True)
    sym = lambda x: 0.5 * (x + x.T)  # noqa: E731
    ref_p = sym((a1p - a0p).cpu().numpy())
    ref_m = sym((a1m - a0m).cpu().numpy())
    assert rel(dp.cpu().numpy(), ref_p) < 1e-10
    assert rel(dm.cpu().numpy(), ref_m) < 1e-10


def test_erpasymm1_aplsqrt(case):
    s, ffoo, fofo, indn = case
    abp, abm, _ = R.ab_cas_fofo(s.occ, s.xone, np.eye(s.n), indn, s.nin, s.nact, ffoo, fofo,
                                s.rdm2act, 0.5)
    Y, eig, P = R.erpasymm1(abp, abm)
    gy, ge, gP = api.erpasymm1_aplsqrt(t(abp), t(abm))
    assert rel(gP.cpu().numpy(), P) < 1e-10
    np.testing.assert_allclose(ge.cpu().numpy(), eig, rtol=1e-9, atol=1e-12)
    w = R.ac_ene_erpa_fofo(Y, eig, s.occ, s.nin, s.nact, indn, fofo)
    gw = api.ace_ne_erpa_fofo(gy, ge, s.occ, indn, s.nact, s.nin, t(fofo))
    assert abs(gw - w) < 1e-9
