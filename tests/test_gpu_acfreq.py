"""ACFREQ (WIter_FOFO, ac_fofo.f90:1-181) through the C ABI against the oracle
(oracle/acfreq_ref.py, the reference's LU form at every frequency).

Tolerances: 1e-9 Eh with FP64 products; 5e-9 Eh with the FP64TC5 sliced
products and the refined eigensolve. The frequency grid matches FreqGrid to
1e-13 relative."""
import numpy as np
import pytest
import torch

from gammcor_gb300 import api, synth
from oracle import ac_cas_ref as R
from oracle import acfreq_ref as F

pytestmark = pytest.mark.gpu
DEV = "cuda:0"


def t(x):
    return torch.as_tensor(np.ascontiguousarray(x), dtype=torch.float64, device=DEV)


def test_freq_grid(gpu_lib):
    for nf in (1, 18, 25):
        x, w = api.freq_grid(nf)
        xr, wr = F.freq_grid(nf)
        # x0 (1 + x) / (1 - x) amplifies the nodes' last bits by 1 / (1 - x) near x = 1
        np.testing.assert_allclose(x, xr, rtol=1e-13, atol=1e-15)
        np.testing.assert_allclose(w, wr, rtol=1e-12, atol=1e-15)


@pytest.mark.parametrize("n,nin,nact,seed", [(16, 2, 4, 0), (20, 2, 2, 1), (24, 3, 4, 3)])
@pytest.mark.parametrize("precision,mode,tol", [("fp64", "cholesky", 1e-9),
                                                ("fp64tc5", "refined", 5e-9)])
def test_acfreq_matches_oracle(gpu_lib, n, nin, nact, seed, precision, mode, tol):
    s = synth.make_system(n=n, nin=nin, nact=nact, rank=4 * n, seed=seed)
    ffoo, fofo = R.transform_fofo_ffoo(s.cmo, s.ao_eri_packed(), s.nin, s.nact)
    indn = R.pair_space(s.occ, s.nele)
    e, ecas = F.witer_fofo(s.occ, s.xone, np.eye(n), indn, nin, nact, ffoo, fofo, s.rdm2act)
    ge, gecas = api.ac_freq_fofo(s.occ, s.xone, indn, nact, nin, t(ffoo), t(fofo), s.rdm2act,
                                 precision=precision, erpa_mode=mode)
    assert abs(ge - e) < tol, (ge, e)
    assert abs(gecas - ecas) < 1e-9


def test_acfreq_indefinite_a_plus_b_takes_the_lu_form(gpu_lib):
    """A+B(0) not positive definite: no Cholesky factor, so the reference's LU form
    runs at every frequency (FP64) and still matches the oracle."""
    s = synth.make_system(n=18, nin=3, nact=4, rank=72, seed=1, eri_scale=0.25)
    ffoo, fofo = R.transform_fofo_ffoo(s.cmo, s.ao_eri_packed(), s.nin, s.nact)
    indn = R.pair_space(s.occ, s.nele)
    a0p, _, _ = R.ab_cas_fofo(s.occ, s.xone, np.eye(s.n), indn, s.nin, s.nact, ffoo, fofo,
                              s.rdm2act, 0.0)
    assert np.linalg.eigvalsh(0.5 * (a0p + a0p.T)).min() < 0
    e, _ = F.witer_fofo(s.occ, s.xone, np.eye(s.n), indn, s.nin, s.nact, ffoo, fofo, s.rdm2act)
    ge, _ = api.ac_freq_fofo(s.occ, s.xone, indn, s.nact, s.nin, t(ffoo), t(fofo), s.rdm2act,
                             precision="fp64tc5", erpa_mode="refined")
    assert abs(ge - e) < 1e-9 * max(1.0, abs(e)), (ge, e)


def test_acfreq_series_orders_and_ure(gpu_lib):
    s = synth.make_system(n=18, nin=2, nact=4, rank=72, seed=6)
    ffoo, fofo = R.transform_fofo_ffoo(s.cmo, s.ao_eri_packed(), s.nin, s.nact)
    indn = R.pair_space(s.occ, s.nele)
    q, _ = np.linalg.qr(np.random.default_rng(4).standard_normal((s.n, s.n)))
    ure = np.eye(s.n) + 0.05 * (q - np.eye(s.n))
    for nf, cn in ((18, 1), (25, 2), (25, 5)):
        e, _ = F.witer_fofo(s.occ, s.xone, ure, indn, s.nin, s.nact, ffoo, fofo, s.rdm2act,
                            ngrid=nf, max_cn=cn)
        ge, _ = api.ac_freq_fofo(s.occ, s.xone, indn, s.nact, s.nin, t(ffoo), t(fofo), s.rdm2act,
                                 nfreq=nf, max_cn=cn, ure=ure)
        assert abs(ge - e) < 1e-9, (nf, cn, ge, e)
