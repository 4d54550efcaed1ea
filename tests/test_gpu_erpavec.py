"""ERPAVEC (interpa.f:962-1070), the GC_ERPA_VEC mode, through the C ABI against
the oracle (oracle/erpavec_ref.py): W(lambda) within 1e-9 Eh, on a positive
definite A+B and on systems whose A+B is indefinite (de-excitations with
negative omega, complex and negative modes dropped), as state-averaged
references give; and the whole quadrature with ERPAVEC at every point."""
import numpy as np
import pytest
import torch

from gammcor_gb300 import api, synth
from oracle import ac_cas_ref as R
from oracle import erpavec_ref as V

pytestmark = pytest.mark.gpu
DEV = "cuda:0"


def t(x):
    return torch.as_tensor(np.ascontiguousarray(x), dtype=torch.float64, device=DEV)


CASES = [dict(n=16, nin=2, nact=4, rank=64, seed=0),
         dict(n=18, nin=3, nact=4, rank=72, seed=1, eri_scale=0.25),
         dict(n=18, nin=3, nact=4, rank=72, seed=6, eri_scale=0.25)]


@pytest.mark.parametrize("case", CASES)
def test_erpavec_integrand_matches_oracle(gpu_lib, case):
    s = synth.make_system(**case)
    ffoo, fofo = R.transform_fofo_ffoo(s.cmo, s.ao_eri_packed(), s.nin, s.nact)
    indn = R.pair_space(s.occ, s.nele)
    for lam in (0.4, 1.0):
        abp, abm, _ = R.ab_cas_fofo(s.occ, s.xone, np.eye(s.n), indn, s.nin, s.nact, ffoo, fofo,
                                    s.rdm2act, lam)
        Y, e = V.erpavec(abp, abm)
        w = R.ac_ene_erpa_fofo(Y, e, s.occ, s.nin, s.nact, indn, fofo)
        gy, ge = api.erpasymm1(t(abp), t(abm), mode="vec")
        gw = api.ace_ne_erpa_fofo(gy, ge, s.occ, indn, s.nact, s.nin, t(fofo))
        assert abs(gw - w) < 1e-9, (lam, gw, w)
        # the same excitation energies, de-excitations (omega < 0) included
        np.testing.assert_allclose(np.sort(ge.cpu().numpy()), np.sort(e), atol=1e-9)


def test_acecorr_with_erpavec(gpu_lib):
    s = synth.make_system(**CASES[1])
    ffoo, fofo = R.transform_fofo_ffoo(s.cmo, s.ao_eri_packed(), s.nin, s.nact)
    indn = R.pair_space(s.occ, s.nele)
    x, w = R.gauleg(0.0, 1.0, 5)
    ws = []
    for lam in x:
        abp, abm, ecas = R.ab_cas_fofo(s.occ, s.xone, np.eye(s.n), indn, s.nin, s.nact, ffoo,
                                       fofo, s.rdm2act, lam)
        Y, e = V.erpavec(abp, abm)
        ws.append(R.ac_ene_erpa_fofo(Y, e, s.occ, s.nin, s.nact, indn, fofo))
    gecas, gecorr, gws = api.acecorr(s.occ, s.xone, indn, s.nact, s.nin, t(ffoo), t(fofo),
                                     s.rdm2act, ngrid=5, erpa_mode="vec")
    np.testing.assert_allclose(gws, ws, atol=1e-9)
    assert abs(gecorr - float(np.dot(w, ws))) < 1e-9
