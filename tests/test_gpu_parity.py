"""Parity of the CUDA path with the oracle, through the C ABI.

Tolerances (FP64 path): integrals 1e-10 absolute; A+-B 1e-10 relative to the
largest element; W(lambda) and energies 1e-9 Eh.
"""
import numpy as np
import pytest
import torch

from gammcor_gb300 import api, synth
from oracle import ac_cas_ref as R

from .helpers import oracle_integrals, small_system

pytestmark = pytest.mark.gpu
DEV = "cuda:0"


def t(x):
    return torch.as_tensor(np.ascontiguousarray(x), dtype=torch.float64, device=DEV)


@pytest.fixture(scope="module")
def sys16(gpu_lib):
    s = small_system()
    G, ffoo, fofo = oracle_integrals(s)
    return s, G, ffoo, fofo


@pytest.fixture(scope="module")
def sys24(gpu_lib):
    s = small_system(n=24, nin=3, nact=4, rank=90, seed=3)
    G, ffoo, fofo = oracle_integrals(s)
    return s, G, ffoo, fofo


def gpu_integrals(s, G, precision="fp64"):
    C = t(s.cmo)
    co = C[:, :s.nocc].contiguous()
    Gd = t(G)
    ffoo = api.tran4_gen(s.n, co, co, C, C, Gd, precision=precision)
    fofo = api.tran4_gen(s.n, C, co, C, co, Gd, precision=precision)
    return ffoo, fofo


@pytest.mark.parametrize("fixture", ["sys16", "sys24"])
def test_tran4_gen_matches_oracle(fixture, request):
    s, G, ffoo, fofo = request.getfixturevalue(fixture)
    gff, gfo = gpu_integrals(s, G)
    assert np.abs(gff.cpu().numpy() - ffoo).max() < 1e-10
    assert np.abs(gfo.cpu().numpy() - fofo).max() < 1e-10


def test_tran4_factored_matches_oracle(sys24):
    s, G, ffoo, fofo = sys24
    C = t(s.cmo)
    co = C[:, :s.nocc].contiguous()
    L = t(s.lfac)
    gfo = api.tran4_factored(s.n, L, C, co, C, co)
    gff = api.tran4_factored(s.n, L, co, co, C, C)
    assert np.abs(gff.cpu().numpy() - ffoo).max() < 1e-10
    assert np.abs(gfo.cpu().numpy() - fofo).max() < 1e-10


def test_tran4_gen_rectangular_blocks(sys16):
    """Distinct nA, nB, nC, nD exercise every dimension of the record layout."""
    s, G, *_ = sys16
    C = s.cmo
    blocks = [C[:, :3], C[:, :5], C[:, :7], C[:, :11]]
    ref = R.tran4_gen(s.n, *blocks, G)
    out = api.tran4_gen(s.n, *[t(b) for b in blocks], t(G))
    assert np.abs(out.cpu().numpy() - ref).max() < 1e-10


@pytest.mark.parametrize("precision,tol", [("fp64", 1e-10), ("fp64tc5", 1e-10)])
def test_tran4_gen_two_orbital_sets(sys16, precision, tol):
    """The SAPT calls of tran4_gen (sapt_main.f90:435-522) put the orbitals of two monomers
    in the four slots, e.g. 'TWOMOAB': A's occupied, A's active and virtual, B's occupied,
    B's active and virtual. Here B's orbitals are an independent orthogonal rotation of
    A's, so every slot holds different coefficients."""
    s, G, *_ = sys16
    CA = s.cmo
    q, _ = np.linalg.qr(np.random.default_rng(21).standard_normal((s.n, s.n)))
    CB = CA @ q
    blocks = [CA[:, :s.nocc], CA[:, s.nin:], CB[:, :s.nocc], CB[:, s.nin:]]
    ref = R.tran4_gen(s.n, *blocks, G)
    out = api.tran4_gen(s.n, *[t(np.ascontiguousarray(b)) for b in blocks], t(G),
                        precision=precision)
    assert np.abs(out.cpu().numpy() - ref).max() < tol


@pytest.mark.parametrize("lam", [0.0, 0.2113248654, 1.0])
def test_ab_cas_fofo_matches_oracle(sys24, lam):
    s, G, ffoo, fofo = sys24
    indn = R.pair_space(s.occ, s.nele)
    abp, abm, e = R.ab_cas_fofo(s.occ, s.xone, np.eye(s.n), indn, s.nin, s.nact, ffoo, fofo,
                                s.rdm2act, lam)
    gp, gm, ge = api.ab_cas_fofo(s.occ, s.xone, indn, s.nact, s.nin, t(ffoo), t(fofo), s.rdm2act, lam)
    scale = max(np.abs(abp).max(), np.abs(abm).max())
    assert np.abs(gp.cpu().numpy() - abp).max() < 1e-10 * scale
    assert np.abs(gm.cpu().numpy() - abm).max() < 1e-10 * scale
    assert abs(ge - e) < 1e-9
    assert abs(ge - s.e_cas) < 1e-9


@pytest.mark.parametrize("mode", ["symm1", "cholesky"])
def test_erpa_and_integrand_match_oracle(sys24, mode):
    s, G, ffoo, fofo = sys24
    indn = R.pair_space(s.occ, s.nele)
    abp, abm, _ = R.ab_cas_fofo(s.occ, s.xone, np.eye(s.n), indn, s.nin, s.nact, ffoo, fofo,
                                s.rdm2act, 0.5)
    Y, eig, _ = R.erpasymm1(abp, abm)
    w_ref = R.ac_ene_erpa_fofo(Y, eig, s.occ, s.nin, s.nact, indn, fofo)
    gy, geig = api.erpasymm1(t(abp), t(abm), mode=mode)
    np.testing.assert_allclose(np.sort(geig.cpu().numpy()), np.sort(eig), rtol=1e-9, atol=1e-10)
    w = api.ace_ne_erpa_fofo(gy, geig, s.occ, indn, s.nact, s.nin, t(fofo))
    assert abs(w - w_ref) < 1e-9
    # integrand alone on the oracle's eigenvectors
    w2 = api.ace_ne_erpa_fofo(t(Y), t(eig), s.occ, indn, s.nact, s.nin, t(fofo))
    assert abs(w2 - w_ref) < 1e-9


@pytest.mark.parametrize("mode", ["symm1", "cholesky"])
def test_acecorr_matches_oracle(sys16, mode):
    s, G, ffoo, fofo = sys16
    indn = R.pair_space(s.occ, s.nele)
    ecas, ecorr, ws, x, w = R.acecorr(s.occ, s.xone, indn, s.nin, s.nact, ffoo, fofo, s.rdm2act)
    gff, gfo = gpu_integrals(s, G)
    gecas, gecorr, gws = api.acecorr(s.occ, s.xone, indn, s.nact, s.nin, gff, gfo, s.rdm2act,
                                     ngrid=5, erpa_mode=mode)
    assert abs(gecas - ecas) < 1e-9
    assert abs(gecorr - ecorr) < 1e-9
    np.testing.assert_allclose(gws, ws, atol=1e-9)


def test_acecorr_n64_golden():
    """64-basis, 6 inactive, CAS(4,4), rank 300, 5 lambda points against the
    committed oracle fixture (inputs and oracle outputs)."""
    from pathlib import Path
    p = Path(__file__).parent / "golden" / "ac_cas_n64.npz"
    d = np.load(p)
    n, nin, nact = int(d["n"]), int(d["nin"]), int(d["nact"])
    L = d["lfac"]
    G = t(L) @ t(L).T
    C = t(d["cmo"])
    co = C[:, :nin + nact].contiguous()
    gff = api.tran4_gen(n, co, co, C, C, G.contiguous())
    gfo = api.tran4_gen(n, C, co, C, co, G.contiguous())
    for mode in ("symm1", "cholesky"):
        ecas, ecorr, ws = api.acecorr(d["occ"], d["xone"], d["indn"], nact, nin, gff, gfo,
                                      d["rdm2act"], ngrid=int(d["ngrid"]), erpa_mode=mode)
        assert abs(ecas - float(d["ecas"])) < 1e-9
        assert abs(ecorr - float(d["ecorr"])) < 1e-9, (mode, ecorr, float(d["ecorr"]))
        np.testing.assert_allclose(ws, d["w_lambda"], atol=1e-9)


@pytest.mark.parametrize("precision,tol", [("bf16x3", 5e-5), ("bf16x6", 2e-7), ("fp64tc5", 1e-10),
                                           ("fp64tc6", 1e-10)])
def test_tran4_mixed_precision_error(sys24, precision, tol):
    """Mixed-precision transform vs the FP64 oracle: max |error| per integral."""
    s, G, ffoo, fofo = sys24
    gff, gfo = gpu_integrals(s, G, precision=precision)
    err = max(np.abs(gff.cpu().numpy() - ffoo).max(), np.abs(gfo.cpu().numpy() - fofo).max())
    assert err < tol, err
    C = t(s.cmo)
    co = C[:, :s.nocc].contiguous()
    gfo2 = api.tran4_factored(s.n, t(s.lfac), C, co, C, co, precision=precision)
    assert np.abs(gfo2.cpu().numpy() - fofo).max() < tol


@pytest.mark.parametrize("precision,tol", [("bf16x3", 1e-4), ("bf16x6", 5e-8), ("fp64tc5", 1e-9),
                                           ("fp64tc6", 1e-9)])
def test_integrand_mixed_precision_error(sys24, precision, tol):
    s, G, ffoo, fofo = sys24
    indn = R.pair_space(s.occ, s.nele)
    abp, abm, _ = R.ab_cas_fofo(s.occ, s.xone, np.eye(s.n), indn, s.nin, s.nact, ffoo, fofo,
                                s.rdm2act, 0.5)
    Y, eig, _ = R.erpasymm1(abp, abm)
    w_ref = R.ac_ene_erpa_fofo(Y, eig, s.occ, s.nin, s.nact, indn, fofo)
    w = api.ace_ne_erpa_fofo(t(Y), t(eig), s.occ, indn, s.nact, s.nin, t(fofo), precision=precision)
    assert abs(w - w_ref) < tol, (w, w_ref)
