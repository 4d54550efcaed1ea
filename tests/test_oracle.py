"""CPU checks of the oracle and the generator (no GPU).

The reference cannot be compiled here and ships no regression outputs, so
parity of the oracle with reference-produced numbers is unpinned; these tests
pin the restatement by the invariants the reference's own algebra implies.
"""
import numpy as np
import pytest

from gammcor_gb300 import synth
from oracle import ac_cas_ref as R
from oracle import incore_ref as IC

from .helpers import oracle_integrals, small_system


@pytest.fixture(scope="module")
def sys16():
    s = small_system()
    G, ffoo, fofo = oracle_integrals(s)
    return s, G, ffoo, fofo


def test_gauleg_matches_legendre_nodes():
    for n in (1, 2, 5, 8, 12):
        x, w = R.gauleg(0.0, 1.0, n)
        xr, wr = np.polynomial.legendre.leggauss(n)
        np.testing.assert_allclose(np.sort(x), 0.5 * (np.sort(xr) + 1), atol=1e-14)
        np.testing.assert_allclose(np.sort(w), np.sort(0.5 * wr), atol=1e-14)
        assert abs(w.sum() - 1.0) < 1e-14


def test_rdm_energy_equals_ci_energy(sys16):
    s, G, ffoo, fofo = sys16
    indn = R.pair_space(s.occ, s.nele)
    _, _, ecas = R.ab_cas_fofo(s.occ, s.xone, np.eye(s.n), indn, s.nin, s.nact, ffoo, fofo,
                               s.rdm2act, 0.5)
    assert abs(ecas - s.e_cas) < 1e-10


def test_transform_equals_einsum(sys16):
    s, G, ffoo, fofo = sys16
    n, nocc = s.n, s.nocc
    C = s.cmo
    co = C[:, :nocc]
    ff4 = synth.mo_eri_from_factor(s.lfac, n, co, co, C, C)
    fo4 = synth.mo_eri_from_factor(s.lfac, n, C, co, C, co)
    np.testing.assert_allclose(ffoo, ff4.transpose(1, 0, 3, 2).reshape(nocc * nocc, n * n), atol=1e-12)
    np.testing.assert_allclose(fofo, fo4.transpose(1, 0, 3, 2).reshape(n * nocc, n * nocc), atol=1e-12)


def test_prepare_nums_and_pairs(sys16):
    s, *_ = sys16
    assert R.prepare_nums(s.occ, s.nele) == (s.nin, s.nact)
    indn = R.pair_space(s.occ, s.nele)
    n, nin, nocc = s.n, s.nin, s.nocc
    nvirt = n - nocc
    assert len(indn) == n * (n - 1) // 2 - nin * (nin - 1) // 2 - nvirt * (nvirt - 1) // 2
    assert np.all(indn[:, 0] > indn[:, 1]) and np.all(indn[:, 1] <= nocc)


def test_pairs_drop_degenerate_and_quasi_virtual():
    occ = np.array([1.0, 1.0, 0.6, 0.6, 1e-9, 0.0, 0.0])
    indn = R.pair_space(occ, nele=3)
    pairs = {tuple(p) for p in indn}
    assert (4, 3) not in pairs          # |n3-n4|/n3 < ThrSelAct
    assert (6, 5) not in pairs          # n5+n6 <= ThrQVirt
    assert (2, 1) not in pairs          # both inactive
    assert (7, 6) not in pairs          # both virtual
    assert (6, 3) in pairs


@pytest.mark.parametrize("lam", [0.0, 0.37, 1.0])
def test_fofo_assembly_equals_incore(sys16, lam):
    s, G, ffoo, fofo = sys16
    n = s.n
    V = synth.mo_eri_from_factor(s.lfac, n, s.cmo, s.cmo, s.cmo, s.cmo)
    indn = R.pair_space(s.occ, s.nele)
    abp, abm, e1 = R.ab_cas_fofo(s.occ, s.xone, np.eye(n), indn, s.nin, s.nact, ffoo, fofo,
                                 s.rdm2act, lam)
    bp, bm, e2 = IC.ab_cas_incore(V, s.occ, synth.unpack_sym(s.xone, n),
                                  synth.unpack_rdm2act(s.rdm2act, s.nact), s.nin, s.nact, indn, lam)
    scale = max(np.abs(abp).max(), np.abs(abm).max())
    assert np.abs(abp - bp).max() < 1e-12 * scale
    assert np.abs(abm - bm).max() < 1e-12 * scale
    assert abs(e1 - e2) < 1e-10
    Y, eig, _ = R.erpasymm1(abp, abm)
    w1 = R.ac_ene_erpa_fofo(Y, eig, s.occ, s.nin, s.nact, indn, fofo)
    w2 = IC.ac_ene_erpa_incore(V, Y, eig, s.occ, s.nin, s.nact, indn)
    assert abs(w1 - w2) < 1e-12 * max(1.0, abs(w1))


def test_assembly_is_affine_in_lambda(sys16):
    s, G, ffoo, fofo = sys16
    indn = R.pair_space(s.occ, s.nele)
    mats = [R.ab_cas_fofo(s.occ, s.xone, np.eye(s.n), indn, s.nin, s.nact, ffoo, fofo,
                          s.rdm2act, lam)[:2] for lam in (0.0, 0.3, 1.0)]
    for k in range(2):
        a0, a3, a1 = mats[0][k], mats[1][k], mats[2][k]
        np.testing.assert_allclose(a3, 0.7 * a0 + 0.3 * a1, atol=1e-11 * np.abs(a1).max())


def test_erpa_residual_and_normalisation(sys16):
    s, G, ffoo, fofo = sys16
    indn = R.pair_space(s.occ, s.nele)
    abp, abm, _ = R.ab_cas_fofo(s.occ, s.xone, np.eye(s.n), indn, s.nin, s.nact, ffoo, fofo,
                                s.rdm2act, 0.6)
    ap = 0.5 * (abp + abp.T)
    am = 0.5 * (abm + abm.T)
    Y, eig, _ = R.erpasymm1(abp, abm)
    keep = eig > 1e-3
    Yk, om = Y[:, keep], eig[keep]
    res = ap @ am @ Yk - Yk * om[None, :] ** 2
    assert np.abs(res).max() < 1e-8 * np.abs(ap @ am).max()
    norm = 2.0 / om * np.einsum('iv,ij,jv->v', Yk, am, Yk)
    np.testing.assert_allclose(norm, 1.0, atol=1e-10)


def test_cholesky_form_gives_same_integrand(sys16):
    """Y = L u / sqrt(2 w) with A+ = L L^T reproduces W of ERPASYMM1."""
    s, G, ffoo, fofo = sys16
    indn = R.pair_space(s.occ, s.nele)
    abp, abm, _ = R.ab_cas_fofo(s.occ, s.xone, np.eye(s.n), indn, s.nin, s.nact, ffoo, fofo,
                                s.rdm2act, 0.6)
    Y, eig, _ = R.erpasymm1(abp, abm)
    ap = 0.5 * (abp + abp.T)
    am = 0.5 * (abm + abm.T)
    L = np.linalg.cholesky(ap)
    w2, U = np.linalg.eigh(L.T @ am @ L)
    om = np.where(w2 > 1e-6, np.sqrt(np.abs(w2)), w2)
    Yc = np.where(w2 > 1e-6, (L @ U) / np.sqrt(2 * np.abs(om)), L @ U)
    wa = R.ac_ene_erpa_fofo(Y, eig, s.occ, s.nin, s.nact, indn, fofo)
    wb = R.ac_ene_erpa_fofo(Yc, om, s.occ, s.nin, s.nact, indn, fofo)
    assert abs(wa - wb) < 1e-10 * max(1.0, abs(wa))


def test_golden_fixture_reproduces():
    """The committed 64-basis fixture (5-point AC-CAS) is reproduced by the oracle's
    cheap parts: inputs regenerate bit-for-bit in meaning and E_CAS matches."""
    from pathlib import Path
    p = Path(__file__).parent / "golden" / "ac_cas_n64.npz"
    if not p.exists():
        pytest.skip("fixture not generated")
    d = np.load(p)
    x, w = R.gauleg(0.0, 1.0, int(d["ngrid"]))
    np.testing.assert_allclose(x, d["x"], atol=1e-15)
    assert abs(np.dot(w, d["w_lambda"]) - float(d["ecorr"])) < 1e-12


@pytest.mark.parametrize("cfg", [dict(n=14, nin=0, nact=4, rank=50),   # no inactive orbitals
                                 dict(n=14, nin=3, nact=2, rank=50),   # CAS(2,2)
                                 dict(n=12, nin=2, nact=6, rank=40)])  # CAS(6,6)
def test_edge_shapes_fofo_equals_incore(cfg):
    """Shapes at the edges of the configs: E_CAS equals the CI energy, the FOFO
    assembly and integrand equal the in-core restatement, and a one-point rule is
    W(1/2)."""
    s = synth.make_system(**cfg, seed=1)
    G, ffoo, fofo = oracle_integrals(s)
    n = s.n
    indn = R.pair_space(s.occ, s.nele)
    V = synth.mo_eri_from_factor(s.lfac, n, s.cmo, s.cmo, s.cmo, s.cmo)
    abp, abm, e1 = R.ab_cas_fofo(s.occ, s.xone, np.eye(n), indn, s.nin, s.nact, ffoo, fofo,
                                 s.rdm2act, 0.5)
    bp, bm, e2 = IC.ab_cas_incore(V, s.occ, synth.unpack_sym(s.xone, n),
                                  synth.unpack_rdm2act(s.rdm2act, s.nact), s.nin, s.nact, indn, 0.5)
    scale = max(np.abs(abp).max(), np.abs(abm).max())
    assert np.abs(abp - bp).max() < 1e-12 * scale and np.abs(abm - bm).max() < 1e-12 * scale
    assert abs(e1 - s.e_cas) < 1e-10 and abs(e2 - s.e_cas) < 1e-10
    Y, eig, _ = R.erpasymm1(abp, abm)
    w1 = R.ac_ene_erpa_fofo(Y, eig, s.occ, s.nin, s.nact, indn, fofo)
    w2 = IC.ac_ene_erpa_incore(V, Y, eig, s.occ, s.nin, s.nact, indn)
    assert abs(w1 - w2) < 1e-12 * max(1.0, abs(w1))
    ecas, ecorr, ws, x, w = R.acecorr(s.occ, s.xone, indn, s.nin, s.nact, ffoo, fofo, s.rdm2act,
                                      ngrid=1)
    assert x[0] == pytest.approx(0.5) and w[0] == pytest.approx(1.0)
    assert abs(ecorr - w1) < 1e-12 * max(1.0, abs(w1))


def test_ac0_oracle_is_the_first_order_connection():
    """AC0CAS_FOFO's energy is the linearised adiabatic connection: with W(0) = 0,
    E_AC0 = W(0) + W'(0)/2, W' from a central difference of the line-faithful
    ACEInteg_FOFO restatement (an independent pin of the AC0 oracle)."""
    from oracle import ac0_ref as A
    from gammcor_gb300 import synth
    s = synth.make_system(n=20, nin=2, nact=2, rank=80, seed=1)
    ffoo, fofo = R.transform_fofo_ffoo(s.cmo, s.ao_eri_packed(), s.nin, s.nact)
    indn = R.pair_space(s.occ, s.nele)
    e0, etot = A.ac0cas_fofo(s.occ, s.xone, np.eye(s.n), indn, s.nin, s.nact, ffoo, fofo,
                             s.rdm2act)

    def W(lam):
        return R.ace_integ_fofo(s.occ, s.xone, indn, s.nin, s.nact, ffoo, fofo, s.rdm2act, lam)[0]
    h = 1e-4
    w0, wp = W(0.0), (W(h) - W(-h)) / (2 * h)
    assert abs(w0) < 1e-12
    assert abs(e0 - (w0 + 0.5 * wp)) < 1e-9, (e0, w0 + 0.5 * wp)
    assert abs(etot - s.e_cas) < 1e-10


def test_acfreq_oracle_first_order_is_ac0():
    """Truncated after the first-order term (Max_Cn = 1), the frequency integral of
    WIter_FOFO must reproduce the AC0 energy (W(0) + W'(0)/2) once the frequency
    grid is fine enough: an independent pin of the ACFREQ oracle's series and
    frequency quadrature."""
    from oracle import ac0_ref as A
    from oracle import acfreq_ref as F
    from gammcor_gb300 import synth
    s = synth.make_system(n=20, nin=2, nact=2, rank=80, seed=1)
    ffoo, fofo = R.transform_fofo_ffoo(s.cmo, s.ao_eri_packed(), s.nin, s.nact)
    indn = R.pair_space(s.occ, s.nele)
    e0, _ = A.ac0cas_fofo(s.occ, s.xone, np.eye(s.n), indn, s.nin, s.nact, ffoo, fofo, s.rdm2act)
    e1, ecas = F.witer_fofo(s.occ, s.xone, np.eye(s.n), indn, s.nin, s.nact, ffoo, fofo,
                            s.rdm2act, ngrid=120, max_cn=1)
    assert abs(e1 - e0) < 1e-10, (e1, e0)
    assert abs(ecas - s.e_cas) < 1e-10
    # the reference settings (25 points, third order) stay close to the lambda quadrature
    e3, _ = F.witer_fofo(s.occ, s.xone, np.eye(s.n), indn, s.nin, s.nact, ffoo, fofo, s.rdm2act)
    eac = R.acecorr(s.occ, s.xone, indn, s.nin, s.nact, ffoo, fofo, s.rdm2act, ngrid=8)[1]
    assert abs(e3 - eac) < 1e-3 * abs(eac)


def test_erpavec_oracle_equals_erpasymm1_for_positive_definite_a_plus():
    """ERPAVEC (interpa.f:962-1070) and ERPASYMM1 give the same W(lambda) when A+B
    is positive definite: the pin of the ERPAVEC restatement."""
    from oracle import erpavec_ref as V
    s = small_system(n=16, nin=2, nact=4, rank=64, seed=0)
    G, ffoo, fofo = oracle_integrals(s)
    indn = R.pair_space(s.occ, s.nele)
    for lam in (0.3, 0.9):
        abp, abm, _ = R.ab_cas_fofo(s.occ, s.xone, np.eye(s.n), indn, s.nin, s.nact, ffoo, fofo,
                                    s.rdm2act, lam)
        Y1, e1, _ = R.erpasymm1(abp, abm)
        Y2, e2 = V.erpavec(abp, abm)
        w1 = R.ac_ene_erpa_fofo(Y1, e1, s.occ, s.nin, s.nact, indn, fofo)
        w2 = R.ac_ene_erpa_fofo(Y2, e2, s.occ, s.nin, s.nact, indn, fofo)
        assert abs(w1 - w2) < 1e-11
