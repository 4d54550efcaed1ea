"""The refined ERPA form (FP32 eigensolve of L^T A- L refined to FP64 accuracy)
and the batched driver, through the C ABI, against the oracle and numpy.

Tolerances:
- W(lambda) and energies: 1e-9 Eh against the oracle with FP64 and FP64TC6
  products, 5e-9 Eh with FP64TC5 (its products carry ~2^-35 relative error).
- The matrix function sum_nu y_nu y_nu^T, which is all W depends on, on spectra
  with planted clusters of close eigenvalues: 1e-9 of its largest element with
  FP64 products and two iterations, 1e-7 with FP64TC5 products (A- itself then
  enters L^T A- L rounded to ~2^-35, and the smallest omega^2 = 0.05 amplifies
  that), 5e-7 after a single iteration.
"""
import numpy as np
import pytest
import torch

from gammcor_gb300 import api, synth
from gammcor_gb300._lib import GcError
from oracle import ac_cas_ref as R

from .helpers import oracle_integrals, small_system

pytestmark = pytest.mark.gpu
DEV = "cuda:0"


def t(x):
    return torch.as_tensor(np.ascontiguousarray(x), dtype=torch.float64, device=DEV)


@pytest.fixture(scope="module")
def sys24(gpu_lib):
    s = small_system(n=24, nin=3, nact=4, rank=90, seed=3)
    G, ffoo, fofo = oracle_integrals(s)
    return s, G, ffoo, fofo


@pytest.mark.parametrize("precision", ["fp64", "fp64tc5", "fp64tc6"])
@pytest.mark.parametrize("lam", [0.0198550718, 0.5, 0.9801449282])
def test_refined_erpa_matches_oracle(sys24, precision, lam):
    s, G, ffoo, fofo = sys24
    indn = R.pair_space(s.occ, s.nele)
    abp, abm, _ = R.ab_cas_fofo(s.occ, s.xone, np.eye(s.n), indn, s.nin, s.nact, ffoo, fofo,
                                s.rdm2act, lam)
    Y, eig, _ = R.erpasymm1(abp, abm)
    w_ref = R.ac_ene_erpa_fofo(Y, eig, s.occ, s.nin, s.nact, indn, fofo)
    ctx = api.Context(0)
    gy, geig = api.erpasymm1(t(abp), t(abm), mode="refined", precision=precision, ctx=ctx)
    rtol = {"fp64": 1e-9, "fp64tc5": 1e-7, "fp64tc6": 1e-9}[precision]
    np.testing.assert_allclose(np.sort(geig.cpu().numpy()), np.sort(eig), rtol=rtol, atol=1e-10)
    w = api.ace_ne_erpa_fofo(gy, geig, s.occ, indn, s.nact, s.nin, t(fofo), ctx=ctx)
    tol = 5e-9 if precision == "fp64tc5" else 1e-9
    assert abs(w - w_ref) < tol, (w, w_ref)
    st = ctx.eig_refine_stats()
    assert st["solves"] == 1 and st["fallbacks"] == 0, st


def planted_spectrum(N, seed, groups):
    """Symmetric M = Q diag(ev) Q^T with eigenvalues in [0.05, 60] and some
    negative ones, plus groups (start, offsets) of close eigenvalues."""
    rng = np.random.default_rng(seed)
    ev = np.sort(np.concatenate([rng.uniform(-20.0, -1.0, N // 10),
                                 rng.uniform(0.05, 60.0, N - N // 10)]))
    for start, offs in groups:
        ev[start:start + len(offs)] = ev[start] + np.asarray(offs)
    ev = np.sort(ev)
    Q, _ = np.linalg.qr(rng.normal(size=(N, N)))
    M = (Q * ev) @ Q.T
    return 0.5 * (M + M.T), ev


def yyT(Y, eig):
    """sum over kept modes (1e-3 < omega < 1e8) of y y^T."""
    keep = (eig > 1e-3) & (eig < 1e8)
    Yk = Y[:, keep]
    return Yk @ Yk.T


def erpa_identity_plus(M, mode, precision, iterations=2):
    """ERPA with A+ = I and A- = M: omega^2 = eig(M), Y = u / sqrt(2 omega)."""
    N = M.shape[0]
    ctx = api.Context(0)
    ctx.set_eig_refinement(iterations)
    y, e = api.erpasymm1(t(np.eye(N)), t(M), mode=mode, precision=precision, ctx=ctx)
    return y.cpu().numpy(), e.cpu().numpy(), ctx.eig_refine_stats()


@pytest.mark.parametrize("precision", ["fp64", "fp64tc5"])
@pytest.mark.parametrize("iterations", [1, 2])
def test_refined_erpa_clustered_spectrum(gpu_lib, precision, iterations):
    groups = [(100, [0.0, 1e-7, 3e-6]), (200, [0.0, 1e-9, 2e-9, 3e-9, 4e-9]), (50, [0.0, 0.0]),
              (300, [0.0, 1e-4]), (330, list(np.arange(40) * 1e-8))]
    M, ev = planted_spectrum(400, 11, groups)
    w, U = np.linalg.eigh(M)
    om = np.sqrt(np.abs(w))
    ref = yyT(U / np.sqrt(2 * np.where(w > 1e-6, om, 1.0))[None, :], np.where(w > 1e-6, om, w))
    Y, e, st = erpa_identity_plus(M, "refined", precision, iterations)
    got = yyT(Y, e)
    assert st["fallbacks"] == 0 and st["max_cluster"] >= 2, st
    # one iteration from cuSOLVER's FP32 eigenvectors leaves ~angle^2 ~ 1e-8 behind
    tol = {("fp64", 2): 1e-9, ("fp64tc5", 2): 1e-7}.get((precision, iterations), 5e-7)
    assert np.abs(got - ref).max() < tol * np.abs(ref).max(), np.abs(got - ref).max()
    np.testing.assert_allclose(np.sort(e[e > 1e-3]), np.sort(om[w > 1e-6]), rtol=tol)


def test_refined_erpa_falls_back_on_a_wide_cluster(gpu_lib):
    """80 equal eigenvalues exceed the 64-wide block solver: the solve falls back to
    dsyevd and the result is still the FP64 one."""
    M, ev = planted_spectrum(300, 12, [(120, [0.0] * 80)])
    w, U = np.linalg.eigh(M)
    om = np.sqrt(np.abs(w))
    ref = yyT(U / np.sqrt(2 * np.where(w > 1e-6, om, 1.0))[None, :], np.where(w > 1e-6, om, w))
    Y, e, st = erpa_identity_plus(M, "refined", "fp64")
    assert st["solves"] == 1 and st["fallbacks"] == 1, st
    assert np.abs(yyT(Y, e) - ref).max() < 1e-9 * np.abs(ref).max()


def test_refinement_iterations_are_validated(gpu_lib):
    ctx = api.Context(0)
    with pytest.raises(GcError):
        ctx.set_eig_refinement(0)
    with pytest.raises(GcError):
        ctx.set_eig_refinement(5)


@pytest.fixture(scope="module")
def batch3(gpu_lib):
    systems = [small_system(n=16, nin=2, nact=4, rank=60, seed=0),
               small_system(n=24, nin=3, nact=4, rank=90, seed=3),
               small_system(n=20, nin=2, nact=2, rank=80, seed=5)]
    refs = []
    for s in systems:
        G, ffoo, fofo = oracle_integrals(s)
        indn = R.pair_space(s.occ, s.nele)
        ecas, ecorr, ws, x, w = R.acecorr(s.occ, s.xone, indn, s.nin, s.nact, ffoo, fofo,
                                          s.rdm2act, ngrid=8)
        refs.append((ecas, ecorr, np.array(ws)))
    return api.BatchInputs(systems, DEV), refs


@pytest.mark.parametrize("cfg", [
    dict(precision="fp64", erpa_mode="symm1", affine=False, nstreams=1),
    dict(precision="fp64", erpa_mode="cholesky", affine=True, nstreams=2),
    dict(precision="fp64tc5", erpa_mode="cholesky", affine=True, nstreams=3),
    dict(precision="fp64tc5", erpa_mode="refined", affine=True, nstreams=3),
    dict(precision="fp64tc6", erpa_mode="refined", affine=True, nstreams=2, eig_refine=2),
])
def test_batched_energies_match_oracle(batch3, cfg):
    batch, refs = batch3
    ecorr, ecas, wl, status = api.ac_energy_batched(batch, ngrid=8, **cfg)
    assert (status == 0).all()
    tol = 5e-9 if cfg["precision"] == "fp64tc5" else 1e-9
    for i, (rc, re, rw) in enumerate(refs):
        assert abs(ecas[i] - rc) < 1e-9
        assert abs(ecorr[i] - re) < tol, (cfg, i, ecorr[i], re)
        np.testing.assert_allclose(wl[i], rw, atol=tol)


def test_refined_batch_agrees_with_fp64_on_larger_systems(gpu_lib):
    """Two generator systems with N of a few thousand: the refined form on the
    sliced tensor-core GEMM against plain FP64 ERPASYMM1, 1 microhartree and
    better."""
    shapes = [dict(n=90, nin=8, nact=4, rank=540), dict(n=120, nin=12, nact=6, rank=720)]
    systems = [synth.make_system_device(**sh, seed=40 + i, device=DEV) for i, sh in enumerate(shapes)]
    batch = api.BatchInputs(systems, DEV)
    ctx = api.Context(0)
    plain = api.ac_energy_batched(batch, ngrid=8, precision="fp64", erpa_mode="symm1",
                                  affine=False, nstreams=1, ctx=ctx)
    fast = api.ac_energy_batched(batch, ngrid=8, precision="fp64tc5", erpa_mode="refined",
                                 affine=True, nstreams=2, ctx=ctx)
    assert (plain[3] == 0).all() and (fast[3] == 0).all()
    err = np.abs(fast[0] - plain[0]).max()
    assert err < 1e-8, err
    st = ctx.eig_refine_stats()
    assert st["solves"] == 16 and st["fallbacks"] == 0, st


def spd(N, seed, lo=1.0, hi=1e3, negative=0):
    """Q diag(ev) Q^T with ev geometric in [lo, hi]; the first `negative` set to -1."""
    rng = np.random.default_rng(seed)
    Q, _ = np.linalg.qr(rng.normal(size=(N, N)))
    ev = np.geomspace(lo, hi, N)
    ev[:negative] = -1.0
    A = (Q * ev) @ Q.T
    return 0.5 * (A + A.T)


@pytest.mark.parametrize("N", [50, 64, 65, 200, 1800])
def test_blocked_cholesky_matches_plain_and_numpy(gpu_lib, N):
    """The library's blocked Cholesky (64-wide FP64 blocks, row-wise panel solves,
    tensor-core trailing updates), at orders below, at and just above one block
    and with a ragged last block, gives the omega and sum y y^T of the single-dpotrf
    form and of numpy. Both forms build L^T A- L from FP64TC5 products (~2^-35 of
    |A||B| per element); with |L^T A- L| <= 50 and omega^2 >= 0.5 that moves omega
    by ~1e-8 relative, checked at 1e-6."""
    ap, am = spd(N, 1, 1.0, 10.0), spd(N, 2, 0.5, 5.0)
    res = []
    for blocked in (True, False):
        ctx = api.Context(0)
        ctx.set_chol_blocked(blocked)
        y, e = api.erpasymm1(t(ap), t(am), mode="refined", precision="fp64tc5", ctx=ctx)
        res.append((np.sort(e.cpu().numpy()), yyT(y.cpu().numpy(), e.cpu().numpy())))
    L = np.linalg.cholesky(ap)
    om = np.sqrt(np.linalg.eigvalsh(L.T @ am @ L))
    for e, _ in res:
        np.testing.assert_allclose(e, om, rtol=1e-6)
    assert np.abs(res[0][1] - res[1][1]).max() < 1e-6 * np.abs(res[1][1]).max()


def test_cholesky_reports_not_positive_definite(gpu_lib):
    """Both Cholesky forms return GC_ENOTPD and name the same first leading minor
    that is not positive definite."""
    N = 1700
    ap, am = spd(N, 3, negative=1), spd(N, 4)
    minors = []
    for blocked in (True, False):
        ctx = api.Context(0)
        ctx.set_chol_blocked(blocked)
        with pytest.raises(GcError) as ei:
            api.erpasymm1(t(ap), t(am), mode="refined", precision="fp64tc5", ctx=ctx)
        assert ei.value.code == 5  # GC_ENOTPD
        minors.append(int(str(ei.value).split("minor")[1].strip(" )")))
    assert minors[0] == minors[1] > 0


def test_batch_reports_the_system_without_a_cholesky_factor(batch3):
    """A system whose A+B is not positive definite goes through the batched Cholesky of
    its points beside the others: its status is GC_ENOTPD, and the other systems'
    energies still match the oracle."""
    from gammcor_gb300 import synth
    batch, refs = batch3
    bad = synth.make_system(n=18, nin=3, nact=4, rank=72, seed=1, eri_scale=0.25)
    G, ffoo, fofo = oracle_integrals(bad)
    indn = R.pair_space(bad.occ, bad.nele)
    x, _ = R.gauleg(0.0, 1.0, 8)
    not_pd = []
    for lam in x:
        abp, _, _ = R.ab_cas_fofo(bad.occ, bad.xone, np.eye(bad.n), indn, bad.nin, bad.nact, ffoo,
                                  fofo, bad.rdm2act, lam)
        not_pd.append(np.linalg.eigvalsh(0.5 * (abp + abp.T)).min() <= 0.0)
    assert any(not_pd)  # the case this test is about
    mixed = api.BatchInputs([batch.systems[0], bad, batch.systems[2]], DEV)
    ecorr, ecas, wl, status = api.ac_energy_batched(mixed, ngrid=8, precision="fp64tc5",
                                                    erpa_mode="refined", nstreams=2)
    assert status[1] == 5  # GC_ENOTPD
    assert status[0] == 0 and status[2] == 0
    assert abs(ecorr[0] - refs[0][1]) < 5e-9
    assert abs(ecorr[2] - refs[2][1]) < 5e-9
