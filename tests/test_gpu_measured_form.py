"""The measured form (FP64-accurate sliced tcgen05 products, FP32 eigensolve
refined to FP64 accuracy, batched worker streams, batch session, integrand
surrogate gate) on the committed 64-basis fixture, against the oracle's
energies stored in it.

Tolerance: 5e-9 Eh for the exact quadratures (the FP64TC5 products carry
~2^-35 of |A||B|^T); an energy the surrogate accepts is held to its own gate,
1e-6 Eh.
"""
from pathlib import Path
from types import SimpleNamespace

import numpy as np
import pytest

from gammcor_gb300 import api, surrogate, synth

pytestmark = pytest.mark.gpu
GOLDEN = Path(__file__).parent / "golden" / "ac_cas_n64.npz"


@pytest.fixture(scope="module")
def golden(gpu_lib):
    d = np.load(GOLDEN)
    s = synth.System(n=int(d["n"]), nin=int(d["nin"]), nact=int(d["nact"]), rank=int(d["rank"]),
                     seed=int(d["seed"]), lfac=d["lfac"], h_ao=np.zeros(1), cmo=d["cmo"],
                     occ=d["occ"], xone=d["xone"], rdm2act=d["rdm2act"], e_cas=float(d["e_ci"]),
                     nele=int(d["nele"]), extra={"fock_diag": d["fock_diag"]})
    batch = api.BatchInputs([s], device="cuda:0")
    np.testing.assert_array_equal(batch.indn[0], d["indn"])
    return d, batch


@pytest.mark.parametrize("nstreams", [1, 3])
def test_session_fp64tc5_refined_matches_oracle(golden, nstreams):
    d, batch = golden
    with api.AcSession(batch, precision="fp64tc5", erpa_mode="refined", nstreams=nstreams) as ses:
        w5, ecas, st = ses.points([0], d["x"])
        w8, _, st8 = ses.points([0], d["x8"])
    assert st[0] == 0 and st8[0] == 0
    assert abs(ecas[0] - float(d["ecas"])) < 1e-9
    np.testing.assert_allclose(w5[0], d["w_lambda"], atol=5e-9)
    assert abs(w5[0] @ d["w"] - float(d["ecorr"])) < 5e-9
    assert abs(w8[0] @ d["w8"] - float(d["ecorr8"])) < 5e-9


def test_batched_fp64tc5_refined_matches_oracle(golden):
    d, batch = golden
    ec, ecas, wl, st = api.ac_energy_batched(batch, ngrid=8, precision="fp64tc5",
                                             erpa_mode="refined", nstreams=2)
    assert st[0] == 0
    assert abs(ec[0] - float(d["ecorr8"])) < 5e-9
    np.testing.assert_allclose(wl[0], d["w_lambda8"], atol=5e-9)


def test_surrogate_gated_energy_matches_oracle(golden):
    d, batch = golden
    ens = surrogate.Ensemble.load(surrogate.MODEL)
    e, fb, est, st = surrogate.energies(batch, ens, threshold=1e-6, nstreams=2)
    assert st[0] == 0
    tol = 5e-9 if fb[0] else 1e-6
    assert abs(e[0] - float(d["ecorr8"])) < tol, (e[0], float(d["ecorr8"]), bool(fb[0]))


def test_phase_timing_counts_every_phase_and_changes_no_result(golden):
    """gc_set_phase_timing records each phase of the batched path on the workers
    and hands the totals to the calling context; the energies are bit-identical
    with timing on and off."""
    d, batch = golden
    ctx = api.Context(0)
    try:
        kw = dict(ngrid=4, precision="fp64tc5", erpa_mode="refined", nstreams=2, ctx=ctx)
        e_off, _, _, st = api.ac_energy_batched(batch, **kw)
        assert all(n == 0 for _, n in ctx.phase_times().values())
        ctx.set_phase_timing(True)
        e_on, _, _, st_on = api.ac_energy_batched(batch, **kw)
        ph = ctx.phase_times()
        ctx.set_phase_timing(False)
    finally:
        ctx.close()
    assert st[0] == 0 and st_on[0] == 0
    assert e_on[0] == e_off[0]
    assert ph["transform"][1] == 2                # FOFO and FFOO
    assert ph["assembly"][1] == 2 + 4             # A+-B at 0 and 1, one combination per point
    assert ph["integrand"][1] == 4
    assert ph["cholesky"][1] == 1                 # the four points' factors in one batch
    assert ph["eigen"][1] == 1                    # the four points' FP32 solves in one batch
    assert ph["products"][1] >= 4
    assert all(ms > 0.0 for ms, _ in ph.values()), ph


def test_batched_fp32_eigensolves_match_one_at_a_time(golden):
    """The FP32 eigensolves of a system's points in one cusolverDnXsyevBatched call (the
    default) and one ssyevd per point give the same refined energies: both starts are
    refined to FP64 accuracy, so they agree far inside the 5e-9 Eh bar, and both match
    the oracle's 8-point energy."""
    d, batch = golden
    out = []
    for on in (True, False):
        ctx = api.Context(0)
        try:
            ctx.set_eig_batch(on)
            ec, _, wl, st = api.ac_energy_batched(batch, ngrid=8, precision="fp64tc5",
                                                  erpa_mode="refined", nstreams=2, ctx=ctx)
        finally:
            ctx.close()
        assert st[0] == 0
        out.append((ec[0], wl[0]))
    assert abs(out[0][0] - out[1][0]) < 1e-9
    np.testing.assert_allclose(out[0][1], out[1][1], atol=1e-9)
    assert abs(out[0][0] - float(d["ecorr8"])) < 5e-9
