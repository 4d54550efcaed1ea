"""The learned integrand reconstruction: trained on data of the exact path by
this library's kernels, it must predict held-out energies better than the same
two-node quadrature without the network (W linear in lambda)."""
import pytest

from gammcor_gb300 import surrogate

pytestmark = pytest.mark.gpu


def test_surrogate_beats_the_method_without_it(gpu_lib):
    quiet = lambda *a: None  # noqa: E731
    tr = surrogate.build_dataset(48, seed=5, chunk=24, nmin=30, nmax=60, log=quiet)
    te = surrogate.build_dataset(16, seed=6, chunk=16, nmin=30, nmax=60, log=quiet)
    ens = surrogate.Ensemble(members=3)
    ens.fit(tr["X"], surrogate.targets(tr["W"]), epochs=1500, log=quiet)
    res = surrogate.evaluate(ens, te, thresholds=(1e-3,))
    assert res["mae_network"] < res["mae_without_network"], res


def test_gated_energies_equal_the_exact_quadrature(gpu_lib):
    """surrogate.energies with the threshold at zero rejects every prediction: the
    end-node pass plus the interior pass of the batch session must then give the
    8-point energies of the one-call batch. The two passes solve their points' FP32
    eigenproblems in other batched calls than the one-call batch, so the refinements
    start from other FP32 vectors and agree to the FP64TC5 products' accuracy (about
    1e-10 Eh here), checked at 1e-9."""
    import numpy as np
    from gammcor_gb300 import api, synth
    shapes = surrogate.shapes(5, seed=9, nmin=30, nmax=50)
    systems = [synth.make_system_device(d["n"], d["nin"], d["nact"], d["rank"], d["seed"])
               for d in shapes]
    batch = api.BatchInputs(systems, "cuda:0")
    ens = surrogate.Ensemble.load(surrogate.MODEL)
    e, fb, est, st = surrogate.energies(batch, ens, threshold=0.0, nstreams=3)
    assert fb.all() and (st == 0).all()
    ref = api.ac_energy_batched(batch, ngrid=8, precision="fp64tc5", erpa_mode="refined",
                                nstreams=3)[0]
    np.testing.assert_allclose(e, ref, atol=1e-9, rtol=0)


def test_session_points_reuse_state_and_validate(gpu_lib):
    """Points added to a session reuse its integrals and A+-B: E_CAS is identical, and
    W(lambda) agrees to the FP64TC5 products' accuracy (the points' FP32 eigenproblems
    are solved in other batched calls, so the refinements start from other vectors)."""
    import numpy as np
    from gammcor_gb300 import api, synth
    from gammcor_gb300._lib import GcError
    shapes = surrogate.shapes(8, seed=10, nmin=30, nmax=50)
    systems = [synth.make_system_device(d["n"], d["nin"], d["nact"], d["rank"], d["seed"])
               for d in shapes]
    # keep systems whose A+B is positive definite on all eight points
    full = api.ac_energy_batched(api.BatchInputs(systems, "cuda:0"), ngrid=8,
                                 precision="fp64tc5", erpa_mode="refined", nstreams=2)
    systems = [s for s, st in zip(systems, full[3]) if st == 0][:4]
    assert len(systems) == 4
    batch = api.BatchInputs(systems, "cuda:0")
    x8, w8 = surrogate.gauss8()
    with api.AcSession(batch, nstreams=2) as ses:
        w1, ecas1, st1 = ses.points([2, 0], x8[:3])
        w2, ecas2, st2 = ses.points([0, 1, 2, 3], x8)
        assert (st1 == 0).all() and (st2 == 0).all()
        np.testing.assert_allclose(w2[[2, 0], :3], w1, atol=1e-9, rtol=0)
        np.testing.assert_allclose(ecas2[[2, 0]], ecas1, atol=1e-12, rtol=0)
        ref = api.ac_energy_batched(batch, ngrid=8, precision="fp64tc5", erpa_mode="refined",
                                    nstreams=2)
        np.testing.assert_allclose(w2 @ w8, ref[0], atol=1e-9, rtol=0)
        np.testing.assert_allclose(ecas2, ref[1], atol=1e-10, rtol=0)
        with pytest.raises(GcError):
            ses.points([1, 1], x8[:1])
        with pytest.raises(GcError):
            ses.points([4], x8[:1])


def test_autotune_streams_picks_a_candidate(gpu_lib):
    from gammcor_gb300 import api, synth
    shapes = surrogate.shapes(3, seed=11, nmin=30, nmax=40)
    systems = [synth.make_system_device(d["n"], d["nin"], d["nact"], d["rank"], d["seed"])
               for d in shapes]
    batch = api.BatchInputs(systems, "cuda:0")
    best, times = api.autotune_streams(batch, candidates=(1, 2), sample=3, points=1)
    assert best in (1, 2) and set(times) == {1, 2} and all(t > 0 for t in times.values())
