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
