"""Failure paths that need no GPU fault.

* A bounded pipeline wait of the tensor-core GEMMs is made to run out by
  shortening the context's limit: the call returns GC_ETIMEOUT, the kernel has
  drained its copies and products and freed its tensor memory, and the next
  call on the same context succeeds with the right result.
* Non-finite inputs (planted on the host) come back as GC_ENONFINITE instead
  of a NaN energy; in a batch only the affected system is reported.
"""
import numpy as np
import pytest
import torch

from gammcor_gb300 import _lib, api, synth
from oracle import ac_cas_ref as R

from .helpers import oracle_integrals, small_system

pytestmark = pytest.mark.gpu
DEV = "cuda:0"


def t(x):
    return torch.as_tensor(np.ascontiguousarray(x), dtype=torch.float64, device=DEV)


@pytest.mark.parametrize("precision", ["fp64tc5", "bf16x6"])
def test_gemm_wait_timeout_then_recovery(gpu_lib, precision):
    ctx = api.Context(0)
    rng = np.random.default_rng(1)
    A = rng.standard_normal((1024, 2048))
    B = rng.standard_normal((768, 2048))
    Ad, Bd = t(A), t(B)
    ctx.set_pipeline_wait(2000)  # 2 us: far shorter than the product takes
    with pytest.raises(_lib.GcError) as e:
        api.tc_gemm_nt(Ad, Bd, precision=precision, ctx=ctx)
    assert e.value.code == 6  # GC_ETIMEOUT
    ctx.set_pipeline_wait(0)  # back to 1 s
    C = api.tc_gemm_nt(Ad, Bd, precision=precision, ctx=ctx).cpu().numpy()
    ref = A @ B.T
    tol = (5e-10 if precision == "fp64tc5" else 2e-5) * (np.abs(A) @ np.abs(B).T).max()
    assert np.abs(C - ref).max() < tol
    ctx.close()


def test_nonfinite_host_input_is_reported(gpu_lib):
    s = small_system()
    G, ffoo, fofo = oracle_integrals(s)
    indn = R.pair_space(s.occ, s.nele)
    xone = s.xone.copy()
    xone[3] = np.nan
    with pytest.raises(_lib.GcError) as e:
        api.ab_cas_fofo(s.occ, xone, indn, s.nact, s.nin, t(ffoo), t(fofo), s.rdm2act, 0.5)
    assert e.value.code == 9  # GC_ENONFINITE


def test_nonfinite_integrals_are_reported_not_solved(gpu_lib):
    s = small_system()
    G, ffoo, fofo = oracle_integrals(s)
    indn = R.pair_space(s.occ, s.nele)
    bad = fofo.copy()
    bad[5, 7] = np.nan
    for mode in ("symm1", "cholesky"):
        with pytest.raises(_lib.GcError) as e:
            api.acecorr(s.occ, s.xone, indn, s.nact, s.nin, t(ffoo), t(bad), s.rdm2act,
                        ngrid=3, erpa_mode=mode)
        assert e.value.code == 9, mode
    # the context is still usable
    ecas, ecorr, _ = api.acecorr(s.occ, s.xone, indn, s.nact, s.nin, t(ffoo), t(fofo),
                                 s.rdm2act, ngrid=3, erpa_mode="cholesky")
    assert np.isfinite(ecorr)


def test_batch_reports_the_nonfinite_system_only(gpu_lib):
    systems = [synth.make_system(n=18, nin=2, nact=4, rank=60, seed=k) for k in range(3)]
    clean = api.BatchInputs(systems, device=DEV)
    e0, _, _, st0 = api.ac_energy_batched(clean, ngrid=4, precision="fp64tc5",
                                          erpa_mode="refined", nstreams=2)
    assert (st0 == 0).all()
    batch = api.BatchInputs(systems, device=DEV)
    batch.lfac[1][10] = float("nan")
    e1, _, _, st1 = api.ac_energy_batched(batch, ngrid=4, precision="fp64tc5",
                                          erpa_mode="refined", nstreams=2)
    assert st1[1] == 9 and st1[0] == 0 and st1[2] == 0, st1
    np.testing.assert_allclose(e1[[0, 2]], e0[[0, 2]], atol=1e-12)
