"""The allocation-free integrand entry point against the regular one.

Some callers of this library cannot allocate device memory when they need
W(lambda): their device memory belongs to their own pool, or their device
footprint must not grow after start-up. gc_ace_ne_erpa_fofo_noalloc serves
them from one fixed device array; this test calls it twice in a row through
the C ABI and checks
both results against gc_ace_ne_erpa_fofo within the 1e-9 Eh tolerance of the
other integrand tests. The file sorts last so that a run stopping at the first
failure has run every other test before it.
"""
import ctypes as C

import numpy as np
import pytest
import torch

from gammcor_gb300 import _lib, api
from oracle import ac_cas_ref as R

from .helpers import oracle_integrals, small_system

pytestmark = pytest.mark.gpu


def test_noalloc_integrand_matches_regular_entry_point(gpu_lib):
    s = small_system(n=24, nin=3, nact=4, rank=90, seed=3)
    G, ffoo, fofo = oracle_integrals(s)
    indn = R.pair_space(s.occ, s.nele)
    dev = "cuda:0"
    tf = lambda x: torch.as_tensor(np.ascontiguousarray(x), dtype=torch.float64, device=dev)
    abp, abm, _ = R.ab_cas_fofo(s.occ, s.xone, np.eye(s.n), indn, s.nin, s.nact, ffoo, fofo,
                                s.rdm2act, 0.5)
    y, eig = api.erpasymm1(tf(abp), tf(abm), mode="symm1")
    fofo_d = tf(fofo)
    w_ref = api.ace_ne_erpa_fofo(y, eig, s.occ, indn, s.nact, s.nin, fofo_d)
    w1 = api.ace_ne_erpa_fofo_noalloc(y, eig, s.occ, indn, s.nact, s.nin, fofo_d)
    w2 = api.ace_ne_erpa_fofo_noalloc(y, eig, s.occ, indn, s.nact, s.nin, fofo_d)
    assert abs(w1 - w_ref) < 1e-9, (w1, w_ref)
    assert abs(w2 - w_ref) < 1e-9, (w2, w_ref)
    # a second system of another size through the same shared array
    s2 = small_system(n=16, nin=2, nact=4, rank=60, seed=0)
    G2, ffoo2, fofo2 = oracle_integrals(s2)
    indn2 = R.pair_space(s2.occ, s2.nele)
    a2p, a2m, _ = R.ab_cas_fofo(s2.occ, s2.xone, np.eye(s2.n), indn2, s2.nin, s2.nact, ffoo2,
                                fofo2, s2.rdm2act, 0.7)
    y2, e2 = api.erpasymm1(tf(a2p), tf(a2m), mode="cholesky")
    f2 = tf(fofo2)
    assert abs(api.ace_ne_erpa_fofo_noalloc(y2, e2, s2.occ, indn2, s2.nact, s2.nin, f2)
               - api.ace_ne_erpa_fofo(y2, e2, s2.occ, indn2, s2.nact, s2.nin, f2)) < 1e-9


def test_noalloc_rejects_sizes_beyond_its_array(gpu_lib):
    ctx = api.default_context(0)
    lib = _lib.load()
    occ = np.ones(4000)
    ind = np.zeros(2, dtype=np.int32)
    w = C.c_double()
    dummy = C.c_void_p(1)
    rc = lib.gc_ace_ne_erpa_fofo_noalloc(ctx.h, 4000, 10, 4, 1, api._dptr(occ), api._iptr(ind),
                                         dummy, dummy, dummy, C.byref(w))
    assert rc == 1  # GC_EINVAL
    assert "limits" in lib.gc_last_error(ctx.h).decode()


def test_noalloc_wrapper_rejects_wrong_layouts(gpu_lib):
    s = small_system(n=16, nin=2, nact=4, rank=60, seed=0)
    G, ffoo, fofo = oracle_integrals(s)
    indn = R.pair_space(s.occ, s.nele)
    N = len(indn)
    dev = "cuda:0"
    y = torch.zeros((N, N), dtype=torch.float64, device=dev).t()
    e = torch.ones(N, dtype=torch.float64, device=dev)
    f = torch.as_tensor(fofo, device=dev)
    with pytest.raises(ValueError):
        api.ace_ne_erpa_fofo_noalloc(y, e.float(), s.occ, indn, s.nact, s.nin, f)
    with pytest.raises(ValueError):
        api.ace_ne_erpa_fofo_noalloc(y, e[::1].repeat(2)[::2], s.occ, indn, s.nact, s.nin, f)
    with pytest.raises(ValueError):
        api.ace_ne_erpa_fofo_noalloc(y, e, s.occ, indn, s.nact, s.nin, f.t())
