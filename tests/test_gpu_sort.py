"""The AO integral sort (readtwoint, sorter.f90:31-395) and the on-device ERI
build against the oracle (oracle/sorter_ref.py). Integer and byte work: the
sorted tensor must match bit for bit, including slots written twice (the later
integral wins), labels in every format, and chunks applied one after another."""
import numpy as np
import pytest
import torch

from gammcor_gb300 import api, synth
from oracle import ac_cas_ref as R
from oracle import sorter_ref as S

pytestmark = pytest.mark.gpu
DEV = "cuda:0"


def quadruples(n, count, rng):
    p = rng.integers(1, n + 1, count)
    q = rng.integers(1, n + 1, count)
    r = rng.integers(1, n + 1, count)
    s = rng.integers(1, n + 1, count)
    return p, q, r, s


@pytest.mark.parametrize("fmt", ["pqrs", "dalton8", "dalton16"])
def test_sort_matches_oracle_bitwise(gpu_lib, fmt):
    rng = np.random.default_rng({"pqrs": 1, "dalton8": 2, "dalton16": 3}[fmt])
    n = 11
    count = 3000                      # far more than the 66^2 slots: many slots written twice
    p, q, r, s = quadruples(n, count, rng)
    if fmt != "pqrs":                 # Dalton labels carry p <= q and r <= s
        p, q = np.minimum(p, q), np.maximum(p, q)
        r, s = np.minimum(r, s), np.maximum(r, s)
    if fmt == "pqrs":
        lab = np.stack([p, q, r, s], 1).ravel().astype(np.int32)
    elif fmt == "dalton8":
        lab = (p | (q << 8) | (r << 16) | (s << 24)).astype(np.uint32).view(np.int32)
    else:
        lab = np.stack([r | (s << 16), p | (q << 16)], 1).ravel().astype(np.uint32).view(np.int32)
    vals = rng.standard_normal(count)
    ref = S.readtwoint(n, vals, lab, fmt)
    got = api.readtwoint(n, torch.as_tensor(vals, device=DEV), torch.as_tensor(lab, device=DEV),
                         fmt)
    assert np.array_equal(got.cpu().numpy(), ref)
    # a second chunk on top of the first
    vals2 = rng.standard_normal(500)
    lab2 = lab[: len(lab) * 500 // count].copy()
    ref = S.readtwoint(n, vals2, lab2, fmt, out=ref)
    got = api.readtwoint(n, torch.as_tensor(vals2, device=DEV), torch.as_tensor(lab2, device=DEV),
                         fmt, out=got)
    assert np.array_equal(got.cpu().numpy(), ref)


def test_triangle_stream_of_real_integrals(gpu_lib):
    s = synth.make_system(n=14, nin=2, nact=2, rank=40, seed=2)
    G = s.ao_eri_packed()                                   # (ntr, ntr), G[rs, pq] = (pq|rs)
    ntr = G.shape[0]
    stream = np.array([G[rs, pq] for pq in range(ntr) for rs in range(pq + 1)])
    ref = S.readtwoint(s.n, stream, None, "triangle")
    assert np.array_equal(ref, G)
    got = api.readtwoint(s.n, torch.as_tensor(stream, device=DEV), None, "triangle")
    assert np.array_equal(got.cpu().numpy(), ref)


def test_factored_eri_feeds_tran4_gen(gpu_lib):
    """AOTWOSORT built on the device from the factor (FP64 1e-12 relative) and
    transformed by tran4_gen equals the oracle's FFOO/FOFO (1e-10)."""
    s = synth.make_system(n=16, nin=2, nact=4, rank=60, seed=0)
    G = s.ao_eri_packed()
    L = torch.as_tensor(s.lfac, device=DEV)
    Gd = api.ao_eri_factored(s.n, L)
    assert np.abs(Gd.cpu().numpy() - G).max() < 1e-12 * np.abs(G).max()
    ffoo, fofo = R.transform_fofo_ffoo(s.cmo, G, s.nin, s.nact)
    C = torch.as_tensor(s.cmo, device=DEV)
    co = C[:, :s.nocc].contiguous()
    gfo = api.tran4_gen(s.n, C, co, C, co, Gd)
    gff = api.tran4_gen(s.n, co, co, C, C, Gd)
    assert np.abs(gfo.cpu().numpy() - fofo).max() < 1e-10
    assert np.abs(gff.cpu().numpy() - ffoo).max() < 1e-10
