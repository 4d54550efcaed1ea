"""AC0-CAS (AC0CAS_FOFO, abfofo.f90:1485-1750) through the C ABI against the
oracle (oracle/ac0_ref.py). Tolerance: 1e-9 Eh on the energy, as the other
FP64 energies; E_CAS 1e-9 Eh."""
import numpy as np
import pytest
import torch

from gammcor_gb300 import api, synth
from oracle import ac0_ref as A
from oracle import ac_cas_ref as R

pytestmark = pytest.mark.gpu
DEV = "cuda:0"


def t(x):
    return torch.as_tensor(np.ascontiguousarray(x), dtype=torch.float64, device=DEV)


@pytest.mark.parametrize("n,nin,nact,seed", [(16, 2, 4, 0), (24, 3, 4, 3), (20, 2, 2, 1),
                                             (22, 0, 4, 2), (18, 3, 6, 4)])
def test_ac0_matches_oracle(gpu_lib, n, nin, nact, seed):
    s = synth.make_system(n=n, nin=nin, nact=nact, rank=4 * n, seed=seed)
    ffoo, fofo = R.transform_fofo_ffoo(s.cmo, s.ao_eri_packed(), s.nin, s.nact)
    indn = R.pair_space(s.occ, s.nele)
    e0, etot = A.ac0cas_fofo(s.occ, s.xone, np.eye(n), indn, nin, nact, ffoo, fofo, s.rdm2act)
    ge, get = api.ac0cas_fofo(s.occ, s.xone, indn, nact, nin, t(ffoo), t(fofo), s.rdm2act)
    assert abs(ge - e0) < 1e-9, (ge, e0)
    assert abs(get - etot) < 1e-9


def test_ac0_with_ure_matches_oracle(gpu_lib):
    s = synth.make_system(n=20, nin=2, nact=4, rank=80, seed=5)
    ffoo, fofo = R.transform_fofo_ffoo(s.cmo, s.ao_eri_packed(), s.nin, s.nact)
    indn = R.pair_space(s.occ, s.nele)
    q, _ = np.linalg.qr(np.random.default_rng(3).standard_normal((s.n, s.n)))
    ure = np.eye(s.n) + 0.05 * (q - np.eye(s.n))
    e0, etot = A.ac0cas_fofo(s.occ, s.xone, ure, indn, s.nin, s.nact, ffoo, fofo, s.rdm2act)
    ge, get = api.ac0cas_fofo(s.occ, s.xone, indn, s.nact, s.nin, t(ffoo), t(fofo), s.rdm2act,
                              ure=ure)
    assert abs(ge - e0) < 1e-9, (ge, e0)
    assert abs(get - etot) < 1e-9


def test_ac0_from_the_factored_transform_on_a_batch_system(gpu_lib):
    """The same energy from integrals the device transform produces (FP64), at a
    larger pair dimension, against the oracle on the oracle's own integrals."""
    s = synth.make_system(n=40, nin=4, nact=4, rank=160, seed=11)
    ffoo, fofo = R.transform_fofo_ffoo(s.cmo, s.ao_eri_packed(), s.nin, s.nact)
    indn = R.pair_space(s.occ, s.nele)
    e0, _ = A.ac0cas_fofo(s.occ, s.xone, np.eye(s.n), indn, s.nin, s.nact, ffoo, fofo, s.rdm2act)
    C = t(s.cmo)
    co = C[:, :s.nocc].contiguous()
    L = t(s.lfac)
    gfo = api.tran4_factored(s.n, L, C, co, C, co)
    gff = api.tran4_factored(s.n, L, co, co, C, C)
    ge, _ = api.ac0cas_fofo(s.occ, s.xone, indn, s.nact, s.nin, gff, gfo, s.rdm2act)
    assert abs(ge - e0) < 1e-9, (ge, e0)
