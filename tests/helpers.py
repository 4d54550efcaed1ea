"""Shared builders for the parity tests (inputs through the generator,
reference results through the oracle)."""
from __future__ import annotations

import numpy as np

from gammcor_gb300 import synth
from oracle import ac_cas_ref as R


def small_system(n=16, nin=2, nact=4, rank=60, seed=0):
    return synth.make_system(n=n, nin=nin, nact=nact, rank=rank, seed=seed)


def oracle_integrals(s):
    G = s.ao_eri_packed()
    ffoo, fofo = R.transform_fofo_ffoo(s.cmo, G, s.nin, s.nact)
    return G, ffoo, fofo
