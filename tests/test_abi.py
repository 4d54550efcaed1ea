"""The C-ABI library loads and exports every symbol include/gammcor_gpu.h
declares; its host-only helpers agree with the oracle. No GPU needed."""
import re
from pathlib import Path

import numpy as np
import pytest

from gammcor_gb300 import _lib, api, build
from oracle import ac_cas_ref as R

ROOT = Path(__file__).resolve().parent.parent


@pytest.fixture(scope="module")
def lib():
    build.build()
    return _lib.load()


def declared_symbols():
    text = (ROOT / "include" / "gammcor_gpu.h").read_text()
    return sorted(set(re.findall(r"^\s*(?:int|const char \*|long long)\s*\**\s*(gc_\w+)\s*\(",
                                 text, re.M)))


def test_header_symbols_exported(lib):
    syms = declared_symbols()
    assert len(syms) >= 12
    for s in syms:
        assert hasattr(lib, s), s
    # the ctypes table covers the header exactly
    assert set(syms) == set(_lib.SIGNATURES)


def test_host_gauleg_matches_oracle(lib):
    for n in (1, 5, 8, 13):
        x, w = api.gauleg(0.0, 1.0, n)
        xr, wr = R.gauleg(0.0, 1.0, n)
        np.testing.assert_allclose(x, xr, atol=1e-15)
        np.testing.assert_allclose(w, wr, atol=1e-15)


def test_host_pair_space_matches_oracle(lib):
    rng = np.random.default_rng(5)
    for _ in range(5):
        n, nin, nact = 20, 3, 6
        occ = np.zeros(n)
        occ[:nin] = 1.0
        occ[nin:nin + nact] = np.sort(rng.uniform(0.0, 1.0, nact))[::-1]
        occ[nin + 2] = occ[nin + 1]          # a degenerate active pair
        occ[nin + nact - 1] = 1e-9            # a quasi-virtual active orbital
        nele = nin + nact // 2
        np.testing.assert_array_equal(api.pair_space(occ, nele), R.pair_space(occ, nele))
        assert api.prepare_nums(occ, nele) == R.prepare_nums(occ, nele)
        np.testing.assert_array_equal(api.pair_space(occ, nele, ifl_core=0),
                                      R.pair_space(occ, nele, ifl_core=0))


def test_fortran_module_binds_declared_symbols():
    """Every bind(C) name of the Fortran module is declared in the C header (or is a
    CUDA runtime call the wrappers use to move their host arrays)."""
    text = (ROOT / "include" / "gammcor_gpu.f90").read_text()
    names = set(re.findall(r'bind\(C,\s*name="(\w+)"\)', text))
    assert {"gc_ab_cas_fofo_ex", "gc_erpasymm1", "gc_ace_ne_erpa_fofo", "gc_tran4_gen"} <= names
    declared = set(declared_symbols())
    for nm in names:
        assert nm in declared or nm in {"cudaMalloc", "cudaFree", "cudaMemcpy"}, nm


def test_header_is_c99_and_every_symbol_links(lib, tmp_path):
    """The header is plain C (a C or Fortran host includes or binds it, not C++): a C99
    program that takes the address of every declared entry point compiles with
    -pedantic -Werror, links against the library and runs."""
    import shutil
    import subprocess
    if shutil.which("gcc") is None:
        pytest.skip("no C compiler")
    syms = declared_symbols()
    src = tmp_path / "abi.c"
    src.write_text('#include "gammcor_gpu.h"\n#include <stdio.h>\n'
                   "typedef void (*fn)(void);\nint main(void) {\n  fn p[] = {"
                   + ", ".join(f"(fn){s}" for s in syms)
                   + '};\n  printf("%d\\n", (int)(sizeof p / sizeof p[0]));\n  return 0;\n}\n')
    exe = tmp_path / "abi"
    libdir = ROOT / "gammcor_gb300"
    cc = subprocess.run(["gcc", "-std=c99", "-Wall", "-Wextra", "-Werror", "-pedantic",
                         "-I", str(ROOT / "include"), str(src), "-L", str(libdir),
                         "-lgammcor_gpu", f"-Wl,-rpath,{libdir}", "-o", str(exe)],
                        capture_output=True, text=True)
    assert cc.returncode == 0, cc.stderr
    run = subprocess.run([str(exe)], capture_output=True, text=True)
    assert run.returncode == 0 and int(run.stdout) == len(syms), run.stderr
