"""ctypes binding of libgammcor_gpu.so (the C ABI declared in include/gammcor_gpu.h).

The library is loaded from the package directory. There is no fallback: if the
shared object is missing or does not load, every call raises.
"""
from __future__ import annotations

import ctypes as C
from pathlib import Path

_HERE = Path(__file__).resolve().parent
LIB_PATH = _HERE / "libgammcor_gpu.so"

GC_OK = 0
STATUS_NAMES = {0: "GC_OK", 1: "GC_EINVAL", 2: "GC_ECUDA", 3: "GC_ECUBLAS", 4: "GC_ECUSOLVER",
                5: "GC_ENOTPD", 6: "GC_ETIMEOUT", 7: "GC_ENOMEM", 8: "GC_EUNSUPPORTED",
                9: "GC_ENONFINITE"}
PREC = {"fp64": 0, "bf16x3": 1, "bf16x6": 2, "fp64tc5": 3, "fp64tc6": 4, "fp64tc4": 5}
ERPA = {"symm1": 0, "cholesky": 1, "refined": 2, "vec": 3}
TWOINT = {"dalton8": 0, "dalton16": 1, "pqrs": 2, "triangle": 3}

_dp = C.POINTER(C.c_double)
_ip = C.POINTER(C.c_int)
_vp = C.c_void_p

class GcSystem(C.Structure):
    _fields_ = [("nbas", C.c_int), ("ninact", C.c_int), ("nact", C.c_int), ("ndimx", C.c_int),
                ("rank", C.c_int), ("occ", _dp), ("xone", _dp), ("indn", _ip), ("rdm2act", _dp),
                ("cmo_dev", _vp), ("lfac_dev", _vp)]


class GcAcParams(C.Structure):
    _fields_ = [("ngrid", C.c_int), ("precision", C.c_int), ("erpa_mode", C.c_int),
                ("affine", C.c_int), ("nstreams", C.c_int), ("eig_emulation", C.c_int),
                ("eig_refine", C.c_int), ("lam", _dp), ("weight", _dp)]


# name -> (restype, argtypes); the list mirrors include/gammcor_gpu.h
SIGNATURES = {
    "gc_create": (C.c_int, [C.POINTER(C.c_void_p), C.c_int, _vp]),
    "gc_destroy": (C.c_int, [_vp]),
    "gc_last_error": (C.c_char_p, [_vp]),
    "gc_synchronize": (C.c_int, [_vp]),
    "gc_kernel_launches": (C.c_longlong, [_vp]),
    "gc_eig_time": (C.c_int, [_vp, _dp, C.POINTER(C.c_longlong)]),
    "gc_set_phase_timing": (C.c_int, [_vp, C.c_int]),
    "gc_phase_time": (C.c_int, [_vp, C.c_int, _dp, C.POINTER(C.c_longlong)]),
    "gc_set_eig_emulation": (C.c_int, [_vp, C.c_int]),
    "gc_set_eig_refinement": (C.c_int, [_vp, C.c_int]),
    "gc_set_chol_blocked": (C.c_int, [_vp, C.c_int]),
    "gc_set_pipeline_wait": (C.c_int, [_vp, C.c_ulonglong]),
    "gc_set_gemm_tile": (C.c_int, [_vp, C.c_int]),
    "gc_set_eig_batch": (C.c_int, [_vp, C.c_int]),
    "gc_eig_refine_stats": (C.c_int, [_vp, C.POINTER(C.c_longlong), C.POINTER(C.c_longlong),
                                      C.POINTER(C.c_int)]),
    "gc_gauleg": (C.c_int, [C.c_double, C.c_double, _dp, _dp, C.c_int]),
    "gc_prepare_nums": (C.c_int, [C.c_int, _dp, C.c_int, _ip, _ip]),
    "gc_pair_space": (C.c_int, [C.c_int, _dp, C.c_int, C.c_int, C.c_double, C.c_double, _ip, _ip]),
    "gc_tran4_gen": (C.c_int, [_vp, C.c_int, C.c_int, _vp, C.c_int, _vp, C.c_int, _vp, C.c_int, _vp,
                               _vp, _vp, C.c_int]),
    "gc_sort_twoint": (C.c_int, [_vp, C.c_int, C.c_longlong, _vp, _vp, C.c_int, C.c_int, _vp]),
    "gc_ao_eri_factored": (C.c_int, [_vp, C.c_int, C.c_int, _vp, _vp, C.c_int]),
    "gc_tran4_factored": (C.c_int, [_vp, C.c_int, C.c_int, _vp, C.c_int, _vp, C.c_int, _vp, C.c_int,
                                    _vp, C.c_int, _vp, _vp, C.c_int]),
    "gc_ab_cas_fofo": (C.c_int, [_vp, C.c_int, C.c_int, C.c_int, C.c_int, _dp, _dp, _ip, _dp, _vp,
                                 _vp, C.c_double, _vp, _vp, _dp]),
    "gc_ab_cas_fofo_ex": (C.c_int, [_vp, C.c_int, C.c_int, C.c_int, C.c_int, _dp, _dp, _dp, _ip,
                                    _dp, _vp, _vp, C.c_double, C.c_int, _vp, _vp, _dp]),
    "gc_erpasymm1": (C.c_int, [_vp, C.c_int, _vp, _vp, _vp, _vp]),
    "gc_ac0cas_fofo": (C.c_int, [_vp, C.c_int, C.c_int, C.c_int, C.c_int, _dp, _dp, _dp, _ip, _dp,
                                 _vp, _vp, _dp, _dp]),
    "gc_freq_grid": (C.c_int, [C.c_int, _dp, _dp]),
    "gc_ac_freq_fofo": (C.c_int, [_vp, C.c_int, C.c_int, C.c_int, C.c_int, _dp, _dp, _dp, _ip, _dp,
                                  _vp, _vp, C.c_int, C.c_int, C.c_int, C.c_int, _dp, _dp]),
    "gc_erpa": (C.c_int, [_vp, C.c_int, _vp, _vp, _vp, _vp, C.c_int]),
    "gc_erpa_ex": (C.c_int, [_vp, C.c_int, _vp, _vp, _vp, _vp, C.c_int, C.c_int]),
    "gc_ace_ne_erpa_fofo": (C.c_int, [_vp, C.c_int, C.c_int, C.c_int, C.c_int, _dp, _ip, _vp, _vp,
                                      _vp, C.c_int, _dp]),
    "gc_ac_energy_batched": (C.c_int, [_vp, C.c_int, C.POINTER(GcSystem), C.POINTER(GcAcParams),
                                       _dp, _dp, _dp, _dp, _ip]),
    "gc_ac_session_create": (C.c_int, [_vp, C.c_int, C.POINTER(GcSystem), C.POINTER(GcAcParams),
                                       C.POINTER(C.c_void_p)]),
    "gc_ac_session_points": (C.c_int, [_vp, C.c_int, _ip, C.c_int, _dp, _dp, _dp, _dp, _ip]),
    "gc_ac_session_destroy": (C.c_int, [_vp]),
    "gc_mlp_create": (C.c_int, [_vp, C.c_int, C.c_int, C.c_int, C.c_ulonglong, C.POINTER(C.c_void_p)]),
    "gc_mlp_destroy": (C.c_int, [_vp]),
    "gc_mlp_num_params": (C.c_longlong, [_vp]),
    "gc_mlp_set_params": (C.c_int, [_vp, _vp, _vp]),
    "gc_mlp_get_params": (C.c_int, [_vp, _vp, _vp]),
    "gc_mlp_forward": (C.c_int, [_vp, _vp, C.c_int, _vp, _vp]),
    "gc_mlp_gradients": (C.c_int, [_vp, _vp, C.c_int, _vp, _vp, _vp, C.POINTER(C.c_float)]),
    "gc_mlp_train_step": (C.c_int, [_vp, _vp, C.c_int, _vp, _vp, C.c_float, C.POINTER(C.c_float)]),
    "gc_tc_gemm_time": (C.c_int, [_vp, C.c_int, C.c_int, C.c_int, C.c_int, C.c_int, _dp]),
    "gc_tc_gemm_nt": (C.c_int, [_vp, C.c_int, C.c_int, C.c_int, C.c_int, _vp, C.c_int, _vp, C.c_int,
                                _vp, C.c_int]),
    "gc_ace_ne_erpa_fofo_noalloc": (C.c_int, [_vp, C.c_int, C.c_int, C.c_int, C.c_int, _dp, _ip,
                                              _vp, _vp, _vp, _dp]),
    "gc_acecorr": (C.c_int, [_vp, C.c_int, C.c_int, C.c_int, C.c_int, _dp, _dp, _ip, _dp, _vp, _vp,
                             C.c_int, C.c_int, C.c_int, _dp, _dp, _dp]),
}

_lib = None


class GcError(RuntimeError):
    def __init__(self, code: int, msg: str):
        super().__init__(f"{STATUS_NAMES.get(code, code)}: {msg}")
        self.code = code


def load(path: Path | None = None):
    """Load the library (once) and declare every entry point's prototype."""
    global _lib
    if _lib is not None:
        return _lib
    p = Path(path) if path else LIB_PATH
    if not p.exists():
        raise RuntimeError(f"{p} is missing: build it with gammcor_gb300.build.build()")
    lib = C.CDLL(str(p))
    for name, (res, args) in SIGNATURES.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    _lib = lib
    return lib


def check(ctx, code: int):
    if code != GC_OK:
        msg = load().gc_last_error(ctx).decode() if ctx else ""
        raise GcError(code, msg)
