"""Host-side mirror of the reference routines on the AC-CAS (FOFO) path.

Each function keeps the name and argument meaning of the GAMMCOR subroutine it
replaces and calls the CUDA library through its C ABI. Device memory is held
in torch tensors (plumbing only; no torch op computes anything on the path).
Matrices returned with Fortran meaning are column-major: ``A[i, j]`` is
``A(i+1, j+1)`` of the reference.
"""
from __future__ import annotations

import ctypes as C

import numpy as np
import torch

from . import _lib
from ._lib import ERPA, PREC, check, load

THR_SEL_ACT = 1e-8
THR_QVIRT = 1e-7


class Context:
    """A library context bound to one device and one CUDA stream."""

    def __init__(self, device: int = 0, stream: torch.cuda.Stream | None = None):
        lib = load()
        self.device = device
        self.stream = stream
        h = C.c_void_p()
        if stream is None:
            stream = torch.cuda.current_stream(device)
        self.stream = stream
        s = C.c_void_p(stream.cuda_stream)
        check(None, lib.gc_create(C.byref(h), device, s))
        self.h = h

    def close(self):
        if self.h:
            load().gc_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def launches(self) -> int:
        return int(load().gc_kernel_launches(self.h))

    def eig_time(self) -> tuple[float, int]:
        """(milliseconds, calls) of the cuSOLVER eigensolves run on this context so far."""
        ms, n = C.c_double(), C.c_longlong()
        check(self.h, load().gc_eig_time(self.h, C.byref(ms), C.byref(n)))
        return ms.value, n.value

    PHASES = ("transform", "assembly", "cholesky", "products", "eigen", "integrand")

    def set_phase_timing(self, on: bool):
        """Record CUDA events around each phase of the AC path (gc_phase)."""
        check(self.h, load().gc_set_phase_timing(self.h, int(on)))

    def phase_times(self) -> dict:
        """{phase: (milliseconds, calls)} accumulated on this context so far."""
        out = {}
        for i, name in enumerate(self.PHASES):
            ms, n = C.c_double(), C.c_longlong()
            check(self.h, load().gc_phase_time(self.h, i, C.byref(ms), C.byref(n)))
            out[name] = (ms.value, n.value)
        return out

    def sync(self):
        check(self.h, load().gc_synchronize(self.h))

    def set_eig_emulation(self, on: bool):
        """cuSOLVER FP64 emulation strategy for the eigensolver (EAGER when on) and
        BF16x9 math for the FP32 eigensolver of the refined ERPA form."""
        check(self.h, load().gc_set_eig_emulation(self.h, int(on)))

    def set_eig_refinement(self, iterations: int):
        """Refinement iterations of the refined ERPA form (1..4)."""
        check(self.h, load().gc_set_eig_refinement(self.h, int(iterations)))

    def set_chol_blocked(self, on: bool):
        """This library's blocked Cholesky of A+B (64-wide FP64 blocks, tensor-core
        trailing updates) on the sliced path; off: one cuSOLVER dpotrf."""
        check(self.h, load().gc_set_chol_blocked(self.h, int(on)))

    def set_pipeline_wait(self, ns: int):
        """Limit of the tensor-core GEMMs' pipeline waits in ns (0: the 1 s default);
        shortening it injects a timeout for tests."""
        check(self.h, load().gc_set_pipeline_wait(self.h, int(ns)))

    def set_eig_batch(self, on: bool):
        """Batch the FP32 eigensolves of all lambda points of a system (batched calls)."""
        check(self.h, load().gc_set_eig_batch(self.h, int(on)))

    def set_gemm_tile(self, width: int):
        """Column tile of the sliced FP64-accurate GEMMs: 0 picks per product,
        64/96/128 forces it (capped by the slice count); results are identical."""
        check(self.h, load().gc_set_gemm_tile(self.h, int(width)))

    def eig_refine_stats(self) -> dict:
        """Refined ERPA counters: solves, dsyevd fallbacks, largest block cluster."""
        s, f, m = C.c_longlong(), C.c_longlong(), C.c_int()
        check(self.h, load().gc_eig_refine_stats(self.h, C.byref(s), C.byref(f), C.byref(m)))
        return {"solves": s.value, "fallbacks": f.value, "max_cluster": m.value}


_default: dict[int, Context] = {}


def default_context(device: int = 0) -> Context:
    if device not in _default:
        _default[device] = Context(device)
    return _default[device]


def _ptr(t: torch.Tensor) -> C.c_void_p:
    if not t.is_cuda:
        raise ValueError("expected a CUDA tensor")
    if not t.is_contiguous():
        raise ValueError("expected a contiguous tensor")
    return C.c_void_p(t.data_ptr())


def _dptr(a: np.ndarray):
    return a.ctypes.data_as(C.POINTER(C.c_double))


def _iptr(a: np.ndarray):
    return a.ctypes.data_as(C.POINTER(C.c_int))


def _fortran_cols(t: torch.Tensor) -> torch.Tensor:
    """Device copy of a matrix laid out column-major (Fortran), as a (cols, rows) tensor."""
    return t.t().contiguous()


# --------------------------------------------------------------- host helpers
def gauleg(x1: float, x2: float, n: int):
    """GauLeg (misc.f:828-865)."""
    x = np.zeros(n)
    w = np.zeros(n)
    check(None, load().gc_gauleg(x1, x2, _dptr(x), _dptr(w), n))
    return x, w


def prepare_nums(occ: np.ndarray, nele: int):
    """prepare_nums (initia.f:2996-3035) -> (Num0, Num1)."""
    occ = np.ascontiguousarray(occ, dtype=np.float64)
    a, b = C.c_int(), C.c_int()
    check(None, load().gc_prepare_nums(occ.shape[0], _dptr(occ), nele, C.byref(a), C.byref(b)))
    return a.value, b.value


def pair_space(occ: np.ndarray, nele: int, ifl_core: int = 1, thr_sel_act: float = THR_SEL_ACT,
               thr_qvirt: float = THR_QVIRT) -> np.ndarray:
    """Pair builder of ACCAS (accas.f:30-106). Returns IndN as (NDimX, 2), 1-based."""
    occ = np.ascontiguousarray(occ, dtype=np.float64)
    n = occ.shape[0]
    buf = np.zeros(max(1, n * (n - 1)), dtype=np.int32)
    nd = C.c_int()
    check(None, load().gc_pair_space(n, _dptr(occ), nele, ifl_core, thr_sel_act, thr_qvirt,
                                     _iptr(buf), C.byref(nd)))
    return buf[: 2 * nd.value].reshape(-1, 2).astype(np.int64)


# ----------------------------------------------------------------- transform
def tran4_gen(nbas: int, CA: torch.Tensor, CB: torch.Tensor, CC: torch.Tensor, CD: torch.Tensor,
              ao_sorted: torch.Tensor, precision: str = "fp64", ctx: Context | None = None,
              out: torch.Tensor | None = None) -> torch.Tensor:
    """tran4_gen (tran.f90:313-423).

    CA..CD: AO x MO blocks as (nbas, nX) tensors with Fortran meaning (they are
    made column-major here). ao_sorted: (ntr, ntr) AOTWOSORT records. Returns
    the output file as (nA*nB, nC*nD): row = record ab, column = element cd.
    """
    ctx = ctx or default_context(CA.device.index or 0)
    cols = [_fortran_cols(c.to(torch.float64)) for c in (CA, CB, CC, CD)]
    nA, nB, nC, nD = (c.shape[0] for c in cols)
    if out is None:
        out = torch.empty((nA * nB, nC * nD), dtype=torch.float64, device=CA.device)
    check(ctx.h, load().gc_tran4_gen(ctx.h, nbas, nA, _ptr(cols[0]), nB, _ptr(cols[1]), nC,
                                     _ptr(cols[2]), nD, _ptr(cols[3]), _ptr(ao_sorted), _ptr(out),
                                     PREC[precision]))
    return out


def readtwoint(nbas: int, values: torch.Tensor, labels: torch.Tensor | None, fmt: str,
               out: torch.Tensor | None = None, ctx: Context | None = None) -> torch.Tensor:
    """readtwoint (sorter.f90:31-395) for one chunk of integrals already on the device:
    values (FP64) and labels (int32, fmt 'dalton8', 'dalton16', 'pqrs', or None for
    'triangle'). Returns the AOTWOSORT tensor (ntr, ntr), record rs = row; pass the
    tensor of an earlier chunk as `out` to add a further chunk."""
    ctx = ctx or default_context(values.device.index or 0)
    ntr = nbas * (nbas + 1) // 2
    init = out is None
    if out is None:
        out = torch.empty((ntr, ntr), dtype=torch.float64, device=values.device)
    if values.dtype != torch.float64 or (labels is not None and labels.dtype != torch.int32):
        raise ValueError("values must be float64 and labels int32")
    check(ctx.h, load().gc_sort_twoint(ctx.h, nbas, values.numel(), _ptr(values),
                                       _ptr(labels) if labels is not None else None,
                                       _lib.TWOINT[fmt], int(init), _ptr(out)))
    return out


def ao_eri_factored(nbas: int, lfac: torch.Tensor, precision: str = "fp64",
                    ctx: Context | None = None) -> torch.Tensor:
    """The AOTWOSORT tensor L L^T from the ERI factor (ntr, rank) with Fortran meaning."""
    ctx = ctx or default_context(lfac.device.index or 0)
    ntr = nbas * (nbas + 1) // 2
    lcol = _fortran_cols(lfac)
    out = torch.empty((ntr, ntr), dtype=torch.float64, device=lfac.device)
    check(ctx.h, load().gc_ao_eri_factored(ctx.h, nbas, lfac.shape[1], _ptr(lcol), _ptr(out),
                                           PREC[precision]))
    return out


def tran4_factored(nbas: int, lfac: torch.Tensor, CA, CB, CC, CD, precision: str = "fp64",
                   ctx: Context | None = None, out: torch.Tensor | None = None) -> torch.Tensor:
    """tran4_gen's output from the ERI factor; lfac is (ntr, rank) with Fortran meaning."""
    ctx = ctx or default_context(CA.device.index or 0)
    cols = [_fortran_cols(c.to(torch.float64)) for c in (CA, CB, CC, CD)]
    nA, nB, nC, nD = (c.shape[0] for c in cols)
    lcol = _fortran_cols(lfac)
    rank = lfac.shape[1]
    if out is None:
        out = torch.empty((nA * nB, nC * nD), dtype=torch.float64, device=CA.device)
    same = CA is CC and CB is CD
    cc = cols[0] if same else cols[2]
    cd = cols[1] if same else cols[3]
    check(ctx.h, load().gc_tran4_factored(ctx.h, nbas, rank, _ptr(lcol), nA, _ptr(cols[0]), nB,
                                          _ptr(cols[1]), nC, _ptr(cc), nD, _ptr(cd), _ptr(out),
                                          PREC[precision]))
    return out


# ------------------------------------------------------------------ assembly
def ab_cas_fofo(occ: np.ndarray, xone: np.ndarray, indn: np.ndarray, nact: int, inactive: int,
                ffoo: torch.Tensor, fofo: torch.Tensor, rdm2act: np.ndarray, acalpha: float,
                ure: np.ndarray | None = None, ab1: bool = False, ctx: Context | None = None):
    """AB_CAS_FOFO (abfofo.f90:8-293). Returns (ABPLUS, ABMIN, ETot); the
    matrices are (NDimX, NDimX) views with Fortran meaning (column-major storage).
    ure: the URe rotation of the one-electron integrals (None: identity); ab1: the
    AB1 form (the lambda derivative of A+-B)."""
    ctx = ctx or default_context(ffoo.device.index or 0)
    occ = np.ascontiguousarray(occ, dtype=np.float64)
    xone = np.ascontiguousarray(xone, dtype=np.float64)
    ind = np.ascontiguousarray(indn, dtype=np.int32).ravel()
    rdm = np.ascontiguousarray(rdm2act, dtype=np.float64)
    n = occ.shape[0]
    N = ind.shape[0] // 2
    u = None if ure is None else np.asfortranarray(ure, dtype=np.float64)
    abp = torch.empty((N, N), dtype=torch.float64, device=ffoo.device)
    abm = torch.empty_like(abp)
    etot = C.c_double()
    check(ctx.h, load().gc_ab_cas_fofo_ex(ctx.h, n, inactive, nact, N, _dptr(occ),
                                          _dptr(u.ravel(order="F")) if u is not None else None,
                                          _dptr(xone), _iptr(ind), _dptr(rdm), _ptr(ffoo),
                                          _ptr(fofo), float(acalpha), int(ab1), _ptr(abp),
                                          _ptr(abm), C.byref(etot)))
    return abp.t(), abm.t(), etot.value


def erpasymm1(abplus: torch.Tensor, abmin: torch.Tensor, mode: str = "symm1",
              precision: str = "fp64", ctx: Context | None = None):
    """ERPASYMM1 (interpa.f:1652-1781) or its Cholesky forms ("cholesky",
    "refined": FP32 eigensolve refined to FP64 accuracy). abplus/abmin are
    Fortran-meaning (N, N) matrices (column-major storage, e.g. the views
    returned by ab_cas_fofo). precision ("fp64", "fp64tc5", "fp64tc6") is the
    arithmetic of the Cholesky forms' matrix products. Returns (EigVecR, Eig)
    with EigVecR[:, nu] = Y_nu."""
    ctx = ctx or default_context(abplus.device.index or 0)
    ap = abplus.t().contiguous()   # column-major storage
    am = abmin.t().contiguous()
    N = ap.shape[0]
    y = torch.empty_like(ap)
    eig = torch.empty(N, dtype=torch.float64, device=ap.device)
    check(ctx.h, load().gc_erpa_ex(ctx.h, N, _ptr(ap), _ptr(am), _ptr(y), _ptr(eig), ERPA[mode],
                                   PREC[precision]))
    return y.t(), eig


def erpasymm1_aplsqrt(abplus: torch.Tensor, abmin: torch.Tensor, ctx: Context | None = None):
    """ERPASYMM1 (interpa.f:1652-1781) with the routine's APLSQRT output: returns
    (EigVecR, Eig, APLSQRT = A+^1/2), all with Fortran meaning. FP64."""
    ctx = ctx or default_context(abplus.device.index or 0)
    ap = abplus.t().contiguous()
    am = abmin.t().contiguous()
    N = ap.shape[0]
    y = torch.empty_like(ap)
    eig = torch.empty(N, dtype=torch.float64, device=ap.device)
    check(ctx.h, load().gc_erpasymm1(ctx.h, N, _ptr(ap), _ptr(am), _ptr(y), _ptr(eig)))
    return y.t(), eig, ap.t()


def ace_ne_erpa_fofo(evec: torch.Tensor, evals: torch.Tensor, occ: np.ndarray, indn: np.ndarray,
                     nact: int, inactive: int, fofo: torch.Tensor, precision: str = "fp64",
                     ctx: Context | None = None) -> float:
    """ACEneERPA_FOFO (abfofo.f90:3791-3927): W(lambda)."""
    ctx = ctx or default_context(fofo.device.index or 0)
    occ = np.ascontiguousarray(occ, dtype=np.float64)
    ind = np.ascontiguousarray(indn, dtype=np.int32).ravel()
    ycol = evec.t().contiguous()
    w = C.c_double()
    check(ctx.h, load().gc_ace_ne_erpa_fofo(ctx.h, occ.shape[0], inactive, nact, ind.shape[0] // 2,
                                            _dptr(occ), _iptr(ind), _ptr(ycol),
                                            _ptr(evals.contiguous()), _ptr(fofo), PREC[precision],
                                            C.byref(w)))
    return w.value


def ace_ne_erpa_fofo_noalloc(evec: torch.Tensor, evals: torch.Tensor, occ: np.ndarray,
                             indn: np.ndarray, nact: int, inactive: int, fofo: torch.Tensor,
                             ctx: Context | None = None) -> float:
    """W(lambda) through the entry point that allocates no device memory, for
    callers whose device memory belongs to their own pool or must not grow
    (limits nbas <= 2048, NDimX <= 16384). Nothing is copied here: evec must
    already be a Fortran-layout (column-major) FP64 device matrix, e.g. the view
    returned by erpasymm1, and evals and fofo contiguous FP64 tensors on the
    context's device."""
    ctx = ctx or default_context(fofo.device.index or 0)
    occ = np.ascontiguousarray(occ, dtype=np.float64)
    ind = np.ascontiguousarray(indn, dtype=np.int32).ravel()
    ycol = evec.t()
    if not ycol.is_contiguous():
        raise ValueError("evec must be column-major (a .t() view of a contiguous tensor)")
    for name, x in (("evec", evec), ("evals", evals), ("fofo", fofo)):
        if x.dtype != torch.float64:
            raise ValueError(f"{name} must be float64, got {x.dtype}")
        if not x.is_cuda or x.device.index != ctx.device:
            raise ValueError(f"{name} must be on cuda:{ctx.device}, got {x.device}")
    for name, x in (("evals", evals), ("fofo", fofo)):
        if not x.is_contiguous():
            raise ValueError(f"{name} must be contiguous")
    w = C.c_double()
    check(ctx.h, load().gc_ace_ne_erpa_fofo_noalloc(ctx.h, occ.shape[0], inactive, nact,
                                                    ind.shape[0] // 2, _dptr(occ), _iptr(ind),
                                                    _ptr(ycol), _ptr(evals), _ptr(fofo),
                                                    C.byref(w)))
    return w.value


def ac0cas_fofo(occ, xone, indn, nact, inactive, ffoo, fofo, rdm2act, ure=None,
                ctx: Context | None = None):
    """AC0CAS_FOFO (abfofo.f90:1485-1750): returns (ECorr, ETot), the AC0 correlation
    energy and E_CAS (without ENuc)."""
    ctx = ctx or default_context(ffoo.device.index or 0)
    occ = np.ascontiguousarray(occ, dtype=np.float64)
    xone = np.ascontiguousarray(xone, dtype=np.float64)
    ind = np.ascontiguousarray(indn, dtype=np.int32).ravel()
    rdm = np.ascontiguousarray(rdm2act, dtype=np.float64)
    u = None if ure is None else np.asfortranarray(ure, dtype=np.float64)
    ec, et = C.c_double(), C.c_double()
    check(ctx.h, load().gc_ac0cas_fofo(ctx.h, occ.shape[0], inactive, nact, ind.shape[0] // 2,
                                       _dptr(occ),
                                       _dptr(u.ravel(order="F")) if u is not None else None,
                                       _dptr(xone), _iptr(ind), _dptr(rdm), _ptr(ffoo), _ptr(fofo),
                                       C.byref(ec), C.byref(et)))
    return ec.value, et.value


def freq_grid(nfreq: int):
    """FreqGrid (ac_iter.f:414-429): frequencies and weights of the ACFREQ integral."""
    x = np.zeros(nfreq)
    w = np.zeros(nfreq)
    check(None, load().gc_freq_grid(nfreq, _dptr(x), _dptr(w)))
    return x, w


def ac_freq_fofo(occ, xone, indn, nact, inactive, ffoo, fofo, rdm2act, nfreq: int = 25,
                 max_cn: int = 3, precision: str = "fp64", erpa_mode: str = "cholesky", ure=None,
                 ctx: Context | None = None):
    """WIter_FOFO (ac_fofo.f90:1-181), the ACFREQ energy: returns (ECorr, ECASSCF)."""
    ctx = ctx or default_context(ffoo.device.index or 0)
    occ = np.ascontiguousarray(occ, dtype=np.float64)
    xone = np.ascontiguousarray(xone, dtype=np.float64)
    ind = np.ascontiguousarray(indn, dtype=np.int32).ravel()
    rdm = np.ascontiguousarray(rdm2act, dtype=np.float64)
    u = None if ure is None else np.asfortranarray(ure, dtype=np.float64)
    ec, et = C.c_double(), C.c_double()
    check(ctx.h, load().gc_ac_freq_fofo(ctx.h, occ.shape[0], inactive, nact, ind.shape[0] // 2,
                                        _dptr(occ),
                                        _dptr(u.ravel(order="F")) if u is not None else None,
                                        _dptr(xone), _iptr(ind), _dptr(rdm), _ptr(ffoo),
                                        _ptr(fofo), int(nfreq), int(max_cn), PREC[precision],
                                        ERPA[erpa_mode], C.byref(ec), C.byref(et)))
    return ec.value, et.value


def acecorr(occ, xone, indn, nact, inactive, ffoo, fofo, rdm2act, ngrid: int = 5,
            erpa_mode: str = "symm1", precision: str = "fp64", ctx: Context | None = None):
    """ACECORR (acfd.f:117-209). Returns (E_CAS, ECorr, [W(lambda_i)])."""
    ctx = ctx or default_context(ffoo.device.index or 0)
    occ = np.ascontiguousarray(occ, dtype=np.float64)
    xone = np.ascontiguousarray(xone, dtype=np.float64)
    ind = np.ascontiguousarray(indn, dtype=np.int32).ravel()
    rdm = np.ascontiguousarray(rdm2act, dtype=np.float64)
    ec, ecas = C.c_double(), C.c_double()
    ws = np.zeros(ngrid)
    check(ctx.h, load().gc_acecorr(ctx.h, occ.shape[0], inactive, nact, ind.shape[0] // 2,
                                   _dptr(occ), _dptr(xone), _iptr(ind), _dptr(rdm), _ptr(ffoo),
                                   _ptr(fofo), ngrid, ERPA[erpa_mode], PREC[precision],
                                   C.byref(ec), C.byref(ecas), _dptr(ws)))
    return ecas.value, ec.value, list(ws)


def tc_gemm_nt(A: torch.Tensor, B: torch.Tensor, precision: str = "bf16x3",
               ctx: Context | None = None) -> torch.Tensor:
    """C = A @ B.T (FP64 in and out) through the tensor-core contraction engine."""
    ctx = ctx or default_context(A.device.index or 0)
    m, k = A.shape
    n = B.shape[0]
    acol = _fortran_cols(A)
    bcol = _fortran_cols(B)
    c = torch.empty((n, m), dtype=torch.float64, device=A.device)   # column-major m x n
    check(ctx.h, load().gc_tc_gemm_nt(ctx.h, PREC[precision], m, n, k, _ptr(acol), m, _ptr(bcol),
                                      n, _ptr(c), m))
    return c.t()


# ---------------------------------------------------------------------- batch
class BatchInputs:
    """Device-resident inputs of a batch of systems for ac_energy_batched."""

    def __init__(self, systems, device="cuda:0"):
        self.systems = list(systems)
        self.device = device
        self.cmo = [torch.as_tensor(np.asfortranarray(s.cmo).ravel(order="F"), device=device)
                    for s in self.systems]
        self.lfac = [torch.as_tensor(np.asfortranarray(s.lfac).ravel(order="F"), device=device)
                     for s in self.systems]
        self._host = []
        self.indn = []
        self.structs = (_lib.GcSystem * len(self.systems))()
        for i, s in enumerate(self.systems):
            indn = pair_space(s.occ, s.nele)
            self.indn.append(indn)
            occ = np.ascontiguousarray(s.occ, dtype=np.float64)
            xone = np.ascontiguousarray(s.xone, dtype=np.float64)
            ind = np.ascontiguousarray(indn, dtype=np.int32).ravel()
            rdm = np.ascontiguousarray(s.rdm2act, dtype=np.float64)
            self._host.append((occ, xone, ind, rdm))
            st = self.structs[i]
            st.nbas, st.ninact, st.nact, st.ndimx, st.rank = s.n, s.nin, s.nact, len(indn), s.rank
            st.occ, st.xone, st.indn, st.rdm2act = _dptr(occ), _dptr(xone), _iptr(ind), _dptr(rdm)
        self.refresh_pointers()

    def subset(self, idx) -> "BatchInputs":
        """A batch of some of these systems that shares their device buffers."""
        sub = BatchInputs.__new__(BatchInputs)
        idx = [int(i) for i in idx]
        sub.systems = [self.systems[i] for i in idx]
        sub.device = self.device
        sub.cmo = [self.cmo[i] for i in idx]
        sub.lfac = [self.lfac[i] for i in idx]
        sub._host = [self._host[i] for i in idx]
        sub.indn = [self.indn[i] for i in idx]
        sub.structs = (_lib.GcSystem * len(idx))()
        for k, i in enumerate(idx):
            sub.structs[k] = self.structs[i]
        return sub

    def refresh_pointers(self):
        for i in range(len(self.systems)):
            self.structs[i].cmo_dev = self.cmo[i].data_ptr()
            self.structs[i].lfac_dev = self.lfac[i].data_ptr()

    def ndimx(self):
        return [len(x) for x in self.indn]


def ac_energy_batched(batch: BatchInputs, ngrid: int = 8, precision: str = "fp64tc5",
                      erpa_mode: str = "cholesky", affine: bool = True, nstreams: int = 8,
                      eig_emulation: bool = False, lambdas=None, weights=None,
                      omega_stats: bool = False, eig_refine: int = 0, ctx: Context | None = None):
    """ACECORR over a batch. Returns (ecorr, ecas, W[nsys, npoints], status) and,
    with omega_stats, the excitation-energy statistics [nsys, npoints, 6].
    lambdas/weights select explicit quadrature points instead of Gauss-Legendre."""
    ctx = ctx or default_context(torch.device(batch.device).index or 0)
    nsys = len(batch.systems)
    lam = wts = None
    if lambdas is not None:
        lam = np.ascontiguousarray(lambdas, dtype=np.float64)
        ngrid = lam.shape[0]
        wts = np.ascontiguousarray(weights if weights is not None else np.zeros(ngrid),
                                   dtype=np.float64)
    par = _lib.GcAcParams(ngrid, PREC[precision], ERPA[erpa_mode], int(affine), nstreams,
                          int(eig_emulation), int(eig_refine),
                          _dptr(lam) if lam is not None else None,
                          _dptr(wts) if wts is not None else None)
    ecorr = np.zeros(nsys)
    ecas = np.zeros(nsys)
    wl = np.zeros((nsys, ngrid))
    st = np.zeros((nsys, ngrid, 6)) if omega_stats else None
    status = np.zeros(nsys, dtype=np.int32)
    check(ctx.h, load().gc_ac_energy_batched(ctx.h, nsys, batch.structs, C.byref(par),
                                             _dptr(ecorr), _dptr(ecas), _dptr(wl),
                                             _dptr(st) if st is not None else None,
                                             _iptr(status)))
    if omega_stats:
        return ecorr, ecas, wl, status, st
    return ecorr, ecas, wl, status

def autotune_streams(batch: BatchInputs, candidates=(4, 8, 12, 16), sample: int = 16,
                     points: int = 2, precision: str = "fp64tc5", erpa_mode: str = "refined",
                     ctx: Context | None = None):
    """Choose the worker-stream count of ac_energy_batched for a batch: one pass of
    `points` lambda points over the `sample` largest systems per candidate (after
    one untimed pass), timed on the device; returns (best, {candidate: seconds}).
    The large systems set the step time, and concurrency between their library
    eigensolves is what the stream count trades against memory."""
    import time
    ctx = ctx or default_context(torch.device(batch.device).index or 0)
    nd = np.asarray(batch.ndimx())
    sub = batch.subset(np.argsort(-nd, kind="stable")[:sample])
    lams = np.linspace(0.1, 0.9, points)
    kw = dict(lambdas=lams, precision=precision, erpa_mode=erpa_mode, ctx=ctx)
    ac_energy_batched(sub, nstreams=candidates[0], **kw)
    times = {}
    for ns in candidates:
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        ac_energy_batched(sub, nstreams=int(ns), **kw)
        torch.cuda.synchronize()
        times[int(ns)] = time.perf_counter() - t0
    return min(times, key=times.get), times


class AcSession:
    """Batch with per-system device state kept between calls (gc_ac_session_*):
    points(idx, lambdas) evaluates W(lambda) for some systems, building a
    system's integrals and A+-B at lambda = 0, 1 on its first use only."""

    def __init__(self, batch: BatchInputs, precision: str = "fp64tc5",
                 erpa_mode: str = "refined", nstreams: int = 8, eig_emulation: bool = False,
                 eig_refine: int = 0, ctx: Context | None = None):
        self.ctx = ctx or default_context(torch.device(batch.device).index or 0)
        self.batch = batch  # keeps the host arrays and device buffers alive
        par = _lib.GcAcParams(0, PREC[precision], ERPA[erpa_mode], 1, nstreams,
                              int(eig_emulation), int(eig_refine), None, None)
        h = C.c_void_p()
        check(self.ctx.h, load().gc_ac_session_create(self.ctx.h, len(batch.systems),
                                                      batch.structs, C.byref(par), C.byref(h)))
        self.h = h

    def points(self, idx, lambdas, omega_stats: bool = False):
        """W[len(idx), len(lambdas)], E_CAS[len(idx)], status[len(idx)] (and the
        excitation statistics [len(idx), len(lambdas), 6] with omega_stats)."""
        idx = np.ascontiguousarray(idx, dtype=np.int32)
        lam = np.ascontiguousarray(lambdas, dtype=np.float64)
        w = np.zeros((idx.size, lam.size))
        st = np.zeros((idx.size, lam.size, 6)) if omega_stats else None
        ecas = np.zeros(idx.size)
        status = np.zeros(idx.size, dtype=np.int32)
        check(self.ctx.h, load().gc_ac_session_points(self.h, idx.size, _iptr(idx), lam.size,
                                                      _dptr(lam), _dptr(w),
                                                      _dptr(st) if st is not None else None,
                                                      _dptr(ecas), _iptr(status)))
        return (w, ecas, status, st) if omega_stats else (w, ecas, status)

    def close(self):
        if self.h:
            load().gc_ac_session_destroy(self.h)
            self.h = None

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def tc_gemm_time(m: int, n: int, k: int, precision: str = "bf16x6", reps: int = 10,
                 ctx: Context | None = None) -> float:
    """Milliseconds per launch of the tensor-core GEMM kernel (CUDA events)."""
    ctx = ctx or default_context(0)
    ms = C.c_double()
    check(ctx.h, load().gc_tc_gemm_time(ctx.h, PREC[precision], m, n, k, reps, C.byref(ms)))
    return ms.value


# ------------------------------------------------------------------ surrogate
class Mlp:
    """The integrand surrogate network, trained and evaluated by this library's kernels."""

    def __init__(self, in_dim: int, hidden: int = 256, out_dim: int = 8, seed: int = 0,
                 ctx: Context | None = None):
        self.ctx = ctx or default_context(0)
        self.in_dim, self.hidden, self.out_dim = in_dim, hidden, out_dim
        h = C.c_void_p()
        check(self.ctx.h, load().gc_mlp_create(self.ctx.h, in_dim, hidden, out_dim, seed,
                                               C.byref(h)))
        self.h = h
        self.nparam = int(load().gc_mlp_num_params(h))

    def __del__(self):
        try:
            if self.h:
                load().gc_mlp_destroy(self.h)
        except Exception:
            pass

    @staticmethod
    def _dev(x) -> torch.Tensor:
        return torch.as_tensor(x).to(device="cuda", dtype=torch.float32).contiguous()

    def params(self) -> torch.Tensor:
        p = torch.empty(self.nparam, dtype=torch.float32, device="cuda")
        check(self.ctx.h, load().gc_mlp_get_params(self.ctx.h, self.h, _ptr(p)))
        return p

    def set_params(self, p):
        p = self._dev(p)
        check(self.ctx.h, load().gc_mlp_set_params(self.ctx.h, self.h, _ptr(p)))

    def forward(self, x) -> torch.Tensor:
        x = self._dev(x)
        y = torch.empty((x.shape[0], self.out_dim), dtype=torch.float32, device="cuda")
        check(self.ctx.h, load().gc_mlp_forward(self.ctx.h, self.h, x.shape[0], _ptr(x), _ptr(y)))
        return y

    def gradients(self, x, t):
        x, t = self._dev(x), self._dev(t)
        g = torch.empty(self.nparam, dtype=torch.float32, device="cuda")
        loss = C.c_float()
        check(self.ctx.h, load().gc_mlp_gradients(self.ctx.h, self.h, x.shape[0], _ptr(x), _ptr(t),
                                                  _ptr(g), C.byref(loss)))
        return loss.value, g

    def train_step(self, x, t, lr: float) -> float:
        x, t = self._dev(x), self._dev(t)
        loss = C.c_float()
        check(self.ctx.h, load().gc_mlp_train_step(self.ctx.h, self.h, x.shape[0], _ptr(x), _ptr(t),
                                                   float(lr), C.byref(loss)))
        return loss.value
