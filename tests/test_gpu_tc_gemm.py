"""The split-precision tcgen05 GEMM against an FP64 product.

Error bounds, relative to the entries of |A| |B|^T: 3-pass BF16 (hi*hi +
hi*lo + lo*hi) 2e-5; 6-pass BF16 (three planes) 1e-6 (FP32 accumulation
dominates); sliced forms (exact integer partial sums) 2e-8 with 4 slices,
5e-10 with 5 and 5e-12 with 6 (truncation after 28 / 35 / 42 bits of the row
maxima; a CPU emulation of the same slicing gives up to 1.5e-10 / 1.2e-12 for
5 / 6 slices).
"""
import pytest
import torch

from gammcor_gb300 import api
from gammcor_gb300._lib import GcError

pytestmark = pytest.mark.gpu
BOUND = {"bf16x3": 2e-5, "bf16x6": 1e-6, "fp64tc4": 2e-8, "fp64tc5": 5e-10, "fp64tc6": 5e-12}


@pytest.mark.parametrize("precision", ["bf16x3", "bf16x6", "fp64tc4", "fp64tc5", "fp64tc6"])
@pytest.mark.parametrize("m,n,k", [(128, 128, 64), (200, 150, 300), (1000, 700, 513),
                                   (7, 300, 40), (640, 90, 1500)])
def test_tc_gemm_matches_fp64(gpu_lib, precision, m, n, k):
    g = torch.Generator(device="cuda").manual_seed(m * 7 + n * 3 + k)
    A = torch.randn(m, k, dtype=torch.float64, device="cuda", generator=g)
    B = torch.randn(n, k, dtype=torch.float64, device="cuda", generator=g)
    A[:, ::3] *= 1e-3          # mixed magnitudes
    C = api.tc_gemm_nt(A, B, precision)
    ref = A @ B.T
    scale = (A.abs() @ B.abs().T)
    err = ((C - ref).abs() / scale).max().item()
    assert err < BOUND[precision], err


def test_sliced_gemm_long_k_and_wide_range(gpu_lib):
    """K spanning many exact chunks, rows 1e12 apart and B rows dominated by a
    1e6-scaled block (the exact-slicing emulation gives 6.5e-10 / 5.1e-12 here)."""
    g = torch.Generator(device="cuda").manual_seed(7)
    A = torch.randn(300, 5000, dtype=torch.float64, device="cuda", generator=g)
    B = torch.randn(260, 5000, dtype=torch.float64, device="cuda", generator=g)
    A[::2] *= 1e-12
    B[:, 100:200] *= 1e6
    ref = A @ B.T
    scale = A.abs() @ B.abs().T
    for prec, bound in (("fp64tc5", 2e-9), ("fp64tc6", 2e-11)):
        C = api.tc_gemm_nt(A, B, prec)
        assert ((C - ref).abs() / scale).max().item() < bound


def test_tc_gemm_repeated_calls_agree(gpu_lib):
    A = torch.randn(300, 257, dtype=torch.float64, device="cuda")
    B = torch.randn(190, 257, dtype=torch.float64, device="cuda")
    c1 = api.tc_gemm_nt(A, B, "bf16x6")
    c2 = api.tc_gemm_nt(A, B, "bf16x6")
    assert torch.equal(c1, c2)


@pytest.mark.parametrize("precision,widths", [("fp64tc4", (64, 96, 128)), ("fp64tc5", (64, 96)),
                                              ("fp64tc6", (64,))])
def test_sliced_gemm_tile_widths_give_identical_bits(gpu_lib, precision, widths):
    """Every column tile width computes each element from the same exact integer
    sums, so forced widths and the automatic choice agree bit for bit, ragged
    edges included (n not a multiple of any width)."""
    g = torch.Generator(device="cuda").manual_seed(11)
    A = torch.randn(1000, 513, dtype=torch.float64, device="cuda", generator=g)
    B = torch.randn(700, 513, dtype=torch.float64, device="cuda", generator=g)
    A[:, ::5] *= 1e-4
    ctx = api.Context(0)
    try:
        ref = api.tc_gemm_nt(A, B, precision, ctx=ctx)
        for w in widths:
            ctx.set_gemm_tile(w)
            assert torch.equal(api.tc_gemm_nt(A, B, precision, ctx=ctx), ref), w
        ctx.set_gemm_tile(0)
    finally:
        ctx.close()
    exact = A @ B.T
    assert ((ref - exact).abs() / (A.abs() @ B.abs().T)).max().item() < BOUND[precision]


def test_gemm_tile_setting_rejects_other_widths(gpu_lib):
    ctx = api.Context(0)
    try:
        with pytest.raises(GcError):
            ctx.set_gemm_tile(80)
    finally:
        ctx.close()
