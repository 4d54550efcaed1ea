"""The surrogate network's kernels against the CPU restatement (oracle/mlp_ref.py).

Forward outputs and gradients of every parameter block agree to 1e-4 relative
to the block's largest entry (FP32 accumulation on the GPU, FP64 in the oracle,
same BF16 weights); a few hundred Adam steps lower the loss tenfold.
"""
import numpy as np
import pytest
import torch

from gammcor_gb300 import api
from oracle import mlp_ref

pytestmark = pytest.mark.gpu


def test_mlp_forward_and_gradients_match_oracle(gpu_lib):
    rng = np.random.default_rng(3)
    din, hid, dout, B = 19, 256, 8, 96
    net = api.Mlp(din, hid, dout, seed=11)
    x = rng.standard_normal((B, din)).astype(np.float32)
    t = rng.standard_normal((B, dout)).astype(np.float32)
    p = net.params().cpu().numpy()
    dims = [din, hid, hid, hid, dout]
    y_ref, _, _ = mlp_ref.forward(p, dims, x)
    y = net.forward(x).cpu().numpy()
    assert np.abs(y - y_ref).max() < 1e-4 * np.abs(y_ref).max()
    loss_ref, g_ref = mlp_ref.loss_and_grad(p, dims, x, t)
    loss, g = net.gradients(x, t)
    g = g.cpu().numpy()
    assert abs(loss - loss_ref) < 1e-4 * loss_ref
    off = 0
    for l in range(4):
        for size in (dims[l] * dims[l + 1], dims[l + 1]):
            blk, ref = g[off:off + size], g_ref[off:off + size]
            assert np.abs(blk - ref).max() < 1e-4 * max(np.abs(ref).max(), 1e-12), (l, size)
            off += size


def test_mlp_training_lowers_loss(gpu_lib):
    rng = np.random.default_rng(4)
    din, B = 12, 256
    x = rng.standard_normal((B, din)).astype(np.float32)
    w = rng.standard_normal((din, 8)).astype(np.float32)
    t = np.tanh(x @ w).astype(np.float32)
    net = api.Mlp(din, 256, 8, seed=1)
    xd, td = torch.tensor(x, device="cuda"), torch.tensor(t, device="cuda")
    first = net.train_step(xd, td, 1e-3)
    for _ in range(300):
        last = net.train_step(xd, td, 1e-3)
    assert last < 0.1 * first, (first, last)
