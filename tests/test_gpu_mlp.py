"""The learned-mixing network's tensor-core kernels against the CPU oracle."""
import numpy as np
import pytest

from oracle import mlp as orc
from quantum_transport_gb300.mlp import Mlp

pytestmark = pytest.mark.gpu

# the mixing network's shape: 6 x 64 Chebyshev coefficients + 2 residual features -> 2 weights
DIMS = (386, 512, 4, 2)


def _data(seed, batch, dims):
    rng = np.random.default_rng(seed)
    X = rng.normal(size=(batch, dims[0])).astype(np.float32)
    T = rng.normal(size=(batch, dims[3])).astype(np.float32)
    return X, T


@pytest.mark.parametrize("batch", [1, 130, 300])
def test_forward_matches_oracle(ctx, batch):
    p = orc.glorot(*DIMS, seed=5)
    net = Mlp(ctx, *DIMS, max_batch=512, params=p)
    X, _ = _data(1, batch, DIMS)
    y = net.infer(X)
    ref, _ = orc.forward(p, X, DIMS, emulate=True)
    # same BF16 operands; FP32 accumulation order differs from the float64 oracle
    assert np.abs(y - ref).max() <= 1e-3 * max(1.0, np.abs(ref).max()), np.abs(y - ref).max()


@pytest.mark.parametrize("dims", [DIMS, (7, 40, 2, 3), (64, 128, 1, 130)])
def test_gradient_matches_oracle(ctx, dims):
    p = orc.glorot(*dims, seed=6)
    rng = np.random.default_rng(7)
    lay, n = orc.layout(*dims)
    for din, dout, wo, bo in lay:
        p[bo:bo + dout] = 0.1 * rng.normal(size=dout)
    net = Mlp(ctx, *dims, max_batch=256, params=p)
    X, T = _data(2, 200, dims)
    loss, g = net.grad(X, T)
    lref, gref = orc.loss_and_grad(p, X, T, dims, emulate=True)
    assert abs(loss - lref) <= 1e-4 * lref
    for din, dout, wo, bo in lay:
        for lo, hi in ((wo, wo + din * dout), (bo, bo + dout)):
            err = np.linalg.norm(g[lo:hi] - gref[lo:hi]) / np.linalg.norm(gref[lo:hi])
            assert err <= 5e-3, (lo, hi, err)


def test_adamw_step_matches_oracle(ctx):
    dims = (33, 64, 2, 4)
    p = orc.glorot(*dims, seed=8)
    net = Mlp(ctx, *dims, max_batch=64, params=p)
    X, T = _data(3, 50, dims)
    _, g = net.grad(X, T)
    net.train_step(X, T, lr=3e-3, weight_decay=0.01)
    q = net.params()
    ref, _, _ = orc.adamw(p, g, np.zeros_like(p), np.zeros_like(p), 1, lr=3e-3, wd=0.01)
    np.testing.assert_allclose(q, ref, rtol=1e-5, atol=1e-6)


def test_training_fits_a_smooth_map(ctx):
    """The GPU training loop (forward, backward, AdamW kernels) learns y = sin(a.x)."""
    dims = (16, 128, 2, 2)
    rng = np.random.default_rng(9)
    A = rng.normal(size=(dims[0], dims[3])) / 4
    X = rng.normal(size=(1024, dims[0])).astype(np.float32)
    T = np.sin(X @ A).astype(np.float32)
    net = Mlp(ctx, *dims, max_batch=1024, seed=11)
    first = net.train_step(X, T, lr=3e-3)
    for _ in range(300):
        last = net.train_step(X, T, lr=3e-3, want_loss=False)
    last = net.train_step(X, T, lr=3e-3)
    assert last < 0.05 * first, (first, last)
