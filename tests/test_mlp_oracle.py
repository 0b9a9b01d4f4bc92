"""The network oracle: analytic gradient against finite differences, BF16 rounding."""
import numpy as np

from oracle import mlp


def test_bf16_round_to_nearest_even():
    x = np.array([1.0, 1.0 + 2.0 ** -8, 1.0 + 3 * 2.0 ** -8, 1.0 + 2.0 ** -9, -2.5, 3.0e38],
                 dtype=np.float32)
    r = mlp.bf16(x)
    # 1 + 2^-8 is a tie between 1 and 1 + 2^-7: even mantissa (1) wins
    assert r[0] == 1.0 and r[1] == 1.0
    assert r[2] == np.float32(1.0 + 2.0 ** -6)  # tie, rounds up to the even neighbour
    assert r[3] == 1.0
    assert r[4] == -2.5
    assert np.isfinite(r[5])
    assert np.isnan(mlp.bf16(np.array([np.nan], dtype=np.float32)))[0]


def test_gradient_matches_finite_differences():
    dims = (7, 16, 2, 3)
    rng = np.random.default_rng(3)
    p = mlp.glorot(*dims, seed=1).astype(np.float64)
    _, n = mlp.layout(*dims)
    p[:] += 0.05 * rng.normal(size=n)  # non-zero biases as well
    X = rng.normal(size=(5, dims[0]))
    T = rng.normal(size=(5, dims[3]))
    loss, g = mlp.loss_and_grad(p, X, T, dims, emulate=False)
    h = 1e-6
    fd = np.empty(n)
    for i in range(n):
        e = np.zeros(n)
        e[i] = h
        lp, _ = mlp.loss_and_grad(p + e, X, T, dims, emulate=False)
        lm, _ = mlp.loss_and_grad(p - e, X, T, dims, emulate=False)
        fd[i] = (lp - lm) / (2 * h)
    assert np.abs(g - fd).max() <= 1e-7 * max(1.0, np.abs(fd).max()), np.abs(g - fd).max()


def test_emulated_gradient_close_to_exact():
    """BF16 operand rounding perturbs the gradient at the 2^-8 level, not more."""
    dims = (33, 64, 3, 2)
    rng = np.random.default_rng(4)
    p = mlp.glorot(*dims, seed=2)
    X = rng.normal(size=(40, dims[0])).astype(np.float32)
    T = rng.normal(size=(40, dims[3])).astype(np.float32)
    _, g64 = mlp.loss_and_grad(p, X, T, dims, emulate=False)
    _, gbf = mlp.loss_and_grad(p, X, T, dims, emulate=True)
    assert np.linalg.norm(gbf - g64) <= 2e-2 * np.linalg.norm(g64)


def test_adamw_first_step_is_signed_lr():
    p = np.array([1.0, -2.0, 0.5])
    g = np.array([0.3, -1e-3, 2.0])
    q, m, v = mlp.adamw(p, g, np.zeros(3), np.zeros(3), 1, lr=1e-2, wd=0.0)
    np.testing.assert_allclose(q, p - 1e-2 * np.sign(g), rtol=1e-6)
