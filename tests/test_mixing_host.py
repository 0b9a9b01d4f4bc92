"""Host-side pieces of the learned SCBA mixing: the Chebyshev projector behind the features,
the DIIS (Pulay) coefficients, and the training targets (each orbital's step along R_bar
towards the fixed point)."""
import numpy as np

from quantum_transport_gb300 import mixing


def test_chebyshev_projector_recovers_coefficients():
    nE = 256
    Qt = mixing.chebyshev_projector(nE)
    assert Qt.shape == (nE, mixing.NCOEF)
    c = np.random.default_rng(0).normal(size=mixing.NCOEF)
    s = np.polynomial.chebyshev.chebval(np.linspace(-1.0, 1.0, nE), c)
    np.testing.assert_allclose(Qt.T @ s, c, atol=1e-8)


def test_pulay_coefficients_minimise_the_combined_residual():
    rng = np.random.default_rng(1)
    R = rng.normal(size=(3, 40))
    c = mixing.pulay_coefficients(R @ R.T)
    assert abs(c.sum() - 1.0) < 1e-12
    w = np.linalg.solve(R @ R.T, np.ones(3))
    np.testing.assert_allclose(c, w / w.sum(), rtol=1e-8)
    best = np.linalg.norm(c @ R)
    for _ in range(16):  # any other affine combination leaves a larger residual
        d = rng.normal(size=3)
        d -= d.mean()
        assert np.linalg.norm((c + 0.1 * d) @ R) >= best


def test_pulay_coefficients_take_a_vanished_residual():
    R = np.array([[1.0, 2.0, 3.0], [0.0, 0.0, 0.0], [3.0, 1.0, 2.0]])
    c = mixing.pulay_coefficients(R @ R.T)
    assert abs(c.sum() - 1.0) < 1e-12
    assert np.linalg.norm(c @ R) < 1e-10


def test_recorder_targets_are_the_clipped_steps_to_the_fixed_point():
    rng = np.random.default_rng(2)
    nE, norb = 16, 6
    a_true = np.array([0.5, 1.0, 2.0, 3.9, 5.0, -1.0])
    s_star = rng.normal(size=(2, nE, norb))
    r = rng.normal(size=(2, nE, norb))
    rec = mixing.Recorder()
    feats = rng.normal(size=(norb, mixing.N_IN)).astype(np.float32)
    rec.add(feats, s_star - a_true * r, r)
    X, T = rec.targets(s_star)
    assert X.shape == (norb, mixing.N_IN) and T.shape == (norb, 1)
    np.testing.assert_array_equal(X, feats)
    np.testing.assert_allclose(T[:, 0], np.clip(a_true, 0.0, mixing.ALPHA_MAX), rtol=1e-6)
    X0, T0 = mixing.Recorder().targets(s_star)
    assert X0.shape == (0, mixing.N_IN) and T0.shape == (0, 1)
