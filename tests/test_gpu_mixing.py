"""Learned SCBA mixing: its kernels against numpy, and what the trained network gains.

The learned mixer has no reference counterpart (the reference mixes linearly,
src/gw_mod.f90:747-749).  It is pinned by (a) its kernels against numpy
restatements, (b) the network's gradients against the oracle
(test_gpu_mlp.py), and (c) the plain loop's fixed point: the learned loop must
converge to the same self-energy.
"""
import numpy as np
import pytest

from quantum_transport_gb300 import gw, mixing
from quantum_transport_gb300.devices import disordered_gw_device

pytestmark = pytest.mark.gpu


def _rand_sigma(rng, shape):
    return rng.normal(size=shape) + 1j * rng.normal(size=shape)


def _system(ctx, seed, **kw):
    d = disordered_gw_device(seed, **kw)
    return gw.GwSystem(ctx, d.H00, d.H10, d.E, d.nx, d.V, mu=(0.1, -0.1))


def test_mix_kernels_match_numpy(ctx):
    import torch
    s = _system(ctx, 0, nE=32)
    rng = np.random.default_rng(1)
    shape = (s.nE, s.nx, s.nm, s.nm)
    A = [_rand_sigma(rng, shape) for _ in range(6)]
    dA = [gw.to_dev(a) for a in A]
    ops = mixing.MixOps(s)
    # diagonal series: Im X[e][l][i,i] -> [2][nE][l*nm + i]
    out = torch.empty((2, s.nE, s.nx * s.nm), dtype=torch.float64, device="cuda")
    ops.diag(dA[0], dA[1], out)
    ref = np.stack([np.diagonal(a, axis1=2, axis2=3).imag.reshape(s.nE, -1) for a in A[:2]])
    np.testing.assert_array_equal(out.cpu().numpy(), ref)
    # Gram matrix and affine combination
    G = ops.gram(dA[0:3], dA[3:6])
    Gref = np.array([[np.real(np.vdot(A[i], A[j]) + np.vdot(A[3 + i], A[3 + j]))
                      for j in range(3)] for i in range(3)])
    np.testing.assert_allclose(G, Gref, rtol=1e-12)
    c = np.array([0.5, -0.25, 0.75])
    o = ops.combine(c, dA[0:3], dA[3:6], 0.3, torch.empty_like(dA[0]))
    np.testing.assert_allclose(gw.from_dev(o), sum(c[i] * (A[i] + 0.3 * A[3 + i]) for i in range(3)),
                               rtol=1e-13, atol=1e-13)
    # learned update with per-orbital (a, b) or a alone, clamped
    amax, bmin, bmax = 4.0, -0.5, 0.95
    for ncols in (2, 1):
        ab = rng.uniform(-1.0, 5.0, size=(s.nx * s.nm, ncols)).astype(np.float32)
        abd = torch.from_numpy(ab).cuda()
        o = torch.empty_like(dA[0])
        mixing.check(ctx._lib.qt_mix_apply(ctx.handle, s.nE, s.nx, s.nm, mixing._vp(abd), ncols,
                                           amax, bmin, bmax, mixing._vp(dA[0]), mixing._vp(dA[1]),
                                           mixing._vp(dA[2]), mixing._vp(o), 4))
        a = np.clip(ab[:, 0].astype(np.float64), 0, amax).reshape(s.nx, s.nm)
        b = (np.clip(ab[:, 1].astype(np.float64), bmin, bmax) if ncols == 2
             else np.zeros(s.nx * s.nm)).reshape(s.nx, s.nm)
        aij = 0.5 * (a[:, :, None] + a[:, None, :])
        bij = 0.5 * (b[:, :, None] + b[:, None, :])
        ref = A[0] + aij[None] * A[1] + bij[None] * (A[0] - A[2])
        np.testing.assert_allclose(gw.from_dev(o), ref, rtol=1e-6, atol=1e-6 * np.abs(ref).max())


def test_mix_features_match_numpy(ctx):
    import torch
    nE, norb = 48, 20
    rng = np.random.default_rng(2)
    ring = rng.normal(size=(mixing.NHIST, 2, nE, norb))
    Qt = mixing.chebyshev_projector(nE)
    mixer = mixing.LearnedMixer(ctx, nE, width=32, depth=1, max_batch=64)
    f = torch.empty((norb, mixing.N_IN), dtype=torch.float32, device="cuda")
    mixer.features(torch.from_numpy(ring).cuda(), -3.0, f)
    c = np.einsum("em,hqeo->ohqm", Qt, ring)          # coefficients [o][h][q][m]
    n0 = np.sqrt((c[:, 0] ** 2).sum(axis=(1, 2)))
    n1 = np.sqrt((c[:, 1] ** 2).sum(axis=(1, 2)))
    ref = np.concatenate([np.clip(c / n0[:, None, None, None], -8, 8).reshape(norb, -1),
                          np.full((norb, 1), -3.0 / 8.0),
                          np.clip(np.log10(n0 / n1), -4, 4)[:, None]], axis=1)
    np.testing.assert_allclose(f.cpu().numpy(), ref, rtol=2e-6, atol=2e-6)


def test_chebyshev_projector_is_exact_on_polynomials():
    nE = 100
    x = np.linspace(-1, 1, nE)
    coef = np.random.default_rng(3).normal(size=mixing.NCOEF)
    s = np.polynomial.chebyshev.chebval(x, coef)
    np.testing.assert_allclose(mixing.chebyshev_projector(nE).T @ s, coef, atol=1e-8)


def test_pulay_matches_plain_fixed_point(ctx):
    s = _system(ctx, 7)
    plain = mixing.run_scba(s, method="plain", tol=1e-8, max_iter=200)
    pul = mixing.run_scba(s, method="pulay", tol=1e-8, max_iter=200)
    assert plain.residuals[-1] <= 1e-8 and pul.residuals[-1] <= 1e-8
    assert pul.evaluations < plain.evaluations
    for a, b in zip(pul.sigma, plain.sigma):
        a, b = gw.from_dev(a), gw.from_dev(b)
        assert np.abs(a - b).max() <= 1e-6 * np.abs(b).max()


def test_learned_mixing_gain(ctx):
    """Trained on 12 seeded disorder realisations (Pulay-loop histories, then one round of
    the learned loop's own iterates), evaluated on 4 held-out seeds.  The learned loop
    needs at most half the GW evaluations of plain mixing, no more than the Pulay loop it
    falls back to, and reaches the same fixed point (max |diff| <= 1e-6 of max |Sigma|)."""
    train_sys = [_system(ctx, 100 + i) for i in range(12)]
    test_sys = [_system(ctx, 200 + i) for i in range(4)]
    mixer = mixing.LearnedMixer(ctx, train_sys[0].nE, seed=5)
    X, T, fps, _ = mixing.collect(train_sys)
    mixing.train(mixer, X, T, steps=800, batch=2048, lr=1e-3)
    X2, T2, _, _ = mixing.collect(train_sys, mixer=mixer, fixed_points=fps)
    mixing.train(mixer, np.concatenate([X, X2]), np.concatenate([T, T2]), steps=800,
                 batch=2048, lr=5e-4, seed=1)
    plain_n, pulay_n, learned_n = [], [], []
    for s in test_sys:
        p = mixing.run_scba(s, method="plain", tol=1e-8, max_iter=200)
        u = mixing.run_scba(s, method="pulay", tol=1e-8, max_iter=200)
        q = mixing.run_scba(s, method="learned", mixer=mixer, tol=1e-8, max_iter=200)
        assert p.residuals[-1] <= 1e-8 and u.residuals[-1] <= 1e-8 and q.residuals[-1] <= 1e-8
        for a, b in zip(q.sigma, p.sigma):
            a, b = gw.from_dev(a), gw.from_dev(b)
            assert np.abs(a - b).max() <= 1e-6 * np.abs(b).max()
        plain_n.append(p.evaluations)
        pulay_n.append(u.evaluations)
        learned_n.append(q.evaluations)
    print("plain", plain_n, "pulay", pulay_n, "learned", learned_n)
    assert np.mean(learned_n) <= 0.5 * np.mean(plain_n), (plain_n, learned_n)
    assert np.mean(learned_n) <= np.mean(pulay_n), (pulay_n, learned_n)
