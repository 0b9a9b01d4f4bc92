"""The GW map over a k-point grid and with the ndiag band on the GPU, against the oracle's
k-pair sums, which tests/test_gw_kpoints.py pins to the reference's literal loops
(src/gw_mod.f90:466-555, 640-730)."""
import numpy as np
import pytest

from oracle import gw as ogw
from quantum_transport_gb300.devices import make_chain_device
from test_gpu_gw import _physical_sigma

pytestmark = pytest.mark.gpu

MU, TEMP = (0.1, -0.1), (300.0, 300.0)


def _kproblem(nky, nkz, nE=48, nx=6, nm=6):
    nk = nky * nkz
    dev = make_chain_device(nx, nm, nE, -4.0, 4.0, seed=11, nk=nk)
    V0 = ogw.coulomb_blocks(nm)
    V = np.stack([V0 * (1.0 + 0.1 * np.cos(2 * np.pi * q / nk)) for q in range(nk)])
    parts = [_physical_sigma(nE, nx, nm, seed=k) for k in range(nk)]
    SR = np.stack([p[0] for p in parts])
    SL = np.stack([p[1] for p in parts])
    return dev, V, SR, SL


def _gpu_system(ctx, dev, V, nky, nkz, ndiag):
    from quantum_transport_gb300 import gw
    nk = nky * nkz
    H00 = dev.H00 if nk > 1 else dev.H00[0]
    return gw.GwSystem(ctx, H00, dev.H10, dev.E, dev.nx, V if nk > 1 else V[0], mu=MU,
                       kgrid=(nky, nkz), ndiag=ndiag)


def _host(T, nk):
    from quantum_transport_gb300 import gw
    g = gw.from_dev(T)
    return g if nk > 1 else g[None]


@pytest.mark.parametrize("nky,nkz,ndiag", [(1, 2, None), (2, 2, None), (1, 3, 2), (1, 1, 1)])
def test_gw_step_kgrid_vs_oracle(ctx, nky, nkz, ndiag):
    from quantum_transport_gb300 import gw
    nk = nky * nkz
    dev, V, SR0, SL0 = _kproblem(nky, nkz)
    s = _gpu_system(ctx, dev, V, nky, nkz, ndiag)
    sr, sl = (SR0, SL0) if nk > 1 else (SR0[0], SL0[0])
    N = s.step(gw.to_dev(sr), gw.to_dev(sl))
    H10k = np.repeat(dev.H10[None], nk, axis=0)
    ref = ogw.gw_map_k(dev.E, dev.H00, H10k, V, dev.nx, SR0, SL0, nky=nky, nkz=nkz, mu=MU,
                       temp=TEMP, ndiag=ndiag)
    outside = ~ogw.band_mask(dev.nm, ndiag)
    for got, exp in zip(N, ref):
        g = _host(got, nk)
        assert np.isfinite(exp).all() and np.abs(exp).max() > 0
        np.testing.assert_allclose(g, exp, rtol=0, atol=1e-8 * np.abs(exp).max())
        assert (g[..., outside] == 0).all()


def test_scba_kgrid_converges_like_oracle(ctx):
    nky, nkz, ndiag = 1, 2, 3
    dev, V, _, _ = _kproblem(nky, nkz, nE=32)
    s = _gpu_system(ctx, dev, V, nky, nkz, ndiag)
    SR, SL, SG, res = s.scba(alpha=0.3, tol=1e-8, max_iter=60)
    assert res[-1] <= 1e-8
    H10k = np.repeat(dev.H10[None], 2, axis=0)
    oR, oL, oG, ores = ogw.scba_k(dev.E, dev.H00, H10k, V, dev.nx, nky=nky, nkz=nkz, mu=MU,
                                  temp=TEMP, max_iter=60, ndiag=ndiag)
    assert abs(len(res) - len(ores)) <= 1
    for got, exp in zip((SR, SL, SG), (oR, oL, oG)):
        np.testing.assert_allclose(_host(got, 2), exp, rtol=0, atol=1e-7 * np.abs(exp).max())


def _cplx(rng, shape):
    return rng.normal(size=shape) + 1j * rng.normal(size=shape)


def test_stage_entries_sum_over_k_pairs(ctx):
    """qt_gw_polarization / qt_gw_selfenergy with the context's 2 x 2 grid: arrays
    [nk][n][nseries], P_q = sum_k corr(X_k, Y_kd), Sigma_k = sum_q conv(X_kd, Y_q)."""
    import torch
    from quantum_transport_gb300 import _lib
    from quantum_transport_gb300.rgf import _ptr
    nky, nkz = 2, 2
    nk, n, ns = 4, 40, 7
    rng = np.random.default_rng(2)
    A = [_cplx(rng, (nk, n, ns)) for _ in range(6)]
    dev = [torch.from_numpy(a).cuda() for a in A]
    lib = ctx._lib
    flags = _lib.QT_FLAG_DEVICE_POINTERS | _lib.QT_FLAG_SYNC
    _lib.check(lib.qt_ctx_set_gw_grid(ctx.handle, nky, nkz, -1))
    try:
        P = [torch.zeros_like(dev[0]) for _ in range(3)]
        _lib.check(lib.qt_gw_polarization(ctx.handle, n, ns, *[_ptr(d) for d in dev[:5]], 0.37,
                                          *[_ptr(p) for p in P], flags))
        S = [torch.zeros_like(dev[0]) for _ in range(3)]
        _lib.check(lib.qt_gw_selfenergy(ctx.handle, n, ns, *[_ptr(d) for d in dev], 0.21,
                                        *[_ptr(x) for x in S], flags))
    finally:
        _lib.check(lib.qt_ctx_set_gw_grid(ctx.handle, 1, 1, -1))
    im = lambda X: 1j * X.imag
    ser = lambda X: X.T  # (n, ns) -> (ns, n): series along the last axis
    gr, gl, gg, glt, ggt = (np.array([im(a[k]) for k in range(nk)]) for a in A[:5])
    refP = [np.zeros((nk, n, ns), dtype=complex) for _ in range(3)]
    for q in range(nk):
        for k in range(nk):
            d = ogw.kd_index(k, q, nky, nkz)
            refP[0][q] += (ogw.corr(ser(gl[k]), np.conj(ser(gr[d])))
                           + ogw.corr(ser(gr[k]), ser(glt[d]))).T
            refP[1][q] += ogw.corr(ser(gl[k]), ser(ggt[d])).T
            refP[2][q] += ogw.corr(ser(gg[k]), ser(glt[d])).T
    for got, exp in zip(P, refP):
        exp = -0.37j * exp
        np.testing.assert_allclose(got.cpu().numpy(), exp, rtol=0, atol=1e-12 * np.abs(exp).max())
    wr, wl, wg = A[3], A[4], A[5]
    refS = [np.zeros((nk, n, ns), dtype=complex) for _ in range(3)]
    for k in range(nk):
        for q in range(nk):
            d = ogw.kd_index(k, q, nky, nkz)
            refS[0][k] += (ogw.conv(ser(gl[d]), ser(wr[q])) + ogw.conv(ser(gr[d]), ser(wl[q]))
                           + ogw.conv(ser(gr[d]), ser(wr[q]))).T
            refS[1][k] += ogw.conv(ser(gl[d]), ser(wl[q])).T
            refS[2][k] += ogw.conv(ser(gg[d]), ser(wg[q])).T
    for got, exp in zip(S, refS):
        exp = 0.21j * exp
        np.testing.assert_allclose(got.cpu().numpy(), exp, rtol=0, atol=1e-12 * np.abs(exp).max())


@pytest.mark.parametrize("nky,nkz", [(1, 1), (1, 2)])
def test_gw_step_per_slab_coulomb_blocks(ctx, nky, nkz):
    """V per momentum transfer and slab (the reference's Vii(nm, nm, nx, nk)):
    QT_FLAG_V_PER_SLAB, W of slab x from V_{q,x}."""
    from quantum_transport_gb300 import gw
    nk = nky * nkz
    dev, V, SR0, SL0 = _kproblem(nky, nkz, nE=32)
    Vs = np.stack([[V[q] * (1.0 + 0.05 * x) for x in range(dev.nx)] for q in range(nk)])
    H00 = dev.H00 if nk > 1 else dev.H00[0]
    s = gw.GwSystem(ctx, H00, dev.H10, dev.E, dev.nx, Vs if nk > 1 else Vs[0], mu=MU,
                    kgrid=(nky, nkz), ndiag=2)
    sr, sl = (SR0, SL0) if nk > 1 else (SR0[0], SL0[0])
    N = s.step(gw.to_dev(sr), gw.to_dev(sl))
    H10k = np.repeat(dev.H10[None], nk, axis=0)
    ref = ogw.gw_map_k(dev.E, dev.H00, H10k, Vs, dev.nx, SR0, SL0, nky=nky, nkz=nkz, mu=MU,
                       temp=TEMP, ndiag=2)
    for got, exp in zip(N, ref):
        np.testing.assert_allclose(_host(got, nk), exp, rtol=0, atol=1e-8 * np.abs(exp).max())
