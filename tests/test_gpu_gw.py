"""GW/SCBA GPU path against the FP64 GW oracle (parity of the reference unpinned:
its GW module does not build and has no fixtures)."""
import numpy as np
import pytest

from oracle import gw as ogw
from quantum_transport_gb300.devices import make_chain_device

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("n", [16, 64, 255, 2048])
def test_corr_conv_batch(ctx, n):
    import torch
    from quantum_transport_gb300 import gw
    rng = np.random.default_rng(n)
    X = rng.normal(size=(n, 5)) + 1j * rng.normal(size=(n, 5))
    Y = rng.normal(size=(n, 5)) + 1j * rng.normal(size=(n, 5))
    Xd, Yd = torch.from_numpy(X).cuda(), torch.from_numpy(Y).cuda()
    for mode, f in (("corr", ogw.corr), ("conv", ogw.conv)):
        Z = gw.corr(ctx, Xd, Yd, mode).cpu().numpy()
        ref = f(X.T, Y.T).T
        np.testing.assert_allclose(Z, ref, rtol=0, atol=1e-11 * np.abs(ref).max())
    if n <= 64:
        np.testing.assert_allclose(gw.corr(ctx, Xd, Yd, "corr").cpu().numpy(),
                                   ogw.corr_direct(X.T, Y.T).T, atol=1e-10)


def _system(ctx, precision="fp64"):
    from quantum_transport_gb300 import gw
    dev = make_chain_device(6, 8, 64, -4.0, 4.0, seed=3)
    V = ogw.coulomb_blocks(8)
    s = gw.GwSystem(ctx, dev.H00[0], dev.H10, dev.E, dev.nx, V, mu=(0.1, -0.1),
                    precision=precision)
    return dev, V, s


def test_gw_step_vs_oracle(ctx):
    from quantum_transport_gb300 import gw
    dev, V, s = _system(ctx)
    rng = np.random.default_rng(0)
    shape = (len(dev.E), dev.nx, 8, 8)
    SL0 = 1e-2 * (rng.normal(size=shape) + 1j * rng.normal(size=shape))
    SL0 = (SL0 - np.conj(np.swapaxes(SL0, -1, -2))) / 2      # anti-Hermitian Sigma^<
    SR0 = 1e-2 * (rng.normal(size=shape) - 1j * np.abs(rng.normal(size=shape)))
    SR0 = (SR0 + np.swapaxes(SR0, -1, -2)) / 2
    NR, NL, NG = s.step(gw.to_dev(SR0), gw.to_dev(SL0))
    GR, GL, GG = ogw.green(dev.E, dev.H00[0], dev.H10, dev.nx, SR0, SL0, mu=(0.1, -0.1),
                           temp=(300.0, 300.0))
    GR, GL, GG = ogw.zero_real(GR, GL, GG)
    dE = dev.E[1] - dev.E[0]
    P = ogw.polarization(GR, GL, GG, dE)
    W = ogw.screened(V, *P)
    ref = [ogw.copy_edges(x) for x in ogw.self_energy(GR, GL, GG, *W, dE)]
    for got, exp in zip((NR, NL, NG), ref):
        g = gw.from_dev(got)
        np.testing.assert_allclose(g, exp, rtol=0, atol=1e-8 * np.abs(exp).max())


def test_scba_converges_like_oracle(ctx):
    from quantum_transport_gb300 import gw
    dev, V, s = _system(ctx)
    SR, SL, SG, res = s.scba(alpha=0.3, tol=1e-8, max_iter=80)
    assert res[-1] <= 1e-8
    oR, oL, oG, ores = ogw.scba(dev.E, dev.H00[0], dev.H10, V, dev.nx, mu=(0.1, -0.1),
                               temp=(300.0, 300.0), max_iter=80)
    assert abs(len(res) - len(ores)) <= 1
    for got, exp in zip((SR, SL, SG), (oR, oL, oG)):
        np.testing.assert_allclose(gw.from_dev(got), exp, rtol=0, atol=1e-7 * np.abs(exp).max())
