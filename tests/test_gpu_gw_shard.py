"""The GW map in stages on the GPU: the four stage entry points against the oracle, and the
sharded driver on one rank against qt_gw_step / qt_scba_solve (same kernels, same numbers).
More than one rank needs more than one GPU; the exchange itself is covered on host ranks."""
import math

import numpy as np
import pytest

from oracle import gw as ogw
from quantum_transport_gb300.devices import make_chain_device
from test_gpu_gw import _physical_sigma

pytestmark = pytest.mark.gpu


def _system(ctx, precision="fp64", nE=64):
    from quantum_transport_gb300 import gw
    dev = make_chain_device(6, 8, nE, -4.0, 4.0, seed=3)
    V = ogw.coulomb_blocks(8)
    s = gw.GwSystem(ctx, dev.H00[0], dev.H10, dev.E, dev.nx, V, mu=(0.1, -0.1),
                    precision=precision)
    return dev, V, s


def _cplx(rng, shape):
    return rng.normal(size=shape) + 1j * rng.normal(size=shape)


def test_stage_entries_vs_oracle(ctx):
    import torch
    from quantum_transport_gb300.gw_shard import GpuStages
    from test_gw_shard import OracleStages
    rng = np.random.default_rng(7)
    n, nx, c, nm = 40, 3, 5, 4
    dev = make_chain_device(nx, nm, n, -2.0, 2.0, seed=1)
    V = ogw.coulomb_blocks(nm)
    gpu = GpuStages(ctx, dev.H00[0], dev.H10, dev.E, nx, V)
    cpu = OracleStages(dev.E, dev.H00[0], dev.H10, nx, V)
    series = [torch.from_numpy(_cplx(rng, (n, nx, c))) for _ in range(6)]
    on_gpu = lambda ts: [t.cuda() for t in ts]
    close = lambda a, b: np.testing.assert_allclose(
        a.cpu().numpy(), b.numpy(), rtol=0, atol=1e-12 * np.abs(b.numpy()).max())
    for a, b in zip(gpu.polarization(*on_gpu(series[:5]), 0.37), cpu.polarization(*series[:5], 0.37)):
        close(a, b)
    for a, b in zip(gpu.self_energy(*on_gpu(series), 0.21), cpu.self_energy(*series, 0.21)):
        close(a, b)
    P = [torch.from_numpy(1e-2 * _cplx(rng, (n, nx, nm, nm))) for _ in range(3)]
    for a, b in zip(gpu.screened(*on_gpu(P)), cpu.screened(*P)):
        close(a, b)
    S = [torch.from_numpy(_cplx(rng, (n, 6, nm, nm))) for _ in range(3)]
    Sg = on_gpu(S)
    gpu.post(*Sg)
    cpu.post(*S)
    for a, b in zip(Sg, S):
        close(a, b)


@pytest.mark.parametrize("precision", ["fp64", "mixed-fp64"])
def test_one_rank_step_is_qt_gw_step(ctx, precision):
    """Same kernels on the same numbers: the staged map equals the fused one bit for bit."""
    from quantum_transport_gb300 import gw
    from quantum_transport_gb300.gw_shard import ShardedGw
    dev, V, s = _system(ctx, precision)
    SR0, SL0 = _physical_sigma(len(dev.E), dev.nx, 8)
    SR, SL = gw.to_dev(SR0), gw.to_dev(SL0)
    fused = s.step(SR, SL)
    g = ShardedGw.on_gpu(ctx, dev.H00[0], dev.H10, dev.E, dev.nx, V, mu=(0.1, -0.1),
                         precision=precision)
    staged = g.step(SR, SL)
    for a, b in zip(staged, fused):
        b = b.cpu().numpy()
        assert np.isfinite(b).all() and np.abs(b).max() > 0
        np.testing.assert_array_equal(a.cpu().numpy(), b)


def test_one_rank_scba_matches_qt_scba_solve(ctx):
    from quantum_transport_gb300.gw_shard import ShardedGw
    dev, V, s = _system(ctx, nE=48)
    SR, SL, SG, res = s.scba(alpha=0.3, tol=1e-8, max_iter=40)
    g = ShardedGw.on_gpu(ctx, dev.H00[0], dev.H10, dev.E, dev.nx, V, mu=(0.1, -0.1))
    R, L, G, r2 = g.scba(alpha=0.3, tol=1e-8, max_iter=40)
    # the maps agree bit for bit; the mixing and the residual sums round differently, and a
    # residual of 1e-6 carries the round-off of |S| ~ 1 relative to it
    assert len(r2) == len(res)
    np.testing.assert_allclose(r2, res, rtol=1e-6)
    for a, b in zip((R, L, G), (SR, SL, SG)):
        b = b.cpu().numpy()
        assert np.isfinite(b).all()
        np.testing.assert_allclose(a.cpu().numpy(), b, rtol=0, atol=1e-12 * np.abs(b).max())


def test_stage_entries_reject_bad_arguments(ctx):
    import torch
    from quantum_transport_gb300 import _lib
    from quantum_transport_gb300.rgf import _ptr
    lib, h = ctx._lib, ctx.handle
    f = _lib.QT_FLAG_DEVICE_POINTERS
    t = torch.zeros((4, 2, 2), dtype=torch.complex128, device="cuda")
    p = _ptr(t)
    assert lib.qt_gw_polarization(h, 4097 // 2 + 1, 4, p, p, p, p, p, 1.0, p, p, p, f) == \
        _lib.QT_ERR_UNSUPPORTED
    assert lib.qt_gw_selfenergy(h, 4, 4, p, p, p, p, p, p, 1.0, p, p, p, 0) == \
        _lib.QT_ERR_UNSUPPORTED
    q = _ptr(torch.zeros_like(t))
    assert lib.qt_gw_screened(h, 2, 4, q, p, q, q, p, q, q, _lib.QT_PREC_FP64, f) == \
        _lib.QT_ERR_ARG
    assert lib.qt_gw_sigma_post(h, 0, 1, 1, p, p, p, f) == _lib.QT_ERR_ARG
    assert math.isfinite(float(t.abs().sum()))


def _two_rank_child(rank, world, port, q, precision):
    """One rank of a gloo group whose ranks share cuda:0: the sharded map and three SCBA
    iterations of the _system problem, computed by GpuStages through the C-ABI."""
    import os
    import torch
    import torch.distributed as dist
    from quantum_transport_gb300 import gw
    from quantum_transport_gb300.gw_shard import ShardedGw
    from quantum_transport_gb300.rgf import Context
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    torch.cuda.set_device(0)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    ctx = Context(0)
    try:
        dev = make_chain_device(6, 8, 64, -4.0, 4.0, seed=3)
        V = ogw.coulomb_blocks(8)
        g = ShardedGw.on_gpu(ctx, dev.H00[0], dev.H10, dev.E, dev.nx, V, world=world,
                             rank=rank, mu=(0.1, -0.1), precision=precision)
        SR0, SL0 = _physical_sigma(len(dev.E), dev.nx, 8)
        SR, SL = gw.to_dev(SR0[g.lo:g.hi]), gw.to_dev(SL0[g.lo:g.hi])
        N = [gw.from_dev(x) for x in g.step(SR, SL)]
        R, L, G, res = g.scba(alpha=0.3, tol=0.0, max_iter=3)
        out = (g.lo, g.hi, N, [gw.from_dev(x) for x in (R, L, G)], np.asarray(res))
    finally:
        ctx.close()
        dist.destroy_process_group()
    q.put((rank, out))


@pytest.mark.parametrize("precision", ["fp64", "mixed-fp64"])
def test_two_gloo_ranks_on_one_gpu_match_fused(ctx, precision):
    """Two ranks of a gloo group on cuda:0, each with its own library context: the
    fourteen all-to-alls of the map move the ranks' G, P, W and Sigma (through host memory
    for gloo), and the product's stage kernels compute on each share.  The map equals
    qt_gw_step bit for bit; three SCBA iterations equal qt_scba_solve's to round-off of the
    mixing."""
    import multiprocessing as mp
    import socket
    from quantum_transport_gb300 import gw
    dev, V, s = _system(ctx, precision)
    SR0, SL0 = _physical_sigma(len(dev.E), dev.nx, 8)
    fused = [gw.from_dev(x) for x in s.step(gw.to_dev(SR0), gw.to_dev(SL0))]
    R, L, G, res = s.scba(alpha=0.3, tol=0.0, max_iter=3)
    mixed = [gw.from_dev(x) for x in (R, L, G)]
    with socket.socket() as so:
        so.bind(("127.0.0.1", 0))
        port = so.getsockname()[1]
    spawn = mp.get_context("spawn")
    q = spawn.Queue()
    world = 2
    procs = [spawn.Process(target=_two_rank_child, args=(r, world, port, q, precision))
             for r in range(world)]
    for p in procs:
        p.start()
    out = dict(q.get(timeout=600) for _ in range(world))
    for p in procs:
        p.join(timeout=120)
        assert p.exitcode == 0
    assert [out[r][:2] for r in range(world)] == [(0, 32), (32, 64)]
    for c in range(3):
        got = np.concatenate([out[r][2][c] for r in range(world)])
        assert np.abs(fused[c]).max() > 0
        np.testing.assert_array_equal(got, fused[c])
        got = np.concatenate([out[r][3][c] for r in range(world)])
        np.testing.assert_allclose(got, mixed[c], rtol=0, atol=1e-12 * np.abs(mixed[c]).max())
    for r in range(world):
        np.testing.assert_allclose(out[r][4], res, rtol=1e-9)


def test_one_rank_kgrid_step_is_qt_gw_step(ctx):
    """A 1 x 2 k-point grid with the ndiag band: the staged map (k axis through the
    exchange, k-pair sums in the stage entry points) equals the fused one bit for bit."""
    from quantum_transport_gb300 import gw
    from quantum_transport_gb300.gw_shard import ShardedGw
    nk, nE, nx, nm = 2, 32, 6, 6
    dev = make_chain_device(nx, nm, nE, -4.0, 4.0, seed=11, nk=nk)
    V = np.stack([ogw.coulomb_blocks(nm) * (1.0 + 0.1 * q) for q in range(nk)])
    parts = [_physical_sigma(nE, nx, nm, seed=k) for k in range(nk)]
    SR = gw.to_dev(np.stack([p[0] for p in parts]))
    SL = gw.to_dev(np.stack([p[1] for p in parts]))
    s = gw.GwSystem(ctx, dev.H00, dev.H10, dev.E, nx, V, mu=(0.1, -0.1), kgrid=(1, nk),
                    ndiag=2)
    fused = s.step(SR, SL)
    g = ShardedGw.on_gpu(ctx, dev.H00, dev.H10, dev.E, nx, V, mu=(0.1, -0.1), kgrid=(1, nk),
                         ndiag=2)
    staged = g.step(SR, SL)
    for a, b in zip(staged, fused):
        b = b.cpu().numpy()
        assert b.shape[0] == nk and np.abs(b).max() > 0
        np.testing.assert_array_equal(a.cpu().numpy(), b)
