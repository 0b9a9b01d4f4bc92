"""The GW loop over energy shards on host ranks (gloo, world sizes 2 to 4): the energies <->
(i, j) all-to-all against the oracle's restatement of energies_to_ijs_2, its inverse, and the
sharded SCBA map (compute by the oracle) against the oracle's one-process SCBA."""
import math
import os
import socket

import numpy as np
import pytest

from oracle import gw as ogw

NM, NX, MU, TEMP = 3, 5, (0.2, -0.2), (300.0, 300.0)


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _spawn(target, world, *args):
    import multiprocessing as mp
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=target, args=(r, world, port, q) + args) for r in range(world)]
    for p in procs:
        p.start()
    out = dict(q.get(timeout=300) for _ in range(world))
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    return [out[r] for r in range(world)]


def _global_blocks(nE, nx, nm, seed):
    rng = np.random.default_rng(seed)
    return rng.normal(size=(nE, nx, nm * nm)) + 1j * rng.normal(size=(nE, nx, nm * nm))


# ---------------------------------------------------------------- the exchange
def _exchange_rank(rank, world, port, q, nE, nm):
    import torch
    import torch.distributed as dist
    from quantum_transport_gb300.shard import (energies_to_ijs, energy_range, ij_range,
                                               ijs_to_energies)
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    G = _global_blocks(nE, NX, nm, 5)
    lo, hi = energy_range(nE, world, rank)
    x = torch.from_numpy(np.ascontiguousarray(G[lo:hi]))
    y = energies_to_ijs(x, nE, world, rank)
    back = ijs_to_energies(y, nm * nm, world, rank)
    dist.destroy_process_group()
    q.put((rank, (y.numpy().copy(), back.numpy().copy(), ij_range(nm * nm, world, rank))))


@pytest.mark.parametrize("world", [2, 4])
def test_exchange_matches_reference_partition(world):
    """nm*nm and nE divisible by the rank count: the reference's own partition.  Rank r's
    result holds, for every energy, the elements energies_to_ijs_2 gives rank r."""
    nm, ne_loc = 4, 3
    nE = ne_loc * world
    res = _spawn(_exchange_rank, world, nE, nm)
    G = _global_blocks(nE, NX, nm, 5)
    # the local buffers in the reference's layout g(nm, nm, nx, local_ne, nk = 1): the same
    # memory order as the (nE_local, nx, nm*nm) C-order arrays here
    bufs = [np.ascontiguousarray(G[r * ne_loc:(r + 1) * ne_loc]).reshape(-1)
            for r in range(world)]
    ref = ogw.energies_to_ijs_2(bufs, nm, NX, 1, ne_loc)
    for r, (y, back, _) in enumerate(res):
        o = ref[r][:, :, 0]                       # [e, s, x, a]
        want = np.transpose(o, (1, 0, 2, 3)).reshape(nE, NX, -1)  # global energy s*ne + e
        np.testing.assert_array_equal(y, want)
        np.testing.assert_array_equal(back, G[r * ne_loc:(r + 1) * ne_loc])
    # the oracle's inverse brings the reference's buffers back
    for a, b in zip(ogw.ijs_to_energies_2(ref, nm, NX, 1, ne_loc), bufs):
        np.testing.assert_array_equal(a, b)


def test_exchange_uneven_shares():
    """nE = 7 and nm*nm = 9 over 2 ranks (4 + 3 energies, 5 + 4 elements): the remainders go
    to the first rank and the round trip is exact."""
    nE, nm, world = 7, 3, 2
    res = _spawn(_exchange_rank, world, nE, nm)
    G = _global_blocks(nE, NX, nm, 5)
    from quantum_transport_gb300.shard import energy_range
    for r, (y, back, (lo, hi)) in enumerate(res):
        np.testing.assert_array_equal(y, G[:, :, lo:hi])
        elo, ehi = energy_range(nE, world, r)
        np.testing.assert_array_equal(back, G[elo:ehi])


def test_single_rank_exchange_is_identity():
    import torch
    from quantum_transport_gb300.shard import energies_to_ijs, ijs_to_energies
    x = torch.from_numpy(_global_blocks(6, NX, 3, 1))
    assert energies_to_ijs(x, 6, 1, 0) is x
    assert ijs_to_energies(x, 9, 1, 0) is x
    with pytest.raises(ValueError):
        energies_to_ijs(x[:5], 6, 1, 0)


# ---------------------------------------------------------------- the sharded SCBA map
def _rm(T):
    """torch blocks stored column-major -> row-major numpy"""
    return np.ascontiguousarray(np.swapaxes(T.numpy(), -1, -2))


def _cm(A):
    import torch
    return torch.from_numpy(np.ascontiguousarray(np.swapaxes(A, -1, -2)))


class OracleStages:
    """The stage interface of gw_shard.GpuStages computed by the oracle on host tensors."""

    def __init__(self, E_local, H00, H10, nx, V):
        self.E, self.H00, self.H10, self.nx, self.V = E_local, H00, H10, nx, V

    def zeros(self, shape):
        import torch
        return torch.zeros(shape, dtype=torch.complex128)

    def green(self, SR, SL):
        G = ogw.green(self.E, self.H00, self.H10, self.nx, _rm(SR), _rm(SL), mu=MU, temp=TEMP)
        return tuple(_cm(A) for A in G)

    @staticmethod
    def _series(fn, scale, *pairs):
        import torch
        z = lambda t: 1j * np.moveaxis(t.numpy(), 0, -1).imag if t is not None else None
        acc = 0
        for X, Y, conj, zero_y in pairs:
            y = z(Y) if zero_y else np.moveaxis(Y.numpy(), 0, -1)
            acc = acc + fn(z(X), np.conj(y) if conj else y)
        return torch.from_numpy(np.ascontiguousarray(np.moveaxis(acc * scale, -1, 0)))

    def polarization(self, gr, gl, gg, glt, ggt, scale):
        s = -1j * scale
        return (self._series(ogw.corr, s, (gl, gr, True, True), (gr, glt, False, True)),
                self._series(ogw.corr, s, (gl, ggt, False, True)),
                self._series(ogw.corr, s, (gg, glt, False, True)))

    def screened(self, PR, PL, PG):
        return tuple(_cm(A) for A in ogw.screened(self.V, _rm(PR), _rm(PL), _rm(PG)))

    def self_energy(self, gr, gl, gg, wr, wl, wg, scale):
        s = 1j * scale
        return (self._series(ogw.conv, s, (gl, wr, False, False), (gr, wl, False, False),
                             (gr, wr, False, False)),
                self._series(ogw.conv, s, (gl, wl, False, False)),
                self._series(ogw.conv, s, (gg, wg, False, False)))

    def post(self, SR, SL, SG):
        import torch
        r, l, g = SR.numpy(), SL.numpy(), SG.numpy()
        r = r.real + 1j * (g - l).imag / 2
        sym = lambda A: (A + np.swapaxes(A, -1, -2)) / 2
        for T, A in ((SR, r), (SL, l), (SG, g)):
            T.copy_(torch.from_numpy(ogw.copy_edges(sym(A))))


def _problem(nE=12):
    rng = np.random.default_rng(21)
    H00 = rng.normal(size=(NM, NM)) * 0.3
    H00 = H00 + H00.T
    H10 = -1.0 * np.eye(NM) + 0.05 * rng.normal(size=(NM, NM))
    V = ogw.coulomb_blocks(NM)
    E = np.linspace(-2.5, 2.5, nE)
    return E, H00, H10, V


def _scba_rank(rank, world, port, q, nE, iters):
    import torch.distributed as dist
    from quantum_transport_gb300.gw_shard import ShardedGw
    from quantum_transport_gb300.shard import energy_range
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    E, H00, H10, V = _problem(nE)
    lo, hi = energy_range(nE, world, rank)
    g = ShardedGw(OracleStages(E[lo:hi], H00, H10, NX, V), nE, NX, NM, E[1] - E[0],
                  world=world, rank=rank)
    SR, SL, SG, res = g.scba(alpha=0.3, tol=0.0, max_iter=iters)
    dist.destroy_process_group()
    q.put((rank, (_rm(SR), _rm(SL), _rm(SG), res)))


def _check_against_oracle(parts, nE, iters):
    E, H00, H10, V = _problem(nE)
    SR, SL, SG, res = ogw.scba(E, H00, H10, V, NX, mu=MU, temp=TEMP, alpha=0.3, tol=0.0,
                               max_iter=iters)
    got = [np.concatenate([p[i] for p in parts]) for i in range(3)]
    for a, b in zip(got, (SR, SL, SG)):
        assert np.abs(b).max() > 0
        np.testing.assert_allclose(a, b, rtol=0, atol=1e-10 * np.abs(b).max())
    for p in parts:
        np.testing.assert_allclose(p[3], res, rtol=1e-9)


@pytest.mark.parametrize("world,nE", [(2, 12), (3, 13), (4, 13)])
def test_sharded_scba_matches_one_process(world, nE):
    """Three maps of the SCBA loop split over ranks agree with the oracle's one-process
    loop, self-energies and residuals. The shares are uneven: nm*nm = 9 elements split 5/4,
    3/3/3 and 3/2/2/2, and 13 energies split 5/4/4 and 4/3/3/3."""
    iters = 3
    parts = _spawn(_scba_rank, world, nE, iters)
    _check_against_oracle(parts, nE, iters)


def test_ranks_without_energies_still_exchange():
    """Three ranks over two energies: the third owns none and still takes part in every
    all-to-all; the maps agree with one process."""
    nE, iters, world = 2, 2, 3
    parts = _spawn(_scba_rank, world, nE, iters)
    assert parts[2][0].shape[0] == 0
    _check_against_oracle(parts, nE, iters)


def test_one_rank_scba_needs_no_process_group():
    from quantum_transport_gb300.gw_shard import ShardedGw
    nE, iters = 10, 2
    E, H00, H10, V = _problem(nE)
    g = ShardedGw(OracleStages(E, H00, H10, NX, V), nE, NX, NM, E[1] - E[0])
    SR, SL, SG, res = g.scba(tol=0.0, max_iter=iters)
    _check_against_oracle([(_rm(SR), _rm(SL), _rm(SG), res)], nE, iters)


def test_scale_factors_follow_the_reference():
    """P takes dE/(2 pi) spindeg/nk and Sigma dE/(2 pi)/nk (src/gw_mod.f90:516, 694)."""
    from quantum_transport_gb300.gw_shard import ShardedGw
    seen = {}

    class Probe(OracleStages):
        def polarization(self, gr, gl, gg, glt, ggt, scale):
            seen["P"] = scale
            return super().polarization(gr, gl, gg, glt, ggt, scale)

        def self_energy(self, gr, gl, gg, wr, wl, wg, scale):
            seen["S"] = scale
            return super().self_energy(gr, gl, gg, wr, wl, wg, scale)

    E, H00, H10, V = _problem(8)
    g = ShardedGw(Probe(E, H00, H10, NX, V), 8, NX, NM, E[1] - E[0], spindeg=2.0)
    g.step(g.zeros(), g.zeros())
    dE = E[1] - E[0]
    assert seen["P"] == dE / (2 * math.pi) * 2.0 and seen["S"] == dE / (2 * math.pi)
