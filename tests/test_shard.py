"""Point sharding over ranks (gloo on CPU, world size 2): disjoint energy blocks,
no exchange until the final gather, result identical to one process."""
import os
import socket

import numpy as np
import pytest

from quantum_transport_gb300.shard import energy_range


@pytest.mark.parametrize("nE,world", [(10, 2), (11, 3), (4096, 8), (3, 4)])
def test_energy_ranges_partition_the_grid(nE, world):
    seen = []
    for r in range(world):
        lo, hi = energy_range(nE, world, r)
        seen.extend(range(lo, hi))
    assert seen == list(range(nE))


def test_reference_split_drops_the_remainder():
    # src/main.f90:100-101: local_NE = nen / comm_size, first = local_NE * rank + 1
    assert [energy_range(11, 3, r, drop_remainder=True) for r in range(3)] == \
        [(0, 3), (3, 6), (6, 9)]


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, world, port, nE, q):
    import torch.distributed as dist
    from oracle import cref
    from quantum_transport_gb300.devices import make_chain_device
    from quantum_transport_gb300.shard import energy_range, gather_points, max_over_ranks
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    dev = make_chain_device(4, 8, nE, -2.0, 2.0, seed=11, nk=2)
    lo, hi = energy_range(nE, world, rank)
    r = cref.rgf(dev.H00, dev.H10, dev.E[lo:hi], dev.nx, mul=0.1, mur=-0.1, sancho_tol=1e-10,
                 threads=1)
    T = gather_points(r["T"].reshape(hi - lo, -1), nE, world, rank)
    t = max_over_ranks(float(rank + 1))
    dist.destroy_process_group()
    q.put((rank, T, t))


def test_two_rank_solve_matches_one_process():
    import multiprocessing as mp
    from oracle import cref
    from quantum_transport_gb300.devices import make_chain_device
    cref.build()
    nE, world = 9, 2
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank, args=(r, world, port, nE, q)) for r in range(world)]
    for p in procs:
        p.start()
    got = [q.get(timeout=300) for _ in range(world)]
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    dev = make_chain_device(4, 8, nE, -2.0, 2.0, seed=11, nk=2)
    ref = cref.rgf(dev.H00, dev.H10, dev.E, dev.nx, mul=0.1, mur=-0.1, sancho_tol=1e-10,
                   threads=1)["T"].reshape(nE, -1)
    for rank, T, t in got:
        np.testing.assert_array_equal(T, ref)   # same arithmetic per point: bit-identical
        assert t == float(world)                # max over ranks


def _photon_data(nE=13, nx=2, nm=3, seed=4):
    rng = np.random.default_rng(seed)
    shape = (nE, nx, nm, nm)
    GL = rng.normal(size=shape) + 1j * rng.normal(size=shape)
    GG = rng.normal(size=shape) + 1j * rng.normal(size=shape)
    M = rng.normal(size=(nx, nm, nm)) + 1j * rng.normal(size=(nx, nm, nm))
    return M, GL, GG


def _halo_rank(rank, world, port, nop, q):
    import torch.distributed as dist
    from oracle import gw as ogw
    from quantum_transport_gb300.shard import energy_halo, energy_range
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    M, GL, GG = _photon_data()
    lo, hi = energy_range(GL.shape[0], world, rank)
    xl = energy_halo(GL[lo:hi], nop, world, rank)
    xg = energy_halo(GG[lo:hi], nop, world, rank)
    S = ogw.ephoton_sigma(M, xl, xg, nop, 1.0, 2.0, 0.5, halo=True)
    dist.destroy_process_group()
    q.put((rank, lo, hi, xl, S))


@pytest.mark.parametrize("world", [2, 3])
def test_energy_halo_feeds_the_photon_self_energy(world):
    """Each energy shard receives nop energies from its neighbours (zeros beyond the grid);
    the e-photon self-energy of every shard then equals the one-process result."""
    import multiprocessing as mp
    from oracle import gw as ogw
    nop = 2
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_halo_rank, args=(r, world, port, nop, q)) for r in range(world)]
    for p in procs:
        p.start()
    got = [q.get(timeout=300) for _ in range(world)]
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    M, GL, GG = _photon_data()
    full = ogw.ephoton_sigma(M, GL, GG, nop, 1.0, 2.0, 0.5)
    padded = np.zeros((GL.shape[0] + 2 * nop,) + GL.shape[1:], dtype=GL.dtype)
    padded[nop:nop + GL.shape[0]] = GL
    for rank, lo, hi, xl, S in got:
        np.testing.assert_array_equal(xl, padded[lo:hi + 2 * nop])
        for a, b in zip(S, full):
            np.testing.assert_array_equal(a, b[lo:hi])


def test_energy_halo_single_rank_pads_with_zeros():
    from quantum_transport_gb300.shard import energy_halo
    x = np.arange(5.0)
    np.testing.assert_array_equal(energy_halo(x, 2, 1, 0), [0, 0, 0, 1, 2, 3, 4, 0, 0])
