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
