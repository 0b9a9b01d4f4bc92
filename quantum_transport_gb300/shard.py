"""Sharding the (E, k) points over ranks: one process per GPU.

Every (E, k) point of the RGF sweep is independent.  As in the reference, each
rank takes a contiguous block of the energy grid (src/main.f90:100-101,
src/negf_mod.f90:100-103).  It solves all k-points of its energies and
exchanges nothing until the final gather of the per-point results.  The
reference gives every rank nen / comm_size energies and drops the remaining
nen mod comm_size; ``energy_range`` spreads them over the first ranks instead,
and reproduces the reference's split with ``drop_remainder=True``.  The RGF path
has no data-path collective.  The GW self-energy loop has two exchange steps:
``energy_halo``, for the e-photon self-energy, which needs nop energies from each
neighbouring shard, and the all-to-all transposes ``energies_to_ijs`` /
``ijs_to_energies`` around the energy correlations and convolutions.
"""
from __future__ import annotations

import numpy as np


def energy_range(nE, world, rank, drop_remainder=False):
    """[lo, hi) of the energies of ``rank`` among ``world`` ranks."""
    if world <= 0 or not 0 <= rank < world:
        raise ValueError("need 0 <= rank < world")
    base, extra = divmod(nE, world)
    if drop_remainder:
        return base * rank, base * (rank + 1)
    lo = base * rank + min(rank, extra)
    return lo, lo + base + (1 if rank < extra else 0)


def gather_points(local, nE, world, rank, group=None):
    """All ranks' per-energy results, concatenated in energy order.

    ``local``: numpy array whose first axis is this rank's energies; returns the
    (nE, ...) array on every rank.  Uses torch.distributed.all_gather: gloo for
    host ranks, NCCL for GPU ranks (CPU tensors are moved to the rank's device).
    """
    import torch
    import torch.distributed as dist
    if world == 1:
        return np.asarray(local)
    local = np.ascontiguousarray(local)
    counts = [energy_range(nE, world, r)[1] - energy_range(nE, world, r)[0] for r in range(world)]
    if local.shape[0] != counts[rank]:
        raise ValueError("local block does not match energy_range")
    cuda = dist.get_backend(group) == "nccl"
    dev = torch.device("cuda", torch.cuda.current_device()) if cuda else torch.device("cpu")
    width = max(counts)
    buf = np.zeros((width,) + local.shape[1:], dtype=local.dtype)
    buf[:local.shape[0]] = local
    t = torch.from_numpy(buf).to(dev)
    outs = [torch.empty_like(t) for _ in range(world)]
    dist.all_gather(outs, t, group=group)
    return np.concatenate([o.cpu().numpy()[:c] for o, c in zip(outs, counts)])


def max_over_ranks(x, group=None):
    """The maximum of a host scalar over all ranks (e.g. the slowest rank's time)."""
    import torch
    import torch.distributed as dist
    if not dist.is_initialized() or dist.get_world_size(group) == 1:
        return float(x)
    cuda = dist.get_backend(group) == "nccl"
    t = torch.tensor([float(x)], dtype=torch.float64,
                     device=torch.device("cuda", torch.cuda.current_device()) if cuda else "cpu")
    dist.all_reduce(t, op=dist.ReduceOp.MAX, group=group)
    return float(t.item())


def energy_halo(local, nop, world, rank, group=None):
    """This rank's energies with ``nop`` energies of each neighbouring shard around them.

    The e-photon self-energy at energy E needs G(E -+ hw), nop = floor(hw / dE) grid
    steps away, so each rank receives the last ``nop`` energies of rank - 1 and the first
    ``nop`` of rank + 1, and zeros beyond the global grid (src/gw_mod.f90:845-863, with the
    buffer layout of :226-239).  Returns an array of nE_local + 2 nop energies, numpy or
    torch like ``local``.  Point-to-point sends and receives only; gloo for host tensors,
    NCCL for device tensors.
    """
    import torch
    import torch.distributed as dist
    is_np = isinstance(local, np.ndarray)
    t = torch.from_numpy(np.ascontiguousarray(local)) if is_np else local.contiguous()
    n = t.shape[0]
    if nop < 0 or nop > n:
        raise ValueError("need 0 <= nop <= local energies")
    ext = torch.zeros((n + 2 * nop,) + tuple(t.shape[1:]), dtype=t.dtype, device=t.device)
    ext[nop:nop + n] = t
    if world > 1 and nop > 0:
        real = (lambda x: torch.view_as_real(x)) if t.is_complex() else (lambda x: x)
        if dist.get_backend(group) == "nccl" and t.device.type != "cuda":
            raise ValueError("NCCL halo exchange needs device tensors")
        reqs, keep = [], []
        if rank > 0:
            send = t[:nop].contiguous()
            keep.append(send)
            reqs.append(dist.isend(real(send), rank - 1, group=group, tag=0))
            reqs.append(dist.irecv(real(ext[:nop]), rank - 1, group=group, tag=1))
        if rank < world - 1:
            send = t[n - nop:].contiguous()
            keep.append(send)
            reqs.append(dist.isend(real(send), rank + 1, group=group, tag=1))
            reqs.append(dist.irecv(real(ext[nop + n:]), rank + 1, group=group, tag=0))
        for r in reqs:
            r.wait()
    return ext.numpy() if is_np else ext


def ij_range(nij, world, rank):
    """[lo, hi) of the block elements (i, j) that ``rank`` owns in the GW convolutions.

    The reference gives every rank local_Nij = nm*nm / comm_size consecutive elements of the
    column-major block, rank r from r * local_Nij (src/gw_mod.f90:171-172); a remainder of
    nm*nm mod comm_size goes to the first ranks here, one each."""
    return energy_range(nij, world, rank)


def _all_to_all(send, out_counts, in_counts, group):
    """One all_to_all_single; over gloo, device tensors go through host memory (ranks on
    GPUs of one host without NCCL, or several ranks on one GPU)."""
    import torch
    import torch.distributed as dist
    backend = dist.get_backend(group)
    if backend == "nccl" and send.device.type != "cuda":
        raise ValueError("NCCL all-to-all needs device tensors")
    dev = send.device
    if backend == "gloo" and dev.type == "cuda":
        send = send.cpu()
    recv = torch.empty(sum(out_counts), dtype=send.dtype, device=send.device)
    real = torch.view_as_real if send.is_complex() else (lambda t: t)
    dist.all_to_all_single(real(recv), real(send.contiguous()), out_counts, in_counts,
                           group=group)
    return recv.to(dev)


def energies_to_ijs(x, nE, world, rank, group=None):
    """Energy shards to element shards: energies_to_ijs_2 (src/gw_mod.f90:41-73).

    ``x``: this rank's energies of a block quantity, a torch tensor (nE_local, nx, nij) with
    nij = nm*nm elements in column-major order and nE_local from ``energy_range``.  Returns
    (nE, nx, nij_local): every energy of the elements ``ij_range`` gives this rank, the
    series layout of the energy correlations.  One all-to-all with the reference's
    partition (each rank sends element range r of its energies to rank r and receives its
    element range of every rank's energies); gloo for host tensors, NCCL for device
    tensors.  The reference keeps the energy series contiguous per element
    ((NE, nk, nx, local_Nij) in Fortran order); here they are interleaved across elements
    (energy slowest), which the correlation kernel reads coalesced.
    """
    import torch
    ne_loc, nx, nij = x.shape
    counts = [energy_range(nE, world, r) for r in range(world)]
    if ne_loc != counts[rank][1] - counts[rank][0]:
        raise ValueError("local energies do not match energy_range")
    if world == 1:
        return x
    ijr = [ij_range(nij, world, r) for r in range(world)]
    c = ijr[rank][1] - ijr[rank][0]
    send = torch.cat([x[:, :, lo:hi].reshape(-1) for lo, hi in ijr])
    recv = _all_to_all(send, [(hi - lo) * nx * c for lo, hi in counts],
                       [ne_loc * nx * (hi - lo) for lo, hi in ijr], group)
    return recv.view(nE, nx, c)


def ijs_to_energies(y, nij, world, rank, group=None):
    """Element shards back to energy shards, the inverse of ``energies_to_ijs`` (the
    reference calls it ijs_to_energies_2, src/gw_mod.f90:522-524, 700-702; its source is
    absent).  ``y``: (nE, nx, nij_local) on this rank; returns (nE_local, nx, nij)."""
    import torch
    nE, nx, c = y.shape
    ijr = [ij_range(nij, world, r) for r in range(world)]
    if c != ijr[rank][1] - ijr[rank][0]:
        raise ValueError("local elements do not match ij_range")
    if world == 1:
        return y
    counts = [energy_range(nE, world, r) for r in range(world)]
    ne_loc = counts[rank][1] - counts[rank][0]
    recv = _all_to_all(y.reshape(-1), [ne_loc * nx * (hi - lo) for lo, hi in ijr],
                       [(hi - lo) * nx * c for lo, hi in counts], group)
    parts = recv.split([ne_loc * nx * (hi - lo) for lo, hi in ijr])
    return torch.cat([p.view(ne_loc, nx, hi - lo) for p, (lo, hi) in zip(parts, ijr)], dim=2)
