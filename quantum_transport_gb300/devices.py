"""Seeded synthetic block-tridiagonal devices (the benchmark workloads).

These generate the Hamiltonians the reference's driver would receive from
``devH_build_fromWannierFile`` (src/deviceHam_mod.f90:234-290): on-site blocks
``Hii`` per slab and couplings ``H1i`` (H1i[l] = H_{l,l-1}, with H1i[0] the
left-lead coupling and H1i[nx] the right-lead coupling), identical in every
slab and in both semi-infinite leads, ``S = I``.

Statistics (all energies in eV):
* on-site block H_ii: Hermitian, diagonal ~ U[-1, 1], off-diagonal complex
  entries with standard deviation ``offdiag`` (real and imaginary parts each
  N(0, offdiag/sqrt 2)), symmetrised as U + U^+ from the strict upper triangle;
* coupling H_{i,i+1} = -2.7 I + N(0, 0.05) + i N(0, 0.05), so that
  H1i[l] = H_{l,l-1} = (H_{l-1,l})^+;
* optional transverse dispersion H_ii(k) = H_ii + H_y e^{ik} + H_y^+ e^{-ik}
  with H_y drawn like the off-diagonal part of H_ii, k_j = -pi + 2 pi j / nk.
"""
from __future__ import annotations

import dataclasses

import numpy as np


@dataclasses.dataclass
class ChainDevice:
    """A device of ``nx`` identical slabs of ``nm`` orbitals, at ``nk`` k-points.

    ``H00[k]`` (nk, nm, nm) on-site block at k, ``H10`` (nm, nm) the coupling
    H_{l,l-1}; energies ``E`` (nE,).  Arrays are complex128, row-major numpy
    (the C-ABI converts to the column-major layout of the reference).
    """
    nx: int
    nm: int
    H00: np.ndarray
    H10: np.ndarray
    E: np.ndarray
    kpts: np.ndarray

    @property
    def nk(self):
        return self.H00.shape[0]

    @property
    def npoints(self):
        return self.E.shape[0] * self.nk


def _hermitian_offdiag(rng, n, sigma):
    s = sigma / np.sqrt(2.0)
    X = rng.normal(0.0, s, (n, n)) + 1j * rng.normal(0.0, s, (n, n))
    U = np.triu(X, 1)
    return U + U.conj().T


def make_chain_device(nx, nm, nE, emin, emax, seed, nk=1, offdiag=0.1,
                      coupling=-2.7, coupling_noise=0.05):
    rng = np.random.default_rng(seed)
    H0 = _hermitian_offdiag(rng, nm, offdiag) + np.diag(rng.uniform(-1.0, 1.0, nm))
    T = coupling * np.eye(nm) + rng.normal(0.0, coupling_noise, (nm, nm)) \
        + 1j * rng.normal(0.0, coupling_noise, (nm, nm))  # H_{i,i+1}
    H10 = T.conj().T                                      # H_{i+1,i}
    if nk > 1:
        Hy = rng.normal(0.0, offdiag / np.sqrt(2.0), (nm, nm)) \
            + 1j * rng.normal(0.0, offdiag / np.sqrt(2.0), (nm, nm))
        kpts = -np.pi + 2.0 * np.pi * np.arange(nk) / nk
        H00 = np.stack([H0 + Hy * np.exp(1j * k) + Hy.conj().T * np.exp(-1j * k) for k in kpts])
    else:
        kpts = np.zeros(1)
        H00 = H0[None].copy()
    E = np.linspace(emin, emax, nE) if nE > 1 else np.array([emin], dtype=np.float64)
    return ChainDevice(nx=nx, nm=nm, H00=H00.astype(np.complex128),
                       H10=H10.astype(np.complex128), E=E, kpts=kpts)


def config_ballistic_small(seed=1234):
    """64 slabs x 32 orbitals, 512 energies on [-3, 3] eV, one k."""
    return make_chain_device(64, 32, 512, -3.0, 3.0, seed)


def config_batched(seed=2024, nE=4096, nk=16, nx=100, nm=128):
    """100 slabs x 128 orbitals, 4096 energies on [-2, 2] eV x 16 k in [-pi, pi)."""
    return make_chain_device(nx, nm, nE, -2.0, 2.0, seed, nk=nk)


@dataclasses.dataclass
class GwDevice:
    """A GW/SCBA problem: per-slab on-site blocks ``H00`` (nx, nm, nm), coupling
    ``H10``, energies ``E`` and the Coulomb block ``V`` (nm, nm)."""
    H00: np.ndarray
    H10: np.ndarray
    E: np.ndarray
    V: np.ndarray

    @property
    def nx(self):
        return self.H00.shape[0]

    @property
    def nm(self):
        return self.H00.shape[-1]


def coulomb_block(nm, spacing_nm=0.25, strength=14.4):
    """V_ij = 14.4 / (|r_i - r_j| + 1) eV, orbitals on a 1-D grid of 0.25 nm."""
    r = np.arange(nm) * spacing_nm
    return strength / (np.abs(r[:, None] - r[None, :]) + 1.0)


def disordered_gw_device(seed, nx=6, nm=8, nE=64, emin=-4.0, emax=4.0, sigma=None,
                         base_seed=3):
    """One disorder realisation of the GW device family: the seeded chain of
    ``make_chain_device(seed=base_seed)`` plus on-site disorder N(0, sigma) on
    every orbital of every slab, sigma ~ U[0.05, 0.3] eV drawn from ``seed``
    unless given."""
    base = make_chain_device(nx, nm, nE, emin, emax, seed=base_seed)
    rng = np.random.default_rng(seed)
    s = rng.uniform(0.05, 0.3) if sigma is None else sigma
    H = np.repeat(base.H00[:1], nx, axis=0).copy()
    H[:, np.arange(nm), np.arange(nm)] += rng.normal(0.0, s, (nx, nm))
    return GwDevice(H00=H, H10=base.H10, E=base.E, V=coulomb_block(nm))


@dataclasses.dataclass
class UnevenDevice:
    """A device sliced from an atomistic graph: slabs of different sizes.

    ``Hii[l]`` (nk, n_l, n_l) and ``H1i[l]`` = H_{l,l-1} (nk, n_l, n_{l-1}) for
    1 <= l < nx; ``H1i[0]`` (nk, n_0, n_0) and ``H1i[nx]`` (nk, n_N, n_N) the leads'
    couplings.  ``layer`` gives each atom's slab, ``order`` the atoms in orbital order."""
    Hii: list
    H1i: list
    E: np.ndarray
    kpts: np.ndarray
    layer: np.ndarray
    order: np.ndarray

    @property
    def nx(self):
        return len(self.Hii)

    @property
    def sizes(self):
        return [h.shape[-1] for h in self.Hii]


def bfs_layers(nat, bonds, edge):
    """Graph distance of every atom from the ``edge`` atoms: slice_1contact's slicing
    (src/graph_partition.f90:282-316, 426-450), slice number = distance."""
    nbr = [[] for _ in range(nat)]
    for i, j in bonds:
        nbr[i].append(j)
        nbr[j].append(i)
    D = np.full(nat, -1, dtype=np.int64)
    D[edge] = 0
    front = list(edge)
    while front:
        nxt = []
        for a in front:
            for b in nbr[a]:
                if D[b] < 0:
                    D[b] = D[a] + 1
                    nxt.append(b)
        front = nxt
    if (D < 0).any():
        raise ValueError("graph is not connected to the edge")
    return D


def config_uneven(seed=4000, natoms=4000, box=(60.0, 6.0, 6.0), cutoff=2.6, nE=2048,
                  emin=-2.0, emax=2.0, nk=8, t_lead=-2.7):
    """Random 3-D tight-binding graph sliced into blocks of different sizes.

    ``natoms`` atoms uniform in ``box`` (Angstrom), bonds below ``cutoff`` with hopping
    t(d) = -2.7 exp(-3 (d / 1.42 - 1)) eV, on-site energies N(0, 0.2) eV, one orbital per
    atom.  The box is periodic along y, and a bond that crosses the y boundary w times
    carries the Bloch phase exp(i k w), k_j = -pi + 2 pi j / nk.  Slabs are the BFS
    layers from the atoms within ``cutoff`` of x = 0, so every bond joins the same or
    neighbouring slabs; a last layer of a few stragglers is merged into the one before.
    Each lead repeats its end slab, consecutive copies coupled by t_lead I."""
    rng = np.random.default_rng(seed)
    L = np.asarray(box, dtype=np.float64)
    pos = rng.uniform(0.0, 1.0, (natoms, 3)) * L
    onsite = rng.normal(0.0, 0.2, natoms)
    bi, bj, bd, bw = [], [], [], []
    for i0 in range(0, natoms, 512):
        d = pos[None, :, :] - pos[i0:i0 + 512, None, :]  # r_j - r_i
        w = -np.round(d[..., 1] / L[1])                  # image of j nearest to i
        d[..., 1] += w * L[1]
        r = np.sqrt((d * d).sum(axis=-1))
        ii, jj = np.nonzero(r < cutoff)
        keep = jj > ii + i0
        bi.append(ii[keep] + i0)
        bj.append(jj[keep])
        bd.append(r[ii[keep], jj[keep]])
        bw.append(w[ii[keep], jj[keep]])
    bi, bj, bd, bw = (np.concatenate(x) for x in (bi, bj, bd, bw))
    t = -2.7 * np.exp(-3.0 * (bd / 1.42 - 1.0))
    layer = bfs_layers(natoms, zip(bi, bj), np.nonzero(pos[:, 0] < cutoff)[0])
    # a last layer of a few stragglers joins its neighbour (layers two apart share no bond)
    counts = np.bincount(layer)
    if len(counts) > 2 and counts[-1] < counts.mean() / 4:
        layer[layer == len(counts) - 1] = len(counts) - 2
    nx = int(layer.max()) + 1
    order = np.lexsort((np.arange(natoms), layer))
    local = np.empty(natoms, dtype=np.int64)
    sizes = np.bincount(layer, minlength=nx)
    start = np.concatenate([[0], np.cumsum(sizes)])
    local[order] = np.arange(natoms) - start[layer[order]]
    kpts = -np.pi + 2.0 * np.pi * np.arange(nk) / nk
    ph = np.exp(1j * np.outer(kpts, bw))  # (nk, nbonds): H_ij = t e^{i k w}
    Hii = [np.zeros((nk, n, n), dtype=np.complex128) for n in sizes]
    H1i = [None] + [np.zeros((nk, sizes[l], sizes[l - 1]), dtype=np.complex128)
                    for l in range(1, nx)] + [None]
    for l in range(nx):
        a = order[start[l]:start[l + 1]]
        Hii[l][:, np.arange(sizes[l]), np.arange(sizes[l])] = onsite[a]
    li, lj = layer[bi], layer[bj]
    for l in range(nx):
        m = (li == l) & (lj == l)
        r, c = local[bi[m]], local[bj[m]]
        np.add.at(Hii[l], (slice(None), r, c), t[m] * ph[:, m])
        np.add.at(Hii[l], (slice(None), c, r), np.conj(t[m] * ph[:, m]))
    for l in range(1, nx):
        # bonds between slab l (rows) and l-1 (columns): H_{ij} for i in l, j in l-1
        m1 = (li == l) & (lj == l - 1)   # i in l, j in l-1: H_ij = t e^{ikw}
        m2 = (li == l - 1) & (lj == l)   # i in l-1, j in l: H_ji = conj(t e^{ikw})
        np.add.at(H1i[l], (slice(None), local[bi[m1]], local[bj[m1]]), t[m1] * ph[:, m1])
        np.add.at(H1i[l], (slice(None), local[bj[m2]], local[bi[m2]]), np.conj(t[m2] * ph[:, m2]))
        if ((np.abs(li - lj) > 1)).any():
            raise AssertionError("BFS layers must be block-tridiagonal")
    H1i[0] = np.broadcast_to(t_lead * np.eye(sizes[0]), (nk, sizes[0], sizes[0])).copy()
    H1i[nx] = np.broadcast_to(t_lead * np.eye(sizes[-1]), (nk, sizes[-1], sizes[-1])).copy()
    E = np.linspace(emin, emax, nE)
    return UnevenDevice(Hii=Hii, H1i=H1i, E=E, kpts=kpts, layer=layer, order=order)
