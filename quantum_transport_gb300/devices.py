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
