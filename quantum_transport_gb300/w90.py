"""Device Hamiltonians from a Wannier90 tight-binding model, built on the GPU.

Mirrors the reference's input side for the RGF path: ``w90_load_from_file``
(src/wannierHam3d.f90:72-152) reads the model, and ``w90_MAT_DEF``
(src/wannierHam3d.f90:273-301) turns it into the on-site block H_ii and the
coupling H_{i+1,i} of a slab of ``ns`` cells at transverse momentum (ky, kz).
Here the blocks of all k-points are built in one launch (``qt_w90_blocks``),
ready for ``rgf_solve`` with per-k on-site blocks.
"""
from __future__ import annotations

import ctypes as C
import dataclasses

import numpy as np

from ._lib import check


@dataclasses.dataclass
class W90Model:
    """H(R) of a Wannier90 model: ``Hr`` (nb, nb, nxr, nyr, nzr) complex128 for
    R in ``ranges`` = (xmin, xmax, ymin, ymax, zmin, zmax), cell vectors alpha,
    beta, gamm (Angstrom)."""
    Hr: np.ndarray
    ranges: tuple
    alpha: np.ndarray
    beta: np.ndarray
    gamm: np.ndarray

    @property
    def nb(self):
        return self.Hr.shape[0]

    @property
    def axes(self):
        """Transport and transverse unit vectors (xhat, yhat, zhat), src/wannierHam3d.f90:130-135."""
        xhat = self.alpha / np.linalg.norm(self.alpha)
        yhat = -np.cross(xhat, self.gamm)
        yhat = yhat / np.linalg.norm(yhat)
        return xhat, yhat, self.gamm / np.linalg.norm(self.gamm)

    @property
    def Lx(self):
        """Cell length along transport (Angstrom)."""
        return abs(float(np.dot(self.alpha, self.axes[0])))

    def kvec(self, kx, ky, kz):
        """Cartesian k vectors kx xhat + ky yhat + kz zhat for arrays of (kx, ky, kz)."""
        xhat, yhat, zhat = self.axes
        kx, ky, kz = (np.atleast_1d(np.asarray(v, dtype=np.float64)) for v in (kx, ky, kz))
        return kx[:, None] * xhat + ky[:, None] * yhat + kz[:, None] * zhat


def load(path):
    """Read a Wannier90-style model file: a header line (bands, spin degeneracy), 'cell'
    and three cell vectors, 'hamiltonian', the entry count, then rows
    Rx Ry Rz m n Re Im with 1-based orbital indices (src/wannierHam3d.f90:72-152)."""
    with open(path) as f:
        lines = [l for l in f.read().split("\n")]
    pos = 2
    cell = np.array([[float(x) for x in lines[pos + i].split()[:3]] for i in range(3)])
    pos += 4
    count = int(lines[pos].split()[0])
    rows = np.array([[float(x) for x in lines[pos + 1 + i].split()[:7]] for i in range(count)])
    R = np.floor(rows[:, :3]).astype(int)
    mn = np.floor(rows[:, 3:5]).astype(int) - 1
    lo, hi = R.min(axis=0), R.max(axis=0)
    nb = int(mn.max()) + 1
    Hr = np.zeros((nb, nb) + tuple(hi - lo + 1), dtype=np.complex128)
    Hr[mn[:, 0], mn[:, 1], R[:, 0] - lo[0], R[:, 1] - lo[1], R[:, 2] - lo[2]] = \
        rows[:, 5] + 1j * rows[:, 6]
    ranges = (lo[0], hi[0], lo[1], hi[1], lo[2], hi[2])
    return W90Model(Hr, tuple(int(x) for x in ranges), cell[0], cell[1], cell[2])


def slab_blocks(ctx, model, ns, kx=0.0, ky=0.0, kz=0.0):
    """(H00, H10) of a slab of ``ns`` cells at every k: arrays (nk, nm, nm), nm = nb*ns,
    row-major (numpy indexing), built on the GPU."""
    kv = np.ascontiguousarray(model.kvec(kx, ky, kz))
    nk, nm = kv.shape[0], model.nb * ns
    Hr = np.asfortranarray(model.Hr)  # Fortran Hr(nb, nb, nxr, nyr, nzr)
    rng = np.ascontiguousarray(model.ranges, dtype=np.int32)
    cell = np.ascontiguousarray(np.stack([model.alpha, model.beta, model.gamm]), dtype=np.float64)
    H00 = np.zeros((nk, nm, nm), dtype=np.complex128)
    H10 = np.zeros_like(H00)
    p = lambda a: a.ctypes.data_as(C.c_void_p)
    check(ctx._lib.qt_w90_blocks(ctx.handle, model.nb, ns, p(rng), p(Hr), p(cell), nk, p(kv),
                                 p(H00), p(H10), 0))
    # the library writes column-major blocks
    return np.swapaxes(H00, -1, -2), np.swapaxes(H10, -1, -2)
