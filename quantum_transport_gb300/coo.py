"""Device Hamiltonian blocks from a COO matrix file, built on the GPU.

Mirrors the reference's COO input path: ``load_COOmatrix``
(src/deviceHam_mod.f90:40-91) reads "i j re [im]" rows, and the blocksize
branch of ``devH_build_fromCOOfile`` (src/deviceHam_mod.f90:168-224) scatters
them into Hii (Hermitian-filled), H1i and Sii.  ``main`` takes this path for
any ``calc_type`` other than 'w90' (src/main.f90:112-114) with
``use0index=.true., iscomplex=.false., blocksize=nb``.  The scatter runs as one
GPU call (``qt_coo_blocks``); its result does not depend on thread order.
"""
from __future__ import annotations

import ctypes as C
import dataclasses

import numpy as np

from ._lib import check


@dataclasses.dataclass
class CooMatrix:
    """COO entries with 0-based ``row``/``col`` (int32) and complex128 ``h``.
    ``norb`` is the largest index as written in the file: the reference's
    ``nm = max(i, j)`` (src/deviceHam_mod.f90:58-62,73), taken before any
    0-based shift."""
    row: np.ndarray
    col: np.ndarray
    h: np.ndarray
    norb: int

    def slabs(self, bs):
        """Slab count of the reference, ``nx = norb / blocksize`` (src/deviceHam_mod.f90:169-170).
        For a 0-based file whose orbital count is a multiple of ``bs`` this drops the
        last slab, as the reference does."""
        return self.norb // bs


def load(path, use0index=False, iscomplex=False):
    """Read a COO file: one entry "i j re" (or "i j re im" with ``iscomplex``) per line,
    1-based unless ``use0index``."""
    a = np.loadtxt(path, ndmin=2, usecols=(0, 1, 2, 3) if iscomplex else (0, 1, 2))
    if a.size == 0:
        z = np.zeros(0, dtype=np.int32)
        return CooMatrix(z, z.copy(), np.zeros(0, dtype=np.complex128), 0)
    i = a[:, 0].astype(np.int64)
    j = a[:, 1].astype(np.int64)
    h = a[:, 2] + 1j * a[:, 3] if iscomplex else a[:, 2].astype(np.complex128)
    base = 0 if use0index else 1
    norb = int(max(i.max(), j.max()))
    return CooMatrix((i - base).astype(np.int32), (j - base).astype(np.int32),
                     np.ascontiguousarray(h, dtype=np.complex128), norb)


def device_blocks(ctx, m, bs, nx=None, s=None):
    """(Hii, H1i, Sii) as (nx, bs, bs), (nx+1, bs, bs), (nx, bs, bs) complex128 arrays in
    numpy [row, col] indexing, built on the GPU.  ``nx`` defaults to ``m.slabs(bs)``;
    ``s`` holds overlap values on the same entries as ``m.h`` (None: Sii = I)."""
    nx = m.slabs(bs) if nx is None else int(nx)
    if nx <= 0:
        raise ValueError("no complete slab of %d orbitals" % bs)
    row = np.ascontiguousarray(m.row, dtype=np.int32)
    col = np.ascontiguousarray(m.col, dtype=np.int32)
    h = np.ascontiguousarray(m.h, dtype=np.complex128)
    sv = None if s is None else np.ascontiguousarray(s, dtype=np.complex128)
    if sv is not None and sv.shape != h.shape:
        raise ValueError("overlap values must sit on the Hamiltonian's entries")
    Hii = np.empty((nx, bs, bs), dtype=np.complex128)
    H1i = np.empty((nx + 1, bs, bs), dtype=np.complex128)
    Sii = np.empty_like(Hii)
    p = lambda a: None if a is None else a.ctypes.data_as(C.c_void_p)
    check(ctx._lib.qt_coo_blocks(ctx.handle, nx, bs, len(h), p(row), p(col), 0, p(h), p(sv),
                                 p(Hii), p(H1i), p(Sii), 0))
    # the library writes column-major blocks
    return (np.swapaxes(Hii, -1, -2), np.swapaxes(H1i, -1, -2), np.swapaxes(Sii, -1, -2))
