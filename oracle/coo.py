"""COO Hamiltonian reader and block builder (oracle side).

TEST INFRASTRUCTURE ONLY: the serial restatement that the GPU block builder is
checked against.  Restates

* ``load_COOmatrix``          src/deviceHam_mod.f90:40-91  (rows "i j re [im]",
  optionally 0-based; nm = the largest index seen)
* ``devH_build_fromCOOfile``  src/deviceHam_mod.f90:93-232 (the ``blocksize``
  branch, the one ``main`` calls at src/main.f90:112-114)

The block loop (src/deviceHam_mod.f90:203-224) visits the entries in file order
and, for entry (row, col, h) in slab ix:

* col inside slab ix:        Hii(ix)[mm, nn] = h, then Hii(ix)[nn, mm] = conj(h),
  and Sii(ix)[mm, nn] = s when an overlap is given;
* col inside slab ix + 1:    H1i(ix)[mm, nn - bs] = h;
* anything else is dropped.

Then H1i(nx+1) = H1i(nx) and, without an overlap, Sii = I.  Later entries
overwrite earlier ones.

Two index quirks of the reference are resolved here by its evident intent, with
0-based (slab, local) = divmod(row0, bs):

* the reference computes ix = row/bs + 1 from the 1-based row, which puts the
  last orbital of each slab at local index 0 (outside the block);
* an entry whose column lies before its slab's first orbital gives a negative
  local index.

Both cases write outside the block arrays in the reference.  Wherever the
reference stays inside its arrays the two mappings agree.  Entries of the second
kind are dropped here.
"""
from __future__ import annotations

import numpy as np


def load_coo(path, use0index=False, iscomplex=False):
    """(h, row0, col0, norb): values, 0-based indices, orbital count.

    ``norb`` is the largest index in the file as written, as the reference's
    ``M = max(i, j)`` (src/deviceHam_mod.f90:58-62); with ``use0index`` that
    is one less than the orbital count, which the reference uses as is."""
    rows = []
    with open(path) as f:
        for line in f:
            parts = line.split()
            if len(parts) < 3:
                continue
            rows.append(parts)
    i = np.array([int(p[0]) for p in rows], dtype=np.int64)
    j = np.array([int(p[1]) for p in rows], dtype=np.int64)
    re = np.array([float(p[2]) for p in rows])
    im = np.array([float(p[3]) for p in rows]) if iscomplex else np.zeros_like(re)
    norb = int(max(i.max(), j.max())) if len(rows) else 0
    base = 0 if use0index else 1
    return re + 1j * im, i - base, j - base, norb


def coo_blocks(nx, bs, row0, col0, h, s=None):
    """(Hii, H1i, Sii): (nx, bs, bs), (nx+1, bs, bs), (nx, bs, bs) complex128,
    numpy [row, col] indexing.  Serial, in entry order."""
    Hii = np.zeros((nx, bs, bs), dtype=np.complex128)
    H1i = np.zeros((nx + 1, bs, bs), dtype=np.complex128)
    Sii = np.zeros((nx, bs, bs), dtype=np.complex128)
    for e in range(len(h)):
        ix, mm = divmod(int(row0[e]), bs)
        if ix >= nx:
            continue
        nn = int(col0[e]) - ix * bs
        if 0 <= nn < bs:
            Hii[ix, mm, nn] = h[e]
            Hii[ix, nn, mm] = np.conj(h[e])
            if s is not None:
                Sii[ix, mm, nn] = s[e]
        elif bs <= nn < 2 * bs:
            H1i[ix, mm, nn - bs] = h[e]
    H1i[nx] = H1i[nx - 1]
    if s is None:
        Sii[:] = np.eye(bs)
    return Hii, H1i, Sii
