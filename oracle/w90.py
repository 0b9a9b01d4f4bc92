"""Wannier90-style Hamiltonian reader and slab-block builder (oracle side).

TEST INFRASTRUCTURE ONLY (used to turn the reference's test_cnt/ham_dat into
committed fixtures).  Restates

* ``w90_load_from_file``  src/wannierHam3d.f90:72-152 (header, cell, H(R) list;
  band-edge search and Wannier centres are not needed for the blocks)
* ``w90_MAT_DEF``         src/wannierHam3d.f90:273-301 (H_ii and H_{i+1,i} of a
  slab of ``ns`` cells at transverse momentum (ky, kz))
"""
from __future__ import annotations

import numpy as np


class W90:
    def __init__(self, path):
        with open(path) as f:
            lines = f.read().split("\n")
        it = iter(lines)
        self.nvb, self.spin_deg = (int(x) for x in next(it).split()[:2])
        next(it)  # "cell"
        self.alpha = np.array([float(x) for x in next(it).split()[:3]])
        self.beta = np.array([float(x) for x in next(it).split()[:3]])
        self.gamm = np.array([float(x) for x in next(it).split()[:3]])
        next(it)  # "hamiltonian"
        n = int(next(it).split()[0])
        ham = np.array([[float(x) for x in next(it).split()[:7]] for _ in range(n)])
        self.xmin, self.xmax = int(ham[:, 0].min()), int(ham[:, 0].max())
        self.ymin, self.ymax = int(ham[:, 1].min()), int(ham[:, 1].max())
        self.zmin, self.zmax = int(ham[:, 2].min()), int(ham[:, 2].max())
        self.nb = int(ham[:, 3].max())
        nxr = self.xmax - self.xmin + 1
        nyr = self.ymax - self.ymin + 1
        nzr = self.zmax - self.zmin + 1
        # Hr(m, n, Rx, Ry, Rz) = Re + i Im      src/wannierHam3d.f90:147-152
        self.Hr = np.zeros((self.nb, self.nb, nxr, nyr, nzr), dtype=np.complex128)
        for row in ham:
            m, nn = int(np.floor(row[3])) - 1, int(np.floor(row[4])) - 1
            self.Hr[m, nn, int(np.floor(row[0])) - self.xmin,
                    int(np.floor(row[1])) - self.ymin,
                    int(np.floor(row[2])) - self.zmin] = row[5] + 1j * row[6]
        self._axes()

    def _axes(self):
        # transport / transverse unit vectors and the cell length, src/wannierHam3d.f90:130-136
        xhat = self.alpha / np.linalg.norm(self.alpha)
        yhat = -np.cross(xhat, self.gamm)
        yhat = yhat / np.linalg.norm(yhat)
        zhat = self.gamm / np.linalg.norm(self.gamm)
        self.xhat, self.yhat, self.zhat = xhat, yhat, zhat
        self.Lx = abs(np.dot(self.alpha, xhat))

    @classmethod
    def from_arrays(cls, Hr, ranges, alpha, beta, gamm):
        """A model from Hr (nb, nb, nxr, nyr, nzr) and ranges (xmin, xmax, ymin, ymax, zmin,
        zmax), as stored in the committed fixture."""
        w = cls.__new__(cls)
        w.Hr = np.asarray(Hr, dtype=np.complex128)
        w.nb = w.Hr.shape[0]
        w.xmin, w.xmax, w.ymin, w.ymax, w.zmin, w.zmax = (int(x) for x in ranges)
        w.alpha, w.beta, w.gamm = (np.asarray(v, dtype=np.float64) for v in (alpha, beta, gamm))
        w._axes()
        return w

    def mat_def(self, ns, kx=0.0, ky=0.0, kz=0.0):
        """(H00, H10) slab blocks of ``ns`` cells, src/wannierHam3d.f90:273-301."""
        nb = self.nb
        H00 = np.zeros((nb * ns, nb * ns), dtype=np.complex128)
        H10 = np.zeros_like(H00)
        kv = kx * self.xhat + ky * self.yhat + kz * self.zhat
        for i in range(1, ns + 1):
            for k in range(1, ns + 1):
                for j in range(self.ymin, self.ymax + 1):
                    for l in range(self.zmin, self.zmax + 1):
                        r = (i - k) * self.alpha + j * self.beta + l * self.gamm
                        ph = np.exp(-1j * np.dot(r, kv))
                        rows = slice((i - 1) * nb, i * nb)
                        cols = slice((k - 1) * nb, k * nb)
                        if self.xmin <= i - k <= self.xmax:
                            H00[rows, cols] += self.Hr[:, :, i - k - self.xmin,
                                                       j - self.ymin, l - self.zmin] * ph
                        if self.xmin <= i - k + ns <= self.xmax:
                            H10[rows, cols] += self.Hr[:, :, i - k + ns - self.xmin,
                                                       j - self.ymin, l - self.zmin] * ph
        return H00, H10
