"""Regenerate the committed known-answer fixtures from the reference's test_cnt/.

Reads (only in the build container, where the reference tree is mounted):
  <ref>/test_cnt/ham_dat                      Wannier90-style CNT Hamiltonian
  <ref>/test_cnt/sancho_g00.dat, sancho_gbb.dat  -Im Tr G00 / GBB per (E, lead)
  <ref>/test_cnt/ldos0000.dat, ndos0000.dat, pdos0000.dat  per-cell spectra
and writes
  cnt_blocks.npz  H00, H10 slab blocks (ns = 3 cells of nb = 32 orbitals, k = 0),
                  built by oracle.w90 (src/wannierHam3d.f90:273-301), plus Lx, nb, ns
  cnt_hr.npz      the model itself: Hr(nb, nb, nxr, nyr, nzr), R ranges, cell vectors
  cnt_golden.npz  the reference outputs as arrays on the exact energy grid
                  E = -6 + ie*5/199 (src/negf_mod.f90:100-101)
  cnt_text.npz    the text of ldos0000.dat, ndos0000.dat, pdos0000.dat, for
                  line-by-line checks of the (4E18.4) writer

The run that produced the .dat files used main.f90's defaults nx = 5, ns = 3
(src/main.f90:75-76), 200 energies on [-6, -1] eV, mu = -3.7 eV, T = 300 K.

Usage: python tests/golden/make_golden.py <reference checkout>   (the path is required)
"""
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))

from oracle.w90 import W90  # noqa: E402


def main(ref):
    tc = os.path.join(ref, "test_cnt")
    w = W90(os.path.join(tc, "ham_dat"))
    ns = 3
    H00, H10 = w.mat_def(ns)
    np.savez_compressed(os.path.join(HERE, "cnt_blocks.npz"), H00=H00, H10=H10, Lx=w.Lx,
                        nb=w.nb, ns=ns)
    np.savez_compressed(os.path.join(HERE, "cnt_hr.npz"), Hr=w.Hr,
                        ranges=np.array([w.xmin, w.xmax, w.ymin, w.ymax, w.zmin, w.zmax]),
                        alpha=w.alpha, beta=w.beta, gamm=w.gamm)
    nen = 200
    E = -6.0 + np.arange(nen) * (5.0 / (nen - 1))
    g00 = np.loadtxt(os.path.join(tc, "sancho_g00.dat"))
    gbb = np.loadtxt(os.path.join(tc, "sancho_gbb.dat"))

    def by_lead(a):
        out = np.zeros((nen, 2))  # [:,0] left lead (tag 2), [:,1] right lead (tag 1)
        for ie in range(nen):
            rows = a[2 * ie: 2 * ie + 2]
            assert np.allclose(rows[:, 0], E[ie], atol=1e-12)
            out[ie, 0] = rows[rows[:, 1] == 2, 2][0]
            out[ie, 1] = rows[rows[:, 1] == 1, 2][0]
        return out

    spec = {}
    for name in ("ldos", "ndos", "pdos"):
        d = np.loadtxt(os.path.join(tc, f"{name}0000.dat"))
        assert d.shape == (nen * 15, 4)
        spec[name] = d[:, 2:].reshape(nen, 15, 2)
        spec["x"] = d[:15, 0]
    text = {}
    for name in ("ldos", "ndos", "pdos"):
        with open(os.path.join(tc, f"{name}0000.dat")) as f:
            text[name] = np.array(f.read())
    np.savez_compressed(os.path.join(HERE, "cnt_text.npz"), **text)
    np.savez_compressed(os.path.join(HERE, "cnt_golden.npz"), E=E, sancho_g00=by_lead(g00),
                        sancho_gbb=by_lead(gbb), ldos=spec["ldos"], ndos=spec["ndos"],
                        pdos=spec["pdos"], x=spec["x"], nx=5, mu=-3.7, temp=300.0)


if __name__ == "__main__":
    if len(sys.argv) != 2:
        sys.exit("usage: python tests/golden/make_golden.py <reference checkout>")
    main(sys.argv[1])
