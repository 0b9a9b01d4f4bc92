"""Spectrum files in the reference's format.

``write_spectrum_summed_over_k`` (src/output_mod.f90:14-61) writes, for every energy
and every cell c of every slab, one record ``(4E18.4) x, E, Re(t) c1, Im(t) c2`` with
t = sum_k sum_b G_bb / nk over the cell's NB orbitals, then an empty record after each
energy.  ``negf_solve`` names the files ldos/ndos/pdos + ``%04d`` + ``.dat`` with the
coefficients (1, -2), (1, 1), (1, -1) (src/negf_mod.f90:140-149).  The same records are
produced here from the diagonals the GPU sweep returns, so the files compare line by
line with the reference's (test_cnt/ldos0000.dat and the others).
"""
from __future__ import annotations

import math
import os

import numpy as np


def fortran_e(x, w=18, d=4):
    """Fortran ``Ew.d`` edit descriptor: 0.ddddE+ee right-justified in ``w`` columns (the
    exponent letter is dropped for |exponent| > 99, as the standard prescribes)."""
    x = float(x)
    if math.isnan(x) or math.isinf(x):
        return ("NaN" if math.isnan(x) else ("-Infinity" if x < 0 else "Infinity")).rjust(w)
    neg = math.copysign(1.0, x) < 0
    if x == 0.0:
        digits, e = "0" * d, 0
    else:
        mant, ex = f"{abs(x):.{d - 1}e}".split("e")
        digits, e = mant.replace(".", ""), int(ex) + 1
    es = f"E{e:+03d}" if abs(e) <= 99 else f"{e:+04d}"
    return (("-" if neg else "") + "0." + digits + es).rjust(w)


def spectrum_records(diag, E, NB, NS, Lx, coeff):
    """The file's text: ``diag`` (nE, nk, nx, nm) complex diagonals, nm = NB*NS."""
    diag = np.asarray(diag)
    nE, nk, nx, nm = diag.shape
    if nm != NB * NS:
        raise ValueError("nm must be NB * NS")
    # sum over k and the cell's orbitals, then / nk (src/output_mod.f90:45-55)
    t = diag.reshape(nE, nk, nx, NS, NB).sum(axis=(1, 4)) / nk
    return format_records(t.real * coeff[0], t.imag * coeff[1], E, Lx)


def format_records(c1, c2, E, Lx):
    """Records of the two value columns ``c1``, ``c2`` (nE, ncells): x accumulates Lx over
    the cells, E per energy, an empty record after each energy."""
    c1 = np.asarray(c1).reshape(len(E), -1)
    c2 = np.asarray(c2).reshape(len(E), -1)
    lines = []
    for ie in range(len(E)):
        xx = 0.0
        en = fortran_e(E[ie])
        for c in range(c1.shape[1]):
            xx = xx + Lx  # accumulated, as the reference does
            lines.append(fortran_e(xx) + en + fortran_e(c1[ie, c]) + fortran_e(c2[ie, c]) + "\n")
        lines.append("\n")
    return "".join(lines)


def write_spectrum_summed_over_k(dataset, i, diag, E, NB, NS, Lx, coeff, append=False,
                                 directory="."):
    """Write ``<directory>/<dataset><i:04d>.dat``; returns the path."""
    path = os.path.join(directory, f"{dataset}{i:04d}.dat")
    with open(path, "a" if append else "w") as f:
        f.write(spectrum_records(diag, E, NB, NS, Lx, coeff))
    return path


SPECTRA = (("ldos", "diag_gr", (1.0, -2.0)), ("ndos", "diag_gl", (1.0, 1.0)),
           ("pdos", "diag_gg", (1.0, -1.0)))


def write_negf_spectra(result, E, NB, NS, Lx, i=0, directory=".", append=False):
    """ldos/ndos/pdos files of ``negf_solve`` (src/negf_mod.f90:140-149) from an
    ``rgf_solve`` result holding diag_gr, diag_gl and diag_gg."""
    return [write_spectrum_summed_over_k(name, i, result[key], E, NB, NS, Lx, c, append,
                                         directory) for name, key, c in SPECTRA]
