"""Energy integrals of the currents the RGF returns (host side, numpy).

* ``terminal_current``  the Id_iteration.dat figure (src/gw_mod.f90:413-428):
                        sum over energies and k of a contact current spectrum,
                        x dE e0^2 spindeg / (2 pi hbar nk), in A
* ``block_current``     what the reference's ``calc_block_current`` call
                        (src/gw_mod.f90:384, the routine itself is absent)
                        feeds into gw_I / gw_EI: per bond and k, the
                        energy-integrated current and energy current

Both use the reference's constants (src/static.f90:10,14; src/fft_mod.f90:19),
so the figures agree with its output files to rounding.
"""
from __future__ import annotations

import numpy as np

E0 = 1.6022e-19                # C
HBAR = 1.0546e-34              # J s
TPI = 3.14159265359 * 2.0


def prefactor(dE, spindeg=2.0, nk=1):
    """A per (eV x dimensionless current spectrum) on a grid of spacing dE (eV)."""
    return dE * E0 / TPI / HBAR * E0 * float(spindeg) / float(nk)


def terminal_current(spectrum, E, spindeg=2.0, nk=1):
    """Total current (A) of a contact spectrum tr or tre of shape (nE,) or (nE, nk)."""
    E = np.asarray(E, dtype=np.float64)
    return float(np.sum(spectrum)) * prefactor(E[1] - E[0], spindeg, nk)


def block_current(bond_cur, E, spindeg=2.0, nk=1):
    """(I, EI): bond currents integrated over energy, each (nk, nx-1).

    ``bond_cur`` is (nE, nk, nx-1) as ``rgf_solve(..., want_bond=True)`` returns it, or
    (nE, nx-1) for one k.  I is in A; EI = sum_E E J(E) x the same factor, in W."""
    J = np.asarray(bond_cur, dtype=np.float64)
    if J.ndim == 2:
        J = J[:, None, :]
    E = np.asarray(E, dtype=np.float64)
    f = prefactor(E[1] - E[0], spindeg, nk)
    return J.sum(axis=0) * f, np.einsum("e,ekb->kb", E, J) * f
