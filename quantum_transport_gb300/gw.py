"""GW/SCBA self-energy loop on the GPU (host-side mirror of gw_ephoton_3d_ijs).

* ``corr`` / ``conv``  corr1d2 / conv1d2 (src/fft_mod.f90:58-168), batched
* ``gw_step``          one evaluation Sigma -> Sigma_new of the SCBA map
                       (src/gw_mod.f90:368-749, 950-959), at one k-point or summed
                       over the k-pairs of an nky x nkz grid, optionally banded
                       (ndiag)
* ``scba``             the plain linear-mixing loop (src/gw_mod.f90:349-749)
                       run to a residual tolerance, optionally with the terminal
                       currents of every iteration (Id_iteration.dat, :413-428)
* ``currents``         the per-energy contact and bond currents of green_RGF_RS
                       (:1131-1345) at given self-energies
* ``ephoton_sigma``    the e-photon self-energy in the monochromatic approximation
                       (:1075-1122); with ``shard.energy_halo`` across energy shards

All arrays are torch CUDA tensors (device pointers); energy-resolved blocks
are complex128 tensors of shape (nE, nx, nm, nm) stored column-major per
block (``to_dev`` / ``from_dev`` convert from/to row-major numpy).
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import _lib
from ._lib import QtContacts, QtDevice, check
from .rgf import OUT_KEYS, PREC, _ptr, colmajor


def to_dev(A):
    import torch
    return torch.from_numpy(colmajor(A)).cuda()


def from_dev(T):
    return np.swapaxes(T.cpu().numpy(), -1, -2)


def corr(ctx, X, Y, mode="corr"):
    """Z = corr/conv of energy-major series X, Y: tensors (n, nseries) complex128 on the GPU."""
    import torch
    n, ns = X.shape
    Z = torch.empty_like(X)
    check(ctx._lib.qt_corr_batch(ctx.handle, n, ns, _ptr(X), _ptr(Y), _ptr(Z),
                                 0 if mode == "corr" else 1,
                                 _lib.QT_FLAG_DEVICE_POINTERS | _lib.QT_FLAG_SYNC))
    return Z


class GwSystem:
    """Device, energy grid, contacts and Coulomb blocks of one SCBA problem.

    One k-point (``kgrid=(1, 1)``): ``H00`` one on-site block shared by all slabs
    (nm, nm), or one per slab (nx, nm, nm); ``H10`` (nm, nm); ``V`` (nm, nm), or one
    Coulomb block per slab (nx, nm, nm).  A grid of nk = nky * nkz k-points
    (``kgrid=(nky, nkz)``, k = kz + ky nkz): ``H00`` (nk, nm, nm) or (nk, nx, nm, nm),
    ``H10`` (nm, nm) or (nk, nm, nm), ``V`` (nk, nm, nm) one block per momentum transfer q,
    (nk, nx, nm, nm) one per q and slab (the reference's Vii), or (nm, nm) for all; the
    self-energies are then (nk, nE, nx, nm, nm).  The leads continue the first and last
    slab.  ``ndiag``: keep only |i - j| <= ndiag of P and Sigma (src/gw_mod.f90:471-475),
    None for full blocks.
    ``sancho_reset`` selects green_RGF_RS's lead decimation as written
    (src/gw_mod.f90:1440-1445): points not converged after ``sancho_max_iter`` steps take
    the isolated-slab surface function; by default they keep their last iterate and are
    flagged."""

    def __init__(self, ctx, H00, H10, E, nx, V, *, mu=(0.0, 0.0), temp=(300.0, 300.0),
                 eta_lead=1e-3, sancho_max_iter=100, sancho_tol=1e-100, spindeg=2.0,
                 precision="fp64", sancho_reset=False, kgrid=(1, 1), ndiag=None):
        import torch
        self.ctx = ctx
        self.nky, self.nkz = int(kgrid[0]), int(kgrid[1])
        self.nk = self.nky * self.nkz
        self.ndiag = -1 if ndiag is None else int(ndiag)
        H00, H10, V = np.asarray(H00), np.asarray(H10), np.asarray(V)
        nk = self.nk
        if nk > 1:
            if H00.shape[0] != nk or H00.ndim not in (3, 4):
                raise ValueError("with several k-points H00 is (nk, [nx,] nm, nm)")
            if V.ndim == 2:
                V = np.repeat(V[None], nk, axis=0)
            if V.shape[0] != nk or V.ndim not in (3, 4):
                raise ValueError("V must be (nk, [nx,] nm, nm) or (nm, nm)")
            per_slab = H00.ndim == 4
            h10_k = H10.ndim == 3
            v_slab = V.ndim == 4
        else:
            per_slab = H00.ndim == 3
            h10_k = False
            v_slab = V.ndim == 3
        if v_slab and V.shape[-3] != nx:
            raise ValueError("per-slab V must have nx blocks")
        self.vflag = _lib.QT_FLAG_V_PER_SLAB if v_slab else 0
        self.nm = H00.shape[-1]
        self.nx = nx
        self.nE = len(E)
        if per_slab and H00.shape[-3] != nx:
            raise ValueError("per-slab H00 must have nx blocks")
        nm2 = self.nm * self.nm
        hl = nm2 if per_slab else 0  # per-slab blocks or one shared block
        hk = (nx * nm2 if per_slab else nm2) if nk > 1 else 0
        h1k = nm2 if h10_k else 0
        self.H00 = to_dev(H00)
        self.H10 = to_dev(H10)
        self.E = torch.from_numpy(np.ascontiguousarray(E, dtype=np.float64)).cuda()
        self.V = to_dev(V)
        self.spindeg = spindeg
        self.prec = PREC[precision]
        self.dev = QtDevice(self.nm, nx, nk, _ptr(self.H00), hk, hl, _ptr(self.H10), h1k, 0,
                            None, 0, 0)
        # one k-point each, for the per-energy currents
        h0, h1 = self.H00.data_ptr(), self.H10.data_ptr()
        self.devk = [QtDevice(self.nm, nx, 1, C.c_void_p(h0 + 16 * k * hk), 0, hl,
                              C.c_void_p(h1 + 16 * k * h1k), 0, 0, None, 0, 0)
                     for k in range(nk)]
        self.con = QtContacts(mu[0], mu[1], temp[0], temp[1], eta_lead, 0.0, sancho_tol,
                              int(sancho_max_iter),
                              _lib.QT_QUIRK_GW_SANCHO_RESET if sancho_reset else 0)

    def _grid(self):
        """The context's GW grid and band, set before every call (contexts may be shared)."""
        check(self.ctx._lib.qt_ctx_set_gw_grid(self.ctx.handle, self.nky, self.nkz, self.ndiag))

    def zeros(self):
        import torch
        shape = (self.nE, self.nx, self.nm, self.nm)
        if self.nk > 1:
            shape = (self.nk,) + shape
        return torch.zeros(shape, dtype=torch.complex128, device="cuda")

    def step(self, SR, SL):
        """Sigma_new (R, <, >) from Sigma (R, <): one SCBA map evaluation."""
        NR, NL, NG = self.zeros(), self.zeros(), self.zeros()
        self._grid()
        check(self.ctx._lib.qt_gw_step(self.ctx.handle, C.byref(self.dev), _ptr(self.E), self.nE,
                                       C.byref(self.con), _ptr(self.V), self.spindeg, self.prec,
                                       _lib.QT_FLAG_DEVICE_POINTERS | self.vflag, _ptr(SR),
                                       _ptr(SL), _ptr(NR), _ptr(NL), _ptr(NG)))
        return NR, NL, NG

    def scba(self, alpha=0.3, tol=1e-8, max_iter=60, start=None, with_currents=False):
        """Plain linear mixing to tol; returns (SR, SL, SG, residuals), and with
        ``with_currents`` also the (iterations, 2) left/right terminal currents in A, the
        columns of Id_iteration.dat."""
        SR, SL, SG = start if start is not None else (self.zeros(), self.zeros(), self.zeros())
        res = np.zeros(max_iter)
        cur = np.zeros((max_iter, 2)) if with_currents else None
        it = C.c_int()
        self._grid()
        check(self.ctx._lib.qt_scba_solve(self.ctx.handle, C.byref(self.dev), _ptr(self.E),
                                          self.nE, C.byref(self.con), _ptr(self.V), self.spindeg,
                                          alpha, tol, max_iter, self.prec,
                                          _lib.QT_FLAG_DEVICE_POINTERS | self.vflag, _ptr(SR),
                                          _ptr(SL), _ptr(SG), res.ctypes.data_as(C.c_void_p),
                                          C.byref(it),
                                          _ptr(cur)))
        if with_currents:
            return SR, SL, SG, res[:it.value], cur[:it.value]
        return SR, SL, SG, res[:it.value]

    def currents(self, SR, SL):
        """Per-energy currents of the RGF with self-energies (SR, SL): dict of numpy arrays
        tr, tre (nE,) (green_RGF_RS's right- and left-contact currents), bond_cur
        (nE, nx-1), the traces of its cur blocks (src/gw_mod.f90:1254-1276), and diag_gr
        (nE, nx*nm), the diagonal of G^R behind the LDOS; with several k-points each has a
        leading k axis."""
        import torch
        res = []
        SRk = SR if self.nk > 1 else SR[None]
        SLk = SL if self.nk > 1 else SL[None]
        for k in range(self.nk):
            out = {"tr": torch.zeros(self.nE, dtype=torch.float64, device="cuda"),
                   "diag_gr": torch.zeros((self.nE, self.nx * self.nm), dtype=torch.complex128,
                                          device="cuda"),
                   "tre": torch.zeros(self.nE, dtype=torch.float64, device="cuda"),
                   "bond_cur": torch.zeros((self.nE, self.nx - 1), dtype=torch.float64,
                                           device="cuda"),
                   "status": torch.zeros(self.nE, dtype=torch.int32, device="cuda")}
            o = _lib.QtOutputs(*[_ptr(out.get(n)) for n in OUT_KEYS])
            sr, sl = SRk[k].contiguous(), SLk[k].contiguous()
            check(self.ctx._lib.qt_rgf_solve(self.ctx.handle, C.byref(self.devk[k]),
                                             _ptr(self.E), self.nE, C.byref(self.con),
                                             _ptr(sr), _ptr(sl), self.prec,
                                             _lib.QT_FLAG_DEVICE_POINTERS | _lib.QT_FLAG_SYNC,
                                             C.byref(o)), allow_points=True)
            res.append({n: v.cpu().numpy() for n, v in out.items()})
        if self.nk == 1:
            return res[0]
        return {n: np.stack([r[n] for r in res]) for n in res[0]}


# (hbar/m0)^2 / (2 eps0 c0^3) with the reference's constants (src/gw_mod.f90:92,
# src/static.f90:10-14)
PHOTON_PRE_FACT = ((1.0546e-34 / 9.109e-31) ** 2) / (2.0 * 8.854e-12 * 2.998e8 ** 3)


def photon_steps(hw, dE):
    """nop = floor(hw / dE): the photon energy in grid steps (src/gw_mod.f90:194)."""
    return int(np.floor(hw / dE))


def ephoton_sigma(ctx, M, GL, GG, nop, intensity, hw, *, halo=False, precision="fp64"):
    """(SR, SL, SG) e-photon self-energies (nE, nx, nm, nm) on the GPU.

    ``M``: (nx, nm, nm) interaction blocks; ``GL``, ``GG``: (nE, nx, nm, nm) G^<, G^>,
    or (nE + 2 nop, ...) with ``halo`` (from ``shard.energy_halo``).  All torch CUDA
    tensors, column-major blocks (``to_dev``)."""
    import torch
    nEx, nx, nm = GL.shape[0], GL.shape[1], GL.shape[-1]
    nE = nEx - 2 * nop if halo else nEx
    shape = (nE, nx, nm, nm)
    SR, SL, SG = (torch.empty(shape, dtype=torch.complex128, device=GL.device) for _ in range(3))
    scale = PHOTON_PRE_FACT * intensity / hw ** 2
    check(ctx._lib.qt_ephoton_sigma(ctx.handle, nm, nx, nE, int(nop), 1 if halo else 0, _ptr(M),
                                    _ptr(GL), _ptr(GG), scale, PREC[precision],
                                    _lib.QT_FLAG_DEVICE_POINTERS | _lib.QT_FLAG_SYNC, _ptr(SR),
                                    _ptr(SL), _ptr(SG)))
    return SR, SL, SG

