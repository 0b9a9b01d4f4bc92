"""The GW/SCBA loop over ranks that share the energy grid (gw_ephoton_3d_ijs with
comm_size > 1, src/gw_mod.f90:78-1070).

Each rank holds the self-energies of its energies (``shard.energy_range``). Per evaluation
of the SCBA map it:

1. solves the RGF with them on its energies (green_RGF_RS, src/gw_mod.f90:368-411);
2. moves G^R, G^<, G^> and the transposed G^<t, G^>t to its block elements over the whole
   energy grid (``shard.energies_to_ijs``, :440-456);
3. takes P by energy correlations there (:458-519);
4. moves P back to its energies (:522-524) and solves W per block (:582-604);
5. moves W to its elements (:636-638) and takes Sigma by energy convolutions (:646-698);
6. moves Sigma back to its energies (:700-702), recombines, symmetrises and copies the
   edge blocks (:698, 731-743, 950-959), and mixes linearly (:747-749).

That is fourteen all-to-alls per map, as in the reference. The residual of the mixing
loop is a sum over all energies: one all_reduce per iteration. On one rank the exchanges
are identities and the stages run the same kernels as ``qt_gw_step``, with the same
results.

Blocks are torch complex128 tensors of shape (nE_local, nx, nm, nm), stored column-major
per block: the last two axes are (column, row), as ``gw.to_dev`` makes them. Element
series are (nE, nx, nij_local) tensors.  With a grid of nk > 1 k-points every array has a
leading k axis (k slowest, the reference's (nm, nm, nx, nE, nk) order); one all-to-all
moves all k-points, and the stages sum over the k-pairs. The stage object does the compute: ``GpuStages``
calls the library on this rank's GPU; any object with the same five methods can stand in
for it.
"""
from __future__ import annotations

import ctypes as C
import math

import numpy as np

from . import _lib
from ._lib import check
from .rgf import OUT_KEYS, _ptr
from .shard import energies_to_ijs, energy_range, ijs_to_energies


class GpuStages:
    """The compute of one rank's share through the C-ABI: the batched RGF on its energies
    (``qt_rgf_solve``), ``qt_gw_polarization``, ``qt_gw_screened``, ``qt_gw_selfenergy``
    and ``qt_gw_sigma_post``. Arguments as for ``gw.GwSystem``, with ``E_local`` the rank's
    energies."""

    def __init__(self, ctx, H00, H10, E_local, nx, V, *, mu=(0.0, 0.0), temp=(300.0, 300.0),
                 eta_lead=1e-3, sancho_max_iter=100, sancho_tol=1e-100, precision="fp64",
                 kgrid=(1, 1), ndiag=None):
        from .gw import GwSystem
        self.sys = GwSystem(ctx, H00, H10, E_local, nx, V, mu=mu, temp=temp,
                            eta_lead=eta_lead, sancho_max_iter=sancho_max_iter,
                            sancho_tol=sancho_tol, precision=precision, kgrid=kgrid,
                            ndiag=ndiag)
        if self.sys.vflag:
            raise ValueError("the stages take one Coulomb block per momentum transfer")
        self.ctx = ctx
        self.lib = ctx._lib
        self.flags = _lib.QT_FLAG_DEVICE_POINTERS

    def zeros(self, shape):
        import torch
        return torch.zeros(shape, dtype=torch.complex128, device="cuda")

    def green(self, SR, SL):
        """G^R, G^<, G^> diagonal blocks with scattering self-energies SR, SL, one k-point
        at a time."""
        import torch
        s = self.sys
        G = [s.zeros() for _ in range(3)]
        if s.nE == 0:  # a rank with no energies still takes part in the exchanges
            return tuple(G)
        one = s.nk == 1
        for k in range(s.nk):
            out = {"G_r": G[0] if one else G[0][k], "G_lesser": G[1] if one else G[1][k],
                   "G_greater": G[2] if one else G[2][k],
                   "status": torch.zeros(s.nE, dtype=torch.int32, device="cuda")}
            o = _lib.QtOutputs(*[_ptr(out.get(n)) for n in OUT_KEYS])
            sr = (SR if one else SR[k]).contiguous()  # held until the call has been made
            sl = (SL if one else SL[k]).contiguous()
            check(self.lib.qt_rgf_solve(self.ctx.handle, C.byref(s.devk[k]), _ptr(s.E), s.nE,
                                        C.byref(s.con), _ptr(sr), _ptr(sl), s.prec, self.flags,
                                        C.byref(o)),
                  allow_points=True)
        return tuple(G)

    def _series_shape(self, g):
        """(energies, series per k-point) of an element-series array"""
        if self.sys.nk == 1:
            return g.shape[0], g[0].numel()
        return g.shape[1], g[0, 0].numel()

    def polarization(self, gr, gl, gg, glt, ggt, scale):
        self.sys._grid()
        n, ns = self._series_shape(gr)
        P = [self.zeros(gr.shape) for _ in range(3)]
        if ns == 0:  # no block elements on this rank
            return tuple(P)
        check(self.lib.qt_gw_polarization(self.ctx.handle, n, ns, _ptr(gr), _ptr(gl), _ptr(gg),
                                          _ptr(glt), _ptr(ggt), scale, _ptr(P[0]), _ptr(P[1]),
                                          _ptr(P[2]), self.flags))
        return tuple(P)

    def screened(self, PR, PL, PG):
        self.sys._grid()
        nm = PR.shape[-1]
        nblk = PR.numel() // (nm * nm)
        W = [self.zeros(PR.shape) for _ in range(3)]
        if nblk == 0:
            return tuple(W)
        check(self.lib.qt_gw_screened(self.ctx.handle, nm, nblk, _ptr(self.sys.V), _ptr(PR),
                                      _ptr(PL), _ptr(PG), _ptr(W[0]), _ptr(W[1]), _ptr(W[2]),
                                      self.sys.prec, self.flags))
        return tuple(W)

    def self_energy(self, gr, gl, gg, wr, wl, wg, scale):
        self.sys._grid()
        n, ns = self._series_shape(gr)
        S = [self.zeros(gr.shape) for _ in range(3)]
        if ns == 0:
            return tuple(S)
        check(self.lib.qt_gw_selfenergy(self.ctx.handle, n, ns, _ptr(gr), _ptr(gl), _ptr(gg),
                                        _ptr(wr), _ptr(wl), _ptr(wg), scale, _ptr(S[0]),
                                        _ptr(S[1]), _ptr(S[2]), self.flags))
        return tuple(S)

    def post(self, SR, SL, SG):
        self.sys._grid()
        ne, nx, nm = SR.shape[-4], SR.shape[-3], SR.shape[-1]
        if ne == 0:
            return
        check(self.lib.qt_gw_sigma_post(self.ctx.handle, nm, nx, ne, _ptr(SR), _ptr(SL),
                                        _ptr(SG), self.flags | _lib.QT_FLAG_SYNC))


class ShardedGw:
    """One rank's part of the SCBA loop over ``world`` ranks (``group``: a torch.distributed
    process group, gloo for host tensors, NCCL for device tensors; unused when world = 1).

    ``nE`` energies of uniform spacing ``dE`` on the whole grid; this rank owns
    ``energy_range(nE, world, rank)``. ``stages`` is the compute for those energies."""

    def __init__(self, stages, nE, nx, nm, dE, *, world=1, rank=0, group=None, spindeg=2.0,
                 nk=1):
        if 2 * nE > 4096:
            raise ValueError("nE <= 2048 (FFT length 4096)")
        self.stages = stages
        self.nE, self.nx, self.nm, self.dE = int(nE), int(nx), int(nm), float(dE)
        self.world, self.rank, self.group = int(world), int(rank), group
        self.spindeg, self.nk = float(spindeg), int(nk)
        self.lo, self.hi = energy_range(self.nE, self.world, self.rank)

    @classmethod
    def on_gpu(cls, ctx, H00, H10, E, nx, V, *, world=1, rank=0, group=None, mu=(0.0, 0.0),
               temp=(300.0, 300.0), eta_lead=1e-3, sancho_max_iter=100, sancho_tol=1e-100,
               spindeg=2.0, precision="fp64", kgrid=(1, 1), ndiag=None):
        """The rank's share of a ``gw.GwSystem`` problem on its GPU."""
        E = np.ascontiguousarray(E, dtype=np.float64)
        lo, hi = energy_range(len(E), world, rank)
        st = GpuStages(ctx, H00, H10, E[lo:hi], nx, V, mu=mu, temp=temp, eta_lead=eta_lead,
                       sancho_max_iter=sancho_max_iter, sancho_tol=sancho_tol,
                       precision=precision, kgrid=kgrid, ndiag=ndiag)
        return cls(st, len(E), nx, np.asarray(H00).shape[-1], E[1] - E[0], world=world,
                   rank=rank, group=group, spindeg=spindeg, nk=kgrid[0] * kgrid[1])

    @property
    def local_energies(self):
        return self.hi - self.lo

    def zeros(self):
        shape = (self.local_energies, self.nx, self.nm, self.nm)
        return self.stages.zeros(shape if self.nk == 1 else (self.nk,) + shape)

    def _to_ijs(self, A):
        """(nk,) nE_local, nx, nm, nm blocks -> (nk,) nE, nx, nij_local series; the k-points
        travel in the same all-to-all, as the slabs do"""
        ne, nk, nx = self.local_energies, self.nk, self.nx
        if nk > 1:
            A = A.permute(1, 0, 2, 3, 4)
        y = energies_to_ijs(A.reshape(ne, nk * nx, self.nm * self.nm), self.nE, self.world,
                            self.rank, self.group)
        if nk == 1:
            return y
        return y.view(self.nE, nk, nx, -1).permute(1, 0, 2, 3).contiguous()

    def _to_energies(self, A):
        ne, nk, nx, nm = self.local_energies, self.nk, self.nx, self.nm
        if nk > 1:
            A = A.permute(1, 0, 2, 3).reshape(self.nE, nk * nx, -1)
        x = ijs_to_energies(A, nm * nm, self.world, self.rank, self.group)
        if nk == 1:
            return x.reshape(ne, nx, nm, nm).contiguous()
        return x.view(ne, nk, nx, nm, nm).permute(1, 0, 2, 3, 4).contiguous()

    def step(self, SR, SL):
        """Sigma_new (R, <, >) on this rank's energies from Sigma (R, <) there: one evaluation
        of the SCBA map, collective over the ranks."""
        st = self.stages
        GR, GL, GG = st.green(SR, SL)
        GLt = GL.transpose(-1, -2).contiguous()
        GGt = GG.transpose(-1, -2).contiguous()
        gr, gl, gg, glt, ggt = (self._to_ijs(A) for A in (GR, GL, GG, GLt, GGt))
        # -i dE / (2 pi) spindeg / nk (src/gw_mod.f90:516-519)
        pr, pl, pg = st.polarization(gr, gl, gg, glt, ggt,
                                     self.dE / (2.0 * math.pi) * self.spindeg / self.nk)
        PR, PL, PG = (self._to_energies(A) for A in (pr, pl, pg))
        WR, WL, WG = st.screened(PR, PL, PG)
        wr, wl, wg = (self._to_ijs(A) for A in (WR, WL, WG))
        # i dE / (2 pi) / nk (src/gw_mod.f90:694-697)
        sr, sl, sg = st.self_energy(gr, gl, gg, wr, wl, wg, self.dE / (2.0 * math.pi) / self.nk)
        NR, NL, NG = (self._to_energies(A) for A in (sr, sl, sg))
        st.post(NR, NL, NG)
        return NR, NL, NG

    def _global_sum(self, values):
        import torch
        import torch.distributed as dist
        t = torch.stack([v.to(torch.float64).reshape(()) for v in values])
        if self.world > 1:
            t = t.to("cuda" if dist.get_backend(self.group) == "nccl" else "cpu")
            dist.all_reduce(t, group=self.group)
        return t.cpu().numpy()

    def scba(self, alpha=0.3, tol=1e-8, max_iter=60, start=None):
        """Plain linear mixing until the residual ||S_new - S||_F / ||S_new||_F over Sigma^<
        and Sigma^> of all energies is <= tol (the reference runs a fixed niter, with no
        test). Returns this rank's (SR, SL, SG) and the residual of every map evaluated."""
        SR, SL, SG = start if start is not None else (self.zeros(), self.zeros(), self.zeros())
        res = []
        for _ in range(max_iter):
            NR, NL, NG = self.step(SR, SL)
            d, m = self._global_sum([((NL - SL).abs() ** 2).sum() + ((NG - SG).abs() ** 2).sum(),
                                     (NL.abs() ** 2).sum() + (NG.abs() ** 2).sum()])
            r = math.sqrt(d) / max(math.sqrt(m), 1e-300)
            res.append(r)
            SR = SR + alpha * (NR - SR)
            SL = SL + alpha * (NL - SL)
            SG = SG + alpha * (NG - SG)
            if r <= tol:
                break
        return SR, SL, SG, np.array(res)
