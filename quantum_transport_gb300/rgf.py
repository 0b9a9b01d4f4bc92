"""Host-side mirror of the reference's RGF interface on top of libqtgpu.so.

Names, argument meaning and error behaviour follow the Fortran routines:

* ``Context``                  cuda_rgf_init / cuda_rgf_finish (src/cuda_rgf_mod.f90:32-51)
* ``cuda_rgf_constblocksize``  src/cuda_rgf_mod.f90:53-413 (one energy point)
* ``rgf_solve``                the ``do ie / do ik`` loop of negf_solve
                               (src/negf_mod.f90:115-127) as one batched call
* ``negf_solve``               src/negf_mod.f90:41-165 incl. the per-cell spectra of
                               write_spectrum_summed_over_k (src/output_mod.f90:14-61)
* ``sancho``                   src/rgf_mod.f90:482 / src/cuda_rgf_mod.f90:657-765
* ``mul_c``, ``invert``        src/matrix_c.f90:615-660, src/linalg.f90:42-62 (batched)

Arrays are numpy complex128 in mathematical (row, col) indexing; they are
converted to the column-major layout of the C-ABI here.  torch CUDA tensors
in column-major layout (i.e. ``X.mT.contiguous()`` of a row-major block) may
be passed instead and are used in place (device-pointer mode).

Errors: a failing call raises ``QtError``.  Point-level failures (singular
block, Sancho not converged, NaN) do not raise; they are reported in the
``status`` array, in contrast to the reference's abort()
(src/cuda_rgf_mod.f90:180-187).
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import _lib
from ._lib import QtContacts, QtDevice, QtOutputs, check

PREC = {"fp64": _lib.QT_PREC_FP64, "mixed": _lib.QT_PREC_MIXED,
        "mixed-fp64": _lib.QT_PREC_MIXED_FP64}


class Context:
    """GPU context: device scratch and the stream it launches on (cuda_rgf_init/finish).

    By default the library launches on PyTorch's current stream of ``device``, so that
    torch tensors passed in place (allocated, sliced or zeroed by torch) are ordered with
    the library's kernels.  ``torch_stream=False`` keeps the context's own stream; callers
    then order their work with ``sync()``.
    """

    def __init__(self, device=0, torch_stream=True):
        self._lib = _lib.load()
        h = C.c_void_p()
        check(self._lib.qt_ctx_create(C.byref(h), int(device)))
        self.handle = h
        self.device = device
        if torch_stream:
            import torch
            s = torch.cuda.current_stream(device).cuda_stream
            check(self._lib.qt_ctx_set_stream(h, C.c_void_p(s), 0))

    def close(self):
        if self.handle:
            self._lib.qt_ctx_destroy(self.handle)
            self.handle = None

    def sync(self):
        check(self._lib.qt_ctx_sync(self.handle))

    def set_scratch_limit(self, nbytes):
        check(self._lib.qt_ctx_set_scratch_limit(self.handle, int(nbytes)))

    def set_wave_points(self, points):
        """Points per wave of the batched sweeps (0: the library's default of 608)."""
        check(self._lib.qt_ctx_set_wave_points(self.handle, int(points)))

    def profile(self, enable=True):
        """Event-time every block product / inverse launch on this context's stream, and the
        phases of each GW map."""
        check(self._lib.qt_ctx_profile(self.handle, int(bool(enable))))

    # kinds 5-8 are phases of the GW map; the products and inverses inside them are also
    # counted in kinds 0-4
    PROFILE_KINDS = {0: "zgemm_oz_c64", 1: "zgemm_oz_c128", 2: "zgemm_f64", 3: "zinv_f32",
                     4: "zinv_f64", 5: "gw_rgf", 6: "gw_corrconv", 7: "gw_screened",
                     8: "gw_post"}

    def profile_read(self):
        """{kind name: (launches, ms, algorithmic flops, executed tensor flops)} since last read."""
        out = {}
        for k, name in self.PROFILE_KINDS.items():
            nl, ms, fa, ft = C.c_int64(), C.c_double(), C.c_double(), C.c_double()
            check(self._lib.qt_ctx_profile_read(self.handle, k, C.byref(nl), C.byref(ms),
                                                C.byref(fa), C.byref(ft)))
            if nl.value:
                out[name] = (nl.value, ms.value, fa.value, ft.value)
        return out

    def inverse_fallbacks(self, reset=True):
        """Block inverses the split path redid in FP64 since the last reset (ill-conditioned
        blocks whose first refinement residual was too large)."""
        n = C.c_int64()
        check(self._lib.qt_ctx_inverse_fallbacks(self.handle, C.byref(n), 1 if reset else 0))
        return n.value

    @property
    def stream_ptr(self):
        p = C.c_void_p()
        check(self._lib.qt_ctx_stream(self.handle, C.byref(p)))
        return p.value or 0


    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def kernel_launches():
    """Kernels launched by libqtgpu.so in this process."""
    return int(_lib.load().qt_kernel_launches())


def colmajor(A):
    """Row-major numpy blocks (..., n, n) -> contiguous column-major complex128."""
    return np.ascontiguousarray(np.swapaxes(np.asarray(A, dtype=np.complex128), -1, -2))


def from_colmajor(buf):
    return np.swapaxes(buf, -1, -2)


def _ptr(a):
    if a is None:
        return None
    if hasattr(a, "data_ptr"):
        return C.c_void_p(a.data_ptr())
    return a.ctypes.data_as(C.c_void_p)


def _blocks(H, nk, nslab):
    """Normalise (nm,nm) | (nk,nm,nm) | (nk,nslab,nm,nm) to column-major + strides."""
    H = np.asarray(H, dtype=np.complex128)
    nm = H.shape[-1]
    nm2 = nm * nm
    if H.ndim == 2:
        return colmajor(H), 0, 0, nm
    if H.ndim == 3:
        if H.shape[0] != nk:
            raise ValueError("3-D block array must be (nk, nm, nm)")
        return colmajor(H), (nm2 if nk > 1 else 0), 0, nm
    if H.ndim == 4:
        if H.shape[0] != nk or H.shape[1] != nslab:
            raise ValueError("4-D block array must be (nk, nslab, nm, nm)")
        return colmajor(H), nslab * nm2, nm2, nm
    raise ValueError("bad block array rank")


# field order of qt_outputs
OUT_KEYS = ("tr", "tre", "T", "diag_gr", "diag_gl", "diag_gg", "G_r", "G_lesser", "G_greater",
            "status", "sancho_iters", "bond_cur", "Jdens")


def rgf_solve(ctx, Hii, H1i, E, nx, *, nk=1, mul=0.0, mur=0.0, templ=300.0, tempr=300.0,
              eta_lead=1e-5, eta_interior=0.0, sancho_tol=1e-100, sancho_max_iter=50,
              precision="fp64", caroli=False, want_diag=True, want_blocks=False,
              want_bond=False, sigma_r_ph=None, sigma_lesser_ph=None, quirks=0):
    """Batched RGF over all (E, k) points (points ordered p = ie*nk + ik).

    Returns a dict of numpy arrays: tr, tre (nE, nk); T (nE, nk) if caroli;
    diag_gr/gl/gg (nE, nk, nx, nm) if want_diag; G_r/G_lesser/G_greater and the
    bond-current blocks Jdens (nE, nk, nx, nm, nm) if want_blocks; bond_cur
    (nE, nk, nx-1), the bond currents Re Tr Jdens_l, if want_bond; status (nE, nk);
    sancho_iters (nE, nk, 2).

    ``precision``: "fp64" (FP64 pipes), "mixed" (tensor-core split products,
    complex64 sweep storage) or "mixed-fp64" (the same products with complex128
    storage, FP64-grade results).
    """
    lib = ctx._lib
    E = np.ascontiguousarray(np.asarray(E, dtype=np.float64).ravel())
    nE = E.shape[0]
    hii, hk, hl, nm = _blocks(Hii, nk, nx)
    h1i, h1k, h1l, nm1 = _blocks(H1i, nk, nx + 1)
    if nm1 != nm:
        raise ValueError("Hii and H1i block sizes differ")
    dev = QtDevice(nm, nx, nk, _ptr(hii), hk, hl, _ptr(h1i), h1k, h1l, None, 0, 0)
    con = QtContacts(mul, mur, templ, tempr, eta_lead, eta_interior, sancho_tol,
                     int(sancho_max_iter), int(quirks))
    npts = nE * nk
    res = {"tr": np.zeros(npts), "tre": np.zeros(npts),
           "status": np.zeros(npts, dtype=np.int32),
           "sancho_iters": np.zeros((npts, 2), dtype=np.int32)}
    if caroli:
        res["T"] = np.zeros(npts)
    if want_diag:
        for k in ("diag_gr", "diag_gl", "diag_gg"):
            res[k] = np.zeros((npts, nx, nm), dtype=np.complex128)
    if want_blocks:
        for k in ("G_r", "G_lesser", "G_greater") + (() if quirks & 1 else ("Jdens",)):
            res[k] = np.zeros((npts, nx, nm, nm), dtype=np.complex128)
    if want_bond:
        res["bond_cur"] = np.zeros((npts, nx - 1))
    out = QtOutputs(*[_ptr(res.get(k)) for k in OUT_KEYS])
    sr = None if sigma_r_ph is None else colmajor(sigma_r_ph)
    sl = None if sigma_lesser_ph is None else colmajor(sigma_lesser_ph)
    flags = _lib.QT_FLAG_SYNC | (_lib.QT_FLAG_CAROLI if caroli else 0)
    check(lib.qt_rgf_solve(ctx.handle, C.byref(dev), _ptr(E), nE, C.byref(con), _ptr(sr),
                           _ptr(sl), PREC[precision], flags, C.byref(out)), allow_points=True)
    for k in ("G_r", "G_lesser", "G_greater", "Jdens"):
        if k in res:
            res[k] = from_colmajor(res[k]).reshape(nE, nk, nx, nm, nm)
    for k in ("tr", "tre", "T", "status"):
        if k in res:
            res[k] = res[k].reshape(nE, nk)
    for k in ("diag_gr", "diag_gl", "diag_gg"):
        if k in res:
            res[k] = res[k].reshape(nE, nk, nx, nm)
    if want_bond:
        res["bond_cur"] = res["bond_cur"].reshape(nE, nk, nx - 1)
    res["sancho_iters"] = res["sancho_iters"].reshape(nE, nk, 2)
    return res


def pack_blocks(blocks, nk):
    """Blocks of different shapes, each (r, c) or (nk, r, c), packed column-major per block
    into one (nk, sum r c) array: returns (packed, per-block offsets, k stride)."""
    blocks = [np.asarray(b, dtype=np.complex128) for b in blocks]
    per_k = [b if b.ndim == 3 else np.broadcast_to(b, (nk,) + b.shape) for b in blocks]
    offs = np.cumsum([0] + [b.shape[1] * b.shape[2] for b in per_k])[:-1].astype(np.int64)
    kstride = int(sum(b.shape[1] * b.shape[2] for b in per_k))
    flat = np.concatenate([np.swapaxes(b, -1, -2).reshape(nk, -1) for b in per_k], axis=1)
    return np.ascontiguousarray(flat), offs, kstride


def rgf_variableblock_device(ctx, sizes, hii, hoff, h1i, h1off, nk, E, nE, out, *,
                             mul=0.0, mur=0.0, templ=300.0, tempr=300.0, eta_lead=1e-5,
                             eta_interior=0.0, sancho_tol=1e-100, sancho_max_iter=50,
                             precision="mixed", caroli=True, quirks=0, sync=False):
    """Device-pointer form of ``rgf_variableblock_forward``: ``hii``/``h1i`` torch CUDA
    tensors from ``pack_blocks`` (k stride = their second dimension), ``sizes``/``hoff``/
    ``h1off`` host numpy arrays, ``E`` a CUDA float64 tensor, ``out`` a dict of CUDA
    tensors for any of tr, tre, T, diag_gr, diag_gl, diag_gg, status, sancho_iters,
    bond_cur.  Asynchronous on ctx's stream unless ``sync``."""
    lib = ctx._lib
    sizes = np.ascontiguousarray(sizes, dtype=np.int32)
    hoff = np.ascontiguousarray(hoff, dtype=np.int64)
    h1off = np.ascontiguousarray(h1off, dtype=np.int64)
    dev = _lib.QtDeviceVB(len(sizes), nk, _ptr(sizes), _ptr(hii), _ptr(hoff),
                          hii.shape[-1] if nk > 1 else 0, _ptr(h1i), _ptr(h1off),
                          h1i.shape[-1] if nk > 1 else 0)
    con = QtContacts(mul, mur, templ, tempr, eta_lead, eta_interior, sancho_tol,
                     int(sancho_max_iter), int(quirks))
    o = QtOutputs(*[_ptr(out.get(k)) for k in OUT_KEYS])
    flags = _lib.QT_FLAG_DEVICE_POINTERS | (_lib.QT_FLAG_CAROLI if caroli else 0) | \
        (_lib.QT_FLAG_SYNC if sync else 0)
    return check(lib.qt_rgf_solve_vb(ctx.handle, C.byref(dev), _ptr(E), int(nE), C.byref(con),
                                     PREC[precision], flags, C.byref(o)), allow_points=True)


def rgf_variableblock_forward(ctx, Hii, H1i, E, *, nk=1, mul=0.0, mur=0.0, templ=300.0,
                              tempr=300.0, eta_lead=1e-5, eta_interior=0.0, sancho_tol=1e-100,
                              sancho_max_iter=50, precision="fp64", caroli=False, quirks=0,
                              want_bond=False):
    """Batched RGF over slabs of different orbital counts (rgf_variableblock_forward,
    src/rgf_mod.f90:46-269) for all (E, k) points.

    ``Hii``: nx blocks H_ll, each (n_l, n_l) or (nk, n_l, n_l).  ``H1i``: nx + 1 blocks,
    H1i[l] = H_{l,l-1} (n_l, n_{l-1}) for 1 <= l < nx, H1i[0] and H1i[nx] the leads' own
    couplings (square), each optionally per k.  Returns tr, tre (and T) (nE, nk), status,
    sancho_iters and the diagonals diag_gr / diag_gl / diag_gg as lists of nx arrays
    (nE, nk, n_l); with ``want_bond`` the bond currents bond_cur (nE, nk, nx-1).
    """
    lib = ctx._lib
    E = np.ascontiguousarray(np.asarray(E, dtype=np.float64).ravel())
    nE, nx = E.shape[0], len(Hii)
    if len(H1i) != nx + 1:
        raise ValueError("H1i needs nx + 1 blocks")
    sizes = np.array([np.shape(h)[-1] for h in Hii], dtype=np.int32)
    hii, hoff, hk = pack_blocks(Hii, nk)
    h1i, h1off, h1k = pack_blocks(H1i, nk)
    dev = _lib.QtDeviceVB(nx, nk, _ptr(sizes), _ptr(hii), _ptr(hoff), hk if nk > 1 else 0,
                          _ptr(h1i), _ptr(h1off), h1k if nk > 1 else 0)
    con = QtContacts(mul, mur, templ, tempr, eta_lead, eta_interior, sancho_tol,
                     int(sancho_max_iter), int(quirks))
    npts, dsum = nE * nk, int(sizes.sum())
    res = {"tr": np.zeros(npts), "tre": np.zeros(npts),
           "status": np.zeros(npts, dtype=np.int32),
           "sancho_iters": np.zeros((npts, 2), dtype=np.int32)}
    if caroli:
        res["T"] = np.zeros(npts)
    for k in ("diag_gr", "diag_gl", "diag_gg"):
        res[k] = np.zeros((npts, dsum), dtype=np.complex128)
    if want_bond:
        res["bond_cur"] = np.zeros((npts, nx - 1))
    out = QtOutputs(*[_ptr(res.get(k)) for k in OUT_KEYS])
    flags = _lib.QT_FLAG_SYNC | (_lib.QT_FLAG_CAROLI if caroli else 0)
    check(lib.qt_rgf_solve_vb(ctx.handle, C.byref(dev), _ptr(E), nE, C.byref(con),
                              PREC[precision], flags, C.byref(out)), allow_points=True)
    for k in ("tr", "tre", "T", "status"):
        if k in res:
            res[k] = res[k].reshape(nE, nk)
    cut = np.cumsum(sizes)[:-1]
    for k in ("diag_gr", "diag_gl", "diag_gg"):
        res[k] = [d.reshape(nE, nk, -1) for d in np.split(res[k], cut, axis=1)]
    if want_bond:
        res["bond_cur"] = res["bond_cur"].reshape(nE, nk, nx - 1)
    res["sancho_iters"] = res["sancho_iters"].reshape(nE, nk, 2)
    return res


def cuda_rgf_constblocksize(ctx, nm, nx, En, mul, mur, TEMPl, TEMPr, Hii, H1i, Sii=None,
                            sigma_lesser_ph=None, sigma_r_ph=None):
    """One point with the reference's argument list (src/cuda_rgf_mod.f90:53-59).

    Hii (nx, nm, nm), H1i (nx+1, nm, nm), optional Sii / sigmas (nx, nm, nm).
    mu/T may be scalars or the reference's constant nm x nm matrices.
    Returns (G_r, G_lesser, G_greater, Jdens, tr, tre).  Jdens[l] is the bond-current
    block H^+ G^<_{l+1,l} - H G^<_{l,l+1} (src/cuda_rgf_mod.f90:293-318); Jdens[nx-1]
    is zero, as the reference never writes it.
    """
    def scalar(x):
        x = np.asarray(x, dtype=np.float64)
        if x.ndim and not np.all(x == x.flat[0]):
            raise ValueError("mu/T matrices must be constant (src/negf_mod.f90:82-85)")
        return float(x.flat[0])

    lib = ctx._lib
    hii = colmajor(Hii)
    h1i = colmajor(H1i)
    sii = None if Sii is None else colmajor(Sii)
    sl = None if sigma_lesser_ph is None else colmajor(sigma_lesser_ph)
    sr = None if sigma_r_ph is None else colmajor(sigma_r_ph)
    Gr = np.zeros((nx, nm, nm), dtype=np.complex128)
    Gl = np.zeros_like(Gr)
    Gg = np.zeros_like(Gr)
    Jd = np.zeros_like(Gr)
    tr = C.c_double()
    tre = C.c_double()
    check(lib.qt_rgf_constblocksize(ctx.handle, nm, nx, float(En), scalar(mul), scalar(mur),
                                    scalar(TEMPl), scalar(TEMPr), _ptr(hii), _ptr(h1i), _ptr(sii),
                                    _ptr(sl), _ptr(sr), _ptr(Gr), _ptr(Gl), _ptr(Gg), _ptr(Jd),
                                    C.byref(tr), C.byref(tre)), allow_points=True)
    return (from_colmajor(Gr), from_colmajor(Gl), from_colmajor(Gg), from_colmajor(Jd),
            tr.value, tre.value)


def sancho(ctx, E, H00, H10, *, eta=1e-5, tol=1e-100, max_iter=50, precision="fp64",
           reset_on_nmax=False):
    """Batched Sancho-Rubio: E (npts,), H00/H10 (nm,nm) shared or (npts,nm,nm).

    ``reset_on_nmax`` is green_RGF_RS's variant (src/gw_mod.f90:1440-1445): a point not
    converged after ``max_iter`` steps restarts from H_SS = H_BB = H00.
    Returns (G00, GBB, iters, status) with G00/GBB (npts, nm, nm).
    """
    lib = ctx._lib
    E = np.ascontiguousarray(np.atleast_1d(np.asarray(E, dtype=np.float64)))
    npts = E.shape[0]
    H00 = np.asarray(H00, dtype=np.complex128)
    H10 = np.asarray(H10, dtype=np.complex128)
    nm = H00.shape[-1]
    h00, h10 = colmajor(H00), colmajor(H10)
    G00 = np.zeros((npts, nm, nm), dtype=np.complex128)
    GBB = np.zeros_like(G00)
    iters = np.zeros(npts, dtype=np.int32)
    status = np.zeros(npts, dtype=np.int32)
    check(lib.qt_sancho_batch(ctx.handle, nm, npts, _ptr(E), _ptr(h00), nm * nm if H00.ndim == 3 else 0,
                              _ptr(h10), nm * nm if H10.ndim == 3 else 0, None, 0, eta, tol,
                              int(max_iter), PREC[precision],
                              _lib.QT_FLAG_SANCHO_RESET if reset_on_nmax else 0, _ptr(G00),
                              _ptr(GBB), _ptr(iters),
                              _ptr(status)))
    return from_colmajor(G00), from_colmajor(GBB), iters, status


def mul_c(ctx, A, B, opA="N", opB="N", alpha=1.0, beta=0.0, D=None, precision="fp64", slices=0):
    """Batched C = alpha op(A) op(B) + beta D for (batch, n, n) arrays (or shared (n, n))."""
    lib = ctx._lib
    A = np.asarray(A, dtype=np.complex128)
    B = np.asarray(B, dtype=np.complex128)
    n = A.shape[-1]
    batch = max(A.shape[0] if A.ndim == 3 else 1, B.shape[0] if B.ndim == 3 else 1)
    a, b = colmajor(A), colmajor(B)
    d = None if D is None else colmajor(D)
    Cm = np.zeros((batch, n, n), dtype=np.complex128)
    al = np.array([complex(alpha).real, complex(alpha).imag])
    be = np.array([complex(beta).real, complex(beta).imag])
    st = lambda X: (n * n if X is not None and X.ndim == 3 else 0)
    check(lib.qt_zgemm_batch(ctx.handle, n, batch, opA.encode(), _ptr(a), st(A), opB.encode(),
                             _ptr(b), st(B), _ptr(al), _ptr(be), _ptr(d),
                             st(None if D is None else np.asarray(D)), _ptr(Cm), n * n,
                             PREC[precision], int(slices), 0))
    return from_colmajor(Cm)


def invert(ctx, A, precision="fp64"):
    """Batched block inverse of (batch, n, n); returns (X, status)."""
    lib = ctx._lib
    A = np.asarray(A, dtype=np.complex128)
    if A.ndim == 2:
        A = A[None]
    batch, n = A.shape[0], A.shape[-1]
    a = colmajor(A)
    X = np.zeros_like(a)
    status = np.zeros(batch, dtype=np.int32)
    check(lib.qt_zinv_batch(ctx.handle, n, batch, _ptr(a), n * n, _ptr(X), n * n,
                            PREC[precision], 0, _ptr(status)))
    return from_colmajor(X), status


def cell_spectra(diag, nbnd, nslab, nk_axis=1):
    """write_spectrum_summed_over_k's per-cell traces (src/output_mod.f90:37-59).

    diag: (nE, nk, nx, nm) diagonals.  Returns (nE, nx*nslab) complex traces
    averaged over k.
    """
    nE, nk, nx, nm = diag.shape
    t = diag.reshape(nE, nk, nx, nslab, nbnd).sum(axis=4).mean(axis=1)
    return t.reshape(nE, nx * nslab)


def negf_solve(ctx, Hii, H1i, nx, nen, emin, emax, temp, mu, nbnd, nslab, *, nk=1,
               precision="fp64", Lx=None, write_dir=None, **kw):
    """Ballistic NEGF driver (src/negf_mod.f90:41-165).

    Energy grid E_ie = emin + ie (emax-emin)/(nen-1) (src/negf_mod.f90:100-101).
    Returns dict with E, tr, tre (nen, nk) and the ldos/ndos/pdos spectra
    (nen, nx*nslab, 2) = (Re*c1, Im*c2) columns with the reference coefficients
    (1,-2), (1,1), (1,-1) (src/negf_mod.f90:142-149).  With ``write_dir`` (and the cell
    length ``Lx``) it also writes ldos0000.dat, ndos0000.dat and pdos0000.dat there in the
    reference's format; their paths are returned under "files".
    """
    E = emin + np.arange(nen) * ((emax - emin) / (nen - 1))
    r = rgf_solve(ctx, Hii, H1i, E, nx, nk=nk, mul=mu[0], mur=mu[1], templ=temp[0],
                  tempr=temp[1], precision=precision, **kw)
    out = {"E": E, "tr": r["tr"], "tre": r["tre"], "status": r["status"]}
    for name, key, c in (("ldos", "diag_gr", (1.0, -2.0)), ("ndos", "diag_gl", (1.0, 1.0)),
                         ("pdos", "diag_gg", (1.0, -1.0))):
        t = cell_spectra(r[key], nbnd, nslab)
        out[name] = np.stack([t.real * c[0], t.imag * c[1]], axis=-1)
    if write_dir is not None:
        from .output import write_negf_spectra
        if Lx is None:
            raise ValueError("writing the spectra needs the cell length Lx")
        out["files"] = write_negf_spectra(r, E, nbnd, nslab, Lx, directory=write_dir)
    return out


def rgf_solve_device(ctx, Hii, hk, hl, H1i, h1k, h1l, nm, nx, nk, E, nE, out, *, mul=0.0,
                     mur=0.0, templ=300.0, tempr=300.0, eta_lead=1e-5, eta_interior=0.0,
                     sancho_tol=1e-100, sancho_max_iter=50, precision="mixed", caroli=True,
                     quirks=0, sync=False):
    """Device-pointer form of ``rgf_solve`` (no host copies; asynchronous on ctx's stream).

    Hii/H1i/E: torch CUDA tensors (column-major complex128 blocks, float64
    energies); ``out``: dict of torch CUDA tensors for any of tr, tre, T,
    diag_gr, diag_gl, diag_gg, status, sancho_iters, bond_cur.  Strides in complex elements.
    Returns the status code (QT_OK or QT_ERR_POINTS when synchronised).
    """
    lib = ctx._lib
    dev = QtDevice(nm, nx, nk, _ptr(Hii), hk, hl, _ptr(H1i), h1k, h1l, None, 0, 0)
    con = QtContacts(mul, mur, templ, tempr, eta_lead, eta_interior, sancho_tol,
                     int(sancho_max_iter), int(quirks))
    o = QtOutputs(*[_ptr(out.get(k)) for k in OUT_KEYS])
    flags = _lib.QT_FLAG_DEVICE_POINTERS | (_lib.QT_FLAG_CAROLI if caroli else 0) | \
        (_lib.QT_FLAG_SYNC if sync else 0)
    return check(lib.qt_rgf_solve(ctx.handle, C.byref(dev), _ptr(E), int(nE), C.byref(con),
                                  None, None, PREC[precision], flags, C.byref(o)),
                 allow_points=True)
