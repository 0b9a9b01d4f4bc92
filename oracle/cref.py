"""ctypes binding of the C restatement (oracle/c/librgf_ref.so).

TEST INFRASTRUCTURE ONLY: the checker and the timed CPU baseline, never the
product path.  Build with ``make -C oracle/c`` (``__graft_entry__.build()``
does it).
"""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB = os.path.join(HERE, "c", "librgf_ref.so")
_lib = None


def build():
    import subprocess
    r = subprocess.run(["make", "-s", "-C", os.path.join(HERE, "c")], capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("oracle/c build failed:\n" + r.stderr)
    return LIB


def load():
    global _lib
    if _lib is None:
        if not os.path.exists(LIB):
            build()
        lib = C.CDLL(LIB)
        vp, ci, d = C.c_void_p, C.c_int, C.c_double
        lib.qt_ref_rgf.argtypes = [ci, ci, ci, vp, vp, ci, vp, d, d, d, ci, d, d, d, d, ci,
                                   vp, vp, vp, vp, vp, vp]
        lib.qt_ref_rgf.restype = ci
        _lib = lib
    return _lib


def rgf(H00, H10, E, nx, *, mul=0.0, mur=0.0, templ=300.0, tempr=300.0, eta_lead=1e-5,
        eta_interior=0.0, sancho_tol=1e-100, sancho_max_iter=50, threads=0, want_diag=True):
    """C restatement over points p = ie*nk + ik.  H00 (nk, nm, nm) or (nm, nm), H10 (nm, nm).

    Returns T (Caroli), tr, tre (nE, nk), diag_gr/diag_gl (nE, nk, nx, nm), status.
    """
    H00 = np.asarray(H00, dtype=np.complex128)
    if H00.ndim == 2:
        H00 = H00[None]
    nk, nm = H00.shape[0], H00.shape[-1]
    h00 = np.ascontiguousarray(np.swapaxes(H00, -1, -2))
    h10 = np.ascontiguousarray(np.asarray(H10, dtype=np.complex128).T)
    E = np.ascontiguousarray(np.asarray(E, dtype=np.float64).ravel())
    npts = E.shape[0] * nk
    out = {k: np.zeros(npts) for k in ("T", "tr", "tre")}
    out["status"] = np.zeros(npts, dtype=np.int32)
    if want_diag:
        out["diag_gr"] = np.zeros((npts, nx, nm), dtype=np.complex128)
        out["diag_gl"] = np.zeros((npts, nx, nm), dtype=np.complex128)
    p = lambda a: None if a is None else a.ctypes.data_as(C.c_void_p)
    load().qt_ref_rgf(nm, nx, nk, p(h00), p(h10), E.shape[0], p(E), eta_lead, eta_interior,
                      sancho_tol, int(sancho_max_iter), mul, mur, templ, tempr, int(threads),
                      p(out["T"]), p(out["tr"]), p(out["tre"]), p(out.get("diag_gr")),
                      p(out.get("diag_gl")), p(out["status"]))
    nE = E.shape[0]
    for k in ("T", "tr", "tre", "status"):
        out[k] = out[k].reshape(nE, nk)
    if want_diag:
        for k in ("diag_gr", "diag_gl"):
            out[k] = out[k].reshape(nE, nk, nx, nm)
    return out
