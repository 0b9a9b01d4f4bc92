"""ctypes binding of libqtgpu.so (include/qt_rgf.h).

The library is built in-tree by ``quantum_transport_gb300.build``.  There is
no CPU fallback: if the shared library is missing or cannot be loaded, every
entry point raises.
"""
from __future__ import annotations

import ctypes as C
import os

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "libqtgpu.so")

QT_OK, QT_ERR_ARG, QT_ERR_CUDA, QT_ERR_NOMEM, QT_ERR_UNSUPPORTED, QT_ERR_POINTS = range(6)
QT_PREC_FP64, QT_PREC_MIXED, QT_PREC_MIXED_FP64 = 0, 1, 2
QT_FLAG_DEVICE_POINTERS, QT_FLAG_CAROLI, QT_FLAG_SYNC, QT_FLAG_SANCHO_RESET = 1, 2, 4, 8
QT_FLAG_COMPLEX64 = 16
QT_QUIRK_CPU_FERMI, QT_QUIRK_GLP_ZERO, QT_QUIRK_BACK_H1I_NEXT = 1, 2, 4
QT_QUIRK_GW_SANCHO_RESET = 8
QT_FLAG_V_PER_SLAB = 32
QT_PT_SINGULAR, QT_PT_SANCHO_NOT_CONVERGED, QT_PT_NONFINITE = 1, 2, 4

# every symbol include/qt_rgf.h declares
EXPORTS = [
    "qt_ctx_create", "qt_ctx_destroy", "qt_ctx_sync", "qt_ctx_set_scratch_limit",
    "qt_last_error", "qt_version", "qt_rgf_solve", "qt_rgf_constblocksize",
    "qt_sancho_batch", "qt_zgemm_batch", "qt_zinv_batch", "qt_kernel_launches",
    "qt_ctx_profile", "qt_ctx_profile_read", "qt_ctx_stream", "qt_gw_step", "qt_scba_solve",
    "qt_corr_batch", "qt_zgemm_batch_noalloc", "qt_noalloc_timeouts",
    "qt_mlp_create", "qt_mlp_destroy", "qt_mlp_num_params", "qt_mlp_get_params",
    "qt_mlp_set_params", "qt_mlp_infer", "qt_mlp_grad", "qt_mlp_train_step",
    "qt_mix_diag", "qt_mix_features", "qt_mix_apply", "qt_mix_gram", "qt_mix_combine",
    "qt_rgf_solve_vb", "qt_ctx_set_stream", "qt_w90_blocks", "qt_coo_blocks",
    "qt_ephoton_sigma", "qt_ctx_inverse_fallbacks", "qt_gw_polarization", "qt_gw_screened",
    "qt_gw_selfenergy", "qt_gw_sigma_post", "qt_ctx_set_wave_points", "qt_ctx_set_gw_grid",
]


class QtDevice(C.Structure):
    _fields_ = [("nm", C.c_int), ("nx", C.c_int), ("nk", C.c_int),
                ("Hii", C.c_void_p), ("hii_kstride", C.c_int64), ("hii_lstride", C.c_int64),
                ("H1i", C.c_void_p), ("h1i_kstride", C.c_int64), ("h1i_lstride", C.c_int64),
                ("Sii", C.c_void_p), ("sii_kstride", C.c_int64), ("sii_lstride", C.c_int64)]


class QtDeviceVB(C.Structure):
    _fields_ = [("nx", C.c_int), ("nk", C.c_int), ("nm", C.c_void_p),
                ("Hii", C.c_void_p), ("hii_off", C.c_void_p), ("hii_kstride", C.c_int64),
                ("H1i", C.c_void_p), ("h1i_off", C.c_void_p), ("h1i_kstride", C.c_int64)]


class QtContacts(C.Structure):
    _fields_ = [("mul", C.c_double), ("mur", C.c_double), ("templ", C.c_double),
                ("tempr", C.c_double), ("eta_lead", C.c_double), ("eta_interior", C.c_double),
                ("sancho_tol", C.c_double), ("sancho_max_iter", C.c_int), ("quirks", C.c_uint)]


class QtOutputs(C.Structure):
    _fields_ = [(n, C.c_void_p) for n in ("tr", "tre", "T", "diag_gr", "diag_gl", "diag_gg",
                                          "G_r", "G_lesser", "G_greater", "status",
                                          "sancho_iters", "bond_cur", "Jdens")]


class QtError(RuntimeError):
    def __init__(self, code, msg):
        super().__init__(f"qt status {code}: {msg}")
        self.code = code


_lib = None


def load(path=LIB_PATH):
    """Load libqtgpu.so (raises if absent: the CUDA path has no fallback)."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(path):
        raise QtError(-1, f"{path} not built; run quantum_transport_gb300.build.build()")
    lib = C.CDLL(path)
    vp, i64, dbl, ci = C.c_void_p, C.c_int64, C.c_double, C.c_int
    lib.qt_ctx_create.argtypes = [C.POINTER(vp), ci]
    lib.qt_ctx_destroy.argtypes = [vp]
    lib.qt_ctx_sync.argtypes = [vp]
    lib.qt_ctx_set_scratch_limit.argtypes = [vp, i64]
    lib.qt_ctx_set_wave_points.argtypes = [vp, i64]
    lib.qt_ctx_set_gw_grid.argtypes = [vp, ci, ci, ci]
    lib.qt_ctx_set_stream.argtypes = [vp, vp, ci]
    lib.qt_ctx_inverse_fallbacks.argtypes = [vp, C.POINTER(i64), ci]
    lib.qt_w90_blocks.argtypes = [vp, ci, ci, vp, vp, vp, ci, vp, vp, vp, C.c_uint]
    lib.qt_coo_blocks.argtypes = [vp, ci, ci, C.c_longlong, vp, vp, ci, vp, vp, vp, vp, vp, C.c_uint]
    lib.qt_last_error.restype = C.c_char_p
    lib.qt_version.restype = C.c_char_p
    lib.qt_rgf_solve.argtypes = [vp, C.POINTER(QtDevice), vp, ci, C.POINTER(QtContacts), vp, vp,
                                 ci, C.c_uint, C.POINTER(QtOutputs)]
    lib.qt_rgf_constblocksize.argtypes = [vp, ci, ci, dbl, dbl, dbl, dbl, dbl] + [vp] * 9 + [vp, vp]
    lib.qt_sancho_batch.argtypes = [vp, ci, ci, vp, vp, i64, vp, i64, vp, i64, dbl, dbl, ci, ci,
                                    C.c_uint, vp, vp, vp, vp]
    lib.qt_zgemm_batch.argtypes = [vp, ci, ci, C.c_char, vp, i64, C.c_char, vp, i64, vp, vp, vp,
                                   i64, vp, i64, ci, ci, C.c_uint]
    lib.qt_zinv_batch.argtypes = [vp, ci, ci, vp, i64, vp, i64, ci, C.c_uint, vp]
    lib.qt_kernel_launches.argtypes = []
    lib.qt_kernel_launches.restype = C.c_int64
    lib.qt_ctx_profile.argtypes = [vp, ci]
    lib.qt_ctx_profile_read.argtypes = [vp, ci, C.POINTER(C.c_int64), C.POINTER(dbl),
                                        C.POINTER(dbl), C.POINTER(dbl)]
    lib.qt_ctx_stream.argtypes = [vp, C.POINTER(vp)]
    lib.qt_gw_step.argtypes = [vp, C.POINTER(QtDevice), vp, ci, C.POINTER(QtContacts), vp, dbl,
                               ci, C.c_uint, vp, vp, vp, vp, vp]
    lib.qt_scba_solve.argtypes = [vp, C.POINTER(QtDevice), vp, ci, C.POINTER(QtContacts), vp,
                                  dbl, dbl, dbl, ci, ci, C.c_uint, vp, vp, vp, vp, vp, vp]
    lib.qt_corr_batch.argtypes = [vp, ci, i64, vp, vp, vp, ci, C.c_uint]
    lib.qt_gw_polarization.argtypes = [vp, ci, i64, vp, vp, vp, vp, vp, dbl, vp, vp, vp,
                                       C.c_uint]
    lib.qt_gw_screened.argtypes = [vp, ci, i64, vp, vp, vp, vp, vp, vp, vp, ci, C.c_uint]
    lib.qt_gw_selfenergy.argtypes = [vp, ci, i64, vp, vp, vp, vp, vp, vp, dbl, vp, vp, vp,
                                     C.c_uint]
    lib.qt_gw_sigma_post.argtypes = [vp, ci, ci, ci, vp, vp, vp, C.c_uint]
    lib.qt_ephoton_sigma.argtypes = [vp, ci, ci, ci, ci, ci, vp, vp, vp, dbl, ci, C.c_uint, vp, vp,
                                     vp]
    lib.qt_zgemm_batch_noalloc.argtypes = [ci, ci, C.c_char, vp, i64, C.c_char, vp, i64, vp, vp,
                                           vp, i64, vp, i64, ci, vp]
    lib.qt_noalloc_timeouts.argtypes = [C.POINTER(ci), vp]
    flt = C.c_float
    lib.qt_mlp_create.argtypes = [vp, ci, ci, ci, ci, ci, vp, C.c_uint64, C.POINTER(vp)]
    lib.qt_mlp_destroy.argtypes = [vp]
    lib.qt_mlp_num_params.argtypes = [vp, C.POINTER(C.c_int64)]
    lib.qt_mlp_get_params.argtypes = [vp, vp]
    lib.qt_mlp_set_params.argtypes = [vp, vp]
    lib.qt_mlp_infer.argtypes = [vp, ci, vp, vp, C.c_uint]
    lib.qt_mlp_grad.argtypes = [vp, ci, vp, vp, vp, C.POINTER(dbl), C.c_uint]
    lib.qt_mlp_train_step.argtypes = [vp, ci, vp, vp, flt, flt, C.POINTER(dbl), C.c_uint]
    pvp = C.POINTER(vp)
    lib.qt_rgf_solve_vb.argtypes = [vp, C.POINTER(QtDeviceVB), vp, ci, C.POINTER(QtContacts), ci,
                                    C.c_uint, C.POINTER(QtOutputs)]
    lib.qt_mix_diag.argtypes = [vp, ci, ci, ci, vp, vp, vp, C.c_uint]
    lib.qt_mix_features.argtypes = [vp, ci, i64, ci, vp, vp, dbl, vp, C.c_uint]
    lib.qt_mix_apply.argtypes = [vp, ci, ci, ci, vp, ci, dbl, dbl, dbl, vp, vp, vp, vp, C.c_uint]
    lib.qt_mix_gram.argtypes = [vp, i64, ci, pvp, pvp, vp]
    lib.qt_mix_combine.argtypes = [vp, i64, ci, vp, pvp, pvp, dbl, vp, C.c_uint]
    for name in EXPORTS:
        f = getattr(lib, name)
        if name not in ("qt_last_error", "qt_version", "qt_kernel_launches"):
            f.restype = C.c_int
    _lib = lib
    return lib


def check(code, allow_points=False):
    if code == QT_OK or (allow_points and code == QT_ERR_POINTS):
        return code
    raise QtError(code, load().qt_last_error().decode())
