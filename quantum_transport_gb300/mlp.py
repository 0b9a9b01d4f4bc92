"""Host mirror of the learned-mixing network (``qt_mlp_*`` in include/qt_rgf.h).

A multilayer perceptron n_in -> width (GELU) x depth -> n_out with BF16
weights and activations and FP32 accumulation on the tensor cores, trained
with AdamW on the mean squared error.  It has no reference counterpart: the
reference's SCBA loop mixes linearly (src/gw_mod.f90:747-749).
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import _lib
from ._lib import check


def _p(a):
    if a is None:
        return None
    if hasattr(a, "data_ptr"):
        return C.c_void_p(a.data_ptr())
    return a.ctypes.data_as(C.c_void_p)


class Mlp:
    """Network of ``depth`` GELU layers of ``width`` on the context's GPU.

    Arrays are float32, row-major: numpy (host copies) or torch CUDA tensors
    (used in place).
    """

    def __init__(self, ctx, n_in, width, depth, n_out, max_batch, params=None, seed=0):
        self.ctx = ctx
        self.dims = (n_in, width, depth, n_out)
        self.max_batch = max_batch
        self._lib = ctx._lib
        h = C.c_void_p()
        init = None if params is None else np.ascontiguousarray(params, dtype=np.float32)
        check(self._lib.qt_mlp_create(ctx.handle, n_in, width, depth, n_out, max_batch,
                                      _p(init), C.c_uint64(seed), C.byref(h)))
        self.handle = h
        n = C.c_int64()
        check(self._lib.qt_mlp_num_params(h, C.byref(n)))
        self.nparams = n.value

    def close(self):
        if self.handle:
            self._lib.qt_mlp_destroy(self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    @staticmethod
    def _flags(*arrays):
        dev = [hasattr(a, "data_ptr") for a in arrays if a is not None]
        if any(dev) and not all(dev):
            raise ValueError("mix of host and device arrays")
        return _lib.QT_FLAG_DEVICE_POINTERS if dev and dev[0] else 0

    @staticmethod
    def _host(a):
        return a if hasattr(a, "data_ptr") else np.ascontiguousarray(a, dtype=np.float32)

    def params(self):
        out = np.empty(self.nparams, dtype=np.float32)
        check(self._lib.qt_mlp_get_params(self.handle, _p(out)))
        return out

    def set_params(self, p):
        p = np.ascontiguousarray(p, dtype=np.float32)
        if p.size != self.nparams:
            raise ValueError("parameter count mismatch")
        check(self._lib.qt_mlp_set_params(self.handle, _p(p)))

    def infer(self, X, out=None):
        X = self._host(X)
        b = X.shape[0]
        if out is None:
            if hasattr(X, "data_ptr"):
                import torch
                out = torch.empty((b, self.dims[3]), dtype=torch.float32, device=X.device)
            else:
                out = np.empty((b, self.dims[3]), dtype=np.float32)
        flags = self._flags(X, out) | _lib.QT_FLAG_SYNC
        check(self._lib.qt_mlp_infer(self.handle, b, _p(X), _p(out), flags))
        return out

    def grad(self, X, T):
        """(loss, flat gradient) at the current parameters; no update."""
        X, T = self._host(X), self._host(T)
        g = np.empty(self.nparams, dtype=np.float32)
        loss = C.c_double()
        check(self._lib.qt_mlp_grad(self.handle, X.shape[0], _p(X), _p(T), _p(g),
                                    C.byref(loss), self._flags(X, T)))
        return loss.value, g

    def train_step(self, X, T, lr=1e-3, weight_decay=0.0, want_loss=True):
        """One AdamW step; returns the loss before the step (None if not wanted)."""
        X, T = self._host(X), self._host(T)
        loss = C.c_double()
        check(self._lib.qt_mlp_train_step(self.handle, X.shape[0], _p(X), _p(T), float(lr),
                                          float(weight_decay),
                                          C.byref(loss) if want_loss else None,
                                          self._flags(X, T)))
        return loss.value if want_loss else None
