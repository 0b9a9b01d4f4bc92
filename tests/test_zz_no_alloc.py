"""The allocation-free split product (qt_zgemm_batch_noalloc) against qt_zgemm_batch.

qt_zgemm_batch_noalloc serves callers that must not allocate device memory
(their device memory belongs to another allocator, or cudaMalloc's implicit
device synchronisation is not acceptable): its exponent scratch is a fixed
512-entry file-scope device array shared by all calls.  This file is collected
last so that, if it fails, a run that stops at the first failure has already
run every other test; it also passes on its own in a fresh process.
"""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

# tolerance of the split product used by tests/test_gpu_mixed.py
TOL = {4: 2.0 ** -28, 6: 2.0 ** -44, 7: 2.0 ** -50}


def _bound(A, B, opa, opb):
    op = {"N": lambda X: X, "C": lambda X: np.conj(np.swapaxes(X, -1, -2))}
    a, b = np.abs(op[opa](A)), np.abs(op[opb](B))
    return (a.max(axis=-1, keepdims=True) * b.sum(axis=-2, keepdims=True)
            + a.sum(axis=-1, keepdims=True) * b.max(axis=-2, keepdims=True))


def _timeouts(stream):
    from quantum_transport_gb300 import _lib
    lib = _lib.load()
    count = C.c_int(-1)
    _lib.check(lib.qt_noalloc_timeouts(C.byref(count), C.c_void_p(stream.cuda_stream)))
    return count.value


def _run_both(ctx, rng, n, batch, opa, opb, slices, alpha, beta, stream=None):
    import torch
    from quantum_transport_gb300 import _lib
    from quantum_transport_gb300.rgf import _ptr, colmajor, from_colmajor
    lib = _lib.load()
    A = rng.normal(size=(batch, n, n)) + 1j * rng.normal(size=(batch, n, n))
    B = rng.normal(size=(batch, n, n)) + 1j * rng.normal(size=(batch, n, n))
    D = rng.normal(size=(batch, n, n)) + 1j * rng.normal(size=(batch, n, n))
    dev = lambda X: torch.from_numpy(colmajor(X)).cuda()
    Ad, Bd, Dd = dev(A), dev(B), dev(D)
    C1 = torch.zeros_like(Ad)
    C2 = torch.zeros_like(Ad)
    al = np.array([alpha, 0.0])
    be = np.array([beta, 0.0])
    nm2 = n * n
    flags = _lib.QT_FLAG_DEVICE_POINTERS | _lib.QT_FLAG_SYNC
    _lib.check(lib.qt_zgemm_batch(ctx.handle, n, batch, opa.encode(), _ptr(Ad), nm2, opb.encode(),
                                  _ptr(Bd), nm2, _ptr(al), _ptr(be), _ptr(Dd), nm2, _ptr(C1), nm2,
                                  _lib.QT_PREC_MIXED, slices, flags))
    torch.cuda.synchronize()
    if stream is None:
        stream = torch.cuda.current_stream()
    free0 = torch.cuda.mem_get_info()[0]
    _lib.check(lib.qt_zgemm_batch_noalloc(n, batch, opa.encode(), _ptr(Ad), nm2, opb.encode(),
                                          _ptr(Bd), nm2, _ptr(al), _ptr(be), _ptr(Dd), nm2,
                                          _ptr(C2), nm2, slices, C.c_void_p(stream.cuda_stream)))
    stream.synchronize()  # only the caller's stream: the work must have gone there
    # the call allocated no device memory (the first call of the file warmed the module up)
    assert torch.cuda.mem_get_info()[0] == free0
    # no wait of the tensor-core kernel ran out, so C is complete
    assert _timeouts(stream) == 0
    c1, c2 = from_colmajor(C1.cpu().numpy()), from_colmajor(C2.cpu().numpy())
    tol = TOL[slices] * (abs(alpha) * _bound(A, B, opa, opb) + abs(beta) * np.abs(D))
    assert (np.abs(c2 - c1) <= tol).all()
    op = {"N": lambda X: X, "C": lambda X: np.conj(np.swapaxes(X, -1, -2))}
    ref = alpha * op[opa](A) @ op[opb](B) + beta * D
    assert (np.abs(c2 - ref) <= 4 * tol + 1e-14 * np.abs(ref).max()).all()


def _warm_up(ctx):
    """One small call first: under lazy module loading the first call on a device loads the
    library's device module (which may allocate), as the header documents."""
    rng = np.random.default_rng(1)
    _run_both_unchecked(ctx, rng)


def _run_both_unchecked(ctx, rng):
    import torch
    from quantum_transport_gb300 import _lib
    from quantum_transport_gb300.rgf import _ptr
    lib = _lib.load()
    X = torch.zeros(16 * 16, dtype=torch.complex128, device="cuda")
    Y = torch.zeros_like(X)
    _lib.check(lib.qt_zgemm_batch_noalloc(16, 1, b"N", _ptr(X), 256, b"N", _ptr(X), 256, None,
                                          None, None, 0, _ptr(Y), 256, 4, None))
    torch.cuda.synchronize()


def test_noalloc_matches_split_product_twice(ctx):
    _warm_up(ctx)
    rng = np.random.default_rng(77)
    # two calls in a row share the static scratch; sizes differ between them
    _run_both(ctx, rng, 96, 7, "N", "C", 4, 1.0, 0.0)
    _run_both(ctx, rng, 128, 5, "C", "N", 7, -1.0, 1.0)


def test_noalloc_on_callers_stream(ctx):
    import torch
    _warm_up(ctx)
    rng = np.random.default_rng(78)
    side = torch.cuda.Stream()
    _run_both(ctx, rng, 128, 9, "N", "N", 6, 1.0, -1.0, stream=side)
    _run_both(ctx, rng, 64, 3, "C", "C", 4, 2.0, 0.5, stream=side)


def test_noalloc_rejects_batch_over_limit(ctx):
    from quantum_transport_gb300 import _lib
    lib = _lib.load()
    dummy = C.c_void_p(1)  # never dereferenced: the size check comes first
    rc = lib.qt_zgemm_batch_noalloc(16, 513, b"N", dummy, 256, b"N", dummy, 256, None, None, None,
                                    0, dummy, 256, 4, None)
    assert rc == _lib.QT_ERR_ARG
    assert b"512" in lib.qt_last_error()
