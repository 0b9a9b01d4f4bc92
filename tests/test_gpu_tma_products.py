"""The split products fed by the tensor memory accelerator, against numpy.

qt_zgemm_batch with QT_FLAG_COMPLEX64 runs the complex64 sweep's 4-digit product on
complex64 blocks: the TMA-fed kernel (one work item per product) where the operands'
addressing fits a tensor map (16-byte aligned blocks, even leading dimensions), the
register-staged kernel otherwise (odd block sizes), and tiles of <= 128 above one tile.  The error bound is that of 4
digits (2^-28 of the row / column scales) plus the complex64 rounding of the result.
The complex128 products (4, 6 and 7 digits) always qualify for tensor maps; they are
checked here with a shared operand and above one tile, and per digit count and operation
in tests/test_gpu_mixed.py.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

OP = {"N": lambda X: X, "C": lambda X: np.conj(np.swapaxes(X, -1, -2))}


def _dev(X):
    import torch
    return torch.from_numpy(
        np.ascontiguousarray(np.swapaxes(X, -1, -2)).astype(np.complex64)).cuda()


def _host(T):
    return np.swapaxes(T.cpu().numpy().astype(np.complex128), -1, -2)


def _product(ctx, A, B, D, opa, opb, alpha, beta, b_shared=False):
    import torch
    from quantum_transport_gb300 import _lib
    from quantum_transport_gb300.rgf import _ptr
    lib = ctx._lib
    n = A.shape[-1]
    batch = A.shape[0]
    Ad, Bd = _dev(A), _dev(B[:1] if b_shared else B)
    Dd = None if D is None else _dev(D)
    Cd = torch.zeros((batch, n, n), dtype=torch.complex64, device="cuda")
    al = np.array([alpha, 0.0])
    be = np.array([beta, 0.0])
    nm2 = n * n
    flags = _lib.QT_FLAG_DEVICE_POINTERS | _lib.QT_FLAG_SYNC | _lib.QT_FLAG_COMPLEX64
    _lib.check(lib.qt_zgemm_batch(ctx.handle, n, batch, opa.encode(), _ptr(Ad), nm2,
                                  opb.encode(), _ptr(Bd), 0 if b_shared else nm2, _ptr(al),
                                  _ptr(be), _ptr(Dd), nm2, _ptr(Cd), nm2, _lib.QT_PREC_MIXED, 4,
                                  flags))
    return _host(Cd)


def _bound(A, B, opa, opb):
    a, b = np.abs(OP[opa](A)), np.abs(OP[opb](B))
    return (a.max(axis=-1, keepdims=True) * b.sum(axis=-2, keepdims=True)
            + a.sum(axis=-1, keepdims=True) * b.max(axis=-2, keepdims=True))


@pytest.mark.parametrize("n", [128, 96, 64, 77, 200])
@pytest.mark.parametrize("ops", ["NN", "NC", "CN", "CC"])
def test_c64_product_vs_numpy(ctx, n, ops):
    rng = np.random.default_rng(7 * n + len(ops))
    batch = 37
    A = (rng.normal(size=(batch, n, n)) + 1j * rng.normal(size=(batch, n, n)))
    B = 1e-3 * (rng.normal(size=(batch, n, n)) + 1j * rng.normal(size=(batch, n, n)))
    D = rng.normal(size=(batch, n, n)) + 1j * rng.normal(size=(batch, n, n))
    A[:, 0, :] *= 1e4  # rows of very different magnitude
    # the product sees the complex64-rounded operands
    A, B, D = (X.astype(np.complex64).astype(np.complex128) for X in (A, B, D))
    alpha, beta = -1.0, 0.5
    got = _product(ctx, A, B, D, ops[0], ops[1], alpha, beta)
    exact = alpha * OP[ops[0]](A) @ OP[ops[1]](B) + beta * D
    # 4 digits per operand, the FP32 level-1..3 accumulator, and the complex64 result;
    # tiled sizes add one complex64 rounding of each partial sum
    tiles = -(-n // 128)
    tol = (2.0 ** -28 * _bound(A, B, ops[0], ops[1]) * tiles
           + 2.0 ** -23 * tiles * (np.abs(exact) + abs(beta) * np.abs(D)))
    err = np.abs(got - exact)
    assert (err <= tol).all(), float((err / tol).max())


def test_c64_product_shared_operand(ctx):
    """op(B) shared by every batch entry (stride 0), as H is in the sweep."""
    rng = np.random.default_rng(3)
    n, batch = 128, 300
    A = rng.normal(size=(batch, n, n)) + 1j * rng.normal(size=(batch, n, n))
    B = rng.normal(size=(1, n, n)) + 1j * rng.normal(size=(1, n, n))
    A, B = (X.astype(np.complex64).astype(np.complex128) for X in (A, B))
    for opb in ("N", "C"):
        got = _product(ctx, A, np.broadcast_to(B, A.shape), None, "N", opb, 1.0, 0.0,
                       b_shared=True)
        exact = A @ OP[opb](B)
        tol = 2.0 ** -28 * _bound(A, B, "N", opb) + 2.0 ** -23 * np.abs(exact)
        assert (np.abs(got - exact) <= tol).all()


TOL128 = {4: 2.0 ** -28, 6: 2.0 ** -44, 7: 2.0 ** -50}


@pytest.mark.parametrize("slices", [4, 6, 7])
@pytest.mark.parametrize("n,shared", [(128, True), (200, False), (77, True)])
def test_c128_product_shared_and_tiled(ctx, slices, n, shared):
    """complex128 split product with op(B) shared by all entries (stride 0) or tiled above
    128 (tiles of 100 accumulate into C), against numpy with the digit-count bound (one
    bound per K tile)."""
    from quantum_transport_gb300 import rgf
    rng = np.random.default_rng(11 * n + slices)
    batch = 24
    nb = 1 if shared else batch
    A = rng.normal(size=(batch, n, n)) + 1j * rng.normal(size=(batch, n, n))
    A[:, 1, :] *= 1e3
    B = rng.normal(size=(nb, n, n)) + 1j * rng.normal(size=(nb, n, n))
    for opa, opb in (("N", "N"), ("N", "C"), ("C", "N")):
        got = rgf.mul_c(ctx, A, B[0] if shared else B, opa, opb, precision="mixed",
                        slices=slices)
        exact = OP[opa](A) @ OP[opb](B)
        tiles = -(-n // 128)
        tol = TOL128[slices] * _bound(A, B, opa, opb) * tiles + 4e-16 * tiles * np.abs(exact)
        err = np.abs(got - exact)
        assert (err <= tol).all(), float((err / tol).max())


@pytest.mark.parametrize("kind,slices", [("c64", 4), ("c128", 4), ("c128", 6), ("c128", 7)])
def test_products_repeat_bitwise_with_beta_d(ctx, kind, slices):
    """2048 products per launch (many work items per CTA) with a beta D term give the same
    bits on every call (the 4-digit complex128 product double-buffers its accumulators)."""
    import torch
    from quantum_transport_gb300 import _lib
    from quantum_transport_gb300.rgf import _ptr
    lib = ctx._lib
    n, batch = 128, 2048
    g = torch.Generator(device="cuda").manual_seed(5)
    dt = torch.complex64 if kind == "c64" else torch.complex128
    A = torch.randn(batch, n, n, dtype=dt, device="cuda", generator=g)
    B = 1e-3 * torch.randn(batch, n, n, dtype=dt, device="cuda", generator=g)
    D = torch.randn(batch, n, n, dtype=dt, device="cuda", generator=g)
    one = np.array([1.0, 0.0])
    flags = _lib.QT_FLAG_DEVICE_POINTERS | _lib.QT_FLAG_SYNC | (
        _lib.QT_FLAG_COMPLEX64 if kind == "c64" else 0)
    outs = []
    for _ in range(4):
        C = torch.zeros_like(A)
        _lib.check(lib.qt_zgemm_batch(ctx.handle, n, batch, b"N", _ptr(A), n * n, b"N", _ptr(B),
                                      n * n, _ptr(one), _ptr(one), _ptr(D), n * n, _ptr(C), n * n,
                                      _lib.QT_PREC_MIXED, slices, flags))
        outs.append(C)
    assert all(torch.equal(outs[0], o) for o in outs[1:])


@pytest.mark.parametrize("kind,slices", [("c64", 4), ("c128", 4), ("c128", 6), ("c128", 7)])
def test_raw_slot_reuse_repeats_bitwise(ctx, kind, slices):
    """88 x 88 x 88 products (11 k-chunks per item, so the ring of TMA slots wraps inside
    items) repeated 24 times: every repeat equals the first bit for bit, and the first is
    within the digit bound of numpy.  Without a proxy fence between the producers' reads of
    a slot and its release to the next tensor copy, about one 6-digit launch in five here
    read a refilled slot."""
    import torch
    from quantum_transport_gb300 import _lib
    from quantum_transport_gb300.rgf import _ptr
    lib = ctx._lib
    n, batch = 88, 256
    g = torch.Generator(device="cuda").manual_seed(11)
    dt = torch.complex64 if kind == "c64" else torch.complex128
    A = torch.randn(batch, n, n, dtype=dt, device="cuda", generator=g)
    B = torch.randn(batch, n, n, dtype=dt, device="cuda", generator=g)
    one, zero = np.array([1.0, 0.0]), np.array([0.0, 0.0])
    flags = _lib.QT_FLAG_DEVICE_POINTERS | _lib.QT_FLAG_SYNC | (
        _lib.QT_FLAG_COMPLEX64 if kind == "c64" else 0)
    outs = []
    for _ in range(24):
        C = torch.zeros_like(A)
        _lib.check(lib.qt_zgemm_batch(ctx.handle, n, batch, b"N", _ptr(A), n * n, b"N", _ptr(B),
                                      n * n, _ptr(one), _ptr(zero), None, 0, _ptr(C), n * n,
                                      _lib.QT_PREC_MIXED, slices, flags))
        outs.append(C)
    assert all(torch.equal(outs[0], o) for o in outs[1:])
    # device blocks are column-major: the stored transpose of each operand
    Ah = _host(A.to(torch.complex64) if kind == "c64" else A)
    Bh = _host(B.to(torch.complex64) if kind == "c64" else B)
    got = _host(outs[0])
    exact = Ah @ Bh
    # the digit bound, the rounding of the result, and numpy's own FP64 rounding of the
    # reference (n terms, comparable to the 7-digit bound)
    tol = (TOL128.get(slices, 2.0 ** -28) * _bound(Ah, Bh, "N", "N")
           + (2.0 ** -23 if kind == "c64" else 4e-16) * np.abs(exact)
           + 2 * n * 2.0 ** -53 * (np.abs(Ah) @ np.abs(Bh)))
    assert (np.abs(got - exact) <= tol).all()
