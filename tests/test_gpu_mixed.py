"""Split-precision (tcgen05 Ozaki-digit) path against FP64 references."""
import numpy as np
import pytest

from oracle import rgf as orc
from quantum_transport_gb300 import rgf
from quantum_transport_gb300.devices import make_chain_device
from tests.goldutil import printed_match

pytestmark = pytest.mark.gpu

# S digits keep 8S-1 bits of each operand row (column) relative to its largest entry, and
# every digit level is accumulated exactly, so the error of C_ij is bounded by
#   2^(4-8S) * (max_k |A_ik| sum_k |B_kj| + sum_k |A_ik| max_k |B_kj|)
TOL = {4: 2.0 ** -28, 6: 2.0 ** -44, 7: 2.0 ** -50}


def rand_blocks(rng, b, n, scale=1.0):
    return scale * (rng.normal(size=(b, n, n)) + 1j * rng.normal(size=(b, n, n)))


@pytest.mark.parametrize("slices", [4, 6, 7])
@pytest.mark.parametrize("n", [16, 33, 96, 128])
@pytest.mark.parametrize("ops", ["NN", "NC", "CN", "CC"])
def test_zgemm_split(ctx, slices, n, ops):
    rng = np.random.default_rng(100 * n + slices)
    A = rand_blocks(rng, 3, n)
    B = rand_blocks(rng, 3, n, scale=1e-3)  # scales differ per operand
    A[:, 0, :] *= 1e4                       # rows of very different magnitude
    op = {"N": lambda X: X, "C": lambda X: np.conj(np.swapaxes(X, -1, -2))}
    C = rgf.mul_c(ctx, A, B, ops[0], ops[1], precision="mixed", slices=slices)
    ref = op[ops[0]](A) @ op[ops[1]](B)
    a, b = np.abs(op[ops[0]](A)), np.abs(op[ops[1]](B))
    bound = (a.max(axis=-1, keepdims=True) * b.sum(axis=-2, keepdims=True)
             + a.sum(axis=-1, keepdims=True) * b.max(axis=-2, keepdims=True))
    err = np.abs(C - ref)
    assert (err <= TOL[slices] * bound).all(), (err / bound).max()


def test_zgemm_split_alpha_beta(ctx):
    rng = np.random.default_rng(9)
    n = 64
    A, B, D = rand_blocks(rng, 2, n), rand_blocks(rng, 2, n), rand_blocks(rng, 2, n)
    C = rgf.mul_c(ctx, A, B, "N", "C", alpha=-1.0, beta=1.0, D=D, precision="mixed", slices=7)
    ref = -A @ np.conj(np.swapaxes(B, -1, -2)) + D
    np.testing.assert_allclose(C, ref, rtol=0, atol=1e-12 * np.abs(ref).max())


def test_zinv_split(ctx):
    rng = np.random.default_rng(3)
    A = rand_blocks(rng, 5, 96) + 4 * np.eye(96)
    X, st = rgf.invert(ctx, A, precision="mixed")
    assert (st == 0).all()
    np.testing.assert_allclose(X @ A, np.broadcast_to(np.eye(96), A.shape), atol=1e-12)


def test_sancho_split_cnt_golden(ctx, cnt):
    """FP64-grade digits reproduce the reference's lead traces (file precision ~1e-12)."""
    idx = np.arange(0, 200, 7)
    E = cnt["E"][idx]
    for j, h in enumerate((cnt["H10"].conj().T, cnt["H10"])):
        G00, GBB, it, st = rgf.sancho(ctx, E, cnt["H00"], h, precision="mixed")
        assert (st == 0).all()
        # same sensitivity as the FP64 path at a few energies (see test_gpu_fp64)
        np.testing.assert_allclose(-np.trace(G00, axis1=1, axis2=2).imag,
                                   cnt["sancho_g00"][idx, j], rtol=5e-8)


def _cnt_negf(ctx, cnt, precision):
    return rgf.negf_solve(ctx, cnt["H00"], cnt["H10"], int(cnt["nx"]), 200, -6.0, -1.0,
                          (300.0, 300.0), (-3.7, -3.7), int(cnt["nb"]), int(cnt["ns"]),
                          precision=precision)


def test_rgf_split_fp64grade_cnt_golden(ctx, cnt):
    """The test_cnt run through the complex128 split path (6-digit tensor-core products,
    refined FP32 inverses): every cell of ldos/ndos/pdos0000.dat to the printed digit, or
    within 1e-8 of the column maximum.  The floor covers cells whose value is itself only
    ~1e-6 of the maximum: there the FP64 path and the LAPACK oracle already differ by
    6e-10 of the maximum, and this path by 1.4e-9 (band edge at -3.8 eV, lead eta 1e-5)."""
    r = _cnt_negf(ctx, cnt, "mixed-fp64")
    assert (r["status"] == 0).all()
    for name, col in (("ldos", 0), ("ldos", 1), ("ndos", 1), ("pdos", 1)):
        gold = cnt[name][:, :, col]
        ok = printed_match(r[name][:, :, col], gold, full=gold)
        ok |= np.abs(r[name][:, :, col] - gold) <= 1e-8 * np.abs(gold).max()
        assert ok.all(), (name, col, np.argwhere(~ok)[:5])


# The complex64 sweep stores H and every block to 2^-24 relative.  Near the band edge at
# -3.8 eV (interior eta = 0, lead eta = 1e-5) the inverted blocks reach a condition number of
# 2.3e5.  There, against the FP64 oracle, this path moves Re Tr G by up to 6.6e-5 and
# -Im Tr G by 5.4e-5 of the column maximum (measured on GB300).  A numpy emulation of
# complex64 storage with exact inverses gives 6.3e-5 for Re Tr G.  Each cell must round to
# the printed digits (2 units) or lie within these floors, about 3x above the measurement.
C64_FLOOR = {("ldos", 0): 2e-4, ("ldos", 1): 1.5e-4, ("ndos", 1): 1.5e-4, ("pdos", 1): 1.5e-4}


def test_rgf_split_cnt_golden(ctx, cnt):
    """The test_cnt run through the complex64 split path, within its storage resolution."""
    r = _cnt_negf(ctx, cnt, "mixed")
    assert (r["status"] == 0).all()
    for (name, col), floor in C64_FLOOR.items():
        gold = cnt[name][:, :, col]
        mine = r[name][:, :, col]
        ok = printed_match(mine, gold, full=gold, units=2.0)
        ok |= np.abs(mine - gold) <= floor * np.abs(gold).max()
        assert ok.all(), (name, col, np.argwhere(~ok)[:5])


@pytest.mark.parametrize("eta_lead", [1e-5, 1e-3])
def test_rgf_split_fp64grade_vs_fp64(ctx, eta_lead):
    """The complex128 split path agrees with the FP64 pipes to FP64 grade: T(E) to 1e-10.
    The diagonals are compared at eta = 1e-3 with a bound of 2e-8 of the maximum.  On this
    device two FP64 orderings already differ in diag G^R: the C restatement (Gauss-Jordan) and
    the LAPACK oracle by 2.3e-9 at eta = 1e-3, and the FP64 pipes and the oracle by 3e-8 at
    1e-5.  The bound is 10x the former."""
    dev = make_chain_device(24, 64, 16, -2.0, 2.0, seed=2024, nk=4)
    kw = dict(nk=dev.nk, mul=0.1, mur=-0.1, templ=290.1, tempr=290.1, sancho_tol=1e-10,
              caroli=True, eta_lead=eta_lead)
    r64 = rgf.rgf_solve(ctx, dev.H00, dev.H10, dev.E, dev.nx, **kw)
    rhi = rgf.rgf_solve(ctx, dev.H00, dev.H10, dev.E, dev.nx, precision="mixed-fp64", **kw)
    assert (rhi["status"] == 0).all()
    rel = np.abs(rhi["T"] - r64["T"]) / np.abs(r64["T"])
    assert rel.max() <= 1e-10, rel.max()
    if eta_lead == 1e-3:
        for key in ("diag_gr", "diag_gl", "tr", "tre"):
            err = np.abs(rhi[key] - r64[key]).max() / np.abs(r64[key]).max()
            assert err <= 2e-8, (key, err)


def test_rgf_split_vs_fp64_transmission(ctx):
    """T(E) of the split path within 1e-6 (relative) of the FP64 path."""
    dev = make_chain_device(24, 64, 16, -2.0, 2.0, seed=2024, nk=4)
    kw = dict(nk=dev.nk, mul=0.1, mur=-0.1, templ=290.1, tempr=290.1, sancho_tol=1e-10,
              caroli=True)
    r64 = rgf.rgf_solve(ctx, dev.H00, dev.H10, dev.E, dev.nx, **kw)
    rmx = rgf.rgf_solve(ctx, dev.H00, dev.H10, dev.E, dev.nx, precision="mixed", **kw)
    assert (rmx["status"] == 0).all()
    rel = np.abs(rmx["T"] - r64["T"]) / np.abs(r64["T"])
    assert rel.max() <= 1e-6, rel.max()
    for key in ("diag_gr", "diag_gl"):
        err = np.abs(rmx[key] - r64[key]).max() / np.abs(r64[key]).max()
        assert err <= 1e-5, (key, err)


def test_split_tiny_fermi_factors(ctx):
    """mu about 2 eV below the energies: occupations f from 4e-31 down to 1e-37, so the
    rows of Sigma^< and G^< sit near FP32's smallest normal numbers.  Their digit scale
    2^(8-e) must not overflow: every output stays finite (this produced NaN before the
    scale was split).  Complex64 storage keeps its relative accuracy while G^< is above
    ~1e-33; below that its values approach FP32's subnormal range, where a row whose
    largest entry is subnormal is flushed, and only the complex128 paths resolve them."""
    dev = make_chain_device(8, 32, 8, -2.4, -2.0, seed=77, nk=2)
    kw = dict(nk=dev.nk, mul=-4.2, mur=-4.2, sancho_tol=1e-10, caroli=True)
    r64 = rgf.rgf_solve(ctx, dev.H00, dev.H10, dev.E, dev.nx, **kw)
    for precision, floor in (("mixed", 1e-33), ("mixed-fp64", 0.0)):
        r = rgf.rgf_solve(ctx, dev.H00, dev.H10, dev.E, dev.nx, precision=precision, **kw)
        assert (r["status"] == 0).all()
        a, b = r["diag_gl"], r64["diag_gl"]
        assert np.isfinite(a).all()
        scale = np.abs(b).max(axis=(2, 3), keepdims=True)   # per (E, k)
        assert scale.min() > 0 and scale.max() < 1e-28
        resolved = np.broadcast_to(scale >= floor, a.shape)
        # complex128 path: diagonals at lead eta 1e-5 are conditioned at ~3e-8 (see
        # test_rgf_split_fp64grade_vs_fp64), independent of how small f is
        tol = 1e-4 if precision == "mixed" else 3e-7
        assert resolved.any()
        assert (np.abs(a - b) <= tol * scale)[resolved].all(), precision
