"""FP64 CUDA path against the oracle and the reference's known answers."""
import numpy as np
import pytest

from oracle import rgf as orc
from quantum_transport_gb300 import rgf
from quantum_transport_gb300.devices import make_chain_device
from tests.goldutil import printed_match

pytestmark = pytest.mark.gpu


def rand_blocks(rng, b, n):
    return rng.normal(size=(b, n, n)) + 1j * rng.normal(size=(b, n, n))


@pytest.mark.parametrize("n", [16, 33, 96, 128])
@pytest.mark.parametrize("ops", ["NN", "NC", "CN", "CC", "TN"])
def test_zgemm_f64(ctx, n, ops):
    rng = np.random.default_rng(n)
    A, B, D = rand_blocks(rng, 3, n), rand_blocks(rng, 3, n), rand_blocks(rng, 3, n)
    op = {"N": lambda X: X, "C": lambda X: np.conj(np.swapaxes(X, -1, -2)),
          "T": lambda X: np.swapaxes(X, -1, -2)}
    al, be = 0.7 - 0.2j, -1.3 + 0.4j
    C = rgf.mul_c(ctx, A, B, ops[0], ops[1], al, be, D)
    ref = al * op[ops[0]](A) @ op[ops[1]](B) + be * D
    np.testing.assert_allclose(C, ref, rtol=0, atol=1e-12 * np.abs(ref).max())


def test_zgemm_f64_shared_operand(ctx):
    rng = np.random.default_rng(5)
    A = rand_blocks(rng, 1, 40)[0]
    B = rand_blocks(rng, 4, 40)
    C = rgf.mul_c(ctx, A, B)
    np.testing.assert_allclose(C, A[None] @ B, atol=1e-11)


@pytest.mark.parametrize("n", [8, 32, 96, 128])
def test_zinv_f64(ctx, n):
    rng = np.random.default_rng(n)
    A = rand_blocks(rng, 4, n) + 3 * np.eye(n)
    X, st = rgf.invert(ctx, A)
    assert (st == 0).all()
    np.testing.assert_allclose(X @ A, np.broadcast_to(np.eye(n), A.shape), atol=1e-10)


def test_zinv_singular_flags_point(ctx):
    A = np.zeros((3, 16, 16), dtype=complex)
    A[0] = np.eye(16)
    A[2] = np.eye(16)
    A[2][:, 5] = 0  # rank deficient
    X, st = rgf.invert(ctx, A)
    assert st[0] == 0 and st[1] & 1 and st[2] & 1
    np.testing.assert_allclose(X[0], np.eye(16))


def test_sancho_cnt_golden(ctx, cnt):
    """GPU decimation reproduces test_cnt/sancho_g00.dat and sancho_gbb.dat."""
    E = cnt["E"]
    H00, H10 = cnt["H00"], cnt["H10"]
    for j, h in enumerate((H10.conj().T, H10)):
        G00, GBB, it, st = rgf.sancho(ctx, E, H00, h)
        assert (st == 0).all()
        # the 50-step decimation amplifies rounding differences between this
        # Gauss-Jordan inverse and the reference's LU: a few energies agree to ~1e-8
        np.testing.assert_allclose(-np.trace(G00, axis1=1, axis2=2).imag, cnt["sancho_g00"][:, j],
                                   rtol=5e-8)
        np.testing.assert_allclose(-np.trace(GBB, axis1=1, axis2=2).imag, cnt["sancho_gbb"][:, j],
                                   rtol=5e-8)


def test_rgf_cnt_golden_all_energies(ctx, cnt):
    """The full test_cnt run (200 energies, nx=5, nm=96): ldos/ndos/pdos0000.dat."""
    nx = int(cnt["nx"])
    r = rgf.negf_solve(ctx, cnt["H00"], cnt["H10"], nx, 200, -6.0, -1.0, (300.0, 300.0),
                       (-3.7, -3.7), int(cnt["nb"]), int(cnt["ns"]))
    assert (r["status"] == 0).all()
    for name in ("ldos", "ndos", "pdos"):
        for col in (0, 1):
            if name != "ldos" and col == 0:
                continue  # Re Tr G^< / G^> is pure round-off in the reference
            # G^> = G^< + (G - G^+) (and G^< in the tail above mu) is a difference of order-one
            # terms, and the eta = 1e-5 decimation amplifies rounding ~1e7: entries below
            # 1e-8 of the column maximum are round-off in either code's operation order
            floor = 1e-10 if name == "ldos" else 1e-8
            ok = printed_match(r[name][:, :, col], cnt[name][:, :, col], full=cnt[name][:, :, col],
                               rel_floor=floor)
            assert ok.all(), (name, col, np.argwhere(~ok)[:5])


@pytest.mark.parametrize("quirks", [0, 1, 2, 4])
def test_rgf_vs_oracle_blocks(ctx, quirks):
    dev = make_chain_device(6, 20, 5, -2.5, 2.5, seed=7, nk=2)
    qmap = {0: orc.QUIRKS_GOLDEN, 1: orc.QUIRKS_CPU, 2: orc.QUIRKS_CUDA,
            4: dict(orc.QUIRKS_GOLDEN, back_coupling="next")}
    mu = (0.1, -0.1)
    # eta_lead = 1e-3 (the GW variant's lead broadening): with the ballistic 1e-5 the
    # decimation is so ill-conditioned that two FP64 orderings (LAPACK LU vs Gauss-Jordan)
    # already differ by ~2e-6 at some energies, far above this test's 1e-9 tolerance
    r = rgf.rgf_solve(ctx, dev.H00, dev.H10, dev.E, dev.nx, nk=dev.nk, mul=mu[0], mur=mu[1],
                      templ=300.0, tempr=280.0, want_blocks=True, quirks=quirks, eta_lead=1e-3)
    assert (r["status"] == 0).all()
    for ie in range(len(dev.E)):
        for ik in range(dev.nk):
            Hii = [dev.H00[ik]] * dev.nx
            H1i = [dev.H10] * (dev.nx + 1)
            o = orc.rgf_constblocksize(dev.E[ie], Hii, H1i, mul=mu[0], mur=mu[1], templ=300.0,
                                       tempr=280.0, quirks=qmap[quirks], eta_lead=1e-3)
            for key, okey in (("G_r", "G_r"), ("G_lesser", "G_lesser"), ("G_greater", "G_greater")):
                got = r[key][ie, ik]
                exp = np.stack(o[okey])
                np.testing.assert_allclose(got, exp, rtol=0, atol=1e-8 * np.abs(exp).max() + 1e-14)
            np.testing.assert_allclose(r["tr"][ie, ik], o["tr"], rtol=1e-8, atol=1e-12)
            np.testing.assert_allclose(r["tre"][ie, ik], o["tre"], rtol=1e-8, atol=1e-12)


def test_caroli_vs_oracle(ctx):
    dev = make_chain_device(8, 24, 6, -2.0, 2.0, seed=11, nk=1)
    # a barrier in the middle slabs makes T non-trivial
    Hii = np.stack([dev.H00[0] + (0.8 * np.eye(24) if 3 <= l <= 4 else 0) for l in range(dev.nx)])
    r = rgf.rgf_solve(ctx, Hii[None], dev.H10, dev.E, dev.nx, caroli=True)
    for ie, E in enumerate(dev.E):
        t = orc.caroli_transmission(E, list(Hii), [dev.H10] * (dev.nx + 1))
        np.testing.assert_allclose(r["T"][ie, 0], t, rtol=1e-8)


def test_constblocksize_dropin(ctx, cnt):
    """The single-point entry point with cuda_rgf_constblocksize's argument list."""
    nx, nm = 5, cnt["H00"].shape[0]
    Hii = np.stack([cnt["H00"]] * nx)
    H1i = np.stack([cnt["H10"]] * (nx + 1))
    mu = np.full((nm, nm), -3.7)
    T = np.full((nm, nm), 300.0)
    E = cnt["E"][120]
    Gr, Gl, Gg, Jd, tr, tre = rgf.cuda_rgf_constblocksize(ctx, nm, nx, E, mu, mu, T, T, Hii, H1i,
                                                          np.stack([np.eye(nm)] * nx))
    o = orc.rgf_constblocksize(E, list(Hii), list(H1i), mul=-3.7, mur=-3.7)
    np.testing.assert_allclose(Gr, np.stack(o["G_r"]), atol=1e-9 * np.abs(Gr).max())
    np.testing.assert_allclose(Gl, np.stack(o["G_lesser"]), atol=1e-9 * np.abs(Gl).max() + 1e-30)
    np.testing.assert_allclose(tr, o["tr"], atol=1e-9)


def test_minimum_device_and_odd_sizes(ctx):
    dev = make_chain_device(2, 7, 3, -1.0, 1.0, seed=3)
    r = rgf.rgf_solve(ctx, dev.H00, dev.H10, dev.E, 2, caroli=True)
    for ie, E in enumerate(dev.E):
        o = orc.rgf_constblocksize(E, [dev.H00[0]] * 2, [dev.H10] * 3, mul=0.0, mur=0.0)
        np.testing.assert_allclose(r["diag_gr"][ie, 0], np.stack([np.diag(x) for x in o["G_r"]]),
                                   atol=1e-10)


@pytest.mark.parametrize("precision", ["fp64", "mixed-fp64", "mixed"])
def test_one_chain_leads_single_decimation(ctx, precision):
    """Equal leads (every slab and coupling alike, no scattering self-energy) take one
    dual-surface decimation; a zero scattering self-energy forces the two separate ones.
    With the reference's fixed 50 steps (TOL = 1e-100) both do the same products; only the
    order of H_BB's two additions differs for the right lead, and the ballistic forward
    step forms g^< differently: rounding, amplified by the decimation to ~1e-10 of G^R.
    A wrong right-lead surface would differ at order one."""
    dev = make_chain_device(6, 24, 6, -2.5, 2.5, seed=13, nk=2)
    kw = dict(mul=0.1, mur=-0.1, eta_lead=1e-3, caroli=True, precision=precision,
              want_blocks=True)
    a = rgf.rgf_solve(ctx, dev.H00, dev.H10, dev.E, dev.nx, nk=dev.nk, **kw)
    z = np.zeros((len(dev.E) * dev.nk, dev.nx, dev.nm, dev.nm), dtype=np.complex128)
    b = rgf.rgf_solve(ctx, dev.H00, dev.H10, dev.E, dev.nx, nk=dev.nk, sigma_r_ph=z,
                      sigma_lesser_ph=z, **kw)
    assert (a["status"] == b["status"]).all()
    np.testing.assert_array_equal(a["sancho_iters"], b["sancho_iters"])
    tol = {"fp64": 1e-9, "mixed-fp64": 1e-9, "mixed": 1e-6}[precision]
    for key in ("T", "tr", "tre", "G_r", "G_lesser"):
        # tr, tre are differences of order-one traces: judged on the transmission's scale
        scale = np.abs(b["T" if key in ("tr", "tre") else key]).max()
        np.testing.assert_allclose(a[key], b[key], rtol=0, atol=tol * scale, err_msg=key)
