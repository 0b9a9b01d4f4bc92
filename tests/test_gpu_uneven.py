"""Blocks above one 128-row tile on the split path: tiled products and block inverses
against numpy, and the uneven-block workload (4000-atom graph, 25 slabs of 134-184
orbitals) in FP64 against the oracle and in both split precisions against FP64."""
import numpy as np
import pytest

from oracle import rgf as orc
from quantum_transport_gb300 import rgf
from quantum_transport_gb300.devices import config_uneven

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("n", [200, 260, 384])
def test_tiled_split_product(ctx, n):
    rng = np.random.default_rng(n)
    A = rng.normal(size=(3, n, n)) + 1j * rng.normal(size=(3, n, n))
    B = rng.normal(size=(3, n, n)) + 1j * rng.normal(size=(3, n, n))
    D = rng.normal(size=(3, n, n)) + 1j * rng.normal(size=(3, n, n))
    for opA, opB in (("N", "N"), ("C", "N"), ("N", "C")):
        a = np.conj(np.swapaxes(A, -1, -2)) if opA == "C" else A
        b = np.conj(np.swapaxes(B, -1, -2)) if opB == "C" else B
        ref = 0.5 * a @ b - D
        got = rgf.mul_c(ctx, A, B, opA, opB, alpha=0.5, beta=-1.0, D=D, precision="mixed",
                        slices=7)
        assert np.abs(got - ref).max() <= 1e-13 * np.abs(ref).max(), (opA, opB)


@pytest.mark.parametrize("n", [160, 260, 384])
def test_tiled_split_inverse(ctx, n):
    rng = np.random.default_rng(n + 1)
    A = (rng.normal(size=(4, n, n)) + 1j * rng.normal(size=(4, n, n))) / np.sqrt(n) \
        + 2.0 * np.eye(n)
    got = rgf.invert(ctx, A, precision="mixed")[0]
    ref = np.linalg.inv(A)
    assert np.abs(got - ref).max() <= 1e-11 * np.abs(ref).max()


KW = dict(mul=0.1, mur=-0.1, templ=300.0, tempr=300.0, eta_lead=1e-3, sancho_tol=1e-12)


@pytest.mark.parametrize("nm", [160, 250])
def test_tiled_sweep_matches_fp64(ctx, nm):
    """Equal blocks above one tile on a well-conditioned chain: the tiled split sweep keeps
    the accuracy of the untiled one (complex128 split: FP64 grade)."""
    from quantum_transport_gb300.devices import make_chain_device
    dev = make_chain_device(6, nm, 8, -2.0, 2.0, seed=3)
    kw = dict(mul=0.1, mur=-0.1, eta_lead=1e-3, sancho_tol=1e-12, sancho_max_iter=200,
              caroli=True)
    r64 = rgf.rgf_solve(ctx, dev.H00, dev.H10, dev.E, dev.nx, **kw)
    for precision, tT, td in (("mixed-fp64", 1e-11, 1e-7), ("mixed", 1e-6, 1e-5)):
        r = rgf.rgf_solve(ctx, dev.H00, dev.H10, dev.E, dev.nx, precision=precision, **kw)
        assert (r["status"] == 0).all()
        assert np.abs(r["T"] - r64["T"]).max() <= tT * np.abs(r64["T"]).max(), precision
        assert np.abs(r["diag_gr"] - r64["diag_gr"]).max() <= \
            td * np.abs(r64["diag_gr"]).max(), precision


@pytest.fixture(scope="module")
def uneven():
    d = config_uneven(nE=2048)
    E = d.E[::128][:16]  # 16 energies across [-2, 2] eV
    Hii = [h[:2] for h in d.Hii]  # k-points -pi and -3 pi / 4
    H1i = [h[:2] for h in d.H1i]
    return d, E, Hii, H1i


def test_uneven_fp64_matches_oracle(ctx, uneven):
    d, E, Hii, H1i = uneven
    r = rgf.rgf_variableblock_forward(ctx, Hii, H1i, E[:3], nk=2, sancho_max_iter=200,
                                      caroli=True, **KW)
    assert (r["status"] == 0).all()
    for ie in range(3):
        for ik in range(2):
            o = orc.rgf_constblocksize(E[ie], [h[ik] for h in Hii], [h[ik] for h in H1i],
                                       quirks=dict(orc.QUIRKS_GOLDEN, back_coupling="next",
                                                   right_coupling="nx+1", jdens="cpu"),
                                       sancho_nmax=200, **KW)
            # each lead repeats a dense 134-184 orbital block at eta = 1e-3: its decimation
            # amplifies the rounding-order difference of the two FP64 eliminations
            for l in (0, d.nx // 2, d.nx - 1):
                exp = np.diag(o["G_r"][l])
                np.testing.assert_allclose(r["diag_gr"][l][ie, ik], exp, rtol=0,
                                           atol=1e-6 * np.abs(exp).max())
            np.testing.assert_allclose(r["tr"][ie, ik], o["tr"], rtol=1e-6, atol=1e-10)


@pytest.mark.parametrize("precision,tol", [("mixed-fp64", 1e-7), ("mixed", 1e-3)])
def test_uneven_split_matches_fp64(ctx, uneven, precision, tol):
    d, E, Hii, H1i = uneven
    r64 = rgf.rgf_variableblock_forward(ctx, Hii, H1i, E, nk=2, sancho_max_iter=200,
                                        caroli=True, **KW)
    rs = rgf.rgf_variableblock_forward(ctx, Hii, H1i, E, nk=2, sancho_max_iter=200,
                                       caroli=True, precision=precision, **KW)
    assert (rs["status"] == 0).all() and (r64["status"] == 0).all()
    T64 = r64["T"]
    err = np.abs(rs["T"] - T64).max() / np.abs(T64).max()
    per = [np.abs(a - b).max() / np.abs(b).max() for a, b in zip(rs["diag_gr"], r64["diag_gr"])]
    print(f"{precision}: max |T - T_fp64| / max T = {err:.3e}, diag G^R per slab max "
          f"{max(per):.3e} median {np.median(per):.3e}, inverses redone in FP64: "
          f"{ctx.inverse_fallbacks()}")
    assert err <= tol
    if precision == "mixed-fp64":
        assert max(per) <= 100 * tol
    else:
        # complex64 storage of g_l: the most ill-conditioned slabs lose their diagonal
        # (up to 0.8 relative even with every inverse in FP64); typical slabs keep 1e-3
        assert np.median(per) <= 1e-2


@pytest.mark.parametrize("n", [96, 200])
def test_inverse_guard_redoes_ill_conditioned_blocks(ctx, n):
    """Blocks with condition number 1e9 defeat the FP32 elimination (first residual far
    above 1, so refinement would diverge): the guard redoes exactly those in FP64."""
    rng = np.random.default_rng(n + 7)

    def unitary():
        q, _ = np.linalg.qr(rng.normal(size=(n, n)) + 1j * rng.normal(size=(n, n)))
        return q

    good = [(rng.normal(size=(n, n)) + 1j * rng.normal(size=(n, n))) / np.sqrt(n) + 2 * np.eye(n)
            for _ in range(5)]
    bad = [unitary() @ np.diag(np.logspace(0, -9, n)) @ unitary() for _ in range(2)]
    A = np.stack(good[:2] + bad[:1] + good[2:] + bad[1:])
    ctx.inverse_fallbacks(reset=True)
    X, status = rgf.invert(ctx, A, precision="mixed")
    assert ctx.inverse_fallbacks() == 2
    assert (status == 0).all()
    for a, x in zip(A, X):
        ref = np.linalg.inv(a)
        assert np.abs(x - ref).max() <= 1e-5 * np.abs(ref).max()
