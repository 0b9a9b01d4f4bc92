"""Slabs of different orbital counts (rgf_variableblock_forward, src/rgf_mod.f90:46-269)
through qt_rgf_solve_vb, against the oracle and a dense inversion of the device."""
import numpy as np
import pytest

from oracle import rgf as orc
from quantum_transport_gb300 import rgf
from tests.test_oracle_variable_blocks import SIZES, dense_green, variable_device

pytestmark = pytest.mark.gpu

ENERGIES = np.array([-2.1, -0.4, 0.7, 2.5])
# the CPU routine's Fermi pairings and tr sign, as the oracle's variable-block conventions
KW = dict(mul=0.2, mur=0.2, templ=300.0, tempr=300.0, eta_lead=1e-3, sancho_tol=1e-12,
          sancho_max_iter=200, quirks=rgf._lib.QT_QUIRK_CPU_FERMI)


def _dense_T(E, Hii, H1i):
    """Caroli T = Re Tr[Gam_R G_N1 Gam_L G_N1^+] from the dense Green's function."""
    sizes = [h.shape[0] for h in Hii]
    nx, off = len(sizes), np.concatenate([[0], np.cumsum(sizes)])
    n = off[-1]
    H = np.zeros((n, n), dtype=np.complex128)
    for l in range(nx):
        H[off[l]:off[l + 1], off[l]:off[l + 1]] = Hii[l]
        if l:
            H[off[l]:off[l + 1], off[l - 1]:off[l]] = H1i[l]
            H[off[l - 1]:off[l], off[l]:off[l + 1]] = H1i[l].conj().T
    gL = orc.sancho(E, np.eye(sizes[0]), Hii[0], H1i[0].conj().T, eta=1e-3, nmax=200, tol=1e-12)[0]
    gR = orc.sancho(E, np.eye(sizes[-1]), Hii[-1], H1i[nx], eta=1e-3, nmax=200, tol=1e-12)[0]
    SL = H1i[0] @ gL @ H1i[0].conj().T
    SR = H1i[nx].conj().T @ gR @ H1i[nx]
    A = E * np.eye(n) - H
    A[:sizes[0], :sizes[0]] -= SL
    A[off[-2]:, off[-2]:] -= SR
    G = np.linalg.inv(A)
    GN1 = G[off[-2]:, :sizes[0]]
    gam = lambda S: 1j * (S - S.conj().T)
    return float(np.real(np.trace(gam(SR) @ GN1 @ gam(SL) @ GN1.conj().T)))


def test_fp64_matches_oracle_and_dense(ctx):
    Hii, H1i = variable_device(5)
    r = rgf.rgf_variableblock_forward(ctx, Hii, H1i, ENERGIES, caroli=True, **KW)
    assert (r["status"] == 0).all()
    for ie, E in enumerate(ENERGIES):
        o = orc.rgf_constblocksize(E, Hii, H1i, quirks=orc.QUIRKS_VARIABLE, sancho_nmax=200,
                                   **{k: v for k, v in KW.items()
                                      if k not in ("sancho_max_iter", "quirks")})
        Gd, Gld = dense_green(E, Hii, H1i, 0.2, 300.0, 1e-3)
        for l in range(len(SIZES)):
            got = r["diag_gr"][l][ie, 0]
            np.testing.assert_allclose(got, np.diag(o["G_r"][l]), rtol=0,
                                       atol=1e-10 * np.abs(Gd[l]).max())
            np.testing.assert_allclose(got, np.diag(Gd[l]), rtol=0, atol=1e-9 * np.abs(Gd[l]).max())
            np.testing.assert_allclose(r["diag_gl"][l][ie, 0], np.diag(o["G_lesser"][l]), rtol=0,
                                       atol=1e-10 * max(np.abs(Gld[l]).max(), 1e-300))
        np.testing.assert_allclose(r["tre"][ie, 0], o["tre"], rtol=1e-9, atol=1e-12)
        np.testing.assert_allclose(r["tr"][ie, 0], o["tr"], rtol=1e-9, atol=1e-12)
        np.testing.assert_allclose(r["T"][ie, 0], _dense_T(E, Hii, H1i), rtol=1e-9)


@pytest.mark.parametrize("precision,tol", [("mixed-fp64", 1e-9), ("mixed", 2e-5)])
def test_split_paths_match_fp64(ctx, precision, tol):
    Hii, H1i = variable_device(6)
    r64 = rgf.rgf_variableblock_forward(ctx, Hii, H1i, ENERGIES, caroli=True, **KW)
    rs = rgf.rgf_variableblock_forward(ctx, Hii, H1i, ENERGIES, caroli=True, precision=precision,
                                       **KW)
    assert (rs["status"] == 0).all()
    np.testing.assert_allclose(rs["T"], r64["T"], rtol=tol)
    for key in ("diag_gr", "diag_gl"):
        for a, b in zip(rs[key], r64[key]):
            assert np.abs(a - b).max() <= tol * np.abs(b).max(), (precision, key)


def test_equal_blocks_match_constblocksize(ctx):
    """With equal blocks and slab-independent couplings the variable-block path is the
    constant-block sweep with the CPU routine's conventions.  The constant-block sweep
    decimates its two equal leads in one dual-surface run (the variable-block path runs
    two), which changes the rounding order only."""
    rng = np.random.default_rng(8)
    n, nx = 12, 6
    X = 0.1 * (rng.normal(size=(n, n)) + 1j * rng.normal(size=(n, n)))
    H00 = np.triu(X, 1) + np.triu(X, 1).conj().T + np.diag(rng.uniform(-1, 1, n))
    H10 = -2.0 * np.eye(n) + 0.05 * (rng.normal(size=(n, n)) + 1j * rng.normal(size=(n, n)))
    E = np.linspace(-3.0, 3.0, 7)
    kw = dict(mul=0.3, mur=-0.1, templ=300.0, tempr=250.0, eta_lead=1e-3, sancho_tol=1e-12,
              sancho_max_iter=200, caroli=True)
    q = rgf._lib.QT_QUIRK_CPU_FERMI | rgf._lib.QT_QUIRK_BACK_H1I_NEXT
    a = rgf.rgf_solve(ctx, H00, H10, E, nx, quirks=q, **kw)
    b = rgf.rgf_variableblock_forward(ctx, [H00] * nx, [H10] * (nx + 1), E,
                                      quirks=rgf._lib.QT_QUIRK_CPU_FERMI, **kw)
    for key in ("T", "tr", "tre"):
        np.testing.assert_allclose(b[key], a[key], rtol=1e-10, atol=1e-13)
    for l in range(nx):
        np.testing.assert_allclose(b["diag_gr"][l], a["diag_gr"][:, :, l], rtol=1e-10, atol=1e-13)
