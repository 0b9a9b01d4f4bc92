"""The oracle's sweep with blocks of different sizes against a dense inversion of the
whole device (an independent restatement of the same Green's functions)."""
import numpy as np
import pytest

from oracle import rgf

SIZES = [6, 9, 7, 10, 6]


def variable_device(seed, sizes=SIZES):
    rng = np.random.default_rng(seed)
    nx = len(sizes)
    Hii = []
    for n in sizes:
        X = 0.1 * (rng.normal(size=(n, n)) + 1j * rng.normal(size=(n, n)))
        Hii.append(np.triu(X, 1) + np.triu(X, 1).conj().T + np.diag(rng.uniform(-1, 1, n)))
    H1i = [None] * (nx + 1)
    for l in range(1, nx):
        H1i[l] = -1.0 * np.eye(sizes[l], sizes[l - 1]) + \
            0.05 * (rng.normal(size=(sizes[l], sizes[l - 1])) + 1j * rng.normal(size=(sizes[l], sizes[l - 1])))
    for l, n in ((0, sizes[0]), (nx, sizes[-1])):
        H1i[l] = -2.7 * np.eye(n) + 0.05 * (rng.normal(size=(n, n)) + 1j * rng.normal(size=(n, n)))
    return Hii, H1i


def dense_green(E, Hii, H1i, mu, temp, eta_lead):
    sizes = [h.shape[0] for h in Hii]
    nx, off = len(sizes), np.concatenate([[0], np.cumsum(sizes)])
    n = off[-1]
    H = np.zeros((n, n), dtype=np.complex128)
    for l in range(nx):
        H[off[l]:off[l + 1], off[l]:off[l + 1]] = Hii[l]
        if l:
            H[off[l]:off[l + 1], off[l - 1]:off[l]] = H1i[l]
            H[off[l - 1]:off[l], off[l]:off[l + 1]] = H1i[l].conj().T
    gL = rgf.sancho(E, np.eye(sizes[0]), Hii[0], H1i[0].conj().T, eta=eta_lead)[0]
    gR = rgf.sancho(E, np.eye(sizes[-1]), Hii[-1], H1i[nx], eta=eta_lead)[0]
    SL = np.zeros_like(H)
    SR = np.zeros_like(H)
    SL[:sizes[0], :sizes[0]] = H1i[0] @ gL @ H1i[0].conj().T
    SR[off[-2]:, off[-2]:] = H1i[nx].conj().T @ gR @ H1i[nx]
    G = np.linalg.inv(E * np.eye(n) - H - SL - SR)
    f = rgf.ferm((E - mu) / (rgf.BOLTZ * temp))
    Sless = -(SL - SL.conj().T) * f - (SR - SR.conj().T) * f
    Gl = G @ Sless @ G.conj().T
    return [G[off[l]:off[l + 1], off[l]:off[l + 1]] for l in range(nx)], \
        [Gl[off[l]:off[l + 1], off[l]:off[l + 1]] for l in range(nx)]


@pytest.mark.parametrize("E", [-2.1, -0.4, 0.7, 2.5])
def test_variable_blocks_match_dense_inverse(E):
    Hii, H1i = variable_device(5)
    o = rgf.rgf_constblocksize(E, Hii, H1i, mul=0.2, mur=0.2, templ=300.0, tempr=300.0,
                               quirks=rgf.QUIRKS_VARIABLE, eta_lead=1e-3, sancho_nmax=200,
                               sancho_tol=1e-12)
    Gd, Gld = dense_green(E, Hii, H1i, 0.2, 300.0, 1e-3)
    for l in range(len(Hii)):
        scale = np.abs(Gd[l]).max()
        np.testing.assert_allclose(o["G_r"][l], Gd[l], rtol=0, atol=1e-9 * scale)
        np.testing.assert_allclose(o["G_lesser"][l], Gld[l], rtol=0,
                                   atol=1e-9 * max(np.abs(Gld[l]).max(), 1e-300))
