"""The oracle's k-pair sums and ndiag band (src/gw_mod.f90:466-555, 640-730) against a
literal restatement of the reference's loops: 1-based k indices with the single wrap of
ikzd / ikyd, the column-major element index global_ij with its row/col band test, and
direct (non-FFT) correlations and convolutions."""
import numpy as np
import pytest

from oracle import gw as ogw


def _kd_literal(ik0, iq0, nky, nkz):
    # src/gw_mod.f90:478-487 with 1-based loop variables
    iky, ikz = ik0 // nkz + 1, ik0 % nkz + 1
    iqy, iqz = iq0 // nkz + 1, iq0 % nkz + 1
    ikzd = ikz - iqz + nkz // 2
    ikyd = iky - iqy + nky // 2
    if ikzd < 1:
        ikzd += nkz
    if ikzd > nkz:
        ikzd -= nkz
    if ikyd < 1:
        ikyd += nky
    if ikyd > nky:
        ikyd -= nky
    if nky == 1:
        ikyd = 1
    if nkz == 1:
        ikzd = 1
    return ikzd + (ikyd - 1) * nkz - 1


@pytest.mark.parametrize("nky,nkz", [(1, 1), (1, 2), (1, 3), (1, 4), (2, 2), (3, 2), (2, 5),
                                     (4, 1)])
def test_kd_index_matches_reference_loop(nky, nkz):
    nk = nky * nkz
    for ik in range(nk):
        for iq in range(nk):
            assert ogw.kd_index(ik, iq, nky, nkz) == _kd_literal(ik, iq, nky, nkz)


def _cplx(rng, shape):
    return rng.normal(size=shape) + 1j * rng.normal(size=shape)


def _in_band(row, col, nm, ndiag):
    if ndiag is None:
        return True
    lo, hi = max(row - ndiag, 0), min(nm - 1, row + ndiag)
    return lo <= col <= hi


def _literal_p(GR, GL, GG, dE, nky, nkz, spindeg, ndiag):
    nk, nE, nx, nm, _ = GR.shape
    PR, PL, PG = (np.zeros_like(GR) for _ in range(3))
    for gij in range(nm * nm):           # global_ij - 1, column-major
        col, row = gij // nm, gij % nm
        if not _in_band(row, col, nm, ndiag):
            continue
        for ix in range(nx):
            for iq in range(nk):
                for ik in range(nk):
                    kd = _kd_literal(ik, iq, nky, nkz)
                    gl, gg, gr = GL[ik, :, ix, row, col], GG[ik, :, ix, row, col], GR[ik, :, ix, row, col]
                    ggt, glt = GG[kd, :, ix, col, row], GL[kd, :, ix, col, row]
                    grd = GR[kd, :, ix, row, col]
                    PL[iq, :, ix, row, col] += ogw.corr_direct(gl, ggt)
                    PG[iq, :, ix, row, col] += ogw.corr_direct(gg, glt)
                    PR[iq, :, ix, row, col] += ogw.corr_direct(gl, np.conj(grd)) + \
                        ogw.corr_direct(gr, glt)
    f = -1j * dE / (2 * np.pi) * spindeg / nk
    return PR * f, PL * f, PG * f


def _literal_sigma(GR, GL, GG, WR, WL, WG, dE, nky, nkz, ndiag):
    nk, nE, nx, nm, _ = GR.shape
    SR, SL, SG = (np.zeros_like(GR) for _ in range(3))
    for gij in range(nm * nm):
        col, row = gij // nm, gij % nm
        if not _in_band(row, col, nm, ndiag):
            continue
        for ix in range(nx):
            for ik in range(nk):
                for iq in range(nk):
                    kd = _kd_literal(ik, iq, nky, nkz)
                    g = [A[kd, :, ix, row, col] for A in (GR, GL, GG)]
                    w = [A[iq, :, ix, row, col] for A in (WR, WL, WG)]
                    SL[ik, :, ix, row, col] += ogw.conv_direct(g[1], w[1])
                    SG[ik, :, ix, row, col] += ogw.conv_direct(g[2], w[2])
                    SR[ik, :, ix, row, col] += ogw.conv_direct(g[1], w[0]) + \
                        ogw.conv_direct(g[0], w[1]) + ogw.conv_direct(g[0], w[0])
    f = 1j * dE / (2 * np.pi) / nk
    SR, SL, SG = SR * f, SL * f, SG * f
    SR = SR.real + 1j * (SG - SL).imag / 2
    sym = lambda A: (A + np.swapaxes(A, -1, -2)) / 2
    return sym(SR), sym(SL), sym(SG)


@pytest.mark.parametrize("nky,nkz,ndiag", [(1, 1, None), (1, 3, None), (2, 2, 1), (1, 4, 0)])
def test_k_sums_and_band_match_literal_loops(nky, nkz, ndiag):
    rng = np.random.default_rng(nky * 10 + nkz)
    nk, nE, nx, nm = nky * nkz, 9, 2, 3
    shape = (nk, nE, nx, nm, nm)
    G = [_cplx(rng, shape) for _ in range(3)]
    W = [_cplx(rng, shape) for _ in range(3)]
    dE = 0.05
    got = ogw.polarization_k(*G, dE, nky, nkz, 2.0, ndiag)
    for a, b in zip(got, _literal_p(*G, dE, nky, nkz, 2.0, ndiag)):
        np.testing.assert_allclose(a, b, atol=1e-12 * np.abs(b).max())
    got = ogw.self_energy_k(*G, *W, dE, nky, nkz, ndiag)
    for a, b in zip(got, _literal_sigma(*G, *W, dE, nky, nkz, ndiag)):
        np.testing.assert_allclose(a, b, atol=1e-12 * np.abs(b).max())


def test_one_k_point_is_the_single_k_oracle():
    rng = np.random.default_rng(5)
    shape = (1, 16, 3, 4, 4)
    G = [_cplx(rng, shape) for _ in range(3)]
    W = [_cplx(rng, shape) for _ in range(3)]
    for a, b in zip(ogw.polarization_k(*G, 0.1, 1, 1), ogw.polarization(*(g[0] for g in G), 0.1)):
        np.testing.assert_allclose(a[0], b, rtol=0, atol=1e-13 * np.abs(b).max())
    for a, b in zip(ogw.self_energy_k(*G, *W, 0.1, 1, 1),
                    ogw.self_energy(*(g[0] for g in G), *(w[0] for w in W), 0.1)):
        np.testing.assert_allclose(a[0], b, rtol=0, atol=1e-13 * np.abs(b).max())
