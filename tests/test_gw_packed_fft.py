"""The packed-transform algebra of the GPU's polarisation and self-energy kernels (one k-point),
restated in numpy and checked against the oracle's correlations and convolutions.

Once Re G is zeroed every input of P and every G of Sigma is purely imaginary, i a with a real.
Two such series share one complex FFT: for z = a + i b, A(k) = (Z(k) + conj Z(L-k))/2 and
B(k) = (Z(k) - conj Z(L-k))/(2i) are the transforms of a and b; the transform of i a is i A,
and the product of two imaginary series' transforms is -A B.  The kernels form
P^<, P^>, P^R from the packs (G^<, G^>), (rev G^>t, rev G^<t), (G^R, rev conj G^R), and
Sigma^<, Sigma^R from the pack (G^<, G^R) with the transforms of W^<, W^R."""
import numpy as np
import pytest

from oracle import gw as ogw


def _pad(x, L):
    z = np.zeros(L, dtype=complex)
    z[:len(x)] = x
    return z


def _unpack(Z):
    L = len(Z)
    Q = np.conj(Z[(-np.arange(L)) % L])
    return (Z + Q) / 2, (Z - Q) / 2j


@pytest.mark.parametrize("n", [16, 37, 64, 255])
def test_packed_polarisation_and_self_energy(n):
    rng = np.random.default_rng(n)
    L = 1 << int(np.ceil(np.log2(2 * n)))
    im = lambda: 1j * rng.normal(size=n)
    gl, gg, gr, glt, ggt = im(), im(), im(), im(), im()
    wl, wr = (rng.normal(size=n) + 1j * rng.normal(size=n) for _ in range(2))
    # polarisation: three packed forward transforms, three inverse
    A1, B1 = _unpack(np.fft.fft(_pad(gl.imag + 1j * gg.imag, L)))
    A2, B2 = _unpack(np.fft.fft(_pad(ggt.imag[::-1] + 1j * glt.imag[::-1], L)))
    A3, B3 = _unpack(np.fft.fft(_pad(gr.imag + 1j * np.conj(gr).imag[::-1], L)))
    t = np.arange(n) - n // 2 + n - 1
    pl = np.fft.ifft(-(A1 * A2))[t]
    pg = np.fft.ifft(-(B1 * B2))[t]
    pr = np.fft.ifft(-(A1 * B3 + A3 * B2))[t]
    for got, exp in ((pl, ogw.corr(gl, ggt)), (pg, ogw.corr(gg, glt)),
                     (pr, ogw.corr(gl, np.conj(gr)) + ogw.corr(gr, glt))):
        np.testing.assert_allclose(got, exp, rtol=0, atol=1e-12 * np.abs(exp).max())
    # the products are Hermitian in k: the kernels write conj of the value at k to L - k
    for X in (A1 * A2, B1 * B2, A1 * B3 + A3 * B2):
        np.testing.assert_allclose(X[(-np.arange(L)) % L], np.conj(X), atol=1e-9)
    # self-energy: the pack (G^<, G^R) and the transforms of W^<, W^R
    A, B = _unpack(np.fft.fft(_pad(gl.imag + 1j * gr.imag, L)))
    WL, WR = np.fft.fft(_pad(wl, L)), np.fft.fft(_pad(wr, L))
    u = np.arange(n) + n // 2
    sl = np.fft.ifft(1j * A * WL)[u]
    sr = np.fft.ifft(1j * A * WR + 1j * B * (WL + WR))[u]
    np.testing.assert_allclose(sl, ogw.conv(gl, wl), atol=1e-12 * np.abs(sl).max())
    exp = ogw.conv(gl, wr) + ogw.conv(gr, wl) + ogw.conv(gr, wr)
    np.testing.assert_allclose(sr, exp, atol=1e-12 * np.abs(exp).max())
