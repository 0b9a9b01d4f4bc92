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


LMAX = 4096


def _stage_fft(x, inverse):
    """The GPU kernels' in-place transform, restated stage by stage in numpy (gw.cu,
    fft_smem): bit-reversed input, an odd stage count's first radix-2 pass (twiddle 1),
    then stages fused in pairs over 4h-blocks.  The pair's second twiddle for (h, 3h) is
    applied as the rotation of the (0, 2h) twiddle by -i (+i inverse), using
    tw[j + LMAX/4] = tw[j] (-i); the first pair (h = 1) has twiddles 1, 1 and -i only."""
    L = len(x)
    logL = L.bit_length() - 1
    j = np.arange(LMAX // 2)
    tw = np.exp(-2j * np.pi * j / LMAX)
    if inverse:
        tw = np.conj(tw)
    rot = 1j if inverse else -1j
    r = np.array([int(format(t, f"0{logL}b")[::-1], 2) for t in range(L)]) if logL else [0]
    a = np.empty(L, dtype=complex)
    a[r] = x
    s = 1
    if logL & 1:
        u, v = a[0::2].copy(), a[1::2].copy()
        a[0::2], a[1::2] = u + v, u - v
        s = 2
    while s < logL:
        h = 1 << (s - 1)
        t = np.arange(L // 4)
        k = t & (h - 1)
        b = (t >> (s - 1)) * 4 * h + k
        e0, e1, e2, e3 = a[b], a[b + h], a[b + 2 * h], a[b + 3 * h]
        v1, v2 = tw[k * (LMAX // (2 * h))], tw[k * (LMAX // (4 * h))]
        e0, e1 = e0 + e1 * v1, e0 - e1 * v1
        e2, e3 = e2 + e3 * v1, e2 - e3 * v1
        e0, e2 = e0 + e2 * v2, e0 - e2 * v2
        y = rot * (e3 * v2)
        e1, e3 = e1 + y, e1 - y
        a[b], a[b + h], a[b + 2 * h], a[b + 3 * h] = e0, e1, e2, e3
        s += 2
    return a


def test_rotation_identity_of_the_twiddle_table():
    """The identity the fused stage pairs rely on: the table's entry a quarter period on is
    the entry times -i."""
    j = np.arange(LMAX // 4)
    tw = np.exp(-2j * np.pi * np.arange(LMAX // 2) / LMAX)
    assert np.abs(tw[j + LMAX // 4] - tw[j] * -1j).max() < 1e-15


@pytest.mark.parametrize("L", [2, 4, 8, 32, 128, 2048, 4096])
def test_stage_structure_matches_the_dft(L):
    rng = np.random.default_rng(L)
    x = rng.normal(size=L) + 1j * rng.normal(size=L)
    ref_f, ref_i = np.fft.fft(x), L * np.fft.ifft(x)
    assert np.abs(_stage_fft(x, False) - ref_f).max() <= 1e-13 * np.abs(ref_f).max()
    assert np.abs(_stage_fft(x, True) - ref_i).max() <= 1e-13 * np.abs(ref_i).max()
