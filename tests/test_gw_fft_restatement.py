"""The oracle's energy correlation / convolution against the reference's 'fft' branches.

oracle/gw.py computes corr1d2 / conv1d2 by zero-padded FFTs of a power-of-two length.
Here the reference's 'fft' branches are restated step by step -- the (2n-1)-point padding,
the reversed or rotated Y, one circular convolution (do_mkl_dfti_conv: forward, forward,
product, backward, / length) and the slice -- and the oracle must equal them to rounding.
The reference's 'index' branch of conv1d2 keeps strict inequalities at both ends and so
drops the first and last terms; it is checked here only where it agrees.
"""
import numpy as np
import pytest

from oracle import gw as ogw


def _dfti_conv(X, Y):
    """do_mkl_dfti_conv (src/fft_mod.f90:170-190): circular convolution of length len(X);
    MKL's backward transform is unnormalised and the routine divides by the length, which
    is numpy's normalised inverse."""
    return np.fft.ifft(np.fft.fft(X) * np.fft.fft(Y))


def corr1d2_fft(X, Y):
    """corr1d2(n, X, Y, 'fft'), src/fft_mod.f90:78-90 (1-based slices made 0-based)."""
    n = len(X)
    X_ = np.zeros(2 * n - 1, dtype=np.complex128)
    Y_ = np.zeros(2 * n - 1, dtype=np.complex128)
    X_[:n] = X                     # X_(1:n) = X
    Y_[:n] = Y[::-1]               # Y_(1:n) = Y(n:1:-1)
    Z_ = _dfti_conv(X_, Y_)
    return Z_[n - n // 2 - 1:n + n // 2 - 1]  # Z = Z_(n-n/2 : n+n/2-1)


def conv1d2_fft(X, Y):
    """conv1d2(n, X, Y, 'fft'), src/fft_mod.f90:151-163."""
    n = len(X)
    X_in = np.zeros(2 * n - 1, dtype=np.complex128)
    Y_in = np.zeros(2 * n - 1, dtype=np.complex128)
    X_in[:n] = X                              # X_in(1:n) = X
    Y_in[:n // 2] = Y[n // 2:]                # Y_in(1:n/2) = Y(n/2+1:n)
    Y_in[2 * n - n // 2 - 1:2 * n - 1] = Y[:n // 2]  # Y_in(2n-n/2:2n-1) = Y(1:n/2)
    Z_in = _dfti_conv(Y_in, X_in)
    return Z_in[:n]                           # Z = Z_in(1:n)


def corr1d2_index(X, Y):
    """corr1d2(n, X, Y, 'index'), src/fft_mod.f90:65-71."""
    n = len(X)
    Z = np.zeros(n, dtype=np.complex128)
    for i in range(-n // 2 + 1, n // 2):
        for ie in range(max(i + 1, 1), min(n, n + i) + 1):
            Z[i + n // 2 - 1] += X[ie - 1] * Y[ie - i - 1]
    return Z


@pytest.mark.parametrize("n", [8, 16, 64, 256, 2048])
def test_oracle_corr_equals_reference_fft_branch(n):
    rng = np.random.default_rng(n)
    X = rng.normal(size=(3, n)) + 1j * rng.normal(size=(3, n))
    Y = rng.normal(size=(3, n)) + 1j * rng.normal(size=(3, n))
    got = ogw.corr(X, Y)
    for b in range(3):
        ref = corr1d2_fft(X[b], Y[b])
        np.testing.assert_allclose(got[b], ref, rtol=0, atol=1e-13 * np.abs(ref).max())


@pytest.mark.parametrize("n", [8, 16, 64, 256, 2048])
def test_oracle_conv_equals_reference_fft_branch(n):
    rng = np.random.default_rng(n + 1)
    X = rng.normal(size=(3, n)) + 1j * rng.normal(size=(3, n))
    W = rng.normal(size=(3, n)) + 1j * rng.normal(size=(3, n))
    got = ogw.conv(X, W)
    for b in range(3):
        ref = conv1d2_fft(X[b], W[b])
        np.testing.assert_allclose(got[b], ref, rtol=0, atol=1e-13 * np.abs(ref).max())


@pytest.mark.parametrize("n", [8, 16, 64])
def test_reference_index_branch_is_one_step_off(n):
    """The 'index' branch writes lag i to Z(i + n/2), the 'fft' branch to Z(i + n/2 + 1):
    the oracle follows 'fft' (the form do_mkl_dfti_conv computes), and the two differ by one
    grid step of the lag axis."""
    rng = np.random.default_rng(3 * n)
    X = rng.normal(size=n) + 1j * rng.normal(size=n)
    Y = rng.normal(size=n) + 1j * rng.normal(size=n)
    idx = corr1d2_index(X, Y)
    fft = corr1d2_fft(X, Y)
    np.testing.assert_allclose(idx[:n - 2], fft[1:n - 1], rtol=0, atol=1e-12 * np.abs(fft).max())
