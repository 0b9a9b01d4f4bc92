"""Accuracy of 4096-point transforms built from split-digit products, the planned tensor-core
form of the GW energy correlations (today FP64 radix-2 transforms in shared memory).

A four-step DFT of length 4096 = 64 x 64 is two 64 x 64 complex products around a twiddle
multiply: Y = F Xm with Xm[n1, n2] = x[64 n1 + n2], Y[k1, n2] *= w^(n2 k1), Z = Y F, and
X[k1 + 64 k2] = Z[k1, k2].  Each product is emulated as the split products compute it: every
row of the left operand and every column of the right one scaled to its own power of two and
cut into S base-256 digits, the digit pairs s + t <= S - 1 summed exactly.  The test pins the
error of one correlation (two forward transforms, their product, one inverse) against
numpy's FP64 FFT for the digit counts of the two split modes: 4 digits against the
complex64 sweep's own 1e-7, 6 digits at FP64 level."""
import numpy as np
import pytest

L, N = 4096, 64


def _digits(M, S):
    e = np.ceil(np.log2(np.maximum(np.abs(M).max(axis=1, keepdims=True), 1e-300))) + 1
    R = M / 2.0 ** e
    D = []
    for _ in range(S):
        R = R * 256.0
        d = np.rint(R)
        D.append(d)
        R = R - d
    return e, D


def _split_real(A, B, S):
    ea, DA = _digits(A, S)
    eb, DB = _digits(B.T, S)
    C = np.zeros((A.shape[0], B.shape[1]))
    for s in range(S):
        for t in range(S - s):
            C += (DA[s] @ DB[t].T) * 256.0 ** (-(s + t + 2))
    return C * 2.0 ** ea * 2.0 ** eb.T


def _split_complex(A, B, S):
    AK = np.hstack([A.real, A.imag])  # (Re, Im) interleaved along K, as the kernels do
    return (_split_real(AK, np.vstack([B.real, -B.imag]), S)
            + 1j * _split_real(AK, np.vstack([B.imag, B.real]), S))


_F = np.exp(-2j * np.pi * np.outer(np.arange(N), np.arange(N)) / N)
_TW = np.exp(-2j * np.pi * np.outer(np.arange(N), np.arange(N)) / L)


def _dft(x, S):
    Y = _split_complex(_F, x.reshape(N, N), S) * _TW
    return _split_complex(Y, _F, S).T.reshape(-1)


def _idft(X, S):
    return np.conj(_dft(np.conj(X), S))


def test_four_step_layout_is_the_dft():
    x = np.random.default_rng(1).normal(size=L) + 0j
    Y = (_F @ x.reshape(N, N)) * _TW
    np.testing.assert_allclose((Y @ _F).T.reshape(-1), np.fft.fft(x), atol=1e-9)


@pytest.mark.parametrize("S,bound", [(4, 2e-8), (6, 5e-13)])
def test_correlation_error_by_digit_count(S, bound):
    rng = np.random.default_rng(S)
    n = L // 2
    E = np.linspace(-4, 4, n)
    a = rng.normal(size=n) + 1j * rng.normal(size=n)
    b = 1j * (0.05 / ((E[:, None] - rng.uniform(-3, 3, 40)) ** 2 + 0.05 ** 2)).sum(1)
    x = np.zeros(L, complex)
    y = np.zeros(L, complex)
    x[:n], y[:n] = a, b[::-1]
    ref = np.fft.ifft(np.fft.fft(x) * np.fft.fft(y))
    got = _idft(_dft(x, S) * _dft(y, S), S) / L
    assert np.abs(got - ref).max() <= bound * np.abs(ref).max()
