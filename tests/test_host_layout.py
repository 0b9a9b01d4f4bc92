"""Host-side layout helpers and the seeded synthetic devices: the column-major block images
the C-ABI reads, the packed layout of blocks of different sizes, the per-cell spectrum
reduction, and the statistics the benchmark configurations state."""
import numpy as np
import pytest

from quantum_transport_gb300 import devices, gw, rgf


def test_colmajor_is_the_fortran_image():
    A = np.random.default_rng(0).normal(size=(3, 4, 4)) + 0j
    buf = rgf.colmajor(A)
    assert buf.flags["C_CONTIGUOUS"] and buf.dtype == np.complex128
    # element (i, j) of block b sits at offset i + j n, as in complex(8) :: m(n, n)
    flat = buf.reshape(3, -1)
    assert flat[1, 2 + 3 * 4] == A[1, 2, 3]
    np.testing.assert_array_equal(rgf.from_colmajor(buf), A)
    np.testing.assert_array_equal(buf[0].ravel(), np.asfortranarray(A[0]).ravel(order="K"))


@pytest.mark.parametrize("shape,nk,nslab,strides", [((5, 5), 1, 3, (0, 0)),
                                                    ((2, 5, 5), 2, 3, (25, 0)),
                                                    ((1, 5, 5), 1, 3, (0, 0)),
                                                    ((2, 3, 5, 5), 2, 3, (75, 25))])
def test_block_strides(shape, nk, nslab, strides):
    buf, hk, hl, nm = rgf._blocks(np.zeros(shape, complex), nk, nslab)
    assert (hk, hl, nm) == strides + (5,)
    assert buf.size == int(np.prod(shape))


def test_block_shapes_are_checked():
    with pytest.raises(ValueError):
        rgf._blocks(np.zeros((3, 5, 5), complex), 2, 3)
    with pytest.raises(ValueError):
        rgf._blocks(np.zeros((2, 4, 5, 5), complex), 2, 3)


def test_pack_blocks_offsets_and_broadcast():
    rng = np.random.default_rng(1)
    nk = 2
    blocks = [rng.normal(size=(nk, 3, 3)) + 1j * rng.normal(size=(nk, 3, 3)),
              rng.normal(size=(4, 3)) + 0j,  # one block for every k
              rng.normal(size=(nk, 4, 4)) + 0j]
    packed, offs, kstride = rgf.pack_blocks(blocks, nk)
    assert list(offs) == [0, 9, 21] and kstride == 37 and packed.shape == (nk, 37)
    for k in range(nk):
        for b, o in zip(blocks, offs):
            bk = b[k] if b.ndim == 3 else b
            r, c = bk.shape
            np.testing.assert_array_equal(packed[k, o:o + r * c].reshape(c, r).T, bk)


def test_cell_spectra_sums_bands_and_averages_k():
    nE, nk, nx, nslab, nbnd = 3, 2, 4, 2, 5
    d = np.random.default_rng(2).normal(size=(nE, nk, nx, nslab * nbnd)) + 0j
    t = rgf.cell_spectra(d, nbnd, nslab)
    assert t.shape == (nE, nx * nslab)
    np.testing.assert_allclose(t[1, 2 * nslab + 1], d[1, :, 2, nbnd:2 * nbnd].sum(-1).mean())


def test_photon_steps_floor():
    assert gw.photon_steps(0.5, 0.125) == 4 and gw.photon_steps(0.55, 0.125) == 4
    assert gw.photon_steps(0.1, 0.125) == 0


def test_chain_device_statistics():
    d = devices.config_batched(nE=64, nk=16, nx=4, nm=32)
    assert d.H00.shape == (16, 32, 32) and d.H10.shape == (32, 32) and d.E.shape == (64,)
    np.testing.assert_allclose(d.kpts, -np.pi + 2 * np.pi * np.arange(16) / 16)
    for H in d.H00:  # H_ii(k) = H_ii + H_y e^{ik} + h.c. is Hermitian at every k
        np.testing.assert_allclose(H, H.conj().T, atol=1e-14)
    H0 = d.H00.mean(axis=0)  # the k-average removes H_y e^{ik} + h.c.
    assert np.all(np.abs(np.diag(H0).real) <= 1.0)
    np.testing.assert_allclose(np.diag(d.H10).real.mean(), -2.7, atol=0.05)
    assert d.E[0] == -2.0 and d.E[-1] == 2.0


def test_coulomb_block_and_disorder_family():
    V = devices.coulomb_block(8)
    np.testing.assert_allclose(V, V.T)
    assert V[0, 0] == 14.4 and np.isclose(V[0, 4], 14.4 / 2.0)
    g = devices.disordered_gw_device(7, nx=5, nm=8, nE=32)
    base = devices.make_chain_device(5, 8, 32, -4.0, 4.0, seed=3)
    off = ~np.eye(8, dtype=bool)
    for l in range(5):  # the disorder touches the on-site energies only
        np.testing.assert_array_equal(g.H00[l][off], base.H00[0][off])
    dd = np.diagonal(g.H00 - base.H00[0], axis1=1, axis2=2)
    assert np.all(dd.imag == 0) and 0.02 < dd.real.std() < 0.4
    np.testing.assert_array_equal(g.V, V)
