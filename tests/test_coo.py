"""COO Hamiltonian input: the package's reader against the oracle's, and the oracle's
block builder pinned by the test_cnt device Hamiltonian written as a COO file."""
import os

import numpy as np
import pytest

from oracle import coo as ocoo
from quantum_transport_gb300 import coo

GOLDEN = os.path.join(os.path.dirname(__file__), "golden")


def cnt_device(nx=5):
    """Full test_cnt device Hamiltonian (nx slabs of H00, couplings H10) at k = 0."""
    b = np.load(os.path.join(GOLDEN, "cnt_blocks.npz"))
    H00, H10 = b["H00"], b["H10"]
    bs = H00.shape[0]
    H = np.zeros((nx * bs, nx * bs), dtype=np.complex128)
    for i in range(nx):
        H[i * bs:(i + 1) * bs, i * bs:(i + 1) * bs] = H00
        if i + 1 < nx:
            H[(i + 1) * bs:(i + 2) * bs, i * bs:(i + 1) * bs] = H10
            H[i * bs:(i + 1) * bs, (i + 1) * bs:(i + 2) * bs] = H10.conj().T
    return H, H00, H10


def write_coo(path, row0, col0, h, base=1, iscomplex=True):
    with open(path, "w") as f:
        for r, c, v in zip(row0, col0, h):
            if iscomplex:
                f.write(f"{r + base} {c + base} {v.real:.17g} {v.imag:.17g}\n")
            else:
                f.write(f"{r + base} {c + base} {v.real:.17g}\n")


def upper_entries(H):
    r, c = np.nonzero(np.triu(H))
    return r, c, H[r, c]


@pytest.mark.parametrize("base,iscomplex", [(0, False), (1, False), (1, True)])
def test_reader_matches_oracle(tmp_path, base, iscomplex):
    rng = np.random.default_rng(3)
    n = 200
    r, c = rng.integers(0, 40, n), rng.integers(0, 40, n)
    h = rng.normal(size=n) + 1j * rng.normal(size=n)
    path = tmp_path / "h_dat"
    write_coo(path, r, c, h, base, iscomplex)
    m = coo.load(str(path), use0index=(base == 0), iscomplex=iscomplex)
    oh, orow, ocol, onorb = ocoo.load_coo(str(path), use0index=(base == 0), iscomplex=iscomplex)
    np.testing.assert_array_equal(m.row, orow)
    np.testing.assert_array_equal(m.col, ocol)
    np.testing.assert_array_equal(m.h, oh)
    assert m.norb == onorb


def test_oracle_rebuilds_cnt_device_from_coo(tmp_path):
    """The upper triangle of the test_cnt device Hamiltonian, written 1-based and complex,
    comes back as the test_cnt blocks: Hii = H00 (Hermitian fill), H1i(ix) = H_{ix,ix+1} =
    H10^dagger for the inner slabs, H1i(nx) = H1i(nx-1), Sii = I."""
    nx = 5
    H, H00, H10 = cnt_device(nx)
    bs = H00.shape[0]
    path = tmp_path / "h_dat"
    write_coo(path, *upper_entries(H), base=1, iscomplex=True)
    h, row0, col0, norb = ocoo.load_coo(str(path), use0index=False, iscomplex=True)
    assert norb // bs == nx
    Hii, H1i, Sii = ocoo.coo_blocks(nx, bs, row0, col0, h)
    for i in range(nx):
        np.testing.assert_array_equal(Hii[i], H00)
        np.testing.assert_array_equal(Sii[i], np.eye(bs))
    for i in range(nx - 1):
        np.testing.assert_array_equal(H1i[i], H10.conj().T)
    np.testing.assert_array_equal(H1i[nx], H1i[nx - 1])


def test_zero_based_file_drops_last_slab(tmp_path):
    """With use0index the reference takes nm from the 0-based indices, so nx = nm / bs is
    one slab short when the orbital count is a multiple of bs."""
    H, H00, _ = cnt_device(3)
    path = tmp_path / "h_dat"
    write_coo(path, *upper_entries(H), base=0, iscomplex=True)
    m = coo.load(str(path), use0index=True, iscomplex=True)
    assert m.slabs(H00.shape[0]) == 2


def test_oracle_later_entries_win():
    bs, nx = 2, 2
    row0 = np.array([0, 1, 0, 1, 2])
    col0 = np.array([1, 0, 2, 1, 1])  # (1,0) overwrites the conjugate fill of (0,1);
    h = np.array([1 + 1j, 5 + 0j, 7 + 2j, 3 - 1j, 9 + 9j])  # diagonal ends conjugated
    Hii, H1i, _ = ocoo.coo_blocks(nx, bs, row0, col0, h)
    assert Hii[0, 0, 1] == 5 and Hii[0, 1, 0] == 5
    assert Hii[0, 1, 1] == 3 + 1j
    assert H1i[0, 0, 0] == 7 + 2j
    assert np.all(Hii[1] == 0)  # (2,1) lies before slab 1's first column: dropped
