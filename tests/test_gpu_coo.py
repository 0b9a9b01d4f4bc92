"""COO block builder on the GPU (qt_coo_blocks) against the oracle's serial loop: bit-exact,
including duplicates, conflicting conjugate fills, dropped entries and overlaps."""
import numpy as np
import pytest

from oracle import coo as ocoo
from quantum_transport_gb300 import coo
from test_coo import cnt_device, upper_entries, write_coo

pytestmark = pytest.mark.gpu


def messy_entries(rng, nx, bs, n):
    """Random entries over slabs 0..nx (one past the end), columns from two slabs before to
    three after, with many repeated (row, col) pairs and diagonal hits."""
    norb = nx * bs
    row0 = rng.integers(0, norb + bs, n)
    col0 = np.clip(row0 + rng.integers(-2 * bs, 3 * bs, n), 0, None)
    dup = rng.random(n) < 0.3
    row0[dup] = row0[rng.integers(0, n, dup.sum())]
    diag = rng.random(n) < 0.1
    col0[diag] = row0[diag]
    h = rng.normal(size=n) + 1j * rng.normal(size=n)
    return row0.astype(np.int32), col0.astype(np.int32), h


@pytest.mark.parametrize("nx,bs,n,with_s", [(3, 4, 400, False), (4, 17, 5000, True),
                                            (6, 96, 60000, False), (2, 128, 40000, True)])
def test_matches_oracle_bit_exact(ctx, nx, bs, n, with_s):
    rng = np.random.default_rng(nx * 1000 + bs)
    row0, col0, h = messy_entries(rng, nx, bs, n)
    s = rng.normal(size=n) + 1j * rng.normal(size=n) if with_s else None
    m = coo.CooMatrix(row0, col0, h, nx * bs)
    Hii, H1i, Sii = coo.device_blocks(ctx, m, bs, s=s)
    oHii, oH1i, oSii = ocoo.coo_blocks(nx, bs, row0, col0, h, s)
    np.testing.assert_array_equal(Hii, oHii)
    np.testing.assert_array_equal(H1i, oH1i)
    np.testing.assert_array_equal(Sii, oSii)


def test_cnt_device_from_coo_file(ctx, tmp_path):
    nx = 5
    H, H00, H10 = cnt_device(nx)
    path = tmp_path / "h_dat"
    write_coo(path, *upper_entries(H), base=1, iscomplex=True)
    m = coo.load(str(path), iscomplex=True)
    Hii, H1i, Sii = coo.device_blocks(ctx, m, H00.shape[0])
    for i in range(nx):
        np.testing.assert_array_equal(Hii[i], H00)
        np.testing.assert_array_equal(Sii[i], np.eye(H00.shape[0]))
    for i in range(nx - 1):
        np.testing.assert_array_equal(H1i[i], H10.conj().T)
    np.testing.assert_array_equal(H1i[nx], H1i[nx - 1])


def test_no_entries(ctx):
    z = np.zeros(0, dtype=np.int32)
    m = coo.CooMatrix(z, z, np.zeros(0, dtype=np.complex128), 8)
    Hii, H1i, Sii = coo.device_blocks(ctx, m, 4)
    assert not Hii.any() and not H1i.any()
    np.testing.assert_array_equal(Sii, np.broadcast_to(np.eye(4), (2, 4, 4)))


def test_one_based_indices_on_device_pointers(ctx):
    """index_base = 1 with device pointers, the form a Fortran caller hands over."""
    import ctypes as C
    import torch
    rng = np.random.default_rng(11)
    nx, bs, n = 3, 8, 700
    row0, col0, h = messy_entries(rng, nx, bs, n)
    dev = torch.device("cuda", 0)
    row = torch.from_numpy(row0 + 1).to(dev)
    col = torch.from_numpy(col0 + 1).to(dev)
    hv = torch.from_numpy(h).to(dev)
    Hii = torch.empty((nx, bs, bs), dtype=torch.complex128, device=dev)
    H1i = torch.empty((nx + 1, bs, bs), dtype=torch.complex128, device=dev)
    Sii = torch.empty_like(Hii)
    p = lambda t: C.c_void_p(t.data_ptr())
    from quantum_transport_gb300._lib import check, QT_FLAG_DEVICE_POINTERS, QT_FLAG_SYNC
    check(ctx._lib.qt_coo_blocks(ctx.handle, nx, bs, n, p(row), p(col), 1, p(hv), None,
                                 p(Hii), p(H1i), p(Sii), QT_FLAG_DEVICE_POINTERS | QT_FLAG_SYNC))
    oHii, oH1i, _ = ocoo.coo_blocks(nx, bs, row0, col0, h)
    np.testing.assert_array_equal(Hii.transpose(-1, -2).cpu().numpy(), oHii)
    np.testing.assert_array_equal(H1i.transpose(-1, -2).cpu().numpy(), oH1i)
