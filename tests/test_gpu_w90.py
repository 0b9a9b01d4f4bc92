"""Slab blocks of a Wannier90 model built on the GPU (w90_MAT_DEF,
src/wannierHam3d.f90:273-301) against the oracle and the test_cnt fixture."""
import os

import numpy as np
import pytest

from oracle.w90 import W90
from quantum_transport_gb300 import w90
from tests.test_w90 import synthetic_model

pytestmark = pytest.mark.gpu

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def test_cnt_blocks_match_fixture(ctx):
    f = np.load(os.path.join(GOLDEN, "cnt_hr.npz"))
    b = np.load(os.path.join(GOLDEN, "cnt_blocks.npz"))
    model = w90.W90Model(f["Hr"], tuple(int(x) for x in f["ranges"]), f["alpha"], f["beta"],
                         f["gamm"])
    H00, H10 = w90.slab_blocks(ctx, model, int(b["ns"]))
    np.testing.assert_allclose(H00[0], b["H00"], rtol=0, atol=1e-14)
    np.testing.assert_allclose(H10[0], b["H10"], rtol=0, atol=1e-14)
    assert abs(model.Lx - float(b["Lx"])) < 1e-12


@pytest.mark.parametrize("ns", [1, 3])
def test_blocks_at_transverse_k_match_oracle(ctx, ns):
    Hr, ranges, cell = synthetic_model(np.random.default_rng(2))
    model = w90.W90Model(Hr, ranges, *cell)
    o = W90.from_arrays(Hr, ranges, *cell)
    kx = np.array([0.0, 0.1, -0.2, 0.05])
    ky = np.array([0.0, 0.3, 0.4, -0.7])
    kz = np.array([0.0, -0.5, 0.2, 0.9])
    H00, H10 = w90.slab_blocks(ctx, model, ns, kx, ky, kz)
    for i in range(len(kx)):
        r00, r10 = o.mat_def(ns, kx[i], ky[i], kz[i])
        np.testing.assert_allclose(H00[i], r00, rtol=0, atol=1e-12)
        np.testing.assert_allclose(H10[i], r10, rtol=0, atol=1e-12)
