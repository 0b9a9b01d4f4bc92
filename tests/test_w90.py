"""Wannier90 model input: the package's reader against the oracle's on a synthetic file."""
import numpy as np

from oracle.w90 import W90
from quantum_transport_gb300 import w90


def synthetic_model(rng, nb=4, rx=(-2, 2), ry=(-1, 1), rz=(0, 1)):
    shape = (nb, nb, rx[1] - rx[0] + 1, ry[1] - ry[0] + 1, rz[1] - rz[0] + 1)
    Hr = 0.3 * (rng.normal(size=shape) + 1j * rng.normal(size=shape))
    cell = np.array([[2.5, 0.1, 0.0], [0.0, 7.0, 0.2], [0.1, 0.0, 6.0]])
    return Hr, rx + ry + rz, cell


def write_model(path, Hr, ranges, cell):
    nb = Hr.shape[0]
    rows = []
    for ix in range(Hr.shape[2]):
        for iy in range(Hr.shape[3]):
            for iz in range(Hr.shape[4]):
                for n in range(nb):
                    for m in range(nb):
                        h = Hr[m, n, ix, iy, iz]
                        rows.append(f"{ix + ranges[0]} {iy + ranges[2]} {iz + ranges[4]} "
                                    f"{m + 1} {n + 1} {h.real:.17g} {h.imag:.17g}")
    with open(path, "w") as f:
        f.write(f"{nb} 2\ncell\n")
        for v in cell:
            f.write(" ".join(f"{x:.17g}" for x in v) + "\n")
        f.write(f"hamiltonian\n{len(rows)}\n" + "\n".join(rows) + "\n")


def test_reader_matches_oracle(tmp_path):
    Hr, ranges, cell = synthetic_model(np.random.default_rng(1))
    path = tmp_path / "ham_dat"
    write_model(path, Hr, ranges, cell)
    m = w90.load(str(path))
    o = W90(str(path))
    np.testing.assert_array_equal(m.Hr, o.Hr)
    assert m.ranges == (o.xmin, o.xmax, o.ymin, o.ymax, o.zmin, o.zmax)
    for a, b in zip(m.axes, (o.xhat, o.yhat, o.zhat)):
        np.testing.assert_allclose(a, b, rtol=0, atol=1e-15)
    assert abs(m.Lx - o.Lx) <= 1e-15
