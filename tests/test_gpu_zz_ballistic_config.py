"""The reference's CPU-runnable case at full size: 64 slabs x 32 orbitals, 512 energies on
[-3, 3] eV, eta = 1e-5 leads, Sancho tol 1e-10, mu = +-0.1 eV, kT = 0.025 eV.  All three
paths against the C restatement of the reference sweep on every point.

The device is well conditioned: all 32 channels are open across the window (T = 32 -
O(1e-9)), and the C restatement and the LAPACK oracle agree to 2e-14 in T and 7e-9 in the
LDOS and diag G^< (relative to each point's largest entry).  The bars leave a wide margin
over those spreads and over the split modes' errors on the 100 x 128 benchmark device."""
import numpy as np
import pytest

from quantum_transport_gb300.devices import config_ballistic_small

pytestmark = pytest.mark.gpu

TEMP = 0.025 / 8.61734e-05  # kT = 0.025 eV
KW = dict(mul=0.1, mur=-0.1, templ=TEMP, tempr=TEMP, sancho_tol=1e-10)


@pytest.fixture(scope="module")
def case():
    from oracle import cref
    d = config_ballistic_small()
    return d, cref.rgf(d.H00, d.H10, d.E, d.nx, **KW)


# mixed: an emulation that rounds every stored block of the sweep to complex64 (H, g_l, the
# Caroli chain; leads in FP64) gives T errors of 2.0e-7 at most, 5e-8 median on this device
@pytest.mark.parametrize("precision,t_max,t_med,d_max,d_med", [
    ("fp64", 1e-9, 1e-12, 1e-6, 1e-7),
    ("mixed-fp64", 1e-7, 1e-8, 1e-5, 1e-7),
    ("mixed", 2e-6, 5e-7, 1e-3, 5e-5)])
def test_paths_vs_c_restatement(ctx, case, precision, t_max, t_med, d_max, d_med):
    from quantum_transport_gb300 import rgf
    d, ref = case
    r = rgf.rgf_solve(ctx, d.H00, d.H10, d.E, d.nx, precision=precision, caroli=True,
                      want_diag=True, **KW)
    assert (ref["status"] == 0).all() and (r["status"] == 0).all()
    assert np.abs(ref["T"]).min() > 31.0
    eT = np.abs(r["T"] - ref["T"]) / np.abs(ref["T"])
    assert eT.max() <= t_max and np.median(eT) <= t_med
    npts = d.E.size
    assert np.isfinite(r["diag_gr"]).all() and np.isfinite(r["diag_gl"]).all()
    for x, y in ((r["diag_gr"].imag, ref["diag_gr"].imag), (r["diag_gl"], ref["diag_gl"])):
        x, y = x.reshape(npts, -1), y.reshape(npts, -1)
        scale = np.abs(y).max(axis=1)
        err = np.abs(x - y).max(axis=1) / scale
        if precision == "mixed":
            # complex64 storage resolves G^< down to ~1e-33 (FP32's normal range); above
            # E = mu + 76 kT (about 2 eV here) f and G^< fall below it and are flushed
            keep = scale >= 1e-33
            assert keep.mean() >= 0.75
            err = err[keep]
        assert err.max() <= d_max and np.median(err) <= d_med
