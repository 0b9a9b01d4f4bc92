"""Bond currents from the GPU sweep: the Jdens blocks of cuda_rgf_constblocksize
(src/cuda_rgf_mod.f90:293-318), their traces (bond_cur) in every precision, the CPU
routine's form on variable blocks (src/rgf_mod.f90:215-221), all against the oracle; and
current conservation along ballistic devices up to the 100 x 128 benchmark device."""
import numpy as np
import pytest

from oracle import rgf as orc
from quantum_transport_gb300 import rgf
from quantum_transport_gb300.devices import config_batched, make_chain_device
from tests.test_oracle_variable_blocks import variable_device

pytestmark = pytest.mark.gpu

MU = (0.1, -0.1)
LEAD = dict(eta_lead=1e-3, sancho_tol=1e-12)


def scattering(rng, npts, nx, n):
    """Diagonal scattering self-energies that make the current change along the device:
    Sigma^R = -i gamma/2 and Sigma^< = i gamma f, with random gamma and occupations f."""
    gam = 0.05 + 0.1 * rng.random((npts, nx, n))
    f = rng.random((npts, nx, n))
    sr = np.zeros((npts, nx, n, n), dtype=np.complex128)
    sl = np.zeros_like(sr)
    i = np.arange(n)
    sr[..., i, i] = -0.5j * gam
    sl[..., i, i] = 1j * gam * f
    return sr, sl


def oracle_point(dev, ie, ik, sr, sl, quirks, p):
    Hii = [dev.H00[ik]] * dev.nx
    H1i = [dev.H10] * (dev.nx + 1)
    return orc.rgf_constblocksize(dev.E[ie], Hii, H1i, sigma_lesser_ph=list(sl[p]),
                                  sigma_r_ph=list(sr[p]), mul=MU[0], mur=MU[1], templ=300.0,
                                  tempr=280.0, quirks=quirks, sancho_nmax=200, **LEAD)


def test_jdens_blocks_and_bond_cur_match_oracle(ctx):
    dev = make_chain_device(6, 16, 4, -2.0, 2.0, seed=21, nk=2)
    npts = len(dev.E) * dev.nk
    sr, sl = scattering(np.random.default_rng(1), npts, dev.nx, dev.nm)
    r = rgf.rgf_solve(ctx, dev.H00, dev.H10, dev.E, dev.nx, nk=dev.nk, mul=MU[0], mur=MU[1],
                      templ=300.0, tempr=280.0, sigma_r_ph=sr, sigma_lesser_ph=sl,
                      want_blocks=True, want_bond=True, sancho_max_iter=200, **LEAD)
    assert (r["status"] == 0).all()
    spread = 0.0
    for ie in range(len(dev.E)):
        for ik in range(dev.nk):
            o = oracle_point(dev, ie, ik, sr, sl, orc.QUIRKS_GOLDEN, ie * dev.nk + ik)
            exp = np.stack(o["Jdens"])
            got = r["Jdens"][ie, ik]
            np.testing.assert_allclose(got, exp, rtol=0, atol=1e-9 * np.abs(exp).max())
            assert not got[-1].any()  # Jdens(nx) is never written by the reference
            J = np.real(np.trace(exp[:-1], axis1=1, axis2=2))
            np.testing.assert_allclose(r["bond_cur"][ie, ik], J, rtol=0,
                                       atol=1e-9 * np.abs(J).max())
            spread = max(spread, np.ptp(J) / np.abs(J).max())
    assert spread > 1e-3  # the scattering really makes the currents differ between bonds


@pytest.mark.parametrize("precision,tol", [("fp64", 1e-9), ("mixed-fp64", 1e-8), ("mixed", 2e-4)])
def test_bond_cur_trace_form(ctx, precision, tol):
    """bond_cur alone (the 2-product trace form) in every precision."""
    dev = make_chain_device(5, 24, 5, -2.2, 2.2, seed=5, nk=1)
    npts = len(dev.E)
    sr, sl = scattering(np.random.default_rng(2), npts, dev.nx, dev.nm)
    r = rgf.rgf_solve(ctx, dev.H00, dev.H10, dev.E, dev.nx, mul=MU[0], mur=MU[1], templ=300.0,
                      tempr=280.0, sigma_r_ph=sr, sigma_lesser_ph=sl, want_diag=False,
                      want_bond=True, precision=precision, sancho_max_iter=200, **LEAD)
    assert (r["status"] == 0).all()
    for ie in range(npts):
        o = oracle_point(dev, ie, 0, sr, sl, orc.QUIRKS_GOLDEN, ie)
        J = np.real([np.trace(o["Jdens"][l]) for l in range(dev.nx - 1)])
        np.testing.assert_allclose(r["bond_cur"][ie, 0], J, rtol=0, atol=tol * np.abs(J).max())


def test_cpu_form_on_variable_blocks(ctx):
    """qt_rgf_solve_vb with the CPU routine's conventions: Jdens_l = -2 H^+ G^<_{l+1,l}."""
    Hii, H1i = variable_device(5)
    E = np.array([-1.9, -0.05, 0.1, 0.25])  # one energy outside the window: J = round-off
    kw = dict(mul=0.3, mur=-0.1, templ=300.0, tempr=300.0, eta_lead=1e-3, sancho_tol=1e-12)
    r = rgf.rgf_variableblock_forward(ctx, Hii, H1i, E, sancho_max_iter=200, want_bond=True,
                                      quirks=rgf._lib.QT_QUIRK_CPU_FERMI, **kw)
    assert (r["status"] == 0).all()
    J = np.array([np.real([np.trace(x) for x in orc.rgf_constblocksize(
        e, Hii, H1i, quirks=orc.QUIRKS_VARIABLE, sancho_nmax=200, **kw)["Jdens"][:-1]]) for e in E])
    assert np.abs(J).max() > 1.0
    np.testing.assert_allclose(r["bond_cur"][:, 0], J, rtol=0, atol=1e-9 * np.abs(J).max())


def test_ballistic_currents_are_conserved(ctx):
    """Without scattering every bond carries the terminal current tr."""
    dev = make_chain_device(12, 20, 40, -3.0, 3.0, seed=9, nk=2)
    for precision, tol in (("fp64", 1e-9), ("mixed", 1e-4)):
        r = rgf.rgf_solve(ctx, dev.H00, dev.H10, dev.E, dev.nx, nk=dev.nk, mul=MU[0], mur=MU[1],
                          want_diag=False, want_bond=True, precision=precision)
        ok = r["status"] == 0
        J, tr = r["bond_cur"][ok], r["tr"][ok]
        scale = np.abs(tr).max()
        assert scale > 0.1
        np.testing.assert_allclose(J, np.broadcast_to(tr[:, None], J.shape), rtol=0,
                                   atol=tol * scale)


def test_conservation_on_benchmark_device(ctx):
    """The 100-slab x 128-orbital device of the benchmark, 608 energies around the Fermi
    window x 1 k, complex64 sweep: bond currents equal tr within the storage precision."""
    dev = config_batched(nE=608, nk=1)
    E = np.linspace(-0.3, 0.3, 608)
    r = rgf.rgf_solve(ctx, dev.H00, dev.H10, E, dev.nx, nk=1, mul=0.1, mur=-0.1,
                      want_diag=False, want_bond=True, precision="mixed")
    ok = r["status"] == 0
    assert ok.mean() > 0.95
    J, tr = r["bond_cur"][ok], r["tr"][ok]
    scale = np.abs(tr).max()
    assert scale > 0.1
    assert np.abs(J - tr[:, None]).max() <= 1e-3 * scale
