"""GW/SCBA GPU path against the FP64 GW oracle (parity of the reference unpinned:
its GW module does not build and has no fixtures)."""
import numpy as np
import pytest

from oracle import gw as ogw
from quantum_transport_gb300 import _lib as rgf_lib
from quantum_transport_gb300.devices import make_chain_device

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("n", [16, 64, 255, 2048])
def test_corr_conv_batch(ctx, n):
    import torch
    from quantum_transport_gb300 import gw
    rng = np.random.default_rng(n)
    X = rng.normal(size=(n, 5)) + 1j * rng.normal(size=(n, 5))
    Y = rng.normal(size=(n, 5)) + 1j * rng.normal(size=(n, 5))
    Xd, Yd = torch.from_numpy(X).cuda(), torch.from_numpy(Y).cuda()
    for mode, f in (("corr", ogw.corr), ("conv", ogw.conv)):
        Z = gw.corr(ctx, Xd, Yd, mode).cpu().numpy()
        ref = f(X.T, Y.T).T
        np.testing.assert_allclose(Z, ref, rtol=0, atol=1e-11 * np.abs(ref).max())
    if n <= 64:
        np.testing.assert_allclose(gw.corr(ctx, Xd, Yd, "corr").cpu().numpy(),
                                   ogw.corr_direct(X.T, Y.T).T, atol=1e-10)


def _system(ctx, precision="fp64"):
    from quantum_transport_gb300 import gw
    dev = make_chain_device(6, 8, 64, -4.0, 4.0, seed=3)
    V = ogw.coulomb_blocks(8)
    s = gw.GwSystem(ctx, dev.H00[0], dev.H10, dev.E, dev.nx, V, mu=(0.1, -0.1),
                    precision=precision)
    return dev, V, s


def test_gw_step_vs_oracle(ctx):
    from quantum_transport_gb300 import gw
    dev, V, s = _system(ctx)
    # the self-energies also enter the leads' decimation (src/gw_mod.f90:1173): they must
    # only broaden, or the decimation diverges
    SR0, SL0 = _physical_sigma(len(dev.E), dev.nx, 8)
    NR, NL, NG = s.step(gw.to_dev(SR0), gw.to_dev(SL0))
    GR, GL, GG = ogw.green(dev.E, dev.H00[0], dev.H10, dev.nx, SR0, SL0, mu=(0.1, -0.1),
                           temp=(300.0, 300.0))
    GR, GL, GG = ogw.zero_real(GR, GL, GG)
    dE = dev.E[1] - dev.E[0]
    P = ogw.polarization(GR, GL, GG, dE)
    W = ogw.screened(V, *P)
    ref = [ogw.copy_edges(x) for x in ogw.self_energy(GR, GL, GG, *W, dE)]
    for got, exp in zip((NR, NL, NG), ref):
        g = gw.from_dev(got)
        assert np.isfinite(exp).all() and np.abs(exp).max() > 0
        np.testing.assert_allclose(g, exp, rtol=0, atol=1e-8 * np.abs(exp).max(),
                                   equal_nan=False)


def test_scba_converges_like_oracle(ctx):
    from quantum_transport_gb300 import gw
    dev, V, s = _system(ctx)
    SR, SL, SG, res = s.scba(alpha=0.3, tol=1e-8, max_iter=80)
    assert res[-1] <= 1e-8
    oR, oL, oG, ores = ogw.scba(dev.E, dev.H00[0], dev.H10, V, dev.nx, mu=(0.1, -0.1),
                               temp=(300.0, 300.0), max_iter=80)
    assert abs(len(res) - len(ores)) <= 1
    for got, exp in zip((SR, SL, SG), (oR, oL, oG)):
        np.testing.assert_allclose(gw.from_dev(got), exp, rtol=0, atol=1e-7 * np.abs(exp).max())


def _physical_sigma(nE, nx, nm, seed=0):
    """Sigma^R = -i Gamma/2, Sigma^< = i f Gamma with Gamma Hermitian positive semidefinite
    and 0 < f < 1: broadening only, so the leads' decimation stays bounded."""
    rng = np.random.default_rng(seed)
    X = 0.1 * (rng.normal(size=(nE, nx, nm, nm)) + 1j * rng.normal(size=(nE, nx, nm, nm)))
    gam = X @ np.conj(np.swapaxes(X, -1, -2)) / nm
    f = rng.random((nE, nx, 1, 1))
    return -0.5j * gam, 1j * f * gam


def test_gw_currents_vs_oracle(ctx):
    """tr, tre and the bond currents (traces of cur, src/gw_mod.f90:1254-1276) of the GW
    RGF at given self-energies."""
    from oracle import rgf as orc
    from quantum_transport_gb300 import gw
    dev, V, s = _system(ctx)
    SR0, SL0 = _physical_sigma(len(dev.E), dev.nx, 8)
    c = s.currents(gw.to_dev(SR0), gw.to_dev(SL0))
    # the decimation runs the reference's fixed 100 steps (TOL = 1e-100), so only the
    # "not converged" bit may be set
    assert ((c["status"] & ~rgf_lib.QT_PT_SANCHO_NOT_CONVERGED) == 0).all()
    Hii, H1i = [dev.H00[0]] * dev.nx, [dev.H10] * (dev.nx + 1)
    Js = []
    for ie, e in enumerate(dev.E):
        o = orc.rgf_constblocksize(e, Hii, H1i, None, list(SL0[ie]), list(SR0[ie]), mul=0.1,
                                   mur=-0.1, templ=300.0, tempr=300.0, eta_lead=1e-3,
                                   sancho_nmax=100, sancho_tol=1e-100)
        J = np.real([np.trace(o["Jdens"][l]) for l in range(dev.nx - 1)])
        Js.append(J)
        np.testing.assert_allclose(c["tr"][ie], o["tr"], rtol=1e-8, atol=1e-12)
        np.testing.assert_allclose(c["tre"][ie], o["tre"], rtol=1e-8, atol=1e-12)
        np.testing.assert_allclose(c["bond_cur"][ie], J, rtol=0,
                                   atol=1e-9 * max(np.abs(J).max(), 1e-12))
    assert np.abs(np.array(Js)).max() > 1e-3


def test_scba_iteration_currents(ctx):
    """The Id_iteration.dat columns of qt_scba_solve are the terminal currents of the RGF at
    each iteration's self-energies: sum_E tre and sum_E tr x dE e0^2 spindeg / (2 pi hbar)."""
    from quantum_transport_gb300 import currents
    dev, V, s = _system(ctx)
    _, _, _, res, cur = s.scba(alpha=0.3, tol=0.0, max_iter=3, with_currents=True)
    assert cur.shape == (3, 2)
    z = s.zeros()
    c0 = s.currents(z, z)
    expect0 = [currents.terminal_current(c0["tre"], dev.E), currents.terminal_current(c0["tr"], dev.E)]
    np.testing.assert_allclose(cur[0], expect0, rtol=1e-10)
    SR1, SL1, _, _ = s.scba(alpha=0.3, tol=0.0, max_iter=1)  # the iterate the second map sees
    c1 = s.currents(SR1, SL1)
    expect1 = [currents.terminal_current(c1["tre"], dev.E), currents.terminal_current(c1["tr"], dev.E)]
    np.testing.assert_allclose(cur[1], expect1, rtol=1e-10)
    assert abs(cur[0, 0]) > 0 and not np.allclose(cur[0], cur[1], rtol=1e-6)


@pytest.mark.parametrize("precision,tol", [("fp64", 1e-12), ("mixed", 1e-11)])
def test_ephoton_sigma_vs_oracle(ctx, precision, tol):
    """qt_ephoton_sigma against calc_sigma_ephoton_monochromatic_ext restated, on one shard
    (zeros beyond the grid) and on an inner shard with its energy halo."""
    from quantum_transport_gb300 import gw
    rng = np.random.default_rng(7)
    nE, nx, nm, nop = 24, 4, 12, 3
    shape = (nE, nx, nm, nm)
    GL = 1e-2 * (rng.normal(size=shape) + 1j * rng.normal(size=shape))
    GG = 1e-2 * (rng.normal(size=shape) + 1j * rng.normal(size=shape))
    M = rng.normal(size=(nx, nm, nm)) + 1j * rng.normal(size=(nx, nm, nm))
    intensity, hw = 1e9, 1.5
    ref = ogw.ephoton_sigma(M, GL, GG, nop, ogw.PHOTON_PRE_FACT, intensity, hw)
    got = gw.ephoton_sigma(ctx, gw.to_dev(M), gw.to_dev(GL), gw.to_dev(GG), nop, intensity, hw,
                           precision=precision)
    for g, r in zip(got, ref):
        np.testing.assert_allclose(gw.from_dev(g), r, rtol=0, atol=tol * np.abs(r).max())
    lo, hi = 8, 16  # an inner shard: its halo is the neighbours' energies
    got = gw.ephoton_sigma(ctx, gw.to_dev(M), gw.to_dev(GL[lo - nop:hi + nop]),
                           gw.to_dev(GG[lo - nop:hi + nop]), nop, intensity, hw, halo=True,
                           precision=precision)
    for g, r in zip(got, ref):
        np.testing.assert_allclose(gw.from_dev(g), r[lo:hi], rtol=0, atol=tol * np.abs(r).max())
    assert not gw.from_dev(got[0]).real.any()  # Sigma^R is purely imaginary


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_sancho_reset_on_nmax_vs_oracle(ctx, precision):
    """green_RGF_RS's decimation (src/gw_mod.f90:1440-1445): an entry still unconverged after
    nmax steps restarts from H_SS = H_BB = H00.  With 12 steps at eta = 1e-3 the energies
    outside the band converge in 7-9 steps and those inside reach nmax, so both branches are
    checked."""
    from oracle import rgf as orc
    from quantum_transport_gb300 import rgf
    dev = make_chain_device(2, 8, 24, -9.0, 9.0, seed=5)
    H00, H10, E = dev.H00[0], dev.H10, dev.E
    nmax, tol = 12, 1e-30
    S = np.eye(8, dtype=np.complex128)
    G00, GBB, it, st = rgf.sancho(ctx, E, H00, H10, eta=1e-3, tol=tol, max_iter=nmax,
                                  precision=precision, reset_on_nmax=True)
    hit = it >= nmax
    assert 0 < hit.sum() < len(E)
    tol_rel = 1e-10 if precision == "fp64" else 1e-9
    for ie, e in enumerate(E):
        g00, gbb, oit, _, _ = orc.sancho(e, S, H00, H10, eta=1e-3, nmax=nmax, tol=tol,
                                         reset_on_nmax=True)
        assert (oit >= nmax) == hit[ie]
        for got, exp in ((G00[ie], g00), (GBB[ie], gbb)):
            np.testing.assert_allclose(got, exp, rtol=0, atol=tol_rel * np.abs(exp).max())
        if hit[ie]:
            # the reset leaves the isolated-slab function in both
            bare = np.linalg.inv(complex(e, 1e-3) * S - H00)
            np.testing.assert_allclose(G00[ie], bare, rtol=0, atol=tol_rel * np.abs(bare).max())
    # without the reset the unconverged entries keep their last iterate
    G00n, _, _, _ = rgf.sancho(ctx, E, H00, H10, eta=1e-3, tol=tol, max_iter=nmax,
                               precision=precision)
    assert not np.allclose(G00n[hit], G00[hit])
    np.testing.assert_array_equal(G00n[~hit], G00[~hit])


def test_gw_green_with_sancho_reset_vs_oracle(ctx):
    """qt_rgf_solve under QT_QUIRK_GW_SANCHO_RESET (green_RGF_RS as written) against the
    oracle's green() with the same reset.  At TOL = 1e-100 this device's decimations finish
    within 100 steps, so the step limit is lowered to 12 and the window widened to
    [-9, 9] eV: the in-band energies then reach the limit and restart from H00, the
    others converge."""
    from quantum_transport_gb300 import gw
    dev = make_chain_device(6, 8, 64, -9.0, 9.0, seed=3)
    V = ogw.coulomb_blocks(8)
    SR0, SL0 = _physical_sigma(len(dev.E), dev.nx, 8)
    out = {}
    for reset in (False, True):
        s = gw.GwSystem(ctx, dev.H00[0], dev.H10, dev.E, dev.nx, V, mu=(0.1, -0.1),
                        sancho_max_iter=12, sancho_reset=reset)
        c = s.currents(gw.to_dev(SR0), gw.to_dev(SL0))
        out[reset] = c
        GR, GL, GG = ogw.green(dev.E, dev.H00[0], dev.H10, dev.nx, SR0, SL0, mu=(0.1, -0.1),
                               temp=(300.0, 300.0), sancho_nmax=12, sancho_reset=reset)
        ref = np.stack([np.diagonal(GR[ie], axis1=-2, axis2=-1) for ie in range(len(dev.E))])
        got = c["diag_gr"].reshape(ref.shape)
        np.testing.assert_allclose(got, ref, rtol=0, atol=1e-8 * np.abs(ref).max())
    hit = (out[True]["status"] & rgf_lib.QT_PT_SANCHO_NOT_CONVERGED) != 0
    assert hit.any() and not hit.all()
    assert not np.allclose(out[True]["diag_gr"].reshape(len(dev.E), -1)[hit],
                           out[False]["diag_gr"].reshape(len(dev.E), -1)[hit])


def test_profiler_times_the_map_phases(ctx):
    """With the context's profiler on, one SCBA iteration records each phase of the map once
    (the correlations twice: P, then Sigma), and the phases fit inside the iteration's own
    event time on the same stream."""
    import torch
    dev, V, s = _system(ctx)
    ctx.profile_read()
    ctx.profile(True)
    try:
        ev = [torch.cuda.Event(enable_timing=True) for _ in range(2)]
        ev[0].record()
        s.scba(alpha=0.3, tol=0.0, max_iter=1)
        ev[1].record()
        torch.cuda.synchronize()
    finally:
        ctx.profile(False)
        prof = ctx.profile_read()
    phases = ("gw_rgf", "gw_corrconv", "gw_screened", "gw_post")
    assert {k: prof[k][0] for k in phases} == {"gw_rgf": 1, "gw_corrconv": 2,
                                               "gw_screened": 1, "gw_post": 1}
    assert all(prof[k][1] > 0 for k in phases[:3]) and prof["gw_post"][1] >= 0
    assert sum(prof[k][1] for k in phases) <= ev[0].elapsed_time(ev[1]) + 0.05
