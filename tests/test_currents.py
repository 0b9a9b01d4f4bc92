"""Energy integrals of the currents (host side): the Id_iteration.dat prefactor and the
per-bond integrals, against the reference's formula written out."""
import numpy as np

from quantum_transport_gb300 import currents


def test_terminal_current_is_the_reference_formula():
    E = np.linspace(-1.0, 1.0, 201)
    tr = np.exp(-E ** 2)
    spindeg, nk = 2.0, 4
    # src/gw_mod.f90:427 with e0, hbar of src/static.f90 and tpi of src/fft_mod.f90
    ref = np.sum(tr) * (E[1] - E[0]) * 1.6022e-19 / (3.14159265359 * 2.0) / 1.0546e-34 \
        * 1.6022e-19 * spindeg / nk
    np.testing.assert_allclose(currents.terminal_current(tr, E, spindeg, nk), ref, rtol=1e-14)


def test_block_current_shapes_and_energy_weight():
    rng = np.random.default_rng(0)
    E = np.linspace(-0.5, 0.5, 11)
    J = rng.normal(size=(11, 3, 5))
    I, EI = currents.block_current(J, E, spindeg=1.0, nk=3)
    f = currents.prefactor(E[1] - E[0], 1.0, 3)
    assert I.shape == EI.shape == (3, 5)
    np.testing.assert_allclose(I, J.sum(axis=0) * f, rtol=1e-14)
    np.testing.assert_allclose(EI, (E[:, None, None] * J).sum(axis=0) * f, rtol=1e-14)
    I1, _ = currents.block_current(J[:, 0, :], E, spindeg=1.0, nk=3)
    np.testing.assert_allclose(I1[0], I[0], rtol=1e-14)
