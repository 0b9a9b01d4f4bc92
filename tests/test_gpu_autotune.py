"""The wave size changes the schedule, not the results: the batched sweeps give bit-identical
outputs at every wave size the autotuner may pick; and the autotuner sets its choice."""
import numpy as np
import pytest

from quantum_transport_gb300 import rgf
from quantum_transport_gb300.devices import make_chain_device

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("precision", ["fp64", "mixed", "mixed-fp64"])
def test_results_do_not_depend_on_the_wave(ctx, precision):
    dev = make_chain_device(6, 32, 40, -2.0, 2.0, seed=9, nk=2)   # 80 points
    kw = dict(nk=dev.nk, mul=0.1, mur=-0.1, sancho_tol=1e-10, caroli=True,
              precision=precision)
    outs = []
    try:
        for wave in (0, 16, 30, 80):   # default, several waves (one ragged), one wave
            ctx.set_wave_points(wave)
            outs.append(rgf.rgf_solve(ctx, dev.H00, dev.H10, dev.E, dev.nx, **kw))
    finally:
        ctx.set_wave_points(0)
    for o in outs[1:]:
        for k in ("T", "tr", "tre", "diag_gr", "diag_gl", "status"):
            np.testing.assert_array_equal(o[k], outs[0][k], err_msg=k)


def test_tune_wave_sets_the_fastest(ctx):
    from quantum_transport_gb300 import autotune
    dev = make_chain_device(4, 16, 32, -2.0, 2.0, seed=2, nk=1)
    run = lambda: rgf.rgf_solve(ctx, dev.H00, dev.H10, dev.E, dev.nx, precision="mixed")
    try:
        best, ms = autotune.tune_wave(ctx, run, 32, cands=[8, 16, 32])
        assert best in (8, 16, 32) and set(ms) == {8, 16, 32}
        assert ms[best] == min(ms.values())
    finally:
        ctx.set_wave_points(0)


@pytest.mark.parametrize("precision", ["fp64", "mixed", "mixed-fp64"])
def test_variable_block_results_do_not_depend_on_the_wave(ctx, precision):
    """The same for the variable-block sweep, with blocks above one 128-row tile (tiled
    products, 2 x 2 block inverses)."""
    from tests.test_oracle_variable_blocks import variable_device
    Hii, H1i = variable_device(4, sizes=(40, 150, 97, 133))
    E = np.linspace(-2.0, 2.0, 24)
    kw = dict(mul=0.1, mur=-0.1, sancho_tol=1e-10, caroli=True, precision=precision)
    outs = []
    try:
        for wave in (0, 5, 24):
            ctx.set_wave_points(wave)
            outs.append(rgf.rgf_variableblock_forward(ctx, Hii, H1i, E, **kw))
    finally:
        ctx.set_wave_points(0)
    for o in outs[1:]:
        for k in ("T", "tr", "tre", "status"):
            np.testing.assert_array_equal(o[k], outs[0][k], err_msg=k)
        for a, b in zip(o["diag_gr"], outs[0]["diag_gr"]):
            np.testing.assert_array_equal(a, b)
