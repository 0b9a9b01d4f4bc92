"""The (4E18.4) spectrum writer: the Fortran edit descriptor, and the reference's
test_cnt/*0000.dat text rebuilt byte for byte from its printed values."""
import os

import numpy as np
import pytest

from quantum_transport_gb300 import output

GOLDEN = os.path.join(os.path.dirname(__file__), "golden")


@pytest.mark.parametrize("x,text", [
    (4.2755, "0.4276E+01"), (-6.0, "-0.6000E+01"), (0.0, "0.0000E+00"), (-0.0, "-0.0000E+00"),
    (9.99995, "0.1000E+02"), (1.234e-14, "0.1234E-13"), (1e-100, "0.1000E-99"),
    (1e-101, "0.1000-100"), (123456.0, "0.1235E+06")])
def test_fortran_e(x, text):
    assert output.fortran_e(x) == text.rjust(18)


@pytest.mark.parametrize("name", ["ldos", "ndos", "pdos"])
def test_reference_text_rebuilt(cnt, name):
    """Printed values -> records: the cell positions accumulate Lx, the energies are the
    grid of negf_solve, and the layout (blank record per energy) matches."""
    text = str(np.load(os.path.join(GOLDEN, "cnt_text.npz"))[name])
    vals = cnt[name]
    mine = output.format_records(vals[..., 0], vals[..., 1], cnt["E"], float(cnt["Lx"]))
    assert mine == text
