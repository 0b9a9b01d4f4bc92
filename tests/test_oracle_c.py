"""The C restatement (timed CPU baseline) agrees with the numpy oracle."""
import numpy as np
import pytest

from oracle import cref
from oracle import rgf as orc
from quantum_transport_gb300.devices import make_chain_device


@pytest.mark.parametrize("nm", [7, 12])
def test_c_oracle_matches_numpy_oracle(nm):
    """nm = 7 pads the block product's 4-row panels and 2- or 4-column panels with zeros."""
    dev = make_chain_device(6, nm, 4, -2.5, 2.5, seed=5, nk=2)
    # the C restatement takes slab-identical blocks: use the uniform device
    r = cref.rgf(dev.H00, dev.H10, dev.E, dev.nx, mul=0.1, mur=-0.1, templ=300, tempr=280)
    assert (r["status"] == 0).all()
    for ie, E in enumerate(dev.E):
        for ik in range(dev.nk):
            Hii = [dev.H00[ik]] * dev.nx
            H1i = [dev.H10] * (dev.nx + 1)
            o = orc.rgf_constblocksize(E, Hii, H1i, mul=0.1, mur=-0.1, templ=300, tempr=280)
            np.testing.assert_allclose(r["tr"][ie, ik], o["tr"], rtol=1e-9, atol=1e-12)
            np.testing.assert_allclose(r["tre"][ie, ik], o["tre"], rtol=1e-9, atol=1e-12)
            np.testing.assert_allclose(r["diag_gr"][ie, ik], o["diag_Gr"], atol=1e-10)
            np.testing.assert_allclose(r["diag_gl"][ie, ik], o["diag_Gl"], atol=1e-10)
            t = orc.caroli_transmission(E, Hii, H1i)
            np.testing.assert_allclose(r["T"][ie, ik], t, rtol=1e-9)


def test_c_oracle_cnt_golden(cnt):
    from tests.goldutil import printed_match
    idx = np.arange(0, 200, 40)
    r = cref.rgf(cnt["H00"], cnt["H10"], cnt["E"][idx], int(cnt["nx"]), mul=-3.7, mur=-3.7)
    lt = r["diag_gr"][:, 0].reshape(len(idx), -1, 32).sum(-1)
    assert printed_match(-2 * lt.imag, cnt["ldos"][idx, :, 1], full=cnt["ldos"][:, :, 1]).all()
