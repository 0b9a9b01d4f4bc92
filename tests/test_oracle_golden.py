"""The oracle against the reference's own known-answer outputs (test_cnt/)."""
import numpy as np
import pytest

from oracle import rgf
from tests.goldutil import printed_match

# a spread of energies keeps the CPU suite short; the full 200-energy sweep is
# exercised by the GPU parity tests
SUBSET = list(range(0, 200, 19)) + [199]


def _device(cnt):
    nx = int(cnt["nx"])
    return [cnt["H00"]] * nx, [cnt["H10"]] * (nx + 1)


@pytest.mark.parametrize("ie", SUBSET[:6])
def test_sancho_traces(cnt, ie):
    """-Im Tr G00 / GBB of both leads to ~1e-11 (files carry full precision)."""
    E = cnt["E"][ie]
    H00, H10 = cnt["H00"], cnt["H10"]
    S = np.eye(H00.shape[0])
    gl = rgf.sancho(E, S, H00, H10.conj().T)   # left lead: called with H10^+
    gr = rgf.sancho(E, S, H00, H10)
    for j, g in enumerate((gl, gr)):
        np.testing.assert_allclose(-np.trace(g[0]).imag, cnt["sancho_g00"][ie, j], rtol=1e-10)
        np.testing.assert_allclose(-np.trace(g[1]).imag, cnt["sancho_gbb"][ie, j], rtol=1e-10)


@pytest.mark.parametrize("ie", SUBSET)
def test_spectra(cnt, ie):
    Hii, H1i = _device(cnt)
    E = cnt["E"][ie]
    o = rgf.rgf_constblocksize(E, Hii, H1i, mul=-3.7, mur=-3.7)
    nb, ns = int(cnt["nb"]), int(cnt["ns"])
    lt = rgf.cell_traces(o["diag_Gr"], nb, ns)
    nt = rgf.cell_traces(o["diag_Gl"], nb, ns)
    pt = rgf.cell_traces(o["diag_Gg"], nb, ns)
    check_spectra(cnt, ie, lt, nt, pt)


def check_spectra(cnt, ie, lt, nt, pt):
    """Per-cell traces against ldos/ndos/pdos0000.dat (coefficients of
    src/negf_mod.f90:142-149: ldos (1,-2), ndos (1,1), pdos (1,-1))."""
    for mine, name, col, c in ((lt.real, "ldos", 0, 1), (lt.imag, "ldos", 1, -2),
                               (nt.imag, "ndos", 1, 1), (pt.imag, "pdos", 1, -1)):
        gold = cnt[name][ie, :, col]
        ok = printed_match(c * mine, gold, full=cnt[name][:, :, col])
        assert ok.all(), (name, col, (c * mine)[~ok], gold[~ok])


def test_glp_quirk_is_refuted(cnt):
    """The GPU routine's Glp==0 G^> recursion does NOT reproduce pdos0000.dat."""
    Hii, H1i = _device(cnt)
    ie = 100  # above mu: f ~ 0, G^> carries the full spectral weight
    o = rgf.rgf_constblocksize(cnt["E"][ie], Hii, H1i, mul=-3.7, mur=-3.7, quirks=rgf.QUIRKS_CUDA)
    pt = rgf.cell_traces(o["diag_Gg"], int(cnt["nb"]), int(cnt["ns"]))
    assert not printed_match(-pt.imag, cnt["pdos"][ie, :, 1], full=cnt["pdos"][:, :, 1]).all()
