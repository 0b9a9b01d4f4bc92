"""The test_cnt run on the GPU written as ldos/ndos/pdos0000.dat and compared with the
reference's files record by record (src/output_mod.f90:14-61)."""
import os

import numpy as np
import pytest

from quantum_transport_gb300 import rgf
from tests.goldutil import printed_match

pytestmark = pytest.mark.gpu
GOLDEN = os.path.join(os.path.dirname(__file__), "golden")


def fields(text):
    recs = text.split("\n")
    return recs, np.array([[float(l[i:i + 18]) for i in range(0, 72, 18)]
                           for l in recs if l.strip()])


def test_cnt_spectrum_files(ctx, cnt, tmp_path):
    r = rgf.negf_solve(ctx, cnt["H00"], cnt["H10"], int(cnt["nx"]), 200, -6.0, -1.0,
                       (300.0, 300.0), (-3.7, -3.7), int(cnt["nb"]), int(cnt["ns"]),
                       Lx=float(cnt["Lx"]), write_dir=str(tmp_path))
    assert (r["status"] == 0).all()
    gold = np.load(os.path.join(GOLDEN, "cnt_text.npz"))
    for path in r["files"]:
        name = os.path.basename(path)[:4]
        with open(path) as f:
            mine_text = f.read()
        ref_text = str(gold[name])
        mr, mv = fields(mine_text)
        rr, rv = fields(ref_text)
        assert len(mr) == len(rr) and mv.shape == rv.shape == (3000, 4)
        # layout, cell positions and energies are identical text
        assert [l == "" for l in mr] == [l == "" for l in rr]
        assert all(a[:36] == b[:36] for a, b in zip(mr, rr))
        # values: printed digits against printed digits, so a value on a rounding boundary
        # may differ by one unit in the last digit; the reference's round-off columns skipped
        for col in (2, 3):
            if name != "ldos" and col == 2:
                continue  # Re Tr G^< / G^> is round-off noise in the reference
            ok = printed_match(mv[:, col], rv[:, col], full=rv[:, col], units=1.01,
                               rel_floor=1e-10 if name == "ldos" else 1e-8)
            assert ok.all(), (name, col, np.argwhere(~ok)[:5])
        # the printed text itself is identical for nearly every record that carries data
        # (values above round-off: G^< above and G^> below the Fermi level are noise)
        data = [(a, b) for a, b in zip(mr, rr) if b]
        big = np.abs(rv[:, 3]) >= 1e-6 * np.abs(rv[:, 3]).max()
        keep = (lambda l: l) if name == "ldos" else (lambda l: l[:36] + l[54:])
        same = np.mean([keep(a) == keep(b) for (a, b), g in zip(data, big) if g])
        assert same > 0.97, (name, same)
