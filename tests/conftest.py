import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)
GOLDEN = os.path.join(ROOT, "tests", "golden")


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a)")


@pytest.fixture(scope="session")
def cnt():
    import numpy as np
    b = np.load(os.path.join(GOLDEN, "cnt_blocks.npz"))
    g = np.load(os.path.join(GOLDEN, "cnt_golden.npz"))
    return {**{k: b[k] for k in b.files}, **{k: g[k] for k in g.files}}


@pytest.fixture(scope="session")
def ctx():
    import torch
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from quantum_transport_gb300.build import build
    build()
    from quantum_transport_gb300.rgf import Context
    c = Context(0)
    yield c
    c.close()
