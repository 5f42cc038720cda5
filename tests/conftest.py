import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)
GOLDEN = os.path.join(ROOT, "tests", "golden")


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (run on the GB300 box)")


def load_golden(name):
    path = os.path.join(GOLDEN, name + ".npz")
    if not os.path.exists(path):
        pytest.skip(f"golden fixture {name} not generated")
    g = np.load(path)
    meta = eval(g["meta"].tobytes().decode())  # written by tests/golden/make_golden.py
    pts = [l.split() for l in g["points"].tobytes().decode().splitlines()]
    return g, meta, pts


@pytest.fixture(scope="session")
def ctx():
    import torch
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    import fjmodels_gb300 as F
    c = F.Context(0)
    yield c
    c.close()
