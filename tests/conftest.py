import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
GOLDEN = os.path.join(ROOT, "tests", "golden")
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a)")


def golden(name):
    return dict(np.load(os.path.join(GOLDEN, name + ".npz")))


@pytest.fixture(scope="session")
def goldens():
    return {n: golden(n) for n in ("water_c1", "peptide30", "peptide30_ap", "peptide120")}


def rel_rms(f, ref):
    """Per-atom force error: sqrt(mean |dF|^2) / sqrt(mean |F|^2)."""
    f = np.asarray(f).reshape(-1, 3)
    ref = np.asarray(ref).reshape(-1, 3)
    return float(np.sqrt(((f - ref) ** 2).sum(1).mean() / (ref ** 2).sum(1).mean()))


def rel_err(a, b):
    return abs(a - b) / max(abs(b), 1e-300)
