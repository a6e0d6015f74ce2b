import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

GOLDEN = os.path.join(ROOT, "tests", "golden")


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a)")


def load_golden(name):
    return np.load(os.path.join(GOLDEN, name))


def decode_circuit(blob, prefix):
    """Rebuild a gate list stored by tests/golden/make_golden.py."""
    kinds = blob[prefix + "_kind"]
    targets = blob[prefix + "_target"]
    masks = blob[prefix + "_ctrl"]
    angles = blob[prefix + "_angle"]
    gates = []
    for k, t, m, a in zip(kinds, targets, masks, angles):
        m = int(m)
        ctrl = tuple(q for q in range(64) if (m >> q) & 1)
        gates.append((int(k), int(t), ctrl, float(a)))
    return gates


def rel_err(a, b):
    a = np.asarray(a)
    b = np.asarray(b)
    den = np.linalg.norm(b)
    return float(np.linalg.norm(a - b) / (den if den > 0 else 1.0))


@pytest.fixture(scope="session")
def cuda_available():
    try:
        import torch
        return torch.cuda.is_available()
    except Exception:
        return False
