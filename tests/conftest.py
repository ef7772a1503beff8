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


def golden_cases():
    """Unpadded fixtures (stage outputs and archives)."""
    return sorted(f[:-4] for f in os.listdir(GOLDEN) if f.endswith(".npz") and not f.startswith("p"))


def pad_golden_cases():
    """Padded (-p) fixtures: archive and reconstruction."""
    return sorted(f[:-4] for f in os.listdir(GOLDEN) if f.endswith(".npz") and f.startswith("p"))


def load_golden(name):
    z = np.load(os.path.join(GOLDEN, name + ".npz"))
    g = {k: z[k] for k in z.files}
    g["dims"] = tuple(int(v) for v in g["dims"])
    for k in ("bs", "dict_size", "r2r", "data_size", "n_outlier", "pad_mode", "pad_type"):
        if k in g:
            g[k] = int(g[k])
    for k in ("eb", "eb_final", "pad_const"):
        if k in g:
            g[k] = float(g[k])
    g["name"] = name
    return g


@pytest.fixture(scope="session")
def cuda():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    return torch
