import json
import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
GOLDEN = os.path.join(ROOT, "tests", "golden")
for p in (ROOT, os.path.join(ROOT, "oracle")):
    if p not in sys.path:
        sys.path.insert(0, p)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GB300 and the built libmgx.so")


@pytest.fixture(scope="session")
def golden():
    return np.load(os.path.join(GOLDEN, "llg_golden.npz"))


@pytest.fixture(scope="session")
def golden_models():
    with open(os.path.join(GOLDEN, "models.json")) as f:
        return json.load(f)


@pytest.fixture(scope="session")
def cuda():
    import torch
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from magex_gb300 import build
    build.build_library()
    return torch.device("cuda", 0)
