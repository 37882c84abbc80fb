import json
import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

GOLDEN = os.path.join(ROOT, "tests", "golden")


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300) and libfolgb.so")


def golden(name):
    with open(os.path.join(GOLDEN, name)) as f:
        return json.load(f)


def arr(entry):
    return np.asarray(entry["data"], dtype=np.float64).reshape(entry["shape"])


@pytest.fixture(scope="session")
def cuda():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from folax_gb300 import _capi
    _capi.load()
    return torch
