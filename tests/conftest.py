import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GB300 device (sm_103a)")


@pytest.fixture(scope="session")
def kats():
    import json
    with open(os.path.join(ROOT, "tests", "golden", "kats.json")) as fh:
        return json.load(fh)


@pytest.fixture(scope="session")
def cuda():
    import torch
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    return torch.device("cuda", 0)


def normwise_err(got, ref):
    got, ref = np.asarray(got), np.asarray(ref)
    dt = np.complex128 if (np.iscomplexobj(got) or np.iscomplexobj(ref)) else np.float64
    got, ref = got.astype(dt), ref.astype(dt)
    scale = np.max(np.abs(ref)) if ref.size else 1.0
    if scale == 0:
        scale = 1.0
    return float(np.max(np.abs(got - ref)) / scale) if ref.size else 0.0
