import json
import os
import sys

import pytest

# hardware work queues: set before CUDA starts, as the package does on import
os.environ.setdefault("CUDA_DEVICE_MAX_CONNECTIONS", "32")

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
PKG_ROOT = os.path.join(ROOT, "ted-q_gb300")
for p in (ROOT, PKG_ROOT):
    if p not in sys.path:
        sys.path.insert(0, p)

GOLDEN = os.path.join(ROOT, "tests", "golden", "cases.json")


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300) and the built sm_103a library")


def load_cases():
    with open(GOLDEN) as f:
        return json.load(f)["cases"]


@pytest.fixture(scope="session")
def golden_cases():
    return load_cases()


def cuda_available():
    try:
        import torch
        return torch.cuda.is_available()
    except Exception:
        return False
