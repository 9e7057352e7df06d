import json
import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)
HERE = os.path.dirname(os.path.abspath(__file__))
if HERE not in sys.path:
    sys.path.insert(0, HERE)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300); runs the library's kernels")


@pytest.fixture(scope="session")
def golden():
    with open(os.path.join(HERE, "golden", "reference_tests.json")) as f:
        return json.load(f)


def gpu_available():
    try:
        import torch
        return torch.cuda.is_available()
    except Exception:
        return False


@pytest.fixture(scope="session")
def lib_built():
    from qvnt_gb300 import _abi
    if not os.path.exists(_abi.LIB_PATH):
        from qvnt_gb300 import build
        build.build()
    return _abi.lib()
