"""Shared test setup.

Tests marked ``gpu`` need a CUDA device and the built library; everything
else runs on the CPU.  Both compare against the oracle (oracle/, the CPU
restatement of the reference).
"""
import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

GOLDEN = os.path.join(ROOT, "tests", "golden")


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300) and the built library")


def load_golden(name):
    with np.load(os.path.join(GOLDEN, name), allow_pickle=False) as z:
        return {k: z[k] for k in z.files}


def params_from(b):
    from pibiti_gb300.params import SimParams
    return SimParams.from_bytes(np.asarray(b, np.uint8).tobytes())


@pytest.fixture(scope="session")
def golden():
    return load_golden


@pytest.fixture(scope="session")
def cuda():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from pibiti_gb300 import _lib
    _lib.lib()  # the extension must load: no fallback path exists
    return torch
