import json
import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
GOLDEN = os.path.join(ROOT, "tests", "golden")
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.join(ROOT, "oracle"))


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300); runs the sm_103a kernels")


def golden(name):
    return np.load(os.path.join(GOLDEN, name))


def golden_sim(name):
    d = np.load(os.path.join(GOLDEN, f"sim_{name}.npz"))
    return d, json.loads(str(d["meta"]))


@pytest.fixture(scope="session")
def kernels_npz():
    return golden("kernels.npz")


@pytest.fixture(scope="session")
def lib_built():
    """libnebula.so built in-tree (nvcc cross-compiles without a GPU)"""
    from nebulaviewer_gb300 import build
    build.build(verbose=False)
    from nebulaviewer_gb300 import _lib
    return _lib.load()


def rel_linf(a, b):
    a = np.asarray(a, np.float64)
    b = np.asarray(b, np.float64)
    return float(np.abs(a - b).max() / max(np.abs(b).max(), 1e-30))


def bits_equal(a, b):
    a = np.ascontiguousarray(a, np.float32)
    b = np.ascontiguousarray(b, np.float32)
    return np.array_equal(a.view(np.uint32), b.view(np.uint32))
