"""Shared fixtures.  Tests marked ``gpu`` need a CUDA device and the built library; the rest
run on the CPU (the oracle against the golden fixtures, host-side logic, C-ABI exports)."""
from __future__ import annotations

import importlib
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
    config.addinivalue_line("markers", "gpu: needs a CUDA device (runs on the GB300 box)")


@pytest.fixture(scope="session")
def golden():
    vec = np.load(os.path.join(GOLDEN, "reference_vectors.npz"))
    with open(os.path.join(GOLDEN, "reference_info.json")) as f:
        info = json.load(f)
    return {k: vec[k] for k in vec.files}, info["cases"]


@pytest.fixture(scope="session")
def oracle():
    import pyoracle
    pyoracle.build()
    return pyoracle.Oracle()


@pytest.fixture(scope="session")
def gl():
    """The product package (generic-linalg_gb300), built in-tree if needed."""
    importlib.import_module("generic-linalg_gb300.build").build_library()
    return importlib.import_module("generic-linalg_gb300")


@pytest.fixture(scope="session")
def gpu(gl):
    import torch
    if not torch.cuda.is_available() or gl.lib().glinalg_device_count() < 1:
        pytest.skip("no CUDA device")
    return torch.device("cuda:0")
