"""Shared test set-up: import paths, the `gpu` marker, golden-fixture loaders."""
from __future__ import annotations

import json
import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
GOLDEN = os.path.join(ROOT, "tests", "golden")
for p in (os.path.join(ROOT, "cor-model_gb300"), os.path.join(ROOT, "oracle"), ROOT):
    if p not in sys.path:
        sys.path.insert(0, p)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300) and the built libcortrace.so")


def golden(name: str) -> dict:
    with open(os.path.join(GOLDEN, name)) as f:
        return json.load(f)


def unhex(lst) -> np.ndarray:
    return np.array([float.fromhex(s) for s in lst], dtype=np.float64)


@pytest.fixture(scope="session")
def ctx():
    import cortrace as ct
    c = ct.Context(0)
    yield c
    c.close()
