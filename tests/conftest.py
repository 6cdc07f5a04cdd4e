"""Shared fixtures.  GPU tests are marked ``gpu``; everything else runs on a
CPU-only machine."""

import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (sm_103a)")


@pytest.fixture
def rng():
    # seed 4 is the reference's convention (python/tests/conftest.py)
    return np.random.default_rng(4)
