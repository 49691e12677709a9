"""Shared pytest setup: the ``gpu`` marker and import paths.

Tests marked ``gpu`` need a CUDA device and the compiled extension; everything
else runs on the CPU (``pytest -m "not gpu"``).
"""

import sys
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parents[1]
if str(ROOT) not in sys.path:
    sys.path.insert(0, str(ROOT))

GOLDEN = Path(__file__).resolve().parent / "golden"


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU and the compiled engine")


@pytest.fixture(scope="session")
def golden():
    import numpy as np

    def load(name):
        with np.load(GOLDEN / f"{name}.npz") as f:
            return {k: f[k] for k in f.files}

    load.path = lambda name: GOLDEN / f"{name}.npz"
    return load
