import os
import sys
from pathlib import Path

import numpy as np
import pytest

ROOT = Path(__file__).resolve().parents[1]
sys.path.insert(0, str(ROOT))
sys.path.insert(0, str(ROOT / "oracle"))
GOLDEN = ROOT / "tests" / "golden"


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA device (GB300); runs the CUDA library")
    config.addinivalue_line("markers", "slow: longer CPU test")


@pytest.fixture(scope="session")
def oracle():
    import pyoracle
    pyoracle.load()
    return pyoracle


@pytest.fixture(scope="session")
def ref(oracle):
    """The reference build (oracle/_ref); skipped where the reference tree is absent."""
    if not oracle.ref_available():
        pytest.skip("reference sources not present")
    oracle.load_ref()
    return oracle


@pytest.fixture(scope="session")
def lib():
    from dmrg_c_gb300 import build, lib as L
    build.build()
    return L.load()


@pytest.fixture(scope="session")
def gpu(lib):
    """The CUDA library on a visible device.  On a GPU run this must not skip: a missing
    device or library is an error."""
    from dmrg_c_gb300 import lib as L
    n = L.device_count()
    assert n > 0, "gpu test collected but no CUDA device is visible"
    return L


@pytest.fixture
def in_tmp(tmp_path, monkeypatch):
    """Run in a scratch directory (the drop-in entry points append to ./SML_out/)."""
    monkeypatch.chdir(tmp_path)
    return tmp_path


def golden(name):
    return np.load(GOLDEN / name)


@pytest.fixture
def rng():
    return np.random.default_rng(1234)


def pytest_collection_modifyitems(config, items):
    os.environ.setdefault("OMP_NUM_THREADS", str(min(8, os.cpu_count() or 1)))
