import os
import sys
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parent.parent
sys.path.insert(0, str(ROOT))
sys.path.insert(0, str(Path(__file__).resolve().parent))


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300) and the built sm_103a library")
    # a per-test limit where pytest-timeout is installed; a no-op mark otherwise
    config.addinivalue_line("markers", "timeout(seconds): per-test time limit (pytest-timeout)")


# GPU suites of features whose device code has not yet run on a GPU. They
# are collected after the suites already run on hardware, so that under
# `pytest -x` a first failure in them stops nothing that was passing before.
FIRST_GPU_RUN = ("test_gpu_sources.py", "test_gpu_spherical.py", "test_gpu_transport.py", "test_gpu_output.py",
                 "test_gpu_smr_sph.py")


def pytest_collection_modifyitems(session, config, items):
    items.sort(key=lambda it: Path(str(it.fspath)).name in FIRST_GPU_RUN)


@pytest.fixture(scope="session")
def oracle():
    from oracle_ctypes import Oracle

    return Oracle()


@pytest.fixture(scope="session")
def names():
    from fortrancfd_gb300 import species_names

    return species_names()


def reference_dir():
    """The reference checkout named by $EDYN_REFERENCE, when that variable is
    set and the directory exists; None otherwise (the tests that need it
    skip)."""
    env = os.environ.get("EDYN_REFERENCE")
    if not env:
        return None
    p = Path(env)
    return p if p.exists() else None
