import os
import sys

import pytest

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
for p in (os.path.join(REPO, "gpu-scrimp-large_gb300"), os.path.join(REPO, "oracle"),
          os.path.join(REPO, "tests")):
    if p not in sys.path:
        sys.path.insert(0, p)

PKG_DIR = os.path.join(REPO, "gpu-scrimp-large_gb300", "scamp_gb300")
# The reference tree (its test inputs and sources), where one is present:
# tests that read it skip when SCAMP_REFERENCE_TREE is unset.
REFERENCE_TREE = os.environ.get("SCAMP_REFERENCE_TREE", "")


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300)")


@pytest.fixture(scope="session")
def engine():
    """The engine package with its library loaded (fails loudly if unbuilt)."""
    import scamp_gb300

    scamp_gb300._lib.load()
    return scamp_gb300


@pytest.fixture(scope="session")
def gpu_engine(engine):
    if not engine.gpu_supported():
        pytest.fail("GPU test run without a visible CUDA device")
    return engine


@pytest.fixture(scope="session")
def oracle_mod():
    import oracle

    oracle.load()
    return oracle
