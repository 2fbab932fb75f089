import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a GB300 (sm_103a) GPU")


def _has_gpu():
    try:
        import torch
        return torch.cuda.is_available()
    except Exception:
        return False


def pytest_collection_modifyitems(config, items):
    if _has_gpu():
        return
    skip = pytest.mark.skip(reason="no CUDA device")
    for it in items:
        if "gpu" in it.keywords:
            it.add_marker(skip)


@pytest.fixture
def reference_probe():
    """Path of the renderer's shipped angular light probe
    (environmentmaps/campus_probe.hdr in its source tree, found through
    GBRT_REFERENCE_DIR); the test is skipped where the tree is absent."""
    from tests.golden.make_golden import PROBE
    if not os.path.exists(PROBE):
        pytest.skip("the renderer's shipped probe is not present (set GBRT_REFERENCE_DIR)")
    return PROBE


@pytest.fixture(scope="session")
def gbrt_built():
    """Makes sure the in-tree CUDA library exists (builds it when missing)."""
    from renderer_gb300 import LIB_PATH
    if not os.path.exists(LIB_PATH):
        from renderer_gb300 import build
        build.build()
    return LIB_PATH


@pytest.fixture(scope="session")
def ctx(gbrt_built):
    from renderer_gb300 import Context
    c = Context(0)
    yield c
    c.close()
