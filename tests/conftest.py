import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a)")


def _has_gpu():
    try:
        import torch
        return torch.cuda.is_available()
    except Exception:
        return False


HAS_GPU = _has_gpu()


def pytest_collection_modifyitems(config, items):
    if HAS_GPU:
        return
    skip = pytest.mark.skip(reason="no CUDA GPU on this host")
    for it in items:
        if "gpu" in it.keywords:
            it.add_marker(skip)


@pytest.fixture(scope="session")
def oracle_lib():
    """Builds the CPU oracles once per session (restatement always; the
    reference build only where its checkout exists)."""
    import oracle
    oracle.build()
    return oracle


@pytest.fixture(scope="session")
def photon():
    """The CUDA library, built in-tree for sm_103a."""
    from photon_gb300 import build
    build.build()
    import photon_gb300
    photon_gb300.load()
    return photon_gb300
