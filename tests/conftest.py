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


@pytest.fixture(scope="session")
def host_traverse_lib(tmp_path_factory):
    """tests/native/host_traverse.cpp with the host BVH8 builder and the
    renderer's host scene build, compiled with the host compiler: the device
    traversal code (traverse.cuh) run on the CPU."""
    import ctypes as C
    import shutil
    import subprocess
    cuda = "/usr/local/cuda"
    if not os.path.isdir(os.path.join(cuda, "include")) or not shutil.which("g++"):
        pytest.skip("needs g++ and the CUDA headers")
    csrc = os.path.join(ROOT, "photon_gb300", "csrc")
    out = tmp_path_factory.mktemp("ht") / "libhost_traverse.so"
    subprocess.run(["g++", "-std=c++17", "-O2", "-fPIC", "-shared", "-fopenmp", "-ffp-contract=off",
                    "-I", os.path.join(cuda, "include"), "-I", csrc,
                    os.path.join(ROOT, "tests", "native", "host_traverse.cpp"),
                    os.path.join(csrc, "bvh8.cpp"), os.path.join(csrc, "scene_build.cpp"),
                    os.path.join(csrc, "tuning.cpp"), "-L", os.path.join(cuda, "lib64"), "-lcudart",
                    "-o", str(out)], check=True)
    return C.CDLL(str(out))
