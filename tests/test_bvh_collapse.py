"""The GPU BVH build's surface-area collapse program on the CPU.

tests/native/collapse_test.cpp compiles photon_gb300/csrc/bvh_collapse.cuh
(the functions the build's k_collapse_dp and k_collapse_sah kernels call)
with the host compiler and checks it on random binary trees in the build's
layout: the wide tree it chooses covers every primitive exactly once with
2..8 children per wide node and leaf children within the leaf size, its cost
recomputed from its nodes equals the program's, and on trees of up to 12
primitives the program's cost equals the least cost over every cover written
out explicitly.  The GPU build over these choices is checked against the
reference fixture and the oracle in tests/test_gpu_bvh_build.py.
"""
import ctypes as C
import os
import shutil
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


@pytest.fixture(scope="module")
def lib(tmp_path_factory):
    cuda = "/usr/local/cuda"
    if not os.path.isdir(os.path.join(cuda, "include")) or not shutil.which("g++"):
        pytest.skip("needs g++ and the CUDA headers")
    out = tmp_path_factory.mktemp("collapse") / "libcollapse_test.so"
    subprocess.run(["g++", "-std=c++17", "-O2", "-fPIC", "-shared", "-ffp-contract=off",
                    "-I", os.path.join(cuda, "include"), "-I", os.path.join(ROOT, "photon_gb300", "csrc"),
                    os.path.join(ROOT, "tests", "native", "collapse_test.cpp"), "-o", str(out)], check=True)
    lib = C.CDLL(str(out))
    lib.ct_check.restype = C.c_int
    lib.ct_check.argtypes = [C.c_uint32, C.c_uint, C.c_int, C.c_float, C.POINTER(C.c_double)]
    return lib


def _check(lib, n, seed, max_leaf, ct):
    out = (C.c_double * 5)()
    rc = lib.ct_check(n, seed, max_leaf, ct, out)
    assert rc == 0, (n, seed, max_leaf, ct, rc, list(out))
    return list(out)


@pytest.mark.parametrize("max_leaf", [1, 2, 3])
@pytest.mark.parametrize("ct", [0.05, 0.3, 3.0, 30.0])
def test_program_matches_enumeration_on_small_trees(lib, max_leaf, ct):
    for n in (4, 5, 6, 7, 8, 9, 10, 11, 12):
        for seed in range(1, 31):
            prog, total, nodes, brute, leaves = _check(lib, n, seed, max_leaf, ct)
            assert brute > 0 and abs(brute - prog) <= 1e-5 * prog


@pytest.mark.parametrize("n", [100, 5000, 50000])
@pytest.mark.parametrize("max_leaf", [1, 2, 3])
def test_program_cover_is_complete(lib, n, max_leaf):
    for seed in (1, 2):
        for ct in (0.05, 0.3, 3.0):
            prog, total, nodes, brute, leaves = _check(lib, n, seed, max_leaf, ct)
            assert nodes >= 1 and leaves >= n / max_leaf


def test_cheap_triangles_make_larger_leaves(lib):
    # with triangle tests almost free a leaf child holds as many triangles as
    # allowed, so the wide tree has fewer nodes than with costly triangles
    few = _check(lib, 5000, 3, 3, 0.05)[2]
    many = _check(lib, 5000, 3, 3, 3.0)[2]
    assert few < many
