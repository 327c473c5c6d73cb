"""The BVH8 builder and the device traversal code, run on the CPU.

tests/native/host_traverse.cpp compiles photon_gb300/csrc/traverse.cuh (the
same __host__ __device__ traversal the kernels use) and bvh8.cpp with the
host compiler.  Against the oracle (bit-identical to the reference's
KokkosBackend): hit/miss and t identical for every ray, primitive ids
identical except exact-distance ties, occlusion identical; every leaf size.
"""
import ctypes as C
import os

import numpy as np
import pytest

from tests.golden import fixtures

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


@pytest.fixture(scope="module")
def host_lib(host_traverse_lib):
    return host_traverse_lib


def host_trace(lib, pos, idx, o, d, t0, t1, any_hit, max_leaf=3):
    n = len(t0)
    out = np.zeros((n, 4), np.float32)
    st = np.zeros(5, np.uint64)
    arrs = [np.ascontiguousarray(a) for a in (pos, idx, o, d, t0, t1)]
    lib.ht_trace(C.c_void_p(arrs[0].ctypes.data), C.c_uint64(arrs[0].size // 3), C.c_void_p(arrs[1].ctypes.data),
                 C.c_uint64(arrs[1].size // 3), *[C.c_void_p(a.ctypes.data) for a in arrs[2:]], C.c_uint32(n),
                 C.c_int(int(any_hit)), C.c_int(max_leaf), C.c_void_p(out.ctypes.data), C.c_void_p(st.ctypes.data))
    return out, st


def check(lib, oracle_lib, pos, idx, o, d, t0, t1, max_leaf):
    out, st = host_trace(lib, pos, idx, o, d, t0, t1, False, max_leaf)
    assert st[4] == idx.size // 3  # every triangle once in the leaves
    assert st[3] < 64               # fits the traversal stack
    ref = oracle_lib.trace("oracle", pos, idx, o, d, t0, t1, False)
    prim = out[:, 1].view(np.uint32)
    hit = ref["hit"].astype(bool)
    assert np.array_equal(prim != 0xffffffff, hit)
    assert np.array_equal(out[hit, 0].view(np.uint32), ref["t"][hit].view(np.uint32))
    same = prim[hit] == ref["prim_id"][hit]
    assert (~same).mean() < 0.01
    occ, _ = host_trace(lib, pos, idx, o, d, t0, t1, True, max_leaf)
    rocc = oracle_lib.trace("oracle", pos, idx, o, d, t0, t1, True)
    assert np.array_equal(occ[:, 1].view(np.uint32) != 0xffffffff, rocc != 0)


@pytest.mark.parametrize("max_leaf", [1, 2, 3])
def test_host_traversal_matches_oracle_fixture_mesh(host_lib, oracle_lib, max_leaf):
    z = fixtures.load_trace()
    check(host_lib, oracle_lib, z["positions"], z["indices"], z["orgs"], z["dirs"], z["tmin"], z["tmax"], max_leaf)


def test_host_traversal_matches_oracle_procedural(host_lib, oracle_lib):
    from photon_gb300 import workloads
    sc, _, _ = workloads.procedural_500k(n_objects=40, n_spheres=20, sphere_subdiv=3)
    rng = np.random.default_rng(9)
    n = 50_000
    lo, hi = sc.positions.min(0), sc.positions.max(0)
    o = rng.uniform(lo, hi, (n, 3)).astype(np.float32)
    d = rng.normal(size=(n, 3)).astype(np.float32)
    d /= np.linalg.norm(d, axis=1, keepdims=True)
    t0 = np.zeros(n, np.float32)
    t1 = np.full(n, 1e30, np.float32)
    t1[::3] = rng.uniform(0.05, 4.0, len(t1[::3])).astype(np.float32)
    check(host_lib, oracle_lib, sc.positions, sc.indices, o, d, t0, t1, 3)


def test_degenerate_and_coincident_triangles(host_lib, oracle_lib):
    """Many identical triangles (identical centroids: the SAH cannot split)
    and zero-area ones: the builder must still produce leaves of <= 3 and a
    stack-safe depth, and the traversal must find the reference's hits."""
    rng = np.random.default_rng(2)
    tri = np.array([[0, 0, 0], [1, 0, 0], [0, 1, 0]], np.float32)
    pos = np.concatenate([tri] * 500 + [np.zeros((3, 3), np.float32)] * 100 + [rng.uniform(-1, 2, (300, 3))])
    pos = pos.astype(np.float32)
    idx = np.arange(len(pos), dtype=np.uint32).reshape(-1, 3)
    n = 4000
    o = np.concatenate([rng.uniform(-0.2, 1.2, (n, 2)), np.full((n, 1), 2.0)], 1).astype(np.float32)
    d = np.tile(np.array([0, 0, -1], np.float32), (n, 1))
    t0 = np.zeros(n, np.float32)
    t1 = np.full(n, 1e30, np.float32)
    out, st = host_trace(host_lib, pos, idx, o, d, t0, t1, False)
    assert st[4] == len(idx) and st[3] < 64
    ref = oracle_lib.trace("oracle", pos, idx, o, d, t0, t1, False)
    hit = ref["hit"].astype(bool)
    assert np.array_equal(out[:, 1].view(np.uint32) != 0xffffffff, hit)
    assert np.array_equal(out[hit, 0].view(np.uint32), ref["t"][hit].view(np.uint32))
