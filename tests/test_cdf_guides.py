"""Guide tables of the CDF searches (photon_gb300/csrc/cdf_search.cuh), run on
the CPU: for the emissive-triangle CDF, the environment's marginal CDF and
every environment row, the guided search returns the same index as the
reference's plain bisection (pathtracer.cpp:296-306, environment_map.h:
62-104) for random RNG values and for every value at and next to a guide
grid point or a CDF entry, where an off-by-one would show."""
import ctypes as C

import numpy as np
import pytest


@pytest.fixture(scope="module")
def host_lib(host_traverse_lib):
    return host_traverse_lib


def _us(seed=0, n=1 << 16):
    """RNG values (multiples of 2^-24 in [0, 1)): random, and the grid points
    of every guide (k / 2^8, k / 2^10) with their two neighbours (the values
    next to each CDF entry are added by the C++ side)."""
    q = 2.0 ** -24
    rng = np.random.default_rng(seed)
    base = np.concatenate([rng.integers(0, 1 << 24, n) * q, np.arange(1 << 10) / 1024.0, np.arange(1 << 8) / 256.0])
    u = np.concatenate([base - q, base, base + q])
    u = u[(u >= 0) & (u < 1)]
    return np.ascontiguousarray(np.unique(u).astype(np.float32))


def _check(lib, sc):
    desc, keep = sc.desc()
    us = _us()
    counts = np.zeros(5, np.uint64)
    rc = lib.ht_guide_check(C.byref(desc), C.c_void_p(us.ctypes.data), C.c_uint32(len(us)),
                            C.c_void_p(counts.ctypes.data))
    assert rc == 0
    return counts


def test_guides_match_bisection_procedural_500k(host_lib):
    from photon_gb300 import workloads
    sc, _, _ = workloads.procedural_500k()
    counts = _check(host_lib, sc)
    assert counts[0] == 7  # emissive, marginal and row guides built
    assert counts[1] > 0 and counts[2] > 0 and counts[3] > 0
    assert counts[4] == 0, f"{int(counts[4])} guided searches differ from the bisection"


def test_guides_match_bisection_many_emitters(host_lib):
    """An emissive CDF of many triangles with very uneven weights (one very
    bright small triangle among dim ones)."""
    from photon_gb300 import workloads
    sc, _, _ = workloads.feature_scene("lights")
    counts = _check(host_lib, sc)
    assert counts[1] > 0
    assert counts[4] == 0


def test_guides_peaked_environment(host_lib):
    """A tiny bright sun on a nearly black sky: most rows and columns hold
    almost no probability, so a guide cell spans many entries."""
    from photon_gb300 import workloads
    sc, _, _ = workloads.procedural_500k()
    env = np.full((64, 128, 4), 1e-6, np.float32)
    env[..., 3] = 1.0
    env[40, 77, :3] = 1e6
    env[10, :5, :3] = 0.0  # zero-probability runs: CDF plateaus
    sc.env_pixels = env
    counts = _check(host_lib, sc)
    assert counts[0] & 6 == 6
    assert counts[4] == 0


@pytest.mark.parametrize("shape", [(1, 1), (1, 7), (5, 1), (3, 2)])
def test_guides_tiny_environments(host_lib, shape):
    """Environments of one row or one column (guide cells span the whole
    table) still give the bisection's indices."""
    from photon_gb300 import workloads
    sc, _, _ = workloads.box_room()
    h, w = shape
    rng = np.random.default_rng(h * 10 + w)
    env = rng.uniform(0.0, 2.0, (h, w, 4)).astype(np.float32)
    env[..., 3] = 1.0
    sc.env_pixels = env
    counts = _check(host_lib, sc)
    assert counts[0] & 6 == 6
    assert counts[2] > 0 and counts[4] == 0


def test_guides_black_environment(host_lib):
    """An all-black environment: the CDFs fall back to uniform steps (k / n)."""
    from photon_gb300 import workloads
    sc, _, _ = workloads.box_room()
    env = np.zeros((16, 32, 4), np.float32)
    env[..., 3] = 1.0
    sc.env_pixels = env
    counts = _check(host_lib, sc)
    assert counts[4] == 0
