"""The resumable volume tracking of the shading kernels (VolTrack / vt_step
in photon_gb300/csrc/volume_track.cuh), run on the CPU against the plain
tracking it replaces in the kernels (vol_sample_scatter, vol_transmittance:
the delta / ratio tracking of tf_volume.h:150-283): for every ray the
scattering distance, albedo, transmittance and the random-number state
after the tracking must be identical bit for bit, so that the shading
continues the reference's random stream exactly."""
import ctypes as C

import numpy as np
import pytest

from tests.golden import fixtures


@pytest.fixture(scope="module")
def host_lib(host_traverse_lib):
    return host_traverse_lib


def _rays(lo, hi, n, seed):
    rng = np.random.default_rng(seed)
    c = 0.5 * (lo + hi)
    r = 0.75 * np.linalg.norm(hi - lo)
    u = rng.normal(size=(n, 3))
    o = (c + r * u / np.linalg.norm(u, axis=1, keepdims=True)).astype(np.float32)
    o[: n // 4] = rng.uniform(lo, hi, (n // 4, 3))  # a quarter start inside
    target = rng.uniform(lo, hi, (n, 3))
    d = (target - o).astype(np.float32)
    d /= np.linalg.norm(d, axis=1, keepdims=True)
    t0 = np.zeros(n, np.float32)
    t1 = np.where(rng.random(n) < 0.5, 1e30, rng.uniform(0.1, 4.0 * r, n)).astype(np.float32)
    t1[::29] = 0.0  # empty segments
    seeds = rng.integers(1, 2 ** 32, n, dtype=np.uint64).astype(np.uint32)
    return o, d, t0, t1, seeds


def _check(lib, sc, n=4096, seed=0):
    desc, keep = sc.desc()
    pos = np.asarray(sc.positions, np.float32).reshape(-1, 3)
    lo, hi = pos.min(0), pos.max(0)
    o, d, t0, t1, seeds = _rays(lo, hi, n, seed)
    arrs = [np.ascontiguousarray(a) for a in (o, d, t0, t1, seeds)]
    counts = np.zeros(3, np.uint64)
    rc = lib.ht_volume_check(C.byref(desc), *[C.c_void_p(a.ctypes.data) for a in arrs], C.c_uint32(n),
                             C.c_void_p(counts.ctypes.data))
    assert rc == 0
    return counts


def test_resumable_tracking_matches_volume_fixture(host_lib):
    """The fixture scene the reference build rendered: a heterogeneous and a
    homogeneous transfer-function volume."""
    sc, _, _, _ = fixtures.load_scene("volume")
    assert len(sc.volumes) >= 2
    counts = _check(host_lib, sc)
    assert counts[0] > 100, "too few rays met the volumes"
    assert counts[1] == 0, f"{int(counts[1])} rays differ"


def test_resumable_tracking_matches_fbm_grid(host_lib):
    """The 256^3-style fBm density of the instanced configuration (64^3 here):
    many macro cells, empty and dense regions, Russian roulette in the
    transmittance."""
    from photon_gb300 import workloads
    sc, _, _ = workloads.instanced_2m(res=32, spp=1, tex_res=64, grid=64, n_instances=8, adaptive=0)
    counts = _check(host_lib, sc, n=2048, seed=3)
    assert counts[0] > 100
    assert counts[1] == 0, f"{int(counts[1])} rays differ"
