"""Self-check of the persistent wave kernels on the GPU.

Every persistent traversal / tracking warp counts its loop trips; one that
passes the cap (tuning key wave_trip_cap, default 2^24, where legitimate work
needs a few thousand) stops, records the kernel and bounce iteration in the
wave's error word, and every later kernel of the wave returns at entry.  The
render call then fails with PHC_ERR_DEVICE and a message naming the kernel.

Here the cap is lowered to a few trips so that it runs out on ordinary work:
the call must come back (the kernels return rather than spin), report the
error, and leave the renderer usable: the next render with the default cap
equals the oracle's frame (a failed call does not advance the sample counter).
"""
import time

import numpy as np
import pytest

from tests.parity import MIN_PATH_FRACTION, close_fraction

pytestmark = pytest.mark.gpu

PHC_ERR_DEVICE = -6


def _scene(kind):
    from photon_gb300 import workloads
    if kind == "box_room":
        sc, cam, st = workloads.box_room()
    else:
        sc, cam, st = workloads.feature_scene(kind)
    st.width = st.height = 64
    st.pixel_samples = 1
    st.adaptive_sampling = 0
    return sc, cam, st


@pytest.mark.parametrize("kind,cap", [("box_room", 3), ("volume", 3)])
def test_trip_cap_reports_and_recovers(photon, oracle_lib, kind, cap):
    from photon_gb300 import PhotonError, tuning_get, tuning_set
    sc, cam, st = _scene(kind)
    r = photon.Renderer()
    r.set_scene(sc)
    default = tuning_get("wave_trip_cap")
    assert default == 1 << 24
    try:
        tuning_set("wave_trip_cap", cap)
        t = time.perf_counter()
        with pytest.raises(PhotonError) as ei:
            r.render(cam, st, True)
        dt = time.perf_counter() - t
    finally:
        tuning_set("wave_trip_cap", default)
    msg = str(ei.value)
    print(f"{kind}, cap {cap}: {dt * 1e3:.1f} ms, {msg[:160]}")
    assert ei.value.code == PHC_ERR_DEVICE
    assert "loop-trip cap" in msg
    assert dt < 30.0
    assert r.accumulated_samples() == 0
    # the same renderer, default cap: a normal frame
    r.render(cam, st, True)
    got = r.read("color")
    ref = oracle_lib.CpuRenderer("oracle")
    ref.set_scene(sc)
    ref.render(cam, st, True)
    want = ref.read("color")
    assert np.isfinite(got).all()
    frac = close_fraction(got, want)
    assert frac >= MIN_PATH_FRACTION, frac
    assert r.accumulated_samples() == 1
    r.close()
    ref.close()


def test_trip_cap_range(photon):
    from photon_gb300 import tuning_get, tuning_set
    old = tuning_get("wave_trip_cap")
    for bad in (0, (1 << 30) + 1):
        with pytest.raises(ValueError):
            tuning_set("wave_trip_cap", bad)
    assert tuning_get("wave_trip_cap") == old
