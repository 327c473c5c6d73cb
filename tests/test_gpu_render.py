"""The renderer seam on the GPU (phc_set_scene / phc_render / phc_read_*)
against the reference.

Per-sample parity: each fixture frame is one sample per pixel (spp 1) on the
reference's RNG stream, so every pixel is one path.  Bar: at least 99.9% of
the paths agree within 1e-4 relative (tests/parity.py), and the depth /
normal / albedo channels likewise.
"""
import numpy as np
import pytest

from tests.golden import fixtures
from tests.parity import MIN_PATH_FRACTION, close_fraction, close_mask

pytestmark = pytest.mark.gpu


def render_frames(photon, sc, cam, st, frames):
    r = photon.Renderer()
    r.set_scene(sc)
    out = []
    for _ in range(frames):
        r.render(cam, st, True)
        out.append({ch: r.read(ch) for ch in ("color", "depth", "normal", "albedo")})
    return out


@pytest.mark.parametrize("name", fixtures.scene_names())
def test_render_matches_reference_fixture(photon, name):
    sc, cam, st, ref_frames = fixtures.load_scene(name)
    got = render_frames(photon, sc, cam, st, len(ref_frames))
    for f, (g, r) in enumerate(zip(got, ref_frames)):
        frac = close_fraction(g["color"], r["color"])
        assert frac >= MIN_PATH_FRACTION, f"{name} frame {f}: {frac:.5f} of paths within 1e-4"
        for ch in ("depth", "normal", "albedo"):
            frac = close_fraction(g[ch], r[ch])
            assert frac >= MIN_PATH_FRACTION, f"{name} frame {f} {ch}: {frac:.5f}"


@pytest.mark.parametrize("adaptive", [0, 1])
def test_render_procedural_matches_oracle(photon, oracle_lib, adaptive):
    """The 500K-triangle workload (env map, emissive triangles, glass,
    metal, clearcoat) at 96x96: per-sample radiance against the oracle, and
    with adaptive sampling the accumulated images (the variance gate makes
    the sample counts depend on every earlier sample)."""
    from photon_gb300 import workloads
    sc, cam, st = workloads.procedural_500k()
    st.width = st.height = 96
    st.adaptive_sampling = adaptive
    st.pixel_samples = 20 if adaptive else 1
    frames = 1 if adaptive else 3
    ref = oracle_lib.CpuRenderer("oracle")
    ref.set_scene(sc)
    got = render_frames(photon, sc, cam, st, frames)
    for f in range(frames):
        ref.render(cam, st, True)
        rc = ref.read("color")
        frac = close_fraction(got[f]["color"], rc)
        need = 0.99 if adaptive else MIN_PATH_FRACTION
        assert frac >= need, f"frame {f}: {frac:.5f}"
        assert close_fraction(got[f]["depth"], ref.read("depth")) >= MIN_PATH_FRACTION


def test_render_procedural_full_frame_matches_oracle(photon, oracle_lib):
    """The 500K-triangle workload at its full 1024^2 frame, depth 8, one
    sample per pixel, two frames (sample offsets 0 and 1): 1,048,576 paths
    per frame on the reference's RNG stream against the oracle, every path
    and every channel (colour with alpha, depth, normal, albedo) at the
    per-sample bar (>= 99.9% of paths within 1e-4 relative)."""
    from photon_gb300 import workloads
    sc, cam, st = workloads.procedural_500k()
    assert (st.width, st.height, st.max_depth) == (1024, 1024, 8)
    st.pixel_samples = 1
    st.adaptive_sampling = 0
    r = photon.Renderer()
    r.set_scene(sc)
    ref = oracle_lib.CpuRenderer("oracle")
    ref.set_scene(sc)
    for f in range(2):
        r.render(cam, st, True)
        ref.render(cam, st, True)
        fracs = {}
        for ch in ("color", "depth", "normal", "albedo"):
            g, w = r.read(ch), ref.read(ch)
            fracs[ch] = close_fraction(g, w)
            if ch == "color":
                bad = int((~close_mask(g, w)).sum())
        print(f"500K workload 1024^2 frame {f}: " + ", ".join(f"{k} {v:.6f}" for k, v in fracs.items()) +
              f" of {st.width * st.height} paths within 1e-4 ({bad} colour paths outside)")
        for ch, v in fracs.items():
            assert v >= MIN_PATH_FRACTION, f"frame {f} {ch}: {v:.6f}"
    r.close()
    ref.close()


def test_progressive_accumulation(photon, oracle_lib):
    """render() without reset adds samples (RenderBridge.cpp:923-927);
    accumulated_samples counts them; a size change restarts."""
    from photon_gb300 import workloads
    sc, cam, st = workloads.box_room()
    st.width = st.height = 48
    st.pixel_samples = 2
    r = photon.Renderer()
    o = oracle_lib.CpuRenderer("oracle")
    for x in (r, o):
        x.set_scene(sc)
        x.render(cam, st, True)
        x.render(cam, st, False)
        x.render(cam, st, False)
    assert r.accumulated_samples() == o.accumulated_samples() == 6
    assert close_fraction(r.read("color"), o.read("color")) >= MIN_PATH_FRACTION
    st.width = 40
    r.render(cam, st, False)
    assert r.accumulated_samples() == 2


def test_multi_sample_lanes_match_sequential(photon):
    """Several samples of a pixel in flight at once (the wave lanes) give the
    same image as one sample per wave, up to float summation order."""
    from photon_gb300 import workloads, tuning_get, tuning_set
    sc, cam, st = workloads.feature_scene("glass", res=64)
    st.pixel_samples = 16
    old = tuning_get("wave_paths")
    try:
        imgs = []
        for wp in (64 * 64, 64 * 64 * 16):
            tuning_set("wave_paths", wp)
            r = photon.Renderer()
            r.set_scene(sc)
            r.render(cam, st, True)
            imgs.append(r.read("color"))
        assert close_fraction(imgs[0], imgs[1], rtol=1e-5, atol=1e-6) >= 0.999
    finally:
        tuning_set("wave_paths", old)


def test_api_errors(photon):
    from photon_gb300 import PhotonError, workloads
    sc, cam, st = workloads.box_room()
    r = photon.Renderer()
    assert r.backend_name() == "cuda"
    with pytest.raises(PhotonError, match="NO_SCENE"):
        r.render(cam, st, True)
    r.set_scene(sc)
    r.width = r.height = 4
    with pytest.raises(PhotonError, match="NO_FRAME"):
        r.read("color")
    bad = workloads.settings(0, 16, 1, 1)
    with pytest.raises(PhotonError, match="INVALID"):
        r.render(cam, bad, True)


def test_empty_scene_renders_background(photon):
    """No triangles: the bridge substitutes one degenerate triangle
    (RenderBridge.cpp:445-453) and every camera ray sees the background."""
    from photon_gb300 import workloads
    from photon_gb300.scene import SceneData
    sc = SceneData(positions=np.zeros((0, 3), np.float32), indices=np.zeros((0, 3), np.uint32))
    _, cam, st = workloads.box_room()
    st.width = st.height = 16
    st.pixel_samples = 1
    st.background[:] = (0.25, 0.5, 0.75, 1.0)
    r = photon.Renderer()
    r.set_scene(sc)
    r.render(cam, st, True)
    c = r.read("color")
    assert np.allclose(c[..., :3], [0.25, 0.5, 0.75])
    assert np.all(np.isinf(r.read("depth")))


@pytest.mark.parametrize("scene", ["procedural_500k", "box_room"])
def test_material_sorted_shading_keeps_images(photon, scene):
    """Shading the hit queue unsorted, sorted by material, and sorted by
    shading class with one kernel per class (each compiled without the lobes
    its materials cannot have) gives the same image bit for bit.  The sizes
    make the first iterations' hit queues pass the sort threshold."""
    from photon_gb300 import tuning_get, tuning_set, workloads
    if scene == "box_room":
        sc, cam, st = workloads.box_room()
        st.width = st.height = 512
        st.pixel_samples = 2
    else:
        sc, cam, st = workloads.procedural_500k()
        st.width = st.height = 256
        st.pixel_samples = 8
    old = (tuning_get("sort_threshold"), tuning_get("shade_classes"))
    try:
        imgs = []
        for thr, cls in ((0, 0), (1, 0), (1, 1), (1 << 18, 1)):
            tuning_set("sort_threshold", thr)
            tuning_set("shade_classes", cls)
            r = photon.Renderer()
            r.set_scene(sc)
            r.render(cam, st, True)
            imgs.append(r.read("color").copy())
            r.close()
        for k in range(1, len(imgs)):
            assert np.array_equal(imgs[0].view(np.uint32), imgs[k].view(np.uint32)), k
    finally:
        tuning_set("sort_threshold", old[0])
        tuning_set("shade_classes", old[1])
