"""pbrt-v4 scenes on the GPU: the reader's scene (include/photon_pbrt.h)
rendered by the CUDA renderer against the reference's own pbrt path.

The golden renders (tests/golden/pbrt_ref.npz, made by make_pbrt_golden.py)
are the reference's parse_pbrt_file + convert_pbrt_scene + PathTracer::render
at spp 4 without adaptive sampling; the features scene exercises the
path-tracer-level materials, atlas textures (a checker base colour and an
alpha mask) read through texture coordinates, a rotated environment image,
PLY meshes, spheres, instancing and area lights.  Bar: 99.9% of the pixels
within 1e-4 relative (tests/parity.py).
"""
import os

import numpy as np
import pytest

from tests.parity import MIN_PATH_FRACTION, close_fraction

pytestmark = pytest.mark.gpu

HERE = os.path.dirname(os.path.abspath(__file__))
SCENES = os.path.join(HERE, "golden", "pbrt")
GOLDEN = os.path.join(HERE, "golden", "pbrt_ref.npz")
CASES = [("box_room", "box_room.pbrt", False), ("features", "features.pbrt", False),
         ("features_ias", "features.pbrt", True)]


@pytest.mark.parametrize("case,fname,ias", CASES)
def test_gpu_render_matches_reference_pbrt_render(photon, case, fname, ias):
    from photon_gb300 import pbrt
    g = np.load(GOLDEN)
    w, h, spp, _ = g[f"{case}/render_args"].tolist()
    sc = pbrt.load(os.path.join(SCENES, fname), use_instancing=ias, width=w, height=h, spp=spp)
    st = type(sc.settings).from_buffer_copy(bytes(sc.settings))
    st.adaptive_sampling = 0
    r = photon.Renderer()
    r.set_scene(sc)
    r.render(sc.camera, st, True)
    img = r.read("color")[..., :3]
    frac = close_fraction(img, g[f"{case}/render"])
    assert frac >= MIN_PATH_FRACTION, f"{case}: {frac:.5f} of pixels within 1e-4"


@pytest.mark.parametrize("adaptive", [0, 1])
def test_gpu_features_scene_matches_oracle(photon, oracle_lib, adaptive):
    """Larger image, per-sample frames (and one adaptive accumulation)
    against the CPU oracle on the same converted scene."""
    from photon_gb300 import pbrt
    sc = pbrt.load(os.path.join(SCENES, "features.pbrt"), width=144, height=96, spp=24 if adaptive else 1)
    st = type(sc.settings).from_buffer_copy(bytes(sc.settings))
    st.adaptive_sampling = adaptive
    r = photon.Renderer()
    r.set_scene(sc)
    o = oracle_lib.CpuRenderer("oracle")
    o.set_scene(sc)
    frames = 1 if adaptive else 2
    for f in range(frames):
        r.render(sc.camera, st, f == 0)
        o.render(sc.camera, st, f == 0)
        frac = close_fraction(r.read("color"), o.read("color"))
        need = 0.99 if adaptive else MIN_PATH_FRACTION
        assert frac >= need, f"frame {f}: {frac:.5f}"
    for ch in ("depth", "normal", "albedo"):
        assert close_fraction(r.read(ch), o.read(ch)) >= MIN_PATH_FRACTION, ch


def test_gpu_adjoint_rejects_atlas_textures(photon):
    from photon_gb300 import pbrt
    from photon_gb300.native import PhotonError
    sc = pbrt.load(os.path.join(SCENES, "features.pbrt"), width=16, height=16, spp=1)
    st = type(sc.settings).from_buffer_copy(bytes(sc.settings))
    st.adaptive_sampling = 0
    r = photon.Renderer()
    r.set_scene(sc)
    with pytest.raises(PhotonError, match="atlas"):
        r.adjoint(sc.camera, st, np.ones((16, 16, 4), np.float32))


def test_gpu_box_room_pbrt_full_config(photon):
    """The box-room file at its own settings (512x512, 64 spp, depth 8,
    adaptive sampling as PathTracer's default): renders, finite, lit."""
    from photon_gb300 import pbrt
    sc = pbrt.load(os.path.join(SCENES, "box_room.pbrt"))
    r = photon.Renderer()
    r.set_scene(sc)
    r.render(sc.camera, sc.settings, True)
    img = r.read("color")
    assert img.shape == (512, 512, 4) and np.isfinite(img).all()
    assert 0.05 < float(img[..., :3].mean()) < 2.0
