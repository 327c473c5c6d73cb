"""The 2M-triangle instanced workload (flattened instances, 12 RGBA8 textures
for base colour / roughness / normal maps, emissive meshes, a 256^3 fBm
density volume with sigma_t up to 8, adaptive sampling) on the GPU.

* Per-sample parity against the oracle on the full geometry and volume
  structure with smaller textures and grid (the oracle's single-threaded
  median-split BVH build and per-pixel loop are the cost), one sample per
  pixel, two frames; and with adaptive sampling, the accumulated image.
* The full-size configuration (1920^2, 2048^2 textures, 256^3 grid, depth 12,
  adaptive) renders on the GPU with finite output and the expected sample
  accounting.
"""
import functools

import numpy as np
import pytest

from tests.parity import MIN_PATH_FRACTION, close_fraction

pytestmark = pytest.mark.gpu


@functools.lru_cache(maxsize=2)
def _small():
    from photon_gb300 import workloads
    return workloads.instanced_2m(res=48, spp=1, tex_res=256, grid=64, adaptive=0)


@pytest.mark.parametrize("adaptive", [0, 1])
def test_instanced_matches_oracle(photon, oracle_lib, adaptive):
    sc, cam, st0 = _small()
    st = type(st0).from_buffer_copy(bytes(st0))
    st.adaptive_sampling = adaptive
    st.pixel_samples = 20 if adaptive else 1
    frames = 1 if adaptive else 2
    r = photon.Renderer()
    r.set_scene(sc)
    ref = oracle_lib.CpuRenderer("oracle")
    ref.set_scene(sc)
    for f in range(frames):
        r.render(cam, st, True)
        ref.render(cam, st, True)
        frac = close_fraction(r.read("color"), ref.read("color"))
        need = 0.99 if adaptive else MIN_PATH_FRACTION
        assert frac >= need, f"frame {f}: {frac:.5f}"
        assert close_fraction(r.read("depth"), ref.read("depth")) >= MIN_PATH_FRACTION
        assert close_fraction(r.read("normal"), ref.read("normal")) >= MIN_PATH_FRACTION
    r.close()
    ref.close()


def test_instanced_full_size_renders(photon):
    from photon_gb300 import workloads
    sc, cam, st = workloads.instanced_2m()
    assert sc.triangle_count >= 2_000_000 and len(sc.samplers) == 12
    st.pixel_samples = 32  # past the adaptive gate (16 samples)
    r = photon.Renderer()
    r.set_scene(sc)
    r.render(cam, st, True)
    s = r.stats()
    img = r.read("color")
    print(f"instanced 2M, 1920^2 x 32 spp adaptive: {s['render_ms']:.1f} ms, "
          f"{s['pixel_samples'] / (s['render_ms'] * 1e3):.1f} Msamples/s, {s['pixel_samples']} pixel samples")
    assert np.isfinite(img).all()
    assert 1920 * 1920 * 16 <= s["pixel_samples"] <= 1920 * 1920 * 32
    assert img[..., :3].mean() > 0.0
    assert r.accumulated_samples() == 32
    r.close()
