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


@functools.lru_cache(maxsize=1)
def _full():
    from photon_gb300 import workloads
    return workloads.instanced_2m(spp=1, adaptive=0)


@pytest.mark.parametrize("adaptive", [0, 1])
def test_instanced_full_textures_crop_matches_oracle(photon, oracle_lib, adaptive):
    """The full configuration (2M triangles, twelve 2048^2 textures, 256^3
    density grid, depth 12) on a 320^2 crop of its 1920^2 frame: the
    camera's image_region selects the crop, so each pixel sees the same
    footprint as in the full frame, and the oracle's cost stays bounded.
    One sample per pixel, two frames, per-sample bar on colour, depth and
    normal; with adaptive sampling (20 spp, the gate opens after 16), the
    accumulated image on >= 99% of pixels."""
    sc, cam0, st0 = _full()
    assert sc.triangle_count >= 2_000_000 and len(sc.samplers) == 12
    assert all(s.size[0] == 2048 for s, _ in sc.samplers)
    assert st0.width == 1920 and st0.max_depth == 12
    cam = type(cam0).from_buffer_copy(bytes(cam0))
    st = type(st0).from_buffer_copy(bytes(st0))
    crop = 320
    x0, y0 = 0.40, 0.35
    cam.image_region[:] = (x0, y0, x0 + crop / 1920.0, y0 + crop / 1920.0)
    st.width = st.height = crop
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
        fc = close_fraction(r.read("color"), ref.read("color"))
        fd = close_fraction(r.read("depth"), ref.read("depth"))
        fn = close_fraction(r.read("normal"), ref.read("normal"))
        print(f"2M instanced, full textures and grid, {crop}^2 crop, adaptive {adaptive}, frame {f}: "
              f"colour {fc:.6f}, depth {fd:.6f}, normal {fn:.6f}")
        need = 0.99 if adaptive else MIN_PATH_FRACTION
        assert fc >= need, f"frame {f}: {fc:.5f}"
        assert fd >= MIN_PATH_FRACTION and fn >= MIN_PATH_FRACTION
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


def test_rgba8_texels_match_fp32_storage(photon):
    """Samplers whose texels are all k / 255 are stored as 8-bit RGBA on the
    device (tuning key texels_u8) and decoded through the table of those
    floats: every channel of every frame is bit-identical to the same scene
    stored as fp32 texels, and the scene takes about a quarter of the texel
    bytes."""
    import torch
    from photon_gb300 import tuning_get, tuning_set
    sc, cam, st0 = _small()
    st = type(st0).from_buffer_copy(bytes(st0))
    st.pixel_samples = 2
    old = tuning_get("texels_u8")
    out, mem = {}, {}
    try:
        for mode in (1, 0):
            tuning_set("texels_u8", mode)
            torch.cuda.synchronize()
            free0 = torch.cuda.mem_get_info()[0]
            r = photon.Renderer()
            r.set_scene(sc)
            torch.cuda.synchronize()
            mem[mode] = free0 - torch.cuda.mem_get_info()[0]
            frames = []
            for _ in range(2):
                r.render(cam, st, True)
                frames.append({ch: r.read(ch).copy() for ch in ("color", "depth", "normal", "albedo")})
            out[mode] = frames
            r.close()
    finally:
        tuning_set("texels_u8", old)
    for f in range(2):
        for ch in ("color", "depth", "normal", "albedo"):
            a, b = out[1][f][ch], out[0][f][ch]
            assert np.array_equal(a.view(np.uint32), b.view(np.uint32)), (f, ch)
    texel_bytes = sum(len(t) * 16 for _, t in sc.samplers)
    print(f"scene device memory: {mem[1] / 2**20:.1f} MiB with 8-bit texels, {mem[0] / 2**20:.1f} MiB fp32 "
          f"({texel_bytes / 2**20:.1f} MiB of fp32 texels)")
    assert mem[0] - mem[1] >= 0.6 * texel_bytes
