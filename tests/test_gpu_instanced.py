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


def _render_modes(photon, sc, cam, st, modes):
    """Renders two frames of the scene under each (texels_u8, gpu_tables)
    mode; returns the frames' four channels and the device memory the scene
    took, per mode."""
    import torch
    from photon_gb300 import tuning_get, tuning_set
    old = (tuning_get("texels_u8"), tuning_get("gpu_tables"))
    out, mem = {}, {}
    try:
        for mode in modes:
            tuning_set("texels_u8", mode[0])
            tuning_set("gpu_tables", mode[1])
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
        tuning_set("texels_u8", old[0])
        tuning_set("gpu_tables", old[1])
    return out, mem


def _same_frames(a, b):
    for f in range(2):
        for ch in ("color", "depth", "normal", "albedo"):
            assert np.array_equal(a[f][ch].view(np.uint32), b[f][ch].view(np.uint32)), (f, ch)


def test_rgba8_texels_match_fp32_storage(photon):
    """Samplers whose texels are all k / 255 are stored as 8-bit RGBA on the
    device (tuning key texels_u8) and decoded through the table of those
    floats: every channel of every frame is bit-identical to the same scene
    stored as fp32 texels, whether the upload packs the texels on the device
    (tuning key gpu_tables, the default) or on the host, and the scene takes
    about a quarter of the texel bytes."""
    sc, cam, st0 = _small()
    st = type(st0).from_buffer_copy(bytes(st0))
    st.pixel_samples = 2
    dev, host, fp32 = (1, 1), (1, 0), (0, 1)
    out, mem = _render_modes(photon, sc, cam, st, (dev, host, fp32))
    _same_frames(out[dev], out[fp32])
    _same_frames(out[host], out[fp32])
    texel_bytes = sum(len(t) * 16 for _, t in sc.samplers)
    print(f"scene device memory: {mem[dev] / 2**20:.1f} MiB with 8-bit texels packed on the device, "
          f"{mem[host] / 2**20:.1f} MiB packed on the host, {mem[fp32] / 2**20:.1f} MiB fp32 "
          f"({texel_bytes / 2**20:.1f} MiB of fp32 texels)")
    assert mem[fp32] - mem[dev] >= 0.6 * texel_bytes
    assert mem[fp32] - mem[host] >= 0.6 * texel_bytes


def test_rgba8_packing_falls_back_to_fp32(photon):
    """A sampler with values that are not k / 255 (0.5 on every 7th texel's
    green channel, or -0.0 on every 11th texel's red channel) keeps fp32
    storage: the device packer flags it, the upload moves it to the float4
    array, and the images equal the all-fp32 scene's bit for bit; the other
    samplers stay 8-bit."""
    import copy
    sc0, cam, st0 = _small()
    sc = copy.copy(sc0)
    sc.samplers = list(sc0.samplers)
    planted = []
    for i, v, step, ch in ((0, 0.5, 7, 1), (len(sc.samplers) - 1, -0.0, 11, 0)):
        rec, t = sc.samplers[i]
        t = np.array(t, np.float32, copy=True).reshape(-1, 4)
        t[::step, ch] = v
        sc.samplers[i] = (rec, t)
        planted.append(i)
    st = type(st0).from_buffer_copy(bytes(st0))
    st.pixel_samples = 2
    dev, host, fp32 = (1, 1), (1, 0), (0, 1)
    out, mem = _render_modes(photon, sc, cam, st, (dev, host, fp32))
    _same_frames(out[dev], out[fp32])
    _same_frames(out[host], out[fp32])
    kept = sum(len(t) * 16 for i, (_, t) in enumerate(sc.samplers) if i not in planted)
    print(f"planted samplers {planted}: {mem[dev] / 2**20:.1f} MiB (device packing), "
          f"{mem[host] / 2**20:.1f} MiB (host), {mem[fp32] / 2**20:.1f} MiB fp32")
    assert mem[fp32] - mem[host] >= 0.6 * kept
