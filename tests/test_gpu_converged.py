"""Converged images: GPU against the CPU oracle at 4096 samples per pixel.

The two sides use disjoint sample ranges (the GPU renderer first spends 4096
samples per pixel, so its frames continue from sample 4096), so the images are
independent estimates of the same integral.  Each side renders 16 frames of
256 spp; per pixel, the mean of the frames is the 4096-spp estimate and their
spread gives its standard error.  Bars: relative MSE of the two 4096-spp
images below the scene's REL_MSE (against the image's mean square), and no
more than twice what the two images' own noise explains (the mean squared
standard error over the mean square: the difference of two unbiased
estimates is noise alone); a per-pixel z-test: |z| > Z_MAX on at most
Z_FRACTION of the pixel channels (with 16 frames the standard-error estimate
has a heavy tail; a shared bias of the renderer would push most pixels past
the bound).

The 500K-triangle workload (1024x512 sun+sky environment, glass, metal,
clearcoat, 4 emissive triangles) runs at 128^2: its caustics through glass
and the sun make the estimate noisy (two independent 4096-spp oracle images
differ by a relative MSE of about 4e-3), hence its wider REL_MSE.  Equal
sample counts on the same per-sample stream give equal error, so this is the
matched-MSE check behind comparing the two renderers' Msamples/s.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

FRAMES = 16
SPP = 256
# scene -> (resolution, relative-MSE bar)
SCENES = {"box_room": (40, 2e-3), "glass": (40, 2e-3), "volume": (40, 2e-3), "textures": (40, 2e-3),
          "procedural_500k": (128, 1e-2)}
Z_MAX = 4.0
Z_FRACTION = 0.01


def _frames_gpu(photon, sc, cam, st):
    r = photon.Renderer()
    r.set_scene(sc)
    skip = type(st).from_buffer_copy(bytes(st))
    skip.pixel_samples = FRAMES * SPP
    r.render(cam, skip, True)
    out = []
    for _ in range(FRAMES):
        r.render(cam, st, True)
        out.append(r.read("color")[..., :3].astype(np.float64))
    r.close()
    return np.stack(out)


def _frames_cpu(oracle_lib, sc, cam, st):
    r = oracle_lib.CpuRenderer("oracle")
    r.set_scene(sc)
    out = []
    for _ in range(FRAMES):
        r.render(cam, st, True)
        out.append(r.read("color")[..., :3].astype(np.float64))
    r.close()
    return np.stack(out)


def _scene(kind):
    from photon_gb300 import workloads
    if kind == "box_room":
        sc, cam, st = workloads.box_room()
    elif kind == "procedural_500k":
        sc, cam, st = workloads.procedural_500k()
    else:
        sc, cam, st = workloads.feature_scene(kind)
    st.width = st.height = SCENES[kind][0]
    st.pixel_samples = SPP
    st.adaptive_sampling = 0
    return sc, cam, st


@pytest.mark.parametrize("kind", list(SCENES))
def test_converged_4096spp_matches_oracle(photon, oracle_lib, kind):
    sc, cam, st = _scene(kind)
    g = _frames_gpu(photon, sc, cam, st)
    c = _frames_cpu(oracle_lib, sc, cam, st)
    mg, mc = g.mean(0), c.mean(0)
    rel_mse = float(np.mean((mg - mc) ** 2) / np.mean(mc ** 2))
    se = np.sqrt(g.var(0, ddof=1) / FRAMES + c.var(0, ddof=1) / FRAMES)
    noise_mse = float(np.mean(se ** 2) / np.mean(mc ** 2))
    ok = se > 0
    z = np.zeros_like(mg)
    z[ok] = (mg[ok] - mc[ok]) / se[ok]
    frac = float(np.mean(np.abs(z) > Z_MAX))
    print(f"{kind} {st.width}^2 x {FRAMES * SPP} spp: rel MSE {rel_mse:.2e} (noise alone {noise_mse:.2e}, "
          f"bar {SCENES[kind][1]:.0e}), |z| > {Z_MAX}: {frac:.4f}, mean z {z[ok].mean():+.3f}")
    assert rel_mse <= SCENES[kind][1], rel_mse
    assert rel_mse <= 2.0 * noise_mse, (rel_mse, noise_mse)
    assert frac <= Z_FRACTION, frac
    # no shared bias: the mean z over all pixels is near zero
    assert abs(float(z[ok].mean())) < 0.15
