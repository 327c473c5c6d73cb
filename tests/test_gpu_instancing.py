"""Instanced geometry on the GPU: the two-level BVH8 traversal (k_trace /
k_shadow with INST) and instance hit attributes in the shading kernels,
against the CPU oracle's instanced tracing on the same scene (per-sample
parity, tests/parity.py), and against the same geometry flattened.
"""
import os

import numpy as np
import pytest

from tests.parity import MIN_PATH_FRACTION, close_fraction

pytestmark = pytest.mark.gpu
ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _frames(photon, oracle_lib, sc, cam, st, frames):
    r = photon.Renderer()
    r.set_scene(sc)
    o = oracle_lib.CpuRenderer("oracle")
    o.set_scene(sc)
    out = []
    for f in range(frames):
        r.render(cam, st, True)
        o.render(cam, st, True)
        out.append({ch: (r.read(ch), o.read(ch)) for ch in ("color", "depth", "normal", "albedo")})
    return out


@pytest.mark.parametrize("n_inst", [60, 400])
def test_gpu_instanced_matches_oracle(photon, oracle_lib, n_inst):
    from photon_gb300 import workloads
    sc, cam, st = workloads.instanced_objects(n_instances=n_inst, res=96, spp=1)
    for f, fr in enumerate(_frames(photon, oracle_lib, sc, cam, st, 2)):
        for ch, (g, o) in fr.items():
            frac = close_fraction(g, o)
            assert frac >= MIN_PATH_FRACTION, f"frame {f} {ch}: {frac:.5f}"


def test_gpu_instanced_adaptive_matches_oracle(photon, oracle_lib):
    from photon_gb300 import workloads
    sc, cam, st = workloads.instanced_objects(res=64, spp=16)
    st.adaptive_sampling = 1
    fr = _frames(photon, oracle_lib, sc, cam, st, 1)[0]
    assert close_fraction(*fr["color"]) >= 0.99


def test_gpu_instanced_matches_flattened_image(photon):
    """The same geometry traced two-level and flattened: equal images up to
    the float rounding of the transforms."""
    from photon_gb300 import workloads
    imgs = []
    for flat in (False, True):
        sc, cam, st = workloads.instanced_objects(n_instances=200, res=128, spp=64, flatten=flat)
        r = photon.Renderer()
        r.set_scene(sc)
        r.render(cam, st, True)
        imgs.append(r.read("color")[..., :3])
    a, b = imgs
    assert abs(float(a.mean()) - float(b.mean())) / float(b.mean()) < 0.01
    assert float(np.abs(a - b).mean()) < 0.02 * float(b.mean())


def test_gpu_pbrt_instanced_matches_oracle(photon, oracle_lib):
    from photon_gb300 import pbrt
    sc = pbrt.load(os.path.join(ROOT, "tests", "golden", "pbrt", "features.pbrt"), use_instancing=True,
                   width=96, height=64, spp=1)
    st = type(sc.settings).from_buffer_copy(bytes(sc.settings))
    st.adaptive_sampling = 0
    fr = _frames(photon, oracle_lib, sc, sc.camera, st, 2)
    for f, d in enumerate(fr):
        assert close_fraction(*d["color"]) >= MIN_PATH_FRACTION, f"frame {f}"


def test_gpu_batch_with_an_instanced_job(photon):
    """A batch holding an instanced scene leaves every renderer as its own
    render call would."""
    from photon_gb300 import workloads
    sc1, cam1, st1 = workloads.instanced_objects(res=64, spp=4)
    sc2, cam2, st2 = workloads.box_room()
    st2.width = st2.height = 64
    st2.pixel_samples = 4
    solo = []
    for sc, cam, st in ((sc1, cam1, st1), (sc2, cam2, st2)):
        r = photon.Renderer()
        r.set_scene(sc)
        r.render(cam, st, True)
        solo.append(r.read("color"))
    rs = [photon.Renderer(), photon.Renderer()]
    rs[0].set_scene(sc1)
    rs[1].set_scene(sc2)
    photon.render_batch([(rs[0], cam1, st1, True), (rs[1], cam2, st2, True)])
    for r, s in zip(rs, solo):
        assert np.array_equal(r.read("color"), s)
