"""Batched mode (phc_render_batch) on the GPU.

The bar: every job of a batch leaves its renderer with exactly the image,
channels and sample count its own phc_render call would give, bit for bit,
whatever the batch composition (mixed scene features, sizes, depths, sample
counts, several waves sharing jobs), and across progressive calls.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

CHANNELS = ("color", "depth", "normal", "albedo")


def _jobs():
    from photon_gb300 import workloads
    out = []
    for kind, res, spp, depth in (("glass", 40, 3, 5), ("env", 24, 5, 4), ("textures", 32, 2, 6),
                                  ("lights", 48, 4, 3), ("volume", 20, 2, 6)):
        sc, cam, st = workloads.feature_scene(kind, res=res)
        st.pixel_samples = spp
        st.max_depth = depth
        out.append((sc, cam, st))
    for sc, cam, st in workloads.batched_jobs(seed=3, n=3, max_tris=20_000, min_res=16, max_res=48, spp=(2, 9)):
        out.append((sc, cam, st))
    return out


def _bits(a):
    return np.ascontiguousarray(a, np.float32).view(np.uint32)


@pytest.mark.parametrize("wave_paths", [0, 3000])
def test_batch_matches_plain_bit_for_bit(photon, wave_paths):
    from photon_gb300 import tuning_get, tuning_set
    old = tuning_get("batch_wave_paths")
    try:
        if wave_paths:
            tuning_set("batch_wave_paths", wave_paths)
        jobs = _jobs()
        plain, batch = [], []
        for sc, cam, st in jobs:
            a = photon.Renderer()
            a.set_scene(sc)
            b = photon.Renderer()
            b.set_scene(sc)
            plain.append(a)
            batch.append(b)
        for frame in range(2):  # the second call accumulates onto the first
            for r, (sc, cam, st) in zip(plain, jobs):
                r.render(cam, st, frame == 0)
            stats = photon.render_batch([(r, cam, st, frame == 0) for r, (sc, cam, st) in zip(batch, jobs)])
            want = sum(st.width * st.height * st.pixel_samples for _, _, st in jobs)
            assert stats["pixel_samples"] == want
            for k, (a, b) in enumerate(zip(plain, batch)):
                assert a.accumulated_samples() == b.accumulated_samples()
                for ch in CHANNELS:
                    assert np.array_equal(_bits(a.read(ch)), _bits(b.read(ch))), f"job {k} frame {frame} {ch}"
    finally:
        tuning_set("batch_wave_paths", old)


def test_batch_with_adaptive_job_and_errors(photon):
    from photon_gb300 import PhotonError, workloads
    sc, cam, st = workloads.feature_scene("basic", res=32)
    st.pixel_samples = 20
    st.adaptive_sampling = 1
    sc2, cam2, st2 = workloads.feature_scene("glass", res=24)
    st2.pixel_samples = 3
    a, b = photon.Renderer(), photon.Renderer()
    a.set_scene(sc)
    b.set_scene(sc2)
    photon.render_batch([(a, cam, st, True), (b, cam2, st2, True)])
    ref = photon.Renderer()
    ref.set_scene(sc)
    ref.render(cam, st, True)
    assert np.array_equal(_bits(ref.read("color")), _bits(a.read("color")))
    with pytest.raises(PhotonError, match="twice"):
        photon.render_batch([(a, cam, st, True), (a, cam, st, True)])
    c = photon.Renderer()  # no scene
    with pytest.raises(PhotonError, match="NO_SCENE"):
        photon.render_batch([(b, cam2, st2, True), (c, cam2, st2, True)])


def test_batch_class_kernels_match_plain(photon):
    """Lean jobs only (procedural Disney materials of several shading
    classes), with the material sort and the class kernels forced on for
    every wave (tuning keys sort_threshold 1, class_threshold 0): the
    batched wavefront's class kernels (shade_classes_batch.cu) leave every
    job with the image its own render gives, bit for bit."""
    from photon_gb300 import tuning_get, tuning_set, workloads
    keys = {"sort_threshold": 1, "class_threshold": 0}
    old = {k: tuning_get(k) for k in keys}
    try:
        for k, v in keys.items():
            tuning_set(k, v)
        jobs = list(workloads.batched_jobs(seed=5, n=6, max_tris=30_000, min_res=32, max_res=64, spp=(2, 6)))
        plain, batch = [], []
        for sc, cam, st in jobs:
            a = photon.Renderer()
            a.set_scene(sc)
            b = photon.Renderer()
            b.set_scene(sc)
            plain.append(a)
            batch.append(b)
        for r, (sc, cam, st) in zip(plain, jobs):
            r.render(cam, st, True)
        photon.render_batch([(r, cam, st, True) for r, (sc, cam, st) in zip(batch, jobs)])
        for k, (a, b) in enumerate(zip(plain, batch)):
            for ch in CHANNELS:
                assert np.array_equal(_bits(a.read(ch)), _bits(b.read(ch))), f"job {k} {ch}"
    finally:
        for k, v in old.items():
            tuning_set(k, v)
