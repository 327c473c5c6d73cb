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


def test_gpu_level_a_instanced_accel(photon):
    """RayBackend::build_accel_instanced through phc_accel_create_instanced:
    hit or miss and distance as the flattened accel, and the instanced
    back-end's record fields (object index as inst_id, prim_id within the
    object, the object's material, barycentrics as uv)."""
    import torch
    from photon_gb300 import workloads
    sc, _, _ = workloads.instanced_objects(n_instances=120)
    fl, _, _ = workloads.instanced_objects(n_instances=120, flatten=True)
    objs, insts = sc.pt.objects, sc.pt.instances
    acc = photon.Accel(sc.positions, sc.indices, sc.normals, sc.material_ids, objects=objs, instances=insts)
    flat = photon.Accel(fl.positions, fl.indices, fl.normals, fl.material_ids)
    rng = np.random.default_rng(4)
    n = 100_000
    o = torch.tensor(rng.uniform([-4, 0.05, -4], [4, 2.5, 4], (n, 3)), dtype=torch.float32, device="cuda")
    d = torch.nn.functional.normalize(torch.randn(n, 3, device="cuda"), dim=1)
    t0 = torch.zeros(n, device="cuda")
    t1 = torch.full((n,), 1e30, device="cuda")
    hi = acc.trace_closest(o, d, t0, t1).cpu().numpy()
    hf = flat.trace_closest(o, d, t0, t1).cpu().numpy()
    f32 = lambda r, a, b: r[:, a:b].copy().view(np.float32)  # noqa: E731
    u32 = lambda r, a, b: r[:, a:b].copy().view(np.uint32)  # noqa: E731
    hit_i, hit_f = hi[:, 84] == 1, hf[:, 84] == 1
    assert (hit_i == hit_f).mean() >= 0.9999
    both = hit_i & hit_f
    ti, tf = f32(hi, 0, 4)[both, 0], f32(hf, 0, 4)[both, 0]
    assert np.quantile(np.abs(ti - tf) / np.maximum(tf, 1e-6), 0.99) < 1e-4
    mat_i, mat_f = u32(hi, 80, 84)[:, 0], u32(hf, 80, 84)[:, 0]
    assert (mat_i[both] == mat_f[both]).mean() >= 0.9999
    inst = u32(hi, 76, 80)[:, 0]
    prim = u32(hi, 68, 72)[:, 0]
    on_obj = both & (inst < len(objs))
    assert on_obj.any() and (inst[both & ~on_obj] == len(objs)).all()
    ntri = np.array([len(ob["indices"]) for ob in objs])
    assert (prim[on_obj] < ntri[inst[on_obj]]).all()
    assert np.array_equal(mat_i[on_obj], np.array([ob["material_id"] for ob in objs])[inst[on_obj]])
    assert np.array_equal(f32(hi, 40, 48)[both], f32(hi, 48, 56)[both])  # uv = barycentrics
    occ_i = torch.zeros(n, dtype=torch.int32, device="cuda")
    occ_f = torch.zeros(n, dtype=torch.int32, device="cuda")
    acc.trace_occluded(o, d, t0, t1, occ_i)
    flat.trace_occluded(o, d, t0, t1, occ_f)
    assert (occ_i.cpu().numpy() == occ_f.cpu().numpy()).mean() >= 0.9999
