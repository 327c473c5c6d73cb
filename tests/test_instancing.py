"""Instanced geometry (phc_pt_scene objects + instances) on the CPU.

The renderer traces instances through a two-level BVH8: a top level over the
placements and one bottom level per object, entered with the ray carried
into object space (photon_gb300/csrc/traverse.cuh, trav_step2).  Here the
same __host__ __device__ traversal runs on the CPU over the renderer's own
host scene build (tests/native/host_traverse.cpp) against the single-level
traversal of the same geometry flattened into world space (the reference's
Kokkos back-end handles instances that way): every ray must agree on hit or
miss and on the material, and the distances must agree to float rounding of
the transforms.  The oracle renders both forms to the same image.  The pbrt
reader's instanced geometry (use_instancing) equals the reference's
ConvertedScene::instanced_geometry.
"""
import ctypes as C
import os

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
CSRC = os.path.join(ROOT, "photon_gb300", "csrc")


@pytest.fixture(scope="module")
def host_lib(host_traverse_lib):
    return host_traverse_lib


def _rays(seed, n, lo, hi):
    rng = np.random.default_rng(seed)
    o = rng.uniform(lo, hi, (n, 3)).astype(np.float32)
    d = rng.normal(size=(n, 3)).astype(np.float32)
    d /= np.linalg.norm(d, axis=1, keepdims=True)
    t1 = np.full(n, 1e30, np.float32)
    t1[::4] = rng.uniform(0.1, 3.0, len(t1[::4])).astype(np.float32)
    return o, d, np.zeros(n, np.float32), t1


def trace_instanced(lib, sc, o, d, t0, t1, any_hit=False):
    n = len(t0)
    desc, keep = sc.desc()
    out = np.zeros((n, 4), np.float32)
    obj = np.zeros(n, np.uint32)
    geo = np.zeros((n, 9), np.float32)
    st = np.zeros(5, np.uint64)
    vp = lambda a: a.ctypes.data_as(C.c_void_p)  # noqa: E731
    rc = lib.ht_trace_instanced(C.byref(desc), vp(o), vp(d), vp(t0), vp(t1), C.c_uint32(n), C.c_int(int(any_hit)),
                                vp(out), vp(obj), vp(geo), vp(st))
    assert rc == 0
    return out, obj, geo, st


def trace_flat(lib, sc, o, d, t0, t1, any_hit=False):
    n = len(t0)
    out = np.zeros((n, 4), np.float32)
    st = np.zeros(5, np.uint64)
    vp = lambda a: a.ctypes.data_as(C.c_void_p)  # noqa: E731
    lib.ht_trace(vp(sc.positions), C.c_uint64(len(sc.positions)), vp(sc.indices), C.c_uint64(len(sc.indices)),
                 vp(o), vp(d), vp(t0), vp(t1), C.c_uint32(n), C.c_int(int(any_hit)), C.c_int(1), vp(out), vp(st))
    return out, st


@pytest.mark.parametrize("seed,n_inst", [(0, 60), (5, 400)])
def test_two_level_traversal_matches_flattened(host_lib, seed, n_inst):
    from photon_gb300 import workloads
    sc, _, _ = workloads.instanced_objects(seed=seed, n_instances=n_inst)
    fl, _, _ = workloads.instanced_objects(seed=seed, n_instances=n_inst, flatten=True)
    o, d, t0, t1 = _rays(seed + 11, 100_000, [-4, 0.05, -4], [4, 2.5, 4])
    out, obj, geo, st = trace_instanced(host_lib, sc, o, d, t0, t1)
    assert st[3] < 64 and st[4] == n_inst + 1  # stack bound; placements + the scene's own triangles
    fo, fst = trace_flat(host_lib, fl, o, d, t0, t1)
    hi = out[:, 1].view(np.uint32) != 0xFFFFFFFF
    hf = fo[:, 1].view(np.uint32) != 0xFFFFFFFF
    assert (hi == hf).mean() >= 0.9999
    both = hi & hf
    rel = np.abs(out[both, 0] - fo[both, 0]) / np.maximum(fo[both, 0], 1e-6)
    # grazing hits magnify the float rounding of the transforms
    assert np.quantile(rel, 0.99) < 1e-4 and np.quantile(rel, 0.9999) < 1e-2
    # material of the hit: the object's for instances, the triangle's for the scene's own
    obj_mat = np.array([ob["material_id"] for ob in sc.pt.objects] + [0], np.uint32)
    scene_mat = sc.material_ids[np.minimum(out[:, 1].view(np.uint32), len(sc.material_ids) - 1)]
    mi = np.where(obj == 0xFFFFFFFF, scene_mat, obj_mat[np.minimum(obj, len(obj_mat) - 1)])
    mf = fl.material_ids[np.minimum(fo[:, 1].view(np.uint32), len(fl.material_ids) - 1)]
    assert (mi[both] == mf[both]).mean() >= 0.9999
    # world hit points agree; geometric normals of instance hits are unit length
    pf = o[both] + d[both] * fo[both, :1]
    assert np.quantile(np.abs(geo[both, :3] - pf).max(1), 0.99) < 1e-4
    inst_hit = both & (obj != 0xFFFFFFFF)
    assert np.allclose(np.linalg.norm(geo[inst_hit, 3:6], axis=1), 1.0, atol=1e-5)
    # occlusion
    occ, _, _, _ = trace_instanced(host_lib, sc, o, d, t0, t1, any_hit=True)
    focc, _ = trace_flat(host_lib, fl, o, d, t0, t1, any_hit=True)
    assert ((occ[:, 1].view(np.uint32) != 0xFFFFFFFF) == (focc[:, 1].view(np.uint32) != 0xFFFFFFFF)).mean() >= 0.9999
    # the two-level build holds the objects once
    assert st[2] < fst[2]


def test_oracle_instanced_render_matches_flattened(oracle_lib):
    from photon_gb300 import workloads
    imgs = []
    for flat in (False, True):
        sc, cam, st = workloads.instanced_objects(res=48, spp=16, flatten=flat)
        o = oracle_lib.CpuRenderer("oracle")
        o.set_scene(sc)
        o.render(cam, st, True)
        imgs.append(o.read("color")[..., :3])
    a, b = imgs
    assert abs(float(a.mean()) - float(b.mean())) / float(b.mean()) < 0.01
    assert float(np.abs(a - b).mean()) < 0.01 * float(b.mean()) + 1e-3


def _ref_available():
    import oracle
    return os.path.exists(oracle.REF_LIB)


@pytest.mark.skipif(not _ref_available(), reason="reference build (oracle/_ref) not present")
def test_pbrt_instanced_geometry_matches_reference(photon, oracle_lib):
    from photon_gb300 import pbrt
    path = os.path.join(ROOT, "tests", "golden", "pbrt", "features.pbrt")
    ref = oracle_lib.RefPbrt(path, use_instancing=True).instanced()
    ours = pbrt.load(path, use_instancing=True).arrays()
    assert len(ref["objects"]) == len(ours["objects"]) and len(ref["instances"]) == len(ours["instances"])
    for r, a in zip(ref["objects"], ours["objects"]):
        assert r["positions"].tobytes() == a["positions"].tobytes()
        assert np.array_equal(r["indices"], a["indices"].astype(np.int32))
        assert r["material_id"] == a["material_id"]
        # the reference's back-end uses normals only when there is one per vertex
        ref_has = r["normals"].size >= r["positions"].size
        assert ref_has == (a["normals"].size > 0)
        if ref_has:
            assert r["normals"][: r["positions"].size].tobytes() == a["normals"].tobytes()
    for (ri, rx), (ai, ax) in zip(ref["instances"], ours["instances"]):
        assert ri == ai and rx.tobytes() == ax.tobytes()


def test_instances_out_of_range_and_singular_are_skipped(host_lib):
    """Placements of unknown objects and singular transforms place nothing."""
    from photon_gb300 import workloads
    sc, _, _ = workloads.instanced_objects(n_instances=6)
    good = list(sc.pt.instances)
    sc.pt.instances = good + [(99, good[0][1]), (0, np.zeros(16, np.float32))]
    o, d, t0, t1 = _rays(3, 2000, [-4, 0.05, -4], [4, 2.5, 4])
    out, obj, geo, st = trace_instanced(host_lib, sc, o, d, t0, t1)
    assert st[4] == 7  # six placements and the scene's triangles
