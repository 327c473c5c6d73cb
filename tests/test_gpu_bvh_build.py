"""The GPU BVH8 builder (tuning key "gpu_bvh", photon_gb300/csrc/bvh_gpu.cu).

The BVH's shape never changes what a ray hits, only the order nodes are
visited in, so the GPU-built tree must give the same hit records as the
reference (golden fixture, through Level A) and the oracle: hit/miss, t and
attributes bit-identical, primitive ids identical except exact-distance
ties.  Renders over it keep per-sample parity.  Edge cases: one triangle,
coincident triangles (equal Morton codes, zero-area merges), a flat mesh.
"""
import numpy as np
import pytest

from tests.golden import fixtures
from tests.parity import MIN_PATH_FRACTION, close_fraction

pytestmark = pytest.mark.gpu


@pytest.fixture(params=[(1, 4, 0), (2, 4, 0), (3, 4, 0), (2, 2, 0), (2, 32, 0), (1, 4, 30), (2, 4, 30), (3, 4, 30),
                        (2, 4, 5), (2, 4, 300)],
                ids=lambda p: f"leaf{p[0]}-radius{p[1]}-tricost{p[2]}")
def gpu_bvh(photon, request):
    """The GPU builder, with leaf children of up to 1, 2 or 3 triangles
    (tuning key gpu_max_leaf), clustering radii 2, 4 and 32 (ploc_radius),
    and the greedy collapse or the surface-area collapse at triangle costs
    of 0.05, 0.3 and 3 node visits (collapse_tri_cost)."""
    from photon_gb300 import tuning_get, tuning_set
    keys = ("gpu_bvh", "gpu_max_leaf", "ploc_radius", "collapse_tri_cost")
    old = {k: tuning_get(k) for k in keys}
    tuning_set("gpu_bvh", 1)
    tuning_set("gpu_max_leaf", request.param[0])
    tuning_set("ploc_radius", request.param[1])
    tuning_set("collapse_tri_cost", request.param[2])
    yield
    for k, v in old.items():
        tuning_set(k, v)


def _to_dev(*arrs):
    import torch
    return [torch.from_numpy(np.ascontiguousarray(a)).cuda() for a in arrs]


def _records(buf):
    from photon_gb300 import _abi
    return np.frombuffer(np.ascontiguousarray(buf).tobytes(), _abi.hit_dtype())


def _check_against(got, ref, tie_frac=0.01):
    assert np.array_equal(got["hit"], ref["hit"])
    h = ref["hit"].astype(bool)
    assert np.array_equal(got["t"][h].view(np.uint32), ref["t"][h].view(np.uint32))
    same = got["prim_id"][h] == ref["prim_id"][h]
    assert (~same).mean() <= tie_frac
    for f in ("position", "normal", "shading_normal", "bary"):
        assert np.array_equal(got[f][h][same].view(np.uint32), ref[f][h][same].view(np.uint32)), f


def test_gpu_built_bvh_matches_reference_fixture(photon, gpu_bvh):
    z = fixtures.load_trace()
    acc = photon.Accel(z["positions"], z["indices"], z["normals"], z["material_ids"])
    o, d, t0, t1 = _to_dev(z["orgs"], z["dirs"], z["tmin"], z["tmax"])
    _check_against(_records(acc.trace_closest(o, d, t0, t1).cpu().numpy()), _records(z["hits"]))
    occ = acc.trace_occluded(o, d, t0, t1).cpu().numpy()
    assert np.array_equal(occ.astype(np.uint32), z["occluded"])


def test_gpu_built_bvh_procedural_500k_matches_oracle(photon, oracle_lib, gpu_bvh):
    from photon_gb300 import workloads
    sc, _, _ = workloads.procedural_500k()
    rng = np.random.default_rng(6)
    n = 1 << 18
    lo, hi = sc.positions.min(0), sc.positions.max(0)
    o = rng.uniform(lo, hi, (n, 3)).astype(np.float32)
    o[:, 1] = rng.uniform(0.05, 6.0, n)
    d = rng.normal(size=(n, 3)).astype(np.float32)
    d /= np.linalg.norm(d, axis=1, keepdims=True)
    t0 = np.zeros(n, np.float32)
    t1 = np.full(n, 1e30, np.float32)
    ref = oracle_lib.trace("oracle", sc.positions, sc.indices, o, d, t0, t1, False, sc.normals, sc.material_ids)
    acc = photon.Accel(sc.positions, sc.indices, sc.normals, sc.material_ids)
    assert acc.info()["tri_bytes"] == 48 * sc.triangle_count  # one leaf record per triangle
    do, dd, dt0, dt1 = _to_dev(o, d, t0, t1)
    _check_against(_records(acc.trace_closest(do, dd, dt0, dt1).cpu().numpy()), ref, tie_frac=1e-4)


@pytest.mark.parametrize("kind", ["one", "coincident", "flat"])
def test_gpu_built_bvh_edge_cases(photon, oracle_lib, gpu_bvh, kind):
    rng = np.random.default_rng(2)
    if kind == "one":
        pos = np.array([[0, 0, 0], [1, 0, 0], [0, 1, 0]], np.float32)
        idx = np.array([[0, 1, 2]], np.uint32)
    elif kind == "coincident":  # 300 copies of 4 triangles: equal Morton codes and boxes
        base = rng.uniform(-1, 1, (12, 3)).astype(np.float32)
        pos = np.tile(base, (300, 1))
        idx = (np.arange(1200 * 3, dtype=np.uint32)).reshape(-1, 3)
    else:  # a 64 x 64 grid in the plane y = 0 (zero extent on one axis)
        g = np.stack(np.meshgrid(np.arange(65), np.arange(65), indexing="ij"), -1).reshape(-1, 2).astype(np.float32)
        pos = np.stack([g[:, 0] / 64, np.zeros(len(g)), g[:, 1] / 64], -1).astype(np.float32)
        i, j = np.meshgrid(np.arange(64), np.arange(64), indexing="ij")
        a = (i * 65 + j).ravel()
        idx = np.concatenate([np.stack([a, a + 65, a + 1], 1), np.stack([a + 1, a + 65, a + 66], 1)]).astype(np.uint32)
    n = 20000
    o = rng.uniform(-1.5, 1.5, (n, 3)).astype(np.float32)
    d = rng.normal(size=(n, 3)).astype(np.float32)
    d /= np.linalg.norm(d, axis=1, keepdims=True)
    t0 = np.zeros(n, np.float32)
    t1 = np.full(n, 1e30, np.float32)
    ref = oracle_lib.trace("oracle", pos, idx, o, d, t0, t1, False)
    acc = photon.Accel(pos, idx)
    do, dd, dt0, dt1 = _to_dev(o, d, t0, t1)
    got = _records(acc.trace_closest(do, dd, dt0, dt1).cpu().numpy())
    assert np.array_equal(got["hit"], ref["hit"])
    h = ref["hit"].astype(bool)
    assert np.array_equal(got["t"][h].view(np.uint32), ref["t"][h].view(np.uint32))
    if kind != "coincident":  # coincident copies tie on every hit
        assert (got["prim_id"][h] != ref["prim_id"][h]).mean() < 0.01


@pytest.mark.parametrize("name", ["box_room", "env", "textures"])
def test_render_over_gpu_built_bvh_matches_reference(photon, gpu_bvh, name):
    sc, cam, st, ref_frames = fixtures.load_scene(name)
    r = photon.Renderer()
    r.set_scene(sc)
    for f, ref in enumerate(ref_frames):
        r.render(cam, st, True)
        frac = close_fraction(r.read("color"), ref["color"])
        assert frac >= MIN_PATH_FRACTION, f"{name} frame {f}: {frac:.5f}"
