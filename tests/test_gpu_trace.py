"""Level A on the GPU: phc_trace_closest / phc_trace_occluded through the
C-ABI against the reference's KokkosBackend (golden fixture) and the CPU
oracle (500K-triangle workload).

Bar: hit/miss decisions, t, barycentrics and every attribute of the hit
record bit-identical; the primitive id identical except where two triangles
give exactly the same t (a tie the reference breaks by its own traversal
order), which must stay rare.
"""
import numpy as np
import pytest

from tests.golden import fixtures

pytestmark = pytest.mark.gpu


def _to_dev(*arrs):
    import torch
    return [torch.from_numpy(np.ascontiguousarray(a)).cuda() for a in arrs]


def _records(buf):
    from photon_gb300 import _abi
    return np.frombuffer(np.ascontiguousarray(buf).tobytes(), _abi.hit_dtype())


def _ties(name, got, ref, h):
    """Primitive-id disagreements among rays both sides hit, every one of
    them at the same distance t bit for bit (an exact tie: the reference
    keeps the last triangle its traversal tests with t <= best.t,
    mesh_intersector.h:92-95, a BVH8 tests them in another order).  Prints
    the count and the first few (ray, this library's prim, the reference's
    prim, t) and returns the count."""
    same_t = got["t"][h].view(np.uint32) == ref["t"][h].view(np.uint32)
    diff = got["prim_id"][h] != ref["prim_id"][h]
    assert not (diff & ~same_t).any(), "a primitive-id disagreement that is not an exact tie"
    rays = np.flatnonzero(h)[diff]
    listed = ", ".join(f"ray {i}: {got['prim_id'][i]} vs {ref['prim_id'][i]} at t={ref['t'][i]:.6g}"
                       for i in rays[:4])
    print(f"{name}: {int(h.sum())} hits of {len(h)} rays, {len(rays)} exact-t ties "
          f"({len(rays) / max(1, int(h.sum())):.2e})" + (f"; {listed}" if len(rays) else ""))
    return len(rays)


def test_trace_closest_matches_reference_fixture(photon):
    z = fixtures.load_trace()
    acc = photon.Accel(z["positions"], z["indices"], z["normals"], z["material_ids"])
    o, d, t0, t1 = _to_dev(z["orgs"], z["dirs"], z["tmin"], z["tmax"])
    got = _records(acc.trace_closest(o, d, t0, t1).cpu().numpy())
    ref = _records(z["hits"])
    assert np.array_equal(got["hit"], ref["hit"])
    h = ref["hit"].astype(bool)
    assert np.array_equal(got["t"][h].view(np.uint32), ref["t"][h].view(np.uint32))
    same = got["prim_id"][h] == ref["prim_id"][h]
    # disagreements only on exact ties
    ties = _ties("trace fixture (reference KokkosBackend records)", got, ref, h)
    assert ties < 0.01 * h.sum()
    for f in ("position", "normal", "shading_normal", "bary"):
        a, b = got[f][h][same], ref[f][h][same]
        assert np.array_equal(a.view(np.uint32), b.view(np.uint32)), f
    assert np.array_equal(got["material_id"][h][same], ref["material_id"][h][same])
    occ = acc.trace_occluded(o, d, t0, t1).cpu().numpy()
    assert np.array_equal(occ.astype(np.uint32), z["occluded"])


def test_trace_compact_matches_full(photon):
    z = fixtures.load_trace()
    acc = photon.Accel(z["positions"], z["indices"])
    o, d, t0, t1 = _to_dev(z["orgs"], z["dirs"], z["tmin"], z["tmax"])
    full = _records(acc.trace_closest(o, d, t0, t1).cpu().numpy())
    comp = acc.trace_closest_compact(o, d, t0, t1).cpu().numpy()
    prim = comp[:, 1].view(np.uint32)
    assert np.array_equal(prim != 0xffffffff, full["hit"].astype(bool))
    h = full["hit"].astype(bool)
    assert np.array_equal(prim[h], full["prim_id"][h])
    assert np.array_equal(comp[h, 0].view(np.uint32), full["t"][h].view(np.uint32))


def test_trace_procedural_500k_matches_oracle(photon, oracle_lib):
    from photon_gb300 import workloads
    sc, _, _ = workloads.procedural_500k()
    rng = np.random.default_rng(5)
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
    do, dd, dt0, dt1 = _to_dev(o, d, t0, t1)
    got = _records(acc.trace_closest(do, dd, dt0, dt1).cpu().numpy())
    assert np.array_equal(got["hit"], ref["hit"])
    h = ref["hit"].astype(bool)
    assert np.array_equal(got["t"][h].view(np.uint32), ref["t"][h].view(np.uint32))
    ties = _ties("500K workload, random rays", got, ref, h)
    assert ties <= max(1, int(1e-4 * h.sum()))
    occ = acc.trace_occluded(do, dd, dt0, dt1).cpu().numpy()
    assert np.array_equal(occ != 0, h)


def test_trace_workload_rays_match_oracle(photon, oracle_lib):
    """The 500K workload's own ray distribution at full size: 1024^2 jittered
    camera rays, then cosine bounce rays from their hits.  Hit/miss and t bit
    for bit against the oracle's median-split BVH (the reference's
    traversal); primitive ids equal except exact-t ties, which are counted
    and printed."""
    from photon_gb300 import workloads
    from tests.rays import bounce_rays, camera_rays
    sc, cam, st = workloads.procedural_500k()
    acc = photon.Accel(sc.positions, sc.indices, sc.normals, sc.material_ids)
    scale = float(np.abs(sc.positions).max())
    batch = camera_rays(cam, st.width, st.height)
    total_ties = 0
    for name in ("camera", "bounce"):
        ref = oracle_lib.trace("oracle", sc.positions, sc.indices, *batch, False, sc.normals, sc.material_ids)
        got = _records(acc.trace_closest(*_to_dev(*batch)).cpu().numpy())
        assert np.array_equal(got["hit"], ref["hit"]), name
        h = ref["hit"].astype(bool)
        assert np.array_equal(got["t"][h].view(np.uint32), ref["t"][h].view(np.uint32)), name
        same = got["prim_id"][h] == ref["prim_id"][h]
        for f in ("position", "normal", "shading_normal", "bary"):
            assert np.array_equal(got[f][h][same].view(np.uint32), ref[f][h][same].view(np.uint32)), (name, f)
        total_ties += _ties(f"500K workload, {name} rays", got, ref, h)
        if name == "camera":
            batch = bounce_rays(ref, batch[1], scale)
    assert total_ties <= max(1, int(1e-4 * len(batch[0])))


def test_trace_empty_and_inactive_rays(photon):
    """Rays with tmax < tmin report a miss (the reference's dead-ray
    encoding, pathtracer.cpp:1119-1120); n = 0 is a no-op."""
    z = fixtures.load_trace()
    acc = photon.Accel(z["positions"], z["indices"])
    n = 64
    o = np.zeros((n, 3), np.float32)
    o[:, 2] = 3.0
    d = np.tile(np.array([0, 0, -1], np.float32), (n, 1))
    t0 = np.ones(n, np.float32)
    t1 = np.zeros(n, np.float32)
    do, dd, dt0, dt1 = _to_dev(o, d, t0, t1)
    got = _records(acc.trace_closest(do, dd, dt0, dt1).cpu().numpy())
    assert not got["hit"].any()
    assert not acc.trace_occluded(do, dd, dt0, dt1).cpu().numpy().any()
    dt1[:] = 1e30
    dt0[:] = 0
    got = _records(acc.trace_closest(do, dd, dt0, dt1).cpu().numpy())
    assert got["hit"].all()
