"""The comparator baseline/kokkos_port.cu (the reference's Kokkos BVH
back-end restated for the GPU) run on the CPU: its traversal must reproduce
the reference's own KokkosBackend records (golden fixture written by the
reference build) and the CPU oracle's, primitive ids included, since it
builds the same median-split tree and visits it in the same order.  The GPU
run of the same code is compared with this library's back-end in
test_gpu_kokkos_port.py and timed by bench.py."""
import numpy as np

from tests.golden import fixtures


def _port(*args, **kw):
    import baseline
    return baseline.KokkosPortAccel(*args, device=False, **kw)


def _same_records(got, ref):
    assert np.array_equal(got["hit"], ref["hit"])
    h = ref["hit"].astype(bool)
    for f in ("t", "position", "normal", "shading_normal", "bary"):
        assert np.array_equal(got[f][h].view(np.uint32), ref[f][h].view(np.uint32)), f
    assert np.array_equal(got["prim_id"][h], ref["prim_id"][h])
    assert np.array_equal(got["material_id"][h], ref["material_id"][h])


def test_port_matches_reference_fixture():
    z = fixtures.load_trace()
    acc = _port(z["positions"], z["indices"], z["normals"], z["material_ids"])
    got = acc.trace_host(z["orgs"], z["dirs"], z["tmin"], z["tmax"])
    _same_records(got, z["hits"].view(got.dtype).reshape(-1))
    occ = acc.trace_host(z["orgs"], z["dirs"], z["tmin"], z["tmax"], any_hit=True)
    assert np.array_equal(occ, z["occluded"])
    acc.close()


def test_port_matches_oracle_on_procedural_500k(oracle_lib):
    from photon_gb300 import workloads
    sc, _, _ = workloads.procedural_500k()
    rng = np.random.default_rng(11)
    n = 1 << 13
    lo, hi = sc.positions.min(0), sc.positions.max(0)
    o = rng.uniform(lo, hi, (n, 3)).astype(np.float32)
    o[:, 1] = rng.uniform(0.05, 6.0, n)
    d = rng.normal(size=(n, 3)).astype(np.float32)
    d /= np.linalg.norm(d, axis=1, keepdims=True)
    t0 = np.zeros(n, np.float32)
    t1 = np.full(n, 1e30, np.float32)
    t1[::7] = 0.0  # inactive rays (tmax < tmin) must miss
    acc = _port(sc.positions, sc.indices, sc.normals, sc.material_ids)
    info = acc.info()
    assert info["depth"] <= 64 and info["nodes"] < 2 * sc.triangle_count
    got = acc.trace_host(o, d, t0, t1)
    ref = oracle_lib.trace("oracle", sc.positions, sc.indices, o, d, t0, t1, False, sc.normals, sc.material_ids)
    _same_records(got, ref)
    assert not got["hit"][::7].any()
    occ = acc.trace_host(o, d, t0, t1, any_hit=True)
    ref_occ = oracle_lib.trace("oracle", sc.positions, sc.indices, o, d, t0, t1, True)
    assert np.array_equal(occ, ref_occ)
    acc.close()
