"""The traversal counters behind the roofline's algorithmic bytes (node
visits V_node and triangle tests V_tri, counted by the kernels themselves)
against a CPU replay of the same BVH8 on a 1% ray sample of the 500K
workload: the Level-A back-end built with the host builder (tuning key
gpu_bvh 0, so that the CPU harness builds the identical tree), the same
traversal code run on the CPU (tests/native/host_traverse.cpp).  The box
and triangle tests round identically on both, so the counts must be equal,
not just close."""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _host_counts(lib, pos, idx, o, d, t0, t1, any_hit, max_leaf):
    n = len(t0)
    out = np.zeros((n, 4), np.float32)
    st = np.zeros(5, np.uint64)
    arrs = [np.ascontiguousarray(a) for a in (pos, idx, o, d, t0, t1)]
    lib.ht_trace(C.c_void_p(arrs[0].ctypes.data), C.c_uint64(arrs[0].size // 3), C.c_void_p(arrs[1].ctypes.data),
                 C.c_uint64(arrs[1].size // 3), *[C.c_void_p(a.ctypes.data) for a in arrs[2:]], C.c_uint32(n),
                 C.c_int(int(any_hit)), C.c_int(max_leaf), C.c_void_p(out.ctypes.data), C.c_void_p(st.ctypes.data))
    return out, int(st[0]), int(st[1])


def test_counters_match_cpu_replay(photon, host_traverse_lib):
    import torch
    from photon_gb300 import _abi, tuning_get, tuning_set, workloads
    from tests.rays import bounce_rays, camera_rays
    sc, cam, st = workloads.procedural_500k()
    keys = ("gpu_bvh", "count_traversal", "max_leaf")
    old = {k: tuning_get(k) for k in keys}
    try:
        tuning_set("gpu_bvh", 0)
        tuning_set("count_traversal", 1)
        max_leaf = tuning_get("max_leaf")
        acc = photon.Accel(sc.positions, sc.indices, sc.normals, sc.material_ids)
        cam_rays = [a[::100].copy() for a in camera_rays(cam, st.width, st.height)]  # 1% of the frame
        dev = lambda arrs: [torch.from_numpy(np.ascontiguousarray(a)).cuda() for a in arrs]
        rec = np.frombuffer(acc.trace_closest(*dev(cam_rays)).cpu().numpy().tobytes(), _abi.hit_dtype())
        batches = {"camera": cam_rays,
                   "bounce": bounce_rays(rec, cam_rays[1], float(np.abs(sc.positions).max()))}
        for name, rays in batches.items():
            for any_hit in (False, True):
                if any_hit:
                    occ = acc.trace_occluded(*dev(rays)).cpu().numpy()
                else:
                    got = acc.trace_closest_compact(*dev(rays)).cpu().numpy()
                g_nodes, g_tris = acc.counters()
                out, h_nodes, h_tris = _host_counts(host_traverse_lib, sc.positions, sc.indices, *rays, any_hit,
                                                    max_leaf)
                kind = "any hit" if any_hit else "closest hit"
                n = len(rays[0])
                print(f"{name} rays ({n}), {kind}: GPU {g_nodes} node visits, {g_tris} triangle tests "
                      f"({g_nodes / n:.2f} / {g_tris / n:.2f} per ray); CPU replay {h_nodes}, {h_tris}")
                assert (g_nodes, g_tris) == (h_nodes, h_tris), (name, kind)
                if any_hit:
                    hit = out[:, 1].view(np.uint32) != 0xffffffff
                    assert np.array_equal(occ != 0, hit), (name, kind)
                else:
                    assert np.array_equal(got[:, 1].view(np.uint32), out[:, 1].view(np.uint32)), (name, kind)
                    assert np.array_equal(got[:, 0].view(np.uint32), out[:, 0].view(np.uint32)), (name, kind)
        acc.close()
    finally:
        for k, v in old.items():
            tuning_set(k, v)
