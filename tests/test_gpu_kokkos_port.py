"""The comparator baseline/kokkos_port.cu on the GPU: the reference's Kokkos
BVH back-end restated for the GPU must find the same closest hits and the
same occlusion as its host run (checked against the reference's records in
test_kokkos_port.py) and as this library's BVH8 back-end, on the rays that
bench.py times.  Its device code contracts multiply-adds as the reference's
Kokkos-CUDA build does, so distances agree to rounding, not bit for bit."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _records(t):
    from photon_gb300 import _abi
    return np.frombuffer(t.cpu().numpy().tobytes(), _abi.hit_dtype())


def test_port_gpu_matches_host_and_ours(photon):
    import torch

    import baseline
    import bench
    from photon_gb300 import workloads
    sc, cam, st = workloads.procedural_500k()
    batches = bench.workload_rays(sc, cam, 256, 256)
    port = baseline.KokkosPortAccel(sc.positions, sc.indices, sc.normals, sc.material_ids)
    ours = photon.Accel(sc.positions, sc.indices, sc.normals, sc.material_ids)
    for name in ("camera", "bounce"):
        o, d, t0, t1 = batches[name]
        n = int(t0.numel())
        b = torch.zeros((n, 88), dtype=torch.uint8, device="cuda")
        port.trace(o, d, t0, t1, b)
        torch.cuda.synchronize()
        got = _records(b)
        host = port.trace_host(o.cpu().numpy(), d.cpu().numpy(), t0.cpu().numpy(), t1.cpu().numpy())
        mine = _records(ours.trace_closest(o, d, t0, t1))
        for ref in (host, mine):
            assert np.mean(got["hit"] == ref["hit"]) >= 0.999, name
            both = (got["hit"] != 0) & (ref["hit"] != 0)
            assert np.mean(got["prim_id"][both] == ref["prim_id"][both]) >= 0.995, name
            rel = np.abs(got["t"][both] - ref["t"][both]) / np.maximum(np.abs(ref["t"][both]), 1e-6)
            assert np.quantile(rel, 0.999) < 1e-4, name
    o, d, t0, t1 = batches["shadow"]
    n = int(t0.numel())
    b = torch.zeros(n, dtype=torch.int32, device="cuda")
    port.trace(o, d, t0, t1, b, any_hit=True)
    torch.cuda.synchronize()
    mine = ours.trace_occluded(o, d, t0, t1).cpu().numpy() != 0
    assert np.mean((b.cpu().numpy() != 0) == mine) >= 0.999
    port.close()
    ours.close()
