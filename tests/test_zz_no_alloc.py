"""phc_trace_closest_compact_static: the allocation-free trace entry point.

Some callers cannot allocate device memory while they trace (an application
that owns all device memory through its own pool or budget, or a hot loop in
which cudaMalloc / cudaFree would synchronise the device).  This entry point
gives them the same closest-hit results as phc_trace_closest_compact with the
kernel's scratch counter in an array compiled into the library.  Checked here
through the C-ABI against the allocating entry point, bit for bit (the
tolerance of the other trace tests), on two calls in a row, plus the size
limit.  This file sorts last so a stop-at-first-failure run has already run
every other test.
"""
import ctypes as C

import numpy as np
import pytest

from tests.golden import fixtures

pytestmark = pytest.mark.gpu

PHC_ERR_LIMIT = -7
PHC_STATIC_MAX_RAYS = 0x40000000


def _rays(n, seed):
    rng = np.random.default_rng(seed)
    o = rng.normal(size=(n, 3))
    o = (o / np.linalg.norm(o, axis=1, keepdims=True) * rng.uniform(0.3, 3.0, (n, 1))).astype(np.float32)
    d = (rng.normal(size=(n, 3)) * 0.3 - o).astype(np.float32)
    d /= np.linalg.norm(d, axis=1, keepdims=True)
    t0 = np.zeros(n, np.float32)
    t1 = np.full(n, 1e30, np.float32)
    t1[::9] = rng.uniform(0.1, 2.0, len(t1[::9])).astype(np.float32)
    t0[::17] = 1.0
    t1[::17] = 0.0
    return o, d, t0, t1


def test_static_scratch_trace_matches_allocating_trace(photon):
    import torch
    lib = photon.load()
    fn = lib.phc_trace_closest_compact_static
    z = fixtures.load_trace()
    acc = photon.Accel(z["positions"], z["indices"], z["normals"], z["material_ids"])
    for n, seed in ((2048, 1), (300_000, 2)):
        o, d, t0, t1 = (torch.from_numpy(a).cuda() for a in _rays(n, seed))
        want = acc.trace_closest_compact(o, d, t0, t1)
        torch.cuda.synchronize()
        assert (want[:, 1].view(torch.int32) != -1).any()
        for call in range(2):
            got = torch.full((n, 4), float("nan"), dtype=torch.float32, device="cuda")
            torch.cuda.synchronize()
            rc = fn(acc.h, o.data_ptr(), d.data_ptr(), t0.data_ptr(), t1.data_ptr(), n, got.data_ptr(), None)
            assert rc == 0, lib.phc_accel_error().decode()
            torch.cuda.synchronize()
            assert torch.equal(got.view(torch.int32), want.view(torch.int32)), f"n={n} call {call}"


def test_static_scratch_trace_rejects_oversize(photon):
    import torch
    lib = photon.load()
    z = fixtures.load_trace()
    acc = photon.Accel(z["positions"], z["indices"])
    buf = torch.zeros(16, dtype=torch.float32, device="cuda")
    rc = lib.phc_trace_closest_compact_static(acc.h, buf.data_ptr(), buf.data_ptr(), buf.data_ptr(),
                                              buf.data_ptr(), PHC_STATIC_MAX_RAYS + 1, buf.data_ptr(), None)
    assert rc == PHC_ERR_LIMIT
    assert "exceeds the maximum" in lib.phc_accel_error().decode()
    assert torch.count_nonzero(buf).item() == 0
