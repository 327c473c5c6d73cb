"""The drop-in boundary checked from the reference's side (C++): the
RayBackend and bridge::Renderer adapters of photon_gb300/adapters/ compile
against the reference's own headers (ray_backend.h, scene.h, RenderBridge.h,
through the project's Kokkos stand-in), with static_asserts that HitResult and
phc_hit_result have the same size and field offsets and that the bridge's
arrays keep their extents; they link with libphoton_cuda.so and run (without a
GPU, bridge::Renderer::initialize reports the library's error as the reference
does).  Needs the reference checkout (skipped where it is absent)."""
import os
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def test_adapters_build_against_reference_headers(photon, oracle_lib):
    if not oracle_lib.have_ref():
        pytest.skip("reference checkout not present")
    r = subprocess.run(["make", "-C", os.path.join(ROOT, "oracle"), "adapters"], capture_output=True, text=True)
    assert r.returncode == 0, r.stdout[-3000:] + r.stderr[-3000:]
    exe = os.path.join(ROOT, "oracle", "_ref", "adapter_check")
    out = subprocess.run([exe], capture_output=True, text=True, timeout=120)
    print(out.stdout)
    assert out.returncode == 0, out.stdout + out.stderr
    assert "backend cuda" in out.stdout
