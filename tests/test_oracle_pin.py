"""Pins the CPU restatement oracle (oracle/photon_oracle.cpp).

1. Against the golden fixtures, which were produced by the reference's own
   sources (tests/golden/make_golden.py): every channel of every frame of
   every fixture scene, the Level-A hit records and the BSDF probes must be
   bit-identical.
2. Where the reference checkout is present, against the reference compiled
   here, on scenes the fixtures do not hold (the 500K-triangle workload,
   adaptive sampling, progressive accumulation).
"""

import numpy as np
import pytest

from tests.golden import fixtures


@pytest.fixture(scope="module")
def ref_oracle(oracle_lib):
    """The reference compiled here; built by oracle.build() only where its
    checkout exists, so the tests using it skip elsewhere (the GPU host)."""
    if not oracle_lib.have_ref():
        pytest.skip("reference checkout not present: its oracle is not built")
    return oracle_lib


def bits(a):
    return np.ascontiguousarray(a, np.float32).view(np.uint32)


@pytest.mark.parametrize("name", fixtures.scene_names())
def test_oracle_matches_reference_fixture(oracle_lib, name):
    sc, cam, st, frames = fixtures.load_scene(name)
    r = oracle_lib.CpuRenderer("oracle")
    r.set_scene(sc)
    for f, ref in enumerate(frames):
        r.render(cam, st, True)
        for ch in ("color", "depth", "normal", "albedo"):
            got = r.read(ch)
            assert np.array_equal(bits(got), bits(ref[ch])), f"{name} frame {f} {ch}"


def test_oracle_trace_matches_reference_fixture(oracle_lib):
    z = fixtures.load_trace()
    hits = oracle_lib.trace("oracle", z["positions"], z["indices"], z["orgs"], z["dirs"], z["tmin"], z["tmax"],
                            False, z["normals"], z["material_ids"])
    assert np.array_equal(np.frombuffer(hits.tobytes(), np.uint8).reshape(-1, 88), z["hits"])
    occ = oracle_lib.trace("oracle", z["positions"], z["indices"], z["orgs"], z["dirs"], z["tmin"], z["tmax"],
                           True, z["normals"], z["material_ids"])
    assert np.array_equal(occ, z["occluded"])


def test_oracle_bsdf_matches_reference_fixture(oracle_lib):
    for m, ng, ns, wo, wi, seeds, out, out2 in fixtures.load_bsdf():
        a, b = oracle_lib.bsdf_probe("oracle", m, ng, ns, wo, wi, seeds)
        assert np.array_equal(bits(a), bits(out))
        assert np.array_equal(bits(b), bits(out2))


@pytest.mark.parametrize("adaptive", [0, 1])
def test_oracle_matches_reference_procedural(ref_oracle, adaptive):
    from photon_gb300 import workloads
    oracle_lib = ref_oracle
    sc, cam, st = workloads.procedural_500k()
    st.width = st.height = 40
    st.pixel_samples = 18 if adaptive else 2
    st.adaptive_sampling = adaptive
    out = {}
    for which in ("ref", "oracle"):
        r = oracle_lib.CpuRenderer(which)
        r.set_scene(sc)
        r.render(cam, st, True)
        r.render(cam, st, False)  # progressive accumulation across calls
        out[which] = {ch: r.read(ch) for ch in ("color", "depth", "normal", "albedo")}
        out[which]["n"] = r.accumulated_samples()
    assert out["ref"]["n"] == out["oracle"]["n"] == 2 * st.pixel_samples
    for ch in ("color", "depth", "normal", "albedo"):
        assert np.array_equal(bits(out["ref"][ch]), bits(out["oracle"][ch])), ch


def test_oracle_errors_match_reference(ref_oracle):
    from photon_gb300 import workloads
    oracle_lib = ref_oracle
    sc, cam, st = workloads.box_room()
    for which in ("ref", "oracle"):
        r = oracle_lib.CpuRenderer(which)
        with pytest.raises(RuntimeError, match="no scene"):
            r.render(cam, st, True)
        r.set_scene(sc)
        st0 = workloads.settings(0, 4, 1, 1)
        with pytest.raises(RuntimeError, match="invalid frame size"):
            r.render(cam, st0, True)
