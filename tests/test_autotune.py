"""The autotuner's search on the CPU (a synthetic cost in place of render
times) and, on a GPU, one short tuning run."""
import pytest


def test_search_finds_the_minimum_and_leaves_best_settings(photon):
    from photon_gb300 import autotune
    from photon_gb300.renderer import tuning_get, tuning_set
    space = {"trace_blocks_per_sm": [4, 8, 16, 32], "trace_refill": [1, 8, 32], "sort_threshold": [0, 1 << 16]}
    saved = {k: tuning_get(k) for k in space}
    target = {"trace_blocks_per_sm": 16, "trace_refill": 1, "sort_threshold": 1 << 16}
    calls = []

    def cost():
        calls.append(1)
        return 1.0 + sum(abs(tuning_get(k) - v) / max(v, 1) for k, v in target.items())

    try:
        best, best_ms, base_ms, trials = autotune.search(cost, space=space, passes=3)
        assert best == target
        assert best_ms == pytest.approx(1.0)
        assert all(tuning_get(k) == v for k, v in target.items())
        assert len(trials) == len(calls) - 1
    finally:
        for k, v in saved.items():
            tuning_set(k, v)


def test_scene_keys_trigger_reupload(photon):
    from photon_gb300 import autotune
    from photon_gb300.renderer import tuning_get, tuning_set
    saved = tuning_get("max_leaf")
    uploads = []
    try:
        autotune.search(lambda: float(tuning_get("max_leaf")), keys=["max_leaf"], space={"max_leaf": [1, 2, 3]},
                        passes=1, on_scene_change=lambda: uploads.append(tuning_get("max_leaf")))
        assert tuning_get("max_leaf") == 1
        assert uploads[-1] == 1 and len(uploads) >= 2
    finally:
        tuning_set("max_leaf", saved)


@pytest.mark.gpu
def test_autotune_short_run(photon):
    from photon_gb300 import autotune, workloads
    from photon_gb300.renderer import tuning_get
    sc, cam, st = workloads.box_room()
    st.width = st.height = 128
    st.pixel_samples = 4
    before = {k: tuning_get(k) for k in ("trace_refill", "shade_blocks_per_sm")}
    res = autotune.autotune(sc, cam, st, keys=["trace_refill", "shade_blocks_per_sm"], passes=1, reps=2)
    assert res["best_ms"] <= res["baseline_ms"]
    assert {k: tuning_get(k) for k in before} == before  # apply=False restores
    assert len(res["trials"]) >= 5
