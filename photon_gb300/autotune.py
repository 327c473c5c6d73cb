"""Autotuner of the renderer's launch parameters (the phc_tuning_* keys).

Coordinate descent on one workload: each key in turn takes every candidate
value of SPACE with the other keys fixed, and keeps the value with the lowest
median device time of a render call (phc_render's render_ms, after a warm-up
call).  Passes repeat until a pass changes nothing or `passes` is reached.
"max_leaf", "gpu_bvh", "gpu_max_leaf", "ploc_radius" and "collapse_tri_cost"
change the BVH8 and are applied by re-uploading the scene.

The reference has no tunables on this path; the keys are this renderer's:
queue capacity (wave_paths), persistent grid sizes of the traversal and
shading kernels, the traversal refill threshold, the shading-kernel split and
lean variants, the material-sort threshold and the BVH8 leaf size.

    from photon_gb300 import autotune, workloads
    sc, cam, st = workloads.procedural_500k()
    result = autotune.autotune(sc, cam, st, apply=True)
"""
from __future__ import annotations

import statistics

from .renderer import Renderer, tuning_get, tuning_set

SPACE = {
    "trace_blocks_per_sm": [4, 8, 12, 16, 24, 32],
    "shade_blocks_per_sm": [2, 4, 6, 8, 12, 16],
    "trace_refill": [1, 4, 8, 12, 16, 32],
    "wave_paths": [1 << 20, 1 << 22, 1 << 24, 1 << 25, 1 << 26, 1 << 27],
    "split_shade": [0, 1],
    "shade_lean": [0, 1],
    "sort_threshold": [0, 1 << 12, 1 << 14, 1 << 16, 1 << 18, 1 << 20],
    "max_leaf": [1, 2, 3],
    "gpu_bvh": [0, 1],
    "gpu_max_leaf": [1, 2, 3],
    "ploc_radius": [2, 4, 8, 16, 32],
    "collapse_tri_cost": [0, 20, 30, 50],
}
SCENE_KEYS = {"max_leaf", "gpu_bvh", "gpu_max_leaf", "ploc_radius", "collapse_tri_cost"}  # read at scene upload


class RenderTimer:
    """Median device time (ms) of `reps` render calls of one workload under
    the current tuning, after `warmup` untimed calls."""

    def __init__(self, scene, camera, settings, reps=3, warmup=1):
        self.scene, self.camera, self.settings = scene, camera, settings
        self.reps, self.warmup = reps, warmup
        self.r = Renderer()
        self.r.set_scene(scene)

    def upload(self):
        self.r.set_scene(self.scene)

    def __call__(self) -> float:
        for _ in range(self.warmup):
            self.r.render(self.camera, self.settings, True)
        times = []
        for _ in range(self.reps):
            self.r.render(self.camera, self.settings, True)
            times.append(self.r.stats()["render_ms"])
        return statistics.median(times)

    def close(self):
        self.r.close()


def search(measure, keys=None, space=None, passes=2, on_scene_change=None, log=None):
    """Coordinate descent.  measure() -> time of the current tuning (lower is
    better); on_scene_change() is called after a SCENE_KEYS value is set.
    Returns (best settings of the searched keys, best time, baseline time,
    trials [(key, value, time)]).  Leaves the tuning at the best settings."""
    space = dict(space or SPACE)
    keys = list(keys or space.keys())
    best = {k: tuning_get(k) for k in keys}
    base_ms = measure()
    best_ms = base_ms
    trials = []
    for _ in range(passes):
        changed = False
        for k in keys:
            for v in space[k]:
                if v == best[k]:
                    continue
                tuning_set(k, v)
                if k in SCENE_KEYS and on_scene_change:
                    on_scene_change()
                ms = measure()
                trials.append((k, v, ms))
                if log:
                    log(f"{k}={v}: {ms:.3f} ms (best {best_ms:.3f})")
                if ms < best_ms:
                    best_ms, best[k], changed = ms, v, True
            tuning_set(k, best[k])
            if k in SCENE_KEYS and on_scene_change:
                on_scene_change()
        if not changed:
            break
    return best, best_ms, base_ms, trials


def autotune(scene, camera, settings, keys=None, space=None, passes=2, reps=3, apply=False, log=None):
    """Tunes the launch parameters for one workload on the current GPU.
    apply=False restores the previous settings afterwards."""
    keys = list(keys or (space or SPACE).keys())
    saved = {k: tuning_get(k) for k in keys}
    timer = RenderTimer(scene, camera, settings, reps=reps)
    try:
        best, best_ms, base_ms, trials = search(timer, keys, space, passes, on_scene_change=timer.upload, log=log)
    finally:
        timer.close()
        if not apply:
            for k, v in saved.items():
                tuning_set(k, v)
    return {"best": best, "best_ms": best_ms, "baseline_ms": base_ms, "speedup": base_ms / best_ms,
            "trials": trials, "previous": saved}
