"""Benchmark of the GB300 path tracer on the 500K-triangle workload.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]

One step is one render call of the full workload: 498,726 triangles, 1024x1024
pixels, 128 samples per pixel, max depth 8 (the reference's 1024^2 / depth-8
metric), with a procedural 1024x512 fp32 sun+sky environment and 4 emissive
triangles (seeded synthetic scene: the reference's published scenes are not
available offline).

Our arm prints one JSON line with
  value      Msamples/s over the K timed steps, device time (CUDA events on the
             renderer's stream), scene resident, L2 flushed before every step;
  e2e        the same metric through the public API with host buffers: every
             step renders from host-side camera/settings and reads the colour
             channel back into pinned host memory;
  roofline   the dominant kernel's algorithmic bytes / its event-timed
             duration against the measured HBM copy bandwidth;
  cpu_baseline  the CPU oracle (a restatement of the reference's algorithm)
             on the host cores, on a bounded sample of the same workload;
  batched_vs_plain, adjoint, instancing  the batched mode against one call
             at a time, the path-replay adjoint against the forward pass, and
             the two-level BVH against flattened placements (each skippable).
--impl reference times that CPU implementation as the main line.
Under torchrun (N > 1) every rank renders its own replica (the path is
replicated, not sharded) and rank 0 prints the line.
"""
from __future__ import annotations

import argparse
import json
import os
import subprocess
import sys
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "Msamples/s @1024² d8 vs ref & plain; batched/plain ratio; adjoint/fwd time"
NODE_BYTES = 80   # one BVH8 node
TRI_BYTES = 48    # one triangle record (v0, e1, e2 as float4)
RAY_BYTES = 32    # origin+tmin, direction+tmax
HIT_BYTES = 16    # t, prim, u, v


_T0 = time.perf_counter()


def _log(msg):
    """Progress on stderr (the JSON line alone goes to stdout)."""
    print(f"[bench {time.perf_counter() - _T0:7.1f}s] {msg}", file=sys.stderr, flush=True)


def peaks():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        with open(p) as f:
            d = json.load(f)
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


class ClockSampler:
    """nvidia-smi clock / throttle samples during the timed region."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index):
        self.gpu = gpu_index
        self.proc = None

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--id={self.gpu}", f"--query-gpu={self.FIELDS}", "--format=csv,noheader,nounits",
                 "-lms", "200"], stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
        except Exception:
            self.proc = None
        return self

    def __exit__(self, *exc):
        self.lines = []
        if self.proc:
            self.proc.terminate()
            try:
                out, _ = self.proc.communicate(timeout=5)
            except Exception:
                self.proc.kill()
                out = ""
            self.lines = [l for l in out.splitlines() if l.strip()]

    def summary(self):
        sm, mx, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for l in getattr(self, "lines", []):
            p = [x.strip() for x in l.split(",")]
            if len(p) < 9:
                continue
            try:
                sm.append(float(p[1]))
                mx = float(p[2])
            except ValueError:
                continue
            for n, v in zip(names, p[5:9]):
                if v.lower() == "active":
                    reasons.add(n)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": mx, "reasons": [], "samples": 0}
        sm.sort()
        return {"sm_mhz": sm[len(sm) // 2], "sm_max_mhz": mx, "reasons": sorted(reasons), "samples": len(sm)}


def dist_setup(n_gpus):
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl" if n_gpus > 0 else "gloo")
    return world, rank, local


def _reduce(x, world, op):
    if world == 1:
        return x
    import torch
    import torch.distributed as dist
    dev = "cuda" if dist.get_backend() == "nccl" else "cpu"
    t = torch.tensor([float(x)], dtype=torch.float64, device=dev)
    dist.all_reduce(t, op=op)
    return float(t.item())


def dist_max(x, world):
    """Largest value over the ranks (the slowest replica's time)."""
    import torch.distributed as dist
    return _reduce(x, world, dist.ReduceOp.MAX) if world > 1 else x


def dist_sum(x, world):
    """Sum over the ranks (all replicas' samples)."""
    import torch.distributed as dist
    return _reduce(x, world, dist.ReduceOp.SUM) if world > 1 else x


def barrier(world):
    if world > 1:
        import torch.distributed as dist
        dist.barrier()


def workload():
    from photon_gb300 import workloads
    sc, cam, st = workloads.procedural_500k()
    desc = (f"procedural_500k: {sc.triangle_count} tris (60 displaced icospheres + 140 tori on a ground plane), "
            f"{st.width}x{st.height}, {st.pixel_samples} spp, max depth {st.max_depth}, "
            "1024x512 fp32 sun+sky env + 4 emissive tris, Disney materials per object")
    return sc, cam, st, desc


def cpu_baseline(sc, cam, st, spp=1, frames=2):
    """The CPU oracle on a bounded sample: `frames` full-resolution frames of
    `spp` samples, all host threads."""
    import oracle
    oracle.build()
    r = oracle.CpuRenderer("oracle")
    r.set_scene(sc)
    import ctypes as C
    s = type(st).from_buffer_copy(bytes(st))
    s.pixel_samples = spp
    t = time.perf_counter()
    for f in range(frames):
        r.render(cam, s, True)
    dt = time.perf_counter() - t
    samples = s.width * s.height * spp * frames
    return {"value": samples / dt / 1e6, "unit": "Msamples/s", "cores": os.cpu_count(), "kind": "port",
            "sample": f"{frames} frames of {s.width}x{s.height} at {spp} spp of the same workload "
                      f"({samples} pixel-samples, {dt:.1f} s)"}


def batched_vs_plain(p, n_jobs=64, seed=0, check_jobs=8):
    """The 64-job mix: the same render calls one at a time (phc_render per
    renderer) and as one batch (phc_render_batch), wall-clock, scenes
    resident, after one warm-up of each.  Measured twice: with one sample of
    every pixel per wavefront (the reference's plain structure,
    pathtracer.cpp:688-1127; wave_paths = 1) and with the renderer's default
    sample lanes.  Image identity is checked on `check_jobs` jobs rendered by
    two fresh renderer sets with the same call history (the bridge's sample
    counter advances per call)."""
    import numpy as np
    import torch
    from photon_gb300 import workloads
    jobs = workloads.batched_jobs(seed=seed, n=n_jobs)
    samples = sum(st.width * st.height * st.pixel_samples for _, _, st in jobs)
    tris = [sc.triangle_count for sc, _, _ in jobs]
    old = p.tuning_get("wave_paths")

    def make(js):
        rs = []
        for sc, cam, st in js:
            r = p.Renderer()
            r.set_scene(sc)
            rs.append(r)
        return rs

    def plain(rs, js):
        for r, (sc, cam, st) in zip(rs, js):
            r.render(cam, st, True)

    def batch(rs, js):
        p.render_batch([(r, cam, st, True) for r, (sc, cam, st) in zip(rs, js)])

    out = {"jobs": n_jobs, "pixel_samples": samples,
           "mix": f"{n_jobs} seeded procedural scenes, {min(tris)}-{max(tris)} tris (log-uniform), "
                  "128^2-1024^2, 4-64 spp, depth 4-12"}
    _log("batched: jobs generated")
    try:
        rs = make(jobs)
        _log("batched: scenes uploaded")
        for label, wave_paths in (("one_sample_per_wave", 1024), ("lanes", old)):
            p.tuning_set("wave_paths", wave_paths)
            res = {}
            for name, fn in (("plain", plain), ("batched", batch)):
                fn(rs, jobs)
                torch.cuda.synchronize()
                t = time.perf_counter()
                fn(rs, jobs)
                res[name + "_s"] = time.perf_counter() - t
            res["plain_msamples_per_s"] = samples / res["plain_s"] / 1e6
            res["batched_msamples_per_s"] = samples / res["batched_s"] / 1e6
            res["ratio"] = res["plain_s"] / res["batched_s"]
            _log(f"batched: {label} timed")
            a, b = make(jobs[:check_jobs]), make(jobs[:check_jobs])
            for _ in range(2):
                plain(a, jobs[:check_jobs])
                batch(b, jobs[:check_jobs])
            res["identical_images"] = bool(all(
                np.array_equal(x.read("color").view(np.uint32), y.read("color").view(np.uint32))
                for x, y in zip(a, b)))
            for r in a + b:
                r.close()
            out[label] = res
        for r in rs:
            r.close()
    finally:
        p.tuning_set("wave_paths", old)
    out["ratio"] = out["one_sample_per_wave"]["ratio"]
    out["identical_images"] = out["one_sample_per_wave"]["identical_images"] and out["lanes"]["identical_images"]
    return out


def adjoint_vs_forward(p, reps=3):
    """Differentiable workload (50K triangles, 8 materials with 512^2 fp32
    base-colour textures, homogeneous medium, 256^2, depth 6): device time
    of the 64-spp forward render and of the 16-spp path-replay adjoint with
    material, texel and medium gradients, on an L2 loss against a 1024-spp
    image of perturbed parameters.  Reports both times, their ratio (the
    workload's own numbers) and the ratio per sample."""
    import numpy as np

    from photon_gb300 import workloads
    sc_t, cam, st_t = workloads.differentiable(target=True)
    st_t.pixel_samples = 1024
    rt = p.Renderer()
    rt.set_scene(sc_t)
    rt.render(cam, st_t, True)
    target = rt.read_color()[..., :3].copy()
    rt.close()
    sc, cam, st = workloads.differentiable()
    r = p.Renderer()
    r.set_scene(sc)
    fwd, adj, adj_wall = [], [], []
    for k in range(reps + 1):
        r.render(cam, st, True)
        fwd.append(r.stats()["render_ms"])
        img = r.read_color()[..., :3]
        d = np.zeros((st.height, st.width, 4), np.float32)
        d[..., :3] = 2.0 * (img - target)
        sa = type(st).from_buffer_copy(bytes(st))
        sa.pixel_samples = 16
        t = time.perf_counter()
        g = r.adjoint(cam, sa, d, sample_offset=(1 << 28) + 16 * k)
        adj_wall.append((time.perf_counter() - t) * 1e3)
        adj.append(g["adjoint_ms"])
    r.close()
    f = float(np.median(fwd[1:]))
    a = float(np.median(adj[1:]))
    loss = float(np.sum((img - target) ** 2))
    return {"workload": f"differentiable: {sc.triangle_count} tris, 8 materials x 512^2 fp32 base-colour "
                        f"textures, homogeneous medium; {st.width}x{st.height}, depth {st.max_depth}",
            "forward_spp": st.pixel_samples, "adjoint_spp": 16,
            "forward_ms": f, "adjoint_ms": a, "adjoint_wall_ms": float(np.median(adj_wall[1:])),
            "adjoint_over_forward": a / f,
            "adjoint_over_forward_per_sample": (a / 16) / (f / st.pixel_samples),
            "loss": loss, "grad_norm_materials": float(np.linalg.norm(g["materials"])),
            "grad_norm_texels": float(np.linalg.norm(g["texels"])),
            "grad_volume": g["volumes"][0].tolist()}


def instancing_vs_flat(p, reps=3):
    """Instanced geometry (four objects of 12-1280 triangles placed by random
    rotations, non-uniform scales and translations over a lit ground plane,
    1024^2, 16 spp, depth 6): the two-level BVH8 against the same placements
    flattened into world-space triangles (the reference's single-level
    handling), 2,000 placements; and the two-level form at 20,000 placements,
    where flattening would hold 18M triangles.  Device time per render,
    Msamples/s, device memory of the scene and upload time."""
    import torch

    from photon_gb300 import workloads
    out = {}
    for name, n, flat in (("flat_2k", 2000, True), ("instanced_2k", 2000, False), ("instanced_20k", 20000, False)):
        sc, cam, st = workloads.instanced_objects(n_instances=n, res=1024, spp=16, flatten=flat)
        r = p.Renderer()
        torch.cuda.synchronize()
        free0 = torch.cuda.mem_get_info()[0]
        t = time.perf_counter()
        r.set_scene(sc)
        upload = time.perf_counter() - t
        scene_mb = (free0 - torch.cuda.mem_get_info()[0]) / 2 ** 20
        r.render(cam, st, True)
        ms = []
        for _ in range(reps):
            r.render(cam, st, True)
            ms.append(r.stats()["render_ms"])
        m = sorted(ms)[len(ms) // 2]
        placed = sc.triangle_count if flat else sc.triangle_count + sum(
            len(sc.pt.objects[o]["indices"]) for o, _ in sc.pt.instances)
        out[name] = {"placements": n, "placed_triangles": int(placed), "render_ms": m,
                     "msamples_per_s": st.width * st.height * st.pixel_samples / (m / 1e3) / 1e6,
                     "scene_device_mb": scene_mb, "upload_s": upload,
                     "image_mean": float(r.read("color")[..., :3].mean())}
        r.close()
    out["instanced_over_flat_time"] = out["instanced_2k"]["render_ms"] / out["flat_2k"]["render_ms"]
    out["flat_over_instanced_memory"] = out["flat_2k"]["scene_device_mb"] / max(out["instanced_2k"]["scene_device_mb"], 1e-3)
    return out


def run_reference(args, world, rank):
    if rank != 0:
        return
    sc, cam, st, desc = workload()
    import oracle
    oracle.build()
    r = oracle.CpuRenderer("oracle")
    r.set_scene(sc)
    s = type(st).from_buffer_copy(bytes(st))
    s.pixel_samples = 1
    for _ in range(args.warmup):
        r.render(cam, s, True)
    t = time.perf_counter()
    for _ in range(args.steps):
        r.render(cam, s, True)
    dt = time.perf_counter() - t
    samples = s.width * s.height * args.steps
    v = samples / dt / 1e6
    line = {
        "impl": "reference", "metric": METRIC, "value": v, "unit": "Msamples/s", "n_gpus": args.gpus,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": dt / args.steps * 1e3,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
        "data": "synthetic (seeded procedural scene)",
        "config": {"workload": desc, "sample_per_step": f"{s.width}x{s.height} at 1 spp",
                   "parallelism": "host cores (OpenMP)"},
        "cpu_baseline": {"value": v, "unit": "Msamples/s", "cores": os.cpu_count(), "kind": "port",
                         "sample": f"{args.steps} frames of {s.width}x{s.height} at 1 spp"},
        "e2e": {"value": v, "unit": "Msamples/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)


def run_ours(args, world, rank, local):
    import ctypes as C

    import numpy as np
    import torch

    torch.cuda.set_device(local)
    from photon_gb300 import build as pbuild
    pbuild.build()
    import photon_gb300 as p

    _log("build done")
    sc, cam, st, desc = workload()
    _log("workload generated")
    if args.spp:
        st.pixel_samples = args.spp
    r = p.Renderer()
    t = time.perf_counter()
    r.set_scene(sc)
    scene_s = time.perf_counter() - t
    _log(f"scene uploaded ({scene_s:.1f}s)")
    flush = torch.empty(64 * 1024 * 1024, dtype=torch.float32, device="cuda")  # 256 MiB > 129 MB L2

    for _ in range(args.warmup):
        r.render(cam, st, True)

    # ---- device-timed steps (scene resident)
    barrier(world)
    torch.cuda.synchronize()
    dev_ms, samples, launches, closest, shadow = 0.0, 0, 0, 0, 0
    with ClockSampler(local) as clk:
        t_wall = time.perf_counter()
        for _ in range(args.steps):
            flush.zero_()
            torch.cuda.synchronize()
            r.render(cam, st, True)
            s = r.stats()
            dev_ms += s["render_ms"]
            samples += s["pixel_samples"]
            launches += s["kernel_launches"]
            closest += s["closest_rays"]
            shadow += s["shadow_rays"]
        torch.cuda.synchronize()
        wall = time.perf_counter() - t_wall
    barrier(world)
    t_max = dist_max(dev_ms / 1e3, world)
    total_samples = dist_sum(samples, world)
    value = total_samples / t_max / 1e6

    _log("device-timed steps done")
    # ---- end to end through the public API with host buffers
    out = torch.empty((st.height, st.width, 4), dtype=torch.float32).pin_memory()
    out_np = out.numpy()
    barrier(world)
    torch.cuda.synchronize()
    t = time.perf_counter()
    e2e_samples = 0
    for _ in range(args.steps):
        r.render(cam, st, True)
        r.read("color", out_np)
        e2e_samples += r.stats()["pixel_samples"]
    e2e_s = dist_max(time.perf_counter() - t, world)
    e2e_value = dist_sum(e2e_samples, world) / e2e_s / 1e6

    # ---- per-kernel times (events around every launch, one render) and the
    # traversal counters (a second render with counting on: the counts are
    # deterministic, the timing of that render is not used)
    p.tuning_set("time_kernels", 1)
    flush.zero_()
    torch.cuda.synchronize()
    r.render(cam, st, True)
    prof = r.stats()
    p.tuning_set("time_kernels", 0)
    p.tuning_set("count_traversal", 1)
    r.render(cam, st, True)
    cnt = r.stats()
    p.tuning_set("count_traversal", 0)
    for k in ("node_visits", "tri_tests", "shadow_node_visits", "shadow_tri_tests"):
        prof[k] = cnt[k]
    kinds = ["raygen", "trace_closest", "shade", "trace_shadow", "wave_end+resolve"]
    kms = dict(zip(kinds, prof["kernel_ms"]))
    kcount = dict(zip(kinds, prof["kernel_count"]))
    # algorithmic bytes of the traversal kernels
    b_closest = (prof["closest_rays"] * (RAY_BYTES + HIT_BYTES) + prof["node_visits"] * NODE_BYTES
                 + prof["tri_tests"] * TRI_BYTES)
    b_shadow = (prof["shadow_rays"] * (RAY_BYTES + 16) + prof["shadow_node_visits"] * NODE_BYTES
                + prof["shadow_tri_tests"] * TRI_BYTES)
    peak, peak_kind = peaks()
    dom = max(kinds, key=lambda k: kms[k])
    if dom == "trace_shadow":
        bytes_alg, ms = b_shadow, kms["trace_shadow"]
    else:
        dom_t = "trace_closest"
        bytes_alg, ms = b_closest, kms["trace_closest"]
    achieved = bytes_alg / (ms / 1e3) / 1e9 if ms > 0 else 0.0
    roofline = {
        "kernel": "k_trace (BVH8 closest hit)" if dom != "trace_shadow" else "k_shadow (BVH8 any hit)",
        "dominant_kernel_by_time": dom, "bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
        "frac": achieved / peak, "peak_source": f"{peak_kind} hbm_gbs", "traffic": None,
        "bytes_per_ray": bytes_alg / max(1, prof["closest_rays"] if dom != "trace_shadow" else prof["shadow_rays"]),
        "nodes_per_ray": prof["node_visits"] / max(1, prof["closest_rays"]),
        "tris_per_ray": prof["tri_tests"] / max(1, prof["closest_rays"]),
        "launches": kcount["trace_closest"], "kernel_ms_total": kms["trace_closest"],
    }

    _log("e2e and kernel profile done")
    cpu = None
    if rank == 0 and not args.no_cpu_baseline:
        cpu = cpu_baseline(sc, cam, st)
        _log("cpu baseline done")
    batched = None
    if rank == 0 and not args.no_batch:
        r.close()
        batched = batched_vs_plain(p)
        _log("batched/plain done")
    adjoint = None
    if rank == 0 and not args.no_adjoint:
        adjoint = adjoint_vs_forward(p)
        _log("adjoint/forward done")
    instancing = None
    if rank == 0 and not args.no_instancing:
        instancing = instancing_vs_flat(p)
        _log("instancing/flat done")

    if rank == 0:
        h2d = C.sizeof(cam) + C.sizeof(st)
        line = {
            "metric": METRIC, "value": value, "unit": "Msamples/s", "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": t_max * 1e3 / args.steps, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic (seeded procedural scene)",
            "config": {"workload": desc, "l2": "flushed before every step (256 MiB write)",
                       "parallelism": "replicas" if world > 1 else "single GPU",
                       "lanes_paths_per_wave": p.tuning_get("wave_paths")},
            "mrays_per_s": (closest + shadow) / (dev_ms / 1e3) / 1e6,
            "wall_ms_per_step": wall * 1e3 / args.steps,
            "scene_upload_s": scene_s,
            "e2e": {"value": e2e_value, "unit": "Msamples/s", "h2d_bytes_per_step": h2d,
                    "d2h_bytes_per_step": st.width * st.height * 16},
            "roofline": roofline,
            "kernel_ms": kms, "kernel_launches_profiled": kcount,
            "cpu_baseline": cpu,
            "batched_vs_plain": batched,
            "adjoint": adjoint,
            "instancing": instancing,
            "clocks": clk.summary(),
            "gpu_launches": launches,
        }
        print(json.dumps(line), flush=True)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--spp", type=int, default=0, help="override samples per pixel (testing only)")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-batch", action="store_true", help="skip the 64-job batched/plain measurement")
    ap.add_argument("--no-adjoint", action="store_true", help="skip the adjoint/forward measurement")
    ap.add_argument("--no-instancing", action="store_true", help="skip the instanced/flattened measurement")
    args = ap.parse_args()
    world, rank, local = dist_setup(args.gpus if args.impl == "ours" else 0)
    if args.impl == "reference":
        run_reference(args, world, rank)
    else:
        run_ours(args, world, rank, local)
    if world > 1:
        import torch.distributed as dist
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
