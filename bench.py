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
             duration against the measured HBM copy bandwidth, and against
             the read bandwidth of an L2-resident buffer measured in the same
             run (roofline.l2, baseline/l2_probe.cu);
  cpu_baseline  the CPU oracle (a restatement of the reference's algorithm)
             on the host cores, on a bounded sample of the same workload;
  batched_vs_plain, adjoint, instancing, configs  the batched mode against
             one call at a time, the path-replay adjoint against the forward
             pass, the two-level BVH against flattened placements, and the
             box-room and 2M-triangle instanced configurations (each skippable);
  kokkos_port  Level A of this library against the reference's Kokkos BVH
             back-end restated for the GPU (baseline/kokkos_port.cu) on the
             same rays, and the bound it gives on the reference's frame rate.
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
# DRAM bytes per closest-hit ray of k_trace, from one ncu capture
# (dram__bytes_read.sum + dram__bytes_write.sum = 282.24 + 144.83 MB over the
# 8,388,608 camera rays of bounce iteration 0 at 8 spp; the node and triangle
# reads stay in L2, so the traffic is the ray/hit queues and grows with the
# ray count).  The roofline's `traffic` scales it to the average launch.
TRACE_DRAM_BYTES_PER_RAY = (282.24e6 + 144.83e6) / 8388608
# Instruction issue of k_trace from the same capture: warp instructions per
# camera ray (smsp__inst_executed.sum / rays), the fraction of issue slots
# used, and active threads per warp instruction.
TRACE_ISSUE = {"warp_instructions_per_ray": 1.597e9 / 8388608, "issue_active": 0.793,
               "threads_per_warp_instruction": 20.0,
               "source": "ncu --set full capture of k_trace, bounce iteration 0 of the 500K workload at 8 spp "
                         "(profiles/k_trace_procedural_500k.md)"}
# Shading: algorithmic bytes per shaded hit path: queue and sorted index 8,
# path state 68 (origin+tmin, direction+tmax, throughput+pdf, info, distance),
# hit 16, triangle indices+material 16, three vertex normals 48, triangle
# record 48, material parameters 64, continued path 68, shadow record 48.
SHADE_BYTES_PER_PATH = 8 + 68 + 16 + 16 + 48 + 48 + 64 + 68 + 48
# DRAM bytes per shaded path of the material-sorted hit-shading kernel, from
# one ncu capture (1412.8 + 1897.5 MB over the 8.4M hits of iteration 0 at
# 8 spp, profiles/k_shade_procedural_500k.md).
SHADE_DRAM_BYTES_PER_PATH = (1412.8e6 + 1897.5e6) / 8388608
# Volume tracking: one density lookup reads the 8 grid values of its
# trilinear cell and the 2 transfer-function entries it interpolates.
VOL_LOOKUP_BYTES = 8 * 4 + 2 * 16


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


def scene_configs(p, reps=1, only=None, spp=0):
    """The other single-GPU forward configurations, one render each after a
    warm-up, device time: the box room (about 36 triangles, 512^2, 64 spp,
    depth 8) and the 2M-triangle instanced scene (12 RGBA8 2048^2 noise
    textures, 256^3 fBm volume, 1920^2, 256 spp, depth 12, adaptive
    sampling, so Msamples/s counts the pixel samples actually traced)."""
    from photon_gb300 import workloads
    out = {}
    for name, make in (("box_room_512", workloads.box_room), ("instanced_2m_1920", workloads.instanced_2m)):
        if only and name != only:
            continue
        sc, cam, st = make()
        if spp:
            st.pixel_samples = spp
        _log(f"configs: {name} generated")
        r = p.Renderer()
        t = time.perf_counter()
        r.set_scene(sc)
        upload = time.perf_counter() - t
        r.render(cam, st, True)
        ms, samples = [], []
        for _ in range(reps):
            r.render(cam, st, True)
            s = r.stats()
            ms.append(s["render_ms"])
            samples.append(s["pixel_samples"])
        m = sorted(ms)[len(ms) // 2]
        k = ms.index(m)
        p.tuning_set("time_kernels", 1)  # per-kind device time of one more render
        r.render(cam, st, True)
        kinds = dict(zip(p._abi.KERNEL_KIND_NAMES, r.stats()["kernel_ms"]))
        p.tuning_set("time_kernels", 0)
        out[name] = {"triangles": int(sc.triangle_count), "res": [st.width, st.height],
                     "spp": st.pixel_samples, "depth": st.max_depth, "adaptive": int(st.adaptive_sampling),
                     "render_ms": m, "pixel_samples": int(samples[k]),
                     "msamples_per_s": samples[k] / (m / 1e3) / 1e6, "upload_s": upload,
                     "kernel_ms": kinds}
        if sc.volumes:
            # the tracking kernels' algorithmic bytes: per density lookup the
            # 8 grid values of its trilinear cell and the 2 transfer-function
            # entries it interpolates (the lookups counted on the device)
            p.tuning_set("count_traversal", 1)
            r.render(cam, st, True)
            lookups = r.stats()["volume_lookups"]
            p.tuning_set("count_traversal", 0)
            vol_ms = kinds["volume_scatter"] + kinds["shadow_transmittance"]
            peak, peak_kind = peaks()
            gbs = lookups * VOL_LOOKUP_BYTES / (vol_ms / 1e3) / 1e9 if vol_ms > 0 else 0.0
            out[name]["roofline"] = {
                "kernel": "k_vol_scatter + k_shadow_volume (delta / ratio tracking)", "bound": "latency",
                "density_lookups": int(lookups), "lookups_per_pixel_sample": lookups / max(1, samples[k]),
                "bytes_per_lookup": VOL_LOOKUP_BYTES, "ms_per_frame": vol_ms, "achieved": gbs, "peak": peak,
                "unit": "GB/s", "frac": gbs / peak, "peak_source": f"{peak_kind} hbm_gbs"}
        r.close()
        del sc
    return out


def workload_rays(sc, cam, width, height, seed=1):
    """Three ray batches of the workload, built with this library's Level A:
    camera rays (one jittered ray per pixel), diffuse bounce rays (cosine
    directions about the geometric normal at the camera rays' hits) and
    shadow rays from the same hits (half toward the sun, half over the upper
    hemisphere, unbounded).  Device tensors (o, d, tmin, tmax) per batch."""
    import numpy as np
    import torch
    import photon_gb300 as p
    rng = np.random.default_rng(seed)
    fwd = np.asarray(cam.direction[:], np.float32)
    up = np.asarray(cam.up[:], np.float32)
    right = np.cross(fwd, up)
    right /= np.linalg.norm(right)
    tup = np.cross(right, fwd)
    th = np.tan(0.5 * cam.fovy)
    aspect = cam.aspect if cam.aspect > 0 else width / height
    py, px = np.mgrid[0:height, 0:width].astype(np.float32)
    sx = (2.0 * (px + rng.random(px.shape, np.float32)) / width - 1.0) * th * aspect
    sy = (2.0 * (py + rng.random(py.shape, np.float32)) / height - 1.0) * th
    d = fwd[None] + sx.reshape(-1, 1) * right[None] + sy.reshape(-1, 1) * tup[None]
    d /= np.linalg.norm(d, axis=1, keepdims=True)
    n = d.shape[0]
    o = np.broadcast_to(np.asarray(cam.position[:], np.float32), (n, 3)).copy()
    dev = lambda a: torch.from_numpy(np.ascontiguousarray(a, np.float32)).cuda()
    cam_b = (dev(o), dev(d), dev(np.zeros(n)), dev(np.full(n, 1e30)))
    acc = p.Accel(sc.positions, sc.indices, sc.normals, sc.material_ids)
    rec = np.frombuffer(acc.trace_closest(*cam_b).cpu().numpy().tobytes(), p._abi.hit_dtype())
    acc.close()
    h = rec["hit"].astype(bool)
    pos, ng = rec["position"][h], rec["normal"][h]
    ng = np.where((np.sum(ng * d[h], 1) > 0)[:, None], -ng, ng)
    m = len(pos)
    # cosine-weighted directions about ng
    u1, u2 = rng.random(m, np.float32), rng.random(m, np.float32)
    r, phi = np.sqrt(u1), 2.0 * np.pi * u2
    a = np.where(np.abs(ng[:, :1]) > 0.9, np.array([[0, 1, 0]], np.float32), np.array([[1, 0, 0]], np.float32))
    t1 = np.cross(ng, a)
    t1 /= np.linalg.norm(t1, axis=1, keepdims=True)
    t2 = np.cross(ng, t1)
    bd = (r * np.cos(phi))[:, None] * t1 + (r * np.sin(phi))[:, None] * t2 + np.sqrt(1 - u1)[:, None] * ng
    bd /= np.linalg.norm(bd, axis=1, keepdims=True)
    eps = 1e-4 * float(np.abs(sc.positions).max())
    bo = pos + eps * ng
    bounce_b = (dev(bo), dev(bd), dev(np.zeros(m)), dev(np.full(m, 1e30)))
    sun = np.asarray((0.35, 0.55, -0.75), np.float32)
    sun /= np.linalg.norm(sun)
    sd = rng.normal(size=(m, 3)).astype(np.float32)
    sd[:, 1] = np.abs(sd[:, 1])
    sd /= np.linalg.norm(sd, axis=1, keepdims=True)
    sd[::2] = sun
    shadow_b = (dev(bo), dev(sd), dev(np.zeros(m)), dev(np.full(m, 1e30)))
    return {"camera": cam_b, "bounce": bounce_b, "shadow": shadow_b}


def kokkos_port_vs_ours(p, sc, cam, st, frame, reps=3):
    """Level A of both back-ends on the same GPU and rays: this library's
    BVH8 (phc_trace_closest / phc_trace_occluded, 88-byte HitResult records)
    against the reference's Kokkos BVH back-end restated for the GPU
    (baseline/kokkos_port.cu: binary median-split BVH, one thread per ray,
    64-entry local stack).  Both calls are synchronous; wall time around
    each call, median of `reps` after a warm-up.  Also a bound on the whole
    frame: the reference's render needs at least its own traversal time for
    this frame's closest and shadow rays (at the port's rates) plus this
    library's time for everything else (camera rays, shading, bookkeeping),
    so frame samples over that time bounds its Msamples/s from above; and a
    second bound that adds the fixed cost of the reference's bounce loop (one
    wavefront per sample of every pixel, launches, fences and the host
    read-back of the active count every iteration), measured from C++ on the
    same GPU and host (baseline.loop_overhead_s)."""
    import numpy as np
    import torch
    import baseline
    batches = workload_rays(sc, cam, st.width, st.height)
    _log("kokkos port: ray batches built")
    ours = p.Accel(sc.positions, sc.indices, sc.normals, sc.material_ids)
    t = time.perf_counter()
    port = baseline.KokkosPortAccel(sc.positions, sc.indices, sc.normals, sc.material_ids)
    port_build_s = time.perf_counter() - t
    stream = torch.cuda.current_stream().cuda_stream

    def timed(fn):
        fn()
        torch.cuda.synchronize()
        ts = []
        for _ in range(reps):
            torch.cuda.synchronize()
            t0 = time.perf_counter()
            fn()
            torch.cuda.synchronize()
            ts.append(time.perf_counter() - t0)
        return sorted(ts)[len(ts) // 2]

    out = {"port_bvh": {**port.info(), "build_s": port_build_s}}
    for name, (o, d, t0, t1) in batches.items():
        n = int(t0.numel())
        any_hit = name == "shadow"
        if any_hit:
            a = torch.empty(n, dtype=torch.int32, device="cuda")
            b = torch.empty(n, dtype=torch.int32, device="cuda")
            t_ours = timed(lambda: ours.trace_occluded(o, d, t0, t1, a))
            t_port = timed(lambda: port.trace(o, d, t0, t1, b, any_hit=True, stream=stream))
            agree = float(np.mean((a.cpu().numpy() != 0) == (b.cpu().numpy() != 0)))
        else:
            a = torch.empty((n, 88), dtype=torch.uint8, device="cuda")
            b = torch.zeros((n, 88), dtype=torch.uint8, device="cuda")
            t_ours = timed(lambda: ours.trace_closest(o, d, t0, t1, a))
            t_port = timed(lambda: port.trace(o, d, t0, t1, b, stream=stream))
            ra = np.frombuffer(a.cpu().numpy().tobytes(), p._abi.hit_dtype())
            rb = np.frombuffer(b.cpu().numpy().tobytes(), p._abi.hit_dtype())
            same_hit = ra["hit"] == rb["hit"]
            both = (ra["hit"] != 0) & (rb["hit"] != 0)
            agree = float((same_hit & (~both | (ra["prim_id"] == rb["prim_id"]))).mean())
        out[name] = {"rays": n, "ours_mrays_per_s": n / t_ours / 1e6, "port_mrays_per_s": n / t_port / 1e6,
                     "ours_ms": t_ours * 1e3, "port_ms": t_port * 1e3, "speedup": t_port / t_ours,
                     "agreement": agree}
        _log(f"kokkos port: {name} timed")
    ours.close()
    port.close()
    # the frame bound
    prim = frame["pixel_samples"]
    sec = max(0, frame["closest_rays"] - prim)
    t_trav = (prim / (out["camera"]["port_mrays_per_s"] * 1e6) + sec / (out["bounce"]["port_mrays_per_s"] * 1e6)
              + frame["shadow_rays"] / (out["shadow"]["port_mrays_per_s"] * 1e6))
    t_rest = (frame["render_ms"] - frame["kernel_ms"]["trace_closest"] - frame["kernel_ms"]["trace_shadow"]) / 1e3
    ref_bound = prim / (t_trav + t_rest) / 1e6
    # the reference renders one sample of every pixel per wavefront and pays
    # the fixed cost of its bounce loop per iteration of every sample
    iters = int(frame["iterations"])
    t_iter = baseline.loop_overhead_s()
    t_loop = st.pixel_samples * iters * t_iter
    out["frame_bound"] = {"reference_traversal_s": t_trav, "other_work_s": t_rest,
                          "reference_msamples_per_s_at_most": ref_bound,
                          "closest_rays": int(frame["closest_rays"]), "shadow_rays": int(frame["shadow_rays"]),
                          "pixel_samples": int(prim),
                          "with_bounce_loop": {
                              "iteration_overhead_us": t_iter * 1e6, "iterations_per_sample": iters,
                              "samples_per_pixel": int(st.pixel_samples), "loop_s": t_loop,
                              "reference_msamples_per_s_at_most": prim / (t_trav + t_rest + t_loop) / 1e6}}
    return out


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


def cpu_baseline_configs():
    """The CPU oracle on the other forward configurations, all host threads:
    the box room at its full 64 spp (512^2, depth 8), the differentiable
    workload's forward pass at its full 64 spp (256^2, depth 6, homogeneous
    medium), and the 2M-triangle volume scene at 1 spp of its 1920^2 frame
    (adaptive sampling off for the sample: its gate opens after 16 samples),
    Msamples/s per configuration."""
    import oracle
    from photon_gb300 import workloads
    oracle.build()
    out = {}
    for name, make, spp in (("box_room_512", workloads.box_room, None),
                            ("differentiable_256", workloads.differentiable, None),
                            ("instanced_2m_1920", workloads.instanced_2m, 1)):
        sc, cam, st = make()
        s = type(st).from_buffer_copy(bytes(st))
        if spp:
            s.pixel_samples = spp
            s.adaptive_sampling = 0
        r = oracle.CpuRenderer("oracle")
        r.set_scene(sc)
        t = time.perf_counter()
        r.render(cam, s, True)
        dt = time.perf_counter() - t
        samples = s.width * s.height * s.pixel_samples
        out[name] = {"msamples_per_s": samples / dt / 1e6, "pixel_samples": int(samples), "seconds": dt,
                     "spp": int(s.pixel_samples), "full_spp": spp is None}
        r.close()
        _log(f"cpu baseline: {name} done")
    return out


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

    dev = {"plain": 0.0, "batched": 0.0}

    def plain(rs, js):
        dev["plain"] = 0.0
        for r, (sc, cam, st) in zip(rs, js):
            r.render(cam, st, True)
            dev["plain"] += r.stats()["render_ms"] / 1e3

    def batch(rs, js):
        dev["batched"] = p.render_batch([(r, cam, st, True) for r, (sc, cam, st) in zip(rs, js)])["render_ms"] / 1e3

    out = {"jobs": n_jobs, "pixel_samples": samples,
           "mix": f"{n_jobs} seeded procedural scenes, {min(tris)}-{max(tris)} tris (log-uniform), "
                  "128^2-1024^2, 4-64 spp, depth 4-12"}
    _log("batched: jobs generated")
    try:
        t = time.perf_counter()
        rs = make(jobs)
        torch.cuda.synchronize()
        out["upload_s"] = time.perf_counter() - t  # 64 phc_set_scene calls: host tables, GPU BVH8 build
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
            # device time inside the calls (events around each call's GPU
            # work) against wall time: what is left between the plain calls
            # is GPU idle time that batching can remove; the rest it can only
            # shorten by doing the same paths faster
            res["plain_device_s"] = dev["plain"]
            res["plain_idle_frac"] = max(0.0, 1.0 - dev["plain"] / res["plain_s"])
            res["batched_device_s"] = dev["batched"]
            res["ratio_bound_from_idle"] = res["plain_s"] / dev["plain"] if dev["plain"] > 0 else None
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
    # the headline ratio is against the plain path as shipped (sample lanes);
    # the one-sample-per-wave ratio is the reference's loop structure
    out["ratio"] = out["lanes"]["ratio"]
    out["ratio_vs_one_sample_per_wave"] = out["one_sample_per_wave"]["ratio"]
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
    kinds = list(p._abi.KERNEL_KIND_NAMES)
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
        "dominant_kernel_by_time": dom,
        # what limits it (ncu): instruction issue over an L2-resident BVH and
        # triangle set; `frac` is the metric's figure, algorithmic node /
        # triangle / ray bytes against the measured HBM copy bandwidth
        "bound": "issue", "memory_level": "l2",
        "achieved": achieved, "peak": peak, "unit": "GB/s",
        "frac": achieved / peak, "peak_source": f"{peak_kind} hbm_gbs",
        "issue": TRACE_ISSUE,
        "traffic": (TRACE_DRAM_BYTES_PER_RAY * prof["closest_rays"] / max(1, kcount["trace_closest"])
                    if dom != "trace_shadow" else None),
        "traffic_source": f"ncu capture of k_trace (profiles/k_trace_procedural_500k.md): "
                          f"{TRACE_DRAM_BYTES_PER_RAY:.1f} DRAM bytes per ray, times the rays of the average "
                          "launch of this frame",
        "algorithmic_bytes_per_launch": bytes_alg / max(1, kcount["trace_closest"]),
        "bytes_per_ray": bytes_alg / max(1, prof["closest_rays"] if dom != "trace_shadow" else prof["shadow_rays"]),
        "nodes_per_ray": prof["node_visits"] / max(1, prof["closest_rays"]),
        "tris_per_ray": prof["tri_tests"] / max(1, prof["closest_rays"]),
        "launches": kcount["trace_closest"], "kernel_ms_total": kms["trace_closest"],
    }
    shade_paths = prof["closest_rays"]
    shade_gbs = shade_paths * SHADE_BYTES_PER_PATH / (kms["shade"] / 1e3) / 1e9 if kms["shade"] > 0 else 0.0
    roofline["shade"] = {
        "kernel": "k_shade (hit and miss shading, material-sorted)", "bound": "latency",
        "ms_per_frame": kms["shade"], "paths": shade_paths,
        "algorithmic_bytes_per_path": SHADE_BYTES_PER_PATH,
        "achieved": shade_gbs, "peak": peak, "unit": "GB/s", "frac": shade_gbs / peak,
        "dram_bytes_per_path": SHADE_DRAM_BYTES_PER_PATH,
        "note": "paths = closest-hit rays of the frame, hits and misses (a miss reads fewer bytes, so the "
                "algorithmic figure is an upper bound); DRAM bytes per path from the ncu capture "
                "(profiles/k_shade_procedural_500k.md)",
    }
    import baseline
    try:
        l2 = baseline.l2_read_gbs()
        roofline["l2"] = {"peak": l2, "frac": achieved / l2, "unit": "GB/s",
                          "peak_source": "one-launch read sweeps of a 32 MiB L2-resident buffer, measured in this run"}
    except Exception as e:  # an optional figure: the line is printed without it
        _log(f"l2 probe failed: {e}")
        roofline["l2"] = None

    _log("e2e and kernel profile done")
    cpu = None
    if rank == 0 and not args.no_cpu_baseline:
        cpu = cpu_baseline(sc, cam, st)
        _log("cpu baseline done")
        if not args.no_configs:
            try:
                cpu["configs"] = cpu_baseline_configs()
            except Exception as e:  # optional: the line is printed without it
                _log(f"cpu baseline of the other configurations failed: {e}")
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
    kokkos = None
    if rank == 0 and not args.no_kokkos_port:
        frame = {"pixel_samples": samples / args.steps, "closest_rays": closest / args.steps,
                 "shadow_rays": shadow / args.steps, "render_ms": dev_ms / args.steps, "kernel_ms": kms,
                 "iterations": kcount["trace_closest"] // max(1, kcount["raygen"])}  # per wave
        try:
            kokkos = kokkos_port_vs_ours(p, sc, cam, st, frame)
            fb = kokkos["frame_bound"]
            fb["ours_msamples_per_s"] = value
            fb["speedup_at_least"] = value / fb["reference_msamples_per_s_at_most"]
            fb["with_bounce_loop"]["speedup_at_least"] = (
                value / fb["with_bounce_loop"]["reference_msamples_per_s_at_most"])
            _log("kokkos port comparison done")
        except Exception as e:  # an optional comparison: the line is printed without it
            _log(f"kokkos port comparison failed: {e}")
            kokkos = {"error": str(e)}
    configs = None
    if rank == 0 and not args.no_configs:
        try:
            configs = scene_configs(p)
            _log("other configurations done")
        except Exception as e:  # optional: the line is printed without it
            _log(f"other configurations failed: {e}")
            configs = {"error": str(e)}

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
            "configs": configs,
            "kokkos_port": kokkos,
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
    ap.add_argument("--no-kokkos-port", action="store_true",
                    help="skip the Level-A comparison with the reference's Kokkos BVH back-end restated for the GPU")
    ap.add_argument("--no-configs", action="store_true",
                    help="skip the box-room and 2M-triangle instanced configurations")
    ap.add_argument("--config-only", default="", choices=["", "box_room_512", "instanced_2m_1920"],
                    help="render only this configuration (one warm-up and one timed render) and print its record "
                         "(profiling a small case; not a bench line)")
    ap.add_argument("--config-spp", type=int, default=0, help="samples per pixel of --config-only")
    ap.add_argument("--adjoint-only", action="store_true",
                    help="run only the adjoint/forward measurement and print its record (profiling; not a bench line)")
    args = ap.parse_args()
    if args.adjoint_only:
        import torch
        torch.cuda.set_device(0)
        from photon_gb300 import build as pbuild
        pbuild.build()
        import photon_gb300 as p
        print(json.dumps(adjoint_vs_forward(p)), flush=True)
        return
    if args.config_only:
        import torch
        torch.cuda.set_device(0)
        from photon_gb300 import build as pbuild
        pbuild.build()
        import photon_gb300 as p
        print(json.dumps(scene_configs(p, only=args.config_only, spp=args.config_spp)), flush=True)
        return
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
