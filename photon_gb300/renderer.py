"""Python mirror of photon::bridge::Renderer over the C-ABI.

Method names, argument meaning and error behaviour follow
src/photon/anari/RenderBridge.h:175-214: set_scene / render / read_* raise
PhotonError where the reference returns false with a message, and
accumulated_samples() counts the samples of the accumulated frame.
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import _abi
from .native import PhotonError, load


class Renderer:
    """One GB300 path tracer: scene, BVH8, wavefront buffers, accumulated frame."""

    def __init__(self):
        self.lib = load()
        h = C.c_void_p()
        rc = self.lib.phc_create(C.byref(h))
        if rc != 0:
            raise PhotonError(rc, self.lib.phc_global_error().decode())
        self.h = h
        self.width = self.height = 0
        self._keep = None

    def close(self):
        if getattr(self, "h", None):
            self.lib.phc_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def _check(self, rc):
        if rc != 0:
            raise PhotonError(rc, self.lib.phc_last_error(self.h).decode())

    def backend_name(self) -> str:
        return self.lib.phc_backend_name(self.h).decode()

    def set_scene(self, scene):
        """Uploads a photon_gb300.scene.SceneData (bridge::SceneData)."""
        desc, keep = scene.desc()
        self._check(self.lib.phc_set_scene(self.h, C.addressof(desc)))

    def render(self, camera, settings, reset=True):
        self.width, self.height = settings.width, settings.height
        self._check(self.lib.phc_render(self.h, C.addressof(camera), C.addressof(settings), int(reset)))

    def accumulated_samples(self) -> int:
        return int(self.lib.phc_accumulated_samples(self.h))

    def read(self, channel: str, out: np.ndarray | None = None) -> np.ndarray:
        """channel.color (h, w, 4) / depth (h, w) / normal, albedo (h, w, 3);
        row 0 is the bottom row."""
        n = {"color": 4, "depth": 1, "normal": 3, "albedo": 3}[channel]
        if out is None:
            out = np.empty((self.height, self.width, n), np.float32)
        fn = getattr(self.lib, "phc_read_" + channel)
        self._check(fn(self.h, out.ctypes.data))
        return out[..., 0] if (n == 1 and out.ndim == 3) else out

    def read_color(self):
        return self.read("color")

    def read_depth(self):
        return self.read("depth")

    def read_normal(self):
        return self.read("normal")

    def read_albedo(self):
        return self.read("albedo")

    def adjoint_sizes(self):
        """Element counts of the material, volume and texel gradient buffers."""
        m, v, t = C.c_uint64(), C.c_uint64(), C.c_uint64()
        self._check(self.lib.phc_adjoint_sizes(self.h, C.byref(m), C.byref(v), C.byref(t)))
        return int(m.value), int(v.value), int(t.value)

    def adjoint(self, camera, settings, d_color, sample_offset=0, texels=True, volumes=True, color=False):
        """Path-replay gradients of a loss given dLoss/dImage (h, w, 4) or
        (h, w, 3) float32 (row 0 = bottom row) for the image of
        settings.pixel_samples samples from sample index sample_offset.

        Returns {"materials": (M, 8), "volumes": (V, 4), "texels": (T, 4),
        "color": (h, w, 4) when color=True, "adjoint_ms": float}.
        """
        h, w = settings.height, settings.width
        d = np.asarray(d_color, np.float32)
        if d.shape[:2] != (h, w) or d.ndim != 3 or d.shape[2] not in (3, 4):
            raise ValueError(f"d_color must be ({h}, {w}, 3|4)")
        if d.shape[2] == 3:
            d = np.concatenate([d, np.zeros((h, w, 1), np.float32)], axis=2)
        d = np.ascontiguousarray(d)
        nm, nv, nt = self.adjoint_sizes()
        g_mat = np.zeros((nm // _abi.ADJ_MATERIAL_PARAMS, _abi.ADJ_MATERIAL_PARAMS), np.float32)
        g_vol = np.zeros((nv // _abi.ADJ_VOLUME_PARAMS, _abi.ADJ_VOLUME_PARAMS), np.float32)
        g_tex = np.zeros((nt // 4, 4), np.float32) if texels else None
        img = np.zeros((h, w, 4), np.float32) if color else None
        g = _abi.AdjointGrads()
        g.materials = g_mat.ctypes.data
        g.volumes = g_vol.ctypes.data if (volumes and nv) else None
        g.texels = g_tex.ctypes.data if (g_tex is not None and nt) else None
        g.color = img.ctypes.data if img is not None else None
        self._check(self.lib.phc_adjoint(self.h, C.addressof(camera), C.addressof(settings),
                                         int(sample_offset), d.ctypes.data, C.byref(g)))
        out = {"materials": g_mat, "volumes": g_vol, "adjoint_ms": float(g.adjoint_ms),
               "replay_mismatches": int(g.replay_mismatches)}
        if g_tex is not None:
            out["texels"] = g_tex
        if img is not None:
            out["color"] = img
        return out

    TABLES = {"majorants": 0, "env_marginal": 1, "env_conditional": 2, "emissive_cdf": 3, "prim_light_pdf": 4}

    def scene_table(self, name: str):
        """One of the scene's device tables (phc_scene_table) as a float32 array."""
        import numpy as np
        which = self.TABLES[name]
        n = C.c_uint64(0)
        self._check(self.lib.phc_scene_table(self.h, which, None, 0, C.byref(n)))
        out = np.zeros(n.value, np.float32)
        if n.value:
            self._check(self.lib.phc_scene_table(self.h, which, out.ctypes.data, n.value, C.byref(n)))
        return out

    def stats(self) -> dict:
        s = _abi.RenderStats()
        self._check(self.lib.phc_render_stats_get(self.h, C.byref(s)))
        out = {}
        for k, _ in s._fields_:
            v = getattr(s, k)
            out[k] = list(v) if hasattr(v, "__len__") else v
        return out


def render_batch(jobs) -> dict:
    """Batched mode: jobs is a list of (Renderer, camera, settings, reset);
    all render calls run as one wavefront (phc_render_batch).  Returns the
    batch counters."""
    lib = load()
    arr = (_abi.Job * len(jobs))()
    keep = []
    for k, (r, cam, st, reset) in enumerate(jobs):
        r.width, r.height = st.width, st.height
        arr[k].renderer = r.h
        arr[k].camera = C.pointer(cam)
        arr[k].settings = C.pointer(st)
        arr[k].reset = int(reset)
        keep.append((cam, st))
    s = _abi.RenderStats()
    rc = lib.phc_render_batch(C.addressof(arr), len(jobs), C.byref(s))
    if rc != 0:
        raise PhotonError(rc, lib.phc_last_error(jobs[0][0].h).decode())
    out = {}
    for k, _ in s._fields_:
        v = getattr(s, k)
        out[k] = list(v) if hasattr(v, "__len__") else v
    return out


def tuning_set(key: str, value: int):
    lib = load()
    if lib.phc_tuning_set(key.encode(), int(value)) != 0:
        raise ValueError(f"bad tuning parameter {key}={value}")


def tuning_get(key: str) -> int:
    return int(load().phc_tuning_get(key.encode()))


class Accel:
    """Level A: the ray back-end over caller device pointers (torch tensors)."""

    def __init__(self, positions, indices, normals=None, material_ids=None, objects=None, instances=None):
        """objects / instances: instanced geometry (RayBackend::build_accel_instanced),
        as in scene.PtData: dicts of positions, indices, normals, material_id, and
        (object_id, column-major 4x4 object-to-world) pairs."""
        self.lib = load()
        pos = np.ascontiguousarray(positions, np.float32).reshape(-1)
        idx = np.ascontiguousarray(indices, np.uint32).reshape(-1)
        nrm = None if normals is None else np.ascontiguousarray(normals, np.float32)
        mid = None if material_ids is None else np.ascontiguousarray(material_ids, np.uint32)
        h = C.c_void_p()
        if objects and instances:
            from .scene import PtData
            keep = []
            pt = PtData(objects=list(objects), instances=list(instances)).desc(keep)
            self._keep = keep
            rc = self.lib.phc_accel_create_instanced(
                C.byref(h), pos.ctypes.data if pos.size else None, pos.size // 3,
                idx.ctypes.data if idx.size else None, idx.size // 3, None if nrm is None else nrm.ctypes.data,
                None if mid is None else mid.ctypes.data, C.cast(pt.objects, C.c_void_p), pt.object_count,
                C.cast(pt.instances, C.c_void_p), pt.instance_count)
        else:
            rc = self.lib.phc_accel_create(C.byref(h), pos.ctypes.data, pos.size // 3, idx.ctypes.data, idx.size // 3,
                                           None if nrm is None else nrm.ctypes.data,
                                           None if mid is None else mid.ctypes.data)
        if rc != 0:
            raise PhotonError(rc, self.lib.phc_accel_error().decode())
        self.h = h

    def close(self):
        if getattr(self, "h", None):
            self.lib.phc_accel_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def _run(self, fn, o, d, t0, t1, out, stream=None):
        n = int(t0.numel())
        rc = fn(self.h, o.data_ptr(), d.data_ptr(), t0.data_ptr(), t1.data_ptr(), n, out.data_ptr(), stream)
        if rc != 0:
            raise PhotonError(rc, self.lib.phc_accel_error().decode())
        return out

    def trace_closest(self, o, d, tmin, tmax, out=None):
        """88-byte HitResult records into a uint8 CUDA tensor (n, 88)."""
        import torch
        if out is None:
            out = torch.empty((tmin.numel(), 88), dtype=torch.uint8, device=tmin.device)
        return self._run(self.lib.phc_trace_closest, o, d, tmin, tmax, out)

    def trace_closest_compact(self, o, d, tmin, tmax, out=None):
        import torch
        if out is None:
            out = torch.empty((tmin.numel(), 4), dtype=torch.float32, device=tmin.device)
        return self._run(self.lib.phc_trace_closest_compact, o, d, tmin, tmax, out)

    def trace_occluded(self, o, d, tmin, tmax, out=None):
        import torch
        if out is None:
            out = torch.empty((tmin.numel(),), dtype=torch.int32, device=tmin.device)
        return self._run(self.lib.phc_trace_occluded, o, d, tmin, tmax, out)

    def counters(self):
        a, b = C.c_uint64(), C.c_uint64()
        self.lib.phc_accel_counters(self.h, C.byref(a), C.byref(b))
        return int(a.value), int(b.value)

    def info(self):
        a, b, c = C.c_uint64(), C.c_uint64(), C.c_uint64()
        self.lib.phc_accel_info(self.h, C.byref(a), C.byref(b), C.byref(c))
        return {"node_bytes": a.value, "tri_bytes": b.value, "node_count": c.value}
