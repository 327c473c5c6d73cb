"""Host-side scene container: the Python mirror of bridge::SceneData.

`SceneData` holds numpy arrays and ctypes records, exactly the content of
photon::bridge::SceneData (src/photon/anari/RenderBridge.h:112-126); `desc()`
packs it into the phc_scene_desc of include/photon_cuda.h without copying the
arrays (they stay owned by this object, as the C-ABI requires: the library
copies them during phc_set_scene).
"""
from __future__ import annotations

import ctypes as C
from dataclasses import dataclass, field

import numpy as np

from . import _abi


def _fptr(a):
    if a is None:
        return C.POINTER(C.c_float)()
    return a.ctypes.data_as(C.POINTER(C.c_float))


def _uptr(a):
    if a is None:
        return C.POINTER(C.c_uint32)()
    return a.ctypes.data_as(C.POINTER(C.c_uint32))


def _f32(a, shape_last=None):
    if a is None:
        return None
    a = np.ascontiguousarray(a, dtype=np.float32)
    if shape_last is not None:
        a = a.reshape(-1, shape_last)
    return a


@dataclass
class PtData:
    """The path-tracer-level part of a scene (phc_pt_scene): pt::Material
    records, per-vertex texture coordinates, atlas textures, the environment's
    map-to-world rotation and instanced geometry (objects in their own space,
    placed by column-major object-to-world transforms)."""
    materials: list = field(default_factory=list)   # _abi.PtMaterial
    texcoords: np.ndarray | None = None             # (V, 2) float32
    textures: list = field(default_factory=list)    # (h, w, 3) float32, row 0 = top
    env_map_to_world: tuple | None = None           # 9 floats, row-major
    objects: list = field(default_factory=list)     # dict(positions, indices, normals=None, material_id=0)
    instances: list = field(default_factory=list)   # (object_id, 16 floats column-major)

    def desc(self, keep):
        p = _abi.PtScene()
        if self.materials:
            arr = (_abi.PtMaterial * len(self.materials))(*self.materials)
            keep.append(arr)
            p.materials = C.cast(arr, C.POINTER(_abi.PtMaterial))
        if self.texcoords is not None:
            t = np.ascontiguousarray(self.texcoords, dtype=np.float32).reshape(-1, 2)
            keep.append(t)
            p.texcoords = _fptr(t)
        if self.textures:
            recs = []
            for img in self.textures:
                a = np.ascontiguousarray(img, dtype=np.float32)
                keep.append(a)
                recs.append(_abi.Texture(a.shape[1], a.shape[0], _fptr(a)))
            arr = (_abi.Texture * len(recs))(*recs)
            keep.append(arr)
            p.textures = C.cast(arr, C.POINTER(_abi.Texture))
            p.texture_count = len(recs)
        if self.env_map_to_world is not None:
            p.env_map_to_world_given = 1
            p.env_map_to_world[:] = list(self.env_map_to_world)
        if self.objects:
            recs = []
            for ob in self.objects:
                pos = _f32(ob["positions"], 3)
                idx = np.ascontiguousarray(ob["indices"], dtype=np.uint32).reshape(-1, 3)
                nrm = _f32(ob.get("normals"), 3)
                keep += [pos, idx, nrm]
                recs.append(_abi.Object(_fptr(pos), pos.shape[0], _uptr(idx), idx.shape[0], _fptr(nrm),
                                        int(ob.get("material_id", 0))))
            arr = (_abi.Object * len(recs))(*recs)
            keep.append(arr)
            p.objects = C.cast(arr, C.POINTER(_abi.Object))
            p.object_count = len(recs)
        if self.instances:
            recs = []
            for oid, xf in self.instances:
                r = _abi.Instance()
                r.object_id = int(oid)
                r.transform[:] = [float(x) for x in np.asarray(xf, np.float32).ravel()]
                recs.append(r)
            arr = (_abi.Instance * len(recs))(*recs)
            keep.append(arr)
            p.instances = C.cast(arr, C.POINTER(_abi.Instance))
            p.instance_count = len(recs)
        keep.append(p)
        return p


@dataclass
class SceneData:
    positions: np.ndarray                      # (V, 3) float32
    indices: np.ndarray                        # (T, 3) uint32
    material_ids: np.ndarray | None = None     # (T,) uint32
    normals: np.ndarray | None = None          # (V, 3) float32
    attributes: list = field(default_factory=lambda: [None] * 5)  # (V, 4) float32 each
    materials: list = field(default_factory=list)   # _abi.Material
    samplers: list = field(default_factory=list)    # (_abi.Sampler, texels (N,4) f32)
    lights: list = field(default_factory=list)      # _abi.Light
    env_pixels: np.ndarray | None = None       # (H, W, 3) float32, row 0 = bottom
    env_visible: bool = True
    env_world_to_map: tuple = (1, 0, 0, 0, 1, 0, 0, 0, 1)
    volumes: list = field(default_factory=list)     # (_abi.Volume, values f32, transfer (K,4) f32)
    name: str = "scene"
    pt: PtData | None = None                   # path-tracer-level part (phc_pt_scene)

    def __post_init__(self):
        self.positions = _f32(self.positions, 3)
        self.indices = np.ascontiguousarray(self.indices, dtype=np.uint32).reshape(-1, 3)
        if self.material_ids is not None:
            self.material_ids = np.ascontiguousarray(self.material_ids, dtype=np.uint32).reshape(-1)
        self.normals = _f32(self.normals, 3)
        self.attributes = [_f32(a, 4) for a in (list(self.attributes) + [None] * 5)[:5]]
        if self.env_pixels is not None:
            self.env_pixels = np.ascontiguousarray(self.env_pixels, dtype=np.float32)

    @property
    def triangle_count(self) -> int:
        return int(self.indices.shape[0])

    def desc(self):
        """phc_scene_desc over this scene's arrays (valid while self lives)."""
        d = _abi.SceneDesc()
        keep = []
        d.positions = _fptr(self.positions)
        d.vertex_count = self.positions.shape[0]
        d.normals = _fptr(self.normals)
        for s in range(5):
            d.attributes[s] = _fptr(self.attributes[s])
        d.indices = _uptr(self.indices)
        d.triangle_count = self.indices.shape[0]
        if self.material_ids is not None:
            d.material_ids = _uptr(self.material_ids)
            d.material_id_count = self.material_ids.shape[0]
        if self.materials:
            arr = (_abi.Material * len(self.materials))(*self.materials)
            keep.append(arr)
            d.materials = C.cast(arr, C.POINTER(_abi.Material))
            d.material_count = len(self.materials)
        if self.samplers:
            recs = []
            for rec, texels in self.samplers:
                r = _abi.Sampler()
                C.pointer(r)[0] = rec
                if texels is not None:
                    t = np.ascontiguousarray(texels, dtype=np.float32).reshape(-1, 4)
                    keep.append(t)
                    r.texels = _fptr(t)
                    r.texel_count = t.shape[0]
                recs.append(r)
            arr = (_abi.Sampler * len(recs))(*recs)
            keep.append(arr)
            d.samplers = C.cast(arr, C.POINTER(_abi.Sampler))
            d.sampler_count = len(recs)
        if self.lights:
            arr = (_abi.Light * len(self.lights))(*self.lights)
            keep.append(arr)
            d.lights = C.cast(arr, C.POINTER(_abi.Light))
            d.light_count = len(self.lights)
        if self.env_pixels is not None:
            h, w = self.env_pixels.shape[:2]
            d.environment.present = 1
            d.environment.visible = 1 if self.env_visible else 0
            d.environment.width = w
            d.environment.height = h
            d.environment.pixels = _fptr(self.env_pixels)
            d.environment.world_to_map[:] = self.env_world_to_map
        if self.volumes:
            recs = []
            for rec, values, transfer in self.volumes:
                r = _abi.Volume()
                C.pointer(r)[0] = rec
                v = np.ascontiguousarray(values, dtype=np.float32).reshape(-1)
                t = np.ascontiguousarray(transfer, dtype=np.float32).reshape(-1, 4)
                keep += [v, t]
                r.values = _fptr(v)
                r.value_count = v.shape[0]
                r.transfer = _fptr(t)
                r.transfer_count = t.shape[0]
                recs.append(r)
            arr = (_abi.Volume * len(recs))(*recs)
            keep.append(arr)
            d.volumes = C.cast(arr, C.POINTER(_abi.Volume))
            d.volume_count = len(recs)
        if self.pt is not None:
            p = self.pt.desc(keep)
            d.pt = C.pointer(p)
            d.material_count = len(self.pt.materials)
        return d, keep


def settings(width, height, spp, max_depth, **kw):
    """phc_settings with the bridge defaults and the given overrides."""
    s = _abi.settings_default()
    s.width, s.height, s.pixel_samples, s.max_depth = width, height, spp, max_depth
    for k, v in kw.items():
        if k in ("background", "ambient_color"):
            getattr(s, k)[:] = v
        else:
            setattr(s, k, v)
    return s


def camera(position, look_at, up=(0, 1, 0), fovy_deg=40.0, aspect=0.0, **kw):
    """phc_camera looking from `position` at `look_at`."""
    c = _abi.camera_default()
    p = np.asarray(position, np.float32)
    d = np.asarray(look_at, np.float32) - p
    d = d / np.linalg.norm(d)
    c.position[:] = p.tolist()
    c.direction[:] = d.tolist()
    c.up[:] = list(up)
    c.fovy = float(np.deg2rad(fovy_deg))
    c.aspect = aspect
    for k, v in kw.items():
        if k == "image_region":
            c.image_region[:] = v
        else:
            setattr(c, k, v)
    return c
