"""CPU oracles for the path-tracing hot path (TEST INFRASTRUCTURE ONLY).

Two shared libraries, both built by oracle/Makefile:

* ``_ref/libphoton_ref.so`` — Photon's own sources (pathtracer.cpp, bvh.cpp,
  kokkos_backend.cpp, environment_map.cpp, RenderBridge.cpp) compiled
  unmodified against the project's Kokkos stand-in.  Exists only where the
  reference checkout was present at build time (not on the GPU host).
* ``_build/libphoton_oracle.so`` — the project's CPU restatement of the same
  algorithm (photon_oracle.cpp), bit-identical to the reference on the same
  compiler and flags; it builds anywhere.

Both expose the same renderer calls (create / set_scene / render / read_*),
plus Level-A tracing and BSDF probes.  Only tests/, __graft_entry__.smoke()
and bench.py's CPU-baseline leg may use this package; the product never does.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
REF_LIB = os.path.join(HERE, "_ref", "libphoton_ref.so")
ORACLE_LIB = os.path.join(HERE, "_build", "libphoton_oracle.so")
# the restatement with double-evaluated transcendental functions (a second libm)
ORACLE_DLIBM_LIB = os.path.join(HERE, "_build", "libphoton_oracle_dlibm.so")
_LIBS = {"ref": (REF_LIB, "ref_"), "oracle": (ORACLE_LIB, "orc_"), "oracle_dlibm": (ORACLE_DLIBM_LIB, "orc_")}
# The reference checkout, when it is not where oracle/Makefile looks (REF).
REFERENCE_DIR = os.environ.get("PHOTON_REFERENCE_DIR", "")


def build(ref: bool | None = None, jobs: int = 8, quiet: bool = True):
    """Build the restatement (always) and the reference oracle: where the
    reference checkout exists (ref=None), always (ref=True) or never
    (ref=False)."""
    targets = ["oracle"] + {None: ["ref-if-present"], True: ["ref"], False: []}[ref]
    out = subprocess.run(["make", "-C", HERE, f"-j{jobs}"] + ([f"REF={REFERENCE_DIR}"] if REFERENCE_DIR else [])
                         + targets, capture_output=True, text=True)
    if out.returncode != 0:
        raise RuntimeError("oracle build failed:\n" + out.stdout[-4000:] + out.stderr[-4000:])
    return targets


def have_ref() -> bool:
    """Whether the reference oracle is built (after build())."""
    return os.path.exists(REF_LIB)


_libs = {}


def _load(path, prefix):
    if path in _libs:
        return _libs[path]
    if not os.path.exists(path):
        raise FileNotFoundError(path)
    lib = C.CDLL(path)
    vp, cp = C.c_void_p, C.c_char_p
    fn = lambda n: getattr(lib, prefix + n)  # noqa: E731
    fn("renderer_create").restype = vp
    fn("renderer_create").argtypes = []
    fn("renderer_destroy").argtypes = [vp]
    fn("last_error").restype = cp
    fn("last_error").argtypes = [vp]
    fn("set_scene").argtypes = [vp, vp]
    fn("render").argtypes = [vp, vp, vp, C.c_int]
    fn("accumulated_samples").restype = C.c_uint32
    fn("accumulated_samples").argtypes = [vp]
    for ch in ("color", "depth", "normal", "albedo"):
        fn("read_" + ch).argtypes = [vp, vp]
    fn("trace").argtypes = [vp, C.c_uint64, vp, C.c_uint64, vp, vp, vp, vp, vp, vp, C.c_uint32, C.c_int, vp, vp]
    fn("bsdf_probe").argtypes = [vp, vp, vp, vp, vp, vp, C.c_uint32, vp, vp]
    _libs[path] = lib
    return lib


def _ptr(a):
    return None if a is None else a.ctypes.data


class CpuRenderer:
    """bridge::Renderer-shaped wrapper over one of the two oracle libraries."""

    def __init__(self, which: str = "oracle"):
        self.which = which
        path, self.prefix = _LIBS[which]
        self.lib = _load(path, self.prefix)
        self.h = self._fn("renderer_create")()
        if not self.h:
            raise RuntimeError(f"{which}: renderer_create failed")
        self.width = self.height = 0
        self._keep = None

    def _fn(self, name):
        return getattr(self.lib, self.prefix + name)

    def close(self):
        if self.h:
            self._fn("renderer_destroy")(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def _check(self, rc, what):
        if rc != 0:
            raise RuntimeError(f"{self.which} {what}: {self._fn('last_error')(self.h).decode()}")

    def set_scene(self, scene):
        desc, keep = scene.desc()
        self._keep = (desc, keep)
        self._check(self._fn("set_scene")(self.h, C.addressof(desc)), "set_scene")

    def render(self, cam, settings, reset=True):
        self.width, self.height = settings.width, settings.height
        self._check(self._fn("render")(self.h, C.addressof(cam), C.addressof(settings), int(reset)), "render")

    def accumulated_samples(self):
        return self._fn("accumulated_samples")(self.h)

    def read(self, channel):
        n = {"color": 4, "depth": 1, "normal": 3, "albedo": 3}[channel]
        out = np.empty((self.height, self.width, n), np.float32)
        self._check(self._fn("read_" + channel)(self.h, out.ctypes.data), "read_" + channel)
        return out[..., 0] if n == 1 else out


def trace(which, positions, indices, orgs, dirs, tmin, tmax, any_hit=False, normals=None, material_ids=None):
    """Level-A trace through the reference's KokkosBackend ('ref') or the
    restatement ('oracle'); returns the HitResult records or occluded flags."""
    from photon_gb300 import _abi
    prefix = "ref_" if which == "ref" else "orc_"
    lib = _load(REF_LIB if which == "ref" else ORACLE_LIB, prefix)
    pos = np.ascontiguousarray(positions, np.float32)
    idx = np.ascontiguousarray(indices, np.uint32)
    o = np.ascontiguousarray(orgs, np.float32)
    d = np.ascontiguousarray(dirs, np.float32)
    t0 = np.ascontiguousarray(tmin, np.float32)
    t1 = np.ascontiguousarray(tmax, np.float32)
    nrm = None if normals is None else np.ascontiguousarray(normals, np.float32)
    mid = None if material_ids is None else np.ascontiguousarray(material_ids, np.uint32)
    n = len(t0)
    hits = np.zeros(n, _abi.hit_dtype())
    occ = np.zeros(n, np.uint32)
    rc = getattr(lib, prefix + "trace")(
        _ptr(pos), pos.size // 3, _ptr(idx), idx.size // 3, _ptr(nrm), _ptr(mid), _ptr(o), _ptr(d), _ptr(t0),
        _ptr(t1), n, int(any_hit), hits.ctypes.data, occ.ctypes.data)
    if rc != 0:
        raise RuntimeError("trace failed")
    return occ if any_hit else hits


def adjoint_fp64(renderer, cam, settings, d_color, params, directions=(), sample_offset=0, h=1e-4):
    """FP64 CPU adjoint (adjoint_fp64.inc) on a CpuRenderer("oracle") with a
    scene: gradients of sum(d_color * I) for params [(kind, index, comp)]
    (kind 0 material, 1 volume, 2 texels along directions[index])."""
    if renderer.which != "oracle":
        raise ValueError("the FP64 adjoint lives in the restatement oracle")
    lib = renderer.lib
    fn = lib.orc_adjoint_fp64
    fn.restype = C.c_int
    fn.argtypes = [C.c_void_p, C.c_void_p, C.c_void_p, C.c_uint32, C.c_void_p, C.c_uint32, C.c_void_p, C.c_void_p,
                   C.c_void_p, C.c_void_p, C.c_double, C.c_void_p]
    d = np.ascontiguousarray(d_color, np.float32)
    n = len(params)
    kind = np.array([p[0] for p in params], np.int32)
    index = np.array([p[1] for p in params], np.int32)
    comp = np.array([p[2] for p in params], np.int32)
    dirs = [np.ascontiguousarray(x, np.float32) for x in directions]
    ptrs = (C.c_void_p * max(1, len(dirs)))(*[x.ctypes.data for x in dirs])
    out = np.zeros(n, np.float64)
    rc = fn(renderer.h, C.addressof(cam), C.addressof(settings), int(sample_offset), d.ctypes.data, n,
            kind.ctypes.data, index.ctypes.data, comp.ctypes.data, C.addressof(ptrs), float(h), out.ctypes.data)
    if rc != 0:
        raise RuntimeError("orc_adjoint_fp64: " + renderer._fn("last_error")(renderer.h).decode())
    return out


def bsdf_probe(which, material, n_geo, n_shade, wo, wi, seeds):
    """Disney BSDF eval/pdf/sample at n cases (see ref_harness.cpp)."""
    prefix = "ref_" if which == "ref" else "orc_"
    lib = _load(REF_LIB if which == "ref" else ORACLE_LIB, prefix)
    arrs = [np.ascontiguousarray(a, np.float32) for a in (n_geo, n_shade, wo, wi)]
    s = np.ascontiguousarray(seeds, np.uint32)
    n = len(s)
    out = np.zeros((n, 8), np.float32)
    out2 = np.zeros((n, 4), np.float32)
    getattr(lib, prefix + "bsdf_probe")(C.addressof(material), *[a.ctypes.data for a in arrs], s.ctypes.data, n,
                                        out.ctypes.data, out2.ctypes.data)
    return out, out2


class RefPbrt:
    """The reference's own pbrt path (parse_pbrt_file + convert_pbrt_scene +
    PathTracer::render) from oracle/_ref/libphoton_ref.so.  Exists only where
    the reference checkout was present at build time."""

    COUNTS = ("triangles", "materials", "emissive", "textures", "lights", "width", "height", "spp",
              "max_depth", "meshes", "named_materials", "object_defs", "object_instances", "has_env")

    def __init__(self, path, use_instancing=False, width=0, height=0, spp=0, max_depth=0):
        from photon_gb300 import _abi
        self._abi = _abi
        lib = _load(REF_LIB, "ref_")
        vp = C.c_void_p
        lib.ref_pbrt_load.restype = vp
        lib.ref_pbrt_load.argtypes = [C.c_char_p, C.c_int, C.c_int, C.c_int, C.c_int, C.c_int]
        lib.ref_pbrt_free.argtypes = [vp]
        for n in ("counts", "mesh", "materials", "emissive", "camera", "env", "render"):
            getattr(lib, "ref_pbrt_" + n).restype = C.c_int
        lib.ref_pbrt_counts.argtypes = [vp, vp]
        lib.ref_pbrt_mesh.argtypes = [vp, vp, vp, vp, vp, vp]
        lib.ref_pbrt_materials.argtypes = [vp, vp]
        lib.ref_pbrt_emissive.argtypes = [vp, vp, vp]
        lib.ref_pbrt_camera.argtypes = [vp, vp]
        lib.ref_pbrt_env.argtypes = [vp, vp, vp, vp, vp]
        lib.ref_pbrt_texture.argtypes = [vp, C.c_uint32, vp, vp]
        lib.ref_pbrt_render.argtypes = [vp, C.c_int, C.c_int, vp]
        self.lib = lib
        self.h = lib.ref_pbrt_load(str(path).encode(), int(use_instancing), width, height, spp, max_depth)
        c = np.zeros(len(self.COUNTS), np.uint64)
        lib.ref_pbrt_counts(self.h, c.ctypes.data)
        self.counts = dict(zip(self.COUNTS, (int(x) for x in c)))

    def arrays(self) -> dict:
        n = self.counts
        nt = n["triangles"]
        pos = np.zeros((3 * nt, 3), np.float32)
        nrm = np.zeros((3 * nt, 3), np.float32)
        uv = np.zeros((3 * nt, 2), np.float32)
        mids = np.zeros(nt, np.uint32)
        idx = np.zeros(3 * nt, np.uint32)
        if nt:
            self.lib.ref_pbrt_mesh(self.h, pos.ctypes.data, nrm.ctypes.data, uv.ctypes.data, mids.ctypes.data,
                                   idx.ctypes.data)
        mats = (self._abi.PtMaterial * max(n["materials"], 1))()
        self.lib.ref_pbrt_materials(self.h, C.addressof(mats))
        eids = np.zeros(n["emissive"], np.uint32)
        eareas = np.zeros(n["emissive"], np.float32)
        if n["emissive"]:
            self.lib.ref_pbrt_emissive(self.h, eids.ctypes.data, eareas.ctypes.data)
        cam = np.zeros(23, np.float32)
        self.lib.ref_pbrt_camera(self.h, cam.ctypes.data)
        wh = np.zeros(2, np.uint32)
        w2t = np.zeros(9, np.float32)
        t2w = np.zeros(9, np.float32)
        self.lib.ref_pbrt_env(self.h, wh.ctypes.data, None, w2t.ctypes.data, t2w.ctypes.data)
        env = None
        if wh[0]:
            px = np.zeros((int(wh[1]), int(wh[0]), 3), np.float32)
            self.lib.ref_pbrt_env(self.h, wh.ctypes.data, px.ctypes.data, w2t.ctypes.data, t2w.ctypes.data)
            env = {"pixels": px, "world_to_map": w2t.reshape(3, 3), "map_to_world": t2w.reshape(3, 3)}
        tex = []
        for i in range(n["textures"]):
            twh = np.zeros(2, np.uint32)
            self.lib.ref_pbrt_texture(self.h, i, twh.ctypes.data, None)
            px = np.zeros((int(twh[1]), int(twh[0]), 3), np.float32)
            self.lib.ref_pbrt_texture(self.h, i, twh.ctypes.data, px.ctypes.data)
            tex.append(px)
        return {"positions": pos, "normals": nrm, "texcoords": uv, "material_ids": mids,
                "indices": idx.reshape(-1, 3), "materials": [mats[i] for i in range(n["materials"])],
                "emissive_ids": eids, "emissive_areas": eareas, "camera": cam, "env": env, "textures": tex}

    def instanced(self) -> dict:
        """ConvertedScene::instanced_geometry: objects (positions, indices,
        normals, material id) and instances (object id, column-major 4x4)."""
        lib, vp = self.lib, C.c_void_p
        lib.ref_pbrt_ig_counts.argtypes = [vp, vp]
        lib.ref_pbrt_ig_object.argtypes = [vp, C.c_uint32, vp, vp, vp, vp]
        lib.ref_pbrt_ig_instance.argtypes = [vp, C.c_uint32, vp, vp]
        c = np.zeros(2, np.uint64)
        lib.ref_pbrt_ig_counts(self.h, c.ctypes.data)
        objs = []
        for i in range(int(c[0])):
            sz = np.zeros(4, np.uint64)
            lib.ref_pbrt_ig_object(self.h, i, sz.ctypes.data, None, None, None)
            pos = np.zeros(int(sz[0]), np.float32)
            idx = np.zeros(int(sz[1]), np.int32)
            nrm = np.zeros(int(sz[2]), np.float32)
            lib.ref_pbrt_ig_object(self.h, i, sz.ctypes.data, pos.ctypes.data, idx.ctypes.data, nrm.ctypes.data)
            objs.append({"positions": pos, "indices": idx, "normals": nrm, "material_id": int(sz[3])})
        insts = []
        for i in range(int(c[1])):
            oid = np.zeros(1, np.uint32)
            xf = np.zeros(16, np.float32)
            lib.ref_pbrt_ig_instance(self.h, i, oid.ctypes.data, xf.ctypes.data)
            insts.append((int(oid[0]), xf))
        return {"objects": objs, "instances": insts}

    def render(self, adaptive=False, bottom_up=True) -> np.ndarray:
        """(h, w, 3) radiance; row 0 = the bottom row when bottom_up."""
        w, h = self.counts["width"], self.counts["height"]
        out = np.zeros((h, w, 3), np.float32)
        self.lib.ref_pbrt_render(self.h, int(adaptive), int(bottom_up), out.ctypes.data)
        return out

    def close(self):
        if self.h:
            self.lib.ref_pbrt_free(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
