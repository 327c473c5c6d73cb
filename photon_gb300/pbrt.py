"""pbrt-v4 scenes: the reference's photon_pbrt_render path on the GPU renderer.

    from photon_gb300 import pbrt, Renderer
    sc = pbrt.load("scene.pbrt")            # parse_pbrt_file + convert_pbrt_scene
    r = Renderer(); r.set_scene(sc)         # the converted scene, as uploaded
    r.render(sc.camera, sc.settings)        # camera and PathTracer params of the file
    img = r.read_color()

load() calls phc_pbrt_load (include/photon_pbrt.h), which stands in for
parse_pbrt_file (src/photon/pbrt/pbrt_parser.cpp:272-640) and
convert_pbrt_scene (src/photon/pbrt/pbrt_to_photon.cpp:58-503).  The returned
PbrtScene owns the converted scene; its desc() is what Renderer.set_scene
takes, like a SceneData's.

`python -m photon_gb300.pbrt scene.pbrt -o out.ppm [--width W --height H
--spp N --max-depth D --exposure E]` mirrors app/photon_pbrt_render.cpp:
render, then ACES-filmic tone mapping and gamma 2.2 into a binary PPM with
the top row first.
"""
from __future__ import annotations

import argparse
import ctypes as C
import sys
import time

import numpy as np

from . import _abi
from .native import PhotonError, load as load_lib


class PbrtOptions(C.Structure):
    _fields_ = [("use_instancing", C.c_int32), ("width", C.c_int32), ("height", C.c_int32),
                ("spp", C.c_int32), ("max_depth", C.c_int32)]


class PbrtInfo(C.Structure):
    _fields_ = [("meshes", C.c_uint64), ("named_materials", C.c_uint64), ("textures", C.c_uint64),
                ("loaded_textures", C.c_uint64), ("object_defs", C.c_uint64),
                ("object_instances", C.c_uint64), ("triangles", C.c_uint64),
                ("emissive_triangles", C.c_uint64), ("width", C.c_uint32), ("height", C.c_uint32),
                ("spp", C.c_uint32), ("max_depth", C.c_uint32), ("has_env_map", C.c_int32)]


class PbrtScene:
    """A converted pbrt scene (owned by the library until close())."""

    def __init__(self, handle, lib):
        self.h, self.lib = handle, lib
        dp = C.c_void_p()
        self._check(lib.phc_pbrt_scene_desc(self.h, C.byref(dp)))
        self._desc = _abi.SceneDesc.from_address(dp.value)
        self.camera = _abi.Camera()
        self._check(lib.phc_pbrt_camera(self.h, C.byref(self.camera)))
        self.settings = _abi.Settings()
        self._check(lib.phc_pbrt_settings(self.h, C.byref(self.settings)))
        inf = PbrtInfo()
        self._check(lib.phc_pbrt_info_get(self.h, C.byref(inf)))
        self.info = {k: getattr(inf, k) for k, _ in PbrtInfo._fields_}

    def _check(self, rc):
        if rc != 0:
            raise PhotonError(rc, self.lib.phc_global_error().decode())

    def desc(self):
        """(phc_scene_desc, keep-alive) for Renderer.set_scene."""
        if self.h is None:
            raise ValueError("the pbrt scene is closed")
        return self._desc, self

    def triangle_count(self) -> int:
        return int(self._desc.triangle_count)

    # arrays of the converted scene (copies), for inspection and tests
    def arrays(self) -> dict:
        d, pt = self._desc, self._desc.pt.contents
        nv, nt, nm = int(d.vertex_count), int(d.triangle_count), int(d.material_count)

        def arr(ptr, n, dt):
            if n == 0 or not ptr:
                return np.zeros(0, dt)
            return np.ctypeslib.as_array(ptr, shape=(n,)).copy()

        out = {
            "positions": arr(d.positions, nv * 3, np.float32).reshape(-1, 3),
            "normals": arr(d.normals, nv * 3, np.float32).reshape(-1, 3),
            "indices": arr(d.indices, nt * 3, np.uint32).reshape(-1, 3),
            "material_ids": arr(d.material_ids, nt, np.uint32),
            "texcoords": arr(pt.texcoords, nv * 2, np.float32).reshape(-1, 2),
            "materials": [_abi.PtMaterial.from_buffer_copy(pt.materials[i]) for i in range(nm)],
            "textures": [],
            "env": None,
        }
        for i in range(pt.texture_count):
            t = pt.textures[i]
            out["textures"].append(arr(t.rgb, t.width * t.height * 3, np.float32).reshape(t.height, t.width, 3))
        out["objects"], out["instances"] = [], []
        for i in range(pt.object_count):
            ob = pt.objects[i]
            out["objects"].append({
                "positions": arr(ob.positions, ob.vertex_count * 3, np.float32),
                "indices": arr(ob.indices, ob.triangle_count * 3, np.uint32),
                "normals": arr(ob.normals, ob.vertex_count * 3, np.float32),
                "material_id": int(ob.material_id)})
        for i in range(pt.instance_count):
            ins = pt.instances[i]
            out["instances"].append((int(ins.object_id), np.array(ins.transform[:], np.float32)))
        e = d.environment
        if e.present:
            out["env"] = {
                "pixels": arr(e.pixels, e.width * e.height * 3, np.float32).reshape(e.height, e.width, 3),
                "world_to_map": np.array(e.world_to_map[:], np.float32).reshape(3, 3),
                "map_to_world": np.array(pt.env_map_to_world[:], np.float32).reshape(3, 3),
            }
        return out

    def close(self):
        if self.h is not None:
            self.lib.phc_pbrt_free(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def load(path: str, use_instancing: bool = False, width: int = 0, height: int = 0, spp: int = 0,
         max_depth: int = 0) -> PbrtScene:
    """Parses and converts a pbrt-v4 file; values > 0 override the file's
    Film size, pixel samples and maximum depth (photon_pbrt_render's
    --width/--height/--spp/--max-depth)."""
    lib = load_lib()
    opt = PbrtOptions(int(use_instancing), int(width), int(height), int(spp), int(max_depth))
    h = C.c_void_p()
    rc = lib.phc_pbrt_load(str(path).encode(), C.byref(opt), C.byref(h))
    if rc != 0:
        raise PhotonError(rc, lib.phc_global_error().decode())
    return PbrtScene(h, lib)


def aces_filmic(x):
    """Narkowicz 2015 fit, as photon_pbrt_render.cpp:64-70 applies it."""
    a, b, c, d, e = 2.51, 0.03, 2.43, 0.59, 0.14
    x = np.maximum(x, 0.0)
    return np.minimum((x * (a * x + b)) / (x * (c * x + d) + e), 1.0)


def write_ppm(path: str, rgb_top_down: np.ndarray, exposure: float = 1.0):
    """Binary PPM of an (h, w, 3) radiance image, top row first, with the
    application's tone mapping (photon_pbrt_render.cpp:72-98)."""
    v = np.power(aces_filmic(rgb_top_down.astype(np.float32) * np.float32(exposure)), 1.0 / 2.2)
    u8 = np.floor(v * 255.0 + 0.5).astype(np.uint8)
    h, w = u8.shape[:2]
    with open(path, "wb") as f:
        f.write(f"P6\n{w} {h}\n255\n".encode())
        f.write(u8.tobytes())


def main(argv=None):
    ap = argparse.ArgumentParser(description="Render a pbrt-v4 scene on the GPU renderer")
    ap.add_argument("scene")
    ap.add_argument("-o", "--output", default="pbrt_render.ppm")
    ap.add_argument("--width", type=int, default=-1)
    ap.add_argument("--height", type=int, default=-1)
    ap.add_argument("--spp", type=int, default=-1)
    ap.add_argument("--max-depth", type=int, default=-1)
    ap.add_argument("--use-ias", action="store_true")
    ap.add_argument("--exposure", type=float, default=1.0)
    a = ap.parse_args(argv)
    from .renderer import Renderer
    t0 = time.perf_counter()
    sc = load(a.scene, a.use_ias, a.width, a.height, a.spp, a.max_depth)
    t1 = time.perf_counter()
    inf = sc.info
    print(f"Parsed and converted in {(t1 - t0) * 1e3:.1f} ms: {inf['meshes']} meshes, "
          f"{inf['named_materials']} materials, {inf['triangles']} triangles, "
          f"{inf['width']}x{inf['height']} @ {inf['spp']} spp", file=sys.stderr)
    r = Renderer()
    r.set_scene(sc)
    r.render(sc.camera, sc.settings, True)
    print(f"Rendered in {r.stats()['render_ms']:.1f} ms", file=sys.stderr)
    img = r.read_color()[..., :3][::-1]  # the renderer's row 0 is the bottom row
    write_ppm(a.output, img, a.exposure)
    print(f"Output: {a.output}", file=sys.stderr)
    r.close()
    sc.close()


if __name__ == "__main__":
    main()
