"""Loads the golden fixtures written by make_golden.py back into scenes."""
from __future__ import annotations

import ctypes as C
import glob
import os

import numpy as np

from photon_gb300 import _abi
from photon_gb300.scene import SceneData

HERE = os.path.dirname(os.path.abspath(__file__))


def _records(buf, cls):
    size = C.sizeof(cls)
    raw = bytes(buf)
    return [cls.from_buffer_copy(raw[i:i + size]) for i in range(0, len(raw), size)]


def scene_names():
    return sorted(os.path.basename(p)[6:-4] for p in glob.glob(os.path.join(HERE, "scene_*.npz")))


def load_scene(name):
    """(SceneData, camera, settings, frames) of fixture scene_<name>.npz."""
    z = np.load(os.path.join(HERE, f"scene_{name}.npz"))
    attrs = [z[f"attr{k}"] if f"attr{k}" in z else None for k in range(5)]
    sc = SceneData(positions=z["positions"], indices=z["indices"], material_ids=z["material_ids"],
                   normals=z["normals"] if "normals" in z else None, attributes=attrs, name=name)
    sc.materials = _records(z["materials"], _abi.Material)
    sc.lights = _records(z["lights"], _abi.Light)
    samplers = _records(z["samplers"], _abi.Sampler)
    sc.samplers = [(s, z[f"texels{k}"] if f"texels{k}" in z else None) for k, s in enumerate(samplers)]
    vols = _records(z["volumes"], _abi.Volume)
    sc.volumes = [(v, z[f"vol_values{k}"], z[f"vol_tf{k}"]) for k, v in enumerate(vols)]
    if "env_pixels" in z:
        sc.env_pixels = z["env_pixels"]
        sc.env_visible = bool(z["env_visible"])
        sc.env_world_to_map = tuple(float(x) for x in z["env_world_to_map"])
    cam = _records(z["camera"], _abi.Camera)[0]
    st = _records(z["settings"], _abi.Settings)[0]
    st.background_image = C.POINTER(C.c_float)()
    if "background_image" in z:
        bg = np.ascontiguousarray(z["background_image"], np.float32)
        st._bg = bg
        st.background_image = bg.ctypes.data_as(C.POINTER(C.c_float))
    frames = []
    f = 0
    while f"f{f}_color" in z:
        frames.append({ch: z[f"f{f}_{ch}"] for ch in ("color", "depth", "normal", "albedo")})
        f += 1
    return sc, cam, st, frames


def load_trace():
    return dict(np.load(os.path.join(HERE, "trace.npz")))


def load_bsdf():
    z = np.load(os.path.join(HERE, "bsdf.npz"))
    mats = _records(z["materials"], _abi.Material)
    cases = []
    for k, m in enumerate(mats):
        cases.append((m, z[f"ng{k}"], z[f"ns{k}"], z[f"wo{k}"], z[f"wi{k}"], z[f"seeds{k}"], z[f"out{k}"],
                      z[f"out2{k}"]))
    return cases
