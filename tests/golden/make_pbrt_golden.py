"""Generates tests/golden/pbrt_ref.npz from the REFERENCE's own pbrt path.

Run where the reference sources exist: it builds oracle/_ref/libphoton_ref.so
(which holds the reference's pbrt_parser.cpp, ply_reader.cpp,
pbrt_to_photon.cpp and image_loader.cpp next to its path tracer) and records,
for each scene of tests/golden/pbrt/ (made by make_scenes.py):

  <case>/counts          sizes of the parsed and converted scene
  <case>/sha_<array>     SHA-256 of the converted mesh arrays (positions,
                         normals, texcoords, material ids: three vertices per
                         triangle), of the materials (phc_pt_material
                         records), textures and environment
  <case>/camera          pt::Camera origin, lower_left, horizontal, vertical,
                         u, v, w, lens radius, focus distance
  <case>/render          PathTracer::render of the converted scene at a small
                         size (spp 4, adaptive off, bottom-up rows as the
                         bridge renders), for per-sample comparisons

    python tests/golden/make_pbrt_golden.py
"""
from __future__ import annotations

import hashlib
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

import oracle  # noqa: E402

# (case, file, use_instancing, width, height, spp)
CASES = [
    ("box_room", "box_room.pbrt", False, 48, 48, 4),
    ("features", "features.pbrt", False, 72, 48, 4),
    ("features_ias", "features.pbrt", True, 72, 48, 4),
]


def sha(a) -> str:
    return hashlib.sha256(np.ascontiguousarray(a).tobytes()).hexdigest()


def material_bytes(mats) -> bytes:
    return b"".join(bytes(m) for m in mats)


def digest(arrs) -> dict:
    out = {k: sha(arrs[k]) for k in ("positions", "normals", "texcoords", "material_ids")}
    out["materials"] = hashlib.sha256(material_bytes(arrs["materials"])).hexdigest()
    out["textures"] = sha(np.concatenate([t.ravel() for t in arrs["textures"]])) if arrs["textures"] else sha(
        np.zeros(0, np.float32))
    env = arrs["env"]
    out["env"] = sha(np.concatenate([env[k].ravel() for k in ("pixels", "world_to_map", "map_to_world")])) \
        if env is not None else sha(np.zeros(0, np.float32))
    return out


def main():
    oracle.build(ref=True)
    data = {}
    for case, fname, ias, w, h, spp in CASES:
        path = os.path.join(HERE, "pbrt", fname)
        full = oracle.RefPbrt(path, use_instancing=ias)
        arrs = full.arrays()
        data[f"{case}/counts_names"] = np.array(oracle.RefPbrt.COUNTS)
        data[f"{case}/counts"] = np.array([full.counts[k] for k in oracle.RefPbrt.COUNTS], np.int64)
        for k, v in digest(arrs).items():
            data[f"{case}/sha_{k}"] = np.array(v)
        data[f"{case}/camera"] = arrs["camera"]
        data[f"{case}/emissive_areas"] = arrs["emissive_areas"]
        full.close()
        small = oracle.RefPbrt(path, use_instancing=ias, width=w, height=h, spp=spp)
        data[f"{case}/render"] = small.render(adaptive=False, bottom_up=True)
        data[f"{case}/render_args"] = np.array([w, h, spp, int(ias)], np.int64)
        small.close()
        print(case, full.counts, file=sys.stderr)
    np.savez_compressed(os.path.join(HERE, "pbrt_ref.npz"), **data)


if __name__ == "__main__":
    main()
