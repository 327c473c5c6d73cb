"""Generates the golden fixtures of tests/golden/ from the REFERENCE itself.

Run in a checkout where the reference sources exist: it builds
oracle/_ref/libphoton_ref.so (Photon's own pathtracer.cpp, bvh.cpp,
kokkos_backend.cpp, environment_map.cpp and RenderBridge.cpp compiled against
the project's Kokkos stand-in) and records, through the reference's own
bridge::Renderer and KokkosBackend:

  scene_<name>.npz  the complete scene (arrays + raw C records, so the
                    fixture does not depend on regenerating it), camera and
                    settings, and per frame (spp 1, successive sample offsets)
                    the color / depth / normal / albedo channels;
  trace.npz         a displaced-sphere mesh, seeded rays and the reference's
                    HitResult records and occlusion flags;
  bsdf.npz          Disney BSDF eval / pdf / sample at seeded directions.

    python tests/golden/make_golden.py
"""
from __future__ import annotations

import ctypes as C
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

import oracle  # noqa: E402
from photon_gb300 import _abi, workloads  # noqa: E402

FRAMES = 2
RES = 32


def rec_bytes(recs):
    return np.frombuffer(b"".join(bytes(r) for r in recs), np.uint8) if recs else np.zeros(0, np.uint8)


def save_scene(path, sc, cam, st, frames):
    d = {
        "positions": sc.positions, "indices": sc.indices, "material_ids": sc.material_ids,
        "materials": rec_bytes(sc.materials), "lights": rec_bytes(sc.lights),
        "camera": rec_bytes([cam]), "settings": rec_bytes([st]),
        "env_world_to_map": np.asarray(sc.env_world_to_map, np.float32),
        "env_visible": np.int32(sc.env_visible),
    }
    if sc.normals is not None:
        d["normals"] = sc.normals
    for k, a in enumerate(sc.attributes):
        if a is not None:
            d[f"attr{k}"] = a
    if sc.env_pixels is not None:
        d["env_pixels"] = sc.env_pixels
    d["samplers"] = rec_bytes([s for s, _ in sc.samplers])
    for k, (_, tex) in enumerate(sc.samplers):
        if tex is not None:
            d[f"texels{k}"] = np.asarray(tex, np.float32)
    d["volumes"] = rec_bytes([v for v, _, _ in sc.volumes])
    for k, (_, vals, tf) in enumerate(sc.volumes):
        d[f"vol_values{k}"] = np.asarray(vals, np.float32)
        d[f"vol_tf{k}"] = np.asarray(tf, np.float32)
    bg = getattr(st, "_bg", None)
    if bg is not None:
        d["background_image"] = bg
    for f, ch in enumerate(frames):
        for k, v in ch.items():
            d[f"f{f}_{k}"] = v
    np.savez_compressed(path, **d)


def render_frames(sc, cam, st, frames=FRAMES):
    r = oracle.CpuRenderer("ref")
    r.set_scene(sc)
    out = []
    for _ in range(frames):
        r.render(cam, st, True)
        out.append({ch: r.read(ch) for ch in ("color", "depth", "normal", "albedo")})
    return out


def displaced_sphere(seed=7, subdiv=5):
    v, f = workloads._icosphere(subdiv)
    rng = np.random.default_rng(seed)
    n = v.copy()
    v = workloads._displace(v, n, rng, 0.1)
    return v.astype(np.float32), f.astype(np.uint32)


def main():
    oracle.build(ref=True)
    names = []
    for kind in workloads.FEATURES:
        sc, cam, st = workloads.feature_scene(kind, res=RES)
        st.pixel_samples = 1
        frames = render_frames(sc, cam, st)
        save_scene(os.path.join(HERE, f"scene_{kind}.npz"), sc, cam, st, frames)
        names.append(kind)
    # box room at the image size of the first workload's shape, small
    sc, cam, st = workloads.box_room()
    st.width = st.height = 64
    st.pixel_samples = 1
    save_scene(os.path.join(HERE, "scene_box_room.npz"), sc, cam, st, render_frames(sc, cam, st))
    names.append("box_room")

    # Level-A fixture: rays from a shell around a displaced sphere
    pos, idx = displaced_sphere()
    nrm = workloads._vertex_normals(pos.astype(np.float64), idx.astype(np.int64)).astype(np.float32)
    mid = (np.arange(len(idx)) % 5).astype(np.uint32)
    rng = np.random.default_rng(11)
    n = 2048
    o = rng.normal(size=(n, 3))
    o = (o / np.linalg.norm(o, axis=1, keepdims=True) * rng.uniform(0.5, 3.0, (n, 1))).astype(np.float32)
    tgt = rng.normal(size=(n, 3)) * 0.4
    d = tgt - o
    d = (d / np.linalg.norm(d, axis=1, keepdims=True)).astype(np.float32)
    t0 = np.zeros(n, np.float32)
    t1 = np.full(n, 1e30, np.float32)
    t1[::5] = rng.uniform(0.2, 2.0, len(t1[::5])).astype(np.float32)
    t0[::13] = 1.0
    t1[::13] = 0.0
    hits = oracle.trace("ref", pos, idx, o, d, t0, t1, False, nrm, mid)
    occ = oracle.trace("ref", pos, idx, o, d, t0, t1, True, nrm, mid)
    np.savez_compressed(os.path.join(HERE, "trace.npz"), positions=pos, indices=idx, normals=nrm,
                        material_ids=mid, orgs=o, dirs=d, tmin=t0, tmax=t1,
                        hits=np.frombuffer(hits.tobytes(), np.uint8).reshape(n, 88), occluded=occ)

    # BSDF fixture
    mats = []
    cases = []
    for k, (metal, rough, trans, coat, sheen, spec, thin) in enumerate([
            (0.0, 1.0, 0.0, 0.0, 0.0, 0.5, 0), (1.0, 0.3, 0.0, 0.0, 0.0, 0.5, 0), (0.0, 0.0, 1.0, 0.0, 0.0, 1.0, 0),
            (0.2, 0.6, 0.3, 0.7, 0.5, 0.5, 0), (0.0, 0.5, 1.0, 0.0, 0.0, 0.5, 1), (0.0, 0.02, 0.0, 1.0, 0.0, 0.0, 0)]):
        m = _abi.material_default()
        m.base_color[:] = (0.7, 0.4 + 0.05 * k, 0.2)
        m.metallic, m.roughness, m.transmission, m.clearcoat, m.sheen, m.specular = metal, rough, trans, coat, sheen, spec
        m.thin_walled = thin
        rng = np.random.default_rng(100 + k)
        nn = 256
        ng = np.tile([0, 0, 1.0], (nn, 1)).astype(np.float32)
        ns = ng + rng.normal(size=(nn, 3)) * 0.15
        ns = (ns / np.linalg.norm(ns, axis=1, keepdims=True)).astype(np.float32)
        wo = rng.normal(size=(nn, 3))
        wo[: nn * 3 // 4, 2] = np.abs(wo[: nn * 3 // 4, 2])
        wo = (wo / np.linalg.norm(wo, axis=1, keepdims=True)).astype(np.float32)
        wi = rng.normal(size=(nn, 3))
        wi[:, 2] = np.abs(wi[:, 2])
        wi = (wi / np.linalg.norm(wi, axis=1, keepdims=True)).astype(np.float32)
        seeds = rng.integers(1, 2 ** 32 - 1, nn).astype(np.uint32)
        out, out2 = oracle.bsdf_probe("ref", m, ng, ns, wo, wi, seeds)
        mats.append(m)
        cases.append((ng, ns, wo, wi, seeds, out, out2))
    d = {"materials": rec_bytes(mats)}
    for k, (ng, ns, wo, wi, seeds, out, out2) in enumerate(cases):
        d.update({f"ng{k}": ng, f"ns{k}": ns, f"wo{k}": wo, f"wi{k}": wi, f"seeds{k}": seeds, f"out{k}": out,
                  f"out2{k}": out2})
    np.savez_compressed(os.path.join(HERE, "bsdf.npz"), **d)
    print("wrote", names, "trace.npz bsdf.npz")


if __name__ == "__main__":
    main()
