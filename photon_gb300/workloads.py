"""Seeded synthetic workloads.

The reference's published numbers are on Bitterli pbrt-v4 scenes that are not
available offline; these generators stand in for them with the shapes, sizes
and value ranges of the five workloads the project is measured on:

  box_room          ~36 triangles, 5 diffuse walls, two rotated boxes, a
                    0.25 m^2 quad light of radiance (17, 12, 4); 512^2, 64 spp,
                    depth 8.
  procedural_500k   200 displaced icospheres and tori on a ground plane
                    (~500K triangles), per-object Disney parameters, a
                    1024x512 fp32 sun+sky environment map and 4 emissive
                    triangles; 1024^2, 128 spp, depth 8.
  instanced_2m      ~2M triangles (instances flattened, as the reference
                    does), 12 RGBA8 2048^2 value-noise textures (base colour,
                    roughness, normal maps), emissive meshes and a 256^3 fBm
                    density grid (sigma_t up to 8); 1920^2, 256 spp, depth 12,
                    adaptive sampling.
  batched_jobs      64 independent small renders of uneven size.
  differentiable    50K triangles, 8 textured materials, homogeneous medium.

Geometry and parameters come from numpy's PCG64 with the given seed; the
path sampling itself uses the reference's per-(pixel, sample, dimension)
hash streams, sample offset 0.
"""
from __future__ import annotations

import numpy as np

from . import _abi
from .scene import SceneData, camera, settings

# ----------------------------------------------------------------- primitives


def _quad(p0, p1, p2, p3):
    """Two triangles (p0, p1, p2), (p0, p2, p3)."""
    return np.array([p0, p1, p2, p3], np.float32), np.array([[0, 1, 2], [0, 2, 3]], np.uint32)


def _box(center, size, angle_deg, bottom=True):
    """Axis-aligned box rotated about +y; 10 or 12 triangles."""
    cx, cy, cz = center
    sx, sy, sz = size
    c, s = np.cos(np.deg2rad(angle_deg)), np.sin(np.deg2rad(angle_deg))
    corners = []
    for y in (0.0, sy):
        for (x, z) in ((-sx / 2, -sz / 2), (sx / 2, -sz / 2), (sx / 2, sz / 2), (-sx / 2, sz / 2)):
            corners.append((cx + c * x + s * z, cy + y, cz - s * x + c * z))
    v = np.array(corners, np.float32)
    faces = [
        (4, 7, 6, 5),  # top, normal +y
        (0, 1, 5, 4), (1, 2, 6, 5), (2, 3, 7, 6), (3, 0, 4, 7),  # sides
    ]
    if bottom:
        faces.append((0, 3, 2, 1))
    idx = []
    for a, b, cc, d in faces:
        idx += [[a, b, cc], [a, cc, d]]
    return v, np.array(idx, np.uint32)


class _MeshBuilder:
    def __init__(self):
        self.pos, self.idx, self.mat, self.nrm = [], [], [], []
        self.count = 0
        self.with_normals = False

    def add(self, v, i, mat, n=None):
        self.pos.append(np.asarray(v, np.float32))
        self.idx.append(np.asarray(i, np.uint32) + self.count)
        self.mat.append(np.full(len(i), mat, np.uint32))
        if n is None:
            n = np.zeros_like(v, dtype=np.float32)
        else:
            self.with_normals = True
        self.nrm.append(np.asarray(n, np.float32))
        self.count += len(v)

    def build(self, **kw):
        return SceneData(
            positions=np.concatenate(self.pos), indices=np.concatenate(self.idx),
            material_ids=np.concatenate(self.mat),
            normals=np.concatenate(self.nrm) if self.with_normals else None, **kw)


def diffuse(rgb):
    m = _abi.material_default()
    m.base_color[:] = rgb
    m.roughness = 1.0
    return m


def emitter(radiance, both_sides=False):
    m = _abi.material_default()
    m.base_color[:] = (0.0, 0.0, 0.0)
    m.emission[:] = radiance
    m.emitter_only = 1
    m.emission_side = 2 if both_sides else 0
    return m


# ------------------------------------------------------------------ box room


def box_room():
    """Box room: 5 quads, two rotated boxes, a 0.5 x 0.5 m quad light."""
    mb = _MeshBuilder()
    W = 2.0
    # floor, ceiling, back wall (white); left red; right green
    mb.add(*_quad((-1, 0, -1), (-1, 0, 1), (1, 0, 1), (1, 0, -1)), 0)
    mb.add(*_quad((-1, W, -1), (1, W, -1), (1, W, 1), (-1, W, 1)), 0)
    mb.add(*_quad((-1, 0, -1), (1, 0, -1), (1, W, -1), (-1, W, -1)), 0)
    mb.add(*_quad((-1, 0, -1), (-1, W, -1), (-1, W, 1), (-1, 0, 1)), 1)
    mb.add(*_quad((1, 0, -1), (1, 0, 1), (1, W, 1), (1, W, -1)), 2)
    # the boxes float 1 mm above the floor: no coplanar faces, so no exact
    # distance ties whose winner depends on the traversal order
    mb.add(*_box((-0.33, 1e-3, -0.3), (0.6, 1.2, 0.6), 17.0), 0)
    mb.add(*_box((0.35, 1e-3, 0.3), (0.6, 0.6, 0.6), -18.0), 0)
    ly = W - 1e-3
    mb.add(*_quad((-0.25, ly, -0.25), (0.25, ly, -0.25), (0.25, ly, 0.25), (-0.25, ly, 0.25)), 3)
    sc = mb.build(name="box_room")
    sc.materials = [diffuse((0.73, 0.73, 0.73)), diffuse((0.65, 0.05, 0.05)),
                    diffuse((0.12, 0.45, 0.15)), emitter((17.0, 12.0, 4.0))]
    cam = camera((0.0, 1.0, 3.9), (0.0, 1.0, 0.0), fovy_deg=40.0)
    st = settings(512, 512, 64, 8, adaptive_sampling=0, throughput_clamp=0.0)
    return sc, cam, st


# ---------------------------------------------------------- procedural 500K


def _icosphere(subdiv):
    t = (1.0 + 5 ** 0.5) / 2
    v = [(-1, t, 0), (1, t, 0), (-1, -t, 0), (1, -t, 0), (0, -1, t), (0, 1, t), (0, -1, -t), (0, 1, -t),
         (t, 0, -1), (t, 0, 1), (-t, 0, -1), (-t, 0, 1)]
    f = [(0, 11, 5), (0, 5, 1), (0, 1, 7), (0, 7, 10), (0, 10, 11), (1, 5, 9), (5, 11, 4), (11, 10, 2),
         (10, 7, 6), (7, 1, 8), (3, 9, 4), (3, 4, 2), (3, 2, 6), (3, 6, 8), (3, 8, 9), (4, 9, 5), (2, 4, 11),
         (6, 2, 10), (8, 6, 7), (9, 8, 1)]
    v = np.array(v, np.float64)
    v /= np.linalg.norm(v, axis=1, keepdims=True)
    f = np.array(f, np.int64)
    for _ in range(subdiv):
        nv = len(v)
        e = np.concatenate([f[:, [0, 1]], f[:, [1, 2]], f[:, [2, 0]]])
        e.sort(axis=1)
        key = e[:, 0] * nv + e[:, 1]
        uniq, inv = np.unique(key, return_inverse=True)
        a, b = uniq // nv, uniq % nv
        mid = v[a] + v[b]
        mid /= np.linalg.norm(mid, axis=1, keepdims=True)
        m = inv.reshape(3, -1).T + nv  # midpoints of edges (01, 12, 20)
        v = np.concatenate([v, mid])
        f = np.concatenate([
            np.stack([f[:, 0], m[:, 0], m[:, 2]], 1), np.stack([f[:, 1], m[:, 1], m[:, 0]], 1),
            np.stack([f[:, 2], m[:, 2], m[:, 1]], 1), np.stack([m[:, 0], m[:, 1], m[:, 2]], 1)])
    return v, f


def _torus(nu, nv, R, r):
    u = np.arange(nu) * (2 * np.pi / nu)
    w = np.arange(nv) * (2 * np.pi / nv)
    uu, ww = np.meshgrid(u, w, indexing="ij")
    x = (R + r * np.cos(ww)) * np.cos(uu)
    z = (R + r * np.cos(ww)) * np.sin(uu)
    y = r * np.sin(ww)
    v = np.stack([x, y, z], -1).reshape(-1, 3)
    n = np.stack([np.cos(ww) * np.cos(uu), np.sin(ww), np.cos(ww) * np.sin(uu)], -1).reshape(-1, 3)
    i = np.arange(nu)[:, None]
    j = np.arange(nv)[None, :]
    a = (i * nv + j)
    b = (((i + 1) % nu) * nv + j)
    c = (((i + 1) % nu) * nv + (j + 1) % nv)
    d = (i * nv + (j + 1) % nv)
    f = np.concatenate([np.stack([a, c, b], -1).reshape(-1, 3), np.stack([a, d, c], -1).reshape(-1, 3)])
    return v, n, f


def _vertex_normals(v, f):
    fn = np.cross(v[f[:, 1]] - v[f[:, 0]], v[f[:, 2]] - v[f[:, 0]])
    n = np.zeros_like(v)
    for k in range(3):
        np.add.at(n, f[:, k], fn)
    n /= np.maximum(np.linalg.norm(n, axis=1, keepdims=True), 1e-20)
    return n


def _displace(v, n, rng, amp):
    """Radial displacement by a few random sinusoids (smooth, seeded)."""
    d = np.zeros(len(v))
    for _ in range(4):
        k = rng.normal(size=3) * rng.uniform(2.0, 6.0)
        d += np.sin(v @ k + rng.uniform(0, 2 * np.pi)) / 4
    return v + n * (amp * d)[:, None]


def sun_sky_env(width=1024, height=512, sun_dir=(0.35, 0.55, -0.75), seed=0, sun_radiance=(4000.0, 3600.0, 3000.0)):
    """Procedural fp32 sun+sky environment (rows from the bottom, +y up)."""
    sd = np.asarray(sun_dir, np.float64)
    sd /= np.linalg.norm(sd)
    # the reference maps texel (x, y) to phi = u*2pi - pi, theta = v*pi with
    # direction (sin t cos p, cos t, sin t sin p) (environment_map.h:138-155)
    u = (np.arange(width) + 0.5) / width
    vv = (np.arange(height) + 0.5) / height
    phi = u * 2 * np.pi - np.pi
    theta = vv * np.pi
    st = np.sin(theta)[:, None]
    d = np.stack([st * np.cos(phi)[None, :], np.cos(theta)[:, None] * np.ones((1, width)),
                  st * np.sin(phi)[None, :]], -1)
    up = np.clip(d[..., 1], -1, 1)
    zen = np.array([0.25, 0.45, 1.0])
    hor = np.array([0.9, 0.85, 0.75])
    gnd = np.array([0.18, 0.15, 0.12])
    t = np.clip(up, 0, 1)[..., None] ** 0.5
    sky = hor * (1 - t) + zen * t
    sky = np.where(up[..., None] >= 0, sky, gnd * np.ones_like(sky))
    cosang = np.clip(d @ sd, -1, 1)
    halo = np.exp((cosang - 1) * 40.0)[..., None] * np.array([1.0, 0.9, 0.7]) * 2.0
    sun = (cosang > np.cos(np.deg2rad(1.5)))[..., None] * np.asarray(sun_radiance, np.float64)
    img = (sky + halo + sun).astype(np.float32)
    # texel rows here run v = 0 (theta 0, +y) upward in index; the bridge
    # stores row 0 as given, the map looks texel (y, x) up at v = y / height
    return np.ascontiguousarray(img)


def procedural_500k(seed=0, n_objects=200, n_spheres=60, sphere_subdiv=4, torus_res=(36, 19), env_res=(1024, 512)):
    """~500K triangles: displaced icospheres and tori on a ground plane."""
    rng = np.random.default_rng(seed)
    mb = _MeshBuilder()
    mats = []
    G = 40.0
    mb.add(*_quad((-G, 0, -G), (-G, 0, G), (G, 0, G), (G, 0, -G)), 0, n=np.tile([0, 1, 0], (4, 1)))
    ground = _abi.material_default()
    ground.base_color[:] = (0.5, 0.5, 0.5)
    ground.roughness = 0.8
    ground.specular = 0.5
    mats.append(ground)
    sv, sf = _icosphere(sphere_subdiv)
    for k in range(n_objects):
        px, pz = rng.uniform(-18, 18, 2)
        scale = rng.uniform(0.5, 1.6)
        if k < n_spheres:
            v = sv.copy()
            n = sv.copy()
            v = _displace(v, n, rng, 0.12)
            f = sf
            v = v * scale
            v[:, 1] += scale * 1.05
        else:
            R, r = 1.0, rng.uniform(0.25, 0.45)
            v, n, f = _torus(torus_res[0], torus_res[1], R, r)
            v = _displace(v, n, rng, 0.06)
            ang = rng.uniform(0, np.pi)
            ca, sa = np.cos(ang), np.sin(ang)
            rot = np.array([[1, 0, 0], [0, ca, -sa], [0, sa, ca]])
            v = v @ rot.T * scale
            v[:, 1] += (R + r) * scale * abs(sa) + r * scale + 0.02
        v[:, 0] += px
        v[:, 2] += pz
        nn = _vertex_normals(v, f)
        mb.add(v.astype(np.float32), f, len(mats), n=nn.astype(np.float32))
        m = _abi.material_default()
        m.base_color[:] = rng.uniform(0.05, 0.95, 3).tolist()
        m.metallic = float(rng.integers(0, 2))
        m.roughness = float(rng.uniform(0.05, 1.0))
        m.transmission = 1.0 if rng.uniform() < 0.1 else 0.0
        m.clearcoat = float(rng.uniform(0, 1))
        m.specular = 0.5
        mats.append(m)
    # 4 emissive triangles above the scene
    for k in range(4):
        cx, cz = rng.uniform(-12, 12, 2)
        y = rng.uniform(9, 12)
        s = 1.5
        tri = np.array([[cx - s, y, cz - s], [cx + s, y, cz - s], [cx, y, cz + s]], np.float32)
        mb.add(tri[[0, 2, 1]], np.array([[0, 1, 2]]), len(mats), n=np.tile([0, -1, 0], (3, 1)))
        mats.append(emitter((30.0, 28.0, 24.0)))
    sc = mb.build(name="procedural_500k")
    sc.materials = mats
    sc.env_pixels = sun_sky_env(*env_res)
    cam = camera((0.0, 9.0, 30.0), (0.0, 0.5, 0.0), fovy_deg=45.0)
    st = settings(1024, 1024, 128, 8, adaptive_sampling=0, throughput_clamp=0.0)
    return sc, cam, st


# ----------------------------------------------------------- batched jobs


def batched_jobs(seed=0, n=64, min_tris=1_000, max_tris=200_000, min_res=128, max_res=1024, spp=(4, 64),
                 depth=(4, 12)):
    """n independent renders: procedural scenes of log-uniform triangle
    counts, square resolutions log-uniform in [min_res, max_res], samples per
    pixel and depths uniform in the given ranges.  Returns a list of
    (SceneData, camera, settings)."""
    rng = np.random.default_rng(seed)
    jobs = []
    for k in range(n):
        tris = float(np.exp(rng.uniform(np.log(min_tris), np.log(max_tris))))
        n_obj = 24
        budget = tris / n_obj
        subdiv = int(np.clip(np.round(np.log(max(budget, 20) / 20.0) / np.log(4.0)), 0, 5))
        nu = int(np.clip(np.sqrt(budget), 3, 80))
        nv = int(np.clip(budget / (2 * nu), 3, 80))
        res = int(np.exp(rng.uniform(np.log(min_res), np.log(max_res))))
        sc, cam, st = procedural_500k(seed=1000 + k, n_objects=n_obj, n_spheres=n_obj // 2, sphere_subdiv=subdiv,
                                      torus_res=(nu, nv), env_res=(256, 128))
        st.width = st.height = res
        st.pixel_samples = int(rng.integers(spp[0], spp[1] + 1))
        st.max_depth = int(rng.integers(depth[0], depth[1] + 1))
        sc.name = f"job{k}"
        jobs.append((sc, cam, st))
    return jobs


# ------------------------------------------------------------ differentiable


def _lerp_matrix(n, res):
    """(n, res + 1) linear-interpolation weights of n cell-centred samples of
    a lattice with res cells (two non-zeros per row)."""
    x = (np.arange(n) + 0.5) * (res / n)
    i = np.minimum(np.floor(x).astype(np.int64), res - 1)
    f = (x - i).astype(np.float32)
    w = np.zeros((n, res + 1), np.float32)
    w[np.arange(n), i] = 1.0 - f
    w[np.arange(n), i + 1] += f
    return w


def value_noise(rng, size=512, octaves=(4, 8, 16, 32, 64), channels=4):
    """(size, size, channels) float32 value noise in [0, 1]: random lattices
    of the given resolutions, bilinearly upsampled (wrapping), summed with
    weights halving per octave."""
    out = np.zeros((size, size, channels), np.float32)
    total = 0.0
    for k, res in enumerate(octaves):
        lat = rng.uniform(0, 1, (res + 1, res + 1, channels)).astype(np.float32)
        lat[res, :] = lat[0, :]
        lat[:, res] = lat[:, 0]
        w = _lerp_matrix(size, res)
        rows = np.tensordot(w, lat, axes=(1, 0))                     # (size, res + 1, ch)
        img = np.tensordot(rows, w, axes=(1, 1)).transpose(0, 2, 1)  # (size, size, ch)
        out += np.float32(0.5 ** k) * img
        total += 0.5 ** k
    return out / np.float32(total)


DIFF_MATERIALS = 8
DIFF_TEXTURE = 512


def differentiable(seed=0, res=256, spp=64, depth=6, texture=DIFF_TEXTURE, target=False, param_textures=False):
    """Differentiable workload: ~50K triangles of displaced icospheres and tori
    on a ground plane, 8 materials whose base colour is a texture x texture
    fp32 value-noise image (sampler i for material i, uv in attribute 0) with
    scalar roughness / metallic / specTrans / sheen / clearcoat, a soft sky
    environment and a homogeneous box medium (constant transfer function of
    albedo 0.8, density scale 0.5).  target=True gives the perturbed
    parameters a reference image is rendered from.  param_textures=True
    also reads roughness (materials 0-3), metallic (4-6) and specTrans (7)
    from texture x texture value-noise images (channel r; samplers 8-15).
    Returns (SceneData, camera, settings)."""
    rng = np.random.default_rng(seed)
    mb = _MeshBuilder()
    uvs = []
    G = 12.0
    gv, gf = _quad((-G, 0, -G), (-G, 0, G), (G, 0, G), (G, 0, -G))
    mb.add(gv, gf, 0, n=np.tile([0, 1, 0], (4, 1)))
    uvs.append(np.stack([gv[:, 0] / 6.0, gv[:, 2] / 6.0], -1))
    sv, sf = _icosphere(3)
    for k in range(40):
        px, pz = rng.uniform(-8, 8, 2)
        scale = rng.uniform(0.5, 1.3)
        if k < 20:
            n = sv.copy()
            v = _displace(sv.copy(), n, rng, 0.1) * scale
            f = sf
            uv = np.stack([np.arctan2(sv[:, 2], sv[:, 0]) / (2 * np.pi) + 0.5, np.arccos(np.clip(sv[:, 1], -1, 1)) / np.pi],
                          -1)
            v[:, 1] += scale * 1.05
        else:
            R, r = 1.0, rng.uniform(0.25, 0.4)
            nu, nv = 36, 17
            v, n, f = _torus(nu, nv, R, r)
            v = _displace(v, n, rng, 0.05)
            ang = rng.uniform(0, np.pi)
            ca, sa = np.cos(ang), np.sin(ang)
            v = v @ np.array([[1, 0, 0], [0, ca, -sa], [0, sa, ca]]).T * scale
            v[:, 1] += (R + r) * scale * abs(sa) + r * scale + 0.02
            uu, ww = np.meshgrid(np.arange(nu) / nu, np.arange(nv) / nv, indexing="ij")
            uv = np.stack([uu.reshape(-1) * 2.0, ww.reshape(-1)], -1)
        v[:, 0] += px
        v[:, 2] += pz
        mb.add(v.astype(np.float32), f, k % DIFF_MATERIALS, n=_vertex_normals(v, f).astype(np.float32))
        uvs.append(uv)
    sc = mb.build(name="differentiable")
    attr = np.zeros((sc.positions.shape[0], 4), np.float32)
    attr[:, :2] = np.concatenate(uvs)
    attr[:, 3] = 1.0
    sc.attributes = [attr, None, None, None, None]
    prng = np.random.default_rng(seed + 7)
    mats, samplers = [], []
    for i in range(DIFF_MATERIALS):
        tint = prng.uniform(0.25, 0.9, 3)
        tex = value_noise(prng, texture)
        tex[..., :3] = np.clip(tex[..., :3] * 0.6 + 0.4 * tint, 0, 1)
        tex[..., 3] = 1.0
        m = _abi.material_default()
        m.base_color[:] = (1.0, 1.0, 1.0)
        m.base_color_src.kind, m.base_color_src.index = 2, i
        m.roughness = float(prng.uniform(0.3, 0.8))
        m.metallic = float(prng.uniform(0.05, 0.5))
        m.transmission = float(prng.uniform(0.05, 0.3)) if i % 4 == 3 else 0.0
        m.sheen = float(prng.uniform(0.1, 0.6))
        m.clearcoat = float(prng.uniform(0.1, 0.6))
        m.specular = 0.5
        s = _abi.sampler_default()
        s.type = 1
        s.in_attribute = 0
        s.linear = 1
        s.wrap[:] = (1, 1, 0)
        s.size[:] = (texture, texture, 1)
        mats.append(m)
        samplers.append((s, tex.reshape(-1, 4)))
    vol = _abi.volume_default()
    vol.dims[:] = (2, 2, 2)
    vol.origin[:] = (-6.0, 0.0, -6.0)
    vol.spacing[:] = (12.0, 3.0, 12.0)
    vol.value_range[:] = (0.0, 1.0)
    vol.density_scale = 0.5
    albedo = np.array([0.8, 0.8, 0.8], np.float32)
    if target:
        trng = np.random.default_rng(seed + 99)
        for m, (s, tex) in zip(mats, samplers):
            m.roughness = float(np.clip(m.roughness + trng.uniform(-0.15, 0.15), 0.05, 1.0))
            m.metallic = float(np.clip(m.metallic + trng.uniform(-0.1, 0.1), 0.0, 1.0))
            m.sheen = float(np.clip(m.sheen + trng.uniform(-0.1, 0.1), 0.0, 1.0))
            m.clearcoat = float(np.clip(m.clearcoat + trng.uniform(-0.1, 0.1), 0.0, 1.0))
            if m.transmission > 0:
                m.transmission = float(np.clip(m.transmission + trng.uniform(-0.05, 0.05), 0.0, 1.0))
            tex[:, :3] = np.clip(tex[:, :3] * trng.uniform(0.8, 1.2, 3).astype(np.float32), 0, 1)
        vol.density_scale = 0.5 * float(trng.uniform(0.8, 1.2))
        albedo = np.clip(albedo * trng.uniform(0.9, 1.1, 3), 0, 1).astype(np.float32)
    tf = np.array([list(albedo) + [1.0], list(albedo) + [1.0]], np.float32)
    if param_textures:
        xrng = np.random.default_rng(seed + 13)
        for i, m in enumerate(mats):
            field, lo, hi = (("roughness_src", 0.25, 0.85) if i < 4 else
                             ("metallic_src", 0.05, 0.5) if i < 7 else ("transmission_src", 0.05, 0.3))
            tex = np.zeros((texture, texture, 4), np.float32)
            tex[..., 0] = lo + (hi - lo) * value_noise(xrng, texture)[..., 0]
            tex[..., 3] = 1.0
            s = _abi.sampler_default()
            s.type = 1
            s.in_attribute = 0
            s.linear = 1
            s.wrap[:] = (1, 1, 0)
            s.size[:] = (texture, texture, 1)
            src = getattr(m, field)
            src.kind, src.index = 2, len(samplers)
            samplers.append((s, tex.reshape(-1, 4)))
    sc.materials = mats
    sc.samplers = samplers
    sc.volumes = [(vol, np.ones(8, np.float32), tf)]
    sc.env_pixels = sun_sky_env(256, 128, sun_radiance=(0.0, 0.0, 0.0))
    cam = camera((0.0, 7.0, 17.0), (0.0, 0.8, 0.0), fovy_deg=45.0)
    st = settings(res, res, spp, depth, adaptive_sampling=0, throughput_clamp=0.0)
    return sc, cam, st


# ------------------------------------------------------------- instanced 2M


def fbm_volume(rng, n=256, octaves=(8, 16, 32, 64), gain=0.5):
    """(n, n, n) float32 fBm noise in [0, 1], indexed [z, y, x] (x fastest
    when flattened): random lattices trilinearly upsampled, summed with
    weights falling by `gain` per octave."""
    out = np.zeros((n, n, n), np.float32)
    total = 0.0
    for k, res in enumerate(octaves):
        lat = rng.uniform(0, 1, (res + 1, res + 1, res + 1)).astype(np.float32)
        w = _lerp_matrix(n, res)
        a = np.tensordot(w, lat, axes=(1, 0))                        # (n, r, r)
        a = np.tensordot(a, w, axes=(2, 1))                          # (n, r, n)
        a = np.tensordot(a, w, axes=(1, 1)).transpose(0, 2, 1)       # (n, n, n)
        out += np.float32(gain ** k) * a
        total += gain ** k
    return out / np.float32(total)


def _rot(rng):
    q = rng.normal(size=4)
    q /= np.linalg.norm(q)
    w, x, y, z = q
    return np.array([[1 - 2 * (y * y + z * z), 2 * (x * y - z * w), 2 * (x * z + y * w)],
                     [2 * (x * y + z * w), 1 - 2 * (x * x + z * z), 2 * (y * z - x * w)],
                     [2 * (x * z - y * w), 2 * (y * z + x * w), 1 - 2 * (x * x + y * y)]])


def instanced_2m(seed=0, res=1920, spp=256, depth=12, tex_res=2048, grid=256, n_instances=400, adaptive=1):
    """~2M triangles: two base meshes (displaced icosphere, torus) instanced
    n_instances times with random rotations, scales and positions and
    flattened into one mesh (as the reference flattens instances); 4 textured
    materials, each with an RGBA8 value-noise base-colour, roughness and
    normal map (12 textures of tex_res^2, stored as the 8-bit values / 255 in
    fp32); 6 emissive instances; a grid^3 fp32 fBm density volume whose
    transfer function ramps opacity 0 -> 1 (density scale 8: sigma_t up to 8)
    over part of the scene; a dim sky.  1920^2, 256 spp, depth 12, adaptive
    sampling on."""
    rng = np.random.default_rng(seed)
    sv, sf = _icosphere(4)
    sv = _displace(sv.copy(), sv.copy(), rng, 0.08)
    s_uv = np.stack([np.arctan2(sv[:, 2], sv[:, 0]) / (2 * np.pi) + 0.5,
                     np.arccos(np.clip(sv[:, 1] / np.linalg.norm(sv, axis=1), -1, 1)) / np.pi], -1)
    nu, nv = 72, 36
    tv, tn, tf = _torus(nu, nv, 1.0, 0.35)
    uu, ww = np.meshgrid(np.arange(nu) / nu, np.arange(nv) / nv, indexing="ij")
    t_uv = np.stack([uu.reshape(-1) * 3.0, ww.reshape(-1)], -1)
    bases = [(sv, sf, s_uv, _vertex_normals(sv, sf)), (tv, tf, t_uv, _vertex_normals(tv, tf))]
    mb = _MeshBuilder()
    uvs = []
    G = 30.0
    gv, gf = _quad((-G, 0, -G), (-G, 0, G), (G, 0, G), (G, 0, -G))
    mb.add(gv, gf, 0, n=np.tile([0, 1, 0], (4, 1)))
    uvs.append(np.stack([gv[:, 0] / 4.0, gv[:, 2] / 4.0], -1))
    for k in range(n_instances):
        v, f, uv, vn = bases[k % 2]
        R = _rot(rng)
        scale = rng.uniform(0.4, 1.2)
        pos = np.array([rng.uniform(-22, 22), 0.0, rng.uniform(-22, 22)])
        vw = (v @ R.T) * scale
        pos[1] = -vw[:, 1].min() + 0.01
        vw = vw + pos
        emissive = k < 6
        mat = 4 if emissive else int(rng.integers(0, 4))
        mb.add(vw.astype(np.float32), f, mat, n=(vn @ R.T).astype(np.float32))  # uniform scale: rotate normals
        uvs.append(uv)
    sc = mb.build(name="instanced_2m")
    attr = np.zeros((sc.positions.shape[0], 4), np.float32)
    attr[:, :2] = np.concatenate(uvs)
    attr[:, 3] = 1.0
    sc.attributes = [attr, None, None, None, None]
    trng = np.random.default_rng(seed + 11)
    mats, samplers = [], []

    def sampler(tex):
        s = _abi.sampler_default()
        s.type = 1
        s.in_attribute = 0
        s.linear = 1
        s.wrap[:] = (1, 1, 0)
        s.size[:] = (tex_res, tex_res, 1)
        q = np.round(np.clip(tex, 0, 1) * 255.0) / 255.0  # RGBA8 values
        samplers.append((s, q.astype(np.float32).reshape(-1, 4)))
        return len(samplers) - 1

    for i in range(4):
        tint = trng.uniform(0.2, 0.9, 3)
        base = value_noise(trng, tex_res, octaves=(4, 16, 64))
        base[..., :3] = base[..., :3] * 0.5 + 0.5 * tint
        base[..., 3] = 1.0
        rough = value_noise(trng, tex_res, octaves=(8, 32))
        rough[..., :3] = rough[..., :1] * 0.8 + 0.1
        nrm = value_noise(trng, tex_res, octaves=(16, 64))
        nrm[..., 0:2] = 0.5 + (nrm[..., 0:2] - 0.5) * 0.6
        nrm[..., 2] = 0.9
        m = _abi.material_default()
        m.base_color_src.kind, m.base_color_src.index = 2, sampler(base)
        m.roughness_src.kind, m.roughness_src.index = 2, sampler(rough)
        m.normal_src.kind, m.normal_src.index = 2, sampler(nrm)
        m.metallic = float(trng.uniform(0.0, 0.6))
        m.specular = 0.5
        m.clearcoat = float(trng.uniform(0.0, 0.5))
        mats.append(m)
    mats.append(emitter((12.0, 10.0, 8.0), both_sides=True))
    sc.materials = mats
    sc.samplers = samplers
    vrng = np.random.default_rng(seed + 23)
    dens = fbm_volume(vrng, grid)
    vol = _abi.volume_default()
    vol.dims[:] = (grid, grid, grid)
    vol.origin[:] = (-18.0, 0.0, -16.0)
    vol.spacing[:] = (20.0 / (grid - 1), 7.0 / (grid - 1), 16.0 / (grid - 1))
    vol.value_range[:] = (0.55, 0.8)
    vol.density_scale = 8.0
    tf = np.array([[0.9, 0.9, 0.95, 0.0], [0.85, 0.8, 0.75, 0.5], [0.8, 0.7, 0.6, 1.0]], np.float32)
    sc.volumes = [(vol, dens.reshape(-1), tf)]
    sc.env_pixels = sun_sky_env(256, 128, sun_radiance=(0.0, 0.0, 0.0)) * np.float32(0.3)
    cam = camera((0.0, 14.0, 40.0), (0.0, 1.0, 0.0), fovy_deg=50.0)
    st = settings(res, res, spp, depth, adaptive_sampling=adaptive, throughput_clamp=0.0)
    st.max_volume_bounces = 6
    return sc, cam, st


# ------------------------------------------------------------ feature scenes


def feature_scene(kind: str, seed=0, res=48):
    """Small scenes that each switch on one part of the reference's shading
    path, for parity tests: 'basic', 'glass', 'env', 'lights', 'volume',
    'textures', 'alpha', 'limits', 'camera'."""
    rng = np.random.default_rng(seed)
    sc, cam, st = box_room()
    st.width = st.height = res
    st.pixel_samples = 1
    mats = list(sc.materials)
    if kind == "basic":
        pass
    elif kind == "glass":
        g = _abi.material_default()
        g.base_color[:] = (0.95, 0.95, 0.95)
        g.transmission = 1.0
        g.roughness = 0.0
        g.ior = 1.5
        g.specular = 1.0
        metal = _abi.material_default()
        metal.base_color[:] = (0.9, 0.7, 0.3)
        metal.metallic = 1.0
        metal.roughness = 0.3
        coat = _abi.material_default()
        coat.base_color[:] = (0.2, 0.3, 0.8)
        coat.clearcoat = 1.0
        coat.sheen = 0.5
        coat.specular = 0.5
        coat.roughness = 0.6
        rough_glass = _abi.material_default()
        rough_glass.transmission = 1.0
        rough_glass.roughness = 0.4
        rough_glass.thin_walled = 1
        mats += [g, metal, coat, rough_glass]
        ids = sc.material_ids.copy()
        ids[10:22] = 4
        ids[22:34] = 5
        ids[np.arange(0, 2)] = 6
        ids[np.arange(4, 6)] = 7
        sc.material_ids = ids
    elif kind == "env":
        sc.env_pixels = sun_sky_env(64, 32, sun_dir=(0.3, 0.5, 0.8))
        # open the room: drop ceiling and right wall
        keep = np.ones(sc.triangle_count, bool)
        keep[2:4] = False
        keep[8:10] = False
        sc.indices = sc.indices[keep]
        sc.material_ids = sc.material_ids[keep]
        ang = 0.6
        sc.env_world_to_map = (np.cos(ang), 0, np.sin(ang), 0, 1, 0, -np.sin(ang), 0, np.cos(ang))
    elif kind == "lights":
        pl = _abi.light_default()
        pl.type = 0
        pl.position[:] = (0.3, 1.7, 0.5)
        pl.color[:] = (1.0, 0.8, 0.6)
        pl.intensity = 2.0
        pl.radius = 0.05
        dl = _abi.light_default()
        dl.type = 1
        dl.direction[:] = (-0.3, -1.0, -0.2)
        dl.intensity = 0.8
        dl.radius = 0.02
        spl = _abi.light_default()
        spl.type = 2
        spl.position[:] = (-0.5, 1.9, 0.8)
        spl.direction[:] = (0.3, -1.0, -0.4)
        spl.intensity = 4.0
        spl.spot_angle = 0.5
        spl.spot_falloff = 0.2
        sc.lights = [pl, dl, spl]
        st.ambient_radiance = 0.3
        st.ambient_color[:] = (0.6, 0.7, 1.0)
    elif kind == "volume":
        n = 24
        g = np.linspace(-1, 1, n)
        x, y, z = np.meshgrid(g, g, g, indexing="ij")
        dens = np.clip(1.0 - np.sqrt(x ** 2 + y ** 2 + z ** 2), 0, 1) + 0.2 * np.sin(5 * x) * np.cos(4 * z)
        vals = np.ascontiguousarray(np.transpose(dens, (2, 1, 0)), dtype=np.float32)  # x fastest
        tf = np.array([[0.9, 0.9, 0.9, 0.0], [0.8, 0.6, 0.4, 0.5], [0.9, 0.3, 0.2, 1.0]], np.float32)
        v = _abi.volume_default()
        v.dims[:] = (n, n, n)
        v.origin[:] = (-0.6, 0.2, -0.4)
        v.spacing[:] = (1.2 / (n - 1),) * 3
        v.value_range[:] = (0.0, 1.0)
        v.density_scale = 4.0
        hv = _abi.volume_default()
        hv.dims[:] = (2, 2, 2)
        hv.origin[:] = (-0.9, 0.05, 0.3)
        hv.spacing[:] = (0.6, 0.5, 0.5)
        hv.density_scale = 1.5
        sc.volumes = [(v, vals, tf), (hv, np.ones(8, np.float32), np.array([[0.8, 0.8, 0.8, 1.0]], np.float32))]
        st.max_volume_bounces = 6
    elif kind == "textures":
        V = sc.positions.shape[0]
        uv = np.zeros((V, 4), np.float32)
        uv[:, 0] = sc.positions[:, 0] * 0.7 + sc.positions[:, 2] * 0.3
        uv[:, 1] = sc.positions[:, 1] * 0.6 + sc.positions[:, 2] * 0.2
        uv[:, 3] = 1.0
        sc.attributes = [uv, None, None, None, None]
        col = np.zeros((V, 4), np.float32)
        col[:, :3] = rng.uniform(0.2, 0.9, (V, 3))
        col[:, 3] = 1.0
        sc.attributes[4] = col
        tex = rng.uniform(0, 1, (16, 16, 4)).astype(np.float32)
        s0 = _abi.sampler_default()
        s0.size[:] = (16, 16, 1)
        s0.wrap[:] = (1, 2, 0)
        s1 = _abi.sampler_default()
        s1.type = 1
        s1.linear = 0
        s1.size[:] = (8, 8, 1)
        nrm = np.zeros((8, 8, 4), np.float32)
        nrm[..., 0] = 0.5 + 0.3 * np.sin(np.arange(8))[None, :]
        nrm[..., 1] = 0.5 + 0.3 * np.cos(np.arange(8))[:, None]
        nrm[..., 2] = 0.9
        nrm[..., 3] = 1
        s2 = _abi.sampler_default()
        s2.type = 3
        s2.in_attribute = 4
        s2.out_transform[:] = (0.5, 0, 0, 0, 0, 0.5, 0, 0, 0, 0, 0.5, 0, 0, 0, 0, 1)
        s2.out_offset[:] = (0.1, 0.1, 0.1, 0)
        s3 = _abi.sampler_default()
        s3.type = 0
        s3.size[:] = (5, 1, 1)
        s3.wrap[0] = 2
        s3.in_attribute = 5
        ramp = np.stack([np.linspace(0, 1, 5)] * 4, -1).astype(np.float32)
        s4 = _abi.sampler_default()
        s4.type = 2
        s4.size[:] = (3, 3, 3)
        s4.in_attribute = 5
        s4.in_transform[:] = (0.5, 0, 0, 0.5, 0, 0.5, 0, 0, 0, 0, 0.5, 0.5, 0, 0, 0, 1)
        vol = rng.uniform(0, 1, (27, 4)).astype(np.float32)
        sc.samplers = [(s0, tex), (s1, nrm), (s2, None), (s3, ramp), (s4, vol)]
        m_tex = diffuse((1, 1, 1))
        m_tex.base_color_src.kind, m_tex.base_color_src.index = 2, 0
        m_tex.normal_src.kind, m_tex.normal_src.index = 2, 1
        m_tex.roughness_src.kind, m_tex.roughness_src.index = 2, 3
        m_tex.specular = 0.5
        m_vc = diffuse((1, 1, 1))
        m_vc.base_color_src.kind, m_vc.base_color_src.index = 1, 4
        m_vc.metallic_src.kind, m_vc.metallic_src.index = 2, 4
        m_vc.roughness = 0.5
        m_tr = diffuse((1, 1, 1))
        m_tr.base_color_src.kind, m_tr.base_color_src.index = 2, 2
        m_em = emitter((0, 0, 0))
        m_em.emitter_only = 0
        m_em.emission_src.kind, m_em.emission_src.index = 2, 2
        mats += [m_tex, m_vc, m_tr, m_em]
        ids = sc.material_ids.copy()
        ids[0:2] = 4
        ids[4:6] = 4
        ids[10:22] = 5
        ids[22:34] = 6
        ids[2:4] = 7
        sc.material_ids = ids
    elif kind == "alpha":
        m_blend = diffuse((0.2, 0.8, 0.3))
        m_blend.alpha_mode = 0
        m_blend.opacity = 0.4
        m_mask = diffuse((0.8, 0.2, 0.3))
        m_mask.alpha_mode = 2
        m_mask.opacity = 0.3
        m_mask.alpha_cutoff = 0.5
        m_hidden = diffuse((0.9, 0.9, 0.2))
        m_hidden.hidden_to_camera = 1
        mats += [m_blend, m_mask, m_hidden]
        ids = sc.material_ids.copy()
        ids[10:22] = 4
        ids[22:28] = 5
        ids[28:34] = 6
        sc.material_ids = ids
        st.background[:] = (0.1, 0.2, 0.3, 0.5)
    elif kind == "limits":
        st.max_diffuse_bounces = 1
        st.max_glossy_bounces = 2
        st.clamp_direct = 0.5
        st.clamp_indirect = 0.2
        st.throughput_clamp = 3.0
        st.max_depth = 4
        metal = _abi.material_default()
        metal.base_color[:] = (0.9, 0.9, 0.9)
        metal.metallic = 1.0
        metal.roughness = 0.2
        mats.append(metal)
        ids = sc.material_ids.copy()
        ids[22:34] = 4
        sc.material_ids = ids
    elif kind == "camera":
        cam.aperture_radius = 0.05
        cam.focus_distance = 3.5
        cam.clip_near = 1.0
        cam.clip_far = 4.5
        cam.image_region[:] = (0.1, 0.2, 0.9, 0.8)
    elif kind == "ortho":
        cam.orthographic = 1
        cam.height = 2.2
        bg = rng.uniform(0, 1, (4, 6, 4)).astype(np.float32)
        st._bg = bg
        st.background_width = 6
        st.background_height = 4
        import ctypes as C
        st.background_image = bg.ctypes.data_as(C.POINTER(C.c_float))
        keep = np.ones(sc.triangle_count, bool)
        keep[4:6] = False
        sc.indices = sc.indices[keep]
        sc.material_ids = sc.material_ids[keep]
    else:
        raise ValueError(kind)
    sc.materials = mats
    sc.name = "feature_" + kind
    return sc, cam, st


FEATURES = ("basic", "glass", "env", "lights", "volume", "textures", "alpha", "limits", "camera", "ortho")


# ------------------------------------------------------- instanced objects

def _pt_material(base=(0.8, 0.8, 0.8), roughness=0.5, metallic=0.0, transmission=0.0, ior=1.5, clearcoat=0.0,
                 emission=(0.0, 0.0, 0.0), strength=0.0, base_tex=-1, flags=0):
    """pt::Material record (material.h:35-82 defaults) for PtData scenes."""
    m = _abi.PtMaterial()
    m.base_color[:] = base
    m.metallic, m.roughness, m.ior, m.transmission = metallic, roughness, ior, transmission
    m.specular, m.clearcoat, m.clearcoat_roughness, m.sheen, m.alpha = 0.5, clearcoat, 0.03, 0.0, 1.0
    m.emission[:] = emission
    m.emission_strength = strength
    m.flags, m.base_color_tex, m.alpha_tex = flags, base_tex, -1
    return m


def _random_placement(rng, extent, scale_range):
    """Column-major object-to-world matrix: random rotation, non-uniform
    scale, translation on the ground area."""
    q = rng.normal(size=4)
    q /= np.linalg.norm(q)
    w, x, y, z = q
    R = np.array([[1 - 2 * (y * y + z * z), 2 * (x * y - z * w), 2 * (x * z + y * w)],
                  [2 * (x * y + z * w), 1 - 2 * (x * x + z * z), 2 * (y * z - x * w)],
                  [2 * (x * z - y * w), 2 * (y * z + x * w), 1 - 2 * (x * x + y * y)]])
    S = np.diag(rng.uniform(*scale_range, 3))
    M = np.eye(4)
    M[:3, :3] = R @ S
    M[:3, 3] = (rng.uniform(-extent, extent), rng.uniform(0.3, 1.2), rng.uniform(-extent, extent))
    return M.T.ravel().astype(np.float32)  # column-major


def instanced_objects(seed=0, n_instances=60, res=128, spp=4, depth=6, flatten=False, sphere_subdiv=3):
    """A ground plane and an area light (the scene's own triangles) with
    `n_instances` placements of four objects (a smooth icosphere, a torus, a
    box without normals, a displaced sphere) under random rotations,
    non-uniform scales and translations; path-tracer-level materials.
    flatten=True returns the same geometry with every placement transformed
    into the scene's triangles (float64 transform, then float32), the
    reference's single-level handling of instances."""
    from .scene import PtData
    rng = np.random.default_rng(seed)
    objs = []
    v, f = _icosphere(sphere_subdiv)
    objs.append(dict(positions=0.3 * v, indices=f, normals=v, material_id=1))
    v, n, f = _torus(32, 16, 0.3, 0.1)
    objs.append(dict(positions=v, indices=f, normals=n, material_id=2))
    bv, bi = _box((0.0, -0.2, 0.0), (0.4, 0.4, 0.4), 0.0)
    objs.append(dict(positions=bv, indices=bi, normals=None, material_id=3))
    v, f = _icosphere(sphere_subdiv)
    vn = v.copy()
    v = 0.25 * v * (1.0 + 0.15 * np.sin(7 * v[:, :1]) * np.cos(5 * v[:, 2:3]))
    objs.append(dict(positions=v, indices=f, normals=_vertex_normals(v, f), material_id=4))
    insts = [(int(rng.integers(0, len(objs))), _random_placement(rng, 2.5, (0.6, 1.6)))
             for _ in range(n_instances)]
    mats = [_pt_material((0.7, 0.7, 0.7), roughness=1.0),
            _pt_material((0.7, 0.15, 0.1), roughness=0.6),
            _pt_material((1.0, 0.78, 0.34), roughness=0.25, metallic=1.0),
            _pt_material((1.0, 1.0, 1.0), roughness=0.05, transmission=1.0, ior=1.45, flags=8),
            _pt_material((0.2, 0.4, 0.7), roughness=0.4, clearcoat=1.0),
            _pt_material((0.0, 0.0, 0.0), roughness=1.0, emission=(12.0, 11.0, 9.0), strength=1.0)]
    pos = [np.array([(-4, 0, -4), (4, 0, -4), (4, 0, 4), (-4, 0, 4)], np.float64),
           np.array([(-0.6, 3.0, -0.6), (0.6, 3.0, -0.6), (0.6, 3.0, 0.6), (-0.6, 3.0, 0.6)], np.float64)]
    idx = [np.array([[0, 2, 1], [0, 3, 2]]), np.array([[0, 1, 2], [0, 2, 3]])]
    mid = [np.zeros(2, np.uint32), np.full(2, 5, np.uint32)]
    nrm = [np.tile([0.0, 1.0, 0.0], (4, 1)), np.tile([0.0, -1.0, 0.0], (4, 1))]
    pt = PtData(materials=mats)
    if flatten:
        for oid, xf in insts:
            ob = objs[oid]
            M = np.asarray(xf, np.float64).reshape(4, 4).T
            p = np.asarray(ob["positions"], np.float64)
            pw = p @ M[:3, :3].T + M[:3, 3]
            pos.append(pw)
            idx.append(np.asarray(ob["indices"]))
            mid.append(np.full(len(ob["indices"]), ob["material_id"], np.uint32))
            if ob["normals"] is not None:
                nw = np.asarray(ob["normals"], np.float64) @ np.linalg.inv(M[:3, :3])
                nw /= np.maximum(np.linalg.norm(nw, axis=1, keepdims=True), 1e-30)
            else:  # no normals: zero vectors, for which shading uses the geometric normal
                nw = np.zeros_like(pw)
            nrm.append(nw)
    else:
        pt.objects = objs
        pt.instances = insts
    off = np.cumsum([0] + [len(p) for p in pos[:-1]])
    sc = SceneData(positions=np.concatenate(pos).astype(np.float32),
                   indices=np.concatenate([i + o for i, o in zip(idx, off)]).astype(np.uint32),
                   material_ids=np.concatenate(mid), normals=np.concatenate(nrm).astype(np.float32),
                   name="instanced_objects" + ("_flat" if flatten else ""), pt=pt)
    cam = camera((0.0, 2.6, 6.5), (0.0, 0.6, 0.0), fovy_deg=45.0)
    st = settings(res, res, spp, depth, adaptive_sampling=0)
    return sc, cam, st
