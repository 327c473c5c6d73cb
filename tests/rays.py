"""Seeded ray batches of a workload, built on the CPU (numpy) for the Level-A
parity tests: one jittered pinhole camera ray per pixel, and cosine-weighted
bounce rays about the geometric normal at hit points that the oracle found.
"""
from __future__ import annotations

import numpy as np


def camera_rays(cam, width, height, seed=1):
    """One jittered ray per pixel of a pinhole camera (position, direction,
    up, fovy, aspect of a phc_camera); origins, unit directions, tmin 0,
    tmax 1e30."""
    rng = np.random.default_rng(seed)
    fwd = np.asarray(cam.direction[:], np.float64)
    fwd /= np.linalg.norm(fwd)
    up = np.asarray(cam.up[:], np.float64)
    right = np.cross(fwd, up)
    right /= np.linalg.norm(right)
    tup = np.cross(right, fwd)
    th = np.tan(0.5 * cam.fovy)
    aspect = cam.aspect if cam.aspect > 0 else width / height
    py, px = np.mgrid[0:height, 0:width].astype(np.float64)
    sx = (2.0 * (px + rng.random(px.shape)) / width - 1.0) * th * aspect
    sy = (2.0 * (py + rng.random(py.shape)) / height - 1.0) * th
    d = fwd[None] + sx.reshape(-1, 1) * right[None] + sy.reshape(-1, 1) * tup[None]
    d /= np.linalg.norm(d, axis=1, keepdims=True)
    n = d.shape[0]
    o = np.broadcast_to(np.asarray(cam.position[:], np.float32), (n, 3)).copy()
    return (o, d.astype(np.float32), np.zeros(n, np.float32), np.full(n, 1e30, np.float32))


def bounce_rays(records, dirs, scale, seed=2):
    """Cosine-weighted directions about the geometric normal (turned toward
    the incoming ray) at the hit points of `records` (88-byte HitResult
    records), origins offset by 1e-4 * scale along that normal."""
    rng = np.random.default_rng(seed)
    h = records["hit"].astype(bool)
    pos = records["position"][h].astype(np.float64)
    ng = records["normal"][h].astype(np.float64)
    ng = np.where((np.sum(ng * dirs[h], 1) > 0)[:, None], -ng, ng)
    m = len(pos)
    u1, u2 = rng.random(m), rng.random(m)
    r, phi = np.sqrt(u1), 2.0 * np.pi * u2
    a = np.where(np.abs(ng[:, :1]) > 0.9, np.array([[0.0, 1.0, 0.0]]), np.array([[1.0, 0.0, 0.0]]))
    t1 = np.cross(ng, a)
    t1 /= np.linalg.norm(t1, axis=1, keepdims=True)
    t2 = np.cross(ng, t1)
    bd = (r * np.cos(phi))[:, None] * t1 + (r * np.sin(phi))[:, None] * t2 + np.sqrt(1 - u1)[:, None] * ng
    bd /= np.linalg.norm(bd, axis=1, keepdims=True)
    bo = pos + 1e-4 * scale * ng
    return (bo.astype(np.float32), bd.astype(np.float32), np.zeros(m, np.float32), np.full(m, 1e30, np.float32))
