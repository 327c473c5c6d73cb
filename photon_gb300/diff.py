"""torch.autograd wrapper over the path-replay adjoint (phc_adjoint).

The reference has no derivatives; this is the differentiable-rendering layer
of the GB300 path tracer.  A DiffScene holds a SceneData and a Renderer and
maps three parameter tensors onto the scene:

  materials (M, 8)  base colour r, g, b, roughness (the bridge's perceptual
                    roughness), metallic, specTrans, sheen, clearcoat
  texels    (T, 4)  the texels of every sampler, concatenated in sampler order
  volumes   (V, 4)  density scale, albedo r, g, b (a constant transfer-function
                    colour; the transfer function's opacity is kept)

render(ds, materials, texels, volumes) is the image (h, w, 3), row 0 the
bottom row, of settings.pixel_samples fresh samples; its backward pass runs
phc_adjoint with adjoint_spp samples on a sample range of its own (decorrelated
from the forward samples) and returns the three gradients.
"""
from __future__ import annotations

import numpy as np
import torch

from . import _abi
from .renderer import Renderer

MATERIAL_FIELDS = _abi.ADJ_MATERIAL_NAMES
ADJOINT_SAMPLE_BASE = 1 << 28


class DiffScene:
    def __init__(self, scene, camera, settings, adjoint_spp=16, renderer=None):
        self.scene = scene
        self.camera = camera
        self.settings = settings
        self.adjoint_spp = int(adjoint_spp)
        self.renderer = renderer or Renderer()
        self._adj_offset = ADJOINT_SAMPLE_BASE
        self.texel_counts = [0 if t is None else int(np.asarray(t).reshape(-1, 4).shape[0])
                             for _, t in scene.samplers]
        self.last_adjoint_ms = 0.0
        self.last_forward_ms = 0.0

    # ----------------------------------------------------------- parameters
    def params(self):
        """Current parameters as float32 tensors (materials, texels, volumes)."""
        mats = np.array([[m.base_color[0], m.base_color[1], m.base_color[2], m.roughness, m.metallic,
                          m.transmission, m.sheen, m.clearcoat] for m in self.scene.materials], np.float32)
        tex = [np.asarray(t, np.float32).reshape(-1, 4) for _, t in self.scene.samplers if t is not None]
        tex = np.concatenate(tex) if tex else np.zeros((0, 4), np.float32)
        vols = np.array([[v.density_scale, *np.asarray(tf, np.float32).reshape(-1, 4)[0, :3]]
                         for v, _, tf in self.scene.volumes], np.float32).reshape(-1, 4)
        return torch.from_numpy(mats), torch.from_numpy(tex.copy()), torch.from_numpy(vols)

    def apply(self, materials, texels, volumes):
        """Writes the parameters into the scene and uploads it."""
        mats = _np(materials)
        for m, p in zip(self.scene.materials, mats):
            m.base_color[:] = p[0:3].tolist()
            m.roughness, m.metallic, m.transmission, m.sheen, m.clearcoat = (float(x) for x in p[3:8])
        tex = _np(texels)
        if tex.size:
            off = 0
            recs = []
            for (rec, t), n in zip(self.scene.samplers, self.texel_counts):
                if t is None:
                    recs.append((rec, None))
                    continue
                recs.append((rec, np.ascontiguousarray(tex[off:off + n])))
                off += n
            self.scene.samplers = recs
        vols = _np(volumes)
        recs = []
        for (v, vals, tf), p in zip(self.scene.volumes, vols):
            v.density_scale = float(p[0])
            tf = np.array(tf, np.float32).reshape(-1, 4)
            tf[:, :3] = p[1:4]
            recs.append((v, vals, tf))
        if recs:
            self.scene.volumes = recs
        self.renderer.set_scene(self.scene)

    # --------------------------------------------------------------- passes
    def forward_image(self):
        self.renderer.render(self.camera, self.settings, reset=True)
        self.last_forward_ms = self.renderer.stats()["render_ms"]
        return self.renderer.read_color()[..., :3].copy()

    def adjoint(self, d_image, spp=None, sample_offset=None):
        st = type(self.settings).from_buffer_copy(bytes(self.settings))
        st.pixel_samples = int(spp or self.adjoint_spp)
        if sample_offset is None:
            sample_offset = self._adj_offset
            self._adj_offset += st.pixel_samples
        g = self.renderer.adjoint(self.camera, st, np.asarray(d_image, np.float32), sample_offset=sample_offset)
        self.last_adjoint_ms = g["adjoint_ms"]
        return g


class _Render(torch.autograd.Function):
    @staticmethod
    def forward(ctx, ds, materials, texels, volumes):
        ds.apply(materials, texels, volumes)
        ctx.ds = ds
        ctx.tex_shape = texels.shape
        return torch.from_numpy(ds.forward_image())

    @staticmethod
    def backward(ctx, grad):
        ds = ctx.ds
        g = ds.adjoint(grad.detach().cpu().numpy())
        gt = g.get("texels")
        gt = torch.from_numpy(gt) if gt is not None and gt.size else torch.zeros(ctx.tex_shape)
        return None, torch.from_numpy(g["materials"]), gt, torch.from_numpy(g["volumes"])


def render(ds: DiffScene, materials, texels, volumes):
    """Differentiable image (h, w, 3) of the scene with these parameters."""
    return _Render.apply(ds, materials, texels, volumes)


def _np(x):
    if isinstance(x, torch.Tensor):
        return x.detach().cpu().numpy().astype(np.float32)
    return np.asarray(x, np.float32)
