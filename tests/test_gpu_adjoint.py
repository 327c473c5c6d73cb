"""Path-replay adjoint (phc_adjoint) on the GPU.

Checks, on the same random numbers (common random numbers: a fresh
renderer's first render uses sample indices 0..spp-1, the adjoint is asked
for the same range):
  * the adjoint's own primal pass reproduces the forward renderer's image;
  * the gradients are linear in dLoss/dImage and vanish for a zero one;
  * on a scene whose sampling decisions do not depend on the parameters
    (diffuse walls, no Russian roulette), central finite differences of the
    forward renderer match the adjoint to float precision;
  * on the differentiable workload (textured Disney materials, homogeneous
    medium) central differences match within the stated tolerance, per
    scalar parameter and along random texel directions.
The loss is linear, Loss = sum(W * I) with fixed positive weights W, so
dLoss/dI = W.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

# The finite differences with common random numbers share every sample of the
# adjoint, but a parameter step can still flip a lobe choice or a Russian
# roulette decision of a few paths; those flips are noise of the difference
# quotient, so the Disney / medium comparison is statistical.
FD_REL_TOL_SMOOTH = 2e-3
FD_REL_TOL = 0.02


def _weights(h, w, seed=5):
    rng = np.random.default_rng(seed)
    wt = np.zeros((h, w, 4), np.float32)
    wt[..., :3] = rng.uniform(0.5, 1.5, (h, w, 3))
    return wt


def _image(photon, sc, cam, st):
    r = photon.Renderer()
    r.set_scene(sc)
    r.render(cam, st, True)
    img = r.read_color()[..., :3].astype(np.float64)
    r.close()
    return img


def _loss(photon, sc, cam, st, wt):
    return float(np.sum(_image(photon, sc, cam, st) * wt[..., :3]))


def _adjoint(photon, sc, cam, st, wt, **kw):
    r = photon.Renderer()
    r.set_scene(sc)
    g = r.adjoint(cam, st, wt, sample_offset=0, **kw)
    r.close()
    return g


def _diff_small(res=40, spp=8, texture=64, param_textures=False):
    from photon_gb300 import workloads
    return workloads.differentiable(res=res, spp=spp, depth=6, texture=texture, param_textures=param_textures)


def test_primal_pass_is_the_render(photon):
    """The adjoint's pass 1 is the forward renderer: its image is the render's,
    and the replay walks every forward path (no radiance mismatch)."""
    sc, cam, st = _diff_small()
    img = _image(photon, sc, cam, st)
    g = _adjoint(photon, sc, cam, st, _weights(st.height, st.width), color=True)
    adj = g["color"][..., :3].astype(np.float64)
    close = np.abs(adj - img) <= 1e-4 * np.abs(img) + 1e-6
    assert close.mean() >= 0.999, close.mean()
    assert g["replay_mismatches"] <= 1e-3 * st.width * st.height * st.pixel_samples, g["replay_mismatches"]
    z = _adjoint(photon, sc, cam, st, np.zeros((st.height, st.width, 4), np.float32))
    assert np.all(z["materials"] == 0) and np.all(z["volumes"] == 0) and np.all(z["texels"] == 0)


def test_linear_in_loss_gradient(photon):
    sc, cam, st = _diff_small(res=24, spp=4)
    w1 = _weights(st.height, st.width, 1)
    w2 = _weights(st.height, st.width, 2)
    g1 = _adjoint(photon, sc, cam, st, w1)
    g2 = _adjoint(photon, sc, cam, st, w2)
    g12 = _adjoint(photon, sc, cam, st, w1 + 2 * w2)
    for k in ("materials", "volumes", "texels"):
        want = g1[k].astype(np.float64) + 2 * g2[k].astype(np.float64)
        scale = np.abs(want).max() + 1e-30
        assert np.abs(g12[k] - want).max() <= 1e-4 * scale, k


def test_fd_diffuse_base_colour_exact(photon):
    """Diffuse box room, depth 2: no lobe choice or roulette depends on the
    base colours, the image is a quadratic in them, so central differences
    are exact up to float rounding."""
    from photon_gb300 import workloads
    sc, cam, st = workloads.feature_scene("basic", res=32)
    st.pixel_samples = 8
    st.max_depth = 2
    wt = _weights(st.height, st.width)
    g = _adjoint(photon, sc, cam, st, wt)["materials"]
    h = 1e-2
    for m in range(3):
        for c in range(3):
            base = sc.materials[m].base_color[c]
            sc.materials[m].base_color[c] = base + h
            lp = _loss(photon, sc, cam, st, wt)
            sc.materials[m].base_color[c] = base - h
            lm = _loss(photon, sc, cam, st, wt)
            sc.materials[m].base_color[c] = base
            fd = (lp - lm) / (2 * h)
            assert abs(g[m, c] - fd) <= FD_REL_TOL_SMOOTH * abs(fd) + 1e-3, (m, c, g[m, c], fd)


def _fd_scalar(photon, sc, cam, st, wt, setter, value, h):
    setter(value + h)
    lp = _loss(photon, sc, cam, st, wt)
    setter(value - h)
    lm = _loss(photon, sc, cam, st, wt)
    setter(value)
    return (lp - lm) / (2 * h)


def test_fd_disney_and_medium_parameters(photon):
    """Every scalar Disney parameter of the 8 materials and the medium's
    density scale and albedo: the gradient vector agrees with central
    differences within FD_REL_TOL (4M pixel samples; the residual is the
    finite differences' own noise)."""
    sc, cam, st = _diff_small(res=32, spp=4096)
    wt = _weights(st.height, st.width)
    g = _adjoint(photon, sc, cam, st, wt)
    adj, fd = [], []
    h = 1e-2
    fields = (("roughness", 3), ("metallic", 4), ("transmission", 5), ("sheen", 6), ("clearcoat", 7))
    for m, mat in enumerate(sc.materials):
        for name, k in fields:
            v = getattr(mat, name)
            if name == "transmission" and v <= 0:
                continue
            fd.append(_fd_scalar(photon, sc, cam, st, wt, lambda x, mat=mat, name=name: setattr(mat, name, x), v, h))
            adj.append(g["materials"][m, k])
    vol, vals, tf = sc.volumes[0]

    def set_density(x):
        vol.density_scale = x

    fd.append(_fd_scalar(photon, sc, cam, st, wt, set_density, vol.density_scale, h))
    adj.append(g["volumes"][0, 0])
    for c in range(3):
        base = float(tf[0, c])

        def set_albedo(x, c=c):
            tf[:, c] = x

        fd.append(_fd_scalar(photon, sc, cam, st, wt, set_albedo, base, h))
        adj.append(g["volumes"][0, 1 + c])
    adj, fd = np.array(adj, np.float64), np.array(fd, np.float64)
    err = np.linalg.norm(adj - fd) / np.linalg.norm(fd)
    print("adjoint", np.array2string(adj, precision=3), "\nfd     ", np.array2string(fd, precision=3), "\nrel", err)
    assert err <= FD_REL_TOL, err


def test_fd_texel_directions(photon):
    """Texel gradients along a uniform brightening of whole textures."""
    sc, cam, st = _diff_small(res=32, spp=4096)
    wt = _weights(st.height, st.width)
    g = _adjoint(photon, sc, cam, st, wt)["texels"]
    h = 1e-2
    counts = [t.shape[0] for _, t in sc.samplers]
    offs = np.concatenate([[0], np.cumsum(counts)])
    adj, fd = [], []
    for i in (0, 3, 6):
        rec, tex = sc.samplers[i]
        base = tex.copy()
        v = np.zeros_like(base)
        v[:, :3] = 1.0
        sc.samplers[i] = (rec, base + h * v)
        lp = _loss(photon, sc, cam, st, wt)
        sc.samplers[i] = (rec, base - h * v)
        lm = _loss(photon, sc, cam, st, wt)
        sc.samplers[i] = (rec, base)
        fd.append((lp - lm) / (2 * h))
        adj.append(float(np.sum(g[offs[i]:offs[i + 1]].astype(np.float64) * v)))
    adj, fd = np.array(adj), np.array(fd)
    print("texel directions: adjoint", adj, "fd", fd)
    assert np.all(np.abs(adj - fd) <= FD_REL_TOL * np.abs(fd) + 1e-6), (adj, fd)


def test_fd_parameter_texture_directions(photon):
    """Texel gradients of roughness (materials 0-3), metallic (4-6) and
    specTrans (7) read from textures, along a uniform raise of a whole
    texture's r channel (the channel those parameters read): the gradient
    vector against central differences, as for the scalar parameters (a
    step flips some paths' lobe choices, noise of the difference quotient;
    the FP64 CPU adjoint below checks the same gradients on the estimator
    itself to 1e-5)."""
    sc, cam, st = _diff_small(res=32, spp=4096, param_textures=True)
    wt = _weights(st.height, st.width)
    g = _adjoint(photon, sc, cam, st, wt)["texels"]
    h = 4e-2  # inside (0, 1) for every texel; a larger step, less noise from flipped paths
    counts = [t.shape[0] for _, t in sc.samplers]
    offs = np.concatenate([[0], np.cumsum(counts)])
    adj, fd = [], []
    for i in (8, 11, 12, 15):  # roughness, roughness, metallic, specTrans
        rec, tex = sc.samplers[i]
        base = tex.copy()
        v = np.zeros_like(base)
        v[:, 0] = 1.0
        sc.samplers[i] = (rec, base + h * v)
        lp = _loss(photon, sc, cam, st, wt)
        sc.samplers[i] = (rec, base - h * v)
        lm = _loss(photon, sc, cam, st, wt)
        sc.samplers[i] = (rec, base)
        fd.append((lp - lm) / (2 * h))
        adj.append(float(np.sum(g[offs[i]:offs[i + 1]].astype(np.float64) * v)))
    adj, fd = np.array(adj), np.array(fd)
    err = np.linalg.norm(adj - fd) / np.linalg.norm(fd)
    print("parameter texture directions: adjoint", adj, "fd", fd, "rel", err)
    assert err <= FD_REL_TOL, (adj, fd, err)


@pytest.mark.parametrize("param_textures", [False, True])
def test_gpu_adjoint_matches_fp64_cpu_adjoint(photon, oracle_lib, param_textures):
    """The GPU adjoint against the FP64 CPU adjoint (oracle/adjoint_fp64.inc:
    the same paths replayed by the oracle, derivatives by central differences
    in double of each weight's forward formula) on the same pixel samples:
    every scalar material parameter, the medium's density and albedo, and the
    texels along three random directions; with param_textures, roughness,
    metallic and specTrans are read from textures too, and their texels are
    part of the directions."""
    sc, cam, st = _diff_small(res=16, spp=16, param_textures=param_textures)
    wt = _weights(st.height, st.width)
    g = _adjoint(photon, sc, cam, st, wt)
    ref = oracle_lib.CpuRenderer("oracle")
    ref.set_scene(sc)
    params, gpu = [], []
    for m in range(len(sc.materials)):
        for k in range(3, 8):
            params.append((0, m, k))
            gpu.append(g["materials"][m, k])
    for k in range(4):
        params.append((1, 0, k))
        gpu.append(g["volumes"][0, k])
    rng = np.random.default_rng(3)
    ntex = g["texels"].shape[0]
    dirs = []
    for d in range(3):
        v = np.zeros((ntex, 4), np.float32)
        v[:, :3] = rng.uniform(-1, 1, (ntex, 3))
        dirs.append(v)
        params.append((2, d, 0))
        gpu.append(float(np.sum(g["texels"].astype(np.float64) * v)))
    cpu = oracle_lib.adjoint_fp64(ref, cam, st, wt, params, dirs)
    gpu = np.array(gpu, np.float64)
    err = np.linalg.norm(gpu - cpu) / np.linalg.norm(cpu)
    print("gpu", np.array2string(gpu, precision=4), "\nfp64", np.array2string(cpu, precision=4), "\nrel", err)
    assert err <= 2e-3, err
    scale = np.abs(cpu).max()
    assert np.all(np.abs(gpu - cpu) <= 1e-2 * np.abs(cpu) + 1e-3 * scale), np.abs(gpu - cpu) / scale


def test_adjoint_api_errors(photon):
    sc, cam, st = _diff_small(res=16, spp=2)
    r = photon.Renderer()
    with pytest.raises(photon.PhotonError):
        r.adjoint(cam, st, np.zeros((16, 16, 4), np.float32))  # no scene
    r.set_scene(sc)
    st.adaptive_sampling = 1
    with pytest.raises(photon.PhotonError):
        r.adjoint(cam, st, np.zeros((16, 16, 4), np.float32))
    st.adaptive_sampling = 0
    with pytest.raises(ValueError):
        r.adjoint(cam, st, np.zeros((8, 16, 4), np.float32))
    g = r.adjoint(cam, st, np.ones((16, 16, 3), np.float32))
    assert g["materials"].shape == (8, 8) and g["volumes"].shape == (1, 4)
    assert g["texels"].shape == (8 * 64 * 64, 4)
    assert r.accumulated_samples() == 0  # the adjoint leaves the frame alone
    r.close()


def test_torch_autograd_wrapper(photon):
    import torch
    from photon_gb300 import diff
    sc, cam, st = _diff_small(res=24, spp=4)
    ds = diff.DiffScene(sc, cam, st, adjoint_spp=4)
    mats, tex, vols = ds.params()
    mats.requires_grad_(True)
    tex.requires_grad_(True)
    vols.requires_grad_(True)
    img = diff.render(ds, mats, tex, vols)
    assert img.shape == (24, 24, 3)
    loss = (img * torch.from_numpy(_weights(24, 24)[..., :3])).sum()
    loss.backward()
    assert mats.grad.shape == mats.shape and tex.grad.shape == tex.shape and vols.grad.shape == vols.shape
    assert torch.isfinite(mats.grad).all() and torch.isfinite(tex.grad).all() and torch.isfinite(vols.grad).all()
    assert mats.grad[:, 3:].abs().sum() > 0 and tex.grad.abs().sum() > 0 and vols.grad.abs().sum() > 0
