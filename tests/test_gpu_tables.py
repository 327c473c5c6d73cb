"""Scene tables built on the GPU at upload (tuning key gpu_tables) against
the host builders of the same tables, element for element and bit for bit:
the macro-cell majorant grid (RenderBridge.cpp:668-780), the environment
map's marginal and row CDFs (environment_map.cpp:8-65) and the emissive
triangles' CDF and area densities (pathtracer.cpp:439-487).  Scenes: the
volume fixture scene (a heterogeneous grid and a homogeneous box), the
2M-triangle workload's 256^3 fBm grid and emissive meshes, the environment
feature scene, and the 500K-triangle workload (1024 x 512 sun-and-sky map,
emissive triangles).  Renders with either set of tables (and so either set
of CDF-search guides) are bit-identical.  Upload times of both are
printed."""
import time

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

TABLES = ("majorants", "env_marginal", "env_conditional", "emissive_cdf", "prim_light_pdf")


def _scene(kind):
    from photon_gb300 import workloads
    if kind == "instanced_2m_grid256":
        sc, cam, st = workloads.instanced_2m(res=64, spp=2, tex_res=64, grid=256, adaptive=0, n_instances=20)
    elif kind == "procedural_500k":
        sc, cam, st = workloads.procedural_500k()
        st.width = st.height = 64
        st.pixel_samples = 2
    else:
        sc, cam, st = workloads.feature_scene(kind)
        st.pixel_samples = 2
    return sc, cam, st


@pytest.mark.parametrize("kind", ["volume", "instanced_2m_grid256", "env", "procedural_500k"])
def test_gpu_tables_equal_host_tables(photon, kind):
    from photon_gb300 import tuning_get, tuning_set
    sc, cam, st = _scene(kind)
    old = tuning_get("gpu_tables")
    tables, imgs, upload = {}, {}, {}
    try:
        for mode in (0, 1):
            tuning_set("gpu_tables", mode)
            r = photon.Renderer()
            t = time.perf_counter()
            r.set_scene(sc)
            upload[mode] = time.perf_counter() - t
            tables[mode] = {name: r.scene_table(name) for name in TABLES}
            r.render(cam, st, True)
            imgs[mode] = r.read("color").copy()
            r.close()
    finally:
        tuning_set("gpu_tables", old)
    for name in TABLES:
        a, b = tables[1][name], tables[0][name]
        assert a.shape == b.shape, name
        assert np.array_equal(a.view(np.uint32), b.view(np.uint32)), name
    if kind in ("volume", "instanced_2m_grid256"):
        assert tables[1]["majorants"].size > 0 and np.isfinite(tables[1]["majorants"]).all()
    if kind in ("env", "procedural_500k"):
        assert tables[1]["env_marginal"].size > 0 and tables[1]["env_conditional"].size > 0
    if kind in ("instanced_2m_grid256", "procedural_500k"):
        assert tables[1]["emissive_cdf"].size > 0 and tables[1]["prim_light_pdf"].size > 0
    assert np.array_equal(imgs[0].view(np.uint32), imgs[1].view(np.uint32))
    sizes = ", ".join(f"{name} {tables[1][name].size}" for name in TABLES)
    print(f"{kind}: {sizes}; upload {upload[0] * 1e3:.1f} ms with host tables, "
          f"{upload[1] * 1e3:.1f} ms with GPU tables")


def _edge_scene(kind):
    """The environment feature scene with its map and emitters edited into
    the builders' edge cases."""
    import copy
    from photon_gb300 import workloads
    sc, cam, st = workloads.feature_scene("env")
    sc = copy.copy(sc)
    env = np.array(sc.env_pixels, np.float32, copy=True)
    if kind == "env_zero":
        env[:] = 0.0  # every row sum 0: uniform row and marginal CDFs
    elif kind == "env_bad_texels":
        env[3] = 0.0                 # a black row
        env[5, 7] = (np.nan, 1.0, 2.0)
        env[6, 1] = (np.inf, -np.inf, 3.0)
        env[7, :, 1] = -1.0          # negative texels count as 0
        env[:, 9] = 1e30             # huge luminance in one column
    sc.env_pixels = env
    if kind == "emitters":
        pos = np.asarray(sc.positions, np.float32).reshape(-1, 3)
        mats = list(sc.materials)
        dim = type(mats[0]).from_buffer_copy(bytes(mats[0]))
        dim.emission[:] = (1e-9, 0.0, 0.0)  # power below the 1e-6 floor
        mats.append(dim)
        sc.materials = mats
        n0 = pos.shape[0]
        extra = np.array([[0.1, 0.2, 0.3], [0.1, 0.2, 0.3], [0.4, 0.2, 0.3],  # zero area
                          [0.2, 0.5, 0.1], [0.3, 0.5, 0.1], [0.2, 0.6, 0.1]], np.float32)
        sc.positions = np.concatenate([pos, extra])
        idx = np.asarray(sc.indices, np.uint32).reshape(-1, 3)
        sc.indices = np.concatenate([idx, np.array([[n0, n0 + 1, n0 + 2], [n0 + 3, n0 + 4, n0 + 5]], np.uint32)])
        mid = np.asarray(sc.material_ids, np.uint32)
        emit = [i for i, m in enumerate(mats) if max(m.emission) > 0][0]
        sc.material_ids = np.concatenate([mid, np.array([emit, len(mats) - 1], np.uint32)])
        if sc.normals is not None:
            sc.normals = np.concatenate([np.asarray(sc.normals, np.float32).reshape(-1, 3),
                                         np.tile(np.array([[0.0, 0.0, 1.0]], np.float32), (6, 1))])
    st.pixel_samples = 2
    return sc, cam, st


@pytest.mark.parametrize("kind", ["env_zero", "env_bad_texels", "emitters"])
def test_gpu_tables_edge_cases(photon, kind):
    """Edge cases of the environment and emitter builders: an all-black map
    (uniform CDFs), non-finite, negative and huge texels and a black row, a
    zero-area emissive triangle and an emitter below the power floor: the
    GPU-built tables equal the host-built ones bit for bit and so do the
    images."""
    from photon_gb300 import tuning_get, tuning_set
    sc, cam, st = _edge_scene(kind)
    old = tuning_get("gpu_tables")
    tables, imgs = {}, {}
    try:
        for mode in (0, 1):
            tuning_set("gpu_tables", mode)
            r = photon.Renderer()
            r.set_scene(sc)
            tables[mode] = {name: r.scene_table(name) for name in TABLES}
            r.render(cam, st, True)
            imgs[mode] = r.read("color").copy()
            r.close()
    finally:
        tuning_set("gpu_tables", old)
    for name in TABLES:
        a, b = tables[1][name], tables[0][name]
        assert a.shape == b.shape, name
        assert np.array_equal(a.view(np.uint32), b.view(np.uint32)), name
    assert np.array_equal(imgs[0].view(np.uint32), imgs[1].view(np.uint32))
    if kind == "env_zero":
        h = tables[1]["env_marginal"].size - 1
        assert np.array_equal(tables[1]["env_marginal"], np.arange(h + 1, dtype=np.float32) / np.float32(h))
