"""Scene tables built on the GPU at upload (tuning key gpu_tables) against
the host builders of the same tables (RenderBridge.cpp:668-780 for the
macro-cell majorant grid), element for element and bit for bit, on the
volume fixture scene (a heterogeneous grid and a homogeneous box) and the
2M-triangle workload's 256^3 fBm grid; renders with either set of tables are
bit-identical.  Upload times of both are printed."""
import time

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

TABLES = ("majorants", "env_marginal", "env_conditional", "emissive_cdf", "prim_light_pdf")


def _scene(kind):
    from photon_gb300 import workloads
    if kind == "instanced_2m_grid256":
        sc, cam, st = workloads.instanced_2m(res=64, spp=2, tex_res=64, grid=256, adaptive=0, n_instances=20)
    else:
        sc, cam, st = workloads.feature_scene(kind)
        st.pixel_samples = 2
    return sc, cam, st


@pytest.mark.parametrize("kind", ["volume", "instanced_2m_grid256"])
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
    assert tables[1]["majorants"].size > 0 and np.isfinite(tables[1]["majorants"]).all()
    assert np.array_equal(imgs[0].view(np.uint32), imgs[1].view(np.uint32))
    print(f"{kind}: {tables[1]['majorants'].size} majorant cells; upload {upload[0] * 1e3:.1f} ms with host "
          f"tables, {upload[1] * 1e3:.1f} ms with GPU tables")
