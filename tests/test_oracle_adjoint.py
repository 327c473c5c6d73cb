"""The FP64 CPU adjoint (oracle/adjoint_fp64.inc) on the CPU: on diffuse
walls at depth 2 (no sampling decision depends on the base colours, the
image is a quadratic in them) it equals central differences of the oracle's
own float renders."""
import numpy as np


def test_fp64_adjoint_equals_oracle_differences(oracle_lib):
    from photon_gb300 import workloads
    sc, cam, st = workloads.feature_scene("basic", res=16)
    st.pixel_samples = 4
    st.max_depth = 2
    rng = np.random.default_rng(5)
    wt = np.zeros((16, 16, 4), np.float32)
    wt[..., :3] = rng.uniform(0.5, 1.5, (16, 16, 3))
    r = oracle_lib.CpuRenderer("oracle")
    r.set_scene(sc)
    params = [(0, m, c) for m in range(3) for c in range(3)]
    g = oracle_lib.adjoint_fp64(r, cam, st, wt, params)

    def loss():
        q = oracle_lib.CpuRenderer("oracle")
        q.set_scene(sc)
        q.render(cam, st, True)
        return float(np.sum(q.read("color")[..., :3].astype(np.float64) * wt[..., :3]))

    h = 1e-2
    for k, (_, m, c) in enumerate(params):
        base = sc.materials[m].base_color[c]
        sc.materials[m].base_color[c] = base + h
        lp = loss()
        sc.materials[m].base_color[c] = base - h
        lm = loss()
        sc.materials[m].base_color[c] = base
        fd = (lp - lm) / (2 * h)
        assert abs(g[k] - fd) <= 1e-4 * abs(fd) + 1e-4, (m, c, g[k], fd)
