"""The sine and cosine of the shading code (photon_gb300/csrc/sincos.cuh:
float-float Cody-Waite reduction and Taylor series), run on the CPU; the
device build executes the same IEEE float operations.  Against the
correctly rounded values (double-precision sin / cos rounded to float) they
are never more than one ulp off and almost always equal; against the host C
library, which the reference calls, they differ no more often than the
correctly rounded values do (only where the library is not correctly
rounded)."""
import ctypes as C

import numpy as np


def _run(lib, x):
    x = np.ascontiguousarray(x, np.float32)
    n = x.size
    out = [np.zeros(n, np.float32) for _ in range(4)]
    lib.ht_sincos(C.c_void_p(x.ctypes.data), C.c_uint32(n), *[C.c_void_p(o.ctypes.data) for o in out])
    return out


def _ulps(a, b):
    return np.abs(a.view(np.int32).astype(np.int64) - b.view(np.int32).astype(np.int64))


def test_sincos_against_correct_rounding_and_host_libm(host_traverse_lib):
    rng = np.random.default_rng(0)
    k = np.arange(0, 1 << 24, 13, dtype=np.uint32)
    phi = np.float32(2 * np.pi) * (k.astype(np.float32) * np.float32(2.0 ** -24))   # 2 pi u of the sampling
    th = np.float32(np.pi / 4) * rng.uniform(-1, 1, 1 << 20).astype(np.float32)       # concentric-disk angles
    wide = rng.uniform(-np.pi, 2 * np.pi, 1 << 20).astype(np.float32)
    for name, x in (("2 pi u", phi), ("pi/4 r", th), ("[-pi, 2pi]", wide)):
        s, c, ls, lc = _run(host_traverse_lib, x)
        cs = np.sin(x.astype(np.float64)).astype(np.float32)
        cc = np.cos(x.astype(np.float64)).astype(np.float32)
        assert _ulps(s, cs).max() <= 1 and _ulps(c, cc).max() <= 1, name
        not_cr = float(np.mean(s != cs)), float(np.mean(c != cc))
        vs_libm = float(np.mean(s != ls)), float(np.mean(c != lc))
        cr_vs_libm = float(np.mean(cs != ls)), float(np.mean(cc != lc))
        print(f"{name}: not correctly rounded sin {not_cr[0]:.1e} cos {not_cr[1]:.1e}; differs from the host "
              f"library sin {vs_libm[0]:.2e} cos {vs_libm[1]:.2e} (correct rounding: {cr_vs_libm[0]:.2e} "
              f"{cr_vs_libm[1]:.2e})")
        assert max(not_cr) < 1e-4, (name, not_cr)
        assert vs_libm[0] <= cr_vs_libm[0] + 1e-4 and vs_libm[1] <= cr_vs_libm[1] + 1e-4, name
    s, c, _, _ = _run(host_traverse_lib, np.array([0.0, -0.0, np.nan, 100.0], np.float32))
    assert s[0] == 0 and np.signbit(s[1]) and c[0] == 1 and np.isnan(s[2]) and np.isfinite(s[3])
