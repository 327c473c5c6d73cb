"""The C-ABI library on the CPU host: it loads, exports every function the
header declares, its ctypes mirrors have the C layouts, the defaults are the
bridge's, the tuning keys round-trip, and without a GPU it fails cleanly."""
import ctypes as C
import os
import re
import subprocess

import pytest

from photon_gb300 import _abi

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
HEADER = os.path.join(ROOT, "include", "photon_cuda.h")
HEADERS = [os.path.join(ROOT, "include", h) for h in ("photon_cuda.h", "photon_pbrt.h")]


def header_functions():
    names = set()
    for h in HEADERS:
        text = re.sub(r"/\*.*?\*/", "", open(h).read(), flags=re.S)
        names |= set(re.findall(r"\b(phc_[a-z0-9_]+)\s*\(", text))
    return sorted(names)


def test_library_exports_every_header_function(photon):
    from photon_gb300 import native
    lib = photon.load()
    names = header_functions()
    assert len(names) >= 30
    for n in names:
        assert hasattr(lib, n), f"{n} not exported"
        assert n in native.SIGNATURES, f"{n} has no ctypes signature"
    nm = subprocess.run(["nm", "-D", "--defined-only", native.LIB_PATH], capture_output=True, text=True).stdout
    exported = set(re.findall(r" T (phc_\w+)", nm))
    assert set(names) <= exported
    assert exported <= set(names), f"exported but not declared: {exported - set(names)}"


STRUCTS = {
    "phc_param_source": _abi.ParamSource, "phc_material": _abi.Material, "phc_sampler": _abi.Sampler,
    "phc_light": _abi.Light, "phc_environment": _abi.Environment, "phc_volume": _abi.Volume,
    "phc_scene_desc": _abi.SceneDesc, "phc_camera": _abi.Camera, "phc_settings": _abi.Settings,
    "phc_render_stats": _abi.RenderStats, "phc_hit_result": _abi.HitResult, "phc_job": _abi.Job,
    "phc_pt_material": _abi.PtMaterial, "phc_texture": _abi.Texture, "phc_pt_scene": _abi.PtScene,
    "phc_object": _abi.Object, "phc_instance": _abi.Instance,
}


def test_struct_layouts_match_c(tmp_path):
    src = tmp_path / "sizes.c"
    lines = ['#include <stdio.h>', '#include <stddef.h>', '#include "photon_cuda.h"', "int main(void){"]
    for n in STRUCTS:
        lines.append(f'printf("{n} %zu\\n", sizeof({n}));')
    lines.append('printf("env_off %zu\\n", offsetof(phc_scene_desc, environment));')
    lines.append('printf("stats_ms %zu\\n", offsetof(phc_render_stats, render_ms));')
    lines.append("return 0;}")
    src.write_text("\n".join(lines))
    exe = tmp_path / "sizes"
    subprocess.run(["gcc", "-I", os.path.join(ROOT, "include"), str(src), "-o", str(exe)], check=True)
    out = dict(l.split() for l in subprocess.run([str(exe)], capture_output=True, text=True).stdout.splitlines())
    for n, cls in STRUCTS.items():
        assert int(out[n]) == C.sizeof(cls), n
    assert int(out["env_off"]) == _abi.SceneDesc.environment.offset
    assert int(out["stats_ms"]) == _abi.RenderStats.render_ms.offset
    assert C.sizeof(_abi.HitResult) == 88  # photon::pt::HitResult


def test_defaults_are_the_bridges(photon):
    lib = photon.load()
    for fn, ref in (("phc_material_default", _abi.material_default()), ("phc_sampler_default", _abi.sampler_default()),
                    ("phc_light_default", _abi.light_default()), ("phc_volume_default", _abi.volume_default()),
                    ("phc_camera_default", _abi.camera_default()), ("phc_settings_default", _abi.settings_default())):
        got = type(ref)()
        getattr(lib, fn)(C.addressof(got))
        assert bytes(got) == bytes(ref), fn


def test_tuning_round_trip(photon):
    p = photon
    for key, val in (("wave_paths", 1 << 20), ("trace_refill", 12), ("split_shade", 0), ("batch_wave_paths", 99999),
                     ("gpu_max_leaf", 3), ("ploc_radius", 16), ("split_volume", 0), ("gpu_tables", 0),
                     ("texels_u8", 0), ("shade_classes", 0), ("vol_refill", 4), ("vol_passes", 2), ("adjoint_sort", 0),
                     ("class_threshold", 1 << 20), ("collapse_tri_cost", 30)):
        old = p.tuning_get(key)
        p.tuning_set(key, val)
        assert p.tuning_get(key) == val
        p.tuning_set(key, old)
    for key, bad in (("trace_refill", 0), ("gpu_max_leaf", 4), ("ploc_radius", 1), ("ploc_radius", 33),
                     ("split_volume", 2), ("collapse_tri_cost", -1), ("collapse_tri_cost", 10001)):
        old = p.tuning_get(key)
        with pytest.raises(ValueError):
            p.tuning_set(key, bad)
        assert p.tuning_get(key) == old
    with pytest.raises(ValueError):
        p.tuning_set("no_such_key", 1)
    assert p.tuning_get("no_such_key") == -1


def test_entry_points_reject_bad_arguments_without_gpu(photon):
    lib = photon.load()
    assert lib.phc_abi_version() == 2
    assert lib.phc_create(None) == -1                      # PHC_ERR_INVALID
    assert lib.phc_set_scene(None, None) == -1
    assert lib.phc_render(None, None, None, 1) == -1
    assert lib.phc_read_color(None, None) == -1
    assert lib.phc_render_batch(None, 0, None) == -1
    assert lib.phc_accel_create(None, None, 0, None, 0, None, None) == -1
    assert lib.phc_trace_closest_compact_static(None, None, None, None, None, 0, None, None) == -1


@pytest.mark.skipif(__import__("tests.conftest", fromlist=["HAS_GPU"]).HAS_GPU, reason="GPU present")
def test_create_fails_cleanly_without_gpu(photon):
    with pytest.raises(photon.PhotonError, match="CUDA"):
        photon.Renderer()
