"""pbrt-v4 reader (include/photon_pbrt.h) against the reference's own pbrt path.

The reference's parse_pbrt_file + convert_pbrt_scene ran on the scenes of
tests/golden/pbrt/ (tests/golden/make_pbrt_golden.py, through
oracle/_ref/libphoton_ref.so): the converted mesh, materials, textures and
environment must be bit-identical (SHA-256 of the arrays), and the CPU
oracle's render of the reader's scene must equal the reference's own
PathTracer render of its converted scene sample for sample.  Where the
reference build exists (oracle/_ref), the same comparisons also run live.
"""
import hashlib
import os

import numpy as np
import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
SCENES = os.path.join(HERE, "golden", "pbrt")
GOLDEN = os.path.join(HERE, "golden", "pbrt_ref.npz")
CASES = [("box_room", "box_room.pbrt", False), ("features", "features.pbrt", False),
         ("features_ias", "features.pbrt", True)]


def sha(a):
    return hashlib.sha256(np.ascontiguousarray(a).tobytes()).hexdigest()


def digest(arrs):
    """The digests of make_pbrt_golden.py over the reader's arrays (the
    reader stores the mesh as three vertices per triangle, as the reference)."""
    out = {k: sha(arrs[k]) for k in ("positions", "normals", "texcoords", "material_ids")}
    out["materials"] = hashlib.sha256(b"".join(bytes(m) for m in arrs["materials"])).hexdigest()
    out["textures"] = sha(np.concatenate([t.ravel() for t in arrs["textures"]])) if arrs["textures"] else sha(
        np.zeros(0, np.float32))
    env = arrs["env"]
    out["env"] = sha(np.concatenate([env[k].ravel() for k in ("pixels", "world_to_map", "map_to_world")])) \
        if env is not None else sha(np.zeros(0, np.float32))
    return out


@pytest.fixture(scope="module")
def golden():
    return np.load(GOLDEN)


@pytest.mark.parametrize("case,fname,ias", CASES)
def test_conversion_bit_identical_to_reference(photon, golden, case, fname, ias):
    from photon_gb300 import pbrt
    sc = pbrt.load(os.path.join(SCENES, fname), use_instancing=ias)
    arrs = sc.arrays()
    names = [str(x) for x in golden[f"{case}/counts_names"]]
    counts = dict(zip(names, golden[f"{case}/counts"].tolist()))
    inf = sc.info
    assert inf["triangles"] == counts["triangles"]
    assert len(arrs["materials"]) == counts["materials"]
    assert inf["emissive_triangles"] == counts["emissive"]
    assert inf["loaded_textures"] == counts["textures"]
    assert (inf["width"], inf["height"], inf["spp"], inf["max_depth"]) == tuple(
        counts[k] for k in ("width", "height", "spp", "max_depth"))
    assert inf["meshes"] == counts["meshes"] and inf["named_materials"] == counts["named_materials"]
    assert inf["object_defs"] == counts["object_defs"] and inf["object_instances"] == counts["object_instances"]
    assert inf["has_env_map"] == counts["has_env"]
    # the mesh is flattened: vertex 3t + k is corner k of triangle t
    assert np.array_equal(arrs["indices"].ravel(), np.arange(3 * inf["triangles"], dtype=np.uint32))
    for k, v in digest(arrs).items():
        assert v == str(golden[f"{case}/sha_{k}"]), f"{case}: {k} differs from the reference's conversion"


def _camera_frame(cam, w, h):
    """The bridge's camera construction (RenderBridge.cpp:872-891 with
    Camera::make_perspective), in float64, for a tolerance check."""
    pos = np.array(cam.position[:], np.float64)
    d = np.array(cam.direction[:], np.float64)
    d /= np.linalg.norm(d)
    up = np.array(cam.up[:], np.float64)
    cw = -d
    cu = np.cross(up, cw)
    cu /= np.linalg.norm(cu)
    cv = np.cross(cw, cu)
    deg = np.float32(np.float32(cam.fovy) * np.float32(180.0)) / np.float32(3.14159265358979)
    hh = np.tan(np.deg2rad(float(deg)) * 0.5)
    aspect = cam.aspect if cam.aspect > 0 else w / h
    focus = cam.focus_distance if cam.aperture_radius > 0 else 1.0
    hor = cu * (aspect * 2 * hh * focus)
    ver = cv * (2 * hh * focus)
    ll = pos - hor / 2 - ver / 2 - cw * focus
    return np.concatenate([pos, ll, hor, ver, cu, cv, cw])


@pytest.mark.parametrize("case,fname,ias", CASES)
def test_camera_matches_reference(photon, golden, case, fname, ias):
    from photon_gb300 import pbrt
    sc = pbrt.load(os.path.join(SCENES, fname), use_instancing=ias)
    ref = golden[f"{case}/camera"].astype(np.float64)
    ours = _camera_frame(sc.camera, sc.settings.width, sc.settings.height)
    np.testing.assert_allclose(ours, ref[:21], rtol=0, atol=2e-6)
    assert sc.camera.aperture_radius == np.float32(ref[21])


@pytest.mark.parametrize("case,fname,ias", CASES)
def test_oracle_render_matches_reference_render(photon, oracle_lib, golden, case, fname, ias):
    """Per sample: the oracle renders the reader's scene exactly as the
    reference's PathTracer renders its own conversion (spp 4, adaptive off)."""
    from photon_gb300 import pbrt
    w, h, spp, _ = golden[f"{case}/render_args"].tolist()
    sc = pbrt.load(os.path.join(SCENES, fname), use_instancing=ias, width=w, height=h, spp=spp)
    st = type(sc.settings).from_buffer_copy(bytes(sc.settings))
    st.adaptive_sampling = 0
    o = oracle_lib.CpuRenderer("oracle")
    o.set_scene(sc)
    o.render(sc.camera, st, True)
    img = o.read("color")[..., :3]
    ref = golden[f"{case}/render"]
    rel = np.abs(img - ref) / np.maximum(np.abs(ref), 1e-3)
    assert (rel <= 1e-4).mean() >= 0.999, f"{case}: {(rel > 1e-4).mean():.4%} of pixel channels differ"
    np.testing.assert_allclose(img, ref, rtol=1e-3, atol=1e-5)


def _ref_available():
    import oracle
    return os.path.exists(oracle.REF_LIB)


@pytest.mark.skipif(not _ref_available(), reason="reference build (oracle/_ref) not present")
@pytest.mark.parametrize("case,fname,ias", CASES)
def test_live_reference_conversion(photon, oracle_lib, case, fname, ias):
    """The same identity against the reference library itself, array by array."""
    from photon_gb300 import pbrt
    path = os.path.join(SCENES, fname)
    ref = oracle_lib.RefPbrt(path, use_instancing=ias)
    ra = ref.arrays()
    a = pbrt.load(path, use_instancing=ias).arrays()
    for k in ("positions", "normals", "texcoords"):
        assert a[k].tobytes() == ra[k].tobytes(), k
    assert np.array_equal(a["material_ids"], ra["material_ids"])
    assert [bytes(m) for m in a["materials"]] == [bytes(m) for m in ra["materials"]]
    assert len(a["textures"]) == len(ra["textures"])
    for t1, t2 in zip(a["textures"], ra["textures"]):
        assert t1.tobytes() == t2.tobytes()
    assert (a["env"] is None) == (ra["env"] is None)
    if a["env"] is not None:
        for k in ("pixels", "world_to_map", "map_to_world"):
            assert a["env"][k].tobytes() == ra["env"][k].tobytes(), k


def test_reader_quirks(photon):
    """Forms the reference reads in its own way (pbrt_parser.cpp), kept."""
    from photon_gb300 import pbrt
    sc = pbrt.load(os.path.join(SCENES, "features.pbrt"))
    mats = sc.arrays()["materials"]
    # named materials in name order: alu coat copper floor glass gold leaf odd photo
    by_name = dict(zip(["alu", "coat", "copper", "floor", "glass", "gold", "leaf", "odd", "photo"], mats))
    # an unbracketed named spectrum is not read: copper keeps eta = k = 0,
    # whose Fresnel f0 ((eta-1)^2 + k^2) / ((eta+1)^2 + k^2) is 1
    assert list(by_name["copper"].base_color) == [1.0, 1.0, 1.0]
    assert by_name["copper"].roughness == np.float32(0.2)  # (u + v) / 2
    assert by_name["gold"].metallic == 1.0 and by_name["gold"].base_color[0] > 0.5
    assert by_name["glass"].transmission == 1.0 and by_name["glass"].ior == np.float32(1.33)
    assert by_name["coat"].clearcoat == 1.0 and by_name["coat"].clearcoat_roughness == np.float32(0.15)
    assert by_name["leaf"].transmission == 0.5
    assert by_name["floor"].base_color_tex == 0  # checker.pfm loaded; photo.png has no loader
    assert by_name["photo"].base_color_tex == -1
    assert by_name["odd"].roughness == np.float32(0.4)
    # the alpha-textured PLY mesh got its own copy of "coat" with the mask
    assert any(m.alpha_tex == 1 for m in mats[9:])
    # emitter materials: black, emission (6, 5, 4), strength 1, not squared roughness 1
    em = [m for m in mats if m.emission_strength == 1.0]
    assert len(em) == 2 and all(list(m.emission) == [6.0, 5.0, 4.0] for m in em)


def test_reader_errors(photon, tmp_path):
    from photon_gb300 import pbrt
    from photon_gb300.native import PhotonError
    with pytest.raises(PhotonError, match="cannot open"):
        pbrt.load(str(tmp_path / "missing.pbrt"))
    bad = tmp_path / "bad.pbrt"
    bad.write_text('WorldBegin\nShape "trianglemesh" "point3 P" [ 0 0 0 1 0 0 0 1 0 ] "integer indices" [ 0 1 7 ]\n')
    with pytest.raises(PhotonError, match="out of range"):
        pbrt.load(str(bad))


def test_empty_and_default_scene(photon, tmp_path):
    """No shapes: no triangles, the fallback material, the file's defaults."""
    from photon_gb300 import pbrt
    p = tmp_path / "empty.pbrt"
    p.write_text("# nothing but a world\nWorldBegin\n")
    sc = pbrt.load(str(p))
    assert sc.info["triangles"] == 0 and sc.info["width"] == 512 and sc.info["spp"] == 64
    m = sc.arrays()["materials"]
    assert len(m) == 1 and list(m[0].base_color) == [0.5, 0.5, 0.5] and m[0].roughness == 1.0
    s = sc.settings
    assert s.adaptive_sampling == 1 and s.throughput_clamp == np.float32(10.0) and s.max_depth == 8


def test_ppm_writer(tmp_path):
    from photon_gb300 import pbrt
    img = np.zeros((2, 3, 3), np.float32)
    img[0, 0] = 1.0
    p = tmp_path / "o.ppm"
    pbrt.write_ppm(str(p), img)
    data = p.read_bytes()
    assert data.startswith(b"P6\n3 2\n255\n") and len(data) == len(b"P6\n3 2\n255\n") + 18
    assert data[len(b"P6\n3 2\n255\n")] > 200
