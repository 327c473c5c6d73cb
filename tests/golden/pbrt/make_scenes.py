"""Writes the pbrt-v4 test scenes of this folder and their assets.

    python tests/golden/pbrt/make_scenes.py

box_room.pbrt   the box-room workload (5 quads, two rotated boxes, a 0.25 m^2
                area light of radiance (17, 12, 4); 512x512, 64 spp, depth 8)
                as a pbrt-v4 file.
features.pbrt   every directive and parameter form the reader handles
                (+ features_include.pbrt, mesh_ascii.ply, mesh_binary.ply,
                checker.pfm, alpha.pfm, sky.pfm), including the forms the
                reference reads in its own way (unbracketed named spectra,
                Translate, TransformBegin/End, a texture in a format without
                a loader, an unknown material type and shape).

Deterministic; the files are committed next to this script.
"""
import os
import struct

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))


def fl(v):
    return " ".join(repr(float(np.float32(x))) for x in np.ravel(v))


def ints(v):
    return " ".join(str(int(x)) for x in np.ravel(v))


def col_major(m):
    """pbrt matrix text (column-major) of a row-major 4x4."""
    return fl(np.asarray(m, np.float64).T.ravel())


def box_mesh(size):
    sx, sy, sz = size
    corners = []
    for y in (0.0, sy):
        for (x, z) in ((-sx / 2, -sz / 2), (sx / 2, -sz / 2), (sx / 2, sz / 2), (-sx / 2, sz / 2)):
            corners.append((x, y, z))
    faces = [(4, 7, 6, 5), (0, 1, 5, 4), (1, 2, 6, 5), (2, 3, 7, 6), (3, 0, 4, 7), (0, 3, 2, 1)]
    idx = []
    for a, b, c, d in faces:
        idx += [a, b, c, a, c, d]
    return np.array(corners, np.float32), np.array(idx)


def rot_y_translate(deg, t):
    c, s = np.cos(np.deg2rad(deg)), np.sin(np.deg2rad(deg))
    return np.array([[c, 0, s, t[0]], [0, 1, 0, t[1]], [-s, 0, c, t[2]], [0, 0, 0, 1]])


def quad(name, p, mat=None, extra=""):
    out = "AttributeBegin\n"
    if mat:
        out += f'  NamedMaterial "{mat}"\n'
    out += extra
    out += f'  Shape "trianglemesh" "point3 P" [ {fl(p)} ] "integer indices" [ 0 1 2 0 2 3 ]\n'
    out += "AttributeEnd\n"
    return out


def box_room():
    W = 2.0
    s = ["# Box room: 5 quads, two rotated boxes, one 0.5 x 0.5 m area light.",
         'LookAt 0 1 3.9  0 1 0  0 1 0',
         'Camera "perspective" "float fov" [ 40 ]',
         'Film "rgb" "integer xresolution" [ 512 ] "integer yresolution" [ 512 ] "string filename" "box_room.exr"',
         'Sampler "independent" "integer pixelsamples" [ 64 ]',
         'Integrator "path" "integer maxdepth" [ 8 ]',
         "WorldBegin",
         'MakeNamedMaterial "white" "string type" "diffuse" "rgb reflectance" [ 0.73 0.73 0.73 ]',
         'MakeNamedMaterial "red" "string type" "diffuse" "rgb reflectance" [ 0.65 0.05 0.05 ]',
         'MakeNamedMaterial "green" "string type" "diffuse" "rgb reflectance" [ 0.12 0.45 0.15 ]']
    txt = "\n".join(s) + "\n"
    txt += quad("floor", [(-1, 0, -1), (-1, 0, 1), (1, 0, 1), (1, 0, -1)], "white")
    txt += quad("ceiling", [(-1, W, -1), (1, W, -1), (1, W, 1), (-1, W, 1)], "white")
    txt += quad("back", [(-1, 0, -1), (1, 0, -1), (1, W, -1), (-1, W, -1)], "white")
    txt += quad("left", [(-1, 0, -1), (-1, W, -1), (-1, W, 1), (-1, 0, 1)], "red")
    txt += quad("right", [(1, 0, -1), (1, 0, 1), (1, W, 1), (1, W, -1)], "green")
    for size, deg, t in (((0.6, 1.2, 0.6), 17.0, (-0.33, 1e-3, -0.3)), ((0.6, 0.6, 0.6), -18.0, (0.35, 1e-3, 0.3))):
        v, i = box_mesh(size)
        txt += ("AttributeBegin\n  NamedMaterial \"white\"\n"
                f"  ConcatTransform [ {col_major(rot_y_translate(deg, t))} ]\n"
                f"  Shape \"trianglemesh\" \"point3 P\" [ {fl(v)} ] \"integer indices\" [ {ints(i)} ]\n"
                "AttributeEnd\n")
    ly = W - 1e-3
    txt += quad("light", [(-0.25, ly, -0.25), (0.25, ly, -0.25), (0.25, ly, 0.25), (-0.25, ly, 0.25)],
                extra='  AreaLightSource "diffuse" "rgb L" [ 17 12 4 ]\n')
    return txt


def write_pfm(path, img):
    """img (h, w, c) top row first; PFM stores the bottom row first."""
    h, w = img.shape[:2]
    c = 1 if img.ndim == 2 or img.shape[2] == 1 else 3
    with open(path, "wb") as f:
        f.write(b"PF\n" if c == 3 else b"Pf\n")
        f.write(f"{w} {h}\n-1.0\n".encode())
        data = img.reshape(h, w, c)[::-1].astype("<f4")
        f.write(data.tobytes())


def ply_mesh():
    """A small displaced grid: (x, y, z, nx, ny, nz, u, v) and quad faces."""
    n = 5
    verts, faces = [], []
    for j in range(n):
        for i in range(n):
            x, z = i / (n - 1) - 0.5, j / (n - 1) - 0.5
            y = 0.15 * np.sin(3 * x) * np.cos(2 * z)
            nrm = np.array([-0.45 * np.cos(3 * x) * np.cos(2 * z), 1.0, 0.3 * np.sin(3 * x) * np.sin(2 * z)])
            nrm /= np.linalg.norm(nrm)
            verts.append((x, y, z, *nrm, i / (n - 1), j / (n - 1)))
    for j in range(n - 1):
        for i in range(n - 1):
            a = j * n + i
            faces.append((a, a + 1, a + n + 1, a + n))
    return np.array(verts, np.float32), faces


def write_ply_ascii(path, verts, faces):
    with open(path, "w") as f:
        f.write("ply\nformat ascii 1.0\ncomment written by make_scenes.py\n")
        f.write(f"element vertex {len(verts)}\n")
        for p in ("x", "y", "z", "nx", "ny", "nz", "u", "v"):
            f.write(f"property float {p}\n")
        f.write(f"element face {len(faces)}\nproperty list uchar int vertex_indices\nend_header\n")
        for v in verts:
            f.write(" ".join(repr(float(x)) for x in v) + "\n")
        for fc in faces:
            f.write(f"{len(fc)} " + " ".join(str(i) for i in fc) + "\n")


def write_ply_binary(path, verts, faces):
    with open(path, "wb") as f:
        f.write(b"ply\r\nformat binary_little_endian 1.0\r\n")
        f.write(f"element vertex {len(verts)}\r\n".encode())
        for p in ("x", "y", "z"):
            f.write(f"property float {p}\r\n".encode())
        f.write(b"property uchar flags\r\n")  # skipped by size
        for p in ("s", "t"):
            f.write(f"property float32 {p}\r\n".encode())
        f.write(f"element face {len(faces)}\r\n".encode())
        f.write(b"property list uint8 uint32 vertex_index\r\nproperty int face_tag\r\nend_header\n")
        for v in verts:
            f.write(struct.pack("<3fB2f", v[0], v[1], v[2], 7, v[6], v[7]))
        for k, fc in enumerate(faces):
            tri = fc if k % 2 else (fc[0], fc[1], fc[2])  # quads and triangles
            f.write(struct.pack("<B", len(tri)) + struct.pack(f"<{len(tri)}I", *tri) + struct.pack("<i", k))


def features():
    rng = np.random.default_rng(7)
    yy, xx = np.mgrid[0:16, 0:16]
    checker = np.where(((xx // 4) + (yy // 4)) % 2 == 0, 0.8, 0.1)[..., None] * np.array([1.0, 0.8, 0.6])
    checker = checker + 0.05 * rng.random((16, 16, 3))
    write_pfm(os.path.join(HERE, "checker.pfm"), checker.astype(np.float32))
    alpha = np.clip(0.5 + 0.5 * np.sin(xx / 2.0) * np.cos(yy / 3.0), 0, 1).astype(np.float32)
    write_pfm(os.path.join(HERE, "alpha.pfm"), alpha[..., None])
    th = (np.arange(16) + 0.5) / 16
    sky = np.stack([0.4 + 0.6 * th, 0.5 + 0.4 * th, 0.9 - 0.3 * th], -1)[:, None, :] * np.ones((16, 32, 1))
    sky[3, 20] = [40.0, 36.0, 30.0]  # a small sun
    write_pfm(os.path.join(HERE, "sky.pfm"), sky.astype(np.float32))
    verts, faces = ply_mesh()
    write_ply_ascii(os.path.join(HERE, "mesh_ascii.ply"), verts, faces)
    write_ply_binary(os.path.join(HERE, "mesh_binary.ply"), verts, faces)

    cam = np.array([[1, 0, 0, 0], [0, 0.9701425, -0.2425356, -0.4], [0, 0.2425356, 0.9701425, 3.2], [0, 0, 0, 1]])
    txt = f"""# Reader feature scene: the directive and parameter forms the pbrt reader handles.
Scale -1 1 1   # handedness flip before the camera transform
ConcatTransform [ {col_major(cam)} ]
Camera "perspective" "float fov" 50 "float lensradius" [ 0.01 ] "float focaldistance" 3
Film "rgb" "integer xresolution" [ 96 ] "integer yresolution" 64
    "string filename" "features.exr"
Sampler "zsobol" "integer pixelsamples" [ 16 ]
Integrator "volpath" "integer maxdepth" [ 6 ] "bool regularize" true
PixelFilter "gaussian" "float xradius" [ 1.5 ]
WorldBegin

AttributeBegin
  Rotate -90 1 0 0
  LightSource "infinite" "string filename" "sky.pfm" "rgb scale" [ 1.5 1.2 0.9 ]
AttributeEnd

Texture "checks" "spectrum" "imagemap" "string filename" "checker.pfm"
Texture "mask" "float" "imagemap" "string filename" [ "alpha.pfm" ]
Texture "photo" "spectrum" "imagemap" "string filename" "photo.png"
Texture "marble" "spectrum" "marble" "float scale" 2

MakeNamedMaterial "floor" "string type" "diffuse" "texture reflectance" "checks"
MakeNamedMaterial "gold" "string type" "conductor"
    "spectrum eta" [ "metal-Au-eta" ] "spectrum k" [ "metal-Au-k" ] "float roughness" 0.2
MakeNamedMaterial "copper" "string type" "conductor" "spectrum eta" "metal-Cu-eta"
    "float uroughness" 0.1 "float vroughness" 0.3
MakeNamedMaterial "glass" "string type" "dielectric" "float eta" 1.33 "float roughness" [ 0.05 ]
MakeNamedMaterial "coat" "string type" "coateddiffuse" "rgb reflectance" [ 0.2 0.4 0.7 ]
    "float roughness" 0.3
MakeNamedMaterial "leaf" "string type" "diffusetransmission" "rgb reflectance" [ 0.3 0.6 0.2 ]
MakeNamedMaterial "odd" "string type" "measured" "rgb reflectance" [ 0.5 0.45 0.4 ] "float roughness" 0.4
MakeNamedMaterial "alu" "string type" "conductor" "rgb eta" [ 1.345 0.965 0.612 ]
    "rgb k" [ 7.474 6.4 5.275 ] "float uroughness" [ 0.05 ]
MakeNamedMaterial "photo" "string type" "diffuse" "texture reflectance" "photo"

AttributeBegin
  NamedMaterial "floor"
  Shape "trianglemesh" "point3 P" [ -3 0 -3  3 0 -3  3 0 3  -3 0 3 ]
      "integer indices" [ 0 1 2 0 2 3 ] "point2 uv" [ 0 0 3 0 3 3 0 3 ]
AttributeEnd

AttributeBegin
  NamedMaterial "gold"
  ConcatTransform [ 1 0 0 0  0 1 0 0  0 0 1 0  -0.9 0.5 0.2 1 ]
  Shape "sphere" "float radius" 0.5
AttributeEnd

AttributeBegin
  NamedMaterial "glass"
  Translate 5 0 0   # read and ignored, as the reference does
  Scale 0.8 0.8 0.8
  Rotate 25 0 1 0
  Shape "plymesh" "string filename" "mesh_binary.ply"
AttributeEnd

AttributeBegin
  NamedMaterial "coat"
  Transform [ 0.7 0 0 0  0 0.7 0 0  0 0 0.7 0  0.9 0.35 -0.4 1 ]
  Shape "plymesh" "string filename" "mesh_ascii.ply" "texture alpha" "mask"
AttributeEnd

Include "features_include.pbrt"

TransformBegin
  Rotate 45 0 0 1
TransformEnd
Material "diffuse" "rgb reflectance" [ 0.1 0.1 0.1 ]
MakeNamedMedium "fog" "string type" "homogeneous" "rgb sigma_a" [ 0.1 0.1 0.1 ]
MediumInterface "" "fog"
ReverseOrientation
Shape "cylinder" "float radius" 1 "float zmax" 2

AttributeBegin
  NamedMaterial "alu"
  ConcatTransform [ 1 0 0 0  0 1 0 0  0 0 1 0  0.2 0.01 0.9 1 ]
  Shape "trianglemesh" "point3 P" [ -0.3 0 -0.3  0.3 0 -0.3  0.3 0.4 0.3  -0.3 0.4 0.3 ]
      "normal N" [ 0 0.7 -0.7  0 0.7 -0.7  0 0.7 -0.7  0 0.7 -0.7 ]
      "integer indices" [ 0 1 2 0 2 3 ]
AttributeEnd

AttributeBegin
  NamedMaterial "odd"
  Scale 1 2 1
  Shape "trianglemesh" "point3 P" [ -1.5 0.2 -2  -0.5 0.2 -2  -1 0.9 -2 ] "integer indices" [ 0 1 2 ]
AttributeEnd

AttributeBegin
  NamedMaterial "photo"
  Shape "trianglemesh" "point3 P" [ 1.5 0.1 -2  2.5 0.1 -2  2 0.8 -2 ] "integer indices" [ 0 1 2 ]
      "point2 uv" [ 0 0 1 0 0.5 1 ]
AttributeEnd

AttributeBegin
  NamedMaterial "copper"
  Shape "trianglemesh" "point3 P" [ 0 0 0 1 0 0 0 1 0 ] "integer indices" [ ]
AttributeEnd
"""
    inc = """# Included from features.pbrt: instanced objects and area lights.
ObjectBegin "rock"
  NamedMaterial "leaf"
  Shape "sphere" "float radius" 0.15
  NamedMaterial "copper"
  Shape "trianglemesh" "point3 P" [ -0.2 0 -0.2  0.2 0 -0.2  0 0.3 0 ] "integer indices" [ 0 1 2 ]
ObjectEnd

AttributeBegin
  ConcatTransform [ 1 0 0 0  0 1 0 0  0 0 1 0  -1.8 0.15 1.2 1 ]
  ObjectInstance "rock"
AttributeEnd
AttributeBegin
  ConcatTransform [ 0 0 -1 0  0 1 0 0  1 0 0 0  1.7 0.15 1.0 1 ]
  ObjectInstance "rock"
AttributeEnd
ObjectInstance "nothing"

AttributeBegin
  AreaLightSource "diffuse" "rgb L" [ 6 5 4 ]
  NamedMaterial "leaf"
  Shape "trianglemesh" "point3 P" [ -0.4 2.2 -0.4  0.4 2.2 -0.4  0.4 2.2 0.4  -0.4 2.2 0.4 ]
      "integer indices" [ 0 2 1 0 3 2 ]
  AreaLightSource "diffuse" "blackbody L" [ 5500 ]
  Shape "sphere" "float radius" 0.05
AttributeEnd
"""
    return txt, inc


def main():
    with open(os.path.join(HERE, "box_room.pbrt"), "w") as f:
        f.write(box_room())
    txt, inc = features()
    with open(os.path.join(HERE, "features.pbrt"), "w") as f:
        f.write(txt)
    with open(os.path.join(HERE, "features_include.pbrt"), "w") as f:
        f.write(inc)


if __name__ == "__main__":
    main()
