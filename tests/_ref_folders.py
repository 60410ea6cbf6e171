"""Scene folders that pin the loader to the reference's own loadScene
(test infrastructure).

Each writer makes a folder deterministically from a seed; the golden
generator (tests/golden/gen_golden_io.py) runs the reference's loader on it
(oracle/_ref/libref.so) and the tests re-make the same bytes (checked by
digest) and parse them with er_scene_folder_read.

- `c1_small`: the generator's full-feature scene at a small size (displaced
  spheres, 24-bit BMP textures, flat RGBE environment, 4 point lights),
  written by eleven.scene_folder, plus an hdri.yOffset (which the reference
  stores in the x offset, SceneLoader.hpp:64-65).
- `c0_small`: the small scene (icospheres, ground quad, constant colour
  environment expanded to 1024x1024, HDRI.hpp:22-38).
- `edge`: hand-written files that reach the parsing corners of
  SceneLoader.hpp / ObjLoader.hpp / stb_image: 32-bit and 8-bit paletted
  BMPs read as linear maps (map_Ns, refl), a top-down 24-bit BMP, a texture
  shared by two materials, a run-length-encoded HDR environment with both
  offsets, Ke / Ni / d lines, an unknown and a missing `usemtl`, vertex lines
  before the first `o` (never parsed, so they do not count in the face
  indices), faces given as v, v//vn and v/vt, a number with an exponent
  (read by the reference's digit scanner, Vector.hpp:15-62), a JSON number
  with an exponent, and a light given by r/g/b keys.
- `bare_camera`: a scene.json whose camera has only its resolution (the
  reference reads every other field as 0) and a constant environment with
  an x offset, no .mtl file (one default material, Material.hpp:21-36).

The .mtl of every folder keeps to the keys the reference reads (Kd, Ks, Ke,
Ni, d and the maps): the Pr/Pm/Pc/Ps extension keys of eleven.scene_folder
are removed.
"""
import hashlib
import json
import os
import struct

import numpy as np

from eleven import scene_folder, scenes

FOLDERS = ("c1_small", "c0_small", "edge", "bare_camera")


def _strip_extension_keys(d):
    mtl = os.path.join(d, "scene.mtl")
    lines = [ln for ln in open(mtl).read().splitlines(True) if ln.split(" ")[0] not in ("Pr", "Pm", "Pc", "Ps")]
    with open(mtl, "w") as f:
        f.write("".join(lines))


def c1_small(d):
    arrays = scenes.config1(x_res=48, y_res=27, n_meshes=3, tri_lo=200, tri_hi=400, tex_size=16, n_tex=2,
                            env_w=32, env_h=16)
    scene_folder.write_folder(arrays, d)
    _strip_extension_keys(d)
    p = os.path.join(d, "scene.json")
    j = json.load(open(p))
    j["hdri"]["xOffset"] = 0.375
    j["hdri"]["yOffset"] = 0.25
    with open(p, "w") as f:
        json.dump(j, f, indent=1)
    return d


def c0_small(d):
    scene_folder.write_folder(scenes.config0(32, 24, n_spheres=3, subdiv=1), d)
    _strip_extension_keys(d)
    return d


# ------------------------------------------------------------------ images

def _bmp(path, w, h, bpp, pixel_bytes, palette=None, top_down=False):
    """BMP with a BITMAPINFOHEADER; pixel_bytes = rows as stored (padded)."""
    pal = b"" if palette is None else bytes(palette)
    off = 14 + 40 + len(pal)
    hdr = struct.pack("<2sIHHI", b"BM", off + len(pixel_bytes), 0, 0, off)
    ncol = 0 if palette is None else len(palette) // 4
    info = struct.pack("<IiiHHIIiiII", 40, w, -h if top_down else h, 1, bpp, 0, len(pixel_bytes), 2835, 2835, ncol,
                       0)
    with open(path, "wb") as f:
        f.write(hdr + info + pal + pixel_bytes)


def _rows(img, bytes_per_px):
    h, w = img.shape[:2]
    stride = (w * bytes_per_px + 3) & ~3
    out = bytearray()
    for r in range(h):
        row = img[r].tobytes()
        out += row + b"\0" * (stride - len(row))
    return bytes(out)


def bmp24(path, rgb, top_down=False):
    _bmp(path, rgb.shape[1], rgb.shape[0], 24, _rows(rgb[..., ::-1].copy(), 3), top_down=top_down)


def bmp32(path, rgba):
    bgra = rgba[..., [2, 1, 0, 3]].copy()
    _bmp(path, rgba.shape[1], rgba.shape[0], 32, _rows(bgra, 4))


def bmp8(path, idx, palette_rgb):
    pal = bytearray()
    for r, g, b in palette_rgb:
        pal += bytes((b, g, r, 0))
    _bmp(path, idx.shape[1], idx.shape[0], 8, _rows(idx.astype(np.uint8), 1), palette=pal)


def _rle_channel(v):
    """Radiance new-style run-length coding of one channel of a scanline."""
    out = bytearray()
    i, n = 0, len(v)
    while i < n:
        j = i
        while j < n and j - i < 127 and v[j] == v[i]:
            j += 1
        if j - i >= 3:
            out += bytes((128 + j - i, v[i]))
            i = j
            continue
        j = i
        while j < n and j - i < 128 and not (j + 2 < n and v[j] == v[j + 1] == v[j + 2]):
            j += 1
        out += bytes((j - i,)) + bytes(v[i:j])
        i = j
    return bytes(out)


def hdr_rle(path, rgb):
    rgbe = scenes.rgbe_encode(rgb)
    h, w, _ = rgbe.shape
    body = bytearray()
    for y in range(h):
        body += bytes((2, 2, w >> 8, w & 255))
        for c in range(4):
            body += _rle_channel(rgbe[y, :, c].tolist())
    with open(path, "wb") as f:
        f.write(b"#?RADIANCE\n# run-length coded\nFORMAT=32-bit_rle_rgbe\n\n")
        f.write(f"-Y {h} +X {w}\n".encode())
        f.write(bytes(body))


# ------------------------------------------------------------------ folders

def edge(d, seed=7):
    rng = np.random.default_rng(seed)
    os.makedirs(os.path.join(d, "HDRI"), exist_ok=True)
    os.makedirs(os.path.join(d, "tex"), exist_ok=True)
    # environment: 32x16 with runs (constant spans) and noise
    env = np.exp(rng.normal(0, 1.5, (16, 32, 1))).astype(np.float32) * np.ones(3, np.float32)
    env[:, 8:20] = env[:, 8:9]
    env[3] = [4.0, 2.0, 1.0]
    hdr_rle(os.path.join(d, "HDRI", "sky.hdr"), env)
    # textures
    bmp24(os.path.join(d, "tex", "albedo_td.bmp"), rng.integers(0, 256, (12, 10, 3), dtype=np.uint8), top_down=True)
    rgba = rng.integers(0, 256, (9, 7, 4), dtype=np.uint8)
    bmp32(os.path.join(d, "tex", "rough32.bmp"), rgba)
    pal = [tuple(int(x) for x in rng.integers(0, 256, 3)) for _ in range(16)]
    bmp8(os.path.join(d, "tex", "metal8.bmp"), rng.integers(0, 16, (6, 11)), pal)
    bmp24(os.path.join(d, "tex", "plain.bmp"), rng.integers(0, 256, (5, 6, 3), dtype=np.uint8))
    with open(os.path.join(d, "scene.json"), "w") as f:
        f.write("""{
 "camera": {"xRes": 64, "yRes": 48, "focalLength": 0.05, "focusDistance": 7.5, "aperture": 1.8,
            "bokeh": true, "position": {"x": 0.5, "y": 1.25, "z": -9},
            "rotation": {"x": 5, "y": -10.5, "z": 2.25}},
 "hdri": {"name": "sky", "xOffset": 0.25, "yOffset": 0.125},
 "pointLights": [
  {"position": {"x": 1, "y": 6, "z": -2}, "radiance": {"r": 40, "g": 30.5, "b": 1.5e2}},
  {"position": {"x": -3.25, "y": 2, "z": 4}, "radiance": {"x": 5, "y": 6, "z": 7}}
 ]
}
""")
    with open(os.path.join(d, "scene.mtl"), "w") as f:
        f.write("""# materials
newmtl red
Kd 0.8 0.1 0.05
Ks 0.25 0.9 0.9
Ke 0 0 0
Ni 1.45
d 1
map_Kd tex/albedo_td.bmp
map_Ns tex/rough32.bmp

newmtl lamp
Kd 1 1 1
Ke 2.5 2 1.5
refl tex/metal8.bmp

newmtl shared
Kd .5 -.25 0.125
map_Kd tex/albedo_td.bmp
map_Bump tex/plain.bmp
""")
    # geometry: stray vertices before the first object, then three objects
    lines = ["# stray data: not parsed by the reference\n", "v 9 9 9\n", "v 8 8 8\n", "v 7 7 7\n", "f 1 2 3\n"]
    P = rng.uniform(-2, 2, (12, 3)).round(4)
    T = rng.uniform(0, 1, (12, 2)).round(4)
    N = rng.normal(size=(12, 3)).round(4)
    lines.append("o first\nusemtl red\n")
    for p in P[:6]:
        lines.append(f"v {p[0]} {p[1]} {p[2]}\n")
    lines.append("v 1e-3 2 3\n")  # read as (1, -3, 2) by the digit scanner
    for t in T[:6]:
        lines.append(f"vt {t[0]} {t[1]}\n")
    for n in N[:6]:
        lines.append(f"vn {n[0]} {n[1]} {n[2]}\n")
    lines += ["f 1/1/1 2/2/2 3/3/3\n", "f 4/4/4 5/5/5 6/6/6\n", "f 1//2 3//4 7//6\n", "f 2/3 4/5 6/6\n",
              "f 5 6 7\n"]
    lines.append("o second\nusemtl nosuchmaterial\n")
    for p in P[6:]:
        lines.append(f"v {p[0]} {p[1]} {p[2]}\n")
    for t in T[6:]:
        lines.append(f"vt {t[0]} {t[1]} 0.5\n")
    for n in N[6:]:
        lines.append(f"vn {n[0]} {n[1]} {n[2]}\n")
    lines += ["f 8/7/7 9/8/8 10/9/9\n", "f 11/10/10 12/11/11 13/12/12\n", "f 8/12/7 10/7/8 12/9/11\n"]
    lines.append("o third\n")  # no usemtl: material 0
    lines += ["f 1/1/1 8/7/7 13/12/12\n", "f 2/2/2 3/3/3 9/8/8\n"]
    lines.append("o fourth\nusemtl lamp\nusemtl shared\n")
    lines += ["f 3/3/3 4/4/4 5/5/5\n"]
    with open(os.path.join(d, "scene.obj"), "w") as f:
        f.writelines(lines)
    return d


def bare_camera(d, seed=9):
    rng = np.random.default_rng(seed)
    with open(os.path.join(d, "scene.json"), "w") as f:
        f.write('{"camera": {"xRes": 20, "yRes": 10},\n "hdri": {"color": {"r": 0.25, "g": 0.5, "b": 2}, '
                '"xOffset": 0.5},\n "pointLights": []}\n')
    P = rng.uniform(-1, 1, (4, 3)).round(3)
    with open(os.path.join(d, "scene.obj"), "w") as f:
        f.write("o quad\n")
        for p in P:
            f.write(f"v {p[0]} {p[1]} {p[2]}\n")
        f.write("vn 0 1 0\nvt 0 0\nvt 1 0\nvt 1 1\nvt 0 1\n")
        f.write("f 1/1/1 2/2/1 3/3/1\nf 1/1/1 3/3/1 4/4/1\n")
    return d


WRITERS = {"c1_small": c1_small, "c0_small": c0_small, "edge": edge, "bare_camera": bare_camera}


def write(name, d):
    os.makedirs(d, exist_ok=True)
    WRITERS[name](d)
    return d


def digest(d):
    """sha256 over the folder's regular files (names and bytes)."""
    h = hashlib.sha256()
    for root, _, files in sorted(os.walk(d)):
        for fn in sorted(files):
            p = os.path.join(root, fn)
            if os.path.islink(p) or "\\" in fn:
                continue
            h.update(os.path.relpath(p, d).encode())
            h.update(open(p, "rb").read())
    return h.hexdigest()


def link_reference_names(d):
    """The names the reference's loadScene opens from inside the folder when
    it is given an empty path ("\\scene.json", ...), linked to the files."""
    for name in ("scene.json", "scene.mtl", "scene.obj"):
        if os.path.exists(os.path.join(d, name)):
            os.symlink(name, os.path.join(d, "\\" + name))
    j = json.load(open(os.path.join(d, "scene.json")))
    if "name" in j.get("hdri", {}):
        n = j["hdri"]["name"] + ".hdr"
        os.symlink(os.path.join("HDRI", n), os.path.join(d, "\\HDRI\\" + n))
