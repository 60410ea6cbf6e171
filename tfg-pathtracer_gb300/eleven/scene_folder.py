"""Write a SceneArrays as a reference scene folder.

Layout (SceneLoader.hpp:7-143): scene.json (camera, hdri, pointLights),
scene.obj (one `o` per mesh object, z negated because the loader negates it
back, ObjLoader.hpp:85,91), scene.mtl (Kd / Ks / Ke plus the Pr Pm Pc Ps
extension keys, map_Kd textures), HDRI/<name>.hdr (Radiance RGBE, rows in
file order) and textures/*.bmp (24-bit, bottom-up).

Numbers are written in positional notation with the shortest digits that
round-trip a float32: the reference's number scanner (Vector.hpp:15-62)
does not understand exponents.  Texture bytes must be the 8-bit values the
float texels were decoded from (SceneArrays.texture_bytes); normals should be
fixed points of the loader's normalisation (scenes.ref_normalize), so that
loading the folder reproduces the arrays bit for bit.
"""
from __future__ import annotations

import json
import os
import struct

import numpy as np

from . import scenes


def fnum(x):
    return np.format_float_positional(np.float32(x), unique=True, trim="-")


def write_bmp(path, rgb_rows_bottom_first):
    """24-bit BMP; the first stored row is the bottom of the picture."""
    img = np.ascontiguousarray(rgb_rows_bottom_first, np.uint8)
    h, w, _ = img.shape
    stride = (w * 3 + 3) & ~3
    pixels = bytearray()
    for r in range(h):
        row = img[r][:, ::-1].tobytes()  # BGR
        pixels += row + b"\0" * (stride - 3 * w)
    hdr = struct.pack("<2sIHHI", b"BM", 54 + len(pixels), 0, 0, 54)
    info = struct.pack("<IiiHHIIiiII", 40, w, h, 1, 24, 0, len(pixels), 2835, 2835, 0, 0)
    with open(path, "wb") as f:
        f.write(hdr + info + pixels)


def write_hdr(path, rgb):
    """Flat (uncompressed) Radiance RGBE, -Y h +X w, rows in array order."""
    rgbe = scenes.rgbe_encode(rgb)
    h, w, _ = rgbe.shape
    with open(path, "wb") as f:
        f.write(b"#?RADIANCE\nFORMAT=32-bit_rle_rgbe\n\n")
        f.write(f"-Y {h} +X {w}\n".encode())
        f.write(np.ascontiguousarray(rgbe).tobytes())


def write_folder(arrays, out_dir, env_name="env"):
    os.makedirs(out_dir, exist_ok=True)
    os.makedirs(os.path.join(out_dir, "HDRI"), exist_ok=True)
    cam = arrays.camera
    cj = {
        "xRes": int(cam["x_res"]), "yRes": int(cam["y_res"]),
        "focalLength": float(np.float32(cam["focal_length"])),
        "focusDistance": float(np.float32(cam.get("focus_distance", 1000000.0))),
        "aperture": float(np.float32(cam.get("aperture", 2.8))),
        "bokeh": bool(cam.get("bokeh", False)),
        "position": dict(zip("xyz", (float(np.float32(v)) for v in cam["position"]))),
        "rotation": dict(zip("xyz", (float(np.float32(v)) for v in cam.get("rotation", (0, 0, 0))))),
    }
    env = np.asarray(arrays.env, np.float32)
    const = env.shape[:2] == (1024, 1024) and np.all(env == env[0, 0])
    if const:
        hj = {"color": dict(zip("rgb", (float(v) for v in env[0, 0])))}
    else:
        write_hdr(os.path.join(out_dir, "HDRI", env_name + ".hdr"), env)
        hj = {"name": env_name}
    if arrays.env_offset[0]:
        hj["xOffset"] = float(np.float32(arrays.env_offset[0]))
    lights = []
    if arrays.lights is not None:
        for p, r in arrays.lights:
            lights.append({"position": dict(zip("xyz", (float(v) for v in p))),
                           "radiance": dict(zip("rgb", (float(v) for v in r)))})
    with open(os.path.join(out_dir, "scene.json"), "w") as f:
        json.dump({"camera": cj, "hdri": hj, "pointLights": lights}, f, indent=1)

    # textures
    tex_names = []
    if arrays.textures:
        if arrays.texture_bytes is None:
            raise ValueError("texture_bytes are needed to write textures")
        os.makedirs(os.path.join(out_dir, "textures"), exist_ok=True)
        for i, b in enumerate(arrays.texture_bytes):
            name = f"textures/tex{i}.bmp"
            write_bmp(os.path.join(out_dir, name), b)
            tex_names.append(name)
    # materials
    with open(os.path.join(out_dir, "scene.mtl"), "w") as f:
        for i, m in enumerate(arrays.materials):
            full = dict(scenes.MATERIAL_DEFAULTS)
            full.update(m)
            f.write(f"newmtl mat{i}\n")
            f.write("Kd " + " ".join(fnum(v) for v in full["albedo"]) + "\n")
            f.write("Ks " + " ".join(fnum(full["specular"]) for _ in range(3)) + "\n")
            f.write("Ke " + " ".join(fnum(v) for v in full["emission"]) + "\n")
            f.write(f"Pr {fnum(full['roughness'])}\nPm {fnum(full['metallic'])}\n")
            f.write(f"Pc {fnum(full['clearcoat'])}\nPs {fnum(full['sheen'])}\n")
            if full["albedo_tex"] >= 0:
                f.write(f"map_Kd {tex_names[full['albedo_tex']]}\n")
            f.write("\n")
    # geometry: objects are contiguous runs of tri_object
    P = np.asarray(arrays.positions, np.float32)
    N = np.asarray(arrays.normals, np.float32)
    U = np.asarray(arrays.uvs, np.float32)
    obj = np.asarray(arrays.tri_object)
    with open(os.path.join(out_dir, "scene.obj"), "w") as f:
        vbase = 1
        for o in range(len(arrays.object_material)):
            idx = np.nonzero(obj == o)[0]
            if len(idx) == 0:
                continue
            if not np.all(np.diff(idx) == 1):
                raise ValueError("triangles of an object must be contiguous")
            f.write(f"o obj{o}\nusemtl mat{int(arrays.object_material[o])}\n")
            lines = []
            for t in idx:
                for k in range(3):
                    v = P[t, k]
                    lines.append(f"v {fnum(v[0])} {fnum(v[1])} {fnum(-v[2])}\n")
            for t in idx:
                for k in range(3):
                    lines.append(f"vt {fnum(U[t, k, 0])} {fnum(U[t, k, 1])}\n")
            for t in idx:
                for k in range(3):
                    n = N[t, k]
                    lines.append(f"vn {fnum(n[0])} {fnum(n[1])} {fnum(-n[2])}\n")
            for j in range(len(idx)):
                a = vbase + 3 * j
                lines.append(f"f {a}/{a}/{a} {a + 1}/{a + 1}/{a + 1} {a + 2}/{a + 2}/{a + 2}\n")
            f.writelines(lines)
            vbase += 3 * len(idx)
    return out_dir
