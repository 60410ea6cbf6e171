"""Generate tests/golden/reference_io.npz: golden outputs of the reference's
own scene loader and post-processing, for the host-side rows of the path
(scene folder, texture / HDR decode, post-process).

Every expected output comes from the REFERENCE's code compiled for the host
(oracle/_ref/libref.so, `make -C oracle ref`):
- loadScene (SceneLoader.hpp:7-143) with ObjLoader.hpp, RSJparser.hpp,
  stb_image's BMP / Radiance decode and its fastPow LDR->float mapping
  (stb_image.h:127-135,1855-1866, Texture.hpp:41-68, HDRI.hpp:42-60) and
  the MikkTSpace tangents, through oracle/ref_shim_scene.cpp, on the
  folders of tests/_ref_folders.py;
- applyExposure, basicBlur, reinhardTonemap, acesTonemap, clampPixels,
  applysRGB, flipX, flipY (PostProcessing.cpp:3-211) through
  oracle/ref_shim_post.cpp, on seeded images.

The folders are not stored: the tests re-make them from the same writers
and check their digests first.

Run from the repository root where the reference sources are present:
    python tests/golden/gen_golden_io.py
"""
import ctypes as C
import os
import sys
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, os.path.join(ROOT, "tfg-pathtracer_gb300"))
sys.path.insert(0, os.path.join(ROOT, "tests"))

import _ref_folders as RF  # noqa: E402
from eleven import _abi as A  # noqa: E402
from eleven import build  # noqa: E402

OUT = os.path.join(HERE, "reference_io.npz")

# post-processing cases: (exposure, tonemap, clamp, srgb, flip_x, flip_y, threshold, power, radius)
POST_CASES = [
    (1.0, 0, 1, 0, 0, 0, 0.0, 0.0, 0.0),
    (1.7, 1, 0, 1, 1, 0, 0.0, 0.0, 0.0),
    (0.6, 2, 1, 1, 0, 1, 0.0, 0.0, 0.0),
    (1.0, 0, 0, 0, 1, 1, 0.8, 0.5, 6.0),
    (1.3, 2, 1, 1, 0, 0, 1.5, 0.25, 9.0),
    (2.0, 1, 1, 1, 1, 1, 0.2, 1.0, 3.0),
]


def post_image(rng, w, h):
    px = np.exp(rng.normal(-0.5, 1.2, (h * w, 4))).astype(np.float32)
    px[:, 3] = 1.0
    px[rng.random(h * w) < 0.02, :3] = 0.0
    return px


def ref_lib():
    build.build_ref()
    L = C.CDLL(os.path.join(ROOT, "oracle", "_ref", "libref.so"))
    L.ref_folder_load.restype = C.c_void_p
    L.ref_folder_load.argtypes = [C.c_char_p]
    L.ref_folder_free.argtypes = [C.c_void_p]
    L.ref_folder_counts.argtypes = [C.c_void_p, C.c_void_p]
    L.ref_folder_tris.argtypes = [C.c_void_p] + [C.c_void_p] * 6
    L.ref_folder_objects.argtypes = [C.c_void_p, C.c_void_p, C.c_void_p]
    L.ref_folder_material.argtypes = [C.c_void_p, C.c_int32, C.POINTER(A.er_material)]
    L.ref_folder_texture.argtypes = [C.c_void_p, C.c_int32, C.c_void_p, C.c_void_p]
    L.ref_folder_env.argtypes = [C.c_void_p, C.c_void_p, C.c_void_p]
    L.ref_folder_camera.argtypes = [C.c_void_p, C.POINTER(A.er_camera)]
    L.ref_folder_lights.argtypes = [C.c_void_p, C.c_void_p]
    L.ref_postprocess.argtypes = [C.c_void_p, C.c_int32, C.c_int32, C.POINTER(A.er_post_opts)]
    return L


def p(a):
    return a.ctypes.data_as(C.c_void_p)


def load_reference_folder(L, name, tmp):
    d = RF.write(name, os.path.join(tmp, name))
    dig = RF.digest(d)
    RF.link_reference_names(d)
    h = L.ref_folder_load(os.fsencode(d))
    assert h, f"reference loadScene failed on {name}"
    c = np.zeros(7, np.int64)
    L.ref_folder_counts(h, p(c))
    T, n_obj, n_mat, n_tex, n_light, ew, eh = (int(x) for x in c)
    out = {"digest": np.frombuffer(bytes.fromhex(dig), np.uint8), "counts": c}
    pos, nrm, uv, tan = (np.zeros((T, 3, 3), np.float32) for _ in range(4))
    sign = np.zeros(T, np.float32)
    obj = np.zeros(T, np.int32)
    L.ref_folder_tris(h, p(pos), p(nrm), p(uv), p(tan), p(sign), p(obj))
    out.update(positions=pos, normals=nrm, uvs=uv, tangents=tan, tangent_sign=sign, tri_object=obj)
    om = np.zeros(n_obj, np.int32)
    otc = np.zeros(n_obj, np.int32)
    L.ref_folder_objects(h, p(om), p(otc))
    out.update(object_material=om, object_tri_count=otc)
    mats = (A.er_material * max(n_mat, 1))()
    for i in range(n_mat):
        L.ref_folder_material(h, i, C.byref(mats[i]))
    out["materials"] = np.frombuffer(bytes(mats), np.uint8)[:n_mat * C.sizeof(A.er_material)].copy()
    for i in range(n_tex):
        wh = np.zeros(2, np.int32)
        L.ref_folder_texture(h, i, p(wh), None)
        t = np.zeros((wh[1], wh[0], 3), np.float32)
        L.ref_folder_texture(h, i, p(wh), p(t))
        out[f"tex{i}"] = t
    env = np.zeros((eh, ew, 3), np.float32)
    to = np.zeros(4, np.float32)
    L.ref_folder_env(h, p(env), p(to))
    if ew * eh > 65536 and np.all(env == env[0, 0]):
        out["env_constant"] = env[0, 0].copy()  # the 1024x1024 expansion of a colour
    else:
        out["env"] = env
    out["env_tile_offset"] = to
    cam = A.er_camera()
    L.ref_folder_camera(h, C.byref(cam))
    out["camera"] = np.frombuffer(bytes(cam), np.uint8).copy()
    lights = (A.er_point_light * max(n_light, 1))()
    L.ref_folder_lights(h, lights)
    out["lights"] = np.frombuffer(bytes(lights), np.uint8)[:n_light * C.sizeof(A.er_point_light)].copy()
    L.ref_folder_free(h)
    return {f"{name}__{k}": v for k, v in out.items()}


def post_golden(L):
    rng = np.random.default_rng(11)
    w, h = 37, 23
    out = {}
    for k, case in enumerate(POST_CASES):
        px = post_image(rng, w, h)
        o = A.er_post_opts(*case)
        res = px.copy()
        L.ref_postprocess(p(res), w, h, C.byref(o))
        # pixels and channels basicBlur defines (see oracle/ref_shim_post.cpp)
        mask = np.ones((h, w, 4), bool)
        if case[7] != 0.0:
            b = int(case[8] / 2)
            inner = np.zeros((h, w), bool)
            inner[b:h - b, b:w - b] = True
            mask[~inner] = False
            mask[..., 3] = False
            if case[4]:
                mask = mask[:, ::-1]
            if case[5]:
                mask = mask[::-1]
        out[f"post{k}_in"] = px
        out[f"post{k}_out"] = res
        out[f"post{k}_mask"] = mask.reshape(h * w, 4)
        out[f"post{k}_opts"] = np.array(case, np.float64)
    out["post_wh"] = np.array([w, h], np.int32)
    return out


def main():
    L = ref_lib()
    data = {"folders": np.array(RF.FOLDERS)}
    with tempfile.TemporaryDirectory() as tmp:
        for name in RF.FOLDERS:
            data.update(load_reference_folder(L, name, tmp))
    data.update(post_golden(L))
    np.savez_compressed(OUT, **data)
    print(f"wrote {OUT} ({os.path.getsize(OUT)} bytes)")


if __name__ == "__main__":
    main()
