"""Scene-folder loader (er_scene_load): parsing and its error statuses, on
the host.  Without a GPU a folder that parses completely reaches the device
step and reports ER_ERR_NO_DEVICE; with one it loads."""
import ctypes as C
import os
import shutil

import numpy as np
import pytest

from eleven import _abi as A
from eleven import _lib, scene_folder, scenes


def small_c1():
    return scenes.config1(x_res=48, y_res=27, n_meshes=3, tri_lo=200, tri_hi=400, tex_size=16, n_tex=2,
                          env_w=32, env_h=16)


def load_status(path):
    L = _lib.load()
    h = C.c_void_p()
    st = L.er_scene_load(os.fsencode(str(path)), None, C.byref(h))
    if st == 0:
        L.er_scene_free(h)
    return st, L.er_last_error().decode()


def ok_statuses():
    return (A.ER_OK, A.ER_ERR_NO_DEVICE)


@pytest.fixture()
def folder(tmp_path):
    return scene_folder.write_folder(small_c1(), str(tmp_path / "scene"))


def test_valid_folder_parses(folder):
    st, msg = load_status(folder)
    assert st in ok_statuses(), msg


def test_constant_env_folder_parses(tmp_path):
    d = scene_folder.write_folder(scenes.config0(16, 12, n_spheres=2, subdiv=1), str(tmp_path / "c0"))
    assert '"color"' in open(os.path.join(d, "scene.json")).read()
    st, msg = load_status(d)
    assert st in ok_statuses(), msg


def test_missing_folder_is_io_error(tmp_path):
    st, msg = load_status(tmp_path / "nope")
    assert st == A.ER_ERR_IO and "scene.json" in msg


def test_malformed_json(folder):
    with open(os.path.join(folder, "scene.json"), "w") as f:
        f.write('{"camera": {"xRes": 4, ')
    assert load_status(folder)[0] == A.ER_ERR_PARSE


def test_missing_camera(folder):
    with open(os.path.join(folder, "scene.json"), "w") as f:
        f.write('{"hdri": {"color": {"r": 1, "g": 1, "b": 1}}}')
    assert load_status(folder)[0] == A.ER_ERR_PARSE


def test_missing_obj(folder):
    os.remove(os.path.join(folder, "scene.obj"))
    st, msg = load_status(folder)
    assert st == A.ER_ERR_IO and "scene.obj" in msg


def test_missing_hdr(folder):
    shutil.rmtree(os.path.join(folder, "HDRI"))
    assert load_status(folder)[0] == A.ER_ERR_IO


def test_face_index_out_of_range(folder):
    with open(os.path.join(folder, "scene.obj"), "a") as f:
        f.write("f 1 2 999999\n")
    st, msg = load_status(folder)
    assert st == A.ER_ERR_PARSE and "index" in msg


def test_truncated_texture(folder):
    p = os.path.join(folder, "textures", "tex0.bmp")
    data = open(p, "rb").read()
    open(p, "wb").write(data[:100])
    assert load_status(folder)[0] == A.ER_ERR_PARSE


def test_unsupported_bmp_depth(folder):
    p = os.path.join(folder, "textures", "tex0.bmp")
    data = bytearray(open(p, "rb").read())
    data[28] = 16  # 16 bits per pixel
    open(p, "wb").write(bytes(data))
    assert load_status(folder)[0] == A.ER_ERR_UNSUPPORTED


def test_bad_hdr_header(folder):
    with open(os.path.join(folder, "HDRI", "env.hdr"), "wb") as f:
        f.write(b"#?NOTHDR\n\n")
    assert load_status(folder)[0] == A.ER_ERR_PARSE


def test_objects_before_first_o_line_are_ignored(folder, tmp_path):
    # the reference parses nothing before the first `o` line: a stray
    # triangle there does not change the scene
    obj = os.path.join(folder, "scene.obj")
    txt = open(obj).read()
    open(obj, "w").write("v 0 0 0\nv 1 0 0\nv 0 1 0\nf 1 2 3\n" + txt)
    st, msg = load_status(folder)
    assert st in ok_statuses(), msg


def test_cli_usage_and_errors():
    from eleven.build import CLI, build_product
    build_product()
    import subprocess
    r = subprocess.run([CLI], capture_output=True, text=True)
    assert r.returncode == 2 and "usage" in r.stderr
    r = subprocess.run([CLI, "/no/such/scene", "4", "/tmp/x.png"], capture_output=True, text=True)
    assert r.returncode == 1 and "scene.json" in r.stderr
