"""The C-ABI library loads, exports every symbol include/eleven.h declares,
agrees with the ctypes mirror on struct layouts, and rejects bad arguments
before touching a device."""
import ctypes as C
import os
import re
import subprocess
import sys

import numpy as np
import pytest

from eleven import _abi as A
from eleven import _lib, scenes

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
HEADER = os.path.join(ROOT, "include", "eleven.h")


def declared_functions():
    src = open(HEADER).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    return sorted(set(re.findall(r"\b(er_[a-z_0-9]+)\s*\(", src)))


def test_header_and_exports_agree():
    decl = declared_functions()
    assert sorted(A.EXPORTED) == decl
    L = _lib.load()
    for name in decl:
        assert hasattr(L, name), name


def test_flag_constants_agree():
    """Every `ER_X = 1u << n` / `ER_X = n` enum constant of the header has
    the same value in the ctypes mirror."""
    src = re.sub(r"/\*.*?\*/", "", open(HEADER).read(), flags=re.S)
    found = 0
    for name, shift, val in re.findall(r"\b(ER_[A-Z0-9_]+)\s*=\s*(?:1u?\s*<<\s*(\d+)|(\d+))\s*[,}\n]", src):
        if not hasattr(A, name):
            continue
        want = (1 << int(shift)) if shift else int(val)
        assert getattr(A, name) == want, name
        found += 1
    assert found >= 12


def test_library_exports_in_symbol_table():
    out = subprocess.run(["nm", "-D", "--defined-only", _lib.lib_path()], capture_output=True, text=True).stdout
    syms = {l.split()[-1] for l in out.splitlines() if l.strip()}
    for name in declared_functions():
        assert name in syms, name


STRUCTS = ["er_camera", "er_material", "er_texture", "er_point_light", "er_scene_desc", "er_scene_opts",
           "er_scene_info", "er_render_opts", "er_render_stats", "er_trace_stats", "er_batch_job",
           "er_batch_tuning", "er_post_opts"]


def test_struct_layouts(tmp_path):
    prog = tmp_path / "sz.c"
    body = "".join(f'printf("{s} %zu\\n", sizeof({s}));' for s in STRUCTS)
    prog.write_text(f'#include <stdio.h>\n#include "eleven.h"\nint main(void){{{body}return 0;}}\n')
    exe = tmp_path / "sz"
    subprocess.run(["gcc", "-I", os.path.join(ROOT, "include"), str(prog), "-o", str(exe)], check=True)
    sizes = dict(l.split() for l in subprocess.run([str(exe)], capture_output=True, text=True).stdout.splitlines())
    for s in STRUCTS:
        assert int(sizes[s]) == C.sizeof(getattr(A, s)), s


def test_status_strings_and_version():
    L = _lib.load()
    assert L.er_abi_version() == 1
    for code in range(10):
        assert L.er_status_string(code)
    assert L.er_status_string(12345) == b"unknown status"


def test_invalid_arguments_rejected():
    L = _lib.load()
    h = C.c_void_p()
    assert L.er_scene_create(None, None, C.byref(h)) == A.ER_ERR_INVALID_ARG
    assert L.er_last_error()
    arr = scenes.config0(8, 6, n_spheres=1, subdiv=0)
    arr.positions = arr.positions.copy()
    arr.positions[0, 0, 0] = np.nan
    d, keep = arr.desc()
    assert L.er_scene_create(C.byref(d), None, C.byref(h)) == 1
    arr = scenes.config0(8, 6, n_spheres=1, subdiv=0)
    arr.object_material = np.full_like(arr.object_material, 99)
    d, keep = arr.desc()
    assert L.er_scene_create(C.byref(d), None, C.byref(h)) == 1
    assert b"object_material" in L.er_last_error()
    arr = scenes.config0(0, 6, n_spheres=1, subdiv=0)
    d, keep = arr.desc()
    assert L.er_scene_create(C.byref(d), None, C.byref(h)) == 1
    assert L.er_scene_free(None) == 0
    assert L.er_trace_closest(None, None, 0, None, None, None, 0, None) == 1
    assert L.er_render(None, None, None, None, None, None, None, None, None) == 1
    assert L.er_film_read_sums(None, 0, None, None) == A.ER_ERR_INVALID_ARG


def test_render_options_checked_before_the_scene():
    """Options are validated before the scene handle is touched: the last
    sample index sample_begin + spp - 1 must fit the device's int32 sample
    counter (a large sample_begin, as sharded runs pass it, would otherwise
    wrap and repeat random streams)."""
    L = _lib.load()
    o = A.er_render_opts(4, 2**31 - 2, 4, 0, 0, 0, 0)
    for call in (lambda: L.er_render(None, C.byref(o), None, None, None, None, None, None, None),
                 lambda: L.er_render_noalloc(None, C.byref(o), None, None, None),
                 lambda: L.er_render_paths(None, C.byref(o), None, None)):
        assert call() == A.ER_ERR_INVALID_ARG
        assert b"INT32_MAX" in L.er_last_error()
    o.sample_begin = 2**31 - 5  # the last sample index is INT32_MAX - 1: accepted, then the NULL scene
    assert L.er_render(None, C.byref(o), None, None, None, None, None, None, None) == A.ER_ERR_INVALID_ARG
    assert b"NULL" in L.er_last_error()


def test_descriptor_checks_before_any_device_call():
    """NULL arrays with positive counts and non-finite camera fields are
    rejected as invalid arguments (no device is touched first)."""
    L = _lib.load()
    h = C.c_void_p()
    arr = scenes.config0(8, 6, n_spheres=1, subdiv=0)

    def rejected(edit, word):
        d, keep = arr.desc()
        edit(d)
        assert L.er_scene_create(C.byref(d), None, C.byref(h)) == A.ER_ERR_INVALID_ARG
        assert word in L.er_last_error(), L.er_last_error()
        assert not h.value

    rejected(lambda d: setattr(d, "materials", None), b"materials is NULL")
    def no_textures(d):
        d.texture_count = 1
        d.textures = None
    rejected(no_textures, b"textures is NULL")
    rejected(lambda d: setattr(d, "lights", None), b"lights is NULL")

    def nan_pose(d):
        d.camera.position[1] = float("nan")
    rejected(nan_pose, b"camera pose")

    def inf_focal(d):
        d.camera.focal_length = float("inf")
    rejected(inf_focal, b"camera parameter")
    assert L.er_scene_set_camera(None, None) == A.ER_ERR_INVALID_ARG


def test_host_allocation_failure_is_a_status(tmp_path):
    """A C++ exception does not cross the ABI: a PNG of 2^30 x 2^30 pixels
    (the encoder reserves ~4.6 EB before reading a pixel) is ER_ERR_OOM.
    Run in a child process, so that an escaped exception shows as its exit
    status instead of ending the test run."""
    code = ("import ctypes as C, sys\n"
            f"sys.path.insert(0, {os.path.join(ROOT, 'tfg-pathtracer_gb300')!r})\n"
            "from eleven import _lib\n"
            "L = _lib.load()\n"
            "px = (C.c_uint8 * 4)()\n"
            f"st = L.er_write_image({str(tmp_path / 'big.png').encode()!r}, px, 1 << 30, 1 << 30, 0)\n"
            "print(st, L.er_last_error().decode())\n")
    r = subprocess.run([sys.executable, "-c", code], capture_output=True, text=True, timeout=120)
    assert r.returncode == 0, r.stderr[-2000:]
    st, msg = r.stdout.strip().split(" ", 1)
    assert int(st) == A.ER_ERR_OOM and "er_write_image" in msg, r.stdout
    assert not (tmp_path / "big.png").exists()
    # a BMP's sizes are 32-bit: 70000 x 70000 is refused before any pixel is read
    L = _lib.load()
    px = (C.c_uint8 * 4)()
    assert L.er_write_image(str(tmp_path / "big.bmp").encode(), px, 70000, 70000, 1) == A.ER_ERR_INVALID_ARG
    assert b"BMP" in L.er_last_error()


def test_no_device_is_reported_not_faked():
    """Without a GPU the library reports it; there is no CPU fallback."""
    try:
        import torch
        has_gpu = torch.cuda.is_available()
    except Exception:
        has_gpu = False
    if has_gpu:
        pytest.skip("a GPU is visible")
    with pytest.raises(_lib.ElevenError) as e:
        _lib.Scene(scenes.config0(8, 6, n_spheres=1, subdiv=0))
    assert e.value.status == 9
