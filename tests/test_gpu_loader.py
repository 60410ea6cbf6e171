"""Scene folders on the GPU: a folder written from arrays and loaded back
renders bit for bit like the arrays, and the command-line renderer writes
the reference's encoded image."""
import os
import struct
import subprocess
import zlib

import numpy as np
import pytest

from eleven import _lib, scene_folder, scenes
from eleven.build import CLI

pytestmark = pytest.mark.gpu


def small_c1():
    return scenes.config1(x_res=64, y_res=36, n_meshes=5, tri_lo=300, tri_hi=1500, tex_size=32, n_tex=3,
                          env_w=64, env_h=32)


def test_folder_roundtrip_renders_identically(tmp_path):
    arrays = small_c1()
    d = scene_folder.write_folder(arrays, str(tmp_path / "s"))
    a = _lib.Scene(arrays)
    b = _lib.Scene.load_folder(d)
    assert b.info().tri_count == arrays.tri_count
    assert b.resolution == (64, 36)
    ra = a.render(spp=4, max_depth=6, seed=1)
    rb = b.render(spp=4, max_depth=6, seed=1)
    assert np.array_equal(ra["beauty"], rb["beauty"])
    assert np.array_equal(ra["pathcount"], rb["pathcount"])
    a.close()
    b.close()


def test_constant_env_folder(tmp_path):
    arrays = scenes.config0(48, 36, n_spheres=4, subdiv=2)
    d = scene_folder.write_folder(arrays, str(tmp_path / "c0"))
    a = _lib.Scene(arrays)
    b = _lib.Scene.load_folder(d)
    assert np.array_equal(a.render(spp=2, max_depth=4)["beauty"], b.render(spp=2, max_depth=4)["beauty"])


def read_png(path):
    data = open(path, "rb").read()
    pos, idat, w, h = 8, b"", 0, 0
    while pos < len(data):
        n, = struct.unpack(">I", data[pos:pos + 4])
        typ = data[pos + 4:pos + 8]
        body = data[pos + 8:pos + 8 + n]
        if typ == b"IHDR":
            w, h = struct.unpack(">II", body[:8])
        elif typ == b"IDAT":
            idat += body
        pos += 12 + n
    raw = np.frombuffer(zlib.decompress(idat), np.uint8).reshape(h, 1 + 4 * w)
    return raw[:, 1:].reshape(h, w, 4)


def test_cli_renders_scene_folder(tmp_path):
    arrays = small_c1()
    d = scene_folder.write_folder(arrays, str(tmp_path / "s"))
    out = str(tmp_path / "out.bmp")  # PNG content despite the name, as the reference
    r = subprocess.run([CLI, d, "4", out, "--max-depth", "6", "--seed", "1"], capture_output=True, text=True,
                       timeout=300)
    assert r.returncode == 0, r.stderr
    assert "kPaths/s" in r.stdout
    img = read_png(out)
    with _lib.Scene(arrays) as s:
        beauty = s.render(spp=4, max_depth=6, seed=1)["beauty"]
    ref = _lib.encode_ldr(beauty, 64, 36).reshape(36, 64, 4)
    assert np.array_equal(img, ref)
    bmp = str(tmp_path / "real.bmp")
    r = subprocess.run([CLI, d, "1", bmp, "--bmp"], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0 and open(bmp, "rb").read(2) == b"BM"
