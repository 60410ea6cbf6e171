"""er_scene_load on corrupted scene folders (CPU): truncations, byte flips,
hostile lines in the OBJ/MTL, odd JSON values, and BMP/HDR header fields
out of range.  Every load returns a status (the folder's own, or the device
step's when it parses) and never crashes; headers that claim more pixels
than their files hold are rejected before anything is allocated for them.

The loads run in a child process, so that a crash shows as its exit
signal, from an empty working directory (texture paths are tried against
the working directory first, as the reference does).
"""
import os
import struct
import subprocess
import sys

import pytest

from eleven import _abi as A
from eleven import scene_folder, scenes

PKG = os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))), "tfg-pathtracer_gb300")

CHILD = r"""
import ctypes as C, os, random, shutil, sys
sys.path.insert(0, {pkg!r})
from eleven import _lib
src, work, n, seed = {src!r}, {work!r}, {n}, {seed}
L = _lib.load()
rng = random.Random(seed)
files = sorted(os.path.relpath(os.path.join(d, f), src) for d, _, fs in os.walk(src) for f in fs)
LINES = [b"f", b"f 1", b"f 0 0 0", b"f -1 -2 -3", b"f 1/2/3 4//5 6/7", b"f 2147483647 1 2", b"f 1 2 -2147483648",
         b"v nan nan nan", b"v 1e39 -1e39 0", b"v", b"vt", b"vn 0 0", b"usemtl", b"usemtl nosuch", b"o", b"g",
         b"mtllib", b"mtllib nosuch.mtl", b"newmtl", b"Kd 1", b"Ks", b"map_Kd", b"map_Kd nosuch.bmp",
         b"Ni -1e40", b"Pr nan", b"s off", b"#" + b"x" * 5000, b"\x00\x01\x02", b"f " + b"1 " * 5000]
JSON = [b"1e400", b"-1", b"0", b"NaN", b"99999999999999", b'"s"', b"[]", b"{{}}", b"null", b"-0.0"]
HDR_DIMS = [0, 1, 7, 8, 127, 32767, 32768, 65536, 65537, -5]
seen = {{}}
for it in range(n):
    shutil.rmtree(work, ignore_errors=True)
    shutil.copytree(src, work)
    name = rng.choice(files)
    p = os.path.join(work, name)
    data = bytearray(open(p, "rb").read())
    kind = rng.randrange(5)
    if kind == 0 and data:
        data = data[:rng.randrange(len(data))]
    elif kind == 1 and data:
        for _ in range(rng.randint(1, 8)):
            data[rng.randrange(len(data))] = rng.randrange(256)
    elif kind == 2 and name.endswith((".obj", ".mtl")):
        lines = bytes(data).split(b"\n")
        lines.insert(rng.randrange(len(lines) + 1), rng.choice(LINES))
        data = bytearray(b"\n".join(lines))
    elif kind == 3 and name.endswith(".json"):
        digits = [i for i, c in enumerate(data) if chr(c).isdigit()]
        if digits:
            i = rng.choice(digits)
            j = i
            while j < len(data) and (chr(data[j]).isdigit() or data[j] in b".eE-+"):
                j += 1
            data[i:j] = rng.choice(JSON)
    elif name.endswith(".bmp") and len(data) >= 54:
        off = rng.choice([10, 14, 18, 22, 28, 30, 46])
        data[off:off + 4] = (rng.choice([0, 1, 8, 24, 32, 65536, 65537, 2**31 - 1, 2**32 - 1]) & 0xFFFFFFFF
                             ).to_bytes(4, "little")
    elif name.endswith(".hdr"):
        head, sep, rest = bytes(data).partition(b"\n\n")
        line, nl, body = rest.partition(b"\n")
        dims = b"-Y %d +X %d" % (rng.choice(HDR_DIMS), rng.choice(HDR_DIMS))
        data = bytearray(head + sep + dims + nl + body)
    open(p, "wb").write(bytes(data))
    h = C.c_void_p()
    st = L.er_scene_load(os.fsencode(work), None, C.byref(h))
    if st == 0:
        L.er_scene_free(h)
    seen[st] = seen.get(st, 0) + 1
print(seen)
"""


@pytest.mark.parametrize("seed", [1, 2])
def test_corrupted_folders_return_a_status(tmp_path, seed):
    arrays = scenes.config1(x_res=32, y_res=18, n_meshes=2, tri_lo=100, tri_hi=200, tex_size=16, n_tex=2,
                            env_w=32, env_h=16)
    src = scene_folder.write_folder(arrays, str(tmp_path / "scene"))
    cwd = tmp_path / "cwd"
    cwd.mkdir()
    code = CHILD.format(pkg=PKG, src=src, work=str(tmp_path / "work"), n=400, seed=seed)
    r = subprocess.run([sys.executable, "-c", code], cwd=str(cwd), capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, f"loader crashed (exit {r.returncode}): {r.stderr[-2000:]}"
    seen = eval(r.stdout.strip().splitlines()[-1])
    print(f"\nstatuses over 400 corrupted loads (seed {seed}): {seen}")
    valid = {A.ER_OK, A.ER_ERR_INVALID_ARG, A.ER_ERR_IO, A.ER_ERR_PARSE, A.ER_ERR_UNSUPPORTED, A.ER_ERR_NO_DEVICE,
             A.ER_ERR_OOM}
    assert set(seen) <= valid, seen
    assert sum(seen.values()) == 400
    assert len(seen) >= 3  # the corruptions reach several different checks


def test_hdr_header_larger_than_its_file_is_rejected_before_allocation(tmp_path):
    """A 40-byte file claiming 65536 x 65536 texels (51 GB of floats) is a
    parse error at once."""
    import ctypes as C
    from eleven import _lib
    arrays = scenes.config1(x_res=16, y_res=9, n_meshes=1, tri_lo=100, tri_hi=200, tex_size=8, n_tex=1,
                            env_w=16, env_h=8)
    d = scene_folder.write_folder(arrays, str(tmp_path / "scene"))
    env = [f for f in os.listdir(os.path.join(d, "HDRI"))][0]
    with open(os.path.join(d, "HDRI", env), "wb") as f:
        f.write(b"#?RADIANCE\nFORMAT=32-bit_rle_rgbe\n\n-Y 65536 +X 65536\n" + struct.pack("4B", 2, 2, 1, 0))
    L = _lib.load()
    h = C.c_void_p()
    st = L.er_scene_load(os.fsencode(d), None, C.byref(h))
    assert st == A.ER_ERR_PARSE
    assert b"truncated HDR" in L.er_last_error()
