"""Host-side parts of the C-ABI that need no GPU: the reference output step
(clamp + fastPow gamma, main.cpp:150-165) and the PNG / BMP writers."""
import struct
import zlib

import numpy as np

import _oracle as O
from eleven import _lib, scenes


def test_encode_ldr_matches_oracle():
    rng = np.random.default_rng(0)
    x = rng.uniform(-0.5, 1.5, (64 * 48 * 4,)).astype(np.float32)
    x[:8] = [0, 1, -0, 1e-30, 0.5, np.inf, -np.inf, 2.0]
    x[3::4] = 1.0
    a = _lib.encode_ldr(x, 64, 48)
    b = np.zeros_like(a)
    O.orc().orc_encode_ldr(O._ptr(x), len(x), b.ctypes.data_as(O.C.POINTER(O.C.c_uint8)))
    assert np.array_equal(a, b)
    # alpha 1 encodes to 250 through the approximate pow, as the reference writes it
    assert a[3] == 250


def test_fastpow_decode_matches_c():
    b = np.arange(256, dtype=np.uint8)
    got = scenes.decode_ldr(b, 2.2)
    x = (b.astype(np.float32) / np.float32(255.0)).astype(np.float64)
    ref = np.array([O.orc().orc_fastpow(float(v), float(np.float32(2.2))) for v in x], np.float32)
    assert np.array_equal(got, ref)
    assert np.all(np.diff(got[1:]) > 0)


def _png_pixels(data):
    assert data[:8] == b"\x89PNG\r\n\x1a\n"
    pos, idat, w, h = 8, b"", 0, 0
    while pos < len(data):
        n, = struct.unpack(">I", data[pos:pos + 4])
        typ = data[pos + 4:pos + 8]
        body = data[pos + 8:pos + 8 + n]
        crc, = struct.unpack(">I", data[pos + 8 + n:pos + 12 + n])
        assert crc == zlib.crc32(typ + body) & 0xFFFFFFFF
        if typ == b"IHDR":
            w, h = struct.unpack(">II", body[:8])
        elif typ == b"IDAT":
            idat += body
        pos += 12 + n
    raw = zlib.decompress(idat)
    rows = np.frombuffer(raw, np.uint8).reshape(h, 1 + 4 * w)
    assert (rows[:, 0] == 0).all()
    return rows[:, 1:].reshape(h, w, 4)


def test_png_and_bmp_writers(tmp_path):
    rng = np.random.default_rng(1)
    img = rng.integers(0, 256, (13, 17, 4), dtype=np.uint8)
    p = tmp_path / "out.png"
    _lib.write_image(str(p), img, 17, 13)
    assert np.array_equal(_png_pixels(p.read_bytes()), img)
    b = tmp_path / "out.bmp"
    _lib.write_image(str(b), img, 17, 13, as_bmp=True)
    data = b.read_bytes()
    assert data[:2] == b"BM"
    off, = struct.unpack("<I", data[10:14])
    w, h = struct.unpack("<ii", data[18:26])
    assert (w, h) == (17, 13)
    stride = (17 * 3 + 3) & ~3
    rows = np.frombuffer(data[off:off + stride * 13], np.uint8).reshape(13, stride)[::-1, :51].reshape(13, 17, 3)
    assert np.array_equal(rows[..., ::-1], img[..., :3])


def test_write_image_reports_io_errors(tmp_path):
    img = np.zeros((2, 2, 4), np.uint8)
    try:
        _lib.write_image(str(tmp_path / "no" / "such" / "dir.png"), img, 2, 2)
    except _lib.ElevenError as e:
        assert e.status == 2
    else:
        raise AssertionError("expected ER_ERR_IO")
