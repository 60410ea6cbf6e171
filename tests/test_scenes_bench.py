"""Scene generators (shapes of the benchmark configurations) and the
bench.py reference arm contract, on CPU."""
import json
import os
import subprocess
import sys

import numpy as np

from eleven import scenes

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def test_config0_shape():
    s = scenes.config0()
    assert s.tri_count == 16 * 1280 + 2
    assert s.camera["x_res"] == 320 and s.camera["y_res"] == 240
    assert len(s.materials) == 17 and len(s.lights) == 1
    assert s.env.shape == (1024, 1024, 3) and np.all(s.env == np.float32(0.5))
    # pinhole 45 degree horizontal field of view with the 35 mm sensor
    assert abs(2 * np.degrees(np.arctan(0.0175 / s.camera["focal_length"])) - 45.0) < 1e-4
    n = np.linalg.norm(s.normals.reshape(-1, 3), axis=1)
    assert np.allclose(n, 1, atol=1e-5)


def test_config0_deterministic():
    a, b = scenes.config0(), scenes.config0()
    assert np.array_equal(a.positions, b.positions)
    assert a.materials == b.materials


def test_config1_shape_small():
    s = scenes.config1(x_res=64, y_res=36, n_meshes=6, tex_size=32, n_tex=2, env_w=64, env_h=32)
    assert s.tri_count > 6 * 500
    assert len(s.textures) == 2 and s.textures[0].shape == (32, 32, 3)
    assert s.env.shape == (32, 64, 3) and s.env.max() >= 1e4 * 0.99
    assert s.camera["bokeh"]
    assert len(s.lights) == 4


def test_rgbe_roundtrip_is_idempotent():
    rng = np.random.default_rng(0)
    v = np.exp(rng.normal(0, 2, (100, 3))).astype(np.float32)
    once = scenes.rgbe_decode(scenes.rgbe_encode(v))
    twice = scenes.rgbe_decode(scenes.rgbe_encode(once))
    assert np.array_equal(once, twice)
    # shared exponent: error is relative to the largest channel
    assert (np.abs(once - v) <= v.max(1, keepdims=True) / 128).all()


def test_bench_reference_arm_contract():
    r = subprocess.run([sys.executable, os.path.join(ROOT, "bench.py"), "--impl", "reference", "--config", "c0",
                        "--steps", "1", "--warmup", "1"], capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stderr
    line = json.loads(r.stdout.strip().splitlines()[-1])
    for k in ("metric", "value", "unit", "n_gpus", "steps", "warmup", "ms_per_step", "higher_is_better",
              "scaling", "vs_baseline", "dtype", "data", "config", "cpu_baseline", "e2e"):
        assert k in line, k
    assert line["impl"] == "reference" and line["value"] > 0
    assert line["cpu_baseline"]["kind"] == "port"
    assert line["e2e"]["h2d_bytes_per_step"] == 0
