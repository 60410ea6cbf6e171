"""Host SAH BVH4 builder (csrc/bvh_build.cpp) checked on the CPU.

tests/bvh_check.cpp is compiled with the builder's source and walks the
FP32 tree and its 8-bit form: every triangle sits in exactly one leaf,
every vertex inside its leaf's box, every node is reached once from the
root, leaves hold at most 16 triangles, each 8-bit child box holds its
FP32 box, and the tree is shallow enough for the traversal's 96-entry
stack (3 * depth + 1 <= 96).  Closest hits do not depend on the tree's
shape, so these are the properties the traversal relies on; the GPU tests
check the hits themselves.
"""
import os
import shutil
import subprocess

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
CSRC = os.path.join(ROOT, "tfg-pathtracer_gb300", "csrc")
CUDA_INC = os.path.join(os.environ.get("CUDA_HOME", "/usr/local/cuda"), "include")


@pytest.fixture(scope="module")
def checker(tmp_path_factory):
    gxx = shutil.which("g++")
    if not gxx or not os.path.exists(os.path.join(CUDA_INC, "cuda_runtime.h")):
        pytest.skip("g++ or the CUDA headers are not available")
    exe = str(tmp_path_factory.mktemp("bvh") / "bvh_check")
    subprocess.run([gxx, "-O2", "-std=c++17", "-I" + os.path.join(ROOT, "include"), "-I" + CSRC, "-I" + CUDA_INC,
                    os.path.join(ROOT, "tests", "bvh_check.cpp"), os.path.join(CSRC, "bvh_build.cpp"), "-o", exe],
                   check=True, capture_output=True)
    return exe


def run(checker, tmp_path, tris):
    f = tmp_path / "tris.bin"
    np.ascontiguousarray(tris, np.float32).tofile(f)
    out = subprocess.run([checker, str(f)], check=True, capture_output=True, text=True).stdout
    return {k: int(v) for k, v in (kv.split("=") for kv in out.split())}


def check(r, n):
    assert r["missing"] == 0 and r["repeated"] == 0, r
    assert r["slots"] == n, r
    assert r["outside"] == 0 and r["badref"] == 0 and r["unreached"] == 0, r
    assert r["maxleaf"] <= 16 and r["q8_loose"] == 0, r
    assert 3 * r["depth"] + 1 <= 96, r


def small_triangles(rng, n, extent=10.0, size=0.05):
    c = rng.uniform(-extent, extent, (n, 1, 3))
    return (c + rng.normal(0, size, (n, 3, 3))).astype(np.float32)


def test_small_scene(checker, tmp_path):
    from eleven import scenes
    a = scenes.config0()
    r = run(checker, tmp_path, a.positions)
    check(r, a.tri_count)
    # the 4-wide collapse fills nodes: well under one node per two leaves
    assert r["nodes"] < 0.5 * r["leaves"], r


def test_random_triangles(checker, tmp_path):
    rng = np.random.default_rng(5)
    for n in (0, 1, 2, 3, 5, 17, 1000, 20000):
        check(run(checker, tmp_path, small_triangles(rng, n)), n)


def test_coincident_and_degenerate(checker, tmp_path):
    # one triangle repeated (all centroids equal: split by count), and
    # zero-area triangles at a few points
    t = np.array([[0, 0, 0], [1, 0, 0], [0, 1, 0]], np.float32)
    check(run(checker, tmp_path, np.repeat(t[None], 300, 0)), 300)
    rng = np.random.default_rng(6)
    pts = rng.uniform(-1, 1, (7, 3)).astype(np.float32)
    deg = np.repeat(pts[rng.integers(0, 7, 500)][:, None, :], 3, 1)
    check(run(checker, tmp_path, deg), 500)


def test_exponential_layout(checker, tmp_path):
    # centroids spaced by a constant factor: a deep, one-sided SAH tree
    n = 6000
    x = 1.01 ** np.arange(n)
    tris = np.zeros((n, 3, 3), np.float32)
    tris[:, :, 0] = (x[:, None] * np.array([1.0, 1.001, 1.0])).astype(np.float32)
    tris[:, 1, 1] = 1e-3
    tris[:, 2, 2] = 1e-3
    check(run(checker, tmp_path, tris), n)
