"""GPU BVH builder (ER_BUILDER_GPU): the hit set does not depend on the
tree, so scenes built on the GPU must trace and render exactly like the
host-built ones."""
import dataclasses

import numpy as np
import pytest

from eleven import _abi as A
from eleven import _lib, scenes

pytestmark = pytest.mark.gpu


def _same_hits(a, b, rays):
    t1, d1, uv1, _ = a.trace(rays)
    t2, d2, uv2, _ = b.trace(rays)
    assert np.array_equal(t1, t2), f"{int((t1 != t2).sum())} id mismatches"
    assert np.array_equal(d1.view(np.uint32), d2.view(np.uint32))
    assert np.array_equal(uv1.view(np.uint32), uv2.view(np.uint32))


@pytest.mark.parametrize("fmt", [A.ER_BVH_FP32, A.ER_BVH_Q8])
def test_gpu_built_scene_traces_and_renders_like_host_built(fmt):
    arrays = scenes.config0(x_res=64, y_res=48)
    host = _lib.Scene(arrays, bvh_format=fmt)
    gpu = _lib.Scene(arrays, bvh_format=fmt, builder=A.ER_BUILDER_GPU)
    _same_hits(host, gpu, scenes.random_rays(arrays, 200_000, seed=11))
    a = host.render(4, max_depth=4, seed=2)
    b = gpu.render(4, max_depth=4, seed=2)
    assert np.array_equal(a["beauty"].view(np.uint32), b["beauty"].view(np.uint32))
    assert np.array_equal(a["pathcount"], b["pathcount"])
    ig = gpu.info()
    assert ig.node_count > 0 and ig.leaf_count > 0 and ig.bvh_depth > 0
    host.close()
    gpu.close()


def test_gpu_builder_large_scene_and_build_time():
    arrays = scenes.config1(x_res=96, y_res=54)
    host = _lib.Scene(arrays)
    gpu = _lib.Scene(arrays, builder=A.ER_BUILDER_GPU)
    _same_hits(host, gpu, scenes.random_rays(arrays, 500_000, seed=12))
    hi, gi = host.info(), gpu.info()
    print(f"\nBVH build: host {hi.bvh_build_ms:.1f} ms ({hi.node_count} nodes), "
          f"GPU {gi.bvh_build_ms:.1f} ms ({gi.node_count} nodes)")
    assert gi.bvh_build_ms < hi.bvh_build_ms
    host.close()
    gpu.close()


@pytest.mark.parametrize("n", [1, 3, 5, 40])
def test_gpu_builder_small_and_degenerate(n):
    """Few triangles (a single-leaf root), and many triangles with one
    centroid (all Morton codes equal)."""
    arrays = scenes.config0(x_res=32, y_res=24)
    rng = np.random.default_rng(n)
    base = rng.uniform(-1, 1, (3, 3)).astype(np.float32)
    pos = np.stack([base + rng.normal(0, 0.01, (3, 3)).astype(np.float32) * (n > 5) for _ in range(n)])
    pos = pos - pos.mean(1, keepdims=True) + base.mean(0)  # identical centroids
    nrm = np.tile(np.array([0, 0, -1], np.float32), (n, 3, 1))
    small = dataclasses.replace(arrays, positions=pos.astype(np.float32), normals=nrm,
                                uvs=np.zeros((n, 3, 2), np.float32), tri_object=np.zeros(n, np.int32),
                                object_material=np.zeros(1, np.int32), materials=arrays.materials[:1])
    host = _lib.Scene(small)
    gpu = _lib.Scene(small, builder=A.ER_BUILDER_GPU)
    o = np.tile(np.array([0, 0, -5], np.float32), (4096, 1)) + rng.normal(0, 0.3, (4096, 3)).astype(np.float32)
    d = base.mean(0)[None, :] - o + rng.normal(0, 0.2, (4096, 3)).astype(np.float32)
    _same_hits(host, gpu, np.concatenate([o, d], 1))
    host.close()
    gpu.close()


def test_builder_option_is_checked():
    arrays = scenes.config0(x_res=16, y_res=12)
    with pytest.raises(_lib.ElevenError):
        _lib.Scene(arrays, builder=7)
