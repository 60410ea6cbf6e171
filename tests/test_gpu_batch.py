"""GPU: batched rendering (er_batch) against single-scene renders.

Every job of a batch must produce the film er_render produces for the same
scene, camera and options, bit for bit, whatever the schedule: waves of
any path budget (jobs cut into several sample slices), fused or split
traversal launches, graph replay or direct launches, FP32 or 8-bit BVH.
"""
import ctypes as C

import numpy as np
import pytest

from eleven import _abi as A
from eleven import _lib, scenes

pytestmark = pytest.mark.gpu


def _moved(cam, dx, res=None):
    c = A.er_camera.from_buffer_copy(cam)
    c.position[0] += dx
    c.rotation[1] += 4.0
    if res:
        c.x_res, c.y_res = res
        c.sensor_height = float(np.float32(c.sensor_width) * (np.float32(res[1]) / np.float32(res[0])))
    return c


@pytest.fixture(scope="module")
def world():
    arrays = [
        scenes.config0(x_res=64, y_res=48, seed=3),
        scenes.config1(x_res=80, y_res=56, n_meshes=6, tri_lo=500, tri_hi=3000, tex_size=64, n_tex=3,
                       env_w=64, env_h=32),
        scenes.displaced_spheres(6000, seed=17, x_res=48, y_res=48, n_lights=2, env_w=32, env_h=16),
    ]
    fp32 = [_lib.Scene(a) for a in arrays]
    q8 = [_lib.Scene(a, bvh_format=A.ER_BVH_Q8) for a in arrays]
    cams = [s.camera() for s in fp32]
    jobs = [
        dict(scene=0, spp=5, max_depth=4, seed=1, camera=cams[0]),
        dict(scene=1, spp=3, max_depth=6, seed=2, camera=cams[1]),
        dict(scene=2, spp=8, max_depth=3, seed=3, camera=cams[2], flags=A.ER_RENDER_ENV_ALIAS),
        dict(scene=1, spp=4, max_depth=5, seed=4, camera=_moved(cams[1], 0.7, (72, 40)), sample_begin=3),
        dict(scene=0, spp=2, max_depth=8, seed=5, camera=_moved(cams[0], -1.0), flags=A.ER_RENDER_ACCUM_FP64),
        # a resolution without 8x4 path tiles (raster path order)
        dict(scene=2, spp=3, max_depth=4, seed=6, camera=_moved(cams[2], 0.3, (70, 38))),
    ]
    return arrays, fp32, q8, jobs


def _single(scene, job):
    scene.set_camera(job["camera"])
    out = scene.render(job["spp"], max_depth=job["max_depth"], seed=job["seed"],
                       sample_begin=job.get("sample_begin", 0), flags=job.get("flags", 0))
    return out["beauty"], out["samples"], out["pathcount"]


@pytest.fixture(scope="module")
def singles(world):
    arrays, fp32, q8, jobs = world
    return [_single(fp32[j["scene"]], j) for j in jobs]


def _check(batch, singles):
    for k, (beauty, samples, pc) in enumerate(singles):
        got = batch.read(k)
        assert np.array_equal(got["beauty"].view(np.uint32), beauty.view(np.uint32)), f"job {k} beauty"
        assert np.array_equal(got["samples"], samples), f"job {k} samples"
        assert np.array_equal(got["pathcount"], pc), f"job {k} pathcount"


def _tuning(wave_paths=0, trace=0, shade=0, split=0, graph=1, one_stream=0):
    t = A.er_batch_tuning()
    t.wave_paths, t.trace_blocks_per_sm, t.shade_blocks_per_sm = wave_paths, trace, shade
    t.split_trace, t.use_graph, t.one_stream = split, graph, one_stream
    return t


@pytest.mark.parametrize("tuning", [
    dict(),                                       # defaults: one wave, graph
    dict(wave_paths=9000, graph=0),               # many waves on two streams, jobs in slices, direct launches
    dict(wave_paths=9000),                        # the same captured in a graph (fork / join in the capture)
    dict(wave_paths=9000, one_stream=1),          # many waves on one stream
    dict(wave_paths=12000, split=1, trace=3, shade=2),
])
def test_batch_equals_single_renders(world, singles, tuning):
    arrays, fp32, q8, jobs = world
    with _lib.Batch(fp32) as b:
        b.set_jobs(jobs)
        st = b.render(_tuning(**tuning))
        assert st.samples == sum(j["spp"] * j["camera"].x_res * j["camera"].y_res for j in jobs)
        assert st.rays_closest > 0 and st.kernel_launches > 0
        _check(b, singles)
        # a second render (graph replay) gives the same films
        b.render(_tuning(**tuning))
        _check(b, singles)


def test_batch_q8_equals_single_renders(world, singles):
    arrays, fp32, q8, jobs = world
    with _lib.Batch(q8, bvh_format=A.ER_BVH_Q8) as b:
        b.set_jobs(jobs)
        b.render(_tuning(wave_paths=10000))
        _check(b, singles)


def test_batch_waves_and_autotune(world, singles):
    arrays, fp32, q8, jobs = world
    with _lib.Batch(fp32) as b:
        b.set_jobs(jobs)
        b.render(_tuning(wave_paths=9000))
        n_waves, nbytes = b.info()
        assert n_waves > 3 and nbytes > 0
        t = b.autotune(reps=1)
        assert t.wave_paths > 0
        b.render()  # the tuned schedule
        _check(b, singles)


def test_batch_rejects_bad_input(world):
    arrays, fp32, q8, jobs = world
    L = _lib.load()
    with _lib.Batch(fp32) as b:
        bad = dict(jobs[0], scene=7)
        with pytest.raises(_lib.ElevenError):
            b.set_jobs([bad])
        with pytest.raises(_lib.ElevenError):
            b.render()  # no jobs
    h = C.c_void_p()
    arr = (C.c_void_p * 1)(fp32[0].h)
    opts = A.er_scene_opts(A.ER_BVH_Q8, 0, 0, None)
    assert L.er_batch_create(arr, 1, C.byref(opts), C.byref(h)) == A.ER_ERR_INVALID_ARG
