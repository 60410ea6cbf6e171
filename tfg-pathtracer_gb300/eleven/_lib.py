"""ctypes binding of libeleven.so (the product C-ABI, include/eleven.h).

The library is built in-tree; loading fails loudly when it is missing or a
call returns an error status.  There is no CPU fallback.
"""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

from . import _abi as A

_lib = None


class ElevenError(RuntimeError):
    def __init__(self, status, where, detail):
        self.status = status
        super().__init__(f"{where}: {A.STATUS_NAMES.get(status, status)}: {detail}")


def lib_path():
    from .build import LIB
    return LIB


def load(build_if_missing=True):
    """Load libeleven.so, building it first if it is absent or stale."""
    global _lib
    if _lib is not None:
        return _lib
    path = lib_path()
    if build_if_missing:
        from . import build
        build.build_product()
    if not os.path.exists(path):
        raise ElevenError(A.ER_ERR_UNSUPPORTED if hasattr(A, "ER_ERR_UNSUPPORTED") else 8, "load",
                          f"{path} not built")
    L = C.CDLL(path)
    L.er_status_string.restype = C.c_char_p
    L.er_status_string.argtypes = [A.er_status]
    L.er_last_error.restype = C.c_char_p
    L.er_abi_version.restype = C.c_int32
    L.er_scene_create.restype = A.er_status
    L.er_scene_create.argtypes = [C.POINTER(A.er_scene_desc), C.POINTER(A.er_scene_opts), C.POINTER(C.c_void_p)]
    L.er_scene_load.restype = A.er_status
    L.er_scene_load.argtypes = [C.c_char_p, C.POINTER(A.er_scene_opts), C.POINTER(C.c_void_p)]
    L.er_scene_folder_read.restype = A.er_status
    L.er_scene_folder_read.argtypes = [C.c_char_p, C.POINTER(C.c_void_p)]
    L.er_folder_desc.restype = A.er_status
    L.er_folder_desc.argtypes = [C.c_void_p, C.POINTER(A.er_scene_desc)]
    L.er_folder_free.restype = A.er_status
    L.er_folder_free.argtypes = [C.c_void_p]
    L.er_scene_info_get.restype = A.er_status
    L.er_scene_info_get.argtypes = [C.c_void_p, C.POINTER(A.er_scene_info)]
    L.er_scene_set_camera.restype = A.er_status
    L.er_scene_set_camera.argtypes = [C.c_void_p, C.POINTER(A.er_camera)]
    L.er_scene_get_camera.restype = A.er_status
    L.er_scene_get_camera.argtypes = [C.c_void_p, C.POINTER(A.er_camera)]
    L.er_scene_free.restype = A.er_status
    L.er_scene_free.argtypes = [C.c_void_p]
    L.er_render.restype = A.er_status
    L.er_render.argtypes = [C.c_void_p, C.POINTER(A.er_render_opts), C.c_void_p, C.c_void_p, C.c_void_p,
                            C.c_void_p, C.c_void_p, C.c_void_p, C.POINTER(A.er_render_stats)]
    L.er_film_read.restype = A.er_status
    L.er_film_read.argtypes = [C.c_void_p, C.c_uint32, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p,
                               C.c_void_p, C.c_void_p]
    L.er_film_read_sums.restype = A.er_status
    L.er_film_read_sums.argtypes = [C.c_void_p, C.c_uint32, C.c_void_p, C.c_void_p]
    L.er_snapshot.restype = A.er_status
    L.er_snapshot.argtypes = [C.c_void_p, C.c_void_p, C.c_void_p]
    L.er_env_distribution.restype = A.er_status
    L.er_env_distribution.argtypes = [C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p]
    L.er_env_search_table.restype = A.er_status
    L.er_env_search_table.argtypes = [C.c_void_p, C.c_void_p]
    L.er_render_noalloc.restype = A.er_status
    L.er_render_noalloc.argtypes = [C.c_void_p, C.POINTER(A.er_render_opts), C.c_void_p, C.c_void_p, C.c_void_p]
    L.er_render_paths.restype = A.er_status
    L.er_render_paths.argtypes = [C.c_void_p, C.POINTER(A.er_render_opts), C.c_void_p, C.c_void_p]
    L.er_scene_get_params.restype = A.er_status
    L.er_scene_get_params.argtypes = [C.c_void_p, C.c_void_p, C.c_void_p]
    L.er_scene_set_params.restype = A.er_status
    L.er_scene_set_params.argtypes = [C.c_void_p, C.c_void_p, C.c_void_p, C.c_uint32]
    L.er_render_replay.restype = A.er_status
    L.er_render_replay.argtypes = [C.c_void_p, C.POINTER(A.er_render_opts), C.c_void_p, C.c_void_p, C.c_void_p,
                                   C.c_void_p, C.c_void_p]
    L.er_backward.restype = A.er_status
    L.er_backward.argtypes = [C.c_void_p, C.POINTER(A.er_render_opts), C.c_void_p, C.c_void_p, C.c_void_p,
                              C.c_void_p, C.POINTER(A.er_render_stats)]
    L.er_batch_create.restype = A.er_status
    L.er_batch_create.argtypes = [C.POINTER(C.c_void_p), C.c_int32, C.POINTER(A.er_scene_opts),
                                  C.POINTER(C.c_void_p)]
    L.er_batch_set_jobs.restype = A.er_status
    L.er_batch_set_jobs.argtypes = [C.c_void_p, C.POINTER(A.er_batch_job), C.c_int32]
    L.er_batch_render.restype = A.er_status
    L.er_batch_render.argtypes = [C.c_void_p, C.POINTER(A.er_batch_tuning), C.POINTER(A.er_render_stats)]
    L.er_batch_read.restype = A.er_status
    L.er_batch_read.argtypes = [C.c_void_p, C.c_int32, C.c_uint32, C.c_void_p, C.c_void_p, C.c_void_p]
    L.er_batch_autotune.restype = A.er_status
    L.er_batch_autotune.argtypes = [C.c_void_p, C.c_int32, C.POINTER(A.er_batch_tuning)]
    L.er_batch_info.restype = A.er_status
    L.er_batch_info.argtypes = [C.c_void_p, C.POINTER(C.c_int32), C.POINTER(C.c_int64)]
    L.er_batch_free.restype = A.er_status
    L.er_batch_free.argtypes = [C.c_void_p]
    L.er_trace_closest.restype = A.er_status
    L.er_trace_closest.argtypes = [C.c_void_p, C.c_void_p, C.c_int64, C.c_void_p, C.c_void_p, C.c_void_p,
                                   C.c_uint32, C.POINTER(A.er_trace_stats)]
    L.er_encode_ldr.restype = A.er_status
    L.er_encode_ldr.argtypes = [C.c_void_p, C.c_int32, C.c_int32, C.c_void_p]
    L.er_compute_tangents.restype = A.er_status
    L.er_compute_tangents.argtypes = [C.c_int64, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p]
    L.er_postprocess.restype = A.er_status
    L.er_postprocess.argtypes = [C.c_void_p, C.c_int32, C.c_int32, C.POINTER(A.er_post_opts), C.c_void_p,
                                 C.c_void_p, C.c_uint32]
    L.er_device_bandwidth.restype = A.er_status
    L.er_device_bandwidth.argtypes = [C.c_int32, C.c_int32, C.c_int64, C.c_int32, C.POINTER(C.c_double)]
    L.er_write_image.restype = A.er_status
    L.er_write_image.argtypes = [C.c_char_p, C.c_void_p, C.c_int32, C.c_int32, C.c_int32]
    _lib = L
    return L


def check(status, where):
    if status != A.ER_OK:
        raise ElevenError(status, where, load().er_last_error().decode(errors="replace"))


def _p(a):
    return None if a is None else a.ctypes.data_as(C.c_void_p)


def read_folder(path):
    """Parse a scene folder on the host (er_scene_folder_read): a dict of
    numpy copies of the description's arrays (no device needed)."""
    L = load()
    h = C.c_void_p()
    check(L.er_scene_folder_read(os.fsencode(str(path)), C.byref(h)), "er_scene_folder_read")
    try:
        d = A.er_scene_desc()
        check(L.er_folder_desc(h, C.byref(d)), "er_folder_desc")
        T = int(d.tri_count)

        def arr(ptr, n, dt):
            if not ptr or n == 0:
                return np.zeros(0, dt)
            return np.ctypeslib.as_array(C.cast(ptr, C.POINTER(np.ctypeslib.as_ctypes_type(dt))), (n,)).copy()

        out = dict(
            camera=d.camera,
            positions=arr(d.positions, 9 * T, np.float32).reshape(T, 3, 3),
            normals=arr(d.normals, 9 * T, np.float32).reshape(T, 3, 3),
            uvs=arr(d.uvs, 6 * T, np.float32).reshape(T, 3, 2),
            tangents=arr(d.tangents, 9 * T, np.float32).reshape(T, 3, 3),
            tangent_sign=arr(d.tangent_sign, T, np.float32),
            tri_object=arr(d.tri_object, T, np.int32),
            object_material=arr(d.object_material, d.object_count, np.int32),
            materials=[A.er_material.from_buffer_copy(d.materials[i]) for i in range(d.material_count)],
            lights=[A.er_point_light.from_buffer_copy(d.lights[i]) for i in range(d.light_count)],
        )
        texs = []
        for i in range(d.texture_count):
            t = d.textures[i]
            texs.append(arr(t.data, 3 * t.width * t.height, np.float32).reshape(t.height, t.width, 3))
        out["textures"] = texs
        e = d.env
        out["env"] = arr(e.data, 3 * e.width * e.height, np.float32).reshape(e.height, e.width, 3)
        out["env_offset"] = (float(e.x_offset), float(e.y_offset))
        out["env_tile"] = (float(e.x_tile), float(e.y_tile))
        return out
    finally:
        L.er_folder_free(h)


class Scene:
    """A scene handle on the GPU (er_scene)."""

    def __init__(self, arrays=None, bvh_format=A.ER_BVH_FP32, max_leaf=0, device=0, stream=None, handle=None,
                 builder=A.ER_BUILDER_HOST):
        L = load()
        self.arrays = arrays
        if handle is not None:
            self.h = handle
            return
        desc, keep = arrays.desc()
        opts = A.er_scene_opts(bvh_format, max_leaf, device, stream, builder)
        h = C.c_void_p()
        check(L.er_scene_create(C.byref(desc), C.byref(opts), C.byref(h)), "er_scene_create")
        self.h = h

    @classmethod
    def load_folder(cls, path, bvh_format=A.ER_BVH_FP32):
        L = load()
        opts = A.er_scene_opts(bvh_format, 0, 0, None)
        h = C.c_void_p()
        check(L.er_scene_load(os.fsencode(path), C.byref(opts), C.byref(h)), "er_scene_load")
        return cls(handle=h)

    def close(self):
        if getattr(self, "h", None):
            load().er_scene_free(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    def info(self):
        i = A.er_scene_info()
        check(load().er_scene_info_get(self.h, C.byref(i)), "er_scene_info_get")
        return i

    @property
    def resolution(self):
        c = self.camera()
        return int(c.x_res), int(c.y_res)

    def camera(self):
        c = A.er_camera()
        check(load().er_scene_get_camera(self.h, C.byref(c)), "er_scene_get_camera")
        return c

    def set_camera(self, cam):
        check(load().er_scene_set_camera(self.h, C.byref(cam)), "er_scene_set_camera")

    def trace(self, rays, normalize=True, stats=False):
        rays = np.ascontiguousarray(rays, dtype=np.float32)
        n = len(rays)
        tri = np.zeros(n, np.int32)
        dist = np.zeros(n, np.float32)
        uv = np.zeros((n, 2), np.float32)
        flags = (0 if normalize else A.ER_TRACE_NORMALIZED) | (A.ER_TRACE_STATS if stats else 0)
        st = A.er_trace_stats()
        check(load().er_trace_closest(self.h, _p(rays), n, _p(tri), _p(dist), _p(uv), flags, C.byref(st)),
              "er_trace_closest")
        return tri, dist, uv, st

    def render(self, spp, max_depth=5, seed=0, sample_begin=0, spp_per_wave=0, flags=0, aov=False):
        W, H = self.resolution
        if aov:
            flags |= A.ER_RENDER_AOV
        o = A.er_render_opts(spp, sample_begin, max_depth, spp_per_wave, seed, flags, 0)
        beauty = np.zeros((H * W, 4), np.float32)
        aovs = [np.zeros((H * W, 4), np.float32) for _ in range(3)] if aov else [None] * 3
        samples = np.zeros(H * W, np.uint32)
        pc = np.zeros(H * W, np.uint32)
        st = A.er_render_stats()
        check(load().er_render(self.h, C.byref(o), _p(beauty), _p(aovs[0]), _p(aovs[1]), _p(aovs[2]),
                               _p(samples), _p(pc), C.byref(st)), "er_render")
        return dict(beauty=beauty, normal=aovs[0], tangent=aovs[1], bitangent=aovs[2], samples=samples,
                    pathcount=pc, stats=st)

    # ---- differentiable parameters (host numpy arrays)
    def env_hw(self):
        """(h, w) of the environment texture."""
        i = self.info()
        return int(i.env_height), int(i.env_width)

    def material_count(self):
        return int(self.info().material_count)

    def get_params(self):
        """(materials (n, 5): albedo rgb, roughness, metallic; env (h, w, 3))."""
        h, w = self.env_hw()
        mats = np.zeros((self.material_count(), 5), np.float32)
        env = np.zeros((h, w, 3), np.float32)
        check(load().er_scene_get_params(self.h, _p(mats), _p(env)), "er_scene_get_params")
        return mats, env

    def set_params(self, materials=None, env=None):
        m = None if materials is None else np.ascontiguousarray(materials, np.float32)
        e = None if env is None else np.ascontiguousarray(env, np.float32)
        check(load().er_scene_set_params(self.h, _p(m), _p(e), 0), "er_scene_set_params")

    def render_replay(self, spp, max_depth=5, seed=0, sample_begin=0, materials=None, env=None, flags=0):
        """Forward render by path replay; materials/env = evaluation
        parameters (sampling stays with the scene's)."""
        W, H = self.resolution
        o = A.er_render_opts(spp, sample_begin, max_depth, 0, seed, flags, 0)
        m = None if materials is None else np.ascontiguousarray(materials, np.float32)
        e = None if env is None else np.ascontiguousarray(env, np.float32)
        beauty = np.zeros((H * W, 4), np.float32)
        samples = np.zeros(H * W, np.uint32)
        pc = np.zeros(H * W, np.uint32)
        check(load().er_render_replay(self.h, C.byref(o), _p(m), _p(e), _p(beauty), _p(samples), _p(pc)),
              "er_render_replay")
        return dict(beauty=beauty, samples=samples, pathcount=pc)

    def backward(self, spp, d_beauty, samples, max_depth=5, seed=0, sample_begin=0, flags=0):
        """Gradients (materials (n, 5), env (h, w, 3)) of a loss whose
        derivative with respect to the film is d_beauty ((H*W, 4))."""
        o = A.er_render_opts(spp, sample_begin, max_depth, 0, seed, flags, 0)
        h, w = self.env_hw()
        gm = np.zeros((self.material_count(), 5), np.float32)
        ge = np.zeros((h, w, 3), np.float32)
        db = np.ascontiguousarray(d_beauty, np.float32)
        sa = np.ascontiguousarray(samples, np.uint32)
        st = A.er_render_stats()
        check(load().er_backward(self.h, C.byref(o), _p(db), _p(sa), _p(gm), _p(ge), C.byref(st)), "er_backward")
        return gm, ge, st

    def snapshot(self):
        """Film as of the last finished wave of a render running with
        ER_RENDER_SNAPSHOTS (callable from another thread): (beauty, samples)."""
        W, H = self.resolution
        beauty = np.zeros((H * W, 4), np.float32)
        samples = np.zeros(H * W, np.uint32)
        check(load().er_snapshot(self.h, _p(beauty), _p(samples)), "er_snapshot")
        return beauty, samples

    def read_sums(self):
        """FP64 per-pixel sums ((H*W, 3) float64) and sample counts of the
        film of an ER_RENDER_ACCUM_FP64 render (er_film_read_sums)."""
        W, H = self.resolution
        sums = np.zeros((H * W, 3), np.float64)
        samples = np.zeros(H * W, np.uint32)
        check(load().er_film_read_sums(self.h, 0, _p(sums), _p(samples)), "er_film_read_sums")
        return sums, samples

    def render_paths(self, spp, max_depth=5, seed=0, sample_begin=0):
        W, H = self.resolution
        o = A.er_render_opts(spp, sample_begin, max_depth, 0, seed, 0, 0)
        rad = np.zeros((spp, H * W, 3), np.float32)
        b = np.zeros((spp, H * W), np.int32)
        check(load().er_render_paths(self.h, C.byref(o), _p(rad), _p(b)), "er_render_paths")
        return rad, b


class Batch:
    """Several scenes and views rendered together (er_batch).

    jobs: dicts with scene (index), spp, max_depth, seed, camera (er_camera
    or None for that scene's own camera), optional sample_begin and flags.
    """

    def __init__(self, scenes, bvh_format=A.ER_BVH_FP32):
        L = load()
        self.scenes = list(scenes)  # kept alive: the batch reads their device data
        arr = (C.c_void_p * len(self.scenes))(*[s.h for s in self.scenes])
        opts = A.er_scene_opts(bvh_format, 0, 0, None)
        h = C.c_void_p()
        check(L.er_batch_create(arr, len(self.scenes), C.byref(opts), C.byref(h)), "er_batch_create")
        self.h = h
        self.jobs = []

    def close(self):
        if getattr(self, "h", None):
            load().er_batch_free(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    def set_jobs(self, jobs):
        arr = (A.er_batch_job * len(jobs))()
        for k, j in enumerate(jobs):
            cam = j.get("camera") or self.scenes[j["scene"]].camera()
            arr[k] = A.er_batch_job(j["scene"], j["spp"], j.get("max_depth", 5), j.get("sample_begin", 0),
                                    j.get("seed", 0), j.get("flags", 0), 0, cam)
        check(load().er_batch_set_jobs(self.h, arr, len(jobs)), "er_batch_set_jobs")
        self.jobs = [dict(j, camera=arr[k].camera) for k, j in enumerate(jobs)]

    def render(self, tuning=None):
        st = A.er_render_stats()
        t = C.byref(tuning) if tuning is not None else None
        check(load().er_batch_render(self.h, t, C.byref(st)), "er_batch_render")
        return st

    def read(self, job):
        cam = self.jobs[job]["camera"]
        n = int(cam.x_res) * int(cam.y_res)
        beauty = np.zeros((n, 4), np.float32)
        samples = np.zeros(n, np.uint32)
        pc = np.zeros(n, np.uint32)
        check(load().er_batch_read(self.h, job, 0, _p(beauty), _p(samples), _p(pc)), "er_batch_read")
        return dict(beauty=beauty, samples=samples, pathcount=pc)

    def autotune(self, reps=2):
        t = A.er_batch_tuning()
        check(load().er_batch_autotune(self.h, reps, C.byref(t)), "er_batch_autotune")
        return t

    def info(self):
        nw = C.c_int32(0)
        nb = C.c_int64(0)
        check(load().er_batch_info(self.h, C.byref(nw), C.byref(nb)), "er_batch_info")
        return int(nw.value), int(nb.value)


def encode_ldr(rgba, width, height):
    rgba = np.ascontiguousarray(rgba, np.float32)
    out = np.zeros(width * height * 4, np.uint8)
    check(load().er_encode_ldr(_p(rgba), width, height, _p(out)), "er_encode_ldr")
    return out


def compute_tangents(positions, normals, uvs):
    """Per-corner tangents (T, 3, 3) and per-triangle signs (T,) (er_compute_tangents)."""
    P = np.ascontiguousarray(positions, np.float32).reshape(-1, 9)
    N = np.ascontiguousarray(normals, np.float32).reshape(-1, 9)
    U = np.ascontiguousarray(uvs, np.float32).reshape(-1, 6)
    t = np.zeros((len(P), 3, 3), np.float32)
    s = np.zeros(len(P), np.float32)
    check(load().er_compute_tangents(len(P), _p(P), _p(N), _p(U), _p(t), _p(s)), "er_compute_tangents")
    return t, s


def postprocess(rgba, width, height, exposure=1.0, tonemap=0, clamp=False, srgb=False, flip_x=False, flip_y=False,
                bloom_threshold=0.0, bloom_power=0.0, bloom_radius=0.0):
    """GPU post-processing (er_postprocess): (float RGBA (W*H, 4), LDR bytes)."""
    rgba = np.ascontiguousarray(rgba, np.float32)
    o = A.er_post_opts(exposure, tonemap, int(clamp), int(srgb), int(flip_x), int(flip_y), bloom_threshold,
                       bloom_power, bloom_radius)
    out = np.zeros((width * height, 4), np.float32)
    ldr = np.zeros(width * height * 4, np.uint8)
    check(load().er_postprocess(_p(rgba), width, height, C.byref(o), _p(out), _p(ldr), 0), "er_postprocess")
    return out, ldr


def write_image(path, rgba_u8, width, height, as_bmp=False):
    rgba_u8 = np.ascontiguousarray(rgba_u8, np.uint8)
    check(load().er_write_image(os.fsencode(path), _p(rgba_u8), width, height, int(as_bmp)), "er_write_image")


def device_bandwidth(kind, nbytes, reps, device=0):
    """GB/s measured by er_device_bandwidth (kind: A.ER_BW_L2_READ or
    A.ER_BW_HBM_COPY)."""
    g = C.c_double()
    check(load().er_device_bandwidth(device, kind, nbytes, reps, C.byref(g)), "er_device_bandwidth")
    return g.value
