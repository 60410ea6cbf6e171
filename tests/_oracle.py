"""ctypes access to the oracle (oracle/liborc.so) and, where it was built,
the reference-header shim (oracle/_ref/libref.so).  Test infrastructure."""
import ctypes as C
import os

import numpy as np

from eleven import _abi as A

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
# ORC_LIB selects another build of the same sources (oracle/liborc_ulp.so,
# the rounding-sensitivity probe) for a whole process
ORC_PATH = os.environ.get("ORC_LIB") or os.path.join(ROOT, "oracle", "liborc.so")
REF_PATH = os.path.join(ROOT, "oracle", "_ref", "libref.so")

_orc = None
_ref = None


def _f(a):
    return np.ascontiguousarray(a, dtype=np.float32)


def _ptr(a, t=A.FP):
    return a.ctypes.data_as(t)


def orc():
    global _orc
    if _orc is None:
        if not os.path.exists(ORC_PATH):
            from eleven import build
            build.build_oracle()
        _orc = C.CDLL(ORC_PATH)
        _orc.orc_scene_new.restype = C.c_void_p
        _orc.orc_scene_new.argtypes = [C.POINTER(A.er_scene_desc)]
        _orc.orc_scene_free.argtypes = [C.c_void_p]
        _orc.orc_bvh_node_count.restype = C.c_int64
        _orc.orc_bvh_node_count.argtypes = [C.c_void_p]
        _orc.orc_bvh_export.argtypes = [C.c_void_p, A.FP, A.IP, A.IP]
        _orc.orc_trace.argtypes = [C.c_void_p, A.FP, C.c_int64, C.c_int32, C.c_int32, A.IP, A.FP, A.FP,
                                   C.c_int32]
        _orc.orc_render.argtypes = [C.c_void_p, C.c_void_p, A.FP, A.FP, A.FP, A.FP, A.UP, A.UP]
        _orc.orc_render_paths.argtypes = [C.c_void_p, C.c_void_p, A.FP, A.IP]
        _orc.orc_encode_ldr.argtypes = [A.FP, C.c_int64, C.POINTER(C.c_uint8)]
        _orc.orc_fastpow.restype = C.c_double
        _orc.orc_fastpow.argtypes = [C.c_double, C.c_double]
        _orc.orc_u01.restype = C.c_float
        _orc.orc_u01.argtypes = [C.c_uint32]
        _bind_probes(_orc, "orc_p_")
        _orc.orc_p_sampling.argtypes = [C.c_int64, A.FP, A.FP]
        _orc.orc_p_camera.argtypes = [C.POINTER(A.er_camera), C.c_int64, A.IP, A.FP, A.FP]
        _orc.orc_p_sample_u.argtypes = [C.c_void_p, C.c_int64, A.IP, C.c_int32, A.FP, A.FP]
        _orc.orc_p_philox.argtypes = [C.c_int64, A.UP, C.c_uint32, C.c_uint32, A.UP]
        _orc.orc_p_hdri_counts.argtypes = [A.FP, C.c_int32, A.UP]
        _orc.orc_postprocess.argtypes = [A.FP, C.c_int32, C.c_int32, C.POINTER(A.er_post_opts)]
        _orc.orc64_new.restype = C.c_void_p
        _orc.orc64_new.argtypes = [C.c_void_p]
        _orc.orc64_free.argtypes = [C.c_void_p]
        _orc.orc64_render_pixels.argtypes = [C.c_void_p, A.IP, C.c_int64, C.c_int32, C.c_int32, C.c_int32,
                                             C.c_uint64, C.POINTER(C.c_double), A.UP, C.c_int32]
        _orc.orc64_trace.argtypes = [C.c_void_p, A.FP, C.c_int64, A.IP, C.POINTER(C.c_double), C.c_int32]
        _orc.orc64_render_pixels_eval.argtypes = [C.c_void_p, A.IP, C.c_int64, C.c_int32, C.c_int32, C.c_int32,
                                                  C.c_uint64, A.FP, A.FP, C.POINTER(C.c_double), A.UP, C.c_int32]
    return _orc


def postprocess(rgba, w, h, opts):
    """Oracle restatement of the reference's post-processing (in a copy)."""
    px = np.array(rgba, np.float32, copy=True, order="C")
    orc().orc_postprocess(_ptr(px), w, h, C.byref(opts))
    return px


def hdri_counts(cdf, n):
    """Effective texel counts of the environment search over the 2^24 grid."""
    cdf = _f(cdf)
    counts = np.zeros(n, np.uint32)
    orc().orc_p_hdri_counts(_ptr(cdf), n, _ptr(counts, A.UP))
    return counts


def ref():
    """The reference-header shim, or None where it was not built."""
    global _ref
    if _ref is None:
        if not os.path.exists(REF_PATH):
            return None
        _ref = C.CDLL(REF_PATH)
        _ref.ref_scene_new.restype = C.c_void_p
        _ref.ref_scene_new.argtypes = [C.POINTER(A.er_scene_desc)]
        _ref.ref_scene_free.argtypes = [C.c_void_p]
        _ref.ref_bvh_node_count.restype = C.c_int64
        _ref.ref_bvh_node_count.argtypes = [C.c_void_p]
        _ref.ref_bvh_export.argtypes = [C.c_void_p, A.FP, A.IP, A.IP]
        _ref.ref_trace.argtypes = [C.c_void_p, A.FP, C.c_int64, C.c_int32, A.IP, A.FP]
        _bind_probes(_ref, "ref_p_")
        _ref.ref_p_sampling.argtypes = [C.c_int64, A.FP, A.FP]
    return _ref


def _bind_probes(lib, pre):
    getattr(lib, pre + "tri_hit").argtypes = [C.c_int64, A.FP, A.FP, C.c_int32, A.FP]
    getattr(lib, pre + "disney").argtypes = [C.c_int64, A.FP, A.FP, A.FP, A.FP, A.FP]
    getattr(lib, pre + "spherical").argtypes = [C.c_int64, A.FP, A.FP]
    getattr(lib, pre + "reverse_spherical").argtypes = [C.c_int64, A.FP, A.FP]
    getattr(lib, pre + "hdri_cdf").argtypes = [C.POINTER(A.er_texture), A.FP, A.FP]
    getattr(lib, pre + "hdri_sample").argtypes = [C.POINTER(A.er_texture), A.FP, C.c_float, C.c_int64, A.FP, A.FP]
    getattr(lib, pre + "tex_uv").argtypes = [C.POINTER(A.er_texture), C.c_int64, A.FP, A.FP]


class Probes:
    """Same batched probe calls on either library (prefix orc_p_ / ref_p_)."""

    def __init__(self, lib, pre):
        self.lib, self.pre = lib, pre

    def _fn(self, name):
        return getattr(self.lib, self.pre + name)

    def tri_hit(self, tris, rays, normalize=True):
        tris, rays = _f(tris), _f(rays)
        out = np.zeros((len(tris), 17), np.float32)
        self._fn("tri_hit")(len(tris), _ptr(tris), _ptr(rays), int(normalize), _ptr(out))
        return out

    def disney(self, hd, dirs, Ls, rnd):
        hd, dirs, Ls, rnd = _f(hd), _f(dirs), _f(Ls), _f(rnd)
        out = np.zeros((len(hd), 7), np.float32)
        self._fn("disney")(len(hd), _ptr(hd), _ptr(dirs), _ptr(Ls), _ptr(rnd), _ptr(out))
        return out

    def spherical(self, pts):
        pts = _f(pts)
        out = np.zeros((len(pts), 2), np.float32)
        self._fn("spherical")(len(pts), _ptr(pts), _ptr(out))
        return out

    def reverse_spherical(self, uv):
        uv = _f(uv)
        out = np.zeros((len(uv), 3), np.float32)
        self._fn("reverse_spherical")(len(uv), _ptr(uv), _ptr(out))
        return out

    def sampling(self, u):
        u = _f(u)
        out = np.zeros((len(u), 12), np.float32)
        self._fn("sampling")(len(u), _ptr(u), _ptr(out))
        return out

    def hdri_cdf(self, env, offset=(0.0, 0.0)):
        t, keep = texture(env, offset)
        cdf = np.zeros(env.shape[0] * env.shape[1] + 1, np.float32)
        rs = C.c_float(0)
        self._fn("hdri_cdf")(C.byref(t), _ptr(cdf), C.byref(rs))
        return cdf, rs.value

    def hdri_sample(self, env, cdf, rsum, r, offset=(0.0, 0.0)):
        t, keep = texture(env, offset)
        cdf, r = _f(cdf), _f(r)
        out = np.zeros((len(r), 8), np.float32)
        self._fn("hdri_sample")(C.byref(t), _ptr(cdf), C.c_float(rsum), len(r), _ptr(r), _ptr(out))
        return out

    def tex_uv(self, img, uv, offset=(0.0, 0.0), tile=(1.0, 1.0)):
        t, keep = texture(img, offset, tile)
        uv = _f(uv)
        out = np.zeros((len(uv), 3), np.float32)
        self._fn("tex_uv")(C.byref(t), len(uv), _ptr(uv), _ptr(out))
        return out


def texture(img, offset=(0.0, 0.0), tile=(1.0, 1.0)):
    from eleven.scenes import fill_texture
    t = A.er_texture()
    keep = []
    fill_texture(t, img, keep, offset=offset, tile=tile)
    return t, keep


class Orc64:
    """FP64 restatement of the estimator over an OrcScene (own BVH)."""

    def __init__(self, orc_scene):
        self.base = orc_scene
        self.h = orc().orc64_new(orc_scene.h)

    def close(self):
        if self.h:
            orc().orc64_free(self.h)
            self.h = None

    def __del__(self):
        self.close()

    def render_pixels(self, idx, spp, max_depth, seed=0, sample_begin=0, nthreads=0, eval_mat=None,
                      eval_env=None):
        """Mean of clamp(L, 0, 10) over non-NaN samples for the pixels with
        output indices idx: (rgb (n, 3) float64, counts (n,)).  eval_mat /
        eval_env: evaluation parameters of the detached estimator."""
        idx = np.ascontiguousarray(idx, np.int32)
        rgb = np.zeros((len(idx), 3), np.float64)
        cnt = np.zeros(len(idx), np.uint32)
        em = None if eval_mat is None else _f(eval_mat)
        ee = None if eval_env is None else _f(eval_env)
        orc().orc64_render_pixels_eval(self.h, _ptr(idx, A.IP), len(idx), spp, sample_begin, max_depth, seed,
                                       None if em is None else _ptr(em), None if ee is None else _ptr(ee),
                                       rgb.ctypes.data_as(C.POINTER(C.c_double)), _ptr(cnt, A.UP), nthreads)
        return rgb, cnt

    def trace(self, rays, nthreads=0):
        rays = _f(rays)
        tri = np.zeros(len(rays), np.int32)
        dist = np.zeros(len(rays), np.float64)
        orc().orc64_trace(self.h, _ptr(rays), len(rays), _ptr(tri, A.IP), dist.ctypes.data_as(C.POINTER(C.c_double)),
                          nthreads)
        return tri, dist


class OrcScene:
    """Oracle scene (reference BVH restated) built from SceneArrays."""

    def __init__(self, arrays):
        self.arrays = arrays
        self.desc, self._keep = arrays.desc()
        self.h = orc().orc_scene_new(C.byref(self.desc))

    def close(self):
        if self.h:
            orc().orc_scene_free(self.h)
            self.h = None

    def __del__(self):
        self.close()

    def bvh(self):
        n = orc().orc_bvh_node_count(self.h)
        boxes = np.zeros((n, 6), np.float32)
        meta = np.zeros((n, 5), np.int32)
        ti = np.zeros(max(1, self.arrays.tri_count), np.int32)
        orc().orc_bvh_export(self.h, _ptr(boxes), _ptr(meta, A.IP), _ptr(ti, A.IP))
        return boxes, meta, ti[:self.arrays.tri_count]

    def trace(self, rays, mode=0, normalize=True, nthreads=0):
        rays = _f(rays)
        n = len(rays)
        tri = np.zeros(n, np.int32)
        dist = np.zeros(n, np.float32)
        uv = np.zeros((n, 2), np.float32)
        orc().orc_trace(self.h, _ptr(rays), n, mode, int(normalize), _ptr(tri, A.IP), _ptr(dist), _ptr(uv),
                        nthreads)
        return tri, dist

    def render(self, spp, max_depth, seed=0, sample_begin=0, aov=False, nthreads=0, pixel_stride=1):
        o = OrcRenderOpts(spp, sample_begin, max_depth, int(aov), seed, nthreads, pixel_stride)
        W, H = self.arrays.camera["x_res"], self.arrays.camera["y_res"]
        beauty = np.zeros((H * W, 4), np.float32)
        aovs = [np.zeros((H * W, 4), np.float32) for _ in range(3)] if aov else [None] * 3
        samples = np.zeros(H * W, np.uint32)
        pc = np.zeros(H * W, np.uint32)
        P = lambda a: None if a is None else _ptr(a)
        orc().orc_render(self.h, C.byref(o), _ptr(beauty), P(aovs[0]), P(aovs[1]), P(aovs[2]),
                         _ptr(samples, A.UP), _ptr(pc, A.UP))
        return dict(beauty=beauty, normal=aovs[0], tangent=aovs[1], bitangent=aovs[2], samples=samples,
                    pathcount=pc)

    def render_paths(self, spp, max_depth, seed=0, sample_begin=0, nthreads=0):
        o = OrcRenderOpts(spp, sample_begin, max_depth, 0, seed, nthreads, 1)
        W, H = self.arrays.camera["x_res"], self.arrays.camera["y_res"]
        rad = np.zeros((spp, H * W, 3), np.float32)
        b = np.zeros((spp, H * W), np.int32)
        orc().orc_render_paths(self.h, C.byref(o), _ptr(rad), _ptr(b, A.IP))
        return rad, b

    def sample_u(self, xy, max_depth, u):
        xy = np.ascontiguousarray(xy, np.int32)
        u = _f(u)
        out = np.zeros((len(xy), 4), np.float32)
        orc().orc_p_sample_u(self.h, len(xy), _ptr(xy, A.IP), max_depth, _ptr(u), _ptr(out))
        return out


class OrcRenderOpts(C.Structure):
    _fields_ = [("spp", C.c_int32), ("sample_begin", C.c_int32), ("max_depth", C.c_int32),
                ("aov", C.c_int32), ("seed", C.c_uint64), ("nthreads", C.c_int32),
                ("pixel_stride", C.c_int32)]


class RefScene:
    """The reference's own BVH (host-compiled headers) over SceneArrays."""

    def __init__(self, arrays):
        self.arrays = arrays
        self.desc, self._keep = arrays.desc()
        self.h = ref().ref_scene_new(C.byref(self.desc))

    def close(self):
        if self.h:
            ref().ref_scene_free(self.h)
            self.h = None

    def __del__(self):
        self.close()

    def bvh(self):
        n = ref().ref_bvh_node_count(self.h)
        boxes = np.zeros((n, 6), np.float32)
        meta = np.zeros((n, 5), np.int32)
        ti = np.zeros(max(1, self.arrays.tri_count), np.int32)
        ref().ref_bvh_export(self.h, _ptr(boxes), _ptr(meta, A.IP), _ptr(ti, A.IP))
        return boxes, meta, ti[:self.arrays.tri_count]

    def trace(self, rays, normalize=True):
        rays = _f(rays)
        n = len(rays)
        tri = np.zeros(n, np.int32)
        dist = np.zeros(n, np.float32)
        ref().ref_trace(self.h, _ptr(rays), n, int(normalize), _ptr(tri, A.IP), _ptr(dist))
        return tri, dist


def philox(ctr, key):
    ctr = np.ascontiguousarray(ctr, np.uint32)
    out = np.zeros_like(ctr)
    orc().orc_p_philox(len(ctr), _ptr(ctr, A.UP), key & 0xFFFFFFFF, key >> 32, _ptr(out, A.UP))
    return out
