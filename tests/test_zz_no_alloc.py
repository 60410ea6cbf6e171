"""er_render_noalloc: the allocation-free render, for callers that may not
allocate device memory while they render (a fixed device-memory budget set
at start-up, a render thread that may not enter the CUDA allocator).

Called through the C-ABI with device film buffers owned by the test; its
images must equal er_render's for the same options, on two calls in a row
(the second call sees the scratch array the first one left behind).  This
file is collected last so that a failure here stops a -x run only after
every other test has run; it also passes on its own in a fresh process."""
import ctypes as C

import numpy as np
import pytest

from eleven import _abi as A
from eleven import _lib, scenes

pytestmark = pytest.mark.gpu


def _cudart():
    import ctypes.util
    for name in ("libcudart.so", "libcudart.so.13", ctypes.util.find_library("cudart")):
        if not name:
            continue
        try:
            lib = C.CDLL(name)
            break
        except OSError:
            continue
    else:
        lib = C.CDLL("/usr/local/cuda/lib64/libcudart.so")
    lib.cudaMalloc.argtypes = [C.POINTER(C.c_void_p), C.c_size_t]
    lib.cudaFree.argtypes = [C.c_void_p]
    lib.cudaMemcpy.argtypes = [C.c_void_p, C.c_void_p, C.c_size_t, C.c_int]
    return lib


class DeviceBuffer:
    """Test-owned device memory (the entry point under test allocates none)."""

    def __init__(self, rt, nbytes):
        self.rt, self.nbytes = rt, nbytes
        self.ptr = C.c_void_p()
        assert rt.cudaMalloc(C.byref(self.ptr), nbytes) == 0

    def read(self, dtype, shape):
        out = np.empty(shape, dtype)
        assert self.rt.cudaMemcpy(out.ctypes.data_as(C.c_void_p), self.ptr, self.nbytes, 2) == 0
        return out

    def free(self):
        self.rt.cudaFree(self.ptr)


def test_noalloc_matches_render_on_two_calls():
    L = _lib.load()
    arrays = scenes.config0(x_res=96, y_res=64, n_spheres=6, subdiv=2)
    scene = _lib.Scene(arrays)
    W, H = scene.resolution
    rt = _cudart()
    beauty = DeviceBuffer(rt, W * H * 16)
    samples = DeviceBuffer(rt, W * H * 4)
    pathcount = DeviceBuffer(rt, W * H * 4)
    for seed, spp in ((3, 12), (7, 5)):  # two calls in a row
        o = A.er_render_opts(spp, 0, 4, 0, seed, 0, 0)
        st = L.er_render_noalloc(scene.h, C.byref(o), beauty.ptr, samples.ptr, pathcount.ptr)
        assert st == A.ER_OK, L.er_last_error()
        got = beauty.read(np.float32, (H * W, 4))
        want = scene.render(spp=spp, max_depth=4, seed=seed)
        # same kernels and random numbers: equal within the parity tests'
        # image tolerance, and in practice bit for bit
        rel = np.sqrt(((got - want["beauty"]) ** 2).sum() / max((want["beauty"] ** 2).sum(), 1e-30))
        assert rel <= 1e-6, rel
        assert np.array_equal(samples.read(np.uint32, H * W), want["samples"])
        assert np.array_equal(pathcount.read(np.uint32, H * W), want["pathcount"])
    # continuing the film equals one longer render
    o = A.er_render_opts(4, 5, 4, 0, 7, A.ER_RENDER_CONTINUE, 0)
    assert L.er_render_noalloc(scene.h, C.byref(o), beauty.ptr, samples.ptr, pathcount.ptr) == A.ER_OK
    want = scene.render(spp=9, max_depth=4, seed=7)
    assert np.array_equal(samples.read(np.uint32, H * W), want["samples"])
    got = beauty.read(np.float32, (H * W, 4))
    assert np.sqrt(((got - want["beauty"]) ** 2).sum() / (want["beauty"] ** 2).sum()) <= 1e-6
    for b in (beauty, samples, pathcount):
        b.free()
    scene.close()


def test_noalloc_rejects_oversized_images_and_flags():
    L = _lib.load()
    arrays = scenes.config0(x_res=320, y_res=240, n_spheres=2, subdiv=1)  # 76,800 > 65,536 pixels
    scene = _lib.Scene(arrays)
    o = A.er_render_opts(1, 0, 4, 0, 0, 0, 0)
    st = L.er_render_noalloc(scene.h, C.byref(o), C.c_void_p(16), C.c_void_p(16), C.c_void_p(16))
    assert st == A.ER_ERR_INVALID_ARG
    assert b"ER_NOALLOC_MAX_PATHS" in L.er_last_error()
    o = A.er_render_opts(1, 0, 4, 0, 0, A.ER_RENDER_AOV, 0)
    st = L.er_render_noalloc(scene.h, C.byref(o), C.c_void_p(16), C.c_void_p(16), C.c_void_p(16))
    assert st == A.ER_ERR_INVALID_ARG
    # counters that are not 4-byte aligned are refused before any launch
    # (the pointers are never dereferenced)
    o = A.er_render_opts(1, 0, 4, 0, 0, 0, 0)
    for smp, pc in ((18, 16), (16, 18)):
        st = L.er_render_noalloc(scene.h, C.byref(o), C.c_void_p(16), C.c_void_p(smp), C.c_void_p(pc))
        assert st == A.ER_ERR_INVALID_ARG
        assert b"4-byte aligned" in L.er_last_error()
    scene.close()
