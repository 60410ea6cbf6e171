"""The kernel.h drop-in (tfg-pathtracer_gb300/shim/kernel_shim.cpp) compiles
against the reference's own headers, exports the four C++ symbols of
kernel.h:78-84 with the reference's mangled names, and links against
libeleven.so.  Needs the reference sources (skipped where absent)."""
import os
import subprocess

import pytest

from eleven import _lib
from eleven.build import INCLUDE, PKG_ROOT, REF_SRC

pytestmark = pytest.mark.skipif(not os.path.isdir(REF_SRC), reason="reference sources not present")

FLAGS = ["-std=c++17", "-w", "-include", "math.h", "-include", "cstring", "-DSTB_IMAGE_STATIC",
         "-I" + REF_SRC, "-I" + INCLUDE, "-I/usr/local/cuda/include"]

DRIVER = r"""
#include "Definitions.h"
#include "kernel.h"
#include <cstdio>
int main() {
  Scene scene;
  scene.camera = Camera(16, 8);
  scene.addHDRI(Vector3(0.5f, 0.5f, 0.5f));
  Material m;
  scene.addMaterial(m);
  cudaError_t e = renderSetup(&scene);
  std::printf("renderSetup=%d samples=%d\n", (int)e, getSamples());
  return 0;
}
"""


def test_shim_exports_reference_symbols(tmp_path):
    obj = tmp_path / "shim.o"
    subprocess.run(["g++", "-c", os.path.join(PKG_ROOT, "shim", "kernel_shim.cpp"), "-o", str(obj)] + FLAGS,
                   check=True)
    syms = subprocess.run(["nm", str(obj)], capture_output=True, text=True).stdout
    for s in ("_Z11renderSetupP5Scene", "_Z10renderCudaP5Scenei", "_Z10getBuffersR10RenderDataPii",
              "_Z10getSamplesv"):
        assert f" T {s}" in syms, s


def test_shim_links_and_reports_status(tmp_path):
    lib = _lib.lib_path()
    _lib.load()
    drv = tmp_path / "drv.cpp"
    drv.write_text(DRIVER)
    exe = tmp_path / "drv"
    subprocess.run(["g++", str(drv), os.path.join(PKG_ROOT, "shim", "kernel_shim.cpp"), "-o", str(exe)] + FLAGS +
                   ["-L" + os.path.dirname(lib), "-leleven", "-Wl,-rpath," + os.path.dirname(lib),
                    "-L/usr/local/cuda/lib64", "-lcudart"], check=True)
    r = subprocess.run([str(exe)], capture_output=True, text=True, timeout=120)
    assert r.returncode == 0, r.stderr
    assert "renderSetup=" in r.stdout
    try:
        import torch
        has_gpu = torch.cuda.is_available()
    except Exception:
        has_gpu = False
    if not has_gpu:
        # no device here: the status comes back as an error, not a crash
        assert "renderSetup=0" not in r.stdout
        assert "no CUDA device" in r.stderr
