"""The kernel.h drop-in (tfg-pathtracer_gb300/shim/kernel_shim.cpp) compiles
against the reference's own headers, exports the four C++ symbols of
kernel.h:78-84 with the reference's mangled names, and links against
libeleven.so.  On a GPU, a headless stand-in for the reference's main.cpp
(main.cpp:111-117 loadScene, :51 renderSetup, :53 renderCuda, :97-102
getBuffers / getSamples) loads a scene folder with the reference's own
loadScene, renders through the shim and reads the passes back; the film
equals er_render's of the same folder.  Needs the reference sources
(skipped where absent)."""
import os
import shutil
import subprocess

import numpy as np
import pytest

from eleven import _lib, scene_folder, scenes
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


# The headless caller: the reference's loadScene appends a Windows separator
# to the folder path (SceneLoader.hpp:11,54), so it runs from inside the
# folder with an empty path and reads the files "\\scene.json", ... that the
# test links to the real ones; texture paths in the .mtl are relative to the
# working directory (SceneLoader.hpp:75,104), which is the folder.
RENDER_DRIVER = r"""
#include "Definitions.h"
#include "kernel.h"
#include "SceneLoader.hpp"
#include "mikktspaceCallback.hpp"
#include <cstdio>
#include <cstdlib>
#include <vector>
#include <unistd.h>
static void dump(const char* path, const void* p, size_t n) {
  FILE* f = std::fopen(path, "wb");
  std::fwrite(p, 1, n, f);
  std::fclose(f);
}
int main(int argc, char** argv) {
  if (argc < 4 || chdir(argv[1]) != 0) return 3;
  const int spp = std::atoi(argv[2]);
  Scene scene = loadScene("");
  if (renderSetup(&scene) != cudaSuccess) return 4;
  if (renderCuda(&scene, spp) != cudaSuccess) return 5;
  const int n = (int)(scene.camera.xRes * scene.camera.yRes);
  std::vector<float> pass[PASSES_COUNT];
  RenderData rd;
  for (int i = 0; i < PASSES_COUNT; i++) {
    pass[i].assign((size_t)4 * n, -1.0f);
    rd.passes[i] = pass[i].data();
  }
  std::vector<int> pathcount(n, -1);
  if (getBuffers(rd, pathcount.data(), n) != cudaSuccess) return 6;
  std::printf("samples=%d\n", getSamples());
  std::string o(argv[3]);
  dump((o + ".beauty").c_str(), pass[BEAUTY].data(), pass[BEAUTY].size() * 4);
  dump((o + ".normal").c_str(), pass[NORMAL].data(), pass[NORMAL].size() * 4);
  dump((o + ".pathcount").c_str(), pathcount.data(), pathcount.size() * 4);
  return 0;
}
"""


def _has_gpu():
    try:
        import torch
        return torch.cuda.is_available()
    except Exception:
        return False


@pytest.mark.gpu
def test_shim_renders_like_er_render(tmp_path):
    if not _has_gpu():
        pytest.skip("no GPU")
    lib = _lib.lib_path()
    _lib.load()
    arrays = scenes.config1(x_res=40, y_res=24, n_meshes=4, tri_lo=200, tri_hi=600, tex_size=16, n_tex=2,
                            env_w=64, env_h=32)
    d = scene_folder.write_folder(arrays, str(tmp_path / "s"))
    # the reference's .mtl reader knows Kd/Ks/Ke/Ni/d and the maps only
    # (ObjLoader.hpp:33-69): drop the extension keys so both loaders see the
    # same materials
    mtl = os.path.join(d, "scene.mtl")
    lines = [ln for ln in open(mtl).read().splitlines(True) if ln.split(" ")[0] not in ("Pr", "Pm", "Pc", "Ps")]
    open(mtl, "w").write("".join(lines))
    for name in ("scene.json", "scene.mtl", "scene.obj"):
        os.symlink(os.path.join(d, name), os.path.join(d, "\\" + name))
    os.symlink(os.path.join(d, "HDRI", "env.hdr"), os.path.join(d, "\\HDRI\\env.hdr"))
    drv = tmp_path / "drv.cpp"
    drv.write_text(RENDER_DRIVER)
    exe = tmp_path / "drv"
    subprocess.run(["g++", "-O1", str(drv), os.path.join(PKG_ROOT, "shim", "kernel_shim.cpp"),
                    os.path.join(REF_SRC, "mikktspace.cpp"), "-o", str(exe)] + FLAGS +
                   ["-L" + os.path.dirname(lib), "-leleven", "-Wl,-rpath," + os.path.dirname(lib),
                    "-L/usr/local/cuda/lib64", "-lcudart"], check=True)
    spp = 12  # the shim renders in chunks of 8: one full chunk and a partial one
    out = str(tmp_path / "film")
    r = subprocess.run([str(exe), d, str(spp), out], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stdout[-2000:] + r.stderr[-2000:]
    assert f"samples={spp}" in r.stdout
    W, H = 40, 24
    beauty = np.fromfile(out + ".beauty", np.float32).reshape(W * H, 4)
    normal = np.fromfile(out + ".normal", np.float32).reshape(W * H, 4)
    pathcount = np.fromfile(out + ".pathcount", np.uint32)
    with _lib.Scene.load_folder(d) as s:
        ref = s.render(spp=spp, max_depth=5, seed=0, aov=True)  # MAXBOUNCES = 5 (Definitions.h:9)
    assert np.array_equal(beauty, ref["beauty"])
    assert np.array_equal(normal, ref["normal"])
    assert np.array_equal(pathcount, ref["pathcount"])
    assert (beauty[:, :3] > 0).any()
