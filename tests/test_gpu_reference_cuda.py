"""The reference's own CUDA renderer (kernel.cu, built for sm_103a by
`make -C oracle refcuda` from a scratch copy of the reference tree with the
textual patches the Makefile lists) on the same GPU, through a headless
caller (oracle/ref_cuda_main.cpp) of its renderSetup / renderCuda /
getBuffers.

Its random numbers are cuRAND XORWOW streams, which this library does not
reproduce, so the comparison is statistical: at matched samples per pixel
the reference's film and this library's film are two independent estimates
of the same image.  Their relative RMSE must be that of two of this
library's own films made with different seeds (the noise of the estimate),
and their mean radiance must agree within the standard error.  Needs the
reference sources (skipped where absent).
"""
import json
import os
import subprocess
import sys

import numpy as np
import pytest

from eleven import _lib, scenes
from eleven.build import ORACLE, REF_SRC

pytestmark = [pytest.mark.gpu, pytest.mark.skipif(not os.path.isdir(REF_SRC), reason="reference sources not present")]


def build_refcuda():
    r = subprocess.run(["make", "-s", "-C", ORACLE, "-j4", "refcuda", "REF_DIR=" + REF_SRC], capture_output=True,
                       text=True)
    assert r.returncode == 0, r.stdout[-3000:] + r.stderr[-3000:]


def run_reference(arrays, depth, warm, spp, tmp, beauty=True):
    sys.path.insert(0, ORACLE)
    import refcuda_scene
    f = os.path.join(tmp, "scene.ersc")
    refcuda_scene.write(arrays, f)
    out = os.path.join(tmp, "ref_beauty.f32")
    exe = os.path.join(ORACLE, "_ref", f"ref_cuda_d{depth}")
    r = subprocess.run([exe, f, str(warm), str(spp)] + ([out] if beauty else []), capture_output=True, text=True,
                       timeout=1200)
    assert r.returncode == 0, f"rc {r.returncode}: " + r.stdout[-2000:] + r.stderr[-2000:]
    line = [ln for ln in r.stdout.splitlines() if ln.startswith("{")][-1]
    res = json.loads(line)
    if beauty:
        W, H = arrays.camera["x_res"], arrays.camera["y_res"]
        res["beauty"] = np.fromfile(out, np.float32).reshape(W * H, 4)
    return res


def rel_rmse(a, b):
    a = np.asarray(a, np.float64)
    b = np.asarray(b, np.float64)
    return float(np.sqrt(((a - b) ** 2).sum() / max((b ** 2).sum(), 1e-300)))


def test_reference_cuda_film_matches_statistically(tmp_path):
    build_refcuda()
    arrays = scenes.config0()
    spp = 256
    ref = run_reference(arrays, 4, 0, spp, str(tmp_path))
    assert ref["samples_first_pixel"] <= spp and ref["max_bounces"] == 4
    with _lib.Scene(arrays) as s:
        a = s.render(spp, max_depth=4, seed=0)["beauty"][:, :3]
        b = s.render(spp, max_depth=4, seed=1)["beauty"][:, :3]
    R = ref["beauty"][:, :3]
    assert np.isfinite(R).all()
    e_self = rel_rmse(a, b)
    e_ref = rel_rmse(R, a)
    # per-channel mean radiance and its standard error (pixel-to-pixel
    # differences of two independent films)
    m_ref, m_a = R.mean(0), a.mean(0)
    se = (a - b).std(0) / np.sqrt(len(a))
    z = (m_ref - m_a) / se
    print(f"\nreference CUDA vs this library at {spp} spp (c0, 320x240): rel-RMSE {e_ref:.4f}, two seeds here "
          f"{e_self:.4f}; mean radiance z = {np.round(z, 2)}")
    assert e_ref < 1.15 * e_self, (e_ref, e_self)
    assert np.abs(z).max() < 5, z
