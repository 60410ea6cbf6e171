"""How far per-path results move under last-place rounding differences of
single-precision transcendental functions alone (CPU, oracle only).

oracle/liborc_ulp.so is the oracle built with its sinf, cosf, acosf,
atan2f, powf and logf results moved by a few units in the last place
(oracle/orc_ulp.h; level 1: half of the calls by one ulp, level 2: every
call by one or two).  Per-path radiance and bounce counts of the plain
oracle are compared with it under the same random numbers:

- the 16-icosphere scene (depth 4) barely moves, which is why the GPU
  per-path threshold there is 99.9 %;
- the 1.18M-triangle scene (dense small triangles, an environment whose
  texel radiance spreads over e^(+-2) with a 1e4 sun, depth 8) moves by
  about 1 % of its paths at level 1 and 4 % at level 2: one rounding
  difference at a vertex can carry a ray past a triangle edge or across an
  environment texel boundary, after which the path is another sample.  The
  GPU path, with CUDA's implementations of these functions, differs from
  the oracle by an amount inside that range (97.7 % of paths within 1e-3),
  which sets the threshold of tests/test_gpu_parity_c1.py.
"""
import os
import subprocess
import sys

import numpy as np
import pytest

import _oracle as O
from eleven import scenes

HERE = os.path.dirname(os.path.abspath(__file__))
ULP_LIB = os.path.join(O.ROOT, "oracle", "liborc_ulp.so")

CASES = {
    "c0": (lambda: scenes.config0(x_res=96, y_res=72), dict(spp=2, max_depth=4, seed=11)),
    "c1": (lambda: scenes.config1(x_res=320, y_res=180), dict(spp=1, max_depth=8, seed=5)),
}

CHILD = r"""
import sys
import numpy as np
sys.path[:0] = [{here!r}, {pkg!r}]
import test_oracle_sensitivity as T
import _oracle as O
out = {{}}
for name, (make, opts) in T.CASES.items():
    orc = O.OrcScene(make())
    for level in (1, 2):
        O.orc().orc_ulp_set_level(level)
        out[f"{{name}}_{{level}}_rad"], out[f"{{name}}_{{level}}_b"] = orc.render_paths(**opts)
    orc.close()
np.savez({dst!r}, **out)
"""


def agreement(rad, b, rrad, rb):
    close = np.isclose(rad, rrad, rtol=1e-3, atol=1e-5).all(axis=-1)
    both_nan = np.isnan(rad).any(-1) & np.isnan(rrad).any(-1)
    return float((b == rb).mean()), float((close | both_nan).mean())


@pytest.fixture(scope="module")
def probe(tmp_path_factory):
    subprocess.run(["make", "-s", "-C", os.path.join(O.ROOT, "oracle"), "liborc_ulp.so"], check=True)
    dst = str(tmp_path_factory.mktemp("ulp") / "ulp.npz")
    code = CHILD.format(here=HERE, pkg=os.path.join(O.ROOT, "tfg-pathtracer_gb300"), dst=dst)
    subprocess.run([sys.executable, "-c", code], check=True, env=dict(os.environ, ORC_LIB=ULP_LIB), timeout=900)
    return dict(np.load(dst))


def test_perturbed_build_is_the_oracle_at_level_0():
    """With no perturbation the probe build renders the plain oracle's
    paths bit for bit (the header changes nothing else)."""
    make, opts = CASES["c0"]
    arrays = make()
    orc = O.OrcScene(arrays)
    rad, b = orc.render_paths(**opts)
    orc.close()
    subprocess.run(["make", "-s", "-C", os.path.join(O.ROOT, "oracle"), "liborc_ulp.so"], check=True)
    code = (f"import sys; sys.path[:0] = [{HERE!r}, {os.path.join(O.ROOT, 'tfg-pathtracer_gb300')!r}]\n"
            "import numpy as np, test_oracle_sensitivity as T, _oracle as O\n"
            "make, opts = T.CASES['c0']; orc = O.OrcScene(make()); r, b = orc.render_paths(**opts)\n"
            "sys.stdout.buffer.write(r.tobytes() + b.tobytes())\n")
    raw = subprocess.run([sys.executable, "-c", code], check=True, capture_output=True,
                         env=dict(os.environ, ORC_LIB=ULP_LIB), timeout=600).stdout
    assert raw == rad.tobytes() + b.tobytes()


def test_small_scene_is_insensitive(probe):
    make, opts = CASES["c0"]
    orc = O.OrcScene(make())
    rad, b = orc.render_paths(**opts)
    orc.close()
    for level in (1, 2):
        same_b, within = agreement(probe[f"c0_{level}_rad"], probe[f"c0_{level}_b"], rad, b)
        print(f"\nc0 level {level}: bounces {same_b:.5f}, within 1e-3 {within:.5f}")
        assert same_b > 0.999 and within > 0.9995


def test_full_feature_scene_moves_by_percents(probe):
    make, opts = CASES["c1"]
    orc = O.OrcScene(make())
    rad, b = orc.render_paths(**opts)
    orc.close()
    res = {}
    for level in (1, 2):
        res[level] = agreement(probe[f"c1_{level}_rad"], probe[f"c1_{level}_b"], rad, b)
        print(f"\nc1 level {level}: bounces {res[level][0]:.5f}, within 1e-3 {res[level][1]:.5f}")
    # measured: level 1 bounces 99.87 %, within 1e-3 99.13 %; level 2 99.24 % / 95.75 %
    assert 0.98 < res[1][1] < 0.999
    assert 0.93 < res[2][1] < 0.99
    assert res[2][1] < res[1][1]
