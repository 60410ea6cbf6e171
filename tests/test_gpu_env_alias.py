"""GPU: the alias-table environment sampler (ER_RENDER_ENV_ALIAS).

The reference draws an environment texel with HDRI::binarySearch
(HDRI.hpp:130-142); the texel it returns for a uniform r, not the CDF, sets
the sampling distribution.  The alias table must reproduce that effective
distribution exactly: its counts over the 2^24-value uniform grid equal the
oracle's, and the table's column masses equal counts / 2^24 as exact
integers.  Renders with the table are then the same estimator with other
random numbers, so they agree with the binary-search renders in mean.
"""
import dataclasses

import numpy as np
import pytest

import _oracle as O
from eleven import _abi as A
from eleven import _lib, scenes

pytestmark = pytest.mark.gpu


def _env_scene(w, h, sun):
    arrays = scenes.config0(x_res=64, y_res=48)
    env = scenes.lognormal_env(w, h, seed=5, sigma=1.5, sun=sun, sun_value=2e3)
    return dataclasses.replace(arrays, env=env)


def _distribution(scene, n):
    L = _lib.load()
    counts = np.zeros(n, np.uint32)
    alias = np.zeros(n, np.int32)
    thresh = np.zeros(n, np.uint32)
    _lib.check(L.er_env_distribution(scene.h, _lib._p(counts), _lib._p(alias), _lib._p(thresh)),
               "er_env_distribution")
    return counts, alias, thresh


@pytest.mark.parametrize("w,h,sun", [(64, 32, 4), (128, 64, 0), (48, 24, 3)])
def test_effective_counts_equal_oracle(w, h, sun):
    arrays = _env_scene(w, h, sun)
    cdf, _ = O.Probes(O.orc(), "orc_p_").hdri_cdf(arrays.env)
    want = O.hdri_counts(cdf, w * h)
    assert int(want.sum()) == 1 << 24
    with _lib.Scene(arrays) as s:
        counts, alias, thresh = _distribution(s, w * h)
    np.testing.assert_array_equal(counts, want)
    assert alias.min() >= 0 and alias.max() < w * h


@pytest.mark.parametrize("w,h,sun", [(64, 32, 4), (128, 64, 0)])
def test_alias_table_reproduces_counts_exactly(w, h, sun):
    """Power-of-two texel count n: column i has mass 1/n; a 32-bit coin
    below thresh[i] keeps i, else alias[i].  Total mass of texel t in units
    of 2^-32 / n must equal counts[t] * n * 2^8 (= counts / 2^24)."""
    n = w * h
    arrays = _env_scene(w, h, sun)
    with _lib.Scene(arrays) as s:
        counts, alias, thresh = _distribution(s, n)
    keep = thresh.astype(np.int64)
    full = thresh == 0xFFFFFFFF
    # a full column either keeps itself or aliases itself: all 2^32 coins
    assert np.all(alias[full] == np.nonzero(full)[0])
    keep[full] = 1 << 32
    mass = np.zeros(n, np.int64)
    np.add.at(mass, np.arange(n), keep)
    np.add.at(mass, alias, (1 << 32) - keep)
    np.testing.assert_array_equal(mass, counts.astype(np.int64) * n * 256)


def _mean_z(a, b):
    d = (np.asarray(a, np.float64) - np.asarray(b, np.float64)).ravel()
    return abs(d.mean()) / max(d.std(ddof=1) / np.sqrt(d.size), 1e-30)


def test_alias_render_unbiased_against_search():
    arrays = _env_scene(64, 32, 4)
    with _lib.Scene(arrays) as s:
        base = s.render(64, max_depth=3, seed=11)["beauty"][:, :3]
        other = s.render(64, max_depth=3, seed=12)["beauty"][:, :3]
        alias = s.render(64, max_depth=3, seed=11, flags=A.ER_RENDER_ENV_ALIAS)["beauty"][:, :3]
        assert np.isfinite(alias).all()
        # same estimator: the mean difference is noise (z well under 5)
        assert _mean_z(alias, base) < 5.0
        assert _mean_z(other, base) < 5.0
        # and no noisier than an independent re-render
        err_alias = np.sqrt(((alias - base) ** 2).mean())
        err_other = np.sqrt(((other - base) ** 2).mean())
        assert err_alias <= 1.25 * err_other
        # the flag is deterministic
        again = s.render(64, max_depth=3, seed=11, flags=A.ER_RENDER_ENV_ALIAS)["beauty"][:, :3]
        np.testing.assert_array_equal(again, alias)
