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


def test_search_lookup_table_matches_the_oracle_per_path():
    """Environments of >= 65,536 texels are sampled through a table of the
    CDF search's result for each of its 2^24 inputs (env.cu): the chosen
    texels, and so the paths, are the reference search's.  Per-path parity
    with the oracle (which runs the search) on a 512x256 environment, and
    the film of a second scene handle built the same way is identical."""
    arrays = scenes.displaced_spheres(20000, 5, 64, 48, 2, env_w=512, env_h=256)
    scene = _lib.Scene(arrays)
    orc = O.OrcScene(arrays)
    rad, b = scene.render_paths(spp=2, max_depth=4, seed=13)
    rrad, rb = orc.render_paths(spp=2, max_depth=4, seed=13)
    # measured: bounce counts 100 %, radiance 99.97 % (98.5 % bit for bit)
    assert (b == rb).mean() > 0.999
    close = np.isclose(rad, rrad, rtol=1e-3, atol=1e-5).all(axis=2)
    both_nan = np.isnan(rad).any(2) & np.isnan(rrad).any(2)
    assert (close | both_nan).mean() > 0.999
    a = scene.render(4, max_depth=4, seed=2)["beauty"]
    other = _lib.Scene(arrays)
    c = other.render(4, max_depth=4, seed=2)["beauty"]
    assert np.array_equal(a.view(np.uint32), c.view(np.uint32))
    other.close()
    scene.close()
    orc.close()


@pytest.mark.parametrize("w,h,sun", [(512, 256, 8), (256, 256, 0)])
def test_search_table_is_the_search(w, h, sun):
    """The 2^24-entry table equals the reference search everywhere: it is
    non-decreasing (as the search is in its input) and its histogram equals
    the oracle's per-texel counts of the search, so the two maps agree on
    every input."""
    arrays = _env_scene(w, h, sun)
    cdf, _ = O.Probes(O.orc(), "orc_p_").hdri_cdf(arrays.env)
    want = O.hdri_counts(cdf, w * h)
    table = np.zeros(1 << 24, np.int32)
    with _lib.Scene(arrays) as s:
        _lib.check(_lib.load().er_env_search_table(s.h, _lib._p(table)), "er_env_search_table")
    assert np.all(np.diff(table) >= 0)
    assert table.min() >= 0 and table.max() < w * h
    np.testing.assert_array_equal(np.bincount(table, minlength=w * h), want)


def test_search_table_needs_a_large_environment():
    arrays = _env_scene(64, 32, 0)
    table = np.zeros(1 << 24, np.int32)
    with _lib.Scene(arrays) as s:
        assert _lib.load().er_env_search_table(s.h, _lib._p(table)) == A.ER_ERR_INVALID_ARG
