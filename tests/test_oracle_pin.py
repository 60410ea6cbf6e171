"""The oracle against the reference's own headers compiled here
(oracle/_ref/libref.so), on fresh random inputs.  Skipped where the
reference sources are absent (the GPU machine)."""
import numpy as np
import pytest

import _oracle as O
from eleven import scenes
from test_oracle_golden import hdri_defined, same

pytestmark = pytest.mark.skipif(O.ref() is None, reason="reference sources not present")


@pytest.fixture(scope="module")
def libs():
    return O.Probes(O.orc(), "orc_p_"), O.Probes(O.ref(), "ref_p_")


def test_random_triangles(libs):
    o, r = libs
    rng = np.random.default_rng(1)
    n = 50_000
    tris = np.zeros((n, 37), np.float32)
    tris[:, :9] = rng.uniform(-1, 1, (n, 9))
    tris[:, 9:18] = rng.uniform(0, 1, (n, 9))
    nn = rng.normal(size=(n, 3, 3))
    tris[:, 18:27] = (nn / np.linalg.norm(nn, axis=2, keepdims=True)).reshape(n, 9)
    tris[:, 27:37] = rng.normal(size=(n, 10))
    rays = np.zeros((n, 6), np.float32)
    rays[:, :3] = rng.uniform(-2, 2, (n, 3))
    rays[:, 3:] = -rays[:, :3] + rng.uniform(-0.5, 0.5, (n, 3))
    assert same(o.tri_hit(tris, rays), r.tri_hit(tris, rays)).all()


def test_random_disney(libs):
    o, r = libs
    rng = np.random.default_rng(2)
    n = 50_000
    hd = rng.uniform(0, 1, (n, 27)).astype(np.float32)
    nrm = rng.normal(size=(n, 3))
    nrm /= np.linalg.norm(nrm, axis=1, keepdims=True)
    hd[:, 18:21] = nrm
    d = rng.normal(size=(n, 3))
    L = rng.normal(size=(n, 3))
    d /= np.linalg.norm(d, axis=1, keepdims=True)
    L /= np.linalg.norm(L, axis=1, keepdims=True)
    L *= np.sign(np.sum(L * nrm, 1, keepdims=True))
    d *= -np.sign(np.sum(d * nrm, 1, keepdims=True))
    rnd = rng.uniform(0, 1, (n, 3))
    assert same(o.disney(hd, d, L, rnd), r.disney(hd, d, L, rnd)).all()


def test_sampling_and_mappings(libs):
    o, r = libs
    rng = np.random.default_rng(3)
    u = rng.uniform(0, 1, (20_000, 3))
    assert same(o.sampling(u), r.sampling(u)).all()
    p = rng.normal(size=(20_000, 3))
    p /= np.linalg.norm(p, axis=1, keepdims=True)
    assert same(o.spherical(p), r.spherical(p)).all()
    uv = rng.uniform(0, 1, (20_000, 2))
    assert same(o.reverse_spherical(uv), r.reverse_spherical(uv)).all()


def test_hdri_with_offset(libs):
    o, r = libs
    env = scenes.lognormal_env(256, 128, seed=1)
    c1, s1 = o.hdri_cdf(env, (0.3, 0.0))
    c2, s2 = r.hdri_cdf(env, (0.3, 0.0))
    assert same(c1, c2).all() and s1 == s2
    rv = np.random.default_rng(4).uniform(0, 1, 50_000).astype(np.float32)
    a, b = o.hdri_sample(env, c1, s1, rv, (0.3, 0.0)), r.hdri_sample(env, c1, s1, rv, (0.3, 0.0))
    ok = hdri_defined(b, env.shape[1], 0.3)
    assert same(a[ok], b[ok]).all()
    assert same(a[:, [0, 2, 3, 4]], b[:, [0, 2, 3, 4]]).all()
    a, b = o.hdri_sample(env, *o.hdri_cdf(env), rv), r.hdri_sample(env, *r.hdri_cdf(env), rv)
    assert same(a, b).all()


def test_c0_bvh_and_traversal():
    sc = scenes.config0()
    a, b = O.OrcScene(sc), O.RefScene(sc)
    ba, ma, ta = a.bvh()
    bb, mb, tb = b.bvh()
    assert same(ba, bb).all() and np.array_equal(ma, mb) and np.array_equal(ta, tb)
    rays = scenes.random_rays(sc, 100_000, seed=13)
    ia, da = a.trace(rays)
    ib, db = b.trace(rays)
    assert np.array_equal(ia, ib) and same(da, db).all()
    a.close()
    b.close()


@pytest.mark.gpu
def test_pins_hold_where_the_gpu_runs(libs):
    """The same pins in the GPU session: there the reference headers and the
    oracle are compiled for that machine's host CPU, so this checks that the
    restatement still equals the reference built there."""
    import inspect
    for name, fn in list(globals().items()):
        if name.startswith("test_") and name != "test_pins_hold_where_the_gpu_runs" and callable(fn):
            fn(libs) if inspect.signature(fn).parameters else fn()
