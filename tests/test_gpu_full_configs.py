"""GPU parity at the benchmark configurations' stated sizes.

- Small scene in full: 320x240 pinhole, 16 icospheres + ground quad,
  16 spp, max depth 4.  Every path of every sample against the oracle
  (same random numbers), and the film against the oracle's film.
- Differentiation scene in full: 512x512, 64 icospheres, 256x128 env,
  max depth 6, 98,624 parameters.  The adjoint gradient at 4096 samples per
  pixel against central finite differences (h = 1e-3, the same 4096 samples:
  common random numbers) of the detached estimator on 32 random parameters
  where it is differentiable, relative error below 1e-2; then 100 Adam
  steps (lr 1e-2, 64 spp) lower the loss.  The clamp of kernel.cu:447 and the 2.2 power of
  kernel.cu:103-104 are inside the differentiated estimator.
"""
import numpy as np
import pytest

import _oracle as O
from eleven import _lib, scenes

pytestmark = pytest.mark.gpu


def rel_rmse(a, b):
    a = np.asarray(a, np.float64)
    b = np.asarray(b, np.float64)
    return float(np.sqrt(((a - b) ** 2).sum() / max((b ** 2).sum(), 1e-300)))


@pytest.fixture(scope="module")
def c0_full():
    arrays = scenes.config0()
    assert (arrays.camera["x_res"], arrays.camera["y_res"]) == (320, 240)
    assert arrays.tri_count == 20482
    s = _lib.Scene(arrays)
    orc = O.OrcScene(arrays)
    yield arrays, s, orc
    s.close()
    orc.close()


def test_c0_full_paths_match_oracle(c0_full):
    """All 1,228,800 paths (16 samples of 76,800 pixels, depth 4)."""
    arrays, s, orc = c0_full
    rad, b = s.render_paths(spp=16, max_depth=4, seed=0)
    rrad, rb = orc.render_paths(spp=16, max_depth=4, seed=0)
    assert rad.shape == (16, 320 * 240, 3)
    same_b = (b == rb).mean()
    close = np.isclose(rad, rrad, rtol=1e-3, atol=1e-5).all(axis=2)
    both_nan = np.isnan(rad).any(2) & np.isnan(rrad).any(2)
    frac = (close | both_nan).mean()
    exact = (rad.view(np.uint32) == rrad.view(np.uint32)).all(axis=2).mean()
    print(f"\nc0 full: bounce counts equal {same_b:.5f}, radiance within 1e-3 {frac:.5f}, bit for bit {exact:.4f}")
    assert same_b > 0.999, f"bounce counts agree on {same_b:.5f} of paths"
    assert frac > 0.999, f"per-path radiance agrees on {frac:.5f} of paths"


def test_c0_full_film_matches_oracle(c0_full):
    arrays, s, orc = c0_full
    out = s.render(spp=16, max_depth=4, seed=0)
    ref = orc.render(spp=16, max_depth=4, seed=0)
    e = rel_rmse(out["beauty"][:, :3], ref["beauty"][:, :3])
    print(f"\nc0 full: film rel-RMSE vs oracle {e:.3e}")
    assert e < 1e-4, e  # measured 5.8e-6
    assert (out["beauty"][:, 3] == 1).all()
    assert np.abs(out["samples"].astype(np.int64) - ref["samples"]).max() <= 1
    assert out["samples"].mean() > 15.9
    assert np.abs(out["pathcount"].astype(np.int64) - ref["pathcount"].astype(np.int64)).mean() < 0.05


C4_DEPTH = 6


@pytest.fixture(scope="module")
def c4_full():
    arrays = scenes.config4()
    target = scenes.config4(param_seed=41)
    s = _lib.Scene(arrays)
    with _lib.Scene(target) as t:
        T = t.render(64, max_depth=C4_DEPTH, seed=99)["beauty"]
    m0, e0 = s.get_params()
    assert m0.size + e0.size == 98_624
    yield arrays, s, T
    s.close()


def _loss(beauty, T):
    d = beauty[:, :3].astype(np.float64) - T[:, :3].astype(np.float64)
    return float((d * d).sum())


def _loss_exact(sums, samples, T):
    """The loss of the film's exact (FP64) pixel means."""
    img = sums / np.maximum(samples, 1)[:, None]
    d = img - T[:, :3].astype(np.float64)
    return float((d * d).sum())


def test_c4_full_gradient_matches_fd_4096spp(c4_full):
    """32 random parameters: 16 of the 256 albedo and roughness parameters
    and 16 of the 98,304 environment texel channels.  The metallic
    parameters are excluded: the configuration draws them from {0, 1}, where
    the estimator is not differentiable (below 0 the 2.2 power of
    kernel.cu:104 is undefined; at 1 the diffuse lobe's (1 - metallic)
    changes sign and the samples it alone lights are clamped at 0 on one
    side, kernel.cu:447), so a central difference there does not estimate
    the gradient.  The finite differences are taken of the films' FP64 sums
    (ER_RENDER_ACCUM_FP64, er_film_read_sums): neither the FP32 running mean
    nor the final rounding of each pixel to float enters the differences,
    whose step of 1e-3 would otherwise move the loss by less than that
    rounding for the smaller gradients."""
    from eleven import _abi as A
    arrays, s, T = c4_full
    spp, h, seed = 4096, 1e-3, 5
    m0, e0 = s.get_params()
    out = s.render(spp, max_depth=C4_DEPTH, seed=seed)
    d = np.zeros_like(out["beauty"])
    d[:, :3] = 2.0 * (out["beauty"][:, :3] - T[:, :3])
    gm, ge, _ = s.backward(spp, d, out["samples"], max_depth=C4_DEPTH, seed=seed)
    g = np.concatenate([gm.ravel(), ge.ravel()]).astype(np.float64)
    assert np.isfinite(g).all()
    gmax = np.abs(g).max()
    rng = np.random.default_rng(32)
    smooth = np.nonzero(np.arange(m0.size) % 5 != 4)[0]  # albedo r, g, b and roughness
    idx = list(rng.choice(smooth, 16, replace=False)) + list(m0.size + rng.choice(e0.size, 16, replace=False))
    rows = []
    for k in idx:
        vals = []
        for sign in (1, -1):
            m, e = m0.copy(), e0.copy()
            if k < m0.size:
                m.ravel()[k] += sign * h
            else:
                e.ravel()[k - m0.size] += sign * h
            s.render_replay(spp, max_depth=C4_DEPTH, seed=seed, materials=m, env=e, flags=A.ER_RENDER_ACCUM_FP64)
            vals.append(_loss_exact(*s.read_sums(), T))
        fd = (vals[0] - vals[1]) / (2 * h)
        big = max(abs(fd), abs(g[k]))
        rows.append((int(k), float(g[k]), fd, abs(fd - g[k]) / big if big > 0 else 0.0, big))
    print("\nc4 full, 4096 spp: (param, adjoint, finite difference, rel) " +
          "; ".join(f"{k} {a:.5g} {b:.5g} {r:.2e}" for k, a, b, r, _ in rows))
    # parameters whose gradient is below 1e-7 of the largest one: reported,
    # not checked
    checked = [r for r in rows if r[4] >= 1e-7 * gmax]
    bad = [r for r in checked if r[3] >= 1e-2]
    assert not bad, f"relative error >= 1e-2: {bad}"
    assert len(checked) >= 28, f"only {len(checked)} of 32 parameters above the noise floor"


def test_c4_full_adam_100_steps(c4_full):
    torch = pytest.importorskip("torch")
    from eleven import adjoint
    arrays, s, T = c4_full
    m0, e0 = s.get_params()
    dev = torch.device("cuda:0")
    Tt = torch.tensor(T, device=dev)
    try:
        _, _, hist = adjoint.optimize(s, Tt, torch.tensor(m0, device=dev), torch.tensor(e0, device=dev), steps=100,
                                      lr=1e-2, spp=64, max_depth=C4_DEPTH)
    finally:
        s.set_params(m0, e0)
    print(f"\nc4 full, Adam lr 1e-2: loss {hist[0]:.4g} -> {hist[-1]:.4g} (min {min(hist):.4g})")
    assert len(hist) == 100
    assert np.mean(hist[-10:]) < 0.8 * np.mean(hist[:3])
