"""GPU: path replay and the adjoint (er_render_replay, er_backward).

1. The replay walk re-traces every path from its counter-based random
   numbers; as a forward render it equals er_render bit for bit.
2. Gradients of an L2 image loss against central finite differences
   (step 1e-3, common random numbers) of the detached estimator the
   adjoint differentiates (er_render_replay with evaluation parameters
   theta +- h, sampling at theta): relative error below 1e-2 on every
   checked parameter whose gradient is not negligible.
3. The torch.autograd.Function returns the same gradients, and Adam steps
   on it lower the loss.
4. The FP64 oracle's gradient (central differences of the same detached
   estimator evaluated in double) agrees with the FP32 adjoint.
"""
import numpy as np
import pytest

import _oracle as O
from eleven import _abi as A
from eleven import _lib, scenes

pytestmark = pytest.mark.gpu

SPP, DEPTH, SEED = 16, 4, 7


@pytest.fixture(scope="module")
def small():
    arrays = scenes.config4(x_res=48, y_res=40, n_obj=12, env_w=32, env_h=16)
    target = scenes.config4(x_res=48, y_res=40, n_obj=12, env_w=32, env_h=16, param_seed=41)
    s = _lib.Scene(arrays)
    t = _lib.Scene(target)
    T = t.render(SPP, max_depth=DEPTH, seed=99)["beauty"]
    t.close()
    return arrays, s, T


def test_replay_equals_render(small):
    arrays, s, T = small
    for flags in (0, A.ER_RENDER_ENV_ALIAS):
        a = s.render(5, max_depth=5, seed=3, sample_begin=2, flags=flags)
        b = s.render_replay(5, max_depth=5, seed=3, sample_begin=2, flags=flags)
        assert np.array_equal(a["beauty"].view(np.uint32), b["beauty"].view(np.uint32))
        assert np.array_equal(a["samples"], b["samples"])
        assert np.array_equal(a["pathcount"], b["pathcount"])
    q8 = _lib.Scene(arrays, bvh_format=A.ER_BVH_Q8)
    c = q8.render_replay(5, max_depth=5, seed=3, sample_begin=2)
    a = s.render(5, max_depth=5, seed=3, sample_begin=2)
    assert np.array_equal(a["beauty"].view(np.uint32), c["beauty"].view(np.uint32))
    q8.close()


def test_replay_with_scene_params_equals_eval_params(small):
    """Evaluation parameters equal to the scene's: the same film up to the
    compiler's choice of fused multiply-adds in the re-evaluated BRDF."""
    arrays, s, T = small
    m, e = s.get_params()
    a = s.render_replay(3, max_depth=4, seed=1)
    b = s.render_replay(3, max_depth=4, seed=1, materials=m, env=e)
    np.testing.assert_allclose(b["beauty"], a["beauty"], rtol=2e-6, atol=1e-7)
    assert np.array_equal(a["samples"], b["samples"])


def _loss(beauty, T):
    d = beauty[:, :3].astype(np.float64) - T[:, :3].astype(np.float64)
    return float((d * d).sum())


def test_gradients_match_finite_differences(small):
    arrays, s, T = small
    m0, e0 = s.get_params()
    out = s.render(SPP, max_depth=DEPTH, seed=SEED)
    I0 = out["beauty"]
    d = np.zeros_like(I0)
    d[:, :3] = 2.0 * (I0[:, :3] - T[:, :3])
    gm, ge, st = s.backward(SPP, d, out["samples"], max_depth=DEPTH, seed=SEED)
    assert np.isfinite(gm).all() and np.isfinite(ge).all()
    assert st.ms > 0
    rng = np.random.default_rng(0)
    # parameters: the 6 largest material gradients, 6 random material
    # parameters, the 6 largest env gradients, 6 random seen env texels
    gmf, gef = gm.ravel(), ge.ravel()
    mat_idx = list(np.argsort(-np.abs(gmf))[:6]) + list(rng.choice(np.nonzero(gmf)[0], 6, replace=False))
    seen = np.nonzero(gef)[0]
    env_idx = list(np.argsort(-np.abs(gef))[:6]) + list(rng.choice(seen, 6, replace=False))
    h = 1e-3
    gmax_m, gmax_e = np.abs(gmf).max(), np.abs(gef).max()
    checked = 0
    for kind, idx in [("m", i) for i in mat_idx] + [("e", i) for i in env_idx]:
        vals = []
        for sign in (+1, -1):
            m, e = m0.copy(), e0.copy()
            if kind == "m":
                m.ravel()[idx] += sign * h
            else:
                e.ravel()[idx] += sign * h
            r = s.render_replay(SPP, max_depth=DEPTH, seed=SEED, materials=m, env=e)
            vals.append(_loss(r["beauty"], T))
        fd = (vals[0] - vals[1]) / (2 * h)
        g = float(gmf[idx] if kind == "m" else gef[idx])
        gmax = gmax_m if kind == "m" else gmax_e
        if max(abs(fd), abs(g)) < 1e-3 * gmax:
            continue  # negligible: FP32 loss differences dominate
        rel = abs(fd - g) / max(abs(fd), abs(g))
        assert rel < 1e-2, f"{kind}[{idx}]: adjoint {g:.6g} vs finite difference {fd:.6g} (rel {rel:.3g})"
        checked += 1
    assert checked >= 12


def test_torch_autograd_and_adam(small):
    torch = pytest.importorskip("torch")
    from eleven import adjoint
    arrays, s, T = small
    m0, e0 = s.get_params()
    dev = torch.device("cuda:0")
    m = torch.tensor(m0, device=dev, requires_grad=True)
    e = torch.tensor(e0, device=dev, requires_grad=True)
    Tt = torch.tensor(T, device=dev)
    img = adjoint.render(s, m, e, SPP, max_depth=DEPTH, seed=SEED)
    loss = adjoint.l2_loss(img, Tt)
    loss.backward()
    # same gradients as the numpy path
    s.set_params(m0, e0)
    out = s.render(SPP, max_depth=DEPTH, seed=SEED)
    d = np.zeros_like(out["beauty"])
    d[:, :3] = 2.0 * (out["beauty"][:, :3] - T[:, :3])
    gm, ge, _ = s.backward(SPP, d, out["samples"], max_depth=DEPTH, seed=SEED)
    np.testing.assert_allclose(m.grad.cpu().numpy(), gm, rtol=1e-4, atol=1e-6 * np.abs(gm).max())
    np.testing.assert_allclose(e.grad.cpu().numpy(), ge, rtol=1e-4, atol=1e-6 * np.abs(ge).max())
    # a few Adam steps lower the loss
    _, _, hist = adjoint.optimize(s, Tt, torch.tensor(m0, device=dev), torch.tensor(e0, device=dev), steps=8,
                                  lr=2e-2, spp=8, max_depth=DEPTH)
    assert hist[-1] < hist[0]
    s.set_params(m0, e0)


def test_gradients_match_fp64_oracle(small):
    """The GPU adjoint (FP32) against the FP64 oracle's gradient: central
    differences (h = 1e-4) of the same detached estimator evaluated in
    double (oracle/orc64.c), same samples.  Paths on which FP32 and FP64
    round a discrete decision apart make the two estimators differ slightly,
    so the bar is looser than the FP32 finite-difference check."""
    arrays, s, T = small
    m0, e0 = s.get_params()
    out = s.render(SPP, max_depth=DEPTH, seed=SEED)
    I0 = out["beauty"]
    d = np.zeros_like(I0)
    d[:, :3] = 2.0 * (I0[:, :3] - T[:, :3])
    gm, ge, _ = s.backward(SPP, d, out["samples"], max_depth=DEPTH, seed=SEED)
    orc = O.OrcScene(arrays)
    o64 = O.Orc64(orc)
    W, H = 48, 40
    idx = np.arange(W * H)
    T64 = T[:, :3].astype(np.float64)

    def loss(m, e):
        rgb, _ = o64.render_pixels(idx, SPP, DEPTH, seed=SEED, eval_mat=m, eval_env=e)
        return float(((rgb - T64) ** 2).sum())

    gmf, gef = gm.ravel(), ge.ravel()
    picks = [("m", i) for i in np.argsort(-np.abs(gmf))[:6]] + [("e", i) for i in np.argsort(-np.abs(gef))[:6]]
    h = 1e-4
    errs = []
    for kind, i in picks:
        vals, xs = [], []
        for sign in (1, -1):
            m, e = m0.copy(), e0.copy()
            (m if kind == "m" else e).ravel()[i] += sign * h
            xs.append(float((m if kind == "m" else e).ravel()[i]))  # the float32 value actually used
            vals.append(loss(m, e))
        fd = (vals[0] - vals[1]) / (xs[0] - xs[1])
        g = float(gmf[i] if kind == "m" else gef[i])
        errs.append(abs(fd - g) / max(abs(fd), abs(g)))
    print("\nadjoint vs FP64 oracle gradient, relative errors:", np.round(errs, 5))
    assert np.median(errs) < 1e-2
    assert max(errs) < 5e-2
    o64.close()
    orc.close()


def test_kept_paths_give_the_same_gradient(small):
    """er_render with ER_RENDER_KEEP_PATHS lets er_backward skip its forward
    pass; the gradient is the one er_backward computes on its own (up to the
    order of the float atomics), and a backward with other options, or after
    a parameter change, does not use the kept radiance."""
    arrays, s, T = small
    m0, e0 = s.get_params()

    def grads(seed, keep, other_seed=None):
        out = s.render(SPP, max_depth=DEPTH, seed=seed, flags=A.ER_RENDER_KEEP_PATHS if keep else 0)
        d = np.zeros_like(out["beauty"])
        d[:, :3] = 2.0 * (out["beauty"][:, :3] - T[:, :3])
        bs = seed if other_seed is None else other_seed
        gm, ge, st = s.backward(SPP, d, out["samples"], max_depth=DEPTH, seed=bs)
        # launches: per gradient wave raygen, DEPTH + 1 traces, DEPTH shades,
        # the resolve; without kept radiance also the forward's own waves
        # (raygen, traces, shades, the per-path dump)
        waves = 2  # 16 spp at 48x40: waves of 8 samples
        grad = waves * (2 * DEPTH + 3)
        assert st.kernel_launches == (grad if keep else grad + waves * (2 * DEPTH + 3)), st.kernel_launches
        return gm, ge, d, out["samples"]

    def close(a, b):
        np.testing.assert_allclose(a, b, rtol=1e-4, atol=1e-6 * max(np.abs(b).max(), 1e-30))

    gm_k, ge_k, d, smp = grads(7, True)
    gm_n, ge_n, _, _ = grads(7, False)
    close(gm_k, gm_n)
    close(ge_k, ge_n)
    # kept radiance of seed 7, backward of seed 8: recomputed, not reused
    s.render(SPP, max_depth=DEPTH, seed=7, flags=A.ER_RENDER_KEEP_PATHS)
    gm_8a, ge_8a, _ = s.backward(SPP, d, smp, max_depth=DEPTH, seed=8)
    s.render(SPP, max_depth=DEPTH, seed=1)
    gm_8b, ge_8b, _ = s.backward(SPP, d, smp, max_depth=DEPTH, seed=8)
    close(gm_8a, gm_8b)
    close(ge_8a, ge_8b)
    # a parameter change after the kept render: recomputed with the new parameters
    s.render(SPP, max_depth=DEPTH, seed=7, flags=A.ER_RENDER_KEEP_PATHS)
    m1 = m0.copy()
    m1[:, 3] = np.clip(m1[:, 3] * 0.5, 0.05, 1.0)
    s.set_params(m1, e0)
    gm_c, ge_c, _ = s.backward(SPP, d, smp, max_depth=DEPTH, seed=7)
    s.render(SPP, max_depth=DEPTH, seed=1)
    gm_d, ge_d, _ = s.backward(SPP, d, smp, max_depth=DEPTH, seed=7)
    close(gm_c, gm_d)
    close(ge_c, ge_d)
    assert not np.allclose(gm_c, gm_k)
    s.set_params(m0, e0)
