"""GPU post-processing (er_postprocess) against the oracle's restatement of
the reference's PostProcessing.cpp, and its LDR output against the host
encoder (er_encode_ldr)."""
import numpy as np
import pytest

import _oracle as O
from eleven import _abi as A
from eleven import _lib

pytestmark = pytest.mark.gpu

W, H = 67, 45


def _image(seed=0):
    rng = np.random.default_rng(seed)
    img = np.exp(rng.normal(-0.5, 1.5, (W * H, 4))).astype(np.float32)
    img[:, 3] = 1.0
    img[rng.integers(0, W * H, 40), 0] = -0.3      # negative channels
    img[rng.integers(0, W * H, 40), 1] = 0.0
    img[7, 2] = np.nan                               # a NaN survives as in the reference
    return img


CASES = [
    dict(),
    dict(exposure=1.7, clamp=1),
    dict(tonemap=A.ER_TONEMAP_REINHARD, srgb=1),
    dict(tonemap=A.ER_TONEMAP_ACES, exposure=0.8),
    dict(clamp=1, srgb=1, flip_x=1),
    dict(flip_y=1, tonemap=A.ER_TONEMAP_ACES, srgb=1),
    dict(bloom_threshold=1.0, bloom_power=0.3, bloom_radius=5.0),
    dict(exposure=1.2, bloom_threshold=0.5, bloom_power=0.7, bloom_radius=9.0, tonemap=A.ER_TONEMAP_REINHARD,
         clamp=1, srgb=1, flip_x=1, flip_y=1),
]


@pytest.mark.parametrize("case", CASES)
def test_postprocess_matches_oracle(case):
    img = _image(1)
    kw = dict(exposure=1.0, tonemap=0, clamp=0, srgb=0, flip_x=0, flip_y=0, bloom_threshold=0.0, bloom_power=0.0,
              bloom_radius=0.0)
    kw.update(case)
    out, ldr = _lib.postprocess(img, W, H, **kw)
    o = A.er_post_opts(kw["exposure"], kw["tonemap"], kw["clamp"], kw["srgb"], kw["flip_x"], kw["flip_y"],
                       kw["bloom_threshold"], kw["bloom_power"], kw["bloom_radius"])
    want = O.postprocess(img, W, H, o)
    if kw["srgb"]:
        # double pow of CUDA and of the host libm may round 1 ulp apart
        # before the conversion to float
        fin = np.isfinite(want)
        np.testing.assert_array_max_ulp(out[fin], want[fin], maxulp=1)
        assert np.array_equal(np.isnan(out), np.isnan(want))
    else:
        assert np.array_equal(out.view(np.uint32), want.view(np.uint32)) or np.allclose(
            out, want, rtol=0, atol=0, equal_nan=True)
    # the LDR bytes are er_encode_ldr of the float result
    assert np.array_equal(ldr, _lib.encode_ldr(out, W, H))


def test_postprocess_rejects_bad_input():
    img = _image(2)
    with pytest.raises(_lib.ElevenError):
        _lib.postprocess(img, W, H, tonemap=7)
    with pytest.raises(_lib.ElevenError):
        _lib.postprocess(img, 0, H)


def test_postprocess_matches_reference_golden():
    """er_postprocess against the reference's own PostProcessing.cpp
    (golden outputs in tests/golden/reference_io.npz), on the pixels and
    channels the reference defines; the sRGB power within 1 ulp."""
    from test_loader_reference import GOLD, _post_cases
    G = dict(np.load(GOLD))
    n = 0
    for k, w, h, o, px, ref, mask in _post_cases(G):
        out, _ = _lib.postprocess(px, w, h, exposure=o.exposure, tonemap=o.tonemap, clamp=o.clamp, srgb=o.srgb,
                                  flip_x=o.flip_x, flip_y=o.flip_y, bloom_threshold=o.bloom_threshold,
                                  bloom_power=o.bloom_power, bloom_radius=o.bloom_radius)
        a = out.view(np.uint32)[mask].astype(np.int64)
        b = ref.view(np.uint32)[mask].astype(np.int64)
        assert np.abs(a - b).max() <= (1 if o.srgb else 0), k
        n += int(mask.sum())
    assert n > 10_000
