"""The FP64 oracle (oracle/orc64.c) against the FP32 oracle.

Its own BVH and pruned traversal must select the same closest triangles as
the restated reference traversal (BVH::transverse) except where the two
precisions rank nearly equal distances differently, and its images must
agree with the FP32 oracle's to within the precision difference (same
random numbers, same texel choices).
"""
import numpy as np

import _oracle as O
from eleven import scenes


def test_fp64_hit_selection_matches_reference_traversal():
    arrays = scenes.config0(x_res=32, y_res=24)
    orc = O.OrcScene(arrays)
    o64 = O.Orc64(orc)
    rays = scenes.random_rays(arrays, 40_000, seed=9)
    t32, d32 = orc.trace(rays)
    t64, d64 = o64.trace(rays)
    assert (t32 >= 0).sum() > 10_000
    bad = np.nonzero(t32 != t64)[0]
    # every disagreement is a near tie: the FP32 distances agree to 1e-5
    near = np.isfinite(d32[bad]) & (np.abs(d32[bad] - d64[bad]) <= 1e-5 * np.maximum(1.0, d64[bad]))
    assert near.all(), f"{(~near).sum()} non-tie selection differences of {len(rays)}"
    assert len(bad) < 1e-3 * len(rays)
    o64.close()
    orc.close()


def test_fp64_image_close_to_fp32_oracle():
    arrays = scenes.config0(x_res=40, y_res=30)
    orc = O.OrcScene(arrays)
    o64 = O.Orc64(orc)
    W, H = 40, 30
    img32 = orc.render(spp=4, max_depth=4, seed=5)["beauty"][:, :3].astype(np.float64)
    rgb, cnt = o64.render_pixels(np.arange(W * H), spp=4, max_depth=4, seed=5)
    assert (cnt > 0).all()
    # Same random numbers: almost every pixel agrees to the precision
    # difference; a few paths take another branch where FP32 and FP64 round
    # a discrete decision (lobe choice, visibility, a grazing hit) apart.
    close = np.abs(rgb - img32).max(1) <= 1e-3 * np.maximum(np.abs(img32).max(1), 0.01)
    assert close.mean() > 0.97, close.mean()
    o64.close()
    orc.close()
