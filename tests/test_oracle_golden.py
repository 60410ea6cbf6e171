"""The oracle against the golden vectors produced by the reference's own
headers (tests/golden/gen_golden.py).  Bit for bit; NaNs compare equal to
NaNs (their payload differs between x86 and Arm)."""
import os

import numpy as np
import pytest

import _oracle as O
from eleven import scenes

GOLD = os.path.join(os.path.dirname(__file__), "golden", "reference_vectors.npz")


@pytest.fixture(scope="module")
def G():
    return dict(np.load(GOLD))


@pytest.fixture(scope="module")
def orc():
    return O.Probes(O.orc(), "orc_p_")


def same(a, b):
    a = np.asarray(a, np.float32)
    b = np.asarray(b, np.float32)
    return (a.view(np.uint32) == b.view(np.uint32)) | (np.isnan(a) & np.isnan(b))


def test_tri_hit(G, orc):
    out = orc.tri_hit(G["tri_in"], G["tri_rays"])
    assert same(out, G["tri_out"]).all()
    assert G["tri_out"][:, 0].sum() > 100  # enough hits exercised


def test_disney_eval_pdf_sample(G, orc):
    out = orc.disney(G["dis_hd"], G["dis_dir"], G["dis_L"], G["dis_rnd"])
    assert same(out, G["dis_out"]).all()


def test_sampling(G):
    if O.ref() is None:
        out = np.zeros_like(G["samp_out"])
        u = np.ascontiguousarray(G["samp_u"])
        O.orc().orc_p_sampling(len(u), O._ptr(u), O._ptr(out))
    else:
        out = O.Probes(O.orc(), "orc_p_").sampling(G["samp_u"])
    assert same(out, G["samp_out"]).all()


def test_spherical_mappings(G, orc):
    assert same(orc.spherical(G["sph_in"]), G["sph_out"]).all()
    assert same(orc.reverse_spherical(G["rsph_in"]), G["rsph_out"]).all()


def hdri_defined(out, w, x_offset):
    """Rows whose inverse offset transform (Texture.hpp:177-193) stays in
    range.  For the others the reference indexes texels outside the array
    (its C remainder of a negative value), which the oracle defines by
    wrapping; only the texel index and direction are compared there."""
    x = (out[:, 0].astype(np.int64) % w).astype(np.float32)
    ix = np.trunc((x / np.float32(w)) * np.float32(w))
    ix2 = np.trunc(ix - np.float32(x_offset) * np.float32(w))
    return ix2 >= 0


@pytest.mark.parametrize("tag,off", [("a", (0.0, 0.0)), ("b", (0.25, 0.0))])
def test_hdri_cdf_and_sampling(G, orc, tag, off):
    cdf, rs = orc.hdri_cdf(G["env"], off)
    assert same(cdf, G[f"cdf_{tag}"]).all()
    assert np.float32(rs) == G[f"rsum_{tag}"]
    out = orc.hdri_sample(G["env"], cdf, rs, G[f"hdri_r_{tag}"], off)
    ref = G[f"hdri_out_{tag}"]
    ok = hdri_defined(ref, G["env"].shape[1], off[0])
    assert ok.sum() > len(ok) // 2
    assert same(out[ok], ref[ok]).all()
    cols = [0, 2, 3, 4]
    assert same(out[:, cols], ref[:, cols]).all()


def test_texture_fetch(G, orc):
    out = orc.tex_uv(G["tex_img"], G["tex_uv"], (0.25, 0.5), (2.0, 3.0))
    assert same(out, G["tex_out"]).all()


def golden_scene(G):
    T = len(G["scene_pos"])
    return scenes.SceneArrays(
        camera=dict(x_res=32, y_res=24, focal_length=scenes.pinhole_focal(45.0), position=(0, 1, -16)),
        positions=G["scene_pos"], normals=G["scene_nrm"], uvs=G["scene_uv"],
        tri_object=np.zeros(T, np.int32), object_material=np.zeros(1, np.int32), materials=[{}],
        env=scenes.constant_env((0.5, 0.5, 0.5), size=8), lights=None)


def test_reference_bvh_build(G):
    import hashlib
    s = O.OrcScene(golden_scene(G))
    boxes, meta, ti = s.bvh()
    h = hashlib.sha256()
    for a in (boxes, meta, ti):
        h.update(np.ascontiguousarray(a).tobytes())
    assert np.array_equal(np.frombuffer(h.digest(), np.uint8), G["bvh_sha256"])
    assert np.array_equal(meta[:2048], G["bvh_meta_head"])
    assert np.array_equal(ti, G["bvh_tri_indices"])
    s.close()


def test_reference_traversal(G):
    s = O.OrcScene(golden_scene(G))
    tri, dist = s.trace(G["trace_rays"])
    assert np.array_equal(tri, G["trace_tri"])
    assert same(dist, G["trace_dist"]).all()
    assert (tri >= 0).sum() > 1000
    s.close()
