"""The scene-folder loader and the post-process oracle against the
reference's own code (golden outputs in tests/golden/reference_io.npz,
written by tests/golden/gen_golden_io.py from the reference's loadScene,
stb_image decode and PostProcessing.cpp compiled for the host).

Loader (er_scene_folder_read, no device needed): positions, normals, uvs,
object ids, per-object materials, every material field, decoded texels
(fastPow sRGB / linear mapping, vertical flip, 8/24/32-bit BMP), the RGBE
environment (flat and run-length coded, not flipped), its offsets (the
yOffset -> xOffset slip), camera and point lights equal the reference's
bit for bit.  Tangents come from this library's own generator, not
MikkTSpace: signs equal and corners within cos 0.9999 as in test_tangents.

Defined where the reference has no value: a folder without scene.mtl gets
one default material here (the reference has none and would index past
its empty material array when rendering).
"""
import ctypes as C
import os

import numpy as np
import pytest

import _oracle as O
import _ref_folders as RF
from eleven import _abi as A
from eleven import _lib

GOLD = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "reference_io.npz")


@pytest.fixture(scope="module")
def G():
    return dict(np.load(GOLD))


def _struct(raw, cls, n):
    size = C.sizeof(cls)
    return [cls.from_buffer_copy(raw[i * size:(i + 1) * size].tobytes()) for i in range(n)]


def _fields(s):
    out = {}
    for name, _ in s._fields_:
        v = getattr(s, name)
        out[name] = list(v) if hasattr(v, "__len__") else v
    return out


def _bits(a):
    return np.ascontiguousarray(a, np.float32).view(np.uint32)


@pytest.mark.parametrize("name", RF.FOLDERS)
def test_folder_matches_reference_loader(G, name, tmp_path):
    k = lambda s: f"{name}__{s}"  # noqa: E731
    d = RF.write(name, str(tmp_path / name))
    assert RF.digest(d) == bytes(G[k("digest")]).hex(), "folder writer changed: re-run gen_golden_io.py"
    got = _lib.read_folder(d)
    T, n_obj, n_mat, n_tex, n_light, ew, eh = (int(x) for x in G[k("counts")])

    # geometry (ObjLoader.hpp:71-171): z flipped, normals normalised, uv.xy
    assert got["positions"].shape[0] == T
    assert np.array_equal(_bits(got["positions"]), _bits(G[k("positions")]))
    assert np.array_equal(_bits(got["normals"]), _bits(G[k("normals")]))
    assert np.array_equal(_bits(got["uvs"]), _bits(G[k("uvs")][:, :, :2]))
    assert np.array_equal(got["tri_object"], G[k("tri_object")])
    assert np.array_equal(got["object_material"], G[k("object_material")])
    assert np.array_equal(np.bincount(got["tri_object"], minlength=n_obj), G[k("object_tri_count")])

    # tangents: own generator (welded corners, angle-weighted) vs MikkTSpace
    sgn_ok = (got["tangent_sign"] == G[k("tangent_sign")]).mean()
    t, rt = got["tangents"].reshape(-1, 3).astype(np.float64), G[k("tangents")].reshape(-1, 3).astype(np.float64)
    nt, nr = np.linalg.norm(t, axis=1), np.linalg.norm(rt, axis=1)
    both = (nt > 0) & (nr > 0)
    cos = (t[both] * rt[both]).sum(1) / (nt[both] * nr[both])
    if both.sum() >= 100:  # meshes with a texture parametrisation
        assert sgn_ok > 0.95
        assert (cos > 0.9999).mean() > 0.9

    # materials (ObjLoader.hpp:33-69, SceneLoader.hpp:71-107, Material.hpp:21-36)
    ref_mats = _struct(G[k("materials")], A.er_material, n_mat)
    if n_mat == 0:
        assert len(got["materials"]) == 1  # the default material added here
        m = _fields(got["materials"][0])
        assert m["albedo"] == [0.5, 0.5, 0.5] and m["roughness"] == 1 and m["specular"] == 0.5
    else:
        assert len(got["materials"]) == n_mat
        for i, (a, b) in enumerate(zip(got["materials"], ref_mats)):
            fa, fb = _fields(a), _fields(b)
            for f in fa:
                assert np.array_equal(np.float32(fa[f]).view(np.uint32) if isinstance(fa[f], float) else fa[f],
                                      np.float32(fb[f]).view(np.uint32) if isinstance(fb[f], float) else fb[f]) \
                    or fa[f] == fb[f], (i, f, fa[f], fb[f])

    # textures: stb decode through fastPow, flipped rows (Texture.hpp:41-68)
    assert len(got["textures"]) == n_tex
    for i in range(n_tex):
        assert np.array_equal(_bits(got["textures"][i]), _bits(G[k(f"tex{i}")])), f"texture {i}"

    # environment (HDRI.hpp:22-60) and its offsets (SceneLoader.hpp:61-65)
    assert got["env"].shape == (eh, ew, 3)
    if k("env_constant") in G:
        assert np.array_equal(_bits(got["env"]), np.broadcast_to(_bits(G[k("env_constant")]), (eh, ew, 3)))
    else:
        assert np.array_equal(_bits(got["env"]), _bits(G[k("env")]))
    to = G[k("env_tile_offset")]
    assert np.array_equal(np.float32(got["env_tile"] + got["env_offset"]), to)

    # camera (SceneLoader.hpp:25-46) and lights (:125-141)
    cam = _fields(A.er_camera.from_buffer_copy(bytes(G[k("camera")])))
    mine = _fields(got["camera"])
    for f in cam:
        assert np.array_equal(np.float32(mine[f]), np.float32(cam[f])), (f, mine[f], cam[f])
    ref_lights = _struct(G[k("lights")], A.er_point_light, n_light)
    assert len(got["lights"]) == n_light
    for a, b in zip(got["lights"], ref_lights):
        assert np.array_equal(np.float32(list(a.position) + list(a.radiance)),
                              np.float32(list(b.position) + list(b.radiance)))


def _post_cases(G):
    w, h = (int(x) for x in G["post_wh"])
    k = 0
    while f"post{k}_in" in G:
        c = G[f"post{k}_opts"]
        o = A.er_post_opts(float(c[0]), int(c[1]), int(c[2]), int(c[3]), int(c[4]), int(c[5]), float(c[6]),
                           float(c[7]), float(c[8]))
        yield k, w, h, o, G[f"post{k}_in"], G[f"post{k}_out"], G[f"post{k}_mask"]
        k += 1


def test_post_oracle_matches_reference(G):
    """orc_postprocess against PostProcessing.cpp on the pixels and channels
    the reference defines: equal, with the sRGB power within 1 ulp
    (both call pow in double; the libm may differ in the last place)."""
    n = 0
    for k, w, h, o, px, ref, mask in _post_cases(G):
        got = O.postprocess(px, w, h, o)
        a, b = _bits(got)[mask].astype(np.int64), _bits(ref)[mask].astype(np.int64)
        tol = 1 if o.srgb else 0
        assert np.abs(a - b).max() <= tol, (k, np.abs(a - b).max())
        n += int(mask.sum())
    assert n > 10_000
