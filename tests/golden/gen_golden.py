"""Generate the golden vectors in tests/golden/reference_vectors.npz.

Every expected output here comes from the REFERENCE's own code: its
__host__ __device__ headers (Tri.hpp, BVH.hpp, Disney.hpp, Sampling.hpp,
HDRI.hpp, Texture.hpp) compiled for the host through oracle/ref_shim*.cpp
into oracle/_ref/libref.so (`make -C oracle ref`).  The reference ships no
tests or known-answer vectors of its own; these pin the oracle (and, through
it, the GPU path) to the reference's arithmetic.

Inputs are seeded random cases plus hand-picked edge cases (rays through
vertices and edges, grazing and parallel rays, zero and +-y normals,
u = 1 draws).  The golden scene's arrays are stored too, so the vectors do
not depend on the scene generator.

Run from the repository root:  python tests/golden/gen_golden.py
"""
import hashlib
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, os.path.join(ROOT, "tfg-pathtracer_gb300"))
sys.path.insert(0, os.path.join(ROOT, "tests"))

import _oracle as O  # noqa: E402
from eleven import build, scenes  # noqa: E402

OUT = os.path.join(HERE, "reference_vectors.npz")


def tri_cases(rng, n):
    tris = np.zeros((n, 37), np.float32)
    tris[:, :9] = rng.uniform(-1, 1, (n, 9))
    tris[:, 9:18] = rng.uniform(0, 1, (n, 9))
    nn = rng.normal(size=(n, 3, 3))
    nn /= np.linalg.norm(nn, axis=2, keepdims=True)
    tris[:, 18:27] = nn.reshape(n, 9)
    tris[:, 27:36] = rng.normal(size=(n, 9))
    tris[:, 36] = rng.choice([-1.0, 1.0], n)
    rays = np.zeros((n, 6), np.float32)
    rays[:, :3] = rng.uniform(-2, 2, (n, 3))
    # aim at a random barycentric point, some exactly at vertices / edges
    w = rng.dirichlet([1, 1, 1], n)
    k = n // 8
    w[:k] = np.eye(3)[rng.integers(0, 3, k)]                       # vertices
    w[k:2 * k, rng.integers(0, 3)] = 0                              # edges
    w[k:2 * k] /= w[k:2 * k].sum(1, keepdims=True)
    v = tris[:, :9].reshape(n, 3, 3)
    target = (w[:, :, None] * v).sum(1)
    rays[:, 3:] = target - rays[:, :3]
    m = 2 * k
    rays[m:m + k, 3:] = (v[m:m + k, 1] - v[m:m + k, 0])               # parallel to an edge
    rays[m:m + k, :3] = v[m:m + k, 0] + 0.5 * rays[m:m + k, 3:] * 0   # origin on the triangle plane
    return tris, rays


def disney_cases(rng, n):
    hd = rng.uniform(0, 1, (n, 27)).astype(np.float32)
    nrm = rng.normal(size=(n, 3))
    nrm /= np.linalg.norm(nrm, axis=1, keepdims=True)
    k = n // 10
    nrm[:k] = [0, 1, 0]          # degenerate basis (Disney.hpp:41-45)
    nrm[k:2 * k] = [0, -1, 0]
    hd[:, 18:21] = nrm
    hd[:, 6] = rng.uniform(0, 1.2, n)  # transmission, >= 1 disables eval
    dirs = rng.normal(size=(n, 3))
    dirs /= np.linalg.norm(dirs, axis=1, keepdims=True)
    Ls = rng.normal(size=(n, 3))
    Ls /= np.linalg.norm(Ls, axis=1, keepdims=True)
    Ls[::2] *= np.sign(np.sum(Ls[::2] * nrm[::2], 1, keepdims=True))
    dirs[::2] *= -np.sign(np.sum(dirs[::2] * nrm[::2], 1, keepdims=True))
    rnd = rng.uniform(0, 1, (n, 3)).astype(np.float32)
    rnd[:5] = 1.0
    return hd, dirs.astype(np.float32), Ls.astype(np.float32), rnd


def bvh_digest(boxes, meta, ti):
    """sha256 over the node boxes, node metadata and leaf order."""
    h = hashlib.sha256()
    for a in (boxes, meta, ti):
        h.update(np.ascontiguousarray(a).tobytes())
    return h.digest()


def main():
    build.build_oracle()
    if build.build_ref() is None or O.ref() is None:
        raise SystemExit("the reference sources are needed to generate golden vectors")
    r = O.Probes(O.ref(), "ref_p_")
    rng = np.random.default_rng(20261203)
    G = {}
    tris, rays = tri_cases(rng, 1500)
    G["tri_in"], G["tri_rays"], G["tri_out"] = tris, rays, r.tri_hit(tris, rays)
    hd, dirs, Ls, rnd = disney_cases(rng, 1500)
    G["dis_hd"], G["dis_dir"], G["dis_L"], G["dis_rnd"] = hd, dirs, Ls, rnd
    G["dis_out"] = r.disney(hd, dirs, Ls, rnd)
    u = rng.uniform(0, 1, (1000, 3)).astype(np.float32)
    u[:3] = 1.0
    G["samp_u"], G["samp_out"] = u, r.sampling(u)
    pts = rng.normal(size=(2000, 3))
    pts /= np.linalg.norm(pts, axis=1, keepdims=True)
    pts[:6] = [[0, 1, 0], [0, -1, 0], [1, 0, 0], [-1, 0, 0], [0, 0, 1], [0, 0, -1]]
    G["sph_in"], G["sph_out"] = pts.astype(np.float32), r.spherical(pts)
    uv = rng.uniform(0, 1, (2000, 2)).astype(np.float32)
    uv[:4] = [[0, 0], [1, 1], [0.5, 0], [0, 0.5]]
    G["rsph_in"], G["rsph_out"] = uv, r.reverse_spherical(uv)
    env = scenes.lognormal_env(64, 32, seed=5)
    env[3:5, 10:12] = 0.0
    G["env"] = env
    for off, tag in [((0.0, 0.0), "a"), ((0.25, 0.0), "b")]:
        cdf, rs = r.hdri_cdf(env, off)
        rv = rng.uniform(0, 1, 2000).astype(np.float32)
        rv[:4] = [1.0, 2.0 ** -24, cdf[100], cdf[1000]]
        G[f"cdf_{tag}"], G[f"rsum_{tag}"] = cdf, np.float32(rs)
        G[f"hdri_r_{tag}"], G[f"hdri_out_{tag}"] = rv, r.hdri_sample(env, cdf, rs, rv, off)
    img = rng.uniform(0, 1, (48, 64, 3)).astype(np.float32)
    tuv = rng.uniform(0, 1, (2000, 2)).astype(np.float32)
    G["tex_img"], G["tex_uv"] = img, tuv
    G["tex_out"] = r.tex_uv(img, tuv, (0.25, 0.5), (2.0, 3.0))
    # golden scene: reference BVH build and traversal
    sc = scenes.config0(x_res=32, y_res=24, n_spheres=6, subdiv=2, seed=4)
    G["scene_pos"], G["scene_nrm"], G["scene_uv"] = sc.positions, sc.normals, sc.uvs
    ref = O.RefScene(sc)
    boxes, meta, ti = ref.bvh()
    # the fixed-depth tree has 2^19-1 nodes: keep a digest and the first 2048
    G["bvh_sha256"] = np.frombuffer(bvh_digest(boxes, meta, ti), np.uint8)
    G["bvh_boxes_head"], G["bvh_meta_head"], G["bvh_tri_indices"] = boxes[:2048], meta[:2048], ti
    rr = scenes.random_rays(sc, 8192, seed=9)
    tri, dist = ref.trace(rr)
    G["trace_rays"], G["trace_tri"], G["trace_dist"] = rr, tri, dist
    ref.close()
    np.savez_compressed(OUT, **G)
    h = hashlib.sha256(open(OUT, "rb").read()).hexdigest()
    print(OUT, os.path.getsize(OUT), "bytes, sha256", h)


if __name__ == "__main__":
    main()
