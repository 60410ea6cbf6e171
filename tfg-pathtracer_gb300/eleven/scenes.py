"""Seeded synthetic scenes with the shapes of the benchmark configurations.

No reference scene ships with the reference (its scenes/ folder is not in
the repository), so these generators stand in for them.  Every scene is a
`SceneArrays`: flat triangle arrays in the layout of er_scene_desc plus
camera, materials, textures, point lights and the environment map.  Texel
values are produced the way the reference's loaders would decode them from
files (8-bit BMP through the fastPow sRGB decode, Texture.hpp:41-68 and
stb_image.h:1855-1866; Radiance RGBE for the environment), so that writing a
scene folder and loading it back gives the same numbers.
"""
from __future__ import annotations

import ctypes as C
import math
from dataclasses import dataclass, field

import numpy as np

from . import _abi as A

SENSOR_WIDTH = np.float32(35 * 0.001)  # Camera.hpp:14


# --------------------------------------------------------------- decoders

def fastpow(a, b):
    """Ankerl's approximate pow on the high 32 bits of a double
    (stb_image.h:127-135), vectorised.  a: float64 array, b: float."""
    a = np.ascontiguousarray(np.asarray(a, dtype=np.float64))
    bits = a.view(np.int64)
    hi = (bits >> 32).astype(np.int64)
    nh = np.trunc(b * (hi - 1072632447).astype(np.float64) + 1072632447).astype(np.int64)
    nh = nh.astype(np.int32).astype(np.int64)
    out = (nh << 32).view(np.float64)
    return out


def decode_ldr(bytes_u8, gamma):
    """stbi_loadf of an 8-bit image with stbi_ldr_to_hdr_gamma(gamma):
    float((double)fastPow(b/255.0f, gamma) * 1.0f)."""
    x = (bytes_u8.astype(np.float32) / np.float32(255.0)).astype(np.float64)
    return fastpow(x, float(np.float32(gamma))).astype(np.float32)


def rgbe_encode(rgb):
    """Radiance RGBE encoding (Ward, Graphics Gems II), as written to .hdr."""
    rgb = np.asarray(rgb, dtype=np.float32)
    m = rgb.max(axis=-1).astype(np.float64)
    out = np.zeros(rgb.shape[:-1] + (4,), dtype=np.uint8)
    nz = m >= 1e-32
    mant, ex = np.frexp(m[nz])
    scale = mant * 256.0 / m[nz]
    for c in range(3):
        out[..., c][nz] = np.clip(np.floor(rgb[..., c][nz] * scale), 0, 255).astype(np.uint8)
    out[..., 3][nz] = (ex + 128).astype(np.uint8)
    return out


def rgbe_decode(rgbe):
    """stb_image's RGBE decode: f = ldexp(1, e-136); c = byte*f (e=0 -> 0)."""
    rgbe = np.asarray(rgbe, dtype=np.uint8)
    e = rgbe[..., 3].astype(np.int32)
    f = np.ldexp(np.float32(1.0), e - (128 + 8)).astype(np.float32)
    out = rgbe[..., :3].astype(np.float32) * f[..., None]
    out[e == 0] = 0
    return out.astype(np.float32)


# ------------------------------------------------------------------ scene

@dataclass
class SceneArrays:
    camera: dict
    positions: np.ndarray          # (T, 3, 3) float32
    normals: np.ndarray            # (T, 3, 3) float32
    uvs: np.ndarray                # (T, 3, 2) float32
    tri_object: np.ndarray         # (T,) int32
    object_material: np.ndarray    # (O,) int32
    materials: list                # list of dicts (er_material fields)
    textures: list = field(default_factory=list)   # list of (H, W, 3) float32
    lights: np.ndarray = None      # (L, 2, 3) float32: position, radiance
    env: np.ndarray = None         # (H, W, 3) float32
    env_offset: tuple = (0.0, 0.0)
    tangents: np.ndarray = None
    tangent_sign: np.ndarray = None
    tie_key: np.ndarray = None
    texture_bytes: list = None     # 8-bit sources of `textures`, rows bottom-first
    name: str = "scene"

    @property
    def tri_count(self):
        return int(self.positions.shape[0])

    def desc(self):
        """Build an er_scene_desc; returns (desc, keepalive)."""
        keep = []

        def fptr(a):
            if a is None:
                return None
            a = np.ascontiguousarray(a, dtype=np.float32)
            keep.append(a)
            return a.ctypes.data_as(A.FP)

        def iptr(a, t=np.int32, p=A.IP):
            if a is None:
                return None
            a = np.ascontiguousarray(a, dtype=t)
            keep.append(a)
            return a.ctypes.data_as(p)

        d = A.er_scene_desc()
        cam = self.camera
        d.camera.x_res = int(cam["x_res"])
        d.camera.y_res = int(cam["y_res"])
        d.camera.focal_length = float(cam["focal_length"])
        d.camera.sensor_width = float(cam.get("sensor_width", SENSOR_WIDTH))
        sh = cam.get("sensor_height")
        if sh is None:  # Camera.hpp:35-37
            sh = np.float32(d.camera.sensor_width) * (np.float32(cam["y_res"]) / np.float32(cam["x_res"]))
        d.camera.sensor_height = float(sh)
        d.camera.aperture = float(cam.get("aperture", 2.8))
        d.camera.focus_distance = float(cam.get("focus_distance", 1000000.0))
        for i in range(3):
            d.camera.position[i] = float(cam["position"][i])
            d.camera.rotation[i] = float(cam.get("rotation", (0, 0, 0))[i])
        d.camera.bokeh = int(bool(cam.get("bokeh", False)))
        d.tri_count = self.tri_count
        d.positions = fptr(self.positions)
        d.normals = fptr(self.normals)
        d.uvs = fptr(self.uvs)
        d.tangents = fptr(self.tangents)
        d.tangent_sign = fptr(self.tangent_sign)
        d.tri_object = iptr(self.tri_object)
        d.object_count = int(len(self.object_material))
        d.object_material = iptr(self.object_material)
        mats = (A.er_material * max(1, len(self.materials)))()
        for i, m in enumerate(self.materials):
            fill_material(mats[i], m)
        keep.append(mats)
        d.material_count = len(self.materials)
        d.materials = C.cast(mats, C.POINTER(A.er_material))
        texs = (A.er_texture * max(1, len(self.textures)))()
        for i, t in enumerate(self.textures):
            fill_texture(texs[i], t, keep)
        keep.append(texs)
        d.texture_count = len(self.textures)
        d.textures = C.cast(texs, C.POINTER(A.er_texture))
        lights = self.lights if self.lights is not None else np.zeros((0, 2, 3), np.float32)
        la = (A.er_point_light * max(1, len(lights)))()
        for i, l in enumerate(lights):
            for k in range(3):
                la[i].position[k] = float(l[0][k])
                la[i].radiance[k] = float(l[1][k])
        keep.append(la)
        d.light_count = int(len(lights))
        d.lights = C.cast(la, C.POINTER(A.er_point_light))
        fill_texture(d.env, self.env, keep, offset=self.env_offset)
        d.tie_key = iptr(self.tie_key, np.uint32, A.UP)
        return d, keep


MATERIAL_DEFAULTS = dict(  # Material.hpp:21-36
    albedo_tex=-1, emission_tex=-1, roughness_tex=-1, metallic_tex=-1, normal_tex=-1,
    albedo=(0.5, 0.5, 0.5), emission=(0.0, 0.0, 0.0), roughness=1.0, metallic=0.0,
    clearcoat_gloss=0.0, clearcoat=0.0, anisotropic=0.0, eta=0.0, transmission=0.0,
    specular=0.5, specular_tint=0.0, sheen_tint=0.0, subsurface=0.0, sheen=0.0)


def fill_material(dst, m):
    full = dict(MATERIAL_DEFAULTS)
    full.update(m)
    for k, v in full.items():
        if k in ("albedo", "emission"):
            arr = getattr(dst, k)
            for i in range(3):
                arr[i] = float(v[i])
        else:
            setattr(dst, k, v if k.endswith("_tex") else float(v))


def fill_texture(dst, t, keep, offset=(0.0, 0.0), tile=(1.0, 1.0)):
    a = np.ascontiguousarray(t, dtype=np.float32)
    keep.append(a)
    dst.width = int(a.shape[1])
    dst.height = int(a.shape[0])
    dst.data = a.ctypes.data_as(A.FP)
    dst.x_tile, dst.y_tile = float(tile[0]), float(tile[1])
    dst.x_offset, dst.y_offset = float(offset[0]), float(offset[1])


# --------------------------------------------------------------- geometry

def icosphere(subdiv):
    """Unit icosphere: (V,3) vertices, (F,3) faces; 20*4^subdiv faces."""
    t = (1.0 + 5 ** 0.5) / 2.0
    v = [(-1, t, 0), (1, t, 0), (-1, -t, 0), (1, -t, 0), (0, -1, t), (0, 1, t), (0, -1, -t), (0, 1, -t),
         (t, 0, -1), (t, 0, 1), (-t, 0, -1), (-t, 0, 1)]
    f = [(0, 11, 5), (0, 5, 1), (0, 1, 7), (0, 7, 10), (0, 10, 11), (1, 5, 9), (5, 11, 4), (11, 10, 2),
         (10, 7, 6), (7, 1, 8), (3, 9, 4), (3, 4, 2), (3, 2, 6), (3, 6, 8), (3, 8, 9), (4, 9, 5),
         (2, 4, 11), (6, 2, 10), (8, 6, 7), (9, 8, 1)]
    verts = [np.array(p, dtype=np.float64) / np.linalg.norm(p) for p in v]
    faces = f
    for _ in range(subdiv):
        cache = {}
        nf = []

        def mid(a, b):
            key = (min(a, b), max(a, b))
            if key not in cache:
                m = verts[a] + verts[b]
                verts.append(m / np.linalg.norm(m))
                cache[key] = len(verts) - 1
            return cache[key]

        for (a, b, c) in faces:
            ab, bc, ca = mid(a, b), mid(b, c), mid(c, a)
            nf += [(a, ab, ca), (b, bc, ab), (c, ca, bc), (ab, bc, ca)]
        faces = nf
    return np.array(verts), np.array(faces, dtype=np.int64)


def uv_sphere(n_lat, n_lon):
    """Unit UV sphere with pole fans: 2*n_lon*(n_lat-1) triangles."""
    th = np.linspace(0.0, np.pi, n_lat + 1)[1:-1]
    ph = np.linspace(0.0, 2 * np.pi, n_lon + 1)[:-1]
    st, ct = np.sin(th)[:, None], np.cos(th)[:, None]
    ring = np.stack([st * np.cos(ph)[None, :], np.broadcast_to(ct, (n_lat - 1, n_lon)),
                     st * np.sin(ph)[None, :]], -1).reshape(-1, 3)
    verts = np.concatenate([[[0.0, 1.0, 0.0]], ring, [[0.0, -1.0, 0.0]]])
    last = len(verts) - 1
    j = np.arange(n_lon)
    jn = (j + 1) % n_lon
    top = np.stack([np.zeros(n_lon, np.int64), 1 + jn, 1 + j], 1)
    i = np.arange(1, n_lat - 1)[:, None]
    a = 1 + (i - 1) * n_lon + j[None, :]
    b = 1 + (i - 1) * n_lon + jn[None, :]
    c = 1 + i * n_lon + j[None, :]
    d = 1 + i * n_lon + jn[None, :]
    mid = np.stack([np.stack([a, b, d], -1), np.stack([a, d, c], -1)], 2).reshape(-1, 3)
    bot = np.stack([np.full(n_lon, last), 1 + (n_lat - 2) * n_lon + j, 1 + (n_lat - 2) * n_lon + jn], 1)
    return verts, np.concatenate([top, mid, bot]).astype(np.int64)


def value_noise3(p, seed, octaves=1):
    """Smooth 3-D value noise in [-1, 1] (lattice hash + trilinear smoothstep)."""
    p = np.asarray(p, dtype=np.float64)
    total = np.zeros(p.shape[0])
    amp, freq, norm = 1.0, 1.0, 0.0
    for o in range(octaves):
        q = p * freq
        i0 = np.floor(q).astype(np.int64)
        f = q - i0
        f = f * f * (3 - 2 * f)
        acc = np.zeros(p.shape[0])
        for dx in (0, 1):
            for dy in (0, 1):
                for dz in (0, 1):
                    h = _hash3(i0[:, 0] + dx, i0[:, 1] + dy, i0[:, 2] + dz, seed + 101 * o)
                    w = ((f[:, 0] if dx else 1 - f[:, 0]) * (f[:, 1] if dy else 1 - f[:, 1])
                         * (f[:, 2] if dz else 1 - f[:, 2]))
                    acc += w * h
        total += amp * acc
        norm += amp
        amp *= 0.5
        freq *= 2.0
    return total / norm


def _hash3(x, y, z, seed):
    h = (x * 73856093) ^ (y * 19349663) ^ (z * 83492791) ^ (seed * 2654435761)
    h = h & 0xFFFFFFFF
    h = (h ^ (h >> 13)) * 1274126177 & 0xFFFFFFFF
    h = h ^ (h >> 16)
    return (h & 0xFFFFFF) / float(0xFFFFFF) * 2.0 - 1.0


def value_noise2_img(w, h, seed, octaves=4, cells=8):
    """Octave value noise image in [0,1], (h, w): random lattice values,
    smoothstep-interpolated, halving amplitude per octave."""
    rng = np.random.default_rng(seed)
    ys = (np.arange(h) + 0.5) / h
    xs = (np.arange(w) + 0.5) / w
    total = np.zeros((h, w))
    amp, norm = 1.0, 0.0
    for o in range(octaves):
        n = cells * (2 ** o)
        lat = rng.uniform(-1, 1, (n + 1, n + 1))
        fy, fx = ys * n, xs * n
        iy, ix = np.floor(fy).astype(np.int64), np.floor(fx).astype(np.int64)
        ty, tx = fy - iy, fx - ix
        ty, tx = ty * ty * (3 - 2 * ty), tx * tx * (3 - 2 * tx)
        a = lat[iy][:, ix]
        b = lat[iy][:, ix + 1]
        c = lat[iy + 1][:, ix]
        d = lat[iy + 1][:, ix + 1]
        top = a + (b - a) * tx[None, :]
        bot = c + (d - c) * tx[None, :]
        total += amp * (top + (bot - top) * ty[:, None])
        norm += amp
        amp *= 0.5
    return 0.5 + 0.5 * total / norm


def vertex_normals(verts, faces):
    fn = np.cross(verts[faces[:, 1]] - verts[faces[:, 0]], verts[faces[:, 2]] - verts[faces[:, 0]])
    vn = np.zeros_like(verts)
    for k in range(3):
        np.add.at(vn, faces[:, k], fn)
    ln = np.linalg.norm(vn, axis=1, keepdims=True)
    ln[ln == 0] = 1
    return vn / ln


def sphere_uv(verts):
    u = 0.5 + np.arctan2(verts[:, 2], verts[:, 0]) / (2 * np.pi)
    v = 0.5 - np.arcsin(np.clip(verts[:, 1], -1, 1)) / np.pi
    return np.stack([u, v], -1)


def ref_normalize(n):
    """Vector3::normalized in float32 (Vector.hpp:173-176), iterated to a
    fixed point so that a loader that normalises normals again
    (ObjLoader.hpp:118) reproduces them bit for bit."""
    def once(v):
        x, y, z = v[:, 0], v[:, 1], v[:, 2]
        ln = np.sqrt(x * x + y * y + z * z)
        nz = ln != 0
        m = v.copy()
        m[nz] = v[nz] / ln[nz, None]
        return m

    def fixed(v):
        return (once(v).view(np.uint32) == v.view(np.uint32)).all(1)

    n = once(np.asarray(n, np.float32).reshape(-1, 3).copy())
    bad = np.nonzero(~fixed(n))[0]
    if len(bad):
        # some vectors alternate between two roundings: search the 1-ulp
        # neighbourhood for a fixed point
        steps = np.array([(a, b, c) for a in (0, -1, 1) for b in (0, -1, 1) for c in (0, -1, 1)], np.int64)
        v = n[bad]
        bits = v.view(np.int32).astype(np.int64)
        for s in steps[1:]:
            cand = (bits + s[None, :]).astype(np.int32).view(np.float32)
            ok = fixed(cand)
            v[ok] = cand[ok]
            bits[ok] = v[ok].view(np.int32)
            still = ~fixed(v)
            if not still.any():
                break
        n[bad] = v
    return n


def _assemble(meshes):
    """meshes: list of (verts(V,3), faces(F,3), normals(V,3), uv(V,2))."""
    P, N, U, O = [], [], [], []
    for oi, (v, f, n, uv) in enumerate(meshes):
        P.append(v[f])
        N.append(n[f])
        U.append(uv[f])
        O.append(np.full(len(f), oi, np.int32))
    N = ref_normalize(np.concatenate(N)).reshape(-1, 3, 3)
    return (np.concatenate(P).astype(np.float32), N, np.concatenate(U).astype(np.float32), np.concatenate(O))


def ground_quad(y, half):
    v = np.array([[-half, y, -half], [half, y, -half], [half, y, half], [-half, y, half]], np.float64)
    f = np.array([[0, 2, 1], [0, 3, 2]], np.int64)
    n = np.tile(np.array([[0.0, 1.0, 0.0]]), (4, 1))
    uv = np.array([[0, 0], [1, 0], [1, 1], [0, 1]], np.float64)
    return v, f, n, uv


def pinhole_focal(fov_deg):
    """Focal length giving a horizontal field of view with the fixed 35 mm
    sensor width of Camera.hpp:14."""
    return float(np.float32(0.5 * float(SENSOR_WIDTH) / math.tan(math.radians(fov_deg) / 2)))


def constant_env(rgb, size=1024):
    """HDRI(Vector3) fills a 1024x1024 texture (HDRI.hpp:22-38)."""
    e = np.empty((size, size, 3), np.float32)
    e[...] = np.asarray(rgb, np.float32)
    return e


# ---------------------------------------------------------------- configs

def config0(x_res=320, y_res=240, seed=0, n_spheres=16, subdiv=3):
    """Plain method, small scene: 16 icospheres (1280 tris each) + ground
    quad, one point light at (0,8,0), constant environment 0.5."""
    rng = np.random.default_rng(seed)
    base_v, base_f = icosphere(subdiv)
    meshes, mats = [], []
    for i in range(n_spheres):
        c = rng.uniform(-5, 5, 3)
        r = rng.uniform(0.3, 1.0)
        v = base_v * r + c
        meshes.append((v, base_f, base_v.copy(), sphere_uv(base_v)))
        mats.append(dict(albedo=tuple(rng.uniform(0, 1, 3)), roughness=rng.uniform(0.05, 1.0),
                         metallic=float(rng.uniform() < 0.3), specular=0.5, clearcoat=0.0))
    meshes.append(ground_quad(-6.0, 40.0))
    mats.append(dict(albedo=(0.8, 0.8, 0.8), roughness=1.0, metallic=0.0, specular=0.5))
    P, N, U, O = _assemble(meshes)
    cam = dict(x_res=x_res, y_res=y_res, focal_length=pinhole_focal(45.0), position=(0.0, 1.0, -16.0),
               rotation=(0.0, 0.0, 0.0), bokeh=False)
    lights = np.array([[[0, 8, 0], [100, 100, 100]]], np.float32)
    return SceneArrays(camera=cam, positions=P, normals=N, uvs=U, tri_object=O,
                       object_material=np.arange(len(meshes), dtype=np.int32), materials=mats,
                       lights=lights, env=constant_env((0.5, 0.5, 0.5)), name="c0")


def lognormal_env(w, h, seed, mu=0.0, sigma=2.0, sun=32, sun_value=1e4):
    rng = np.random.default_rng(seed + 7)
    lum = np.exp(rng.normal(mu, sigma, (h, w))).astype(np.float32)
    env = np.repeat(lum[..., None], 3, axis=2)
    if sun:
        y0, x0 = h // 4, w // 3
        env[y0:y0 + sun, x0:x0 + sun, :] = np.float32(sun_value)
    return rgbe_decode(rgbe_encode(env))


def noise_textures(n, size, seed):
    texs, raw = [], []
    for i in range(n):
        img = np.stack([value_noise2_img(size, size, seed * 1000 + 3 * i + c) for c in range(3)], -1)
        b = np.clip(np.round(img * 255), 0, 255).astype(np.uint8)
        raw.append(b)
        texs.append(decode_ldr(b, 2.2))
    return texs, raw


def config1(x_res=1920, y_res=1080, seed=1, n_meshes=200, tri_lo=1000, tri_hi=20000, tex_size=512,
            n_tex=10, env_w=2048, env_h=1024, aperture_radius=0.05, focus=10.0):
    """Plain method, full features: ~1M triangles from 200 displaced
    spheres, ten 512^2 value-noise baseColor textures, 2048x1024 log-normal
    environment with a sun patch, 4 point lights, thin lens."""
    rng = np.random.default_rng(seed)
    meshes, mats = [], []
    for i in range(n_meshes):
        target = math.exp(rng.uniform(math.log(tri_lo), math.log(tri_hi)))
        n_lat = max(3, int(round(math.sqrt(target / 4.0))))
        n_lon = 2 * n_lat
        v, f = uv_sphere(n_lat, n_lon)
        disp = 1.0 + 0.2 * value_noise3(v * 2.0, seed * 7919 + i, octaves=3)
        r = rng.uniform(0.4, 1.2)
        c = np.array([rng.uniform(-9, 9), rng.uniform(-4, 4), rng.uniform(-6, 10)])
        vd = v * disp[:, None] * r + c
        n = vertex_normals(vd, f)
        meshes.append((vd, f, n, sphere_uv(v)))
        mats.append(dict(albedo=tuple(rng.uniform(0, 1, 3)), albedo_tex=int(i % n_tex),
                         roughness=rng.uniform(0.05, 1.0), metallic=float(rng.uniform() < 0.3),
                         specular=0.5, clearcoat=rng.uniform(0, 1), sheen=rng.uniform(0, 1)))
    P, N, U, O = _assemble(meshes)
    texs, tex_bytes = noise_textures(n_tex, tex_size, seed)
    focal = pinhole_focal(50.0)
    cam = dict(x_res=x_res, y_res=y_res, focal_length=focal, position=(0.0, 0.5, -16.0),
               rotation=(0.0, 0.0, 0.0), bokeh=True,
               aperture=float(np.float32(focal / (2 * aperture_radius))), focus_distance=focus)
    lights = np.array([[[-6, 8, -4], [60, 60, 60]], [[6, 8, -4], [60, 50, 40]],
                       [[0, 10, 6], [80, 80, 80]], [[0, -2, -10], [30, 30, 40]]], np.float32)
    return SceneArrays(camera=cam, positions=P, normals=N, uvs=U, tri_object=O,
                       object_material=np.arange(len(meshes), dtype=np.int32), materials=mats,
                       textures=texs, texture_bytes=tex_bytes, lights=lights,
                       env=lognormal_env(env_w, env_h, seed), name="c1")


C2_RESOLUTIONS = [(128, 128), (256, 256), (320, 240), (512, 512), (640, 480), (800, 600), (1024, 768)]


def displaced_spheres(n_tris, seed, x_res, y_res, n_lights, env_w=512, env_h=256, mesh_tris=8000):
    """A scene of seeded value-noise-displaced UV spheres with about n_tris
    triangles in total (meshes of about mesh_tris), Disney parameters as in
    the 1M-triangle scene (no textures), n_lights point lights and a
    log-normal environment of env_w x env_h."""
    rng = np.random.default_rng(seed)
    n_meshes = int(min(64, max(2, round(n_tris / mesh_tris))))
    per = n_tris / n_meshes
    meshes, mats = [], []
    for i in range(n_meshes):
        n_lat = max(3, int(round(math.sqrt(per / 4.0))))
        v, f = uv_sphere(n_lat, 2 * n_lat)
        disp = 1.0 + 0.2 * value_noise3(v * 2.0, seed * 7919 + i, octaves=3)
        r = rng.uniform(0.4, 1.2)
        c = np.array([rng.uniform(-7, 7), rng.uniform(-3, 3), rng.uniform(-4, 8)])
        vd = v * disp[:, None] * r + c
        meshes.append((vd, f, vertex_normals(vd, f), sphere_uv(v)))
        mats.append(dict(albedo=tuple(rng.uniform(0, 1, 3)), roughness=rng.uniform(0.05, 1.0),
                         metallic=float(rng.uniform() < 0.3), specular=0.5, clearcoat=rng.uniform(0, 1),
                         sheen=rng.uniform(0, 1)))
    P, N, U, O = _assemble(meshes)
    cam = dict(x_res=x_res, y_res=y_res, focal_length=pinhole_focal(50.0), position=(0.0, 0.5, -16.0),
               rotation=(0.0, 0.0, 0.0), bokeh=False)
    pos = rng.uniform([-8, 4, -8], [8, 10, 8], (n_lights, 3))
    rad = rng.uniform(30, 90, (n_lights, 3))
    lights = np.stack([pos, rad], 1).astype(np.float32)
    return SceneArrays(camera=cam, positions=P, normals=N, uvs=U, tri_object=O,
                       object_material=np.arange(len(meshes), dtype=np.int32), materials=mats,
                       lights=lights, env=lognormal_env(env_w, env_h, seed, sun=8), name=f"c2-{seed}")


def config2(n_jobs=64, seed=2, tri_lo=10_000, tri_hi=500_000, resolutions=C2_RESOLUTIONS, spps=(4, 16, 64),
            depths=(4, 8), env_w=512, env_h=256):
    """Batching: n_jobs heterogeneous scenes/views.  Per job: resolution
    uniform over `resolutions`, spp uniform over `spps`, max depth uniform in
    depths[0]..depths[1], triangle count log-uniform in [tri_lo, tri_hi]
    (displaced spheres), 1-4 point lights, a log-normal environment.
    Returns (scene arrays, job dicts) with job["scene"] = its scene index."""
    rng = np.random.default_rng(seed)
    arrays, jobs = [], []
    for j in range(n_jobs):
        W, H = resolutions[int(rng.integers(len(resolutions)))]
        spp = int(spps[int(rng.integers(len(spps)))])
        depth = int(rng.integers(depths[0], depths[1] + 1))
        tris = math.exp(rng.uniform(math.log(tri_lo), math.log(tri_hi)))
        n_lights = int(rng.integers(1, 5))
        arrays.append(displaced_spheres(tris, seed * 1000 + j, W, H, n_lights, env_w, env_h))
        jobs.append(dict(scene=j, spp=spp, max_depth=depth, seed=j))
    return arrays, jobs


def config4(x_res=512, y_res=512, n_obj=64, geom_seed=4, param_seed=40, env_w=256, env_h=128, subdiv=3):
    """Differentiation: n_obj icospheres placed as in the small scene (centres
    U[-5,5]^3, radii U[0.3,1]), one point light, and a log-normal
    env_w x env_h environment (n_obj * 5 + env_w * env_h * 3 parameters).  The differentiable parameters
    (albedo U[0,1]^3, roughness U[0.05,1], metallic Bernoulli(0.3) per
    object, env texels) are drawn from param_seed, so two param seeds give
    a scene and a target with the same geometry."""
    rng = np.random.default_rng(geom_seed)
    prng = np.random.default_rng(param_seed)
    base_v, base_f = icosphere(subdiv)
    meshes, mats = [], []
    for i in range(n_obj):
        c = rng.uniform(-5, 5, 3)
        r = rng.uniform(0.3, 1.0)
        meshes.append((base_v * r + c, base_f, base_v.copy(), sphere_uv(base_v)))
        mats.append(dict(albedo=tuple(prng.uniform(0, 1, 3)), roughness=prng.uniform(0.05, 1.0),
                         metallic=float(prng.uniform() < 0.3), specular=0.5, clearcoat=0.0))
    P, N, U, O = _assemble(meshes)
    cam = dict(x_res=x_res, y_res=y_res, focal_length=pinhole_focal(45.0), position=(0.0, 1.0, -16.0),
               rotation=(0.0, 0.0, 0.0), bokeh=False)
    lights = np.array([[[0, 8, 0], [100, 100, 100]]], np.float32)
    env = lognormal_env(env_w, env_h, param_seed, sigma=1.0, sun=0)
    return SceneArrays(camera=cam, positions=P, normals=N, uvs=U, tri_object=O,
                       object_material=np.arange(len(meshes), dtype=np.int32), materials=mats,
                       lights=lights, env=env, name="c4")


def random_rays(scene, n, seed=3):
    """Origins uniform in the scene bounds, directions uniform on the sphere
    (z = 1-2u, phi = 2 pi v)."""
    rng = np.random.default_rng(seed)
    lo = scene.positions.reshape(-1, 3).min(0)
    hi = scene.positions.reshape(-1, 3).max(0)
    o = rng.uniform(lo, hi, (n, 3))
    u, v = rng.uniform(0, 1, n), rng.uniform(0, 1, n)
    z = 1 - 2 * u
    r = np.sqrt(np.maximum(0, 1 - z * z))
    d = np.stack([r * np.cos(2 * np.pi * v), r * np.sin(2 * np.pi * v), z], -1)
    return np.concatenate([o, d], 1).astype(np.float32)
