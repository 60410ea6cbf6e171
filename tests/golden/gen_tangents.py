"""Writes tests/golden/reference_tangents.npz: the reference's own tangent
generation (MikkTSpace via CalcTangents, ObjLoader.hpp:167-168), run through
oracle/_ref/libref.so (`make -C oracle ref`, built from the reference tree),
on two seeded meshes with UV seams and poles.  Run from the repository root
where the reference sources exist:  python tests/golden/gen_tangents.py
"""
import ctypes as C
import os
import sys

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, os.path.join(ROOT, "tfg-pathtracer_gb300"))
from eleven import scenes  # noqa: E402


def meshes():
    out = {}
    for name, (v, f) in [("uvsphere", scenes.uv_sphere(12, 24)), ("icosphere", scenes.icosphere(2))]:
        n = scenes.vertex_normals(v, f)
        uv = scenes.sphere_uv(v)
        out[name] = (np.ascontiguousarray(v[f], np.float32), np.ascontiguousarray(n[f], np.float32),
                     np.ascontiguousarray(uv[f], np.float32))
    return out


def main():
    lib = C.CDLL(os.path.join(ROOT, "oracle", "_ref", "libref.so"))
    lib.ref_p_tangents.argtypes = [C.c_int64] + [C.c_void_p] * 5
    data = {}
    for name, (P, N, U) in meshes().items():
        t = np.zeros((len(P), 3, 3), np.float32)
        s = np.zeros(len(P), np.float32)
        lib.ref_p_tangents(len(P), P.ctypes.data, N.ctypes.data, U.ctypes.data, t.ctypes.data, s.ctypes.data)
        data.update({f"{name}_P": P, f"{name}_N": N, f"{name}_U": U, f"{name}_T": t, f"{name}_S": s})
    np.savez_compressed(os.path.join(ROOT, "tests", "golden", "reference_tangents.npz"), **data)


if __name__ == "__main__":
    main()
