"""ORACLE - test infrastructure only.  Writes a scene (eleven.scenes
SceneArrays) as the flat file oracle/ref_cuda_main.cpp reads to build the
reference's own Scene for its CUDA renderer: camera, per-triangle corners,
objects and their materials, textures, environment and point lights, all
little-endian, in er_scene_desc's units."""
import struct

import numpy as np

from eleven import _abi as A


def write(arrays, path):
    desc, keep = arrays.desc()
    c = desc.camera
    T = int(desc.tri_count)

    def f32(p, n):
        if not p or n == 0:
            return np.zeros(n, np.float32)
        return np.ctypeslib.as_array(p, (n,)).astype(np.float32)

    with open(path, "wb") as f:
        f.write(b"ERSC")
        f.write(struct.pack("<ii5f6fi", c.x_res, c.y_res, c.focal_length, c.sensor_width, c.sensor_height,
                            c.aperture, c.focus_distance, *c.position, *c.rotation, c.bokeh))
        f.write(struct.pack("<q", T))
        f.write(f32(desc.positions, 9 * T).tobytes())
        f.write(f32(desc.normals, 9 * T).tobytes())
        f.write(f32(desc.uvs, 6 * T).tobytes())
        f.write(f32(desc.tangents, 9 * T).tobytes())
        sign = f32(desc.tangent_sign, T) if desc.tangent_sign else np.ones(T, np.float32)
        f.write(sign.tobytes())
        tobj = np.ctypeslib.as_array(desc.tri_object, (T,)) if desc.tri_object else np.zeros(T, np.int32)
        f.write(np.ascontiguousarray(tobj, np.int32).tobytes())
        n_obj = max(int(desc.object_count), 1)
        omat = (np.ctypeslib.as_array(desc.object_material, (n_obj,)) if desc.object_count
                else np.zeros(1, np.int32))
        f.write(struct.pack("<i", n_obj) + np.ascontiguousarray(omat, np.int32).tobytes())
        f.write(struct.pack("<i", desc.material_count))
        for i in range(desc.material_count):
            f.write(bytes(desc.materials[i]))
        f.write(struct.pack("<i", desc.texture_count))

        def tex(t):
            f.write(struct.pack("<ii", t.width, t.height))
            f.write(f32(t.data, 3 * t.width * t.height).tobytes())
            f.write(struct.pack("<4f", t.x_tile, t.y_tile, t.x_offset, t.y_offset))

        for i in range(desc.texture_count):
            tex(desc.textures[i])
        tex(desc.env)
        f.write(struct.pack("<i", desc.light_count))
        for i in range(desc.light_count):
            L = desc.lights[i]
            f.write(struct.pack("<6f", *L.position, *L.radiance))
    assert A.er_material.__name__ and keep is not None
    return path
