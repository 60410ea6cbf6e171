"""ctypes mirror of include/eleven.h (the C-ABI of libeleven.so).

Field order and types must match the header exactly; tests check the
struct sizes against the library's own view of them.
"""
import ctypes as C

er_status = C.c_int32

ER_OK = 0
ER_ERR_INVALID_ARG = 1
ER_ERR_IO = 2
ER_ERR_PARSE = 3
ER_ERR_CUDA = 4
ER_ERR_OOM = 5
ER_ERR_DEVICE_CHECK = 6
ER_ERR_TIMEOUT = 7
ER_ERR_UNSUPPORTED = 8
ER_ERR_NO_DEVICE = 9
STATUS_NAMES = {
    0: "ER_OK", 1: "ER_ERR_INVALID_ARG", 2: "ER_ERR_IO", 3: "ER_ERR_PARSE",
    4: "ER_ERR_CUDA", 5: "ER_ERR_OOM", 6: "ER_ERR_DEVICE_CHECK",
    7: "ER_ERR_TIMEOUT", 8: "ER_ERR_UNSUPPORTED", 9: "ER_ERR_NO_DEVICE",
}

ER_BVH_FP32 = 0
ER_BVH_Q8 = 1

ER_RENDER_DEVICE_OUT = 1 << 0
ER_RENDER_ACCUM_FP64 = 1 << 1
ER_RENDER_AOV = 1 << 2
ER_RENDER_ENV_ALIAS = 1 << 3
ER_RENDER_CONTINUE = 1 << 4
ER_RENDER_NO_OUTPUT = 1 << 5

ER_TRACE_DEVICE_PTRS = 1 << 0
ER_TRACE_NORMALIZED = 1 << 1
ER_TRACE_STATS = 1 << 2

FP = C.POINTER(C.c_float)
IP = C.POINTER(C.c_int32)
UP = C.POINTER(C.c_uint32)


class er_camera(C.Structure):
    _fields_ = [
        ("x_res", C.c_int32), ("y_res", C.c_int32),
        ("focal_length", C.c_float), ("sensor_width", C.c_float),
        ("sensor_height", C.c_float), ("aperture", C.c_float),
        ("focus_distance", C.c_float),
        ("position", C.c_float * 3), ("rotation", C.c_float * 3),
        ("bokeh", C.c_int32),
    ]


class er_material(C.Structure):
    _fields_ = [
        ("albedo_tex", C.c_int32), ("emission_tex", C.c_int32),
        ("roughness_tex", C.c_int32), ("metallic_tex", C.c_int32),
        ("normal_tex", C.c_int32),
        ("albedo", C.c_float * 3), ("emission", C.c_float * 3),
        ("roughness", C.c_float), ("metallic", C.c_float),
        ("clearcoat_gloss", C.c_float), ("clearcoat", C.c_float),
        ("anisotropic", C.c_float), ("eta", C.c_float),
        ("transmission", C.c_float), ("specular", C.c_float),
        ("specular_tint", C.c_float), ("sheen_tint", C.c_float),
        ("subsurface", C.c_float), ("sheen", C.c_float),
    ]


class er_texture(C.Structure):
    _fields_ = [
        ("width", C.c_int32), ("height", C.c_int32), ("data", FP),
        ("x_tile", C.c_float), ("y_tile", C.c_float),
        ("x_offset", C.c_float), ("y_offset", C.c_float),
    ]


class er_point_light(C.Structure):
    _fields_ = [("position", C.c_float * 3), ("radiance", C.c_float * 3)]


class er_scene_desc(C.Structure):
    _fields_ = [
        ("camera", er_camera),
        ("tri_count", C.c_int64),
        ("positions", FP), ("normals", FP), ("uvs", FP), ("tangents", FP),
        ("tangent_sign", FP), ("tri_object", IP),
        ("object_count", C.c_int32), ("object_material", IP),
        ("material_count", C.c_int32), ("materials", C.POINTER(er_material)),
        ("texture_count", C.c_int32), ("textures", C.POINTER(er_texture)),
        ("light_count", C.c_int32), ("lights", C.POINTER(er_point_light)),
        ("env", er_texture),
        ("tie_key", UP),
    ]


ER_BUILDER_HOST = 0
ER_BUILDER_GPU = 1


class er_scene_opts(C.Structure):
    _fields_ = [
        ("bvh_format", C.c_int32), ("max_leaf_tris", C.c_int32),
        ("device", C.c_int32), ("stream", C.c_void_p), ("builder", C.c_int32),
    ]


class er_scene_info(C.Structure):
    _fields_ = [
        ("tri_count", C.c_int64), ("node_count", C.c_int64),
        ("leaf_count", C.c_int64), ("device_bytes", C.c_int64),
        ("bvh_build_ms", C.c_double), ("upload_ms", C.c_double),
        ("scene_lo", C.c_float * 3), ("scene_hi", C.c_float * 3),
        ("max_shading_offset", C.c_float),
        ("bvh_depth", C.c_int32), ("bvh_format", C.c_int32),
        ("material_count", C.c_int32), ("env_width", C.c_int32), ("env_height", C.c_int32),
        ("reserved", C.c_int32),
    ]


class er_render_opts(C.Structure):
    _fields_ = [
        ("spp", C.c_int32), ("sample_begin", C.c_int32),
        ("max_depth", C.c_int32), ("spp_per_wave", C.c_int32),
        ("seed", C.c_uint64), ("flags", C.c_uint32), ("reserved", C.c_int32),
    ]


ER_RENDER_PROFILE = 1 << 6
ER_RENDER_COUNT = 1 << 7
ER_RENDER_SNAPSHOTS = 1 << 8
ER_RENDER_ONE_STREAM = 1 << 9
ER_RENDER_KEEP_PATHS = 1 << 10
STAGES = ["raygen", "trace", "shade", "reserved", "accumulate"]


class er_render_stats(C.Structure):
    _fields_ = [
        ("ms", C.c_double), ("samples", C.c_int64),
        ("rays_closest", C.c_int64), ("rays_shadow", C.c_int64),
        ("path_vertices", C.c_int64), ("kernel_launches", C.c_int64),
        ("stage_ms", C.c_double * 5), ("stage_launches", C.c_int64 * 5),
        ("closest_nodes", C.c_int64), ("closest_tris", C.c_int64),
        ("shadow_nodes", C.c_int64), ("shadow_tris", C.c_int64),
    ]


class er_trace_stats(C.Structure):
    _fields_ = [
        ("ms", C.c_double), ("node_visits", C.c_int64),
        ("box_tests", C.c_int64), ("tri_tests", C.c_int64),
    ]


class er_batch_job(C.Structure):
    _fields_ = [
        ("scene", C.c_int32), ("spp", C.c_int32), ("max_depth", C.c_int32),
        ("sample_begin", C.c_int32), ("seed", C.c_uint64), ("flags", C.c_uint32),
        ("reserved", C.c_int32), ("camera", er_camera),
    ]


class er_batch_tuning(C.Structure):
    _fields_ = [
        ("wave_paths", C.c_int32), ("trace_blocks_per_sm", C.c_int32),
        ("shade_blocks_per_sm", C.c_int32), ("split_trace", C.c_int32),
        ("use_graph", C.c_int32), ("one_stream", C.c_int32), ("reserved", C.c_int32 * 2),
    ]


# Every symbol include/eleven.h declares (checked by the CPU tests).
EXPORTED = [
    "er_status_string", "er_last_error", "er_abi_version",
    "er_scene_create", "er_scene_load", "er_scene_info_get",
    "er_scene_set_camera", "er_scene_get_camera", "er_scene_free",
    "er_render", "er_film_read", "er_snapshot", "er_render_paths", "er_render_noalloc", "er_env_distribution",
    "er_env_search_table",
    "er_scene_get_params", "er_scene_set_params", "er_render_replay", "er_backward",
    "er_batch_create", "er_batch_set_jobs", "er_batch_render", "er_batch_read",
    "er_batch_autotune", "er_batch_info", "er_batch_free",
    "er_trace_closest", "er_encode_ldr", "er_write_image", "er_postprocess", "er_compute_tangents",
    "er_scene_folder_read", "er_folder_desc", "er_folder_free", "er_device_bandwidth", "er_film_read_sums",
]

ER_BW_L2_READ, ER_BW_HBM_COPY = 0, 1

ER_TONEMAP_NONE, ER_TONEMAP_REINHARD, ER_TONEMAP_ACES = 0, 1, 2


class er_post_opts(C.Structure):
    _fields_ = [
        ("exposure", C.c_float), ("tonemap", C.c_int32), ("clamp", C.c_int32), ("srgb", C.c_int32),
        ("flip_x", C.c_int32), ("flip_y", C.c_int32),
        ("bloom_threshold", C.c_float), ("bloom_power", C.c_float), ("bloom_radius", C.c_float),
    ]
