/*
 * eleven.h - C-ABI of the GB300-native Eleven Renderer sample path.
 *
 * One shared library (libeleven.so) exports everything below with C linkage,
 * plain pointers and sizes.  It replaces the reference's render boundary
 * (src/tfg-pathtracer/kernel.h:78-84, defined in kernel.cu:566-724):
 *
 *   reference                                   replaced by
 *   cudaError_t renderSetup(Scene*)             er_scene_create / er_scene_load
 *     (kernel.h:80, kernel.cu:566-661)            (scene upload + BVH build)
 *   cudaError_t renderCuda(Scene*, int spp)     er_render
 *     (kernel.h:78, kernel.cu:665-686)
 *   cudaError_t getBuffers(RenderData&, int*,   er_render output buffers /
 *     int) (kernel.h:82, kernel.cu:688-710)       er_film_read
 *   int getSamples() (kernel.h:84,              er_film_read (samples array)
 *     kernel.cu:712-724)
 *   BVH::transverse (BVH.hpp:120-157) via      er_trace_closest (parity gate)
 *     throwRay (kernel.cu:152-173)
 *
 * Every call returns an er_status; no C++ exception crosses the ABI and no
 * device-side trap is used: device checks set an error word that the host
 * turns into ER_ERR_DEVICE_CHECK / ER_ERR_TIMEOUT.
 *
 * Threading: calls on one handle are serialised by the caller; handles are
 * independent of each other (no process globals).  All work of a handle is
 * issued on the stream given at creation (NULL = a stream owned by the handle).
 */
#ifndef ELEVEN_H
#define ELEVEN_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define ER_ABI_VERSION 1

typedef int32_t er_status;
enum {
  ER_OK = 0,
  ER_ERR_INVALID_ARG = 1,   /* NULL pointer, negative size, NaN parameter ... */
  ER_ERR_IO = 2,            /* missing / unreadable scene file */
  ER_ERR_PARSE = 3,         /* malformed JSON / OBJ / MTL / BMP / HDR */
  ER_ERR_CUDA = 4,          /* a CUDA runtime call failed */
  ER_ERR_OOM = 5,           /* device or host allocation failed / over cap */
  ER_ERR_DEVICE_CHECK = 6,  /* a kernel's own bounds check fired */
  ER_ERR_TIMEOUT = 7,       /* a bounded device wait gave up */
  ER_ERR_UNSUPPORTED = 8,   /* feature not available on this device / build */
  ER_ERR_NO_DEVICE = 9      /* no CUDA device visible */
};

/* Static description of a status code. */
const char* er_status_string(er_status s);
/* Detail message of the last failing call on this thread ("" if none). */
const char* er_last_error(void);
/* ABI version of the loaded library (ER_ABI_VERSION). */
int32_t er_abi_version(void);

/* ---------------------------------------------------------------- scene -- */

/* Camera.hpp:6-40.  rotation is XYZ Euler in degrees (kernel.cu:297-306);
 * aperture is the reference's f-number: lens diameter = focal/aperture
 * (kernel.cu:316). */
typedef struct er_camera {
  int32_t x_res, y_res;
  float focal_length;
  float sensor_width;
  float sensor_height;
  float aperture;
  float focus_distance;
  float position[3];
  float rotation[3];
  int32_t bokeh;
} er_camera;

/* Material.hpp:8-37.  Texture ids index er_scene_desc.textures, -1 = none. */
typedef struct er_material {
  int32_t albedo_tex, emission_tex, roughness_tex, metallic_tex, normal_tex;
  float albedo[3];
  float emission[3];
  float roughness, metallic, clearcoat_gloss, clearcoat, anisotropic, eta,
      transmission, specular, specular_tint, sheen_tint, subsurface, sheen;
} er_material;

/* Texture.hpp:15-33 (data, width, height, xTile/yTile, xOffset/yOffset):
 * float RGB texels, row-major, row 0 first as stored after loading (BMP
 * textures are flipped vertically on load, Texture.hpp:49). */
typedef struct er_texture {
  int32_t width, height;
  const float* data; /* width*height*3 */
  float x_tile, y_tile, x_offset, y_offset;
} er_texture;

/* PointLight.hpp:6-18 */
typedef struct er_point_light {
  float position[3];
  float radiance[3];
} er_point_light;

/* Flat triangle soup in the reference's Tri layout (Tri.hpp:13-19), one
 * entry per triangle, vertices in winding order. */
typedef struct er_scene_desc {
  er_camera camera;
  int64_t tri_count;
  const float* positions;    /* tri_count*9                                 */
  const float* normals;      /* tri_count*9, NULL = zero normals            */
  const float* uvs;          /* tri_count*6 (u,v per vertex), NULL = zeros  */
  const float* tangents;     /* tri_count*9, NULL = zero tangents           */
  const float* tangent_sign; /* tri_count, NULL = +1                         */
  const int32_t* tri_object; /* tri_count: mesh object of each triangle     */
  int32_t object_count;
  const int32_t* object_material; /* object_count: material of each object;
                                     ignored (material 0) when object_count
                                     is 0                                    */
  int32_t material_count;
  const er_material* materials;
  int32_t texture_count;
  const er_texture* textures;
  int32_t light_count;
  const er_point_light* lights;
  er_texture env; /* environment map (HDRI.hpp); constant colours are given as
                     a filled texture, as HDRI(Vector3) does (HDRI.hpp:22-38) */
  /* Optional per-triangle tie key: among hits at exactly equal reference
   * distance the lowest key wins.  NULL = triangle index. */
  const uint32_t* tie_key;
} er_scene_desc;

/* BVH node formats. */
enum { ER_BVH_FP32 = 0, ER_BVH_Q8 = 1 };

/* BVH builders: the host SAH builder (default; slower to build, faster to
 * trace) or the GPU linear BVH (Morton order, ~100x faster to build).  The
 * hit set does not depend on the builder. */
enum { ER_BUILDER_HOST = 0, ER_BUILDER_GPU = 1 };

typedef struct er_scene_opts {
  int32_t bvh_format;     /* ER_BVH_FP32 or ER_BVH_Q8 */
  int32_t max_leaf_tris;  /* 1..8, 0 = default (4) */
  int32_t device;         /* CUDA device ordinal */
  void* stream;           /* cudaStream_t, NULL = handle-owned stream */
  int32_t builder;        /* ER_BUILDER_HOST or ER_BUILDER_GPU */
} er_scene_opts;

typedef struct er_scene er_scene;

typedef struct er_scene_info {
  int64_t tri_count;
  int64_t node_count;
  int64_t leaf_count;
  int64_t device_bytes;     /* bytes held on the device by the handle */
  double bvh_build_ms;      /* host BVH build time */
  double upload_ms;         /* host->device upload time */
  float scene_lo[3], scene_hi[3];
  float max_shading_offset; /* bound on |shading position - geometric hit| */
  int32_t bvh_depth;
  int32_t bvh_format;
  int32_t material_count;
  int32_t env_width, env_height;
  int32_t reserved;
} er_scene_info;

/* Build a scene from arrays (the harness / generator path). */
er_status er_scene_create(const er_scene_desc* desc, const er_scene_opts* opts,
                          er_scene** out);
/* Load a reference scene folder: scene.json, scene.obj, scene.mtl, HDRI/ and
 * the textures the .mtl names (SceneLoader.hpp:7-143).  x_res/y_res come
 * from scene.json. */
er_status er_scene_load(const char* dir, const er_scene_opts* opts,
                        er_scene** out);
/* The host half of er_scene_load, without a device: reads and parses a
 * scene folder (SceneLoader.hpp:7-143 loadScene, ObjLoader.hpp:20-206,
 * Texture.hpp:41-68, HDRI.hpp:42-60) into a description whose arrays the
 * er_folder handle owns.  er_folder_desc copies that description (its
 * pointers stay valid until er_folder_free); a caller may adjust it (the
 * reference's harness sets Material fields its .mtl reader cannot express)
 * and pass it to er_scene_create.  er_scene_load(dir) equals
 * er_scene_create(desc of er_scene_folder_read(dir)). */
typedef struct er_folder er_folder;
er_status er_scene_folder_read(const char* dir, er_folder** out);
er_status er_folder_desc(const er_folder* folder, er_scene_desc* out);
er_status er_folder_free(er_folder* folder);
er_status er_scene_info_get(const er_scene* scene, er_scene_info* out);
/* Replace the camera of a built scene (no BVH rebuild). */
er_status er_scene_set_camera(er_scene* scene, const er_camera* cam);
/* Current camera of a scene (resolution of the film; the camera a loaded
 * scene.json describes, SceneLoader.hpp:25-46). */
er_status er_scene_get_camera(const er_scene* scene, er_camera* out);
er_status er_scene_free(er_scene* scene);

/* ---------------------------------------------------------------- render -- */

enum {
  ER_RENDER_DEVICE_OUT = 1u << 0, /* output pointers are device pointers    */
  ER_RENDER_ACCUM_FP64 = 1u << 1, /* FP64 per-pixel sums instead of the
                                     reference FP32 running mean            */
  ER_RENDER_AOV = 1u << 2,        /* also write NORMAL/TANGENT/BITANGENT     */
  ER_RENDER_ENV_ALIAS = 1u << 3,  /* env sampling through the FP64-built
                                     alias table of the reference's effective
                                     texel distribution                     */
  ER_RENDER_CONTINUE = 1u << 4,   /* add samples to the film of the previous
                                     call instead of clearing it            */
  ER_RENDER_NO_OUTPUT = 1u << 5,  /* render into the film only              */
  ER_RENDER_PROFILE = 1u << 6,    /* CUDA-event time per stage (stats)      */
  ER_RENDER_COUNT = 1u << 7,      /* count node visits / triangle tests     */
  ER_RENDER_SNAPSHOTS = 1u << 8,  /* copy the film to the snapshot buffer
                                     after every wave (er_snapshot)         */
  ER_RENDER_KEEP_PATHS = 1u << 10, /* keep every sample's radiance on the
                                     device, so that an er_backward with the
                                     same options (and unchanged parameters
                                     and camera) skips its forward pass     */
  ER_RENDER_ONE_STREAM = 1u << 9  /* run the waves one after another on the
                                     scene's stream.  Default with two or
                                     more waves: two waves in flight on two
                                     streams (the second an internal one),
                                     accumulated in sample order, so the
                                     film is the same; ER_RENDER_PROFILE
                                     implies this flag                      */
};

/* Stages of the wavefront, indices of er_render_stats.stage_ms.  TRACE is
 * the traversal launch of a bounce (its extension rays together with the
 * previous bounce's shadow rays); index 3 is reserved. */
enum { ER_STAGE_RAYGEN = 0, ER_STAGE_TRACE = 1, ER_STAGE_SHADE = 2, ER_STAGE_RESERVED = 3,
       ER_STAGE_ACCUMULATE = 4, ER_STAGE_COUNT = 5 };

typedef struct er_render_opts {
  int32_t spp;            /* samples per pixel of this call                 */
  int32_t sample_begin;   /* first sample index (for split / resumed runs) */
  int32_t max_depth;      /* MAXBOUNCES (Definitions.h:9); 0 = 5            */
  int32_t spp_per_wave;   /* samples per pixel traced together; 0 = auto    */
  uint64_t seed;          /* RNG key                                        */
  uint32_t flags;         /* ER_RENDER_*                                    */
  int32_t reserved;
} er_render_opts;

typedef struct er_render_stats {
  double ms;              /* device time of the call (CUDA events)          */
  int64_t samples;        /* path samples traced                            */
  int64_t rays_closest;   /* extension rays traced                          */
  int64_t rays_shadow;    /* shadow rays traced                             */
  int64_t path_vertices;  /* sum of bounce counts: the reference's "paths"
                             counter (kernel.cu:445, main.cpp:105-106)      */
  int64_t kernel_launches;
  double stage_ms[ER_STAGE_COUNT];        /* with ER_RENDER_PROFILE        */
  int64_t stage_launches[ER_STAGE_COUNT];
  int64_t closest_nodes, closest_tris;    /* with ER_RENDER_COUNT          */
  int64_t shadow_nodes, shadow_tris;
} er_render_stats;

/* Render `opts->spp` samples per pixel.  beauty (and, with ER_RENDER_AOV,
 * normal/tangent/bitangent) are W*H*4 floats in the reference's pass layout
 * (RGBA, alpha = 1, row y = 0 at the top of the image as the reference's
 * vertically flipped index, kernel.cu:378).  samples and pathcount are W*H
 * uint32 (dev_samples / dev_pathcount, kernel.cu:44-45).  Any output pointer
 * may be NULL.  stats may be NULL. */
er_status er_render(er_scene* scene, const er_render_opts* opts, float* beauty,
                    float* normal, float* tangent, float* bitangent,
                    uint32_t* samples, uint32_t* pathcount,
                    er_render_stats* stats);

/* Read the current film (after one or more er_render calls). */
er_status er_film_read(er_scene* scene, uint32_t flags, float* beauty,
                       float* normal, float* tangent, float* bitangent,
                       uint32_t* samples, uint32_t* pathcount);

/* The film's per-pixel FP64 sums of the clamped sample radiance (W*H*3
 * doubles, the film's pixel order) and sample counts, when every render into
 * it since it was last cleared ran with ER_RENDER_ACCUM_FP64
 * (ER_ERR_INVALID_ARG otherwise).  The exact form of the film for callers
 * that merge films of sample ranges rendered apart, or difference two films
 * (the FP32 beauty rounds each pixel's mean once more). */
er_status er_film_read_sums(er_scene* scene, uint32_t flags, double* sums, uint32_t* samples);

/* Progressive readback while er_render runs on another thread (the
 * reference's window loop polls getBuffers during renderCuda, main.cpp:53,
 * kernel.cu:688-710): the film as of the last finished wave of a render
 * made with ER_RENDER_SNAPSHOTS (beauty RGBA float and per-pixel sample
 * counts, host pointers; either may be NULL).  The only call that may run
 * concurrently with another call on the same scene; it uses its own
 * stream.  ER_ERR_INVALID_ARG until a first wave has finished. */
er_status er_snapshot(er_scene* scene, float* beauty, uint32_t* samples);

/* Allocation-free render.  No counterpart in the reference: it is for
 * callers that may not allocate device memory while rendering (a host
 * application with a device-memory budget fixed at start-up, a render thread
 * that may not enter the CUDA allocator).  The call allocates nothing: the
 * path state and ray queues live in one file-scope device array sized for
 * ER_NOALLOC_MAX_PATHS paths (about 19 MB, held on every GPU that loads the
 * library until the process exits), and the film is the caller's device
 * buffers: beauty W*H*4 floats (16-byte aligned), samples and pathcount
 * W*H uint32, laid out as in er_render.
 *  - W*H must not exceed ER_NOALLOC_MAX_PATHS (ER_ERR_INVALID_ARG otherwise);
 *    spp is traced in waves of opts->spp_per_wave samples (0, or a larger
 *    value: floor(ER_NOALLOC_MAX_PATHS / (W*H)) samples).
 *  - Only ER_RENDER_CONTINUE is accepted in opts->flags (FP32 running mean,
 *    no AOVs); without it the film is cleared first.
 *  - beauty must be 16-byte aligned, samples and pathcount 4-byte aligned.
 *  - The array's device address is looked up, with the scene's device
 *    current, when a scene is created (er_scene_create / er_scene_load): under
 *    CUDA's lazy module loading that is when the module holding the array is
 *    loaded and its memory taken, so er_render_noalloc itself allocates
 *    nothing.  If that lookup failed there, the first er_render_noalloc call
 *    on the device repeats it; make that first call before any stream capture.
 *    A cudaDeviceReset ends every scene of the device; the next scene created
 *    there looks the address up again.
 *  - All calls share the array and it keeps the last call's contents (each
 *    wave re-initialises what it reads).  Calls whose work overlaps on the
 *    GPU (other streams, other threads) race on it: serialise them.
 * Synchronous like er_render.  Results equal er_render's for the same
 * options. */
#define ER_NOALLOC_MAX_PATHS 65536
er_status er_render_noalloc(er_scene* scene, const er_render_opts* opts, float* beauty, uint32_t* samples,
                            uint32_t* pathcount);

/* Per-path debug output of one wave: radiance (before the clamp of
 * kernel.cu:447) and bounce count of path (pixel p, sample s) for
 * s in [sample_begin, sample_begin+spp).  radiance is spp*W*H*3 floats,
 * bounces spp*W*H int32, both indexed [s][p] with p the output pixel index. */
er_status er_render_paths(er_scene* scene, const er_render_opts* opts,
                          float* radiance, int32_t* bounces);

/* Environment sampling diagnostics: counts[i] = how many of the 2^24
 * uniform values the reference's HDRI::binarySearch (HDRI.hpp:130-142) maps
 * to texel i (its effective distribution is counts / 2^24), and the alias
 * table ER_RENDER_ENV_ALIAS samples it with (column i is kept when a 32-bit
 * coin is below thresh[i], else alias[i] is taken).  Arrays of env w*h
 * entries; any may be NULL.  Builds the table on first use. */
er_status er_env_distribution(er_scene* scene, uint32_t* counts, int32_t* alias, uint32_t* thresh);

/* The texel HDRI::binarySearch returns for each of its 2^24 inputs
 * k * 2^-24, k = 1..2^24 (table[k - 1]); environments of at least 65,536
 * texels are sampled through this table (one load instead of the search,
 * same texel).  table: 2^24 int32 (host).  ER_ERR_INVALID_ARG for a smaller
 * environment, which is sampled by the search itself. */
er_status er_env_search_table(er_scene* scene, int32_t* table);

/* -------------------------------------------------------------- tangents -- */
/* Per-corner tangents (9 floats per triangle) and a per-triangle sign in
 * the manner of the MikkTSpace generator the reference's loader runs on
 * every object (ObjLoader.hpp:167-168): welded corners, texture-space
 * triangle tangents projected onto the corner normal's plane, angle-weighted
 * per vertex and orientation.  er_scene_load calls it per object. */
er_status er_compute_tangents(int64_t tri_count, const float* positions, const float* normals, const float* uvs,
                              float* tangents, float* tangent_sign);

/* ---------------------------------------------------------- post-process -- */
/* The reference's PostProcessing.cpp as one GPU pass, applied in this
 * order: applyExposure (:3-6), basicBlur bloom (:132-211), Reinhard
 * (:35-39) or ACES (:41-52) tone map, clampPixels (:30-33), applysRGB
 * (:54-57), flipX (:19-28) / flipY (:8-17).  rgba_out receives the float result,
 * ldr_out its 8-bit encoding as er_encode_ldr makes it (either may be
 * NULL).  flags: ER_RENDER_DEVICE_OUT for device pointers. */
enum { ER_TONEMAP_NONE = 0, ER_TONEMAP_REINHARD = 1, ER_TONEMAP_ACES = 2 };

typedef struct er_post_opts {
  float exposure;        /* 1 = unchanged */
  int32_t tonemap;       /* ER_TONEMAP_* */
  int32_t clamp;         /* 1: clamp to [0, 1] */
  int32_t srgb;          /* 1: pow(x, 1/2.2) */
  int32_t flip_x, flip_y;
  float bloom_threshold, bloom_power, bloom_radius;  /* bloom_power 0 = no bloom */
} er_post_opts;

er_status er_postprocess(const float* rgba_in, int32_t width, int32_t height, const er_post_opts* opts,
                         float* rgba_out, uint8_t* ldr_out, uint32_t flags);

/* --------------------------------------------------------------- adjoint -- */
/* Differentiable parameters (no counterpart in the reference): per material
 * 5 floats (albedo r, g, b, roughness, metallic, before the 2.2 power of
 * kernel.cu:103-104) and the environment's texels (w*h*3 floats, storage
 * order).  flags: ER_RENDER_DEVICE_OUT for device arrays.  Setting the
 * environment rebuilds its CDF (HDRI.hpp:107-128). */
er_status er_scene_get_params(er_scene* scene, float* materials, float* env);
er_status er_scene_set_params(er_scene* scene, const float* materials, const float* env, uint32_t flags);

/* Forward render of the detached estimator: sampling (directions, pdfs, MIS
 * weights, chosen texel and light) from the scene's parameters, BRDF values
 * and environment radiance from eval_materials / eval_env (NULL = the
 * scene's).  It runs the er_render wavefront and, like er_render, replaces
 * the scene's film.  With both NULL the film equals er_render's for the
 * same options.  Only ER_RENDER_DEVICE_OUT, ER_RENDER_ENV_ALIAS and
 * ER_RENDER_ACCUM_FP64 apply (FP64 per-pixel sums, so that finite
 * differences of the estimator see no running-mean rounding). */
er_status er_render_replay(er_scene* scene, const er_render_opts* opts, const float* eval_materials,
                           const float* eval_env, float* beauty, uint32_t* samples, uint32_t* pathcount);

/* Gradient of a loss with respect to the parameters, by path replay of the
 * samples er_render made with the same opts: d_beauty = d loss / d beauty
 * (W*H*4 floats, the film's layout), samples = that render's per-pixel
 * sample counts.  The derivative holds the sampling fixed (the detached
 * estimator er_render_replay evaluates).  Outputs: n_materials*5 and
 * env w*h*3 floats.  The samples' radiance comes from the last er_render
 * when it ran with ER_RENDER_KEEP_PATHS and the same seed, sample range,
 * depth and env sampling, with no er_scene_set_params / set_camera since;
 * otherwise er_backward renders them again first.  stats (may be NULL):
 * ms = device time of the replay (and of the forward it renders again),
 * samples, kernel_launches; the ray counters stay 0. */
er_status er_backward(er_scene* scene, const er_render_opts* opts, const float* d_beauty, const uint32_t* samples,
                      float* grad_materials, float* grad_env, er_render_stats* stats);

/* ----------------------------------------------------------------- batch -- */
/* Many scenes and views rendered together.  No counterpart in the
 * reference, whose renderCuda (kernel.cu:665-686) renders one scene per
 * process through device globals.  A batch merges the device data of its
 * scenes (which must outlive it and stay unchanged); each job is a scene,
 * a view and sample options; all jobs share wavefront queues, and one
 * render is one captured CUDA graph.  Each job's film equals er_render's for
 * the same scene, camera and options. */
typedef struct er_batch er_batch;

typedef struct er_batch_job {
  int32_t scene;          /* index into the scenes given to er_batch_create */
  int32_t spp;
  int32_t max_depth;      /* <= 0: 5 */
  int32_t sample_begin;
  uint64_t seed;
  uint32_t flags;         /* ER_RENDER_ENV_ALIAS, ER_RENDER_ACCUM_FP64 */
  int32_t reserved;
  er_camera camera;       /* the view; the film is camera.x_res x y_res */
} er_batch_job;

/* Schedule of a batch render (what er_batch_autotune searches). */
typedef struct er_batch_tuning {
  int32_t wave_paths;           /* paths per wave; 0 = 8,388,608; at least the largest job's pixels */
  int32_t trace_blocks_per_sm;  /* persistent traversal grid = SMs x this; 0 = as many as fit */
  int32_t shade_blocks_per_sm;  /* shading grid = SMs x this; 0 = as many as fit */
  int32_t split_trace;          /* 1: extension, point-light and env rays as three traversal launches */
  int32_t use_graph;            /* 1: capture the launch sequence once and replay it */
  int32_t one_stream;           /* 1: waves one after another; 0: two waves in flight on two streams */
  int32_t reserved[2];
} er_batch_tuning;

/* opts: bvh_format (ER_BVH_Q8 needs scenes built with it) and stream. */
er_status er_batch_create(er_scene* const* scenes, int32_t n_scenes, const er_scene_opts* opts, er_batch** out);
/* Replaces the job list (allocates each job's film). */
er_status er_batch_set_jobs(er_batch* batch, const er_batch_job* jobs, int32_t n_jobs);
/* Renders every job from a cleared film.  tuning NULL: the autotuned
 * schedule if er_batch_autotune ran, else the defaults. */
er_status er_batch_render(er_batch* batch, const er_batch_tuning* tuning, er_render_stats* stats);
/* Film of one job: RGBA float beauty, per-pixel sample and path-vertex
 * counts (flags: ER_RENDER_DEVICE_OUT for device destinations). */
er_status er_batch_read(er_batch* batch, int32_t job, uint32_t flags, float* beauty, uint32_t* samples,
                        uint32_t* pathcount);
/* Times the current jobs under candidate schedules (best of reps renders
 * each) and keeps the fastest for er_batch_render(batch, NULL, ...). */
er_status er_batch_autotune(er_batch* batch, int32_t reps, er_batch_tuning* best);
er_status er_batch_info(const er_batch* batch, int32_t* n_waves, int64_t* device_bytes);
er_status er_batch_free(er_batch* batch);

/* ----------------------------------------------------------------- trace -- */

enum {
  ER_TRACE_DEVICE_PTRS = 1u << 0, /* all pointers are device pointers        */
  ER_TRACE_NORMALIZED = 1u << 1,  /* directions already went through the
                                     reference Ray constructor normalisation  */
  ER_TRACE_STATS = 1u << 2        /* count node / triangle tests             */
};

typedef struct er_trace_stats {
  double ms;
  int64_t node_visits;
  int64_t box_tests;
  int64_t tri_tests;
} er_trace_stats;

/* Closest hit of n rays, each 6 floats (origin xyz, direction xyz).  The
 * direction is normalised as Ray.hpp:14-18 does unless ER_TRACE_NORMALIZED.
 * tri_id[i] = index of the hit triangle in the scene desc or -1; dist[i] =
 * |hit position - origin| with the reference's hit position (smooth-shading
 * position when convex, Tri.hpp:74-92); uv[2i..2i+1] = barycentric (u, v).
 * dist / uv may be NULL. */
er_status er_trace_closest(er_scene* scene, const float* rays, int64_t n,
                           int32_t* tri_id, float* dist, float* uv,
                           uint32_t flags, er_trace_stats* stats);

/* ----------------------------------------------------------- measurement -- */
/* Bandwidth ceilings of a GPU measured by this library's own streaming
 * kernels (no counterpart in the reference; the denominators of the
 * traversal and shading rooflines).  ER_BW_L2_READ: a buffer of `bytes`
 * (1 MiB .. 64 MiB, resident in L2) read `reps` times with 16-byte loads
 * cached in L2 only; ER_BW_HBM_COPY: a buffer of `bytes` (at least 1 MiB,
 * at most 32 GiB; choose it far larger than L2) copied `reps` times, read +
 * written bytes counted.  gbps = bytes moved / CUDA-event time.  Allocates
 * and frees its buffers. */
enum { ER_BW_L2_READ = 0, ER_BW_HBM_COPY = 1 };
er_status er_device_bandwidth(int32_t device, int32_t kind, int64_t bytes, int32_t reps, double* gbps);

/* ----------------------------------------------------------------- image -- */

/* Reference output step (main.cpp:150-165, PostProcessing.cpp:30-33):
 * clamp to [0,1], approximate pow(x, 1/2.2) by the fastPow bit trick
 * (stb_image.h:127-135), *255, truncate.  rgba_in is W*H*4 floats on the
 * host, out is W*H*4 bytes. */
er_status er_encode_ldr(const float* rgba_in, int32_t width, int32_t height,
                        uint8_t* out);
/* Write W*H*4 bytes as PNG (what the reference writes, also for .bmp names)
 * or, when as_bmp != 0, as a 24-bit BMP. */
er_status er_write_image(const char* path, const uint8_t* rgba, int32_t width,
                         int32_t height, int32_t as_bmp);

#ifdef __cplusplus
}
#endif
#endif /* ELEVEN_H */
