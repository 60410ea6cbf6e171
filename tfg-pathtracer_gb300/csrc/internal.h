// Host-side internals of libeleven: device scene layout, film, status helpers.
#pragma once

#include <cuda_runtime.h>

#include <cstdint>
#include <exception>
#include <mutex>
#include <new>
#include <stdexcept>
#include <string>
#include <vector>

#include "eleven.h"

namespace er {

// ---------------------------------------------------------------- status --

void set_error(const std::string& msg);
er_status fail(er_status s, const std::string& msg);
er_status cuda_fail(cudaError_t e, const char* what);

// Runs the body of a C-ABI entry point: a C++ exception (a host allocation
// that failed, a container size out of range) becomes a status instead of
// crossing the C ABI.
template <typename F>
er_status guarded(const char* what, F&& body) noexcept {
  er_status s = ER_ERR_INVALID_ARG;
  const char* why = "unexpected exception";
  try {
    return body();
  } catch (const std::bad_alloc&) {
    s = ER_ERR_OOM;
    why = "host memory allocation failed";
  } catch (const std::length_error&) {
    s = ER_ERR_OOM;
    why = "host buffer size out of range";
  } catch (...) {
  }
  try {
    fail(s, std::string(what) + ": " + why);
  } catch (...) {  // no memory left for the message either
  }
  return s;
}

// Frees a half-built handle when an exception unwinds past it (guarded()
// then reports it); the error returns free it themselves.
template <typename T>
struct FreeOnUnwind {
  T* h;
  er_status (*free_fn)(T*);
  int n = std::uncaught_exceptions();
  ~FreeOnUnwind() {
    if (std::uncaught_exceptions() > n) free_fn(h);
  }
};

#define ER_CUDA(call)                                        \
  do {                                                       \
    cudaError_t e_ = (call);                                 \
    if (e_ != cudaSuccess) return ::er::cuda_fail(e_, #call); \
  } while (0)

// ------------------------------------------------------------ BVH layout --
//
// FP32 BVH4 node, 128 bytes (two 64-byte lines), loaded as 8 float4:
//   [0] lo.x[4] [1] hi.x[4] [2] lo.y[4] [3] hi.y[4] [4] lo.z[4] [5] hi.z[4]
//   [6] child[4] (int bits)  [7] shading-offset bound of each child (float)
// child: >= 0 internal node index; kEmpty = no child; otherwise a leaf:
//   bit 31 set, bits 30..27 = tri count - 1, bits 26..0 = first leaf slot.
// An empty slot's box is inverted, lo = +inf and hi = -inf on every axis,
// so the slab test rejects it for every ray without looking at the child.
constexpr int32_t kEmpty = -1;
constexpr uint32_t kLeafBit = 0x80000000u;
constexpr int kLeafCountShift = 27;
constexpr uint32_t kLeafFirstMask = (1u << 27) - 1;
constexpr int kMaxLeafTris = 16;
constexpr int64_t kMaxTris = (int64_t)kLeafFirstMask - 1;

inline int32_t make_leaf(uint32_t first, uint32_t count) {
  return (int32_t)(kLeafBit | ((count - 1u) << kLeafCountShift) | first);
}

// 8-bit quantised BVH4 node, 64 bytes:
//   [0] origin.xyz (float), w = exponent bytes e.x | e.y<<8 | e.z<<16
//   [1] qlo.x[4] qhi.x[4] qlo.y[4] qhi.y[4] as bytes
//   [2] qlo.z[4] qhi.z[4], child[0..1]
//   [3] child[2..3], shading-offset bound (max of the 4 children), pad
// child box = origin + q * 2^e, rounded outward at build time.
struct QNode {
  float ox, oy, oz;
  uint32_t ex;
  uint8_t qlx[4], qhx[4], qly[4], qhy[4];
  uint8_t qlz[4], qhz[4];
  int32_t child01[2];
  int32_t child23[2];
  float delta;
  uint32_t pad;
};
static_assert(sizeof(QNode) == 64, "QNode is one 64-byte line");

struct BuildResult {
  std::vector<float> nodes;        // 32 floats per FP32 node
  std::vector<QNode> qnodes;       // quantised form (same topology)
  std::vector<int32_t> order;      // leaf slot -> desc triangle index
  int64_t node_count = 0, leaf_count = 0;
  int32_t depth = 0;
  float max_delta = 0;
};

// A BVH4 built on the device (bvh_gpu.cu): node and leaf-order triangle
// arrays allocated on the scene.
struct GpuBvh {
  const float4* nodes;
  const float4* tri_v;
  const float4* tri_n;
  const float2* tri_uv;
  const float4* tri_t;
  int64_t node_count, leaf_count;
  int32_t depth;
  float max_delta;
  double build_ms;
};
er_status build_bvh_gpu(er_scene* s, const er_scene_desc* d, int max_leaf, const float scene_lo[3],
                        const float scene_hi[3], GpuBvh* out);

// Builds the SAH BVH4 over the desc's triangles (bvh_build.cpp).
er_status build_bvh4(const er_scene_desc* d, int max_leaf, BuildResult* out);
void quantize_bvh4(BuildResult* r);
// Bound on |shading position - geometric hit| for triangle i (Tri.hpp:74-92).
double shading_offset_bound(const er_scene_desc* d, int64_t i);

// ----------------------------------------------------------- device scene --

// Texture descriptor on the device (Texture.hpp:196-214).
struct DevTex {
  int32_t w, h;
  int64_t offset;  // float4 texel offset into the texel pool
  float x_tile, y_tile, x_offset, y_offset;
};

// Camera with the per-ray trigonometry hoisted (kernel.cu:297-306).
struct DevCamera {
  int32_t x_res, y_res;
  float focal_length, sensor_width, sensor_height, aperture, focus_distance;
  float px, py, pz;
  float cx, sx, cy, sy, cz, sz;  // cosf / sinf of the rotation in radians
  int32_t bokeh;
};

// Material as the shader reads it (Material.hpp:8-37).
struct DevMaterial {
  int32_t albedo_tex, emission_tex, roughness_tex, metallic_tex, normal_tex, pad0, pad1, pad2;
  float albedo[4];
  float emission[4];
  float roughness, metallic, clearcoat_gloss, clearcoat, anisotropic, eta, transmission, specular;
  float specular_tint, sheen_tint, subsurface, sheen;
};

struct DevScene {
  const float4* nodes;   // FP32 BVH4 (8 float4 per node)
  const uint4* qnodes;   // quantised BVH4 (4 uint4 per node) or null
  const float4* tri_v;   // 3 float4 per leaf slot: v0|desc id, v1|tie key, v2|material
  const float4* tri_n;   // 3 float4 per leaf slot: n0|tangent sign, n1, n2
  const float2* tri_uv;  // 3 float2 per leaf slot
  const float4* tri_t;   // 3 float4 per leaf slot (tangents) or null
  const DevMaterial* mats;
  const DevTex* texs;
  const float4* texels;  // RGB(A) texel pool
  const er_point_light* lights;
  DevTex env;
  const float* cdf;      // env CDF, w*h+1 floats (HDRI.hpp:107-128)
  const int32_t* alias_idx;   // env alias table (w*h) or null (env.cu)
  const uint32_t* alias_thresh;
  const int32_t* env_lut;     // the CDF search's texel for each of its 2^24 inputs, or null (env.cu)
  float radiance_sum;
  int32_t n_lights;
  int32_t n_mats;
  int32_t n_texs;
  int64_t n_tris;
  int64_t n_nodes;
  float scene_eps;       // absolute slack for conservative box tests
  int32_t use_q8;
  DevCamera cam;
};

struct Film {
  int32_t w = 0, h = 0;
  float4* beauty = nullptr;
  float4* aov[3] = {nullptr, nullptr, nullptr};
  double* sum = nullptr;       // FP64 sums (3 per pixel) in FP64 mode
  bool sum_valid = false;      // every sample of the film went into sum
  uint32_t* samples = nullptr;
  uint32_t* pathcount = nullptr;
  bool aov_on = false;
  // optional per-sample radiance (before the clamp), 3 floats at
  // (sample - first sample) * npix + pixel index; keep_s0 = the wave's
  // first sample relative to the call's
  float* keep = nullptr;
  int32_t keep_s0 = 0;
};

struct Wave;  // wavefront buffers (render.cu)

// Per-wave constants of the sample loop (one job's slice of samples).
struct WaveParams {
  int32_t W, H, npix, spp_wave, sample_base, max_depth;
  uint32_t k0, k1;
  uint32_t flags;
};

// ------------------------------------------------------------------ batch --
//
// A batch wave holds slices of several jobs: slice k owns the wave's paths
// [path_base, path_base + spp_wave * npix) and accumulate items
// [pix_base, pix_base + npix).  Jobs see one merged device scene; what
// differs per job (BVH root, environment, lights, camera, film) comes from
// the job table.
struct BatchSeg {
  int32_t path_base, pix_base, job, pad;
  WaveParams P;
};

struct BatchJobDev {
  DevTex env;
  const float* cdf;
  const int32_t* alias_idx;
  const uint32_t* alias_thresh;
  const int32_t* env_lut;
  const er_point_light* lights;
  float radiance_sum;
  int32_t n_lights;
  int32_t root;       // BVH root node in the merged node array
  float scene_eps;
  DevCamera cam;
  Film film;
};

struct BatchView {
  const BatchSeg* segs = nullptr;
  const BatchJobDev* jobs = nullptr;
  int32_t n_segs = 0;
  int32_t n_acc = 0;
};

// One wave of a batch plan: segments [seg_begin, seg_begin + n_segs) of the
// plan's device segment table.
struct BatchWave {
  int32_t seg_begin, n_segs, n_paths, n_acc, max_depth;
};

// Launch schedule knobs (the autotuner's search space).
struct BatchSchedule {
  int32_t trace_blocks_per_sm;  // 0 = as many as fit
  int32_t shade_blocks_per_sm;  // 0 = as many as fit
  bool split_trace;             // extension / point / env traversal as three launches
};

// Second wave pipeline of a batch: waves alternate between (wave, stream)
// and (w2, s2); accumulates are chained by ev_acc in wave order.
struct BatchPair {
  Wave* w2 = nullptr;
  cudaStream_t s2 = nullptr;
  cudaEvent_t ev_fork = nullptr, ev_join = nullptr, ev_acc[2] = {nullptr, nullptr};
};

}  // namespace er

struct er_scene {
  int device = 0;
  cudaStream_t stream = nullptr;
  bool own_stream = false;
  er::DevScene dev{};
  std::vector<void*> allocs;   // device allocations owned by the handle
  int64_t device_bytes = 0;
  er_scene_info info{};
  er_camera camera{};
  int num_sms = 0;
  er::Film film;
  er::Wave* wave = nullptr;
  // adjoint scratch kept between er_backward calls: per-path radiance and
  // vertex counts of the dumped forward pass, gradient accumulators
  float* bw_rad = nullptr;
  int32_t* bw_b = nullptr;
  int64_t bw_cap = 0;
  // radiance kept by er_render (ER_RENDER_KEEP_PATHS) and the options it
  // belongs to; `version` counts parameter and camera changes
  float* kp_rad = nullptr;
  int64_t kp_cap = 0;
  bool kp_valid = false;
  uint64_t kp_seed = 0;
  int32_t kp_begin = 0, kp_spp = 0, kp_depth = 0;
  uint32_t kp_flags = 0;
  uint64_t kp_version = 0, version = 0;
  // second wave in flight (its own buffers and stream), so that one wave's
  // launches fill the other's traversal tails
  er::Wave* wave2 = nullptr;
  cudaStream_t stream2 = nullptr;
  // page-locked words read back by every render call without a blocking
  // copy: the device error word at 0, the statistics counters at 64
  unsigned char* h_pin = nullptr;
  cudaEvent_t ev_fork = nullptr, ev_acc[2] = {nullptr, nullptr};
  uint32_t* err_word = nullptr;   // device error word (bounds / timeout)
  unsigned long long* d_stats = nullptr;  // device ray counters
  std::vector<cudaEvent_t> ev_pool;       // per-launch profiling events
  std::vector<int> ev_stage;
  // environment tables (env.cu): allocated once, refilled after an
  // environment change
  const uint32_t* env_counts = nullptr;   // effective env texel counts
  void* env_q = nullptr;                  // FP64 alias weights
  void* env_alias_buf = nullptr;
  void* env_thresh_buf = nullptr;
  void* env_lut_buf = nullptr;
  bool env_alias_ok = false, env_lut_ok = false;
  int64_t texel_count = 0;                // float4 entries of dev.texels (textures + env)
  cudaEvent_t ev0 = nullptr, ev1 = nullptr;
  // progressive readback (er_snapshot): a copy of the film after each wave
  std::mutex snap_mu;
  float4* snap_beauty = nullptr;
  uint32_t* snap_samples = nullptr;
  int32_t snap_w = 0, snap_h = 0;
  bool snap_valid = false;
  cudaEvent_t snap_event = nullptr;
  cudaStream_t snap_stream = nullptr;
};

namespace er {
er_status dev_alloc(er_scene* s, void** p, size_t bytes);
er_status upload(er_scene* s, void** p, const void* host, size_t bytes);
DevCamera make_dev_camera(const er_camera& c);
void free_wave(er_scene* s);
void free_film(er_scene* s);
// Looks up (again) the device address of er_render_noalloc's scratch array
// on the current device, `device` (render.cu); errors are left to the call.
void noalloc_prepare(int device);
er_status check_device_error(er_scene* s);
// Resolution (1 .. 2^28 pixels) and finite lens and pose parameters.
er_status validate_camera(const er_camera& c);
// Resident blocks of `block` threads per SM for `kernel` on the current
// device (at least 1), cached per kernel, block size and device.
int blocks_per_sm(const void* kernel, int block);
er_status build_env_alias(er_scene* s);
// The search lookup table for environments of at least kEnvLutMinTexels
// texels (no-op below); the tables are refilled after invalidate_env_tables.
er_status build_env_lut(er_scene* s);
void invalidate_env_tables(er_scene* s);
constexpr int64_t kEnvLutMinTexels = 65536;
// Per-corner tangents and per-triangle signs (tangents.cpp).
void compute_tangents(int64_t n_tris, const float* pos, const float* nrm, const float* uv, float* tangents,
                      float* sign);
// Environment CDF and radiance sum as the reference builds them (scene.cpp).
void hdri_cdf(const er_texture& t, std::vector<float>& cdf, float* radiance_sum);

// Inputs and outputs of the gradient wavefront (er_backward): the forward
// dump's per-path radiance (sample-major from sample0, output index order),
// d loss / d beauty and the forward film's sample counts per pixel, and the
// gradient arrays (materials x 5, env texels x 3).
struct GradArgs {
  // forward evaluation parameters (er_render_replay): materials (n x 5) and
  // env texels (w*h*3) the BRDF values and environment radiance are taken
  // from while the sampling stays with the scene's; null = the scene's
  const float* eval_mat = nullptr;
  const float* eval_env = nullptr;
  const float* rad = nullptr;
  const float4* d_beauty = nullptr;
  const uint32_t* nvalid = nullptr;
  float* g_mat = nullptr;
  float* g_env = nullptr;
  int32_t sample0 = 0;
};
// Runs the samples of opts through the wavefront with the gradient variant
// of the shade stage (render.cu); adds its kernel launches to *launches.
er_status render_backward_device(er_scene* s, const er_render_opts* o, const GradArgs& G, int64_t* launches);
// The detached estimator (er_render_replay): the samples of opts through the
// wavefront with BRDF values and environment radiance from the evaluation
// parameters in G (device arrays), into the scene's film; outputs as
// er_render's (render.cu).
er_status render_eval_device(er_scene* s, const er_render_opts* o, const GradArgs& G, float* beauty,
                             uint32_t* samples, uint32_t* pathcount);
// Per-path radiance (spp x npix x 3, sample-major, output index order) and
// vertex counts of the samples er_render makes with opts, into device
// buffers (render.cu).  grad_wave: size the wave buffers for the gradient
// wavefront that follows, so that it reuses them.  launches != null: set to
// the kernel launches it made.
er_status render_paths_device(er_scene* s, const er_render_opts* o, float* d_rad, int32_t* d_b,
                              bool grad_wave = false, int64_t* launches = nullptr);
// Wavefront buffers for `cap` paths (render.cu); stats = device ray counters.
er_status wave_create(int64_t cap, unsigned long long* stats, Wave** out);
void wave_destroy(Wave* w);
er_status film_clear(const Film& F, cudaStream_t stream);
// Launches every wave of a batch plan on `stream` (render.cu).
er_status batch_launch(const DevScene& S, Wave* w, const BatchSeg* d_segs, const BatchJobDev* d_jobs,
                       const std::vector<BatchWave>& waves, const BatchSchedule& sch, int num_sms, uint32_t* err,
                       cudaStream_t stream, int64_t* launches, const BatchPair* pair = nullptr);
}  // namespace er
