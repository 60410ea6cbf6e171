// Batched rendering: many scenes and views in shared wavefront queues.
//
// The reference renders one scene per process (its device state is global,
// kernel.cu:41-52).  A batch instead merges its scenes into one device scene
// (BVH nodes, triangle slots, materials, textures and texels concatenated,
// with child / slot / material / texture / texel indices rebased by small
// fix-up kernels), so the traversal and shading kernels keep a single set of
// scene pointers and a ray only carries its job, whose BVH root it starts
// from.  Jobs (scene, camera, spp, depth, seed) are cut into sample slices
// that fill waves of a fixed path budget; several jobs share each wave, so
// small jobs no longer leave the GPU idle and the deep-bounce tails of many
// jobs are traced together.  The whole launch sequence of a render (film
// clears and every wave) is captured once into a CUDA graph and replayed.
// An autotuner picks the wave budget, the grid sizes of the persistent
// traversal and shading kernels, and whether the three traversal phases run
// fused in one launch or split, by timing the batch itself.
//
// Slices of a job are accumulated in sample order with the single-scene
// accumulation, and the per-sample random numbers depend only on (pixel,
// sample, seed), so every job's film equals er_render's for the same scene,
// camera and options, bit for bit.
#include <algorithm>
#include <chrono>
#include <cstring>
#include <string>
#include <vector>

#include "internal.h"

using namespace er;

struct er_batch {
  int device = 0;
  cudaStream_t stream = nullptr;
  bool own_stream = false;
  int num_sms = 0;
  std::vector<er_scene*> scenes;
  DevScene dev{};                 // merged scene
  std::vector<int32_t> root;      // per scene: BVH root in the merged nodes
  std::vector<int64_t> texel_base;
  std::vector<void*> allocs;      // merged arrays, counters
  int64_t device_bytes = 0;
  uint32_t* err_word = nullptr;
  unsigned long long* d_stats = nullptr;
  // jobs
  std::vector<er_batch_job> jobs;
  std::vector<Film> films;
  BatchJobDev* d_jobs = nullptr;
  // plan for plan_budget paths per wave
  int64_t plan_budget = 0;
  std::vector<BatchWave> waves;
  BatchSeg* d_segs = nullptr;
  Wave* wave = nullptr;
  int64_t wave_cap = 0;
  BatchPair pair;  // second wave pipeline (allocated on first use)
  // captured launch sequence
  cudaGraphExec_t graph = nullptr;
  er_batch_tuning graph_tuning{};
  int64_t graph_launches = 0;
  er_batch_tuning tuned{};
  bool has_tuned = false;
  cudaEvent_t ev0 = nullptr, ev1 = nullptr;
};

namespace {

constexpr int32_t kDefaultWavePaths = 1 << 23;

er_status balloc(er_batch* b, void** p, size_t bytes) {
  *p = nullptr;
  cudaError_t e = cudaMalloc(p, std::max<size_t>(bytes, 16));
  if (e != cudaSuccess) {
    *p = nullptr;
    cudaGetLastError();
    return fail(e == cudaErrorMemoryAllocation ? ER_ERR_OOM : ER_ERR_CUDA, "batch allocation failed");
  }
  b->allocs.push_back(*p);
  b->device_bytes += (int64_t)bytes;
  return ER_OK;
}

void bfree(er_batch* b, void* p) {
  if (!p) return;
  auto it = std::find(b->allocs.begin(), b->allocs.end(), p);
  if (it != b->allocs.end()) b->allocs.erase(it);
  cudaFree(p);
}

// ---- fix-up kernels: rebase indices of one scene's part of a merged array

__device__ __forceinline__ int32_t rebase_child(int32_t c, int32_t node_base, int32_t slot_base) {
  if (c == kEmpty) return c;
  if (c >= 0) return c + node_base;
  uint32_t u = (uint32_t)c;
  return (int32_t)((u & ~kLeafFirstMask) | ((u & kLeafFirstMask) + (uint32_t)slot_base));
}

__global__ void k_fix_nodes(float4* nodes, int64_t n, int32_t node_base, int32_t slot_base) {
  int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  float4 c = nodes[8 * i + 6];
  c.x = __int_as_float(rebase_child(__float_as_int(c.x), node_base, slot_base));
  c.y = __int_as_float(rebase_child(__float_as_int(c.y), node_base, slot_base));
  c.z = __int_as_float(rebase_child(__float_as_int(c.z), node_base, slot_base));
  c.w = __int_as_float(rebase_child(__float_as_int(c.w), node_base, slot_base));
  nodes[8 * i + 6] = c;
}

// QNode as 4 uint4: children in [2].z, [2].w, [3].x, [3].y
__global__ void k_fix_qnodes(uint4* q, int64_t n, int32_t node_base, int32_t slot_base) {
  int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  uint4 a = q[4 * i + 2], b = q[4 * i + 3];
  a.z = (uint32_t)rebase_child((int32_t)a.z, node_base, slot_base);
  a.w = (uint32_t)rebase_child((int32_t)a.w, node_base, slot_base);
  b.x = (uint32_t)rebase_child((int32_t)b.x, node_base, slot_base);
  b.y = (uint32_t)rebase_child((int32_t)b.y, node_base, slot_base);
  q[4 * i + 2] = a;
  q[4 * i + 3] = b;
}

// material id in the w lane of each slot's third vertex
__global__ void k_fix_tri_mat(float4* tv, int64_t nslots, int32_t mat_base) {
  int64_t s = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (s >= nslots) return;
  float4 v = tv[3 * s + 2];
  v.w = __int_as_float(__float_as_int(v.w) + mat_base);
  tv[3 * s + 2] = v;
}

__global__ void k_fix_mats(DevMaterial* m, int32_t n, int32_t tex_base) {
  int32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  DevMaterial& q = m[i];
  if (q.albedo_tex >= 0) q.albedo_tex += tex_base;
  if (q.emission_tex >= 0) q.emission_tex += tex_base;
  if (q.roughness_tex >= 0) q.roughness_tex += tex_base;
  if (q.metallic_tex >= 0) q.metallic_tex += tex_base;
  if (q.normal_tex >= 0) q.normal_tex += tex_base;
}

__global__ void k_fix_texs(DevTex* t, int32_t n, int64_t texel_base) {
  int32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  t[i].offset += texel_base;
}

unsigned blocks(int64_t n, int bs = 256) { return (unsigned)((n + bs - 1) / bs); }

er_status check_err(er_batch* b) {
  uint32_t w = 0;
  ER_CUDA(cudaMemcpyAsync(&w, b->err_word, 4, cudaMemcpyDeviceToHost, b->stream));
  ER_CUDA(cudaStreamSynchronize(b->stream));
  if (w == 0) return ER_OK;
  ER_CUDA(cudaMemsetAsync(b->err_word, 0, 4, b->stream));
  if (w & 2u) return fail(ER_ERR_TIMEOUT, "a bounded device wait gave up");
  return fail(ER_ERR_DEVICE_CHECK, "device bounds check fired (error word " + std::to_string(w) + ")");
}

void drop_graph(er_batch* b) {
  if (b->graph) cudaGraphExecDestroy(b->graph);
  b->graph = nullptr;
}

void drop_plan(er_batch* b) {
  drop_graph(b);
  bfree(b, b->d_segs);
  b->d_segs = nullptr;
  b->waves.clear();
  b->plan_budget = 0;
}

void drop_jobs(er_batch* b) {
  drop_plan(b);
  for (Film& F : b->films) {
    bfree(b, F.beauty);
    bfree(b, F.sum);
    bfree(b, F.samples);
    bfree(b, F.pathcount);
  }
  b->films.clear();
  bfree(b, b->d_jobs);
  b->d_jobs = nullptr;
  b->jobs.clear();
  b->has_tuned = false;
}

int32_t job_npix(const er_batch_job& j) { return j.camera.x_res * j.camera.y_res; }
int32_t job_depth(const er_batch_job& j) { return j.max_depth > 0 ? j.max_depth : 5; }

// Cuts every job into sample slices that fill waves of `budget` paths, in
// job order; each wave holds at most one slice per job and a job's slices
// follow its sample order.
er_status make_plan(er_batch* b, int64_t budget) {
  if (b->plan_budget == budget && b->d_segs) return ER_OK;
  drop_plan(b);
  const size_t nj = b->jobs.size();
  std::vector<int32_t> next(nj, 0);
  std::vector<BatchSeg> segs;
  int64_t cap = 0;
  while (true) {
    BatchWave w{(int32_t)segs.size(), 0, 0, 0, 0};
    int64_t paths = 0;
    for (size_t j = 0; j < nj; j++) {
      const er_batch_job& J = b->jobs[j];
      const int32_t npix = job_npix(J);
      const int32_t rem = J.spp - next[j];
      if (rem <= 0) continue;
      const int64_t fit = (budget - paths) / npix;
      if (fit <= 0) continue;
      const int32_t sw = (int32_t)std::min<int64_t>(rem, fit);
      BatchSeg g{};
      g.path_base = (int32_t)paths;
      g.pix_base = w.n_acc;
      g.job = (int32_t)j;
      g.P.W = J.camera.x_res;
      g.P.H = J.camera.y_res;
      g.P.npix = npix;
      g.P.spp_wave = sw;
      g.P.sample_base = J.sample_begin + next[j];
      g.P.max_depth = job_depth(J);
      g.P.k0 = (uint32_t)J.seed;
      g.P.k1 = (uint32_t)(J.seed >> 32);
      g.P.flags = J.flags;
      segs.push_back(g);
      paths += (int64_t)sw * npix;
      w.n_acc += npix;
      w.n_segs++;
      w.max_depth = std::max(w.max_depth, g.P.max_depth);
      next[j] += sw;
    }
    if (w.n_segs == 0) break;
    w.n_paths = (int32_t)paths;
    cap = std::max(cap, paths);
    b->waves.push_back(w);
  }
  if (!segs.empty()) {
    er_status st = balloc(b, (void**)&b->d_segs, segs.size() * sizeof(BatchSeg));
    if (st != ER_OK) return st;
    ER_CUDA(cudaMemcpyAsync(b->d_segs, segs.data(), segs.size() * sizeof(BatchSeg), cudaMemcpyHostToDevice,
                            b->stream));
    ER_CUDA(cudaStreamSynchronize(b->stream));
  }
  if (!b->wave || b->wave_cap < cap) {
    drop_graph(b);
    wave_destroy(b->wave);
    wave_destroy(b->pair.w2);
    b->wave = nullptr;
    b->pair.w2 = nullptr;
    b->wave_cap = 0;
    er_status st = wave_create(std::max<int64_t>(cap, 1), b->d_stats, &b->wave);
    if (st != ER_OK) return st;
    b->wave_cap = cap;
  }
  b->plan_budget = budget;
  return ER_OK;
}

er_batch_tuning default_tuning() {
  er_batch_tuning t{};
  t.wave_paths = kDefaultWavePaths;
  t.use_graph = 1;
  return t;
}

bool same_tuning(const er_batch_tuning& a, const er_batch_tuning& b) {
  return a.wave_paths == b.wave_paths && a.trace_blocks_per_sm == b.trace_blocks_per_sm &&
         a.shade_blocks_per_sm == b.shade_blocks_per_sm && a.split_trace == b.split_trace &&
         a.one_stream == b.one_stream;
}

// The second pipeline's buffers (the first's capacity), stream and events.
er_status ensure_pair(er_batch* b) {
  BatchPair& p = b->pair;
  if (!p.w2) {
    drop_graph(b);
    er_status st = wave_create(std::max<int64_t>(b->wave_cap, 1), b->d_stats, &p.w2);
    if (st != ER_OK) return st;
  }
  if (!p.s2) ER_CUDA(cudaStreamCreateWithFlags(&p.s2, cudaStreamNonBlocking));
  for (cudaEvent_t* e : {&p.ev_fork, &p.ev_join, &p.ev_acc[0], &p.ev_acc[1]})
    if (!*e) ER_CUDA(cudaEventCreateWithFlags(e, cudaEventDisableTiming));
  return ER_OK;
}

int32_t max_job_npix(const er_batch* b) {
  int32_t m = 1;
  for (const er_batch_job& j : b->jobs) m = std::max(m, job_npix(j));
  return m;
}

// The effective wave budget of a tuning: at least one full image of the
// largest job.
int64_t wave_budget(const er_batch* b, const er_batch_tuning& t) {
  int64_t w = t.wave_paths > 0 ? t.wave_paths : kDefaultWavePaths;
  return std::max<int64_t>(w, max_job_npix(b));
}

er_status enqueue_render(er_batch* b, const er_batch_tuning& t, int64_t* launches) {
  for (const Film& F : b->films) {
    er_status st = film_clear(F, b->stream);
    if (st != ER_OK) return st;
  }
  BatchSchedule sch;
  sch.trace_blocks_per_sm = t.trace_blocks_per_sm;
  sch.shade_blocks_per_sm = t.shade_blocks_per_sm;
  sch.split_trace = t.split_trace != 0;
  int64_t nl = 0;
  const BatchPair* pair = nullptr;
  if (!t.one_stream && b->waves.size() >= 2) {
    if (!b->pair.w2) return fail(ER_ERR_INVALID_ARG, "second wave pipeline missing");
    pair = &b->pair;
  }
  er_status st = batch_launch(b->dev, b->wave, b->d_segs, b->d_jobs, b->waves, sch, b->num_sms, b->err_word,
                              b->stream, &nl, pair);
  if (launches) *launches = nl + (int64_t)b->films.size();
  return st;
}

// Renders every job once with tuning t; ms = device time of the render.
er_status render_once(er_batch* b, const er_batch_tuning& t, double* ms, int64_t* launches) {
  er_status st = make_plan(b, wave_budget(b, t));
  if (st != ER_OK) return st;
  // (allocations happen here, outside any stream capture)
  if (!t.one_stream && b->waves.size() >= 2 && (st = ensure_pair(b)) != ER_OK) return st;
  int64_t nl = 0;
  if (t.use_graph) {
    if (!b->graph || !same_tuning(b->graph_tuning, t)) {
      drop_graph(b);
      cudaGraph_t g = nullptr;
      ER_CUDA(cudaStreamBeginCapture(b->stream, cudaStreamCaptureModeThreadLocal));
      st = enqueue_render(b, t, &b->graph_launches);
      cudaError_t ce = cudaStreamEndCapture(b->stream, &g);
      if (st != ER_OK) {
        if (g) cudaGraphDestroy(g);
        return st;
      }
      if (ce != cudaSuccess) return cuda_fail(ce, "cudaStreamEndCapture");
      ce = cudaGraphInstantiate(&b->graph, g, 0);
      cudaGraphDestroy(g);
      if (ce != cudaSuccess) {
        b->graph = nullptr;
        return cuda_fail(ce, "cudaGraphInstantiate");
      }
      b->graph_tuning = t;
    }
    ER_CUDA(cudaEventRecord(b->ev0, b->stream));
    ER_CUDA(cudaGraphLaunch(b->graph, b->stream));
    ER_CUDA(cudaEventRecord(b->ev1, b->stream));
    nl = b->graph_launches;
  } else {
    ER_CUDA(cudaEventRecord(b->ev0, b->stream));
    if ((st = enqueue_render(b, t, &nl)) != ER_OK) return st;
    ER_CUDA(cudaEventRecord(b->ev1, b->stream));
  }
  ER_CUDA(cudaEventSynchronize(b->ev1));
  if ((st = check_err(b)) != ER_OK) return st;
  float f = 0;
  ER_CUDA(cudaEventElapsedTime(&f, b->ev0, b->ev1));
  if (ms) *ms = f;
  if (launches) *launches = nl;
  return ER_OK;
}

}  // namespace

extern "C" er_status er_batch_create(er_scene* const* scenes, int32_t n_scenes, const er_scene_opts* opts,
                                     er_batch** out) {
  return guarded("er_batch_create", [&]() -> er_status {
    if (!out) return fail(ER_ERR_INVALID_ARG, "out is NULL");
    *out = nullptr;
    if (!scenes || n_scenes <= 0) return fail(ER_ERR_INVALID_ARG, "no scenes");
    for (int32_t i = 0; i < n_scenes; i++)
      if (!scenes[i]) return fail(ER_ERR_INVALID_ARG, "scene is NULL");
    const int device = scenes[0]->device;
    for (int32_t i = 0; i < n_scenes; i++)
      if (scenes[i]->device != device) return fail(ER_ERR_INVALID_ARG, "scenes live on different devices");
    const bool q8 = opts && opts->bvh_format == ER_BVH_Q8;
    if (opts && opts->bvh_format != ER_BVH_FP32 && opts->bvh_format != ER_BVH_Q8)
      return fail(ER_ERR_INVALID_ARG, "bvh_format");
    if (q8)
      for (int32_t i = 0; i < n_scenes; i++)
        if (!scenes[i]->dev.qnodes) return fail(ER_ERR_INVALID_ARG, "ER_BVH_Q8 batch needs scenes built with ER_BVH_Q8");
    // sizes of each scene's arrays (a scene without triangles still has one slot)
    int64_t nodes = 0, slots = 0, texels = 0;
    int64_t mats = 0, texs = 0;
    bool any_tangents = false;
    for (int32_t i = 0; i < n_scenes; i++) {
      const DevScene& S = scenes[i]->dev;
      nodes += S.n_nodes;
      slots += std::max<int64_t>(S.n_tris, 1);
      mats += std::max(S.n_mats, 1);
      texs += std::max(S.n_texs, 1);
      texels += scenes[i]->texel_count;
      any_tangents |= S.tri_t != nullptr;
    }
    if (slots > kMaxTris) return fail(ER_ERR_UNSUPPORTED, "merged triangle count exceeds the leaf encoding");
    if (nodes > 0x7FFFFFFF) return fail(ER_ERR_UNSUPPORTED, "merged node count exceeds int32");
    ER_CUDA(cudaSetDevice(device));

    er_batch* b = new er_batch();
    FreeOnUnwind<er_batch> unwind{b, er_batch_free};
    b->device = device;
    auto bail = [&](er_status e) {
      er_batch_free(b);
      return e;
    };
    cudaDeviceProp prop;
    cudaError_t ce = cudaGetDeviceProperties(&prop, device);
    if (ce != cudaSuccess) return bail(cuda_fail(ce, "cudaGetDeviceProperties"));
    b->num_sms = prop.multiProcessorCount;
    if (opts && opts->stream) {
      b->stream = (cudaStream_t)opts->stream;
    } else {
      ce = cudaStreamCreateWithFlags(&b->stream, cudaStreamNonBlocking);
      if (ce != cudaSuccess) return bail(cuda_fail(ce, "cudaStreamCreate"));
      b->own_stream = true;
    }
    cudaEventCreate(&b->ev0);
    cudaEventCreate(&b->ev1);
    b->scenes.assign(scenes, scenes + n_scenes);
    for (er_scene* s : b->scenes) cudaStreamSynchronize(s->stream);

    er_status st;
    void *p_nodes, *p_q = nullptr, *p_tv, *p_tn, *p_tuv, *p_tt = nullptr, *p_mats, *p_texs, *p_texels, *p_err;
    if ((st = balloc(b, &p_nodes, (size_t)nodes * 128)) != ER_OK) return bail(st);
    if (q8 && (st = balloc(b, &p_q, (size_t)nodes * 64)) != ER_OK) return bail(st);
    if ((st = balloc(b, &p_tv, (size_t)slots * 48)) != ER_OK) return bail(st);
    if ((st = balloc(b, &p_tn, (size_t)slots * 48)) != ER_OK) return bail(st);
    if ((st = balloc(b, &p_tuv, (size_t)slots * 24)) != ER_OK) return bail(st);
    if (any_tangents && (st = balloc(b, &p_tt, (size_t)slots * 48)) != ER_OK) return bail(st);
    if ((st = balloc(b, &p_mats, (size_t)mats * sizeof(DevMaterial))) != ER_OK) return bail(st);
    if ((st = balloc(b, &p_texs, (size_t)texs * sizeof(DevTex))) != ER_OK) return bail(st);
    if ((st = balloc(b, &p_texels, (size_t)std::max<int64_t>(texels, 1) * 16)) != ER_OK) return bail(st);
    if ((st = balloc(b, &p_err, 256)) != ER_OK) return bail(st);
    ce = cudaMemsetAsync(p_err, 0, 256, b->stream);
    if (ce != cudaSuccess) return bail(cuda_fail(ce, "cudaMemsetAsync"));
    if (p_tt) {
      ce = cudaMemsetAsync(p_tt, 0, (size_t)slots * 48, b->stream);
      if (ce != cudaSuccess) return bail(cuda_fail(ce, "cudaMemsetAsync"));
    }

    int64_t nb = 0, sb = 0, tb = 0;
    int32_t mb = 0, xb = 0;
    float eps = 0;
    auto cp = [&](void* dst, const void* src, size_t bytes) {
      return bytes ? cudaMemcpyAsync(dst, src, bytes, cudaMemcpyDeviceToDevice, b->stream) : cudaSuccess;
    };
    for (int32_t i = 0; i < n_scenes; i++) {
      const er_scene* sc = b->scenes[i];
      const DevScene& S = sc->dev;
      const int64_t ns = std::max<int64_t>(S.n_tris, 1);
      const int32_t nm = std::max(S.n_mats, 1), nt = std::max(S.n_texs, 1);
      char* c_nodes = (char*)p_nodes + nb * 128;
      char* c_tv = (char*)p_tv + sb * 48;
      char* c_mats = (char*)p_mats + (size_t)mb * sizeof(DevMaterial);
      char* c_texs = (char*)p_texs + (size_t)xb * sizeof(DevTex);
      cudaError_t e = cudaSuccess;
      if (e == cudaSuccess) e = cp(c_nodes, S.nodes, (size_t)S.n_nodes * 128);
      if (e == cudaSuccess && q8) e = cp((char*)p_q + nb * 64, S.qnodes, (size_t)S.n_nodes * 64);
      if (e == cudaSuccess) e = cp(c_tv, S.tri_v, (size_t)ns * 48);
      if (e == cudaSuccess) e = cp((char*)p_tn + sb * 48, S.tri_n, (size_t)ns * 48);
      if (e == cudaSuccess) e = cp((char*)p_tuv + sb * 24, S.tri_uv, (size_t)ns * 24);
      if (e == cudaSuccess && S.tri_t) e = cp((char*)p_tt + sb * 48, S.tri_t, (size_t)ns * 48);
      if (e == cudaSuccess) e = cp(c_mats, S.mats, (size_t)nm * sizeof(DevMaterial));
      if (e == cudaSuccess) e = cp(c_texs, S.texs, (size_t)nt * sizeof(DevTex));
      if (e == cudaSuccess) e = cp((char*)p_texels + tb * 16, S.texels, (size_t)sc->texel_count * 16);
      if (e != cudaSuccess) return bail(cuda_fail(e, "batch merge copy"));
      k_fix_nodes<<<blocks(S.n_nodes), 256, 0, b->stream>>>((float4*)c_nodes, S.n_nodes, (int32_t)nb, (int32_t)sb);
      if (q8) k_fix_qnodes<<<blocks(S.n_nodes), 256, 0, b->stream>>>((uint4*)((char*)p_q + nb * 64), S.n_nodes,
                                                                      (int32_t)nb, (int32_t)sb);
      k_fix_tri_mat<<<blocks(ns), 256, 0, b->stream>>>((float4*)c_tv, ns, mb);
      k_fix_mats<<<blocks(nm), 256, 0, b->stream>>>((DevMaterial*)c_mats, nm, xb);
      k_fix_texs<<<blocks(nt), 256, 0, b->stream>>>((DevTex*)c_texs, nt, tb);
      ce = cudaGetLastError();
      if (ce != cudaSuccess) return bail(cuda_fail(ce, "batch fix-up"));
      b->root.push_back((int32_t)nb);
      b->texel_base.push_back(tb);
      eps = std::max(eps, S.scene_eps);
      nb += S.n_nodes;
      sb += ns;
      mb += nm;
      xb += nt;
      tb += sc->texel_count;
    }
    ce = cudaStreamSynchronize(b->stream);
    if (ce != cudaSuccess) return bail(cuda_fail(ce, "batch merge"));

    DevScene& M = b->dev;
    M = b->scenes[0]->dev;  // per-job parts (env, lights, camera) come from the job table
    M.nodes = (const float4*)p_nodes;
    M.qnodes = (const uint4*)p_q;
    M.tri_v = (const float4*)p_tv;
    M.tri_n = (const float4*)p_tn;
    M.tri_uv = (const float2*)p_tuv;
    M.tri_t = (const float4*)p_tt;
    M.mats = (const DevMaterial*)p_mats;
    M.texs = (const DevTex*)p_texs;
    M.texels = (const float4*)p_texels;
    M.env.offset += b->texel_base[0];
    M.n_mats = (int32_t)mats;
    M.n_texs = (int32_t)texs;
    M.n_tris = slots;
    M.n_nodes = nodes;
    M.scene_eps = eps;
    M.use_q8 = q8;
    b->err_word = (uint32_t*)p_err;
    b->d_stats = (unsigned long long*)((char*)p_err + 64);
    // occupancy queries of the batch kernels, outside any stream capture
    std::vector<BatchWave> none;
    if ((st = batch_launch(M, nullptr, nullptr, nullptr, none, BatchSchedule{}, b->num_sms, b->err_word, b->stream,
                           nullptr)) != ER_OK)
      return bail(st);
    *out = b;
    return ER_OK;
  });
}

extern "C" er_status er_batch_set_jobs(er_batch* b, const er_batch_job* jobs, int32_t n_jobs) {
  return guarded("er_batch_set_jobs", [&]() -> er_status {
    if (!b) return fail(ER_ERR_INVALID_ARG, "batch is NULL");
    if (n_jobs < 0 || (n_jobs > 0 && !jobs)) return fail(ER_ERR_INVALID_ARG, "bad job list");
    for (int32_t j = 0; j < n_jobs; j++) {
      const er_batch_job& J = jobs[j];
      if (J.scene < 0 || J.scene >= (int32_t)b->scenes.size()) return fail(ER_ERR_INVALID_ARG, "job scene out of range");
      er_status cs = validate_camera(J.camera);
      if (cs != ER_OK) return fail(cs, "job " + std::to_string(j) + ": " + er_last_error());
      if (J.spp < 0 || J.sample_begin < 0 || J.max_depth < 0 || J.max_depth > 64 ||
          (int64_t)J.sample_begin + J.spp > INT32_MAX)
        return fail(ER_ERR_INVALID_ARG, "job options out of range");
      if (J.flags & ~(uint32_t)(ER_RENDER_ENV_ALIAS | ER_RENDER_ACCUM_FP64))
        return fail(ER_ERR_INVALID_ARG, "job flags: only ER_RENDER_ENV_ALIAS and ER_RENDER_ACCUM_FP64");
    }
    ER_CUDA(cudaSetDevice(b->device));
    drop_jobs(b);
    er_status st;
    std::vector<BatchJobDev> table((size_t)n_jobs);
    b->films.resize((size_t)n_jobs);
    for (int32_t j = 0; j < n_jobs; j++) {
      const er_batch_job& J = jobs[j];
      er_scene* sc = b->scenes[(size_t)J.scene];
      if ((J.flags & ER_RENDER_ENV_ALIAS) && (st = build_env_alias(sc)) != ER_OK) return st;
      if ((st = build_env_lut(sc)) != ER_OK) return st;
      Film& F = b->films[(size_t)j];
      F.w = J.camera.x_res;
      F.h = J.camera.y_res;
      const size_t np = (size_t)F.w * F.h;
      if ((st = balloc(b, (void**)&F.beauty, np * sizeof(float4))) != ER_OK) return st;
      if ((st = balloc(b, (void**)&F.samples, np * 4)) != ER_OK) return st;
      if ((st = balloc(b, (void**)&F.pathcount, np * 4)) != ER_OK) return st;
      if ((J.flags & ER_RENDER_ACCUM_FP64) && (st = balloc(b, (void**)&F.sum, np * 3 * sizeof(double))) != ER_OK)
        return st;
      BatchJobDev& D = table[(size_t)j];
      std::memset(&D, 0, sizeof D);
      const DevScene& S = sc->dev;
      D.env = S.env;
      D.env.offset += b->texel_base[(size_t)J.scene];
      D.cdf = S.cdf;
      D.alias_idx = S.alias_idx;
      D.alias_thresh = S.alias_thresh;
      D.env_lut = S.env_lut;
      D.lights = S.lights;
      D.radiance_sum = S.radiance_sum;
      D.n_lights = S.n_lights;
      D.root = b->root[(size_t)J.scene];
      D.scene_eps = S.scene_eps;
      D.cam = make_dev_camera(J.camera);
      D.film = F;
    }
    b->jobs.assign(jobs, jobs + n_jobs);
    if (n_jobs > 0) {
      if ((st = balloc(b, (void**)&b->d_jobs, table.size() * sizeof(BatchJobDev))) != ER_OK) return st;
      ER_CUDA(cudaMemcpyAsync(b->d_jobs, table.data(), table.size() * sizeof(BatchJobDev), cudaMemcpyHostToDevice,
                              b->stream));
      ER_CUDA(cudaStreamSynchronize(b->stream));
    }
    return ER_OK;
  });
}

extern "C" er_status er_batch_render(er_batch* b, const er_batch_tuning* tuning, er_render_stats* stats) {
  return guarded("er_batch_render", [&]() -> er_status {
    if (!b) return fail(ER_ERR_INVALID_ARG, "batch is NULL");
    ER_CUDA(cudaSetDevice(b->device));
    if (b->jobs.empty()) return fail(ER_ERR_INVALID_ARG, "no jobs (er_batch_set_jobs)");
    er_batch_tuning t = tuning ? *tuning : (b->has_tuned ? b->tuned : default_tuning());
    if (t.wave_paths < 0 || t.trace_blocks_per_sm < 0 || t.shade_blocks_per_sm < 0)
      return fail(ER_ERR_INVALID_ARG, "tuning out of range");
    unsigned long long st0[8], st1[8];
    ER_CUDA(cudaMemcpyAsync(st0, b->d_stats, sizeof st0, cudaMemcpyDeviceToHost, b->stream));
    ER_CUDA(cudaStreamSynchronize(b->stream));
    double ms = 0;
    int64_t nl = 0;
    er_status st = render_once(b, t, &ms, &nl);
    if (st != ER_OK) return st;
    if (stats) {
      ER_CUDA(cudaMemcpy(st1, b->d_stats, sizeof st1, cudaMemcpyDeviceToHost));
      std::memset(stats, 0, sizeof *stats);
      stats->ms = ms;
      for (const er_batch_job& J : b->jobs) stats->samples += (int64_t)J.spp * job_npix(J);
      stats->rays_closest = (int64_t)(st1[0] - st0[0]);
      stats->rays_shadow = (int64_t)(st1[1] - st0[1]);
      stats->path_vertices = (int64_t)(st1[6] - st0[6]);
      stats->kernel_launches = nl;
    }
    return ER_OK;
  });
}

extern "C" er_status er_batch_read(er_batch* b, int32_t job, uint32_t flags, float* beauty, uint32_t* samples,
                                   uint32_t* pathcount) {
  return guarded("er_batch_read", [&]() -> er_status {
    if (!b) return fail(ER_ERR_INVALID_ARG, "batch is NULL");
    if (job < 0 || job >= (int32_t)b->films.size()) return fail(ER_ERR_INVALID_ARG, "job out of range");
    ER_CUDA(cudaSetDevice(b->device));
    const Film& F = b->films[(size_t)job];
    const size_t np = (size_t)F.w * F.h;
    const cudaMemcpyKind k = (flags & ER_RENDER_DEVICE_OUT) ? cudaMemcpyDeviceToDevice : cudaMemcpyDeviceToHost;
    if (beauty) ER_CUDA(cudaMemcpyAsync(beauty, F.beauty, np * sizeof(float4), k, b->stream));
    if (samples) ER_CUDA(cudaMemcpyAsync(samples, F.samples, np * 4, k, b->stream));
    if (pathcount) ER_CUDA(cudaMemcpyAsync(pathcount, F.pathcount, np * 4, k, b->stream));
    ER_CUDA(cudaStreamSynchronize(b->stream));
    return ER_OK;
  });
}

// Coordinate descent over the schedule knobs, each candidate timed as the
// best of `reps` graph replays of the current jobs.
extern "C" er_status er_batch_autotune(er_batch* b, int32_t reps, er_batch_tuning* best) {
  return guarded("er_batch_autotune", [&]() -> er_status {
    if (!b) return fail(ER_ERR_INVALID_ARG, "batch is NULL");
    ER_CUDA(cudaSetDevice(b->device));
    if (b->jobs.empty()) return fail(ER_ERR_INVALID_ARG, "no jobs (er_batch_set_jobs)");
    reps = std::max(1, reps);
    auto measure = [&](const er_batch_tuning& t, double* out) -> er_status {
      double m = 1e300;
      for (int32_t r = 0; r <= reps; r++) {  // first run builds the graph
        double ms = 0;
        er_status st = render_once(b, t, &ms, nullptr);
        if (st != ER_OK) return st;
        if (r > 0) m = std::min(m, ms);
      }
      *out = m;
      return ER_OK;
    };
    er_batch_tuning cur = default_tuning();
    double cur_ms = 0;
    er_status st = measure(cur, &cur_ms);
    if (st != ER_OK) return st;
    auto try_knob = [&](auto set, std::initializer_list<int32_t> values) -> er_status {
      er_batch_tuning bestt = cur;
      double best_ms = cur_ms;
      for (int32_t v : values) {
        er_batch_tuning t = cur;
        set(t, v);
        if (same_tuning(t, cur)) continue;
        double ms = 0;
        er_status e = measure(t, &ms);
        if (e != ER_OK) return e;
        if (ms < best_ms) {
          best_ms = ms;
          bestt = t;
        }
      }
      cur = bestt;
      cur_ms = best_ms;
      return ER_OK;
    };
    if ((st = try_knob([](er_batch_tuning& t, int32_t v) { t.wave_paths = v; },
                       {1 << 20, 1 << 21, 1 << 22, 1 << 23, 1 << 24})) != ER_OK)
      return st;
    if ((st = try_knob([](er_batch_tuning& t, int32_t v) { t.trace_blocks_per_sm = v; }, {0, 4, 5, 6})) != ER_OK)
      return st;
    if ((st = try_knob([](er_batch_tuning& t, int32_t v) { t.shade_blocks_per_sm = v; }, {0, 4, 8})) != ER_OK)
      return st;
    if ((st = try_knob([](er_batch_tuning& t, int32_t v) { t.split_trace = v; }, {0, 1})) != ER_OK) return st;
    if ((st = try_knob([](er_batch_tuning& t, int32_t v) { t.one_stream = v; }, {0, 1})) != ER_OK) return st;
    b->tuned = cur;
    b->has_tuned = true;
    if (best) *best = cur;
    return ER_OK;
  });
}

extern "C" er_status er_batch_info(const er_batch* b, int32_t* n_waves, int64_t* device_bytes) {
  return guarded("er_batch_info", [&]() -> er_status {
    if (!b) return fail(ER_ERR_INVALID_ARG, "batch is NULL");
    if (n_waves) *n_waves = (int32_t)b->waves.size();
    if (device_bytes) *device_bytes = b->device_bytes;
    return ER_OK;
  });
}

extern "C" er_status er_batch_free(er_batch* b) {
  return guarded("er_batch_free", [&]() -> er_status {
    if (!b) return ER_OK;
    cudaSetDevice(b->device);
    if (b->stream) cudaStreamSynchronize(b->stream);
    drop_graph(b);
    if (b->pair.s2) cudaStreamSynchronize(b->pair.s2);
    wave_destroy(b->wave);
    wave_destroy(b->pair.w2);
    for (void* p : b->allocs) cudaFree(p);
    if (b->pair.s2) cudaStreamDestroy(b->pair.s2);
    for (cudaEvent_t e : {b->pair.ev_fork, b->pair.ev_join, b->pair.ev_acc[0], b->pair.ev_acc[1]})
      if (e) cudaEventDestroy(e);
    if (b->ev0) cudaEventDestroy(b->ev0);
    if (b->ev1) cudaEventDestroy(b->ev1);
    if (b->own_stream && b->stream) cudaStreamDestroy(b->stream);
    delete b;
    return ER_OK;
  });
}
