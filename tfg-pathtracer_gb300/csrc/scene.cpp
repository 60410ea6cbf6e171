// Scene handle: validation, BVH build, device layout and upload.
//
// Replaces renderSetup (kernel.cu:566-661): instead of ~40 cudaMemcpy calls
// with device pointer fix-ups into process globals, every array is laid out
// on the host once (leaf order for the triangle data) and uploaded into
// allocations owned by the handle.
#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstring>

#include "internal.h"

namespace er {

er_status dev_alloc(er_scene* s, void** p, size_t bytes) {
  *p = nullptr;
  if (bytes == 0) bytes = 16;
  cudaError_t e = cudaMalloc(p, bytes);
  if (e != cudaSuccess) {
    *p = nullptr;
    cudaGetLastError();
    return fail(e == cudaErrorMemoryAllocation ? ER_ERR_OOM : ER_ERR_CUDA,
                std::string("cudaMalloc(") + std::to_string(bytes) + "): " + cudaGetErrorString(e));
  }
  s->allocs.push_back(*p);
  s->device_bytes += (int64_t)bytes;
  return ER_OK;
}

er_status upload(er_scene* s, void** p, const void* host, size_t bytes) {
  er_status st = dev_alloc(s, p, bytes);
  if (st != ER_OK) return st;
  if (bytes) ER_CUDA(cudaMemcpyAsync(*p, host, bytes, cudaMemcpyHostToDevice, s->stream));
  return ER_OK;
}

DevCamera make_dev_camera(const er_camera& c) {
  DevCamera d;
  d.x_res = c.x_res;
  d.y_res = c.y_res;
  d.focal_length = c.focal_length;
  d.sensor_width = c.sensor_width;
  d.sensor_height = c.sensor_height;
  d.aperture = c.aperture;
  d.focus_distance = c.focus_distance;
  d.px = c.position[0];
  d.py = c.position[1];
  d.pz = c.position[2];
  // kernel.cu:299-306: rotation *= (float)(PI/180.0), then cos/sin of each
  // component.  The same libm calls the host oracle makes per ray.
  volatile float k = (float)((double)3.14159265358979323846f / 180.0);
  float rx = c.rotation[0] * k, ry = c.rotation[1] * k, rz = c.rotation[2] * k;
  d.cx = cosf(rx); d.sx = sinf(rx);
  d.cy = cosf(ry); d.sy = sinf(ry);
  d.cz = cosf(rz); d.sz = sinf(rz);
  d.bokeh = c.bokeh;
  return d;
}

er_status check_device_error(er_scene* s) {
  uint32_t w = 0;
  ER_CUDA(cudaMemcpyAsync(&w, s->err_word, 4, cudaMemcpyDeviceToHost, s->stream));
  ER_CUDA(cudaStreamSynchronize(s->stream));
  if (w == 0) return ER_OK;
  uint32_t z = 0;
  ER_CUDA(cudaMemcpyAsync(s->err_word, &z, 4, cudaMemcpyHostToDevice, s->stream));
  if (w & 2u) return fail(ER_ERR_TIMEOUT, "a bounded device wait gave up");
  return fail(ER_ERR_DEVICE_CHECK, "device bounds check fired (error word " + std::to_string(w) + ")");
}

namespace {

bool finite3(const float* p) { return std::isfinite(p[0]) && std::isfinite(p[1]) && std::isfinite(p[2]); }

}  // namespace

er_status validate_camera(const er_camera& c) {
  if (c.x_res <= 0 || c.y_res <= 0 || (int64_t)c.x_res * c.y_res > ((int64_t)1 << 28))
    return fail(ER_ERR_INVALID_ARG, "camera resolution out of range");
  float cf[] = {c.focal_length, c.sensor_width, c.sensor_height, c.aperture, c.focus_distance};
  for (float v : cf)
    if (!std::isfinite(v)) return fail(ER_ERR_INVALID_ARG, "camera parameter is not finite");
  if (!finite3(c.position) || !finite3(c.rotation)) return fail(ER_ERR_INVALID_ARG, "camera pose is not finite");
  return ER_OK;
}

namespace {

er_status validate_texture(const er_texture& t, const char* what) {
  if (t.width <= 0 || t.height <= 0 || !t.data)
    return fail(ER_ERR_INVALID_ARG, std::string(what) + ": empty texture");
  if ((int64_t)t.width * t.height > ((int64_t)1 << 30))
    return fail(ER_ERR_INVALID_ARG, std::string(what) + ": texture too large");
  return ER_OK;
}

er_status validate(const er_scene_desc* d) {
  if (!d) return fail(ER_ERR_INVALID_ARG, "desc is NULL");
  er_status cs = validate_camera(d->camera);
  if (cs != ER_OK) return cs;
  if (d->tri_count < 0 || d->tri_count > kMaxTris - kMaxLeafTris)
    return fail(ER_ERR_INVALID_ARG, "tri_count out of range");
  if (d->tri_count > 0 && !d->positions) return fail(ER_ERR_INVALID_ARG, "positions is NULL");
  for (int64_t i = 0; i < 9 * d->tri_count; i += 3)
    if (!finite3(d->positions + i)) return fail(ER_ERR_INVALID_ARG, "non-finite vertex position");
  if (d->tri_count > 0 && d->material_count <= 0) return fail(ER_ERR_INVALID_ARG, "no materials");
  if (d->object_count < 0 || d->material_count < 0 || d->texture_count < 0 || d->light_count < 0)
    return fail(ER_ERR_INVALID_ARG, "negative count");
  if (d->tri_object) {
    for (int64_t i = 0; i < d->tri_count; i++)
      if (d->tri_object[i] < 0 || d->tri_object[i] >= std::max(1, d->object_count))
        return fail(ER_ERR_INVALID_ARG, "tri_object index out of range");
  }
  if (d->object_count > 0 && !d->object_material) return fail(ER_ERR_INVALID_ARG, "object_material is NULL");
  if (d->material_count > 0 && !d->materials) return fail(ER_ERR_INVALID_ARG, "materials is NULL");
  if (d->texture_count > 0 && !d->textures) return fail(ER_ERR_INVALID_ARG, "textures is NULL");
  for (int32_t i = 0; i < d->object_count; i++)
    if (d->object_material[i] < 0 || d->object_material[i] >= d->material_count)
      return fail(ER_ERR_INVALID_ARG, "object_material index out of range");
  for (int32_t i = 0; i < d->material_count; i++) {
    const er_material& m = d->materials[i];
    int32_t ids[] = {m.albedo_tex, m.emission_tex, m.roughness_tex, m.metallic_tex, m.normal_tex};
    for (int32_t t : ids)
      if (t < -1 || t >= d->texture_count) return fail(ER_ERR_INVALID_ARG, "material texture id out of range");
  }
  for (int32_t i = 0; i < d->texture_count; i++) {
    er_status st = validate_texture(d->textures[i], "texture");
    if (st != ER_OK) return st;
  }
  if (d->light_count > 0 && !d->lights) return fail(ER_ERR_INVALID_ARG, "lights is NULL");
  return validate_texture(d->env, "environment");
}

}  // namespace

// HDRI.hpp:107-128 through Texture::getValueFromCoordinates (Texture.hpp:95-
// 112): FP32 running sums in row-major order.  Sequential on purpose: the
// reference's rounding of the running sum is part of the sampled
// distribution.
void hdri_cdf(const er_texture& t, std::vector<float>& cdf, float* radiance_sum) {
  auto f2i = [](float f) -> int32_t {  // device float->int semantics
    if (f != f) return 0;
    if (f >= 2147483648.0f) return INT32_MAX;
    if (f <= -2147483904.0f) return INT32_MIN;
    return (int32_t)f;
  };
  auto texel = [&](int32_t x, int32_t y) {
    x = f2i(t.x_tile * ((float)x + t.x_offset * (float)t.width)) % t.width;
    y = f2i(t.y_tile * ((float)y + t.y_offset * (float)t.height)) % t.height;
    if (x < 0) x += t.width;
    if (y < 0) y += t.height;
    const float* p = t.data + 3 * ((int64_t)y * t.width + x);
    return (p[0] + p[1]) + p[2];
  };
  int64_t n = (int64_t)t.width * t.height;
  cdf.assign((size_t)n + 1, 0.0f);
  float sum = 0;
  for (int32_t j = 0; j < t.height; j++)
    for (int32_t i = 0; i < t.width; i++) sum += texel(i, j);
  int64_t c = 0;
  for (int32_t j = 0; j < t.height; j++)
    for (int32_t i = 0; i < t.width; i++, c++) cdf[(size_t)c + 1] = cdf[(size_t)c] + texel(i, j) / sum;
  *radiance_sum = sum;
}

namespace {

void pack_texels(const er_texture& t, std::vector<float4>& pool, DevTex* dt) {
  dt->w = t.width;
  dt->h = t.height;
  dt->offset = (int64_t)pool.size();
  dt->x_tile = t.x_tile;
  dt->y_tile = t.y_tile;
  dt->x_offset = t.x_offset;
  dt->y_offset = t.y_offset;
  int64_t n = (int64_t)t.width * t.height;
  pool.resize(pool.size() + (size_t)n);
  float4* dst = pool.data() + dt->offset;
  for (int64_t i = 0; i < n; i++) dst[i] = make_float4(t.data[3 * i], t.data[3 * i + 1], t.data[3 * i + 2], 0.0f);
}

}  // namespace
}  // namespace er

using namespace er;

extern "C" er_status er_scene_create(const er_scene_desc* d, const er_scene_opts* opts, er_scene** out) {
  return guarded("er_scene_create", [&]() -> er_status {
    if (!out) return fail(ER_ERR_INVALID_ARG, "out is NULL");
    *out = nullptr;
    er_status st = validate(d);
    if (st != ER_OK) return st;
    er_scene_opts o{};
    o.bvh_format = ER_BVH_FP32;
    if (opts) o = *opts;
    if (o.bvh_format != ER_BVH_FP32 && o.bvh_format != ER_BVH_Q8) return fail(ER_ERR_INVALID_ARG, "bvh_format");
    if (o.builder != ER_BUILDER_HOST && o.builder != ER_BUILDER_GPU) return fail(ER_ERR_INVALID_ARG, "builder");
    int ndev = 0;
    cudaError_t ce = cudaGetDeviceCount(&ndev);
    if (ce != cudaSuccess || ndev == 0) {
      cudaGetLastError();
      return fail(ER_ERR_NO_DEVICE, "no CUDA device visible");
    }
    if (o.device < 0 || o.device >= ndev) return fail(ER_ERR_INVALID_ARG, "device ordinal out of range");
    ER_CUDA(cudaSetDevice(o.device));

    er_scene* s = new er_scene();
    FreeOnUnwind<er_scene> unwind{s, er_scene_free};
    s->device = o.device;
    s->camera = d->camera;
    auto bail = [&](er_status e) {
      er_scene_free(s);
      return e;
    };
    cudaDeviceProp prop;
    ce = cudaGetDeviceProperties(&prop, o.device);
    if (ce != cudaSuccess) return bail(cuda_fail(ce, "cudaGetDeviceProperties"));
    s->num_sms = prop.multiProcessorCount;
    // er_render_noalloc's scratch address on this device (loads the module
    // that holds the array now rather than in that allocation-free call)
    noalloc_prepare(o.device);
    if (o.stream) {
      s->stream = (cudaStream_t)o.stream;
    } else {
      ce = cudaStreamCreateWithFlags(&s->stream, cudaStreamNonBlocking);
      if (ce != cudaSuccess) return bail(cuda_fail(ce, "cudaStreamCreate"));
      s->own_stream = true;
    }
    cudaEventCreate(&s->ev0);
    cudaEventCreate(&s->ev1);
    ce = cudaHostAlloc((void**)&s->h_pin, 128, cudaHostAllocDefault);
    if (ce != cudaSuccess) return bail(cuda_fail(ce, "cudaHostAlloc"));

    // ---- BVH
    const bool gpu_build = o.builder == ER_BUILDER_GPU;
    auto t0 = std::chrono::steady_clock::now();
    BuildResult br;
    if (!gpu_build) {
      st = build_bvh4(d, o.max_leaf_tris > 0 ? o.max_leaf_tris : 4, &br);
      if (st != ER_OK) return bail(st);
      if (3 * br.depth + 1 > 96) return bail(fail(ER_ERR_UNSUPPORTED, "BVH too deep for the traversal stack"));
      if (o.bvh_format == ER_BVH_Q8) quantize_bvh4(&br);
    }
    auto t1 = std::chrono::steady_clock::now();

    // ---- leaf-ordered triangle data (the GPU builder gathers its own)
    int64_t T = d->tri_count;
    const int64_t T_host = gpu_build ? 0 : T;
    std::vector<float4> tv((size_t)(3 * std::max<int64_t>(T_host, 1))), tn((size_t)(3 * std::max<int64_t>(T_host, 1)));
    std::vector<float2> tuv((size_t)(3 * std::max<int64_t>(T_host, 1)));
    std::vector<float4> tt;
    if (d->tangents && !gpu_build) tt.resize((size_t)(3 * T));
    float lo[3] = {INFINITY, INFINITY, INFINITY}, hi[3] = {-INFINITY, -INFINITY, -INFINITY};
    if (gpu_build)
      for (int64_t i = 0; i < 3 * T; i++)
        for (int a = 0; a < 3; a++) {
          lo[a] = std::min(lo[a], d->positions[3 * i + a]);
          hi[a] = std::max(hi[a], d->positions[3 * i + a]);
        }
    for (int64_t s_ = 0; s_ < T_host; s_++) {
      int32_t i = br.order[(size_t)s_];
      const float* p = d->positions + 9 * (int64_t)i;
      int32_t obj = d->tri_object ? d->tri_object[i] : 0;
      int32_t mat = d->object_material && d->object_count > 0 ? d->object_material[obj] : 0;
      uint32_t key = d->tie_key ? d->tie_key[i] : (uint32_t)i;
      float w[3];
      std::memcpy(&w[0], &i, 4);
      std::memcpy(&w[1], &key, 4);
      std::memcpy(&w[2], &mat, 4);
      for (int k = 0; k < 3; k++) {
        tv[3 * s_ + k] = make_float4(p[3 * k], p[3 * k + 1], p[3 * k + 2], w[k]);
        for (int a = 0; a < 3; a++) { lo[a] = std::min(lo[a], p[3 * k + a]); hi[a] = std::max(hi[a], p[3 * k + a]); }
        const float* n = d->normals ? d->normals + 9 * (int64_t)i + 3 * k : nullptr;
        float ts = d->tangent_sign ? d->tangent_sign[i] : 1.0f;
        tn[3 * s_ + k] = n ? make_float4(n[0], n[1], n[2], k == 0 ? ts : 0.0f) : make_float4(0, 0, 0, k == 0 ? ts : 0.0f);
        tuv[3 * s_ + k] = d->uvs ? make_float2(d->uvs[6 * (int64_t)i + 2 * k], d->uvs[6 * (int64_t)i + 2 * k + 1])
                                 : make_float2(0, 0);
        if (d->tangents) {
          const float* g = d->tangents + 9 * (int64_t)i + 3 * k;
          tt[3 * s_ + k] = make_float4(g[0], g[1], g[2], 0.0f);
        }
      }
    }
    float ext = 0;
    for (int a = 0; a < 3; a++) {
      if (T > 0) ext = std::max(ext, std::max(std::fabs(lo[a]), std::fabs(hi[a])));
      s->info.scene_lo[a] = T > 0 ? lo[a] : 0.0f;
      s->info.scene_hi[a] = T > 0 ? hi[a] : 0.0f;
    }

    // ---- materials, textures, env, lights
    std::vector<DevMaterial> mats((size_t)std::max(1, d->material_count));
    for (int32_t i = 0; i < d->material_count; i++) {
      const er_material& m = d->materials[i];
      DevMaterial& q = mats[i];
      std::memset(&q, 0, sizeof q);
      q.albedo_tex = m.albedo_tex; q.emission_tex = m.emission_tex; q.roughness_tex = m.roughness_tex;
      q.metallic_tex = m.metallic_tex; q.normal_tex = m.normal_tex;
      for (int k = 0; k < 3; k++) { q.albedo[k] = m.albedo[k]; q.emission[k] = m.emission[k]; }
      q.roughness = m.roughness; q.metallic = m.metallic; q.clearcoat_gloss = m.clearcoat_gloss;
      q.clearcoat = m.clearcoat; q.anisotropic = m.anisotropic; q.eta = m.eta; q.transmission = m.transmission;
      q.specular = m.specular; q.specular_tint = m.specular_tint; q.sheen_tint = m.sheen_tint;
      q.subsurface = m.subsurface; q.sheen = m.sheen;
    }
    std::vector<float4> pool;
    std::vector<DevTex> texs((size_t)std::max(1, d->texture_count));
    for (int32_t i = 0; i < d->texture_count; i++) pack_texels(d->textures[i], pool, &texs[i]);
    DevTex env;
    pack_texels(d->env, pool, &env);
    std::vector<float> cdf;
    float rsum = 0;
    hdri_cdf(d->env, cdf, &rsum);

    void *p_nodes = nullptr, *p_q = nullptr, *p_tv, *p_tn, *p_tuv, *p_tt = nullptr, *p_mats, *p_texs, *p_pool, *p_cdf,
         *p_lights, *p_err;
    auto t2 = std::chrono::steady_clock::now();
    double gpu_build_ms = 0;
    if (gpu_build) {
      GpuBvh g{};
      float blo[3], bhi[3];
      for (int a = 0; a < 3; a++) { blo[a] = T > 0 ? lo[a] : 0.f; bhi[a] = T > 0 ? hi[a] : 0.f; }
      if ((st = build_bvh_gpu(s, d, o.max_leaf_tris > 0 ? o.max_leaf_tris : 4, blo, bhi, &g)) != ER_OK) return bail(st);
      if (3 * g.depth + 1 > 96) return bail(fail(ER_ERR_UNSUPPORTED, "BVH too deep for the traversal stack"));
      p_nodes = (void*)g.nodes;
      p_tv = (void*)g.tri_v;
      p_tn = (void*)g.tri_n;
      p_tuv = (void*)g.tri_uv;
      p_tt = (void*)g.tri_t;
      br.node_count = g.node_count;
      br.leaf_count = g.leaf_count;
      br.depth = g.depth;
      br.max_delta = g.max_delta;
      gpu_build_ms = g.build_ms;
      if (o.bvh_format == ER_BVH_Q8) {
        // quantised from the GPU tree on the host (outward rounding checked
        // with the kernel's float operations)
        br.nodes.resize((size_t)g.node_count * 32);
        ce = cudaMemcpy(br.nodes.data(), g.nodes, br.nodes.size() * sizeof(float), cudaMemcpyDeviceToHost);
        if (ce != cudaSuccess) return bail(cuda_fail(ce, "BVH download"));
        quantize_bvh4(&br);
      }
    } else {
      if ((st = upload(s, &p_nodes, br.nodes.data(), br.nodes.size() * sizeof(float))) != ER_OK) return bail(st);
      if ((st = upload(s, &p_tv, tv.data(), tv.size() * sizeof(float4))) != ER_OK) return bail(st);
      if ((st = upload(s, &p_tn, tn.data(), tn.size() * sizeof(float4))) != ER_OK) return bail(st);
      if ((st = upload(s, &p_tuv, tuv.data(), tuv.size() * sizeof(float2))) != ER_OK) return bail(st);
      if (d->tangents && (st = upload(s, &p_tt, tt.data(), tt.size() * sizeof(float4))) != ER_OK) return bail(st);
    }
    if (o.bvh_format == ER_BVH_Q8 &&
        (st = upload(s, &p_q, br.qnodes.data(), br.qnodes.size() * sizeof(QNode))) != ER_OK)
      return bail(st);
    if ((st = upload(s, &p_mats, mats.data(), mats.size() * sizeof(DevMaterial))) != ER_OK) return bail(st);
    if ((st = upload(s, &p_texs, texs.data(), texs.size() * sizeof(DevTex))) != ER_OK) return bail(st);
    if ((st = upload(s, &p_pool, pool.data(), pool.size() * sizeof(float4))) != ER_OK) return bail(st);
    if ((st = upload(s, &p_cdf, cdf.data(), cdf.size() * sizeof(float))) != ER_OK) return bail(st);
    er_point_light dummy{};
    if ((st = upload(s, &p_lights, d->light_count > 0 ? (const void*)d->lights : (const void*)&dummy,
                     (size_t)std::max(1, d->light_count) * sizeof(er_point_light))) != ER_OK)
      return bail(st);
    if ((st = dev_alloc(s, &p_err, 256)) != ER_OK) return bail(st);
    ce = cudaMemsetAsync(p_err, 0, 256, s->stream);
    if (ce != cudaSuccess) return bail(cuda_fail(ce, "cudaMemset"));
    ce = cudaStreamSynchronize(s->stream);
    if (ce != cudaSuccess) return bail(cuda_fail(ce, "upload"));
    auto t3 = std::chrono::steady_clock::now();

    DevScene& S = s->dev;
    S.nodes = (const float4*)p_nodes;
    S.qnodes = (const uint4*)p_q;
    S.tri_v = (const float4*)p_tv;
    S.tri_n = (const float4*)p_tn;
    S.tri_uv = (const float2*)p_tuv;
    S.tri_t = (const float4*)p_tt;
    S.mats = (const DevMaterial*)p_mats;
    S.texs = (const DevTex*)p_texs;
    S.texels = (const float4*)p_pool;
    S.lights = (const er_point_light*)p_lights;
    S.env = env;
    S.cdf = (const float*)p_cdf;
    S.alias_idx = nullptr;
    S.alias_thresh = nullptr;
    S.env_lut = nullptr;
    S.radiance_sum = rsum;
    S.n_lights = d->light_count;
    S.n_mats = d->material_count;
    S.n_texs = d->texture_count;
    S.n_tris = T;
    S.n_nodes = br.node_count;
    S.scene_eps = ext;
    S.use_q8 = o.bvh_format == ER_BVH_Q8;
    S.cam = make_dev_camera(d->camera);
    s->texel_count = (int64_t)pool.size();
    s->err_word = (uint32_t*)p_err;
    s->d_stats = (unsigned long long*)((char*)p_err + 64);

    er_scene_info& I = s->info;
    I.tri_count = T;
    I.node_count = br.node_count;
    I.leaf_count = br.leaf_count;
    I.bvh_build_ms = gpu_build ? gpu_build_ms : std::chrono::duration<double, std::milli>(t1 - t0).count();
    I.upload_ms = std::chrono::duration<double, std::milli>(t3 - t2).count();
    I.max_shading_offset = br.max_delta;
    I.bvh_depth = br.depth;
    I.bvh_format = o.bvh_format;
    I.material_count = d->material_count;
    I.env_width = d->env.width;
    I.env_height = d->env.height;
    I.device_bytes = s->device_bytes;
    *out = s;
    return ER_OK;
  });
}

extern "C" er_status er_scene_info_get(const er_scene* s, er_scene_info* out) {
  return guarded("er_scene_info_get", [&]() -> er_status {
    if (!s || !out) return fail(ER_ERR_INVALID_ARG, "NULL argument");
    *out = s->info;
    out->device_bytes = s->device_bytes;
    return ER_OK;
  });
}

extern "C" er_status er_scene_set_camera(er_scene* s, const er_camera* c) {
  return guarded("er_scene_set_camera", [&]() -> er_status {
    if (!s || !c) return fail(ER_ERR_INVALID_ARG, "NULL argument");
    er_status st = validate_camera(*c);
    if (st != ER_OK) return st;
    s->camera = *c;
    s->dev.cam = make_dev_camera(*c);
    s->version++;
    return ER_OK;
  });
}

extern "C" er_status er_scene_get_camera(const er_scene* s, er_camera* out) {
  return guarded("er_scene_get_camera", [&]() -> er_status {
    if (!s || !out) return fail(ER_ERR_INVALID_ARG, "NULL argument");
    *out = s->camera;
    return ER_OK;
  });
}

extern "C" er_status er_scene_free(er_scene* s) {
  return guarded("er_scene_free", [&]() -> er_status {
    if (!s) return ER_OK;
    cudaSetDevice(s->device);
    // a call that failed part-way may have left work on the second wave's
    // stream or the snapshot reader: nothing is freed under it
    if (s->stream) cudaStreamSynchronize(s->stream);
    if (s->stream2) cudaStreamSynchronize(s->stream2);
    if (s->snap_stream) cudaStreamSynchronize(s->snap_stream);
    free_wave(s);
    free_film(s);
    cudaFree(s->bw_rad);
    cudaFree(s->bw_b);
    cudaFree(s->kp_rad);
    for (void* p : s->allocs) cudaFree(p);
    s->allocs.clear();
    for (cudaEvent_t e : s->ev_pool) cudaEventDestroy(e);
    if (s->ev0) cudaEventDestroy(s->ev0);
    if (s->ev1) cudaEventDestroy(s->ev1);
    if (s->h_pin) cudaFreeHost(s->h_pin);
    cudaFree(s->snap_beauty);
    cudaFree(s->snap_samples);
    if (s->snap_event) cudaEventDestroy(s->snap_event);
    if (s->snap_stream) cudaStreamDestroy(s->snap_stream);
    if (s->stream2) cudaStreamDestroy(s->stream2);
    if (s->ev_fork) cudaEventDestroy(s->ev_fork);
    for (cudaEvent_t e : s->ev_acc)
      if (e) cudaEventDestroy(e);
    if (s->own_stream && s->stream) cudaStreamDestroy(s->stream);
    delete s;
    return ER_OK;
  });
}
