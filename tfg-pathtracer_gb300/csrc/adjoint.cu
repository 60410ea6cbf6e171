// Path-replay adjoint of the sample loop, and the parameter interface it
// differentiates.
//
// No counterpart in the reference (it has no derivatives).  Parameters: per
// material (albedo r, g, b, roughness, metallic) as stored before the 2.2
// power generateHitData applies (kernel.cu:103-104), and every environment
// texel (r, g, b) in storage order.  The gradient is that of the per-sample
// estimator with the sampling held fixed ("detached" sampling, as in path
// replay backpropagation, Vicini et al. 2021): random numbers, sampled
// directions, the chosen env texel and light, hit points, visibility, pdfs
// and MIS weights are constants; the derivative flows through every BRDF
// value (continuation, env and light directions) and every environment
// radiance (escape and next-event texel).
//
// Backward: the wavefront forward first gives every sample's radiance L
// (12 bytes per path; it sets the clamp mask and the NaN drop of the
// accumulation, kernel.cu:445-449).  Then the same wavefront re-traces every
// path from its counter-based random numbers (render.cu, gradient variants
// of raygen and shade).  When a vertex's MIS terms are resolved, the replay
// knows the throughput beta_i before it, the radiance L_<=i gathered so far
// and therefore the radiance still to come, L - L_<=i, which carries vertex
// i's throughput factor f_i |N.L| / pdf_i: its derivative is
// (L - L_<=i) * df_i / f_i per channel (adjoint.cuh: vertex_gradient).  The
// vertex is re-shaded from its stored hit for that; nothing else per vertex
// is kept.  Gradients are scattered with warp-aggregated atomics.
//
// The forward of the detached estimator (er_render_replay) is the same
// wavefront with the shade stage's BRDF values and environment radiance
// taken from separate evaluation parameters (render.cu, k_shade's EVAL
// variant; adjoint.cuh: eval_vertex): with no evaluation parameters it is
// er_render; with others it is the estimator whose finite differences the
// gradient is checked against.
#include <cmath>
#include <cstring>
#include <vector>

#include "adjoint.cuh"
#include "internal.h"

namespace er {
namespace {

// ---------------------------------------------------------------- replay --

struct ReplayArgs {
  WaveParams P;              // W, H, npix, spp_wave = spp, sample_base, max_depth, seed, flags
  const float4* d_beauty;    // d loss / d beauty (output index order)
  const uint32_t* nvalid;    // the forward film's sample counts
  float* g_mat;              // n_mats x 5
  float* g_env;              // w*h*3
  int32_t n_mats;
  uint32_t* err;
};

er_status check_replay_opts(er_scene* s, const er_render_opts* o) {
  if (!s || !o) return fail(ER_ERR_INVALID_ARG, "NULL argument");
  if (o->spp < 0 || o->sample_begin < 0 || o->max_depth < 0 || o->max_depth > 64)
    return fail(ER_ERR_INVALID_ARG, "render options out of range");
  if ((int64_t)o->sample_begin + o->spp > INT32_MAX)
    return fail(ER_ERR_INVALID_ARG, "sample_begin + spp exceeds INT32_MAX");
  if (o->flags & ~(uint32_t)(ER_RENDER_DEVICE_OUT | ER_RENDER_ENV_ALIAS | ER_RENDER_ACCUM_FP64))
    return fail(ER_ERR_INVALID_ARG, "only ER_RENDER_DEVICE_OUT, ER_RENDER_ENV_ALIAS and ER_RENDER_ACCUM_FP64 apply here");
  ER_CUDA(cudaSetDevice(s->device));
  er_status st;
  if ((o->flags & ER_RENDER_ENV_ALIAS) && (st = build_env_alias(s)) != ER_OK) return st;
  return build_env_lut(s);
}

WaveParams replay_params(const er_scene* s, const er_render_opts* o) {
  WaveParams P;
  P.W = s->camera.x_res;
  P.H = s->camera.y_res;
  P.npix = P.W * P.H;
  P.spp_wave = o->spp;
  P.sample_base = o->sample_begin;
  P.max_depth = o->max_depth > 0 ? o->max_depth : 5;
  P.k0 = (uint32_t)o->seed;
  P.k1 = (uint32_t)(o->seed >> 32);
  P.flags = o->flags & ER_RENDER_ENV_ALIAS;
  return P;
}

// Device copy of a caller array (host or device per `dev`); *own set when
// a temporary was allocated.
er_status to_device(er_scene* s, bool dev, const void* src, size_t bytes, void** out, bool* own) {
  *own = false;
  *out = nullptr;
  if (!src) return ER_OK;
  if (dev) {
    *out = const_cast<void*>(src);
    return ER_OK;
  }
  cudaError_t e = cudaMalloc(out, bytes);
  if (e != cudaSuccess) {
    cudaGetLastError();
    return fail(ER_ERR_OOM, "temporary allocation failed");
  }
  *own = true;
  ER_CUDA(cudaMemcpyAsync(*out, src, bytes, cudaMemcpyHostToDevice, s->stream));
  return ER_OK;
}

struct Temps {
  std::vector<void*> p;
  ~Temps() {
    for (void* q : p) cudaFree(q);
  }
  er_status alloc(void** out, size_t bytes) {
    cudaError_t e = cudaMalloc(out, std::max<size_t>(bytes, 16));
    if (e != cudaSuccess) {
      cudaGetLastError();
      return fail(ER_ERR_OOM, "temporary allocation failed");
    }
    p.push_back(*out);
    return ER_OK;
  }
};

}  // namespace
}  // namespace er

using namespace er;

extern "C" er_status er_scene_get_params(er_scene* s, float* materials, float* env) {
  return guarded("er_scene_get_params", [&]() -> er_status {
    if (!s) return fail(ER_ERR_INVALID_ARG, "scene is NULL");
    ER_CUDA(cudaSetDevice(s->device));
    const int32_t nm = s->dev.n_mats;
    if (materials && nm > 0) {
      std::vector<DevMaterial> m((size_t)nm);
      ER_CUDA(cudaMemcpyAsync(m.data(), s->dev.mats, m.size() * sizeof(DevMaterial), cudaMemcpyDeviceToHost, s->stream));
      ER_CUDA(cudaStreamSynchronize(s->stream));
      for (int32_t i = 0; i < nm; i++) {
        float* q = materials + 5 * (size_t)i;
        q[0] = m[i].albedo[0]; q[1] = m[i].albedo[1]; q[2] = m[i].albedo[2];
        q[3] = m[i].roughness; q[4] = m[i].metallic;
      }
    }
    if (env) {
      const DevTex& E = s->dev.env;
      const size_t n = (size_t)E.w * E.h;
      std::vector<float4> t(n);
      ER_CUDA(cudaMemcpyAsync(t.data(), s->dev.texels + E.offset, n * sizeof(float4), cudaMemcpyDeviceToHost, s->stream));
      ER_CUDA(cudaStreamSynchronize(s->stream));
      for (size_t i = 0; i < n; i++) {
        env[3 * i] = t[i].x; env[3 * i + 1] = t[i].y; env[3 * i + 2] = t[i].z;
      }
    }
    return ER_OK;
  });
}

extern "C" er_status er_scene_set_params(er_scene* s, const float* materials, const float* env, uint32_t flags) {
  return guarded("er_scene_set_params", [&]() -> er_status {
    if (!s) return fail(ER_ERR_INVALID_ARG, "scene is NULL");
    ER_CUDA(cudaSetDevice(s->device));
    s->version++;  // radiance kept by an earlier render no longer applies
    const bool dev = flags & ER_RENDER_DEVICE_OUT;
    const int32_t nm = s->dev.n_mats;
    if (materials && nm > 0) {
      std::vector<float> q((size_t)nm * 5);
      ER_CUDA(cudaMemcpyAsync(q.data(), materials, q.size() * 4, dev ? cudaMemcpyDeviceToHost : cudaMemcpyHostToHost,
                              s->stream));
      std::vector<DevMaterial> m((size_t)nm);
      ER_CUDA(cudaMemcpyAsync(m.data(), s->dev.mats, m.size() * sizeof(DevMaterial), cudaMemcpyDeviceToHost, s->stream));
      ER_CUDA(cudaStreamSynchronize(s->stream));
      for (int32_t i = 0; i < nm; i++) {
        const float* p = q.data() + 5 * (size_t)i;
        for (int k = 0; k < 5; k++)
          if (!std::isfinite(p[k])) return fail(ER_ERR_INVALID_ARG, "material parameter is not finite");
        m[i].albedo[0] = p[0]; m[i].albedo[1] = p[1]; m[i].albedo[2] = p[2];
        m[i].roughness = p[3]; m[i].metallic = p[4];
      }
      ER_CUDA(cudaMemcpyAsync(const_cast<DevMaterial*>(s->dev.mats), m.data(), m.size() * sizeof(DevMaterial),
                              cudaMemcpyHostToDevice, s->stream));
      ER_CUDA(cudaStreamSynchronize(s->stream));
    }
    if (env) {
      const DevTex& E = s->dev.env;
      const size_t n = (size_t)E.w * E.h;
      std::vector<float> rgb(3 * n);
      ER_CUDA(cudaMemcpyAsync(rgb.data(), env, rgb.size() * 4, dev ? cudaMemcpyDeviceToHost : cudaMemcpyHostToHost,
                              s->stream));
      ER_CUDA(cudaStreamSynchronize(s->stream));
      for (float v : rgb)
        if (!std::isfinite(v)) return fail(ER_ERR_INVALID_ARG, "environment texel is not finite");
      std::vector<float4> t(n);
      for (size_t i = 0; i < n; i++) t[i] = make_float4(rgb[3 * i], rgb[3 * i + 1], rgb[3 * i + 2], 0.f);
      er_texture et{E.w, E.h, rgb.data(), E.x_tile, E.y_tile, E.x_offset, E.y_offset};
      std::vector<float> cdf;
      float rsum = 0;
      hdri_cdf(et, cdf, &rsum);
      ER_CUDA(cudaMemcpyAsync(const_cast<float4*>(s->dev.texels + E.offset), t.data(), n * sizeof(float4),
                              cudaMemcpyHostToDevice, s->stream));
      ER_CUDA(cudaMemcpyAsync(const_cast<float*>(s->dev.cdf), cdf.data(), cdf.size() * 4, cudaMemcpyHostToDevice,
                              s->stream));
      ER_CUDA(cudaStreamSynchronize(s->stream));
      s->dev.radiance_sum = rsum;
      invalidate_env_tables(s);  // refilled on next use
    }
    return ER_OK;
  });
}

extern "C" er_status er_render_replay(er_scene* s, const er_render_opts* o, const float* eval_materials,
                                      const float* eval_env, float* beauty, uint32_t* samples, uint32_t* pathcount) {
  return guarded("er_render_replay", [&]() -> er_status {
    er_status st = check_replay_opts(s, o);
    if (st != ER_OK) return st;
    if (!beauty || !samples || !pathcount) return fail(ER_ERR_INVALID_ARG, "NULL output");
    const bool dev = o->flags & ER_RENDER_DEVICE_OUT;
    const size_t env_n = (size_t)s->dev.env.w * s->dev.env.h * 3;
    Temps T;
    void *em = nullptr, *ee = nullptr;
    bool own_m = false, own_e = false;
    if ((st = to_device(s, dev, eval_materials, (size_t)s->dev.n_mats * 5 * 4, &em, &own_m)) != ER_OK) return st;
    if (own_m) T.p.push_back(em);
    if ((st = to_device(s, dev, eval_env, env_n * 4, &ee, &own_e)) != ER_OK) return st;
    if (own_e) T.p.push_back(ee);
    GradArgs G;
    G.eval_mat = (const float*)em;
    G.eval_env = (const float*)ee;
    return render_eval_device(s, o, G, beauty, samples, pathcount);
  });
}

extern "C" er_status er_backward(er_scene* s, const er_render_opts* o, const float* d_beauty, const uint32_t* samples,
                                 float* grad_materials, float* grad_env, er_render_stats* stats) {
  return guarded("er_backward", [&]() -> er_status {
    er_status st = check_replay_opts(s, o);
    if (st != ER_OK) return st;
    if (!d_beauty || !samples) return fail(ER_ERR_INVALID_ARG, "NULL input");
    const bool dev = o->flags & ER_RENDER_DEVICE_OUT;
    ReplayArgs A{};
    A.P = replay_params(s, o);
    A.n_mats = s->dev.n_mats;
    A.err = s->err_word;
    const size_t np = (size_t)A.P.npix;
    const size_t mat_n = (size_t)A.n_mats * 5, env_n = (size_t)s->dev.env.w * s->dev.env.h * 3;
    Temps T;
    void *db = nullptr, *nv = nullptr;
    bool own;
    if ((st = to_device(s, dev, d_beauty, np * 16, &db, &own)) != ER_OK) return st;
    if (own) T.p.push_back(db);
    if ((st = to_device(s, dev, samples, np * 4, &nv, &own)) != ER_OK) return st;
    if (own) T.p.push_back(nv);
    A.d_beauty = (const float4*)db;
    A.nvalid = (const uint32_t*)nv;
    if (dev && grad_materials) A.g_mat = grad_materials;
    else if ((st = T.alloc((void**)&A.g_mat, mat_n * 4)) != ER_OK) return st;
    if (dev && grad_env) A.g_env = grad_env;
    else if ((st = T.alloc((void**)&A.g_env, env_n * 4)) != ER_OK) return st;
    ER_CUDA(cudaMemsetAsync(A.g_mat, 0, mat_n * 4, s->stream));
    ER_CUDA(cudaMemsetAsync(A.g_env, 0, env_n * 4, s->stream));
    // the samples' radiance: the wavefront forward with a per-path dump into
    // scratch kept on the scene (grown, never shrunk, between calls)
    const int64_t npaths = (int64_t)np * A.P.spp_wave;
    const bool kept = s->kp_valid && s->kp_version == s->version && s->kp_seed == o->seed &&
                      s->kp_begin == o->sample_begin && s->kp_spp == o->spp &&
                      s->kp_depth == (o->max_depth > 0 ? o->max_depth : 5) &&
                      s->kp_flags == (o->flags & ER_RENDER_ENV_ALIAS);
    if (!kept && npaths > s->bw_cap) {
      ER_CUDA(cudaStreamSynchronize(s->stream));
      cudaFree(s->bw_rad);
      cudaFree(s->bw_b);
      s->bw_rad = nullptr;
      s->bw_b = nullptr;
      s->bw_cap = 0;
      if (cudaMalloc(&s->bw_rad, (size_t)npaths * 12) != cudaSuccess ||
          cudaMalloc(&s->bw_b, (size_t)npaths * 4) != cudaSuccess) {
        cudaGetLastError();
        return fail(ER_ERR_OOM, "adjoint scratch allocation failed");
      }
      s->bw_cap = npaths;
    }
    float* d_rad = kept ? s->kp_rad : s->bw_rad;
    int32_t* d_b = s->bw_b;
    ER_CUDA(cudaEventRecord(s->ev0, s->stream));
    int64_t launches = 0;
    if (npaths > 0) {
      er_render_opts oo = *o;
      oo.flags &= ER_RENDER_ENV_ALIAS;
      if (!kept && (st = render_paths_device(s, &oo, d_rad, d_b, true, &launches)) != ER_OK) return st;
      GradArgs G;
      G.rad = d_rad;
      G.d_beauty = A.d_beauty;
      G.nvalid = A.nvalid;
      G.g_mat = A.g_mat;
      G.g_env = A.g_env;
      G.sample0 = o->sample_begin;
      if ((st = render_backward_device(s, &oo, G, &launches)) != ER_OK) return st;
    }
    ER_CUDA(cudaEventRecord(s->ev1, s->stream));
    if (!dev) {
      if (grad_materials)
        ER_CUDA(cudaMemcpyAsync(grad_materials, A.g_mat, mat_n * 4, cudaMemcpyDeviceToHost, s->stream));
      if (grad_env) ER_CUDA(cudaMemcpyAsync(grad_env, A.g_env, env_n * 4, cudaMemcpyDeviceToHost, s->stream));
    } else {
      if (!grad_materials || !grad_env) {
        // device mode with a NULL destination: the gradient is discarded
      }
    }
    ER_CUDA(cudaStreamSynchronize(s->stream));
    if ((st = check_device_error(s)) != ER_OK) return st;
    if (stats) {
      std::memset(stats, 0, sizeof *stats);
      float ms = 0;
      cudaEventElapsedTime(&ms, s->ev0, s->ev1);
      stats->ms = ms;
      stats->samples = (int64_t)o->spp * (int64_t)np;
      stats->kernel_launches = launches;
    }
    return ER_OK;
  });
}
