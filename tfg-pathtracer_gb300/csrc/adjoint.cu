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
// The same walk without gradients is a complete forward render
// (er_render_replay): with the evaluation parameters equal to the scene's
// it reproduces er_render bit for bit; with other evaluation parameters it
// is the detached estimator itself, which finite differences of the
// gradient are checked against.
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
  const float* eval_mat;     // evaluation parameters (n_mats x 5) or null = the scene's
  const float* eval_env;     // evaluation env texels (w*h*3, storage order) or null
  float4* beauty;            // forward outputs (film, output index order)
  uint32_t* samples;
  uint32_t* pathcount;
  const float4* d_beauty;    // d loss / d beauty (output index order)
  const uint32_t* nvalid;    // the forward film's sample counts
  float* g_mat;              // n_mats x 5
  float* g_env;              // w*h*3
  int32_t n_mats;
  uint32_t* err;
};

template <int MODE, bool Q8>
__device__ __forceinline__ void trace_warp(const DevScene& S, Traverser<MODE, Q8, false>& tr, int2* sstk,
                                          bool active, uint32_t* err) {
  // Called by all 32 lanes together; lanes without a ray pass active =
  // false.  Node and leaf rounds are chosen by warp vote as in the
  // persistent traversal, so the lanes stay converged.  Every node is
  // expanded and every leaf tested at most once per ray: the walk is
  // bounded by a multiple of the node count.
  int2 lstk[kLocalStack];
  TravStats st{0, 0, 0};
  bool busy = active && !tr.done;
  const int64_t lim = 8 * S.n_nodes + 64;
  int64_t it = 0;
  while (__any_sync(0xFFFFFFFFu, busy)) {
    const bool node_only = busy && tr.node >= 0 && tr.leaf == 0;
    const bool leaf_round = !__any_sync(0xFFFFFFFFu, node_only);
    if (busy) {
      if (leaf_round) {
        if (tr.leaf != 0) tr.leaf_step(S, sstk, lstk, st, err);
        else if (tr.node < 0) tr.finish();
      } else if (tr.node >= 0) {
        tr.node_step(S, sstk, lstk, st, err);
      }
      if (++it > lim) {
        atomicOr(err, 4u);
        tr.done = true;
      }
      busy = !tr.done;
    }
  }
}

// One sample of pixel (x, y), called by all 32 lanes of the warp together
// (active = false: a lane without a path this round); returns the sample's
// radiance and vertex count.
template <bool Q8, bool EVAL>
__device__ f3 walk(const DevScene& S, const ReplayArgs& A, int2* sstk, bool active, int32_t x, int32_t y,
                   uint32_t idx, uint32_t sample, int32_t* bounces) {
  const WaveParams& P = A.P;
  uint4 ra = philox(make_uint4(idx, sample, 0u, 0u), P.k0, P.k1);
  uint4 rb = philox(make_uint4(idx, sample, 1u, 0u), P.k0, P.k1);
  f3 o, d;
  camera_ray(S.cam, x, y, u01(ra.x), u01(ra.y), u01(ra.z), u01(ra.w), u01(rb.x), o, d);
  f3 thr = mk1(1.0f);
  float Lx = 0.f, Ly = 0.f, Lz = 0.f;
  *bounces = P.max_depth;
  bool alive = active;
  for (int32_t bounce = 0; bounce < P.max_depth; bounce++) {
    if (!__any_sync(0xFFFFFFFFu, alive)) break;
    int32_t hslot = -1;
    float ht = 0.f, hu = 0.f, hv = 0.f;
    {
      Traverser<kClosest, Q8, false> tr;
      if (alive) tr.init(S, o, d, mk1(0.f), 0.f);
      trace_warp(S, tr, sstk, alive, A.err);
      if (alive) {
        hslot = tr.slot;
        ht = tr.t;
        hu = tr.u;
        hv = tr.v;
      }
    }
    if (alive && hslot < 0) {
      // kernel.cu:414-419
      int64_t te;
      f3 e = escape_radiance(S, d, &te);
      if (EVAL && A.eval_env) e = mk(A.eval_env[3 * te], A.eval_env[3 * te + 1], A.eval_env[3 * te + 2]);
      Lx = __fadd_rn(Lx, __fmul_rn(e.x, thr.x));
      Ly = __fadd_rn(Ly, __fmul_rn(e.y, thr.y));
      Lz = __fadd_rn(Lz, __fmul_rn(e.z, thr.z));
      *bounces = bounce;
      alive = false;
    }
    // The vertex is shaded twice: once for its shadow rays, and again after
    // tracing them (same inputs, same result), so that the shading state
    // does not stay live across the traversals.
    bool vH = false, vP = true, pt = false;
    {
      f3 eo = mk1(0.f), ed = mk1(0.f), po = mk1(0.f), pd = mk1(0.f), pp = mk1(0.f);
      float pdist = 0.f;
      if (alive) {
        VertexShade V0;
        shade_vertex(S, P.flags, P.k0, P.k1, idx, sample, bounce, o, d, ht, hu, hv, hslot, V0);
        eo = V0.env_o;
        ed = V0.env_d;
        pt = V0.has_pt;
        po = V0.pt_o;
        pd = V0.pt_d;
        pp = V0.pos;
        pdist = V0.dist;
      }
      {
        Traverser<kAny, Q8, false> te;
        if (alive) te.init(S, eo, ed, mk1(0.f), 0.f);
        trace_warp(S, te, sstk, alive, A.err);
        vH = alive && !te.occluded;
      }
      {
        Traverser<kPoint, Q8, false> tp;
        if (pt) tp.init(S, po, pd, pp, pdist);
        trace_warp(S, tp, sstk, pt, A.err);
        if (pt) vP = !tp.occluded;
      }
    }
    if (!alive) continue;
    VertexShade V;
    shade_vertex(S, P.flags, P.k0, P.k1, idx, sample, bounce, o, d, ht, hu, hv, hslot, V);
    f3 tH = V.tH, tP = V.tP, tB = V.tB, g = V.g, f = V.f, fH = V.fH, fP = V.fP, eH = V.eH;
    const DevMaterial& M = S.mats[V.mat];
    if (EVAL) {
      // evaluation parameters: the same formulas with this vertex's BRDF
      // and environment values re-evaluated (directions, pdfs, weights kept)
      HitData he = V.hd;
      if (A.eval_mat) {
        const float* q = A.eval_mat + 5 * (size_t)V.mat;
        if (M.albedo_tex < 0) he.albedo = mk(q[0], q[1], q[2]);
        if (M.roughness_tex < 0) he.roughness = powf(q[3], 2.2f);
        if (M.metallic_tex < 0) he.metallic = powf(q[4], 2.2f);
      }
      DisneyCtx Ce = disney_ctx(he, d);
      f = disney_eval(he, Ce, V.dir);
      fH = disney_eval(he, Ce, V.dH);
      if (A.eval_env) {
        int64_t t3 = 3 * V.env_texel;
        eH = mk(A.eval_env[t3], A.eval_env[t3 + 1], A.eval_env[t3 + 2]);
      }
      f3 hdriC = (fH * V.cosH) * eH / V.hdriPdf;
      tH = hdriC * V.w1;
      if (V.has_pt) {
        fP = disney_eval(he, Ce, V.dP);
        f3 pointC = (V.plv * fP) * V.cosP / V.pointPdf;
        tP = pointC * V.w2;
      }
      f3 brdfC = (f * V.ndl) * he.emission / V.brdfPdf;
      tB = brdfC * V.w3;
      g = (f * V.ndl) / V.brdfPdf;
    }
    // resolve in the reference's order (kernel.cu:351-355)
    float w1z = V.w1 * 0.0f, w2z = V.w2 * 0.0f;
    float hx = vH ? tH.x : w1z, hy = vH ? tH.y : w1z, hz = vH ? tH.z : w1z;
    float px = vP ? tP.x : w2z, py = vP ? tP.y : w2z, pz = vP ? tP.z : w2z;
    Lx = __fadd_rn(Lx, __fmul_rn(__fadd_rn(__fadd_rn(hx, px), tB.x), thr.x));
    Ly = __fadd_rn(Ly, __fmul_rn(__fadd_rn(__fadd_rn(hy, py), tB.y), thr.y));
    Lz = __fadd_rn(Lz, __fmul_rn(__fadd_rn(__fadd_rn(hz, pz), tB.z), thr.z));
    thr = mk(__fmul_rn(thr.x, g.x), __fmul_rn(thr.y, g.y), __fmul_rn(thr.z, g.z));
    if (bounce + 1 >= P.max_depth) break;
    // kernel.cu:442
    o = xadd(V.pos, xscale(V.dir, 0.001f));
    d = xnormalize(V.dir);
  }
  return mk(Lx, Ly, Lz);
}

// Forward render by replay: one thread per pixel, samples in order, with
// accumulate_pixel's arithmetic.  Lanes past the image take part in the
// warp's traversals without a path.
template <bool Q8, bool EVAL>
__global__ void __launch_bounds__(kTravBlock) k_replay(DevScene S, ReplayArgs A) {
  __shared__ int2 stk[kSmemStack * kTravBlock];
  const WaveParams& P = A.P;
  const int32_t pix0 = blockIdx.x * blockDim.x + threadIdx.x;
  const bool valid = pix0 < P.npix;
  const int32_t pix = valid ? pix0 : 0;
  const int32_t x = pix % P.W, y = pix / P.W;
  const uint32_t idx = (uint32_t)(P.W * (P.H - y - 1) + x);  // kernel.cu:378
  uint32_t sa = 0, pc = 0;
  float4 bt = make_float4(0.f, 0.f, 0.f, 1.f);
  for (int32_t s = 0; s < P.spp_wave; s++) {
    int32_t nb;
    f3 L = walk<Q8, EVAL>(S, A, stk + threadIdx.x, valid, x, y, idx, (uint32_t)(P.sample_base + s), &nb);
    if (!valid) continue;
    pc += (uint32_t)nb;
    float lx = clampf_(L.x, 0.f, 10.f), ly = clampf_(L.y, 0.f, 10.f), lz = clampf_(L.z, 0.f, 10.f);
    if (isnan(lx) || isnan(ly) || isnan(lz)) continue;
    float inv = __fadd_rn((float)sa, 1.0f);
    if (sa > 0) {
      float k = __fdiv_rn((float)sa, (float)(sa + 1));
      bt.x = __fmul_rn(bt.x, k); bt.y = __fmul_rn(bt.y, k); bt.z = __fmul_rn(bt.z, k);
    }
    bt.x = __fadd_rn(bt.x, __fdiv_rn(lx, inv));
    bt.y = __fadd_rn(bt.y, __fdiv_rn(ly, inv));
    bt.z = __fadd_rn(bt.z, __fdiv_rn(lz, inv));
    sa++;
  }
  if (!valid) return;
  A.beauty[idx] = bt;
  A.samples[idx] = sa;
  A.pathcount[idx] = pc;
}


template <bool EVAL>
er_status launch_replay(er_scene* s, const ReplayArgs& A) {
  const int32_t npix = A.P.npix;
  const unsigned blocks = (unsigned)((npix + kTravBlock - 1) / kTravBlock);
  if (s->dev.use_q8) k_replay<true, EVAL><<<blocks, kTravBlock, 0, s->stream>>>(s->dev, A);
  else k_replay<false, EVAL><<<blocks, kTravBlock, 0, s->stream>>>(s->dev, A);
  ER_CUDA(cudaGetLastError());
  return ER_OK;
}

// ------------------------------------------------------------- host side --

er_status check_replay_opts(er_scene* s, const er_render_opts* o) {
  if (!s || !o) return fail(ER_ERR_INVALID_ARG, "NULL argument");
  if (o->spp < 0 || o->sample_begin < 0 || o->max_depth < 0 || o->max_depth > 64)
    return fail(ER_ERR_INVALID_ARG, "render options out of range");
  if (o->flags & ~(uint32_t)(ER_RENDER_DEVICE_OUT | ER_RENDER_ENV_ALIAS))
    return fail(ER_ERR_INVALID_ARG, "only ER_RENDER_DEVICE_OUT and ER_RENDER_ENV_ALIAS apply here");
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
    ReplayArgs A{};
    A.P = replay_params(s, o);
    A.n_mats = s->dev.n_mats;
    A.err = s->err_word;
    const size_t np = (size_t)A.P.npix;
    const size_t env_n = (size_t)s->dev.env.w * s->dev.env.h * 3;
    Temps T;
    void *em = nullptr, *ee = nullptr;
    bool own_m = false, own_e = false;
    if ((st = to_device(s, dev, eval_materials, (size_t)A.n_mats * 5 * 4, &em, &own_m)) != ER_OK) return st;
    if (own_m) T.p.push_back(em);
    if ((st = to_device(s, dev, eval_env, env_n * 4, &ee, &own_e)) != ER_OK) return st;
    if (own_e) T.p.push_back(ee);
    A.eval_mat = (const float*)em;
    A.eval_env = (const float*)ee;
    if (dev) {
      A.beauty = (float4*)beauty;
      A.samples = samples;
      A.pathcount = pathcount;
    } else {
      if ((st = T.alloc((void**)&A.beauty, np * 16)) != ER_OK) return st;
      if ((st = T.alloc((void**)&A.samples, np * 4)) != ER_OK) return st;
      if ((st = T.alloc((void**)&A.pathcount, np * 4)) != ER_OK) return st;
    }
    if (np > 0) {
      st = (em || ee) ? launch_replay<true>(s, A) : launch_replay<false>(s, A);
      if (st != ER_OK) return st;
    }
    if (!dev) {
      ER_CUDA(cudaMemcpyAsync(beauty, A.beauty, np * 16, cudaMemcpyDeviceToHost, s->stream));
      ER_CUDA(cudaMemcpyAsync(samples, A.samples, np * 4, cudaMemcpyDeviceToHost, s->stream));
      ER_CUDA(cudaMemcpyAsync(pathcount, A.pathcount, np * 4, cudaMemcpyDeviceToHost, s->stream));
    }
    ER_CUDA(cudaStreamSynchronize(s->stream));
    return check_device_error(s);
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
    if (npaths > 0) {
      er_render_opts oo = *o;
      oo.flags &= ER_RENDER_ENV_ALIAS;
      if (!kept && (st = render_paths_device(s, &oo, d_rad, d_b, true)) != ER_OK) return st;
      GradArgs G;
      G.rad = d_rad;
      G.d_beauty = A.d_beauty;
      G.nvalid = A.nvalid;
      G.g_mat = A.g_mat;
      G.g_env = A.g_env;
      G.sample0 = o->sample_begin;
      if ((st = render_backward_device(s, &oo, G)) != ER_OK) return st;
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
      stats->kernel_launches = npaths > 0 ? 2 * A.P.max_depth + 4 : 0;
    }
    return ER_OK;
  });
}
