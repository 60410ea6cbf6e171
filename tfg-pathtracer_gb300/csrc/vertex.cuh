// One path vertex of the reference's sample loop (kernel.cu:404-443):
// generateHitData, the BRDF sample, HDRI and point-light next-event
// estimation and the MIS terms of shade (kernel.cu:339-358), computed from
// a closest hit.  Shared by the wavefront shade kernel and the path-replay
// kernels, which must reproduce the same vertex bit for bit.
#pragma once

#include "shade.cuh"
#include "traverse.cuh"

namespace er {

// Storage index of the texel tex_coord reads (Texture.hpp:95-112).
__device__ __forceinline__ int64_t tex_index(const DevTex& t, int32_t x, int32_t y) {
  x = __float2int_rz(t.x_tile * ((float)x + t.x_offset * (float)t.w)) % t.w;
  y = __float2int_rz(t.y_tile * ((float)y + t.y_offset * (float)t.h)) % t.h;
  if (x < 0) x += t.w;
  if (y < 0) y += t.h;
  return (int64_t)y * t.w + x;
}

// kernel.cu:414-419: environment radiance seen along d; *texel = the env
// texel read (storage index).
__device__ __forceinline__ f3 escape_radiance(const DevScene& S, f3 d, int64_t* texel) {
  float eu, ev;
  spherical_mapping(-d, eu, ev);
  const DevTex& E = S.env;
  if (texel) *texel = tex_index(E, __float2int_rz(eu * (float)E.w), __float2int_rz(ev * (float)E.h));
  return tex_uv(S, E, eu, ev);
}

// kernel.cu:234-235: index of the environment texel HDRI NEE samples with
// the shared light uniform r1 = u01(w): the reference's CDF search, or the
// same search through its 2^24-entry table, or (ER_RENDER_ENV_ALIAS) the
// alias table of its effective distribution (env.cu).
__device__ __forceinline__ int32_t env_pick(const DevScene& S, uint32_t flags, uint32_t idx, uint32_t sample,
                                            int32_t bounce, uint32_t w, uint32_t k0, uint32_t k1) {
  const DevTex& E = S.env;
  if ((flags & ER_RENDER_ENV_ALIAS) && S.alias_idx) {
    // column from the shared light word, coin from a second word
    uint32_t coin = philox(make_uint4(idx, sample, 2u + (uint32_t)bounce, 1u), k0, k1).x;
    int32_t col = (int32_t)__umulhi(w, (uint32_t)(E.w * E.h));
    return coin < __ldg(S.alias_thresh + col) ? col : __ldg(S.alias_idx + col);
  }
  if (S.env_lut) return __ldg(S.env_lut + (w >> 8));  // == hdri_search(S.cdf, u01(w), w*h)
  return hdri_search(S.cdf, u01(w), E.w * E.h);
}

// kernel.cu:236-245: texel index -> pixel -> uv with the env's tile and
// offset (Texture.hpp:177-193), limited to [0, 1] (Math.hpp:38-41).
__device__ __forceinline__ void env_texel_uv(const DevTex& E, int32_t cnt, float& iu, float& iv) {
  float nu = __fdiv_rn((float)(cnt % E.w), (float)E.w), nv = __fdiv_rn((float)(cnt / E.w), (float)E.h);
  int32_t ix = __float2int_rz(nu * (float)E.w), iy = __float2int_rz(nv * (float)E.h);
  ix = __float2int_rz(E.x_tile * ((float)ix - E.x_offset * (float)E.w)) % E.w;
  iy = __float2int_rz(E.y_tile * ((float)iy - E.y_offset * (float)E.h)) % E.h;
  iu = __fdiv_rn((float)ix, (float)E.w);
  iv = __fdiv_rn((float)iy, (float)E.h);
  limit_uv(iu, iv);
}

struct VertexShade {
  f3 pos;            // shading position (Tri.hpp:91)
  f3 sn, tg, bt;     // interpolated normal, tangent, bitangent (AOVs)
  int32_t mat;       // material slot
  float rough_in, metal_in;  // material roughness / metallic before the 2.2 power
  HitData hd;
  DisneyCtx C;
  f3 dir;            // BRDF-sampled continuation direction (not normalised)
  f3 f;              // DisneyEval(dir)
  float brdfPdf, ndl;
  f3 dH, eH, fH;     // HDRI NEE: direction, texel radiance, BRDF
  float hdriPdf, cosH;
  int64_t env_texel;
  bool has_pt;
  f3 dP, fP, plv;    // point-light NEE: direction, BRDF, radiance / dist^2
  float pointPdf, dist, cosP;
  float w1, w2, w3;  // MIS weights
  f3 tH, tP, tB;     // weighted strategy terms (before the path throughput)
  f3 g;              // throughput factor f * |N.L| / pdf
  f3 env_o, env_d, pt_o, pt_d;  // shadow rays
};

// Shades the closest hit (t, u, v, slot) of ray (o, d) at vertex `bounce`
// of the sample with output index idx and sample number `sample`.
template <bool EVAL_LOOP = false>
__device__ __forceinline__ void shade_vertex(const DevScene& S, uint32_t flags, uint32_t k0, uint32_t k1, uint32_t idx,
                                             uint32_t sample, int32_t bounce, f3 o, f3 d, float t, float u, float v,
                                             int32_t slot, VertexShade& V) {
  // Tri.hpp:70-92 + 153-157 rebuilt from (t, u, v) with the same ops
  const float4* tv = S.tri_v + 3 * (size_t)slot;
  const float4* tn = S.tri_n + 3 * (size_t)slot;
  float4 v0 = __ldg(tv), v1 = __ldg(tv + 1), v2 = __ldg(tv + 2);
  float4 n0 = __ldg(tn), n1 = __ldg(tn + 1), n2 = __ldg(tn + 2);
  // The vertex's random numbers and the environment texel they pick for
  // HDRI NEE (kernel.cu:234-245) depend on no surface data: their loads
  // (search table, then texel) are issued here, so that they overlap the
  // triangle -> material -> texture loads below instead of following them.
  uint4 rn = philox(make_uint4(idx, sample, 2u + (uint32_t)bounce, 0u), k0, k1);
  const int32_t cnt = env_pick(S, flags, idx, sample, bounce, rn.w, k0, k1);
  f3 sn;
  f3 pos = ref_position(o, d, t, u, v, from4(v0), from4(v1), from4(v2), from4(n0), from4(n1), from4(n2), &sn);
  const float2* tuv = S.tri_uv + 3 * (size_t)slot;
  float2 uv0 = __ldg(tuv), uv1 = __ldg(tuv + 1), uv2 = __ldg(tuv + 2);
  float iu, iv;
  env_texel_uv(S.env, cnt, iu, iv);
  const DevTex& E = S.env;
  const int32_t ex = __float2int_rz(iu * (float)E.w), ey = __float2int_rz(iv * (float)E.h);
  const f3 eH = tex_coord(S, E, ex, ey);
  float tu = __fadd_rn(__fadd_rn(uv0.x, __fmul_rn(__fsub_rn(uv1.x, uv0.x), u)), __fmul_rn(__fsub_rn(uv2.x, uv0.x), v));
  float tvv = __fadd_rn(__fadd_rn(uv0.y, __fmul_rn(__fsub_rn(uv1.y, uv0.y), u)), __fmul_rn(__fsub_rn(uv2.y, uv0.y), v));
  f3 tg = mk1(0.f), bt = mk1(0.f);
  if (S.tri_t) {
    const float4* tt = S.tri_t + 3 * (size_t)slot;
    f3 g0 = from4(__ldg(tt)), g1 = from4(__ldg(tt + 1)), g2 = from4(__ldg(tt + 2));
    tg = xadd(xadd(g0, xscale(xsub(g1, g0), u)), xscale(xsub(g2, g0), v));
    bt = xscale(xcross(sn, tg), n0.w);
  }
  V.pos = pos;
  V.sn = sn;
  V.tg = tg;
  V.bt = bt;
  // kernel.cu:54-119 generateHitData
  V.mat = __float_as_int(v2.w);
  const DevMaterial& M = S.mats[V.mat];
  HitData& hd = V.hd;
  hd.albedo = M.albedo_tex < 0 ? mk(M.albedo[0], M.albedo[1], M.albedo[2]) : tex_uv(S, S.texs[M.albedo_tex], tu, tvv);
  hd.emission = M.emission_tex < 0 ? mk(M.emission[0], M.emission[1], M.emission[2])
                                   : tex_uv(S, S.texs[M.emission_tex], tu, tvv);
  float rough = M.roughness_tex < 0 ? M.roughness : tex_uv(S, S.texs[M.roughness_tex], tu, tvv).x;
  float metal = M.metallic_tex < 0 ? M.metallic : tex_uv(S, S.texs[M.metallic_tex], tu, tvv).x;
  if (M.normal_tex < 0) {
    hd.normal = sn;
  } else {
    f3 c = tex_uv(S, S.texs[M.normal_tex], tu, tvv);
    f3 ln = c * 2.0f - mk1(1.0f);
    hd.normal = normalized(tg * ln.x - bt * ln.y + sn * ln.z);
  }
  V.rough_in = rough;
  V.metal_in = metal;
  {
    // one copy of powf for both remaps (the pair rotated through a loop):
    // 1.4 % off the shade stage on the 1080p scene
    float pr = rough, pm = metal;
#pragma unroll 1
    for (int k = 0; k < 2; k++) {
      const float r = powf(pr, 2.2f);
      pr = pm;
      pm = r;
    }
    hd.roughness = pr;
    hd.metallic = pm;
  }
  hd.clearcoatGloss = M.clearcoat_gloss;
  hd.clearcoat = M.clearcoat;
  hd.anisotropic = M.anisotropic;
  hd.transmission = M.transmission;
  hd.specular = M.specular;
  hd.specularTint = M.specular_tint;
  hd.sheenTint = M.sheen_tint;
  hd.subsurface = M.subsurface;
  hd.sheen = M.sheen;

  V.C = disney_ctx(hd, d);
  const DisneyCtx& C = V.C;
  f3 dir = disney_sample(hd, C, u01(rn.x), u01(rn.y), u01(rn.z));
  float r1 = u01(rn.w);
  f3 dH = -normalized(reverse_spherical(iu, iv));
  // EVAL_LOOP: the point light's direction first, so that the BRDF is
  // evaluated for the three directions by one copy of its code (a loop, not
  // unrolled), for a smaller hot loop in the instruction cache; the values
  // are the same either way.  Measured per workload (same call): the 64-job
  // batch of small scenes 3.9 % faster with the loop, the 1080p textured
  // scene 6 % slower in the shade stage (more spilling), so the batch and
  // gradient kernels take the loop and the plain kernels the three inlined
  // calls.
  int32_t li = 0;
  f3 toL = mk1(0.f), dP = mk1(0.f);
  auto light_dir = [&]() {
    li = min(__float2int_rz((float)S.n_lights * r1), S.n_lights - 1);
    const er_point_light& Lq = S.lights[li];
    toL = xsub(mk(Lq.position[0], Lq.position[1], Lq.position[2]), pos);
    dP = normalized(toL);
  };
  if (EVAL_LOOP && S.n_lights > 0) light_dir();
  f3 f, fH, fP = mk1(0.f);
  if (EVAL_LOOP) {
    const int n_eval = S.n_lights > 0 ? 3 : 2;
#pragma unroll 1
    for (int k = 0; k < n_eval; k++) {
      const f3 L = k == 0 ? dir : (k == 1 ? dH : dP);
      const f3 e = disney_eval(hd, C, L);
      if (k == 0) f = e;
      else if (k == 1) fH = e;
      else fP = e;
    }
  } else {
    f = disney_eval(hd, C, dir);
    fH = disney_eval(hd, C, dH);
  }
  // shade, kernel.cu:339-358
  float brdfPdf = disney_pdf(C, dir);
  float ndl = fabsf(dot(dir, hd.normal));
  V.dir = dir;
  V.f = f;
  V.brdfPdf = brdfPdf;
  V.ndl = ndl;
  // HDRI NEE, kernel.cu:234-257 (the pdf is defined even when blocked);
  // the texel (iu, iv) and its value eH were fetched above
  float hdriPdf = hdri_pdf(S, eH, ey);
  float cosH = fabsf(dot(dH, hd.normal));
  f3 hdriC = (fH * cosH) * eH / hdriPdf;
  V.dH = dH;
  V.eH = eH;
  V.fH = fH;
  V.hdriPdf = hdriPdf;
  V.cosH = cosH;
  V.env_texel = tex_index(E, ex, ey);
  V.env_o = xadd(pos, xscale(dH, 0.001f));
  V.env_d = xnormalize(dH);
  // point light NEE, kernel.cu:175-205
  float pointPdf = 0.f;
  f3 pointC = mk1(0.f);
  V.has_pt = false;
  V.dP = V.fP = V.plv = V.pt_o = V.pt_d = mk1(0.f);
  V.dist = V.cosP = 0.f;
  if (S.n_lights > 0) {
    pointPdf = (float)S.n_lights / (2.0f * ER_PI);
    if (!EVAL_LOOP) {
      light_dir();
      fP = disney_eval(hd, C, dP);
    }
    const er_point_light& Lp = S.lights[li];
    float dist = xlen(toL);
    f3 plv = mk(Lp.radiance[0], Lp.radiance[1], Lp.radiance[2]) / (dist * dist);
    float cosP = fabsf(dot(dP, hd.normal));
    pointC = (plv * fP) * cosP / pointPdf;
    V.dP = dP;
    V.fP = fP;
    V.plv = plv;
    V.dist = dist;
    V.cosP = cosP;
    V.pt_o = xadd(pos, xscale(dP, 0.001f));
    V.pt_d = xnormalize(dP);
    V.has_pt = true;
  }
  V.pointPdf = pointPdf;
  f3 brdfC = (f * ndl) * hd.emission / brdfPdf;
  float den = hdriPdf + pointPdf + brdfPdf;
  V.w1 = hdriPdf / den;
  V.w2 = pointPdf / den;
  V.w3 = brdfPdf / den;
  V.tH = hdriC * V.w1;
  V.tP = pointC * V.w2;
  V.tB = brdfC * V.w3;
  V.g = (f * ndl) / brdfPdf;
}

}  // namespace er
