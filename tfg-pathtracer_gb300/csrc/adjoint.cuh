// Derivatives of the per-vertex shading for the path-replay adjoint, shared
// by the replay kernels (adjoint.cu) and the gradient variant of the
// wavefront shade stage (render.cu).
#pragma once

#include "vertex.cuh"

namespace er {

constexpr int kParams = 5;  // per material: albedo r, g, b, roughness, metallic

// Closed-form partials of DisneyEval (Disney.hpp:179-253) in albedo,
// metallic and roughness.  With GD = Gs * Ds, A the specular mix and Ctint = Cdlin /
// Cdlum (Cdlum = 0.3 r + 0.6 g + 0.1 b):
//   f_c = (Cdlin_c kd + Fsheen_c)(1 - m) + (Cspec0_c (1 - FH) + FH) GD + cc
//   Cspec0_c = X_c (1 - m) + m Cdlin_c,  X_c = (1 + sT (Ctint_c - 1)) 0.08 s
//   Fsheen_c = (1 + shT (Ctint_c - 1)) FH sheen
// so  d f_c / d Cdlin_j = [c = j] (kd (1 - m) + GD (1 - FH) m)
//                         + d Ctint_c / d Cdlin_j (1 - m)(shT FH sheen + GD (1 - FH) sT 0.08 s)
// with d Ctint_c / d Cdlin_j = ([c = j] - Ctint_c w_j) / Cdlum (zero when
// Cdlum <= 0, where Ctint is the constant 1), and
//   d f_c / d m = -(Cdlin_c kd + Fsheen_c) + GD (1 - FH)(Cdlin_c - X_c).
// Roughness r enters kd through Fd90 = 0.5 + 2 LH^2 r and Fss90 = LH^2 r,
// and GD through ax = max(0.001, r / aspect), ay = max(0.001, r aspect):
//   d f_c / d r = Cdlin_c (1 - m) d kd / d r + Fs_c d GD / d r
//   Ds = 1 / (pi ax ay q^2), q = (HX / ax)^2 + (HY / ay)^2 + NH^2:
//     d Ds / d ax = Ds (4 HX^2 / (ax^3 q) - 1 / ax)   (ay alike)
//   G1 = 1 / (NV + S), S = sqrt((VX ax)^2 + (VY ay)^2 + NV^2):
//     d G1 / d ax = -G1^2 VX^2 ax / S                  (ay alike)
// dA[j] holds d f / d Cdlin_j for the three channels.
struct EvalGrad {
  f3 dA[3];
  f3 dM;
  f3 dR;
};
__device__ __forceinline__ EvalGrad disney_eval_grad(const HitData& hd, const DisneyCtx& c, f3 L) {
  EvalGrad g;
  g.dA[0] = g.dA[1] = g.dA[2] = g.dM = g.dR = mk1(0.f);
  if (!disney_gate(hd, c, L)) return g;
  const f3 H = normalized(L + c.V);
  const float NDotL = fabsf(dot(c.N, L));
  const float NDotV = fabsf(dot(c.N, c.V));
  const float NDotH = fabsf(dot(c.N, H));
  const float LDotH = fabsf(dot(L, H));
  const f3 Cdlin = hd.albedo;
  const float m = hd.metallic;
  const float Cdlum = 0.3f * Cdlin.x + 0.6f * Cdlin.y + 0.1f * Cdlin.z;
  const bool lum = Cdlum > 0.0f;
  const f3 Ctint = lum ? Cdlin / Cdlum : mk1(1.0f);
  const float s08 = hd.specular * 0.08f;
  const f3 X = lerp3(mk1(1.0f), Ctint, hd.specularTint) * s08;
  const f3 Csheen = lerp3(mk1(1.0f), Ctint, hd.sheenTint);
  const float FL = schlick(NDotL), FV = schlick(NDotV);
  const float Fd90 = 0.5f + 2.0f * LDotH * LDotH * hd.roughness;
  const float Fd = lerpf_(1.0f, Fd90, FL) * lerpf_(1.0f, Fd90, FV);
  const float Fss90 = LDotH * LDotH * hd.roughness;
  const float Fss = lerpf_(1.0f, Fss90, FL) * lerpf_(1.0f, Fss90, FV);
  const float ss = 1.25f * (Fss * (1.0f / (NDotL + NDotV) - 0.5f) + 0.5f);
  const float HX = dot(H, c.T), HY = dot(H, c.B);
  const float Ds = gtr2_aniso(NDotH, HX, HY, c.ax, c.ay);
  const float FH = schlick(LDotH);
  const float LX = dot(L, c.T), LY = dot(L, c.B), VX = dot(c.V, c.T), VY = dot(c.V, c.B);
  const float G1L = smith_ggx_aniso(NDotL, LX, LY, c.ax, c.ay);
  const float G1V = smith_ggx_aniso(NDotV, VX, VY, c.ax, c.ay);
  const float Gs = G1L * G1V;
  const float GD = Gs * Ds;
  const float kd = (1.0f / ER_PI) * lerpf_(Fd, ss, hd.subsurface);
  {
    // roughness
    const float LH2 = LDotH * LDotH;
    const float dFd = 2.0f * LH2 * (FL * lerpf_(1.0f, Fd90, FV) + FV * lerpf_(1.0f, Fd90, FL));
    const float dFss = LH2 * (FL * lerpf_(1.0f, Fss90, FV) + FV * lerpf_(1.0f, Fss90, FL));
    const float dss = 1.25f * (1.0f / (NDotL + NDotV) - 0.5f) * dFss;
    const float dkd = (1.0f / ER_PI) * ((1.0f - hd.subsurface) * dFd + hd.subsurface * dss);
    const float aspect = sqrtf(1.0f - hd.anisotropic * 0.9f);
    const float dax = hd.roughness / aspect > 0.001f ? 1.0f / aspect : 0.0f;
    const float day = hd.roughness * aspect > 0.001f ? aspect : 0.0f;
    const float q = (HX / c.ax) * (HX / c.ax) + (HY / c.ay) * (HY / c.ay) + NDotH * NDotH;
    const float dDs_ax = Ds * (4.0f * HX * HX / (c.ax * c.ax * c.ax * q) - 1.0f / c.ax);
    const float dDs_ay = Ds * (4.0f * HY * HY / (c.ay * c.ay * c.ay * q) - 1.0f / c.ay);
    const float SL = sqrtf(LX * c.ax * (LX * c.ax) + LY * c.ay * (LY * c.ay) + NDotL * NDotL);
    const float SV = sqrtf(VX * c.ax * (VX * c.ax) + VY * c.ay * (VY * c.ay) + NDotV * NDotV);
    const float dG1L_ax = -G1L * G1L * LX * LX * c.ax / SL, dG1L_ay = -G1L * G1L * LY * LY * c.ay / SL;
    const float dG1V_ax = -G1V * G1V * VX * VX * c.ax / SV, dG1V_ay = -G1V * G1V * VY * VY * c.ay / SV;
    const float dGD_ax = (dG1L_ax * G1V + G1L * dG1V_ax) * Ds + Gs * dDs_ax;
    const float dGD_ay = (dG1L_ay * G1V + G1L * dG1V_ay) * Ds + Gs * dDs_ay;
    const float dGD = dGD_ax * dax + dGD_ay * day;
    const f3 Cspec0 = lerp3(X, Cdlin, m);
    const f3 Fs = lerp3(Cspec0, mk1(1.0f), FH);
    g.dR = Cdlin * ((1.0f - m) * dkd) + Fs * dGD;
  }
  const f3 Fsheen = Csheen * (FH * hd.sheen);
  const float spec_m = GD * (1.0f - FH);
  g.dM = (Cdlin - X) * spec_m - (Cdlin * kd + Fsheen);
  const float A = kd * (1.0f - m) + spec_m * m;
  const float B = lum ? (1.0f - m) * (hd.sheenTint * FH * hd.sheen + spec_m * hd.specularTint * s08) / Cdlum : 0.0f;
  const float w[3] = {0.3f, 0.6f, 0.1f};
#pragma unroll
  for (int j = 0; j < 3; j++) {
    g.dA[j] = Ctint * (-B * w[j]);
    const float diag = A + B;
    if (j == 0) g.dA[j].x += diag;
    if (j == 1) g.dA[j].y += diag;
    if (j == 2) g.dA[j].z += diag;
  }
  return g;
}

// The detached estimator at a vertex (er_render_replay): the vertex's
// BRDF values and environment radiance re-evaluated with the evaluation
// parameters (albedo, roughness, metallic per material before the 2.2 power
// of kernel.cu:103-104; env texels), with its directions, pdfs, MIS weights,
// chosen texel and light kept from the scene's parameters; updates the
// strategy terms tH, tP, tB and the throughput factor g (kernel.cu:339-357).
__device__ __forceinline__ void eval_vertex(const DevScene& S, const float* eval_mat, const float* eval_env, f3 d,
                                            VertexShade& V) {
  const DevMaterial& M = S.mats[V.mat];
  HitData he = V.hd;
  if (eval_mat) {
    const float* q = eval_mat + 5 * (size_t)V.mat;
    if (M.albedo_tex < 0) he.albedo = mk(q[0], q[1], q[2]);
    if (M.roughness_tex < 0) he.roughness = powf(q[3], 2.2f);
    if (M.metallic_tex < 0) he.metallic = powf(q[4], 2.2f);
  }
  const DisneyCtx Ce = disney_ctx(he, d);
  const f3 f = disney_eval(he, Ce, V.dir);
  const f3 fH = disney_eval(he, Ce, V.dH);
  f3 eH = V.eH;
  if (eval_env) {
    const int64_t t3 = 3 * V.env_texel;
    eH = mk(eval_env[t3], eval_env[t3 + 1], eval_env[t3 + 2]);
  }
  const f3 hdriC = (fH * V.cosH) * eH / V.hdriPdf;
  V.tH = hdriC * V.w1;
  if (V.has_pt) {
    const f3 fP = disney_eval(he, Ce, V.dP);
    const f3 pointC = (V.plv * fP) * V.cosP / V.pointPdf;
    V.tP = pointC * V.w2;
  }
  const f3 brdfC = (f * V.ndl) * he.emission / V.brdfPdf;
  V.tB = brdfC * V.w3;
  V.g = (f * V.ndl) / V.brdfPdf;
}

// base[key * N + k] += v[k], warp-aggregated: the converged lanes that
// share a key (neighbouring pixels see the same env texel and object) are
// summed with shuffles and one lane issues the N atomics.  Non-finite
// contributions are dropped.
template <int N>
__device__ __forceinline__ void agg_add(float* base, int64_t key, float (&v)[N]) {
#pragma unroll
  for (int k = 0; k < N; k++)
    if (!(fabsf(v[k]) < INFINITY)) v[k] = 0.f;
  const unsigned active = __activemask();
  const unsigned peers = __match_any_sync(active, (unsigned long long)key);
  float s[N];
#pragma unroll
  for (int k = 0; k < N; k++) s[k] = 0.f;
  for (unsigned m = peers; m; m &= m - 1) {
    const int src = __ffs(m) - 1;
#pragma unroll
    for (int k = 0; k < N; k++) s[k] += __shfl_sync(peers, v[k], src);
  }
  if ((int)(threadIdx.x & 31u) == __ffs(peers) - 1) {
#pragma unroll
    for (int k = 0; k < N; k++)
      if (s[k] != 0.f) atomicAdd(&base[key * N + k], s[k]);
  }
}

// Gradient contributions of one shaded vertex (the detached estimator of
// adjoint.cu), prepared when the vertex is shaded and applied when its
// shadow rays have been traced.  With thr = path throughput before the
// vertex, dl = d loss / d sample radiance, Lt = the sample's total radiance
// and Lb = the radiance gathered before the vertex, the strategy terms
// resolve to L = Lb + thr (h + p + tB) (h = tH visible, w1*0 occluded; p
// alike), and the derivative of the radiance still to come, Lt - L,
// through the vertex's BRDF f is (Lt - L) df / f per channel.  Every
// parameter's derivative is therefore affine in the two visibility bits:
//   g = K0 + vH dH + vP dP,
// with K0 taken at vH = vP = 0.  The coefficients are stored per path
// (5 float4: K0, dH, dP for the 5 material parameters, the material slot
// or -1 when the sample has no adjoint, the env-texel gradient and texel)
// and apply_vertex_gradient adds g to g_mat[5 * material + k] and, when the
// env ray was visible, the texel's to g_env[3 * texel + c].
__device__ __forceinline__ void vertex_grad_coeffs(const DevScene& S, const VertexShade& V, f3 thr, f3 dl, f3 Lt,
                                                   f3 Lb, float4* out) {
  if (dl.x == 0.f && dl.y == 0.f && dl.z == 0.f) {
    out[3] = make_float4(0.f, 0.f, 0.f, __int_as_float(-1));
    return;
  }
  const DevMaterial& M = S.mats[V.mat];
  const f3 f = V.f, fH = V.fH, eH = V.eH;
  const bool ca = M.albedo_tex < 0, cr = M.roughness_tex < 0, cm = M.metallic_tex < 0;
  const bool dm = cm && V.metal_in > 0.f, dr = cr && V.rough_in > 0.f;
  const DisneyCtx& C = V.C;
  // strategy weights per channel: C_c = thr_c * (kH_c fH_c + kP_c fP_c + kB_c f_c)
  const f3 kH = eH * (V.cosH / V.hdriPdf * V.w1);
  const f3 kB = V.hd.emission * (V.ndl / V.brdfPdf * V.w3);
  const f3 kP = V.has_pt ? V.plv * (V.cosP / V.pointPdf * V.w2) : mk1(0.f);
  const f3 wd = mk(dl.x * thr.x, dl.y * thr.y, dl.z * thr.z);
  // (Lt - L) / f split into its visibility-free part and the h, p parts
  const float oH = V.w1 * 0.0f, oP = V.w2 * 0.0f;
  const f3 q = mk(f.x != 0.f ? dl.x / f.x : 0.f, f.y != 0.f ? dl.y / f.y : 0.f, f.z != 0.f ? dl.z / f.z : 0.f);
  const f3 r0 = mk(q.x * (Lt.x - Lb.x - thr.x * (V.tB.x + oH + oP)), q.y * (Lt.y - Lb.y - thr.y * (V.tB.y + oH + oP)),
                   q.z * (Lt.z - Lb.z - thr.z * (V.tB.z + oH + oP)));
  const f3 rH = mk(-q.x * thr.x * (V.tH.x - oH), -q.y * thr.y * (V.tH.y - oH), -q.z * thr.z * (V.tH.z - oH));
  const f3 rP = mk(-q.x * thr.x * (V.tP.x - oP), -q.y * thr.y * (V.tP.y - oP), -q.z * thr.z * (V.tP.z - oP));
  float k0[kParams] = {0.f, 0.f, 0.f, 0.f, 0.f}, kh[kParams] = {0.f, 0.f, 0.f, 0.f, 0.f},
        kp[kParams] = {0.f, 0.f, 0.f, 0.f, 0.f};
  if (ca || dm || dr) {
    const f3 uB = mk(wd.x * kB.x + r0.x, wd.y * kB.y + r0.y, wd.z * kB.z + r0.z);
    const f3 uH = mk(wd.x * kH.x, wd.y * kH.y, wd.z * kH.z);
    const f3 uP = mk(wd.x * kP.x, wd.y * kP.y, wd.z * kP.z);
    // per parameter k, with g, gh, gp its BRDF derivative for the sampled,
    // env and light directions:
    //   k0 = chain * (uB . g), kh = chain * (rH . g + uH . gh),
    //   kp = chain * (rP . g + uP . gp).
    // The three derivative evaluations run in one loop (one copy of the
    // code; this kernel is bound by instruction fetch), the sums formed in
    // the same order as written out.
    float s0[kParams], sh[kParams], sp[kParams];
#pragma unroll 1
    for (int j = 0; j < 3; j++) {
      EvalGrad E;
      E.dA[0] = E.dA[1] = E.dA[2] = E.dM = E.dR = mk1(0.f);
      if (j < 2 || V.has_pt) E = disney_eval_grad(V.hd, C, j == 0 ? V.dir : (j == 1 ? V.dH : V.dP));
#pragma unroll
      for (int k = 0; k < kParams; k++) {
        const f3 g = k < 3 ? E.dA[k] : (k == 3 ? E.dR : E.dM);
        if (j == 0) {
          s0[k] = dot(uB, g);
          sh[k] = dot(rH, g);
          sp[k] = dot(rP, g);
        } else if (j == 1) {
          sh[k] = sh[k] + dot(uH, g);
        } else {
          sp[k] = sp[k] + dot(uP, g);
        }
      }
    }
    auto put = [&](int k, float chain) {
      k0[k] = chain * s0[k];
      kh[k] = chain * sh[k];
      kp[k] = chain * sp[k];
    };
    if (ca)
#pragma unroll
      for (int j = 0; j < 3; j++) put(j, 1.0f);
    // d x^2.2 / dx = 2.2 x^1.2 = 2.2 x^2.2 / x, x^2.2 being the remapped
    // value the vertex already holds (x > 0 here): no further powf in this
    // instruction-fetch-bound kernel
    if (dr) put(3, 2.2f * (V.hd.roughness / V.rough_in));
    if (dm) put(4, 2.2f * (V.hd.metallic / V.metal_in));
  }
  const float sH = V.cosH / V.hdriPdf * V.w1;
  out[0] = make_float4(k0[0], k0[1], k0[2], k0[3]);
  out[1] = make_float4(k0[4], kh[0], kh[1], kh[2]);
  out[2] = make_float4(kh[3], kh[4], kp[0], kp[1]);
  out[3] = make_float4(kp[2], kp[3], kp[4], __int_as_float(V.mat));
  out[4] = make_float4(wd.x * fH.x * sH, wd.y * fH.y * sH, wd.z * fH.z * sH, __int_as_float((int32_t)V.env_texel));
}

__device__ __forceinline__ void apply_vertex_gradient(const float4* c, bool vH, bool vP, float* g_mat, float* g_env) {
  const int32_t mat = __float_as_int(c[3].w);
  if (mat < 0) return;
  const float h = vH ? 1.f : 0.f, p = vP ? 1.f : 0.f;
  float gk[kParams] = {c[0].x + h * c[1].y + p * c[2].z, c[0].y + h * c[1].z + p * c[2].w,
                       c[0].z + h * c[1].w + p * c[3].x, c[0].w + h * c[2].x + p * c[3].y,
                       c[1].x + h * c[2].y + p * c[3].z};
  agg_add<kParams>(g_mat, mat, gk);
  if (vH) {
    float ge[3] = {c[4].x, c[4].y, c[4].z};
    agg_add<3>(g_env, __float_as_int(c[4].w), ge);
  }
}

}  // namespace er
