// Derivatives of the per-vertex shading for the path-replay adjoint, shared
// by the replay kernels (adjoint.cu) and the gradient variant of the
// wavefront shade stage (render.cu).
#pragma once

#include "vertex.cuh"

namespace er {

// ---------------------------------------------------------------- duals --
// Forward-mode dual number carrying the derivative along one material
// parameter (the replay loops over the kParams parameters of a vertex).
constexpr int kNP = 1;
constexpr int kParams = 5;  // albedo r, g, b, roughness, metallic

struct Dual {
  float v;
  float d[kNP];
};

__device__ __forceinline__ Dual dconst(float v) {
  Dual r;
  r.v = v;
#pragma unroll
  for (int k = 0; k < kNP; k++) r.d[k] = 0.f;
  return r;
}
__device__ __forceinline__ Dual operator+(Dual a, Dual b) {
  Dual r;
  r.v = a.v + b.v;
#pragma unroll
  for (int k = 0; k < kNP; k++) r.d[k] = a.d[k] + b.d[k];
  return r;
}
__device__ __forceinline__ Dual operator-(Dual a, Dual b) {
  Dual r;
  r.v = a.v - b.v;
#pragma unroll
  for (int k = 0; k < kNP; k++) r.d[k] = a.d[k] - b.d[k];
  return r;
}
__device__ __forceinline__ Dual operator*(Dual a, Dual b) {
  Dual r;
  r.v = a.v * b.v;
#pragma unroll
  for (int k = 0; k < kNP; k++) r.d[k] = a.d[k] * b.v + a.v * b.d[k];
  return r;
}
__device__ __forceinline__ Dual operator/(Dual a, Dual b) {
  Dual r;
  r.v = a.v / b.v;
  float ib = 1.0f / b.v;
#pragma unroll
  for (int k = 0; k < kNP; k++) r.d[k] = (a.d[k] - r.v * b.d[k]) * ib;
  return r;
}
__device__ __forceinline__ Dual operator+(Dual a, float b) { a.v += b; return a; }
__device__ __forceinline__ Dual operator+(float b, Dual a) { a.v += b; return a; }
__device__ __forceinline__ Dual operator-(float b, Dual a) {
  Dual r;
  r.v = b - a.v;
#pragma unroll
  for (int k = 0; k < kNP; k++) r.d[k] = -a.d[k];
  return r;
}
__device__ __forceinline__ Dual operator*(Dual a, float b) {
  a.v *= b;
#pragma unroll
  for (int k = 0; k < kNP; k++) a.d[k] *= b;
  return a;
}
__device__ __forceinline__ Dual operator*(float b, Dual a) { return a * b; }
__device__ __forceinline__ Dual operator/(Dual a, float b) { return a * (1.0f / b); }
__device__ __forceinline__ Dual operator/(float a, Dual b) { return dconst(a) / b; }
__device__ __forceinline__ Dual dsqrt(Dual a) {
  Dual r;
  r.v = sqrtf(a.v);
  float k2 = r.v > 0.f ? 0.5f / r.v : 0.f;
#pragma unroll
  for (int k = 0; k < kNP; k++) r.d[k] = a.d[k] * k2;
  return r;
}
// maxf_(lo, a) of the reference: lo > a ? lo : a
__device__ __forceinline__ Dual dmax_lo(float lo, Dual a) { return lo > a.v ? dconst(lo) : a; }
__device__ __forceinline__ Dual dlerp(Dual a, Dual b, Dual c) { return a + c * (b - a); }

struct D3 {
  Dual x, y, z;
};
__device__ __forceinline__ D3 d3(Dual a) { return D3{a, a, a}; }
__device__ __forceinline__ D3 d3c(float a) { return d3(dconst(a)); }
__device__ __forceinline__ D3 operator+(D3 a, D3 b) { return D3{a.x + b.x, a.y + b.y, a.z + b.z}; }
__device__ __forceinline__ D3 operator*(D3 a, Dual s) { return D3{a.x * s, a.y * s, a.z * s}; }
__device__ __forceinline__ D3 operator*(D3 a, float s) { return D3{a.x * s, a.y * s, a.z * s}; }
__device__ __forceinline__ D3 dlerp3(D3 a, D3 b, Dual c) { return D3{dlerp(a.x, b.x, c), dlerp(a.y, b.y, c), dlerp(a.z, b.z, c)}; }
__device__ __forceinline__ D3 dlerp3(D3 a, D3 b, float c) {
  return D3{dlerp(a.x, b.x, dconst(c)), dlerp(a.y, b.y, dconst(c)), dlerp(a.z, b.z, dconst(c))};
}

__device__ __forceinline__ Dual gtr2_aniso_d(float NDotH, float HDotX, float HDotY, Dual ax, Dual ay) {
  Dual a = HDotX / ax, b = HDotY / ay;
  Dual c = a * a + b * b + NDotH * NDotH;
  return 1.0f / (ER_PI * ax * ay * c * c);
}
__device__ __forceinline__ Dual smith_ggx_aniso_d(float NDotV, float VDotX, float VDotY, Dual ax, Dual ay) {
  Dual a = VDotX * ax, b = VDotY * ay;
  return 1.0f / (NDotV + dsqrt(a * a + b * b + NDotV * NDotV));
}

// DisneyEval (Disney.hpp:179-253) with albedo, roughness and metallic as
// duals; the other parameters and all directions are constants.
static __device__ D3 disney_eval_d(const HitData& hd, D3 Cdlin, Dual rough, Dual metal, const DisneyCtx& c, f3 L) {
  if (!(hd.transmission < 1.0f && dot(c.N, L) > 0.0f && dot(c.N, c.V) > 0.0f)) return d3c(0.f);
  f3 H = normalized(L + c.V);
  float NDotL = fabsf(dot(c.N, L));
  float NDotV = fabsf(dot(c.N, c.V));
  float NDotH = fabsf(dot(c.N, H));
  float LDotH = fabsf(dot(L, H));
  Dual Cdlum = Cdlin.x * 0.3f + Cdlin.y * 0.6f + Cdlin.z * 0.1f;
  D3 Ctint = Cdlum.v > 0.0f ? D3{Cdlin.x / Cdlum, Cdlin.y / Cdlum, Cdlin.z / Cdlum} : d3c(1.0f);
  D3 Cspec0 = dlerp3(dlerp3(d3c(1.0f), Ctint, hd.specularTint) * (hd.specular * 0.08f), Cdlin, metal);
  D3 Csheen = dlerp3(d3c(1.0f), Ctint, hd.sheenTint);
  float FL = schlick(NDotL), FV = schlick(NDotV);
  Dual Fd90 = 0.5f + rough * (2.0f * LDotH * LDotH);
  Dual Fd = dlerp(dconst(1.0f), Fd90, dconst(FL)) * dlerp(dconst(1.0f), Fd90, dconst(FV));
  Dual Fss90 = rough * (LDotH * LDotH);
  Dual Fss = dlerp(dconst(1.0f), Fss90, dconst(FL)) * dlerp(dconst(1.0f), Fss90, dconst(FV));
  Dual ss = (Fss * (1.0f / (NDotL + NDotV) - 0.5f) + 0.5f) * 1.25f;
  float aspect = sqrtf(1.0f - hd.anisotropic * 0.9f);
  Dual ax = dmax_lo(0.001f, rough / aspect), ay = dmax_lo(0.001f, rough * aspect);
  Dual Ds = gtr2_aniso_d(NDotH, dot(H, c.T), dot(H, c.B), ax, ay);
  float FH = schlick(LDotH);
  D3 Fs = dlerp3(Cspec0, d3c(1.0f), FH);
  Dual Gs = smith_ggx_aniso_d(NDotL, dot(L, c.T), dot(L, c.B), ax, ay) *
            smith_ggx_aniso_d(NDotV, dot(c.V, c.T), dot(c.V, c.B), ax, ay);
  D3 Fsheen = Csheen * (FH * hd.sheen);
  float Dr = gtr1(NDotH, c.clearcoatAlpha);
  float Fr = lerpf_(0.04f, 1.0f, FH);
  float Gr = smith_ggx(NDotL, 0.25f) * smith_ggx(NDotV, 0.25f);
  Dual kd = dlerp(Fd, ss, dconst(hd.subsurface)) * (1.0f / ER_PI);
  D3 diff = (Cdlin * kd + Fsheen) * (1.0f - metal);
  D3 spec = Fs * (Gs * Ds);
  float cc = 0.25f * hd.clearcoat * Gr * Fr * Dr;
  return diff + spec + d3c(cc);
}

// Closed-form partials of DisneyEval (Disney.hpp:179-253) in albedo and
// metallic.  With GD = Gs * Ds, A the specular mix and Ctint = Cdlin /
// Cdlum (Cdlum = 0.3 r + 0.6 g + 0.1 b):
//   f_c = (Cdlin_c kd + Fsheen_c)(1 - m) + (Cspec0_c (1 - FH) + FH) GD + cc
//   Cspec0_c = X_c (1 - m) + m Cdlin_c,  X_c = (1 + sT (Ctint_c - 1)) 0.08 s
//   Fsheen_c = (1 + shT (Ctint_c - 1)) FH sheen
// so  d f_c / d Cdlin_j = [c = j] (kd (1 - m) + GD (1 - FH) m)
//                         + d Ctint_c / d Cdlin_j (1 - m)(shT FH sheen + GD (1 - FH) sT 0.08 s)
// with d Ctint_c / d Cdlin_j = ([c = j] - Ctint_c w_j) / Cdlum (zero when
// Cdlum <= 0, where Ctint is the constant 1), and
//   d f_c / d m = -(Cdlin_c kd + Fsheen_c) + GD (1 - FH)(Cdlin_c - X_c).
// dA[j] holds d f / d Cdlin_j for the three channels.
struct EvalGrad {
  f3 dA[3];
  f3 dM;
};
__device__ __forceinline__ EvalGrad disney_eval_grad(const HitData& hd, const DisneyCtx& c, f3 L) {
  EvalGrad g;
  g.dA[0] = g.dA[1] = g.dA[2] = g.dM = mk1(0.f);
  if (!(hd.transmission < 1.0f && dot(c.N, L) > 0.0f && dot(c.N, c.V) > 0.0f)) return g;
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
  const float Ds = gtr2_aniso(NDotH, dot(H, c.T), dot(H, c.B), c.ax, c.ay);
  const float FH = schlick(LDotH);
  const float Gs = smith_ggx_aniso(NDotL, dot(L, c.T), dot(L, c.B), c.ax, c.ay) *
                   smith_ggx_aniso(NDotV, dot(c.V, c.T), dot(c.V, c.B), c.ax, c.ay);
  const float GD = Gs * Ds;
  const float kd = (1.0f / ER_PI) * lerpf_(Fd, ss, hd.subsurface);
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
// adjoint.cu): thr = path throughput before the vertex, dl = d loss / d
// sample radiance, (Lx, Ly, Lz) = radiance gathered up to and including
// this vertex, Lt = the sample's total radiance, vH / vP = visibility of
// the env and point-light shadow rays.  Material gradients go to
// g_mat[5 * material + k] (global or shared memory), env gradients to
// g_env[3 * texel + c].
__device__ __forceinline__ void vertex_gradient(const DevScene& S, const VertexShade& V, f3 thr, f3 dl, f3 Lt,
                                                float Lx, float Ly, float Lz, bool vH, bool vP, float* g_mat,
                                                float* g_env) {
  const DevMaterial& M = S.mats[V.mat];
  const f3 f = V.f, fH = V.fH, eH = V.eH;
  const bool ca = M.albedo_tex < 0, cr = M.roughness_tex < 0, cm = M.metallic_tex < 0;
  const DisneyCtx& C = V.C;
  // strategy weights per channel: C_c = thr_c * (kH_c fH_c + kP_c fP_c + kB_c f_c)
  const f3 kH = vH ? eH * (V.cosH / V.hdriPdf * V.w1) : mk1(0.f);
  const f3 kB = V.hd.emission * (V.ndl / V.brdfPdf * V.w3);
  const f3 kP = (V.has_pt && vP) ? V.plv * (V.cosP / V.pointPdf * V.w2) : mk1(0.f);
  const f3 wd = mk(dl.x * thr.x, dl.y * thr.y, dl.z * thr.z);
  // radiance still to come carries f through the throughput
  const f3 La = mk(Lt.x - Lx, Lt.y - Ly, Lt.z - Lz);
  const f3 ra = mk(f.x != 0.f ? dl.x * La.x / f.x : 0.f, f.y != 0.f ? dl.y * La.y / f.y : 0.f,
                   f.z != 0.f ? dl.z * La.z / f.z : 0.f);
  // albedo and metallic: closed-form partials of the three evaluations
  float gk[kParams] = {0.f, 0.f, 0.f, 0.f, 0.f};
  const bool use_p = V.has_pt && vP;
  const bool dm = cm && V.metal_in > 0.f;
  if (ca || dm) {
    const f3 uB = mk(wd.x * kB.x + ra.x, wd.y * kB.y + ra.y, wd.z * kB.z + ra.z);
    const f3 uH = mk(wd.x * kH.x, wd.y * kH.y, wd.z * kH.z);
    const f3 uP = mk(wd.x * kP.x, wd.y * kP.y, wd.z * kP.z);
    const EvalGrad G = disney_eval_grad(V.hd, C, V.dir);
    const EvalGrad GH = disney_eval_grad(V.hd, C, V.dH);
    EvalGrad GP;
    GP.dA[0] = GP.dA[1] = GP.dA[2] = GP.dM = mk1(0.f);
    if (use_p) GP = disney_eval_grad(V.hd, C, V.dP);
    if (ca)
#pragma unroll
      for (int j = 0; j < 3; j++) gk[j] = dot(uB, G.dA[j]) + dot(uH, GH.dA[j]) + dot(uP, GP.dA[j]);
    if (dm) gk[4] = 2.2f * powf(V.metal_in, 1.2f) * (dot(uB, G.dM) + dot(uH, GH.dM) + dot(uP, GP.dM));
  }
  // roughness: a single-partial dual through the three evaluations
  if (cr && V.rough_in > 0.f) {
    D3 alb{dconst(V.hd.albedo.x), dconst(V.hd.albedo.y), dconst(V.hd.albedo.z)};
    Dual rg = dconst(V.hd.roughness), mt = dconst(V.hd.metallic);
    rg.d[0] = 2.2f * powf(V.rough_in, 1.2f);
    D3 Df = disney_eval_d(V.hd, alb, rg, mt, C, V.dir);
    D3 DfH = disney_eval_d(V.hd, alb, rg, mt, C, V.dH);
    float acc = wd.x * (kH.x * DfH.x.d[0] + kB.x * Df.x.d[0]) + wd.y * (kH.y * DfH.y.d[0] + kB.y * Df.y.d[0]) +
                wd.z * (kH.z * DfH.z.d[0] + kB.z * Df.z.d[0]) + ra.x * Df.x.d[0] + ra.y * Df.y.d[0] + ra.z * Df.z.d[0];
    if (use_p) {
      D3 DfP = disney_eval_d(V.hd, alb, rg, mt, C, V.dP);
      acc += wd.x * kP.x * DfP.x.d[0] + wd.y * kP.y * DfP.y.d[0] + wd.z * kP.z * DfP.z.d[0];
    }
    gk[3] = acc;
  }
  agg_add<kParams>(g_mat, V.mat, gk);
  if (vH) {
    float s = V.cosH / V.hdriPdf * V.w1;
    float ge[3] = {wd.x * fH.x * s, wd.y * fH.y * s, wd.z * fH.z * s};
    agg_add<3>(g_env, V.env_texel, ge);
  }
}

}  // namespace er
