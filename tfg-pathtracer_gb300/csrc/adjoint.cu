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
// One thread owns one pixel and walks its samples in order.  Per sample it
// re-traces the path from its counter-based random numbers twice: once for
// the sample's radiance L (which sets the clamp mask and the NaN drop of the
// accumulation, kernel.cu:445-449), once to scatter gradients.  At vertex i
// the replay knows the throughput beta_i, the radiance L_<=i gathered so far
// and therefore the radiance still to come, L - L_<=i, which carries vertex
// i's throughput factor f_i |N.L| / pdf_i: its derivative is
// (L - L_<=i) * df_i / f_i per channel.  Nothing per vertex is stored.
//
// The same walk without gradients is a complete forward render
// (er_render_replay): with the evaluation parameters equal to the scene's
// it reproduces er_render bit for bit; with other evaluation parameters it
// is the detached estimator itself, which finite differences of the
// gradient are checked against.
#include <cmath>
#include <cstring>
#include <vector>

#include "internal.h"
#include "vertex.cuh"

namespace er {
namespace {

// ---------------------------------------------------------------- duals --
// Forward-mode dual number over the 5 material parameters of one vertex.
constexpr int kNP = 5;

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
__device__ D3 disney_eval_d(const HitData& hd, D3 Cdlin, Dual rough, Dual metal, const DisneyCtx& c, f3 L) {
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
  int32_t smem_grad;         // material gradients accumulated in shared memory
  uint32_t* err;
};

template <int MODE, bool Q8>
__device__ __forceinline__ void trace_one(const DevScene& S, Traverser<MODE, Q8, false>& tr, int2* sstk,
                                          uint32_t* err) {
  int2 lstk[kLocalStack];
  TravStats st{0, 0, 0};
  // every node is expanded at most once and every leaf tested at most once
  // per ray, so the walk is bounded by twice the node count
  for (int64_t it = 0; !tr.done; it++) {
    if (tr.leaf != 0) tr.leaf_step(S, sstk, lstk, st, err);
    else if (tr.node >= 0) tr.node_step(S, sstk, lstk, st, err);
    else tr.finish();
    if (it > 8 * S.n_nodes + 64) {
      atomicOr(err, 4u);
      tr.done = true;
    }
  }
}

// Adds v to gradient slot i (shared-memory copy when it fits).
__device__ __forceinline__ void add_mat(const ReplayArgs& A, float* sg, int32_t i, float v) {
  if (v == 0.f || !(fabsf(v) < INFINITY)) return;
  if (A.smem_grad) atomicAdd(&sg[i], v);
  else atomicAdd(&A.g_mat[i], v);
}

// One sample of pixel (x, y).  GRAD = false: returns the sample's radiance
// and vertex count.  GRAD = true: the replay, given the sample's radiance
// Lt and its adjoint dl (d loss / d radiance).
template <bool Q8, bool GRAD, bool EVAL>
__device__ f3 walk(const DevScene& S, const ReplayArgs& A, int2* sstk, float* sg, int32_t x, int32_t y, uint32_t idx,
                   uint32_t sample, f3 Lt, f3 dl, int32_t* bounces) {
  const WaveParams& P = A.P;
  uint4 ra = philox(make_uint4(idx, sample, 0u, 0u), P.k0, P.k1);
  uint4 rb = philox(make_uint4(idx, sample, 1u, 0u), P.k0, P.k1);
  f3 o, d;
  camera_ray(S.cam, x, y, u01(ra.x), u01(ra.y), u01(ra.z), u01(ra.w), u01(rb.x), o, d);
  f3 thr = mk1(1.0f);
  float Lx = 0.f, Ly = 0.f, Lz = 0.f;
  *bounces = P.max_depth;
  for (int32_t bounce = 0; bounce < P.max_depth; bounce++) {
    Traverser<kClosest, Q8, false> tr;
    tr.init(S, o, d, mk1(0.f), 0.f);
    trace_one(S, tr, sstk, A.err);
    if (tr.slot < 0) {
      // kernel.cu:414-419
      int64_t te;
      f3 e = escape_radiance(S, d, &te);
      if (EVAL && A.eval_env) e = mk(A.eval_env[3 * te], A.eval_env[3 * te + 1], A.eval_env[3 * te + 2]);
      Lx = __fadd_rn(Lx, __fmul_rn(e.x, thr.x));
      Ly = __fadd_rn(Ly, __fmul_rn(e.y, thr.y));
      Lz = __fadd_rn(Lz, __fmul_rn(e.z, thr.z));
      if (GRAD) {
        atomicAdd(&A.g_env[3 * te], dl.x * thr.x);
        atomicAdd(&A.g_env[3 * te + 1], dl.y * thr.y);
        atomicAdd(&A.g_env[3 * te + 2], dl.z * thr.z);
      }
      *bounces = bounce;
      break;
    }
    VertexShade V;
    shade_vertex(S, P.flags, P.k0, P.k1, idx, sample, bounce, o, d, tr.t, tr.u, tr.v, tr.slot, V);
    Traverser<kAny, Q8, false> te;
    te.init(S, V.env_o, V.env_d, mk1(0.f), 0.f);
    trace_one(S, te, sstk, A.err);
    const bool vH = !te.occluded;
    bool vP = true;
    if (V.has_pt) {
      Traverser<kPoint, Q8, false> tp;
      tp.init(S, V.pt_o, V.pt_d, V.pos, V.dist);
      trace_one(S, tp, sstk, A.err);
      vP = !tp.occluded;
    }
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
    if (GRAD) {
      // d C_i: BRDF values of the three strategies, env texel of the NEE
      const bool ca = M.albedo_tex < 0, cr = M.roughness_tex < 0, cm = M.metallic_tex < 0;
      D3 alb = d3c(0.f);
      alb.x = dconst(V.hd.albedo.x);
      alb.y = dconst(V.hd.albedo.y);
      alb.z = dconst(V.hd.albedo.z);
      if (ca) { alb.x.d[0] = 1.f; alb.y.d[1] = 1.f; alb.z.d[2] = 1.f; }
      Dual rg = dconst(V.hd.roughness), mt = dconst(V.hd.metallic);
      if (cr && V.rough_in > 0.f) rg.d[3] = 2.2f * powf(V.rough_in, 1.2f);
      if (cm && V.metal_in > 0.f) mt.d[4] = 2.2f * powf(V.metal_in, 1.2f);
      const DisneyCtx& C = V.C;
      D3 Df = disney_eval_d(V.hd, alb, rg, mt, C, V.dir);
      D3 DfH = disney_eval_d(V.hd, alb, rg, mt, C, V.dH);
      // strategy weights per channel: C_c = thr_c * (kH_c fH_c + kP_c fP_c + kB_c f_c)
      f3 kH = vH ? eH * (V.cosH / V.hdriPdf * V.w1) : mk1(0.f);
      f3 kB = V.hd.emission * (V.ndl / V.brdfPdf * V.w3);
      f3 wd = mk(dl.x * thr.x, dl.y * thr.y, dl.z * thr.z);
      float gk[kNP];
#pragma unroll
      for (int k = 0; k < kNP; k++)
        gk[k] = wd.x * (kH.x * DfH.x.d[k] + kB.x * Df.x.d[k]) + wd.y * (kH.y * DfH.y.d[k] + kB.y * Df.y.d[k]) +
                wd.z * (kH.z * DfH.z.d[k] + kB.z * Df.z.d[k]);
      if (V.has_pt && vP) {
        D3 DfP = disney_eval_d(V.hd, alb, rg, mt, C, V.dP);
        f3 kP = V.plv * (V.cosP / V.pointPdf * V.w2);
#pragma unroll
        for (int k = 0; k < kNP; k++)
          gk[k] += wd.x * kP.x * DfP.x.d[k] + wd.y * kP.y * DfP.y.d[k] + wd.z * kP.z * DfP.z.d[k];
      }
      // radiance still to come carries f_i through the throughput
      f3 La = mk(Lt.x - Lx, Lt.y - Ly, Lt.z - Lz);
      f3 ra = mk(f.x != 0.f ? dl.x * La.x / f.x : 0.f, f.y != 0.f ? dl.y * La.y / f.y : 0.f,
                 f.z != 0.f ? dl.z * La.z / f.z : 0.f);
#pragma unroll
      for (int k = 0; k < kNP; k++) {
        gk[k] += ra.x * Df.x.d[k] + ra.y * Df.y.d[k] + ra.z * Df.z.d[k];
        add_mat(A, sg, 5 * V.mat + k, gk[k]);
      }
      if (vH) {
        float s = V.cosH / V.hdriPdf * V.w1;
        int64_t t3 = 3 * V.env_texel;
        float a0 = wd.x * fH.x * s, a1 = wd.y * fH.y * s, a2 = wd.z * fH.z * s;
        if (a0 != 0.f && fabsf(a0) < INFINITY) atomicAdd(&A.g_env[t3], a0);
        if (a1 != 0.f && fabsf(a1) < INFINITY) atomicAdd(&A.g_env[t3 + 1], a1);
        if (a2 != 0.f && fabsf(a2) < INFINITY) atomicAdd(&A.g_env[t3 + 2], a2);
      }
    }
    thr = mk(__fmul_rn(thr.x, g.x), __fmul_rn(thr.y, g.y), __fmul_rn(thr.z, g.z));
    if (bounce + 1 >= P.max_depth) break;
    // kernel.cu:442
    o = xadd(V.pos, xscale(V.dir, 0.001f));
    d = xnormalize(V.dir);
  }
  return mk(Lx, Ly, Lz);
}

template <bool Q8, bool GRAD, bool EVAL>
__global__ void __launch_bounds__(kTravBlock) k_replay(DevScene S, ReplayArgs A) {
  __shared__ int2 stk[kSmemStack * kTravBlock];
  extern __shared__ float sg[];
  const WaveParams& P = A.P;
  if (GRAD && A.smem_grad) {
    for (int32_t i = threadIdx.x; i < 5 * A.n_mats; i += blockDim.x) sg[i] = 0.f;
    __syncthreads();
  }
  const int32_t pix = blockIdx.x * blockDim.x + threadIdx.x;
  if (pix < P.npix) {
    const int32_t x = pix % P.W, y = pix / P.W;
    const uint32_t idx = (uint32_t)(P.W * (P.H - y - 1) + x);  // kernel.cu:378
    if (!GRAD) {
      // forward render with accumulate_pixel's arithmetic
      uint32_t sa = 0, pc = 0;
      float4 bt = make_float4(0.f, 0.f, 0.f, 1.f);
      for (int32_t s = 0; s < P.spp_wave; s++) {
        int32_t nb;
        f3 L = walk<Q8, false, EVAL>(S, A, stk + threadIdx.x, sg, x, y, idx, (uint32_t)(P.sample_base + s),
                                     mk1(0.f), mk1(0.f), &nb);
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
      A.beauty[idx] = bt;
      A.samples[idx] = sa;
      A.pathcount[idx] = pc;
    } else {
      const uint32_t n = A.nvalid[idx];
      const float4 g4 = A.d_beauty[idx];
      if (n > 0 && (g4.x != 0.f || g4.y != 0.f || g4.z != 0.f)) {
        const float inv_n = 1.0f / (float)n;
        for (int32_t s = 0; s < P.spp_wave; s++) {
          int32_t nb;
          const uint32_t sample = (uint32_t)(P.sample_base + s);
          f3 L = walk<Q8, false, false>(S, A, stk + threadIdx.x, sg, x, y, idx, sample, mk1(0.f), mk1(0.f), &nb);
          if (isnan(L.x) || isnan(L.y) || isnan(L.z)) continue;  // dropped by the accumulation
          // clamp(L, 0, 10) passes the derivative only strictly inside
          f3 dl = mk((L.x > 0.f && L.x < 10.f) ? g4.x * inv_n : 0.f, (L.y > 0.f && L.y < 10.f) ? g4.y * inv_n : 0.f,
                     (L.z > 0.f && L.z < 10.f) ? g4.z * inv_n : 0.f);
          if (dl.x == 0.f && dl.y == 0.f && dl.z == 0.f) continue;
          walk<Q8, true, false>(S, A, stk + threadIdx.x, sg, x, y, idx, sample, L, dl, &nb);
        }
      }
    }
  }
  if (GRAD && A.smem_grad) {
    __syncthreads();
    for (int32_t i = threadIdx.x; i < 5 * A.n_mats; i += blockDim.x)
      if (sg[i] != 0.f) atomicAdd(&A.g_mat[i], sg[i]);
  }
}

constexpr int kMaxSmemGrad = 8192;  // floats of shared memory for material gradients

template <bool GRAD, bool EVAL>
er_status launch_replay(er_scene* s, const ReplayArgs& A) {
  const int32_t npix = A.P.npix;
  const unsigned blocks = (unsigned)((npix + kTravBlock - 1) / kTravBlock);
  const size_t smem = (GRAD && A.smem_grad) ? (size_t)5 * A.n_mats * sizeof(float) : 0;
  if (s->dev.use_q8) k_replay<true, GRAD, EVAL><<<blocks, kTravBlock, smem, s->stream>>>(s->dev, A);
  else k_replay<false, GRAD, EVAL><<<blocks, kTravBlock, smem, s->stream>>>(s->dev, A);
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
  if ((o->flags & ER_RENDER_ENV_ALIAS)) {
    er_status st = build_env_alias(s);
    if (st != ER_OK) return st;
  }
  return ER_OK;
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
}

extern "C" er_status er_scene_set_params(er_scene* s, const float* materials, const float* env, uint32_t flags) {
  if (!s) return fail(ER_ERR_INVALID_ARG, "scene is NULL");
  ER_CUDA(cudaSetDevice(s->device));
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
    s->dev.alias_idx = nullptr;  // rebuilt on next use
    s->dev.alias_thresh = nullptr;
  }
  return ER_OK;
}

extern "C" er_status er_render_replay(er_scene* s, const er_render_opts* o, const float* eval_materials,
                                      const float* eval_env, float* beauty, uint32_t* samples, uint32_t* pathcount) {
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
    st = (em || ee) ? launch_replay<false, true>(s, A) : launch_replay<false, false>(s, A);
    if (st != ER_OK) return st;
  }
  if (!dev) {
    ER_CUDA(cudaMemcpyAsync(beauty, A.beauty, np * 16, cudaMemcpyDeviceToHost, s->stream));
    ER_CUDA(cudaMemcpyAsync(samples, A.samples, np * 4, cudaMemcpyDeviceToHost, s->stream));
    ER_CUDA(cudaMemcpyAsync(pathcount, A.pathcount, np * 4, cudaMemcpyDeviceToHost, s->stream));
  }
  ER_CUDA(cudaStreamSynchronize(s->stream));
  return check_device_error(s);
}

extern "C" er_status er_backward(er_scene* s, const er_render_opts* o, const float* d_beauty, const uint32_t* samples,
                                 float* grad_materials, float* grad_env, er_render_stats* stats) {
  er_status st = check_replay_opts(s, o);
  if (st != ER_OK) return st;
  if (!d_beauty || !samples) return fail(ER_ERR_INVALID_ARG, "NULL input");
  const bool dev = o->flags & ER_RENDER_DEVICE_OUT;
  ReplayArgs A{};
  A.P = replay_params(s, o);
  A.n_mats = s->dev.n_mats;
  A.err = s->err_word;
  A.smem_grad = 5 * A.n_mats <= kMaxSmemGrad;
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
  ER_CUDA(cudaEventRecord(s->ev0, s->stream));
  if (np > 0 && (st = launch_replay<true, false>(s, A)) != ER_OK) return st;
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
    stats->kernel_launches = np > 0 ? 1 : 0;
  }
  return ER_OK;
}
