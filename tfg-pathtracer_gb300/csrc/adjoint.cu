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
// accumulation, kernel.cu:445-449).  Then one thread per path re-traces the
// path from its counter-based random numbers and scatters gradients.  At
// vertex i the replay knows the throughput beta_i, the radiance L_<=i
// gathered so far and therefore the radiance still to come, L - L_<=i,
// which carries vertex i's throughput factor f_i |N.L| / pdf_i: its
// derivative is (L - L_<=i) * df_i / f_i per channel.  Nothing per vertex is
// stored.  Material gradients collect in shared memory per block of the
// persistent grid, env gradients with global atomics.
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

// One sample of pixel (x, y), called by all 32 lanes of the warp together
// (active = false: a lane without a path this round).  GRAD = false:
// returns the sample's radiance and vertex count.  GRAD = true: the replay,
// given the sample's radiance Lt and its adjoint dl (d loss / d radiance).
template <bool Q8, bool GRAD, bool EVAL>
__device__ f3 walk(const DevScene& S, const ReplayArgs& A, int2* sstk, float* sg, bool active, int32_t x, int32_t y,
                   uint32_t idx, uint32_t sample, f3 Lt, f3 dl, int32_t* bounces) {
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
      if (GRAD) {
        float ge[3] = {dl.x * thr.x, dl.y * thr.y, dl.z * thr.z};
        agg_add<3>(A.g_env, te, ge);
      }
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
    if (GRAD) {
      // d C_i: BRDF values of the three strategies, env texel of the NEE.
      // One parameter at a time (single-partial duals keep registers low).
      const bool ca = M.albedo_tex < 0, cr = M.roughness_tex < 0, cm = M.metallic_tex < 0;
      const DisneyCtx& C = V.C;
      // strategy weights per channel: C_c = thr_c * (kH_c fH_c + kP_c fP_c + kB_c f_c)
      const f3 kH = vH ? eH * (V.cosH / V.hdriPdf * V.w1) : mk1(0.f);
      const f3 kB = V.hd.emission * (V.ndl / V.brdfPdf * V.w3);
      const f3 kP = (V.has_pt && vP) ? V.plv * (V.cosP / V.pointPdf * V.w2) : mk1(0.f);
      const f3 wd = mk(dl.x * thr.x, dl.y * thr.y, dl.z * thr.z);
      // radiance still to come carries f_i through the throughput
      const f3 La = mk(Lt.x - Lx, Lt.y - Ly, Lt.z - Lz);
      const f3 ra = mk(f.x != 0.f ? dl.x * La.x / f.x : 0.f, f.y != 0.f ? dl.y * La.y / f.y : 0.f,
                       f.z != 0.f ? dl.z * La.z / f.z : 0.f);
      float gk[kParams];
#pragma unroll 1
      for (int k = 0; k < kParams; k++) {
        D3 alb{dconst(V.hd.albedo.x), dconst(V.hd.albedo.y), dconst(V.hd.albedo.z)};
        Dual rg = dconst(V.hd.roughness), mt = dconst(V.hd.metallic);
        bool seeded = false;
        if (k == 0 && ca) { alb.x.d[0] = 1.f; seeded = true; }
        if (k == 1 && ca) { alb.y.d[0] = 1.f; seeded = true; }
        if (k == 2 && ca) { alb.z.d[0] = 1.f; seeded = true; }
        if (k == 3 && cr && V.rough_in > 0.f) { rg.d[0] = 2.2f * powf(V.rough_in, 1.2f); seeded = true; }
        if (k == 4 && cm && V.metal_in > 0.f) { mt.d[0] = 2.2f * powf(V.metal_in, 1.2f); seeded = true; }
        float acc = 0.f;
        if (seeded) {
          D3 Df = disney_eval_d(V.hd, alb, rg, mt, C, V.dir);
          D3 DfH = disney_eval_d(V.hd, alb, rg, mt, C, V.dH);
          acc = wd.x * (kH.x * DfH.x.d[0] + kB.x * Df.x.d[0]) + wd.y * (kH.y * DfH.y.d[0] + kB.y * Df.y.d[0]) +
                wd.z * (kH.z * DfH.z.d[0] + kB.z * Df.z.d[0]) + ra.x * Df.x.d[0] + ra.y * Df.y.d[0] +
                ra.z * Df.z.d[0];
          if (V.has_pt && vP) {
            D3 DfP = disney_eval_d(V.hd, alb, rg, mt, C, V.dP);
            acc += wd.x * kP.x * DfP.x.d[0] + wd.y * kP.y * DfP.y.d[0] + wd.z * kP.z * DfP.z.d[0];
          }
        }
        gk[k] = acc;
      }
      agg_add<kParams>(A.smem_grad ? sg : A.g_mat, V.mat, gk);
      if (vH) {
        float s = V.cosH / V.hdriPdf * V.w1;
        float ge[3] = {wd.x * fH.x * s, wd.y * fH.y * s, wd.z * fH.z * s};
        agg_add<3>(A.g_env, V.env_texel, ge);
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
    f3 L = walk<Q8, false, EVAL>(S, A, stk + threadIdx.x, nullptr, valid, x, y, idx, (uint32_t)(P.sample_base + s),
                                 mk1(0.f), mk1(0.f), &nb);
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

#ifndef ER_BWD_MIN_BLOCKS
#define ER_BWD_MIN_BLOCKS 2
#endif
// Resident blocks of 128 per SM the register budget of k_backward allows.
constexpr int kBackwardMinBlocks = ER_BWD_MIN_BLOCKS;

// Gradient replay: one path per lane over a persistent grid; each warp
// takes 32 consecutive paths (sample-major, so neighbouring lanes trace
// neighbouring pixels).  The sample's radiance comes from the wavefront
// forward's per-path dump.
template <bool Q8>
__global__ void __launch_bounds__(kTravBlock, kBackwardMinBlocks) k_backward(DevScene S, ReplayArgs A, const float* __restrict__ rad) {
  __shared__ int2 stk[kSmemStack * kTravBlock];
  extern __shared__ float sg[];
  const WaveParams& P = A.P;
  if (A.smem_grad) {
    for (int32_t i = threadIdx.x; i < 5 * A.n_mats; i += blockDim.x) sg[i] = 0.f;
    __syncthreads();
  }
  const int64_t N = (int64_t)P.npix * P.spp_wave;
  const int64_t warp = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int64_t nwarps = ((int64_t)gridDim.x * blockDim.x) >> 5;
  const int32_t lane = (int32_t)(threadIdx.x & 31u);
  for (int64_t base = warp * 32; base < N; base += nwarps * 32) {
    const int64_t q = base + lane;
    bool act = q < N;
    const int32_t pix = act ? (int32_t)(q % P.npix) : 0, s = act ? (int32_t)(q / P.npix) : 0;
    const int32_t x = pix % P.W, y = pix / P.W;
    const uint32_t idx = (uint32_t)(P.W * (P.H - y - 1) + x);  // kernel.cu:378
    f3 L = mk1(0.f), dl = mk1(0.f);
    if (act) {
      const uint32_t n = A.nvalid[idx];
      const float4 g4 = A.d_beauty[idx];
      const float* r = rad + 3 * ((int64_t)s * P.npix + idx);
      L = mk(r[0], r[1], r[2]);
      // dropped samples (NaN) get no gradient; clamp(L, 0, 10) passes the
      // derivative only strictly inside
      const float inv_n = n > 0 ? 1.0f / (float)n : 0.f;
      const bool keep = n > 0 && !isnan(L.x) && !isnan(L.y) && !isnan(L.z);
      dl = mk((keep && L.x > 0.f && L.x < 10.f) ? g4.x * inv_n : 0.f,
              (keep && L.y > 0.f && L.y < 10.f) ? g4.y * inv_n : 0.f,
              (keep && L.z > 0.f && L.z < 10.f) ? g4.z * inv_n : 0.f);
      act = dl.x != 0.f || dl.y != 0.f || dl.z != 0.f;
    }
    int32_t nb;
    walk<Q8, true, false>(S, A, stk + threadIdx.x, sg, act, x, y, idx, (uint32_t)(P.sample_base + s), L, dl, &nb);
  }
  if (A.smem_grad) {
    __syncthreads();
    for (int32_t i = threadIdx.x; i < 5 * A.n_mats; i += blockDim.x)
      if (sg[i] != 0.f) atomicAdd(&A.g_mat[i], sg[i]);
  }
}

constexpr int kMaxSmemGrad = 8192;  // floats of shared memory for material gradients

template <bool EVAL>
er_status launch_replay(er_scene* s, const ReplayArgs& A) {
  const int32_t npix = A.P.npix;
  const unsigned blocks = (unsigned)((npix + kTravBlock - 1) / kTravBlock);
  if (s->dev.use_q8) k_replay<true, EVAL><<<blocks, kTravBlock, 0, s->stream>>>(s->dev, A);
  else k_replay<false, EVAL><<<blocks, kTravBlock, 0, s->stream>>>(s->dev, A);
  ER_CUDA(cudaGetLastError());
  return ER_OK;
}

er_status launch_backward(er_scene* s, const ReplayArgs& A, const float* rad) {
  const size_t smem = A.smem_grad ? (size_t)5 * A.n_mats * sizeof(float) : 0;
  int occ = 0;
  if (s->dev.use_q8) cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, k_backward<true>, kTravBlock, smem);
  else cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, k_backward<false>, kTravBlock, smem);
  const int64_t N = (int64_t)A.P.npix * A.P.spp_wave;
  const int64_t want = (N + kTravBlock - 1) / kTravBlock;
  const unsigned blocks = (unsigned)std::max<int64_t>(1, std::min<int64_t>(want, (int64_t)std::max(1, occ) * s->num_sms));
  if (s->dev.use_q8) k_backward<true><<<blocks, kTravBlock, smem, s->stream>>>(s->dev, A, rad);
  else k_backward<false><<<blocks, kTravBlock, smem, s->stream>>>(s->dev, A, rad);
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
  // the samples' radiance: the wavefront forward, one wave, per-path dump
  const int64_t npaths = (int64_t)np * A.P.spp_wave;
  float* d_rad = nullptr;
  int32_t* d_b = nullptr;
  if ((st = T.alloc((void**)&d_rad, (size_t)npaths * 12)) != ER_OK) return st;
  if ((st = T.alloc((void**)&d_b, (size_t)npaths * 4)) != ER_OK) return st;
  ER_CUDA(cudaEventRecord(s->ev0, s->stream));
  if (npaths > 0) {
    er_render_opts oo = *o;
    oo.flags &= ER_RENDER_ENV_ALIAS;
    if ((st = render_paths_device(s, &oo, d_rad, d_b)) != ER_OK) return st;
    if ((st = launch_backward(s, A, d_rad)) != ER_OK) return st;
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
}
