// Wavefront path tracer: the sample loop of the reference's renderingKernel
// (kernel.cu:369-481) split into stages that run over compacted queues:
//
//   raygen -> [ extend (closest hit) -> shade -> shadow ] x max_depth -> accumulate
//
// One wave traces spp_wave samples of every pixel.  Paths are indexed
// p = s * npix + pix; per-path state lives in SoA arrays, queues hold
// (origin|path, direction) pairs and are appended with warp ballots + one
// atomic per warp.  Radiance contributions of a vertex are resolved in the
// reference's order (kernel.cu:351-357) once its two shadow rays are done,
// and samples are accumulated per pixel in sample order, so the image does
// not depend on queue order.
#include <algorithm>
#include <cstring>
#include <map>
#include <mutex>
#include <string>
#include <tuple>

#include "internal.h"
#include "shade.cuh"
#include "traverse.cuh"
#include "vertex.cuh"
#include "adjoint.cuh"

namespace er {

// Device view of the wave buffers (passed to kernels by value).
struct WaveView {
  bool aov = false;
  float4* thr = nullptr;
  float4* light = nullptr;
  float4* pend = nullptr;  // 4 per path
  uint8_t* vis = nullptr;  // 2 per path
  int32_t* bounces = nullptr;
  float4* aovs = nullptr;  // 3 per path
  // gradient replay (er_backward): per path the sample's radiance and its
  // adjoint, and the last shaded vertex (origin|slot, direction|bounce, t u v)
  float4* g_lt = nullptr;
  float4* g_dl = nullptr;
  float4* g_k = nullptr;  // 5 float4 per path: the last vertex's gradient coefficients
  float4* q_o[2] = {nullptr, nullptr};
  float4* q_d[2] = {nullptr, nullptr};
  float4* hits = nullptr;
  float4* s_o = nullptr;
  float4* s_d = nullptr;
  float4* s_p = nullptr;
  int32_t* counts = nullptr;       // queue sizes and claim counters (see k_extend)
  unsigned long long* stats = nullptr;  // [0] closest rays [1] shadow rays (owned by the scene)
  int64_t shadow_half = 0;         // point-light rays start here in the shadow queue
};

struct Wave {
  int64_t cap = 0;
  WaveView v;
  std::vector<void*> mem;
};

// Queue counters (w.counts), by bounce parity q = b & 1:
//   kExt + q      extension rays of bounce b (written by raygen / shade(b-1))
//   kEnv + q      env shadow rays of bounce b (written by shade(b))
//   kPt + q       point-light shadow rays of bounce b (written by shade(b))
//   kClaim + 0..2 claim counters of the trace kernel's three phases
// Each count is zeroed by a kernel that runs after its last reader and
// before its first writer.
constexpr int kExt = 0, kEnv = 2, kPt = 4, kClaim = 8;

namespace {

__device__ __forceinline__ uint32_t lane_id() { return threadIdx.x & 31u; }

// Warp-aggregated append: one atomic per warp, slots ordered by lane.
__device__ __forceinline__ int32_t warp_append(int32_t* counter, bool pred) {
  unsigned mask = __ballot_sync(0xFFFFFFFFu, pred);
  int32_t base = 0;
  if (mask) {
    int leader = __ffs(mask) - 1;
    if ((int)lane_id() == leader) base = atomicAdd(counter, __popc(mask));
    base = __shfl_sync(0xFFFFFFFFu, base, leader);
  }
  unsigned lt = (1u << lane_id()) - 1u;
  return base + __popc(mask & lt);
}

// kernel.cu:378: output index of thread pixel (x, y)
__device__ __forceinline__ int32_t out_index(const WaveParams& P, int32_t x, int32_t y) {
  return P.W * (P.H - y - 1) + x;
}

// Batch slice of wave path p (slices are sorted by path_base).
__device__ __forceinline__ int32_t find_seg(const BatchView& B, int32_t p) {
  int32_t lo = 0, hi = B.n_segs - 1;
  while (lo < hi) {
    int32_t mid = (lo + hi + 1) >> 1;
    if (__ldg(&B.segs[mid].path_base) <= p) lo = mid;
    else hi = mid - 1;
  }
  return lo;
}

// Batch slice of accumulate item i.
__device__ __forceinline__ int32_t find_seg_pix(const BatchView& B, int32_t i) {
  int32_t lo = 0, hi = B.n_segs - 1;
  while (lo < hi) {
    int32_t mid = (lo + hi + 1) >> 1;
    if (__ldg(&B.segs[mid].pix_base) <= i) lo = mid;
    else hi = mid - 1;
  }
  return lo;
}

// Path p's wave constants, index within its job's slice, and job (0 for a
// single-scene render).  Queue entries carry the job in a spare lane so the
// traversal can start at that job's BVH root.
template <bool BATCH>
__device__ __forceinline__ int32_t path_slice(const BatchView& B, int32_t p, WaveParams& P, int32_t& job) {
  if (!BATCH) {
    job = 0;
    return p;
  }
  const BatchSeg& g = B.segs[find_seg(B, p)];
  P = g.P;
  job = g.job;
  return p - g.path_base;
}

// d loss / d radiance of one sample: the pixel's adjoint spread over its
// valid samples, zero for a dropped (NaN) sample and for clamped channels
// (clamp(L, 0, 10) passes the derivative only strictly inside).
__device__ __forceinline__ f3 sample_adjoint(f3 L, float4 g4, uint32_t n) {
  const bool keep = n > 0 && !isnan(L.x) && !isnan(L.y) && !isnan(L.z);
  const float inv_n = n > 0 ? 1.0f / (float)n : 0.f;
  return mk((keep && L.x > 0.f && L.x < 10.f) ? g4.x * inv_n : 0.f,
            (keep && L.y > 0.f && L.y < 10.f) ? g4.y * inv_n : 0.f,
            (keep && L.z > 0.f && L.z < 10.f) ? g4.z * inv_n : 0.f);
}

// Path order within a sample: 8x4 pixel tiles (a warp's 32 paths start in
// one tile, so its primary rays and first hits are coherent) when the image
// divides into them, else raster order.  pix = y * W + x either way; the
// random numbers and the output slot depend only on the pixel, so the order
// changes no result.
__device__ __forceinline__ bool tiled(const WaveParams& P) { return (P.W & 7) == 0 && (P.H & 3) == 0; }
__device__ __forceinline__ int32_t path_pixel(const WaveParams& P, int32_t q) {
  if (!tiled(P)) return q;
  const int32_t t = q >> 5, r = q & 31, tw = P.W >> 3;
  const int32_t x = ((t % tw) << 3) + (r & 7), y = ((t / tw) << 2) + (r >> 3);
  return y * P.W + x;
}
__device__ __forceinline__ int32_t pixel_path(const WaveParams& P, int32_t pix) {
  if (!tiled(P)) return pix;
  const int32_t x = pix % P.W, y = pix / P.W;
  return (((y >> 2) * (P.W >> 3) + (x >> 3)) << 5) + ((y & 3) << 3) + (x & 7);
}

template <bool BATCH, bool GRAD = false>
__global__ void k_raygen(DevScene S, WaveView w, WaveParams P, int32_t n, BatchView B, GradArgs G) {
  int32_t p = blockIdx.x * blockDim.x + threadIdx.x;
  if (p == 0) {
    for (int k = 0; k < 16; k++) w.counts[k] = 0;
    w.counts[kExt] = n;
  }
  if (p >= n) return;
  int32_t job;
  int32_t local = path_slice<BATCH>(B, p, P, job);
  int32_t pix = path_pixel(P, local % P.npix), s = local / P.npix;
  int32_t x = pix % P.W, y = pix / P.W;
  uint32_t idx = (uint32_t)out_index(P, x, y);
  uint32_t sample = (uint32_t)(P.sample_base + s);
  uint4 a = philox(make_uint4(idx, sample, 0u, 0u), P.k0, P.k1);
  uint4 b = philox(make_uint4(idx, sample, 1u, 0u), P.k0, P.k1);
  f3 o, d;
  camera_ray(BATCH ? B.jobs[job].cam : S.cam, x, y, u01(a.x), u01(a.y), u01(a.z), u01(a.w), u01(b.x), o, d);
  w.q_o[0][p] = make_float4(o.x, o.y, o.z, __int_as_float(p));
  w.q_d[0][p] = make_float4(d.x, d.y, d.z, __int_as_float(job));
  w.thr[p] = make_float4(1.f, 1.f, 1.f, 0.f);
  w.light[p] = make_float4(0.f, 0.f, 0.f, 0.f);
  w.pend[4 * (size_t)p + 2] = make_float4(0.f, 0.f, 0.f, 0.f);
  w.bounces[p] = P.max_depth;
  if (GRAD) {
    const float* r = G.rad + 3 * ((int64_t)(sample - (uint32_t)G.sample0) * P.npix + idx);
    const f3 L = mk(r[0], r[1], r[2]);
    const f3 dl = sample_adjoint(L, G.d_beauty[idx], G.nvalid[idx]);
    w.g_lt[p] = make_float4(L.x, L.y, L.z, 0.f);
    w.g_dl[p] = make_float4(dl.x, dl.y, dl.z, 0.f);
  }
  if (w.aov) {
    w.aovs[3 * (size_t)p] = make_float4(0, 0, 0, 0);
    w.aovs[3 * (size_t)p + 1] = make_float4(0, 0, 0, 0);
    w.aovs[3 * (size_t)p + 2] = make_float4(0, 0, 0, 0);
  }
}

// Adds per-thread traversal counters into stats[k], stats[k+1] (one atomic
// per warp).
__device__ __forceinline__ void flush_counts(unsigned long long* stats, int k, const TravStats& st) {
  unsigned long long a = st.nodes, b = st.tris;
  for (int o = 16; o > 0; o >>= 1) {
    a += __shfl_down_sync(0xFFFFFFFFu, a, o);
    b += __shfl_down_sync(0xFFFFFFFFu, b, o);
  }
  if (lane_id() == 0) {
    atomicAdd(&stats[k], a);
    atomicAdd(&stats[k + 1], b);
  }
}

// One traversal launch per bounce: the extension rays of bounce b (closest
// hit) together with the shadow rays of bounce b-1, which are independent
// of them.  Three persistent phases; every warp helps in all of them.
//
// `phases` selects the phases (1 extension, 2 point-light, 4 env); a split
// schedule runs them as three launches, the launch with phase 1 first.
template <bool Q8, bool STATS, bool BATCH>
__global__ void __launch_bounds__(kTravBlock, kTravMinBlocks)
    k_trace(DevScene S, WaveView w, int32_t b, uint32_t* err, BatchView B, uint32_t phases) {
  __shared__ int2 stk[kSmemStack * kTravBlock];
  const int32_t q = b & 1, qp = q ^ 1;
  const int32_t n_ext = (phases & 1u) ? w.counts[kExt + q] : 0;
  const int32_t n_pt = (phases & 2u) ? w.counts[kPt + qp] : 0;
  const int32_t n_env = (phases & 4u) ? w.counts[kEnv + qp] : 0;
  if (blockIdx.x == 0 && threadIdx.x == 0) {
    if (phases & 1u) {
      w.counts[kExt + qp] = 0;  // shade(b) appends the next extension rays
      w.counts[kEnv + q] = 0;   // ... and the shadow rays of bounce b
      w.counts[kPt + q] = 0;
    }
    atomicAdd(&w.stats[0], (unsigned long long)n_ext);
    atomicAdd(&w.stats[1], (unsigned long long)(n_env + n_pt));
  }
  const float4* qo = w.q_o[q];
  const float4* qd = w.q_d[q];
  float4* hits = w.hits;
  const float4* so = w.s_o;
  const float4* sd = w.s_d;
  const float4* spp = w.s_p;
  uint8_t* vis = w.vis;
  const int64_t half = w.shadow_half;
  TravStats st{0, 0, 0}, ss{0, 0, 0};
  persistent_traverse<kClosest, Q8, STATS>(
      S, n_ext, &w.counts[kClaim], stk + threadIdx.x, st, err,
      [&](int32_t i, auto& tr) {
        float4 a = qo[i], d = qd[i];
        if (BATCH) {
          const BatchJobDev& J = B.jobs[__float_as_int(d.w)];
          tr.init_at(S, mk(a.x, a.y, a.z), mk(d.x, d.y, d.z), mk1(0.f), 0.f, J.root, J.scene_eps);
        } else {
          tr.init(S, mk(a.x, a.y, a.z), mk(d.x, d.y, d.z), mk1(0.f), 0.f);
        }
      },
      [&](int32_t i, auto& tr) { hits[i] = make_float4(tr.t, tr.u, tr.v, __int_as_float(tr.slot)); });
  // point-light rays: shadow queue [half, half + n_pt)
  persistent_traverse<kPoint, Q8, STATS>(
      S, n_pt, &w.counts[kClaim + 1], stk + threadIdx.x, ss, err,
      [&](int32_t i, auto& tr) {
        float4 a = so[half + i], d = sd[half + i], p = spp[half + i];
        if (BATCH) {
          const BatchJobDev& J = B.jobs[__float_as_int(p.w)];
          tr.init_at(S, mk(a.x, a.y, a.z), mk(d.x, d.y, d.z), mk(p.x, p.y, p.z), d.w, J.root, J.scene_eps);
        } else {
          tr.init(S, mk(a.x, a.y, a.z), mk(d.x, d.y, d.z), mk(p.x, p.y, p.z), d.w);
        }
      },
      [&](int32_t i, auto& tr) { vis[__float_as_int(so[half + i].w)] = tr.occluded ? 0 : 1; });
  // env rays: shadow queue [0, n_env)
  persistent_traverse<kAny, Q8, STATS>(
      S, n_env, &w.counts[kClaim + 2], stk + threadIdx.x, ss, err,
      [&](int32_t i, auto& tr) {
        float4 a = so[i], d = sd[i];
        if (BATCH) {
          const BatchJobDev& J = B.jobs[__float_as_int(d.w)];
          tr.init_at(S, mk(a.x, a.y, a.z), mk(d.x, d.y, d.z), mk1(0.f), 0.f, J.root, J.scene_eps);
        } else {
          tr.init(S, mk(a.x, a.y, a.z), mk(d.x, d.y, d.z), mk1(0.f), 0.f);
        }
      },
      [&](int32_t i, auto& tr) { vis[__float_as_int(so[i].w)] = tr.occluded ? 0 : 1; });
  if (STATS) {
    flush_counts(w.stats, 2, st);
    flush_counts(w.stats, 4, ss);
  }
}

// Every channel of t has the bits of o.
__device__ __forceinline__ bool same_bits3(f3 t, float o) {
  const uint32_t b = __float_as_uint(o);
  return __float_as_uint(t.x) == b && __float_as_uint(t.y) == b && __float_as_uint(t.z) == b;
}

// Resolve the pending MIS terms of a path's last shaded vertex
// (kernel.cu:351-355,433): light += reduction * ((w1*H + w2*P) + w3*B),
// with an occluded strategy contributing w*0 (NaN when its weight is).
__device__ __forceinline__ void resolve(const WaveView& w, int32_t p, float4& L) {
  float4 tB = w.pend[4 * (size_t)p + 2];
  uint32_t fl = __float_as_uint(tB.w);
  if (!(fl & 1u)) return;
  float4 tH = w.pend[4 * (size_t)p];
  float4 tP = w.pend[4 * (size_t)p + 1];
  float4 rp = w.pend[4 * (size_t)p + 3];
  bool vH = w.vis[2 * (size_t)p] != 0;
  bool vP = (fl & 2u) ? (w.vis[2 * (size_t)p + 1] != 0) : true;
  float hx = vH ? tH.x : tH.w, hy = vH ? tH.y : tH.w, hz = vH ? tH.z : tH.w;
  float px = vP ? tP.x : tP.w, py = vP ? tP.y : tP.w, pz = vP ? tP.z : tP.w;
  L.x = __fadd_rn(L.x, __fmul_rn(__fadd_rn(__fadd_rn(hx, px), tB.x), rp.x));
  L.y = __fadd_rn(L.y, __fmul_rn(__fadd_rn(__fadd_rn(hy, py), tB.y), rp.y));
  L.z = __fadd_rn(L.z, __fmul_rn(__fadd_rn(__fadd_rn(hz, pz), tB.z), rp.z));
  w.pend[4 * (size_t)p + 2].w = __uint_as_float(0u);
}

// Gradient of the vertex whose MIS terms were just resolved: its stored
// coefficients with the visibility its shadow rays found.  fl = the pending
// flags before resolve.
__device__ __forceinline__ void grad_prev_vertex(const WaveView& w, const GradArgs& G, int32_t p, uint32_t fl) {
  const bool vH = w.vis[2 * (size_t)p] != 0;
  const bool vP = (fl & 2u) ? (w.vis[2 * (size_t)p + 1] != 0) : true;
  apply_vertex_gradient(w.g_k + 5 * (size_t)p, vH, vP, G.g_mat, G.g_env);
}

#ifndef ER_SHADE_MIN_BLOCKS
#define ER_SHADE_MIN_BLOCKS 7
#endif
#ifndef ER_SHADE_GRAD_MIN_BLOCKS
#define ER_SHADE_GRAD_MIN_BLOCKS 12
#endif
// Resident 128-thread shade blocks per SM the register budgets are sized
// for.  Both kernels wait on dependent loads (texture, material, env
// lookups, atomics), so occupancy pays for some spilling.  Forward: 73
// registers at 7 blocks (unbounded 117 at 4 blocks: 10 % longer stage on
// the 1080p scene; 8 blocks spill too much).  Gradient: 42 registers at 12
// blocks (unbounded 209 at 2 blocks): backward of the 512x512 adjoint
// workload 34.9 vs 49.7 ms.
constexpr int kShadeMinBlocks = ER_SHADE_MIN_BLOCKS;
constexpr int kShadeGradMinBlocks = ER_SHADE_GRAD_MIN_BLOCKS;

// EVAL: the detached estimator of er_render_replay, BRDF values and
// environment radiance from G's evaluation parameters.
template <bool BATCH, bool GRAD = false, bool EVAL = false>
__global__ void __launch_bounds__(128, GRAD ? kShadeGradMinBlocks : kShadeMinBlocks)
    k_shade(DevScene S0, WaveView w, WaveParams P0, int32_t bounce, BatchView B, GradArgs G) {
  const int32_t qin = bounce & 1;
  const int32_t n = w.counts[kExt + qin];
  const float4* qo = w.q_o[qin];
  const float4* qd = w.q_d[qin];
  const int32_t qout = qin ^ 1;
  if (blockIdx.x == 0 && threadIdx.x == 0) {
    w.counts[kClaim] = 0;  // the next trace launch claims from zero
    w.counts[kClaim + 1] = 0;
    w.counts[kClaim + 2] = 0;
  }
  for (int32_t base = blockIdx.x * blockDim.x; base < n; base += gridDim.x * blockDim.x) {
    int32_t i = base + threadIdx.x;
    bool valid = i < n;
    bool push_next = false, push_env = false, push_pt = false;
    f3 next_o = mk1(0), next_d = mk1(0), env_o = mk1(0), env_d = mk1(0), pt_o = mk1(0), pt_d = mk1(0),
       pt_p = mk1(0);
    float pt_dist = 0.f;
    int32_t p = 0, job = 0;
    if (valid) {
      float4 a = qo[i], b = qd[i];
      p = __float_as_int(a.w);
      // the path's job: its wave constants and the per-scene parts of S
      WaveParams P = P0;
      DevScene S = S0;
      int32_t local = path_slice<BATCH>(B, p, P, job);
      if (BATCH) {
        const BatchJobDev& J = B.jobs[job];
        S.env = J.env;
        S.cdf = J.cdf;
        S.alias_idx = J.alias_idx;
        S.alias_thresh = J.alias_thresh;
        S.env_lut = J.env_lut;
        S.lights = J.lights;
        S.radiance_sum = J.radiance_sum;
        S.n_lights = J.n_lights;
      }
      const bool last = bounce + 1 >= P.max_depth;
      f3 o = mk(a.x, a.y, a.z), d = mk(b.x, b.y, b.z);
      float4 L = w.light[p];
      const uint32_t fl_prev = GRAD ? __float_as_uint(w.pend[4 * (size_t)p + 2].w) : 0u;
      resolve(w, p, L);
      if (GRAD && (fl_prev & 1u)) grad_prev_vertex(w, G, p, fl_prev);
      float4 T4 = w.thr[p];
      f3 thr = mk(T4.x, T4.y, T4.z);
      float4 h = w.hits[i];
      int32_t slot = __float_as_int(h.w);
      if (slot < 0) {
        // kernel.cu:414-419: environment on escape, no MIS weight
        int64_t te = 0;
        f3 e = escape_radiance(S, d, (GRAD || EVAL) ? &te : nullptr);
        if (EVAL && G.eval_env) e = mk(G.eval_env[3 * te], G.eval_env[3 * te + 1], G.eval_env[3 * te + 2]);
        if (GRAD) {
          const float4 dl4 = w.g_dl[p];
          float ge[3] = {dl4.x * thr.x, dl4.y * thr.y, dl4.z * thr.z};
          if (ge[0] != 0.f || ge[1] != 0.f || ge[2] != 0.f) agg_add<3>(G.g_env, te, ge);
        }
        L.x = __fadd_rn(L.x, __fmul_rn(e.x, thr.x));
        L.y = __fadd_rn(L.y, __fmul_rn(e.y, thr.y));
        L.z = __fadd_rn(L.z, __fmul_rn(e.z, thr.z));
        w.bounces[p] = bounce;
      } else {
        int32_t pix = path_pixel(P, local % P.npix), s = local / P.npix;
        uint32_t idx = (uint32_t)out_index(P, pix % P.W, pix / P.W);
        VertexShade V;
        shade_vertex<BATCH || GRAD>(S, P.flags, P.k0, P.k1, idx, (uint32_t)(P.sample_base + s), bounce, o, d, h.x, h.y, h.z,
                            slot, V);
        if (EVAL) eval_vertex(S, G.eval_mat, G.eval_env, d, V);
        if (GRAD) {
          const float4 dl4 = w.g_dl[p], lt = w.g_lt[p];
          vertex_grad_coeffs(S, V, thr, mk(dl4.x, dl4.y, dl4.z), mk(lt.x, lt.y, lt.z), mk(L.x, L.y, L.z),
                             w.g_k + 5 * (size_t)p);
        }
        env_o = V.env_o;
        env_d = V.env_d;
        // A shadow ray whose strategy term is bitwise the same visible or
        // occluded (w * H == w * 0 in every channel: the BRDF is zero
        // towards the light, e.g. it lies below the surface) cannot change
        // the film, so it is not traced; its visibility is set to "visible".
        // The gradient pass also needs the BRDF's partials to vanish there,
        // which holds where DisneyEval's own gate rejects the direction (its
        // env-texel derivative depends on visibility wherever f is not 0).
        const float oH = V.w1 * 0.0f, oP = V.w2 * 0.0f;
        push_env = !same_bits3(V.tH, oH) || (GRAD && disney_gate(V.hd, V.C, V.dH));
        if (!push_env) w.vis[2 * (size_t)p] = 1;
        if (V.has_pt) {
          pt_o = V.pt_o;
          pt_d = V.pt_d;
          pt_p = V.pos;
          pt_dist = V.dist;
          push_pt = !same_bits3(V.tP, oP) || (GRAD && disney_gate(V.hd, V.C, V.dP));
          if (!push_pt) w.vis[2 * (size_t)p + 1] = 1;
        }
        uint32_t fl = 1u | (V.has_pt ? 2u : 0u);
        w.pend[4 * (size_t)p] = make_float4(V.tH.x, V.tH.y, V.tH.z, oH);
        w.pend[4 * (size_t)p + 1] = make_float4(V.tP.x, V.tP.y, V.tP.z, oP);
        w.pend[4 * (size_t)p + 2] = make_float4(V.tB.x, V.tB.y, V.tB.z, __uint_as_float(fl));
        w.pend[4 * (size_t)p + 3] = make_float4(thr.x, thr.y, thr.z, 0.f);
        thr = mk(__fmul_rn(thr.x, V.g.x), __fmul_rn(thr.y, V.g.y), __fmul_rn(thr.z, V.g.z));
        w.thr[p] = make_float4(thr.x, thr.y, thr.z, 0.f);
        if (bounce == 0 && w.aov) {
          w.aovs[3 * (size_t)p] = make_float4(V.sn.x, V.sn.y, V.sn.z, 0.f);
          w.aovs[3 * (size_t)p + 1] = make_float4(V.tg.x, V.tg.y, V.tg.z, 0.f);
          w.aovs[3 * (size_t)p + 2] = make_float4(V.bt.x, V.bt.y, V.bt.z, 0.f);
        }
        if (!last) {
          // kernel.cu:442
          next_o = xadd(V.pos, xscale(V.dir, 0.001f));
          next_d = xnormalize(V.dir);
          push_next = true;
        }
      }
      w.light[p] = L;
    }
    int32_t j = warp_append(&w.counts[kExt + qout], push_next);
    if (push_next) {
      w.q_o[qout][j] = make_float4(next_o.x, next_o.y, next_o.z, __int_as_float(p));
      w.q_d[qout][j] = make_float4(next_d.x, next_d.y, next_d.z, __int_as_float(job));
    }
    int32_t k = warp_append(&w.counts[kEnv + qin], push_env);
    if (push_env) {
      w.s_o[k] = make_float4(env_o.x, env_o.y, env_o.z, __int_as_float(2 * p));
      w.s_d[k] = make_float4(env_d.x, env_d.y, env_d.z, __int_as_float(job));
    }
    k = warp_append(&w.counts[kPt + qin], push_pt);
    if (push_pt) {
      int64_t j = w.shadow_half + k;
      w.s_o[j] = make_float4(pt_o.x, pt_o.y, pt_o.z, __int_as_float(2 * p + 1));
      w.s_d[j] = make_float4(pt_d.x, pt_d.y, pt_d.z, pt_dist);
      w.s_p[j] = make_float4(pt_p.x, pt_p.y, pt_p.z, __int_as_float(job));
    }
  }
}

// Gradient of every path's last shaded vertex (resolved here instead of in
// the accumulation).
__global__ void k_resolve_grad(WaveView w, int32_t n, GradArgs G) {
  int32_t p = blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= n) return;
  const uint32_t fl = __float_as_uint(w.pend[4 * (size_t)p + 2].w);
  if (!(fl & 1u)) return;
  w.pend[4 * (size_t)p + 2].w = __uint_as_float(0u);
  grad_prev_vertex(w, G, p, fl);
}

// kernel.cu:445-478 per pixel, samples in index order.
__device__ __forceinline__ void accumulate_pixel(const WaveView& w, const WaveParams& P, const Film& F, int32_t sw,
                                                 int32_t pix, int32_t path_base, uint32_t& bounce_sum);

// One item per pixel of every slice (a single render: one slice).
template <bool BATCH>
__global__ void k_accumulate(WaveView w, WaveParams P, Film F, int32_t sw, BatchView B) {
  int32_t pix = blockIdx.x * blockDim.x + threadIdx.x;
  uint32_t bsum = 0;
  if (BATCH) {
    if (pix < B.n_acc) {
      const BatchSeg& g = B.segs[find_seg_pix(B, pix)];
      accumulate_pixel(w, g.P, B.jobs[g.job].film, g.P.spp_wave, pix - g.pix_base, g.path_base, bsum);
    }
  } else if (pix < P.npix) {
    accumulate_pixel(w, P, F, sw, pix, 0, bsum);
  }
  // path-vertex counter (the reference's kPaths numerator), one atomic per warp
  unsigned long long v = bsum;
  for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xFFFFFFFFu, v, o);
  if (lane_id() == 0 && v) atomicAdd(&w.stats[6], v);
}

__device__ __forceinline__ void accumulate_pixel(const WaveView& w, const WaveParams& P, const Film& F, int32_t sw,
                                                 int32_t pix, int32_t path_base, uint32_t& bounce_sum) {
  int32_t x = pix % P.W, y = pix / P.W;
  int32_t idx = out_index(P, x, y);
  uint32_t sa = F.samples[idx], pc = F.pathcount[idx];
  const bool fp64 = P.flags & ER_RENDER_ACCUM_FP64;
  float4 bt = F.beauty[idx];
  double s0 = 0, s1 = 0, s2 = 0;
  if (fp64) { s0 = F.sum[3 * (size_t)idx]; s1 = F.sum[3 * (size_t)idx + 1]; s2 = F.sum[3 * (size_t)idx + 2]; }
  float4 a[3];
  if (F.aov_on) for (int k = 0; k < 3; k++) a[k] = F.aov[k][idx];
  for (int32_t s = 0; s < sw; s++) {
    int32_t p = path_base + s * P.npix + pixel_path(P, pix);
    float4 L = w.light[p];
    resolve(w, p, L);
    if (F.keep) {
      float* r = F.keep + 3 * ((int64_t)(F.keep_s0 + s) * P.npix + idx);
      r[0] = L.x; r[1] = L.y; r[2] = L.z;
    }
    pc += (uint32_t)w.bounces[p];
    bounce_sum += (uint32_t)w.bounces[p];
    float lx = clampf_(L.x, 0.f, 10.f), ly = clampf_(L.y, 0.f, 10.f), lz = clampf_(L.z, 0.f, 10.f);
    if (isnan(lx) || isnan(ly) || isnan(lz)) continue;
    float inv = __fadd_rn((float)sa, 1.0f);
    if (fp64) {
      s0 += lx; s1 += ly; s2 += lz;
    } else {
      if (sa > 0) {
        float k = __fdiv_rn((float)sa, (float)(sa + 1));
        bt.x = __fmul_rn(bt.x, k); bt.y = __fmul_rn(bt.y, k); bt.z = __fmul_rn(bt.z, k);
      }
      bt.x = __fadd_rn(bt.x, __fdiv_rn(lx, inv));
      bt.y = __fadd_rn(bt.y, __fdiv_rn(ly, inv));
      bt.z = __fadd_rn(bt.z, __fdiv_rn(lz, inv));
    }
    if (F.aov_on) {
      for (int k = 0; k < 3; k++) {
        float4 v = w.aov ? w.aovs[3 * (size_t)p + k] : make_float4(0, 0, 0, 0);
        if (sa > 0) {
          float kk = __fdiv_rn((float)sa, (float)(sa + 1));
          a[k].x = __fmul_rn(a[k].x, kk); a[k].y = __fmul_rn(a[k].y, kk); a[k].z = __fmul_rn(a[k].z, kk);
        }
        a[k].x = __fadd_rn(a[k].x, __fdiv_rn(v.x, inv));
        a[k].y = __fadd_rn(a[k].y, __fdiv_rn(v.y, inv));
        a[k].z = __fadd_rn(a[k].z, __fdiv_rn(v.z, inv));
      }
    }
    sa++;
  }
  if (fp64) {
    F.sum[3 * (size_t)idx] = s0; F.sum[3 * (size_t)idx + 1] = s1; F.sum[3 * (size_t)idx + 2] = s2;
    if (sa > 0) bt = make_float4((float)(s0 / sa), (float)(s1 / sa), (float)(s2 / sa), 1.0f);
  }
  F.beauty[idx] = bt;
  if (F.aov_on) for (int k = 0; k < 3; k++) F.aov[k][idx] = a[k];
  F.samples[idx] = sa;
  F.pathcount[idx] = pc;
}

// Per-path dump for er_render_paths.
// s_off: the wave's first sample, relative to the call's first.
__global__ void k_dump(WaveView w, WaveParams P, int32_t sw, int32_t s_off, float* rad, int32_t* bnc) {
  int32_t p = blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= sw * P.npix) return;
  float4 L = w.light[p];
  resolve(w, p, L);
  int32_t pix = path_pixel(P, p % P.npix), s = p / P.npix;
  int64_t j = (int64_t)(s + s_off) * P.npix + out_index(P, pix % P.W, pix / P.W);
  rad[3 * j] = L.x; rad[3 * j + 1] = L.y; rad[3 * j + 2] = L.z;
  bnc[j] = w.bounces[p];
}

__global__ void k_film_clear(Film F, int32_t npix) {
  int32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= npix) return;
  F.beauty[i] = make_float4(0.f, 0.f, 0.f, 1.f);
  if (F.aov_on) for (int k = 0; k < 3; k++) F.aov[k][i] = make_float4(0.f, 0.f, 0.f, 1.f);
  if (F.sum) { F.sum[3 * (size_t)i] = 0; F.sum[3 * (size_t)i + 1] = 0; F.sum[3 * (size_t)i + 2] = 0; }
  F.samples[i] = 0;
  F.pathcount[i] = 0;
}

}  // namespace

int blocks_per_sm(const void* kernel, int block) {
  static std::mutex mu;
  static std::map<std::tuple<const void*, int, int>, int> cache;
  int dev = 0;
  cudaGetDevice(&dev);
  const auto key = std::make_tuple(kernel, block, dev);
  std::lock_guard<std::mutex> lk(mu);
  auto it = cache.find(key);
  if (it != cache.end()) return it->second;
  int nb = 0;
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, kernel, block, 0) != cudaSuccess) {
    cudaGetLastError();
    nb = 1;
  }
  nb = std::max(1, nb);
  cache[key] = nb;
  return nb;
}

namespace {

template <typename K>
int grid_for(K kernel, int block, int sms) {
  return blocks_per_sm((const void*)kernel, block) * sms;
}

er_status alloc_w(Wave* w, void** p, size_t bytes) {
  cudaError_t e = cudaMalloc(p, std::max<size_t>(bytes, 16));
  if (e != cudaSuccess) {
    cudaGetLastError();
    return fail(e == cudaErrorMemoryAllocation ? ER_ERR_OOM : ER_ERR_CUDA, "wave buffer allocation failed");
  }
  w->mem.push_back(*p);
  return ER_OK;
}

// Allocates the buffers of `ww` for `cap` paths; on failure the caller
// frees what was allocated.
er_status wave_fill(Wave* ww, int64_t cap, bool aov, bool grad, unsigned long long* stats) {
  ww->cap = cap;
  WaveView* w = &ww->v;
  w->aov = aov;
  w->stats = stats;
  w->shadow_half = cap;
  er_status st;
#define AL(ptr, bytes) \
  if ((st = alloc_w(ww, (void**)&(ptr), (bytes))) != ER_OK) return st;
  AL(w->thr, cap * sizeof(float4));
  AL(w->light, cap * sizeof(float4));
  AL(w->pend, 4 * cap * sizeof(float4));
  AL(w->vis, 2 * cap);
  AL(w->bounces, cap * sizeof(int32_t));
  if (aov) AL(w->aovs, 3 * cap * sizeof(float4));
  for (int q = 0; q < 2; q++) {
    AL(w->q_o[q], cap * sizeof(float4));
    AL(w->q_d[q], cap * sizeof(float4));
  }
  AL(w->hits, cap * sizeof(float4));
  AL(w->s_o, 2 * cap * sizeof(float4));
  AL(w->s_d, 2 * cap * sizeof(float4));
  AL(w->s_p, 2 * cap * sizeof(float4));
  AL(w->counts, 16 * sizeof(int32_t));
  if (grad) {
    AL(w->g_lt, cap * sizeof(float4));
    AL(w->g_dl, cap * sizeof(float4));
    AL(w->g_k, 5 * cap * sizeof(float4));
  }
#undef AL
  return ER_OK;
}

// Default path budget of a wave (about 4.6 GB of buffers; two waves are in
// flight): at 1080p eight samples per pixel.  Larger waves lose less to the
// tails of the traversal launches (per 1080p sample: 8.25 ms at 2^22 paths,
// 8.04 at 2^23, 7.95 at 2^24), but a call keeps at least two waves when it
// has two samples, so that its waves overlap on two streams.
constexpr int64_t kWavePaths = (int64_t)1 << 24;
int32_t default_spp_per_wave(int32_t spp, int32_t npix) {
  const int32_t budget = std::max(1, (int32_t)(kWavePaths / npix));
  return std::max(1, std::min(budget, (spp + 1) / 2));
}

er_status ensure_wave(er_scene* s, int64_t cap, bool aov, bool grad = false) {
  if (s->wave && s->wave->cap >= cap && (!aov || s->wave->v.aov) && (!grad || s->wave->v.g_lt)) return ER_OK;
  free_wave(s);
  s->wave = new Wave();
  er_status st = wave_fill(s->wave, cap, aov, grad, s->d_stats);
  if (st != ER_OK) free_wave(s);
  return st;
}

// The second wave of the two-stream schedule, its stream and events; the
// same capacity and passes as the first.
er_status ensure_wave2(er_scene* s, bool grad = false) {
  const Wave* w1 = s->wave;
  if (!s->wave2 || s->wave2->cap < w1->cap || (w1->v.aov && !s->wave2->v.aov) || (grad && !s->wave2->v.g_lt)) {
    if (s->wave2) {
      for (void* p : s->wave2->mem) cudaFree(p);
      delete s->wave2;
    }
    s->wave2 = new Wave();
    er_status st = wave_fill(s->wave2, w1->cap, w1->v.aov, grad || w1->v.g_lt, s->d_stats);
    if (st != ER_OK) {
      for (void* p : s->wave2->mem) cudaFree(p);
      delete s->wave2;
      s->wave2 = nullptr;
      return st;
    }
  }
  if (!s->stream2) ER_CUDA(cudaStreamCreateWithFlags(&s->stream2, cudaStreamNonBlocking));
  if (!s->ev_fork) ER_CUDA(cudaEventCreateWithFlags(&s->ev_fork, cudaEventDisableTiming));
  for (cudaEvent_t& e : s->ev_acc)
    if (!e) ER_CUDA(cudaEventCreateWithFlags(&e, cudaEventDisableTiming));
  return ER_OK;
}

er_status ensure_film(er_scene* s, bool aov, bool fp64, bool clear) {
  Film& F = s->film;
  int32_t W = s->camera.x_res, H = s->camera.y_res;
  bool realloc = F.w != W || F.h != H || (aov && !F.aov_on) || (fp64 && !F.sum);
  if (realloc) {
    free_film(s);
    F.w = W;
    F.h = H;
    size_t np = (size_t)W * H;
    auto al = [&](void** p, size_t b) -> er_status {
      cudaError_t e = cudaMalloc(p, b);
      if (e != cudaSuccess) {
        cudaGetLastError();
        return fail(ER_ERR_OOM, "film allocation failed");
      }
      return ER_OK;
    };
    er_status st;
    if ((st = al((void**)&F.beauty, np * sizeof(float4))) != ER_OK) return st;
    if ((st = al((void**)&F.samples, np * sizeof(uint32_t))) != ER_OK) return st;
    if ((st = al((void**)&F.pathcount, np * sizeof(uint32_t))) != ER_OK) return st;
    if (aov) {
      for (int k = 0; k < 3; k++)
        if ((st = al((void**)&F.aov[k], np * sizeof(float4))) != ER_OK) return st;
      F.aov_on = true;
    }
    if (fp64 && (st = al((void**)&F.sum, np * 3 * sizeof(double))) != ER_OK) return st;
    clear = true;
  }
  if (clear) {
    int32_t npix = W * H;
    k_film_clear<<<(npix + 255) / 256, 256, 0, s->stream>>>(F, npix);
    ER_CUDA(cudaGetLastError());
  }
  // the FP64 sums hold the whole film only if every render into it since
  // the last clear accumulated them
  if (!fp64) F.sum_valid = false;
  else if (clear) F.sum_valid = true;
  return ER_OK;
}

er_status copy_out(er_scene* s, bool dev, void* dst, const void* src, size_t bytes) {
  if (!dst) return ER_OK;
  ER_CUDA(cudaMemcpyAsync(dst, src, bytes, dev ? cudaMemcpyDeviceToDevice : cudaMemcpyDeviceToHost, s->stream));
  return ER_OK;
}

// Runs the waves of one call.  dump_rad != null: single wave, per-path dump.
// eval != null: the shade stage takes its evaluation parameters (the
// detached estimator of er_render_replay).
er_status run(er_scene* s, const er_render_opts* o, float* dump_rad, int32_t* dump_b, int64_t* launches,
              bool grad_wave = false, const GradArgs* eval = nullptr) {
  const int32_t W = s->camera.x_res, H = s->camera.y_res;
  const int32_t npix = W * H;
  const bool aov = o->flags & ER_RENDER_AOV;
  int32_t max_depth = o->max_depth > 0 ? o->max_depth : 5;
  int32_t sw = o->spp_per_wave > 0 ? o->spp_per_wave : default_spp_per_wave(o->spp, npix);
  sw = std::min(sw, std::max(1, o->spp));
  er_status st = ensure_wave(s, (int64_t)sw * npix, aov, grad_wave);
  if (st != ER_OK) return st;
  WaveParams P;
  P.W = W; P.H = H; P.npix = npix; P.max_depth = max_depth;
  P.k0 = (uint32_t)o->seed; P.k1 = (uint32_t)(o->seed >> 32);
  P.flags = o->flags;
  const bool q8 = s->dev.use_q8;
  const bool count = o->flags & ER_RENDER_COUNT;
  const bool prof = o->flags & ER_RENDER_PROFILE;
  // Two waves in flight: wave k runs on stream k % 2 with its own buffers;
  // accumulate(k) waits for accumulate(k - 1), so the film sees the samples
  // in index order as with one stream.
  const bool two = !dump_rad && !prof && !(o->flags & ER_RENDER_ONE_STREAM) && o->spp > sw;
  if (two) {
    if ((st = ensure_wave2(s)) != ER_OK) return st;
    ER_CUDA(cudaEventRecord(s->ev_fork, s->stream));
    ER_CUDA(cudaStreamWaitEvent(s->stream2, s->ev_fork, 0));
  }
  const int g_tr[4] = {grid_for(k_trace<false, false, false>, kTravBlock, s->num_sms),
                       grid_for(k_trace<true, false, false>, kTravBlock, s->num_sms),
                       grid_for(k_trace<false, true, false>, kTravBlock, s->num_sms),
                       grid_for(k_trace<true, true, false>, kTravBlock, s->num_sms)};
  const int g_shade = grid_for(k_shade<false>, 128, s->num_sms);
  const BatchView NB;
  const int variant = (q8 ? 1 : 0) + (count ? 2 : 0);
  int64_t nl = 0;
  // Profiling: one event after every launch, attributed to its stage.
  s->ev_stage.clear();
  auto mark = [&](int stage) -> er_status {
    nl++;
    if (!prof) return ER_OK;
    size_t k = s->ev_stage.size() + 1;
    while (s->ev_pool.size() <= k) {
      cudaEvent_t e;
      ER_CUDA(cudaEventCreate(&e));
      s->ev_pool.push_back(e);
    }
    ER_CUDA(cudaEventRecord(s->ev_pool[k], s->stream));
    s->ev_stage.push_back(stage);
    return ER_OK;
  };
  if (prof) {
    if (s->ev_pool.empty()) {
      cudaEvent_t e;
      ER_CUDA(cudaEventCreate(&e));
      s->ev_pool.push_back(e);
    }
    ER_CUDA(cudaEventRecord(s->ev_pool[0], s->stream));
  }
  int32_t k = 0;
  for (int32_t s0 = 0; s0 < o->spp; s0 += sw, k++) {
    const bool alt = two && (k & 1);
    WaveView& w = alt ? s->wave2->v : s->wave->v;
    cudaStream_t strm = alt ? s->stream2 : s->stream;
    int32_t cur = std::min(sw, o->spp - s0);
    P.spp_wave = cur;
    P.sample_base = o->sample_begin + s0;
    int32_t n = cur * npix;
    k_raygen<false><<<(n + 255) / 256, 256, 0, strm>>>(s->dev, w, P, n, NB, GradArgs{});
    if ((st = mark(ER_STAGE_RAYGEN)) != ER_OK) return st;
    // trace(b): extension rays of bounce b + shadow rays of bounce b-1;
    // the extra trace(max_depth) finishes the last bounce's shadow rays.
    for (int32_t b = 0; b <= max_depth; b++) {
      uint32_t* err = s->err_word;
      switch (variant) {
        case 0: k_trace<false, false, false><<<g_tr[0], kTravBlock, 0, strm>>>(s->dev, w, b, err, NB, 7u); break;
        case 1: k_trace<true, false, false><<<g_tr[1], kTravBlock, 0, strm>>>(s->dev, w, b, err, NB, 7u); break;
        case 2: k_trace<false, true, false><<<g_tr[2], kTravBlock, 0, strm>>>(s->dev, w, b, err, NB, 7u); break;
        default: k_trace<true, true, false><<<g_tr[3], kTravBlock, 0, strm>>>(s->dev, w, b, err, NB, 7u); break;
      }
      if ((st = mark(ER_STAGE_TRACE)) != ER_OK) return st;
      if (b == max_depth) break;
      if (eval) k_shade<false, false, true><<<g_shade, 128, 0, strm>>>(s->dev, w, P, b, NB, *eval);
      else k_shade<false><<<g_shade, 128, 0, strm>>>(s->dev, w, P, b, NB, GradArgs{});
      if ((st = mark(ER_STAGE_SHADE)) != ER_OK) return st;
    }
    if (dump_rad) {
      k_dump<<<(n + 255) / 256, 256, 0, s->stream>>>(w, P, cur, s0, dump_rad, dump_b);
    } else {
      Film F = s->film;
      if (o->flags & ER_RENDER_KEEP_PATHS) {
        F.keep = s->kp_rad;
        F.keep_s0 = s0;
      }
      if (two && k > 0) ER_CUDA(cudaStreamWaitEvent(strm, s->ev_acc[(k - 1) & 1], 0));
      k_accumulate<false><<<(npix + 127) / 128, 128, 0, strm>>>(w, P, F, cur, NB);
      if (o->flags & ER_RENDER_SNAPSHOTS) {
        // the reader (er_snapshot) holds the lock while it copies the
        // snapshot out, so the buffer is not overwritten under it
        std::lock_guard<std::mutex> lk(s->snap_mu);
        ER_CUDA(cudaMemcpyAsync(s->snap_beauty, F.beauty, (size_t)npix * sizeof(float4), cudaMemcpyDeviceToDevice,
                                strm));
        ER_CUDA(cudaMemcpyAsync(s->snap_samples, F.samples, (size_t)npix * 4, cudaMemcpyDeviceToDevice, strm));
        ER_CUDA(cudaEventRecord(s->snap_event, strm));
        s->snap_valid = true;
      }
      if (two) ER_CUDA(cudaEventRecord(s->ev_acc[k & 1], strm));
    }
    if ((st = mark(ER_STAGE_ACCUMULATE)) != ER_OK) return st;
    ER_CUDA(cudaGetLastError());
  }
  // join: the last accumulate follows every launch of both streams
  if (two) ER_CUDA(cudaStreamWaitEvent(s->stream, s->ev_acc[(k - 1) & 1], 0));
  if (launches) *launches = nl;
  return ER_OK;
}

// Snapshot buffer, event and reader stream of the scene's film size.
er_status ensure_snapshot(er_scene* s) {
  std::lock_guard<std::mutex> lk(s->snap_mu);
  const int32_t W = s->camera.x_res, H = s->camera.y_res;
  if (s->snap_beauty && s->snap_w == W && s->snap_h == H) return ER_OK;
  cudaFree(s->snap_beauty);
  cudaFree(s->snap_samples);
  s->snap_beauty = nullptr;
  s->snap_samples = nullptr;
  s->snap_valid = false;
  const size_t np = (size_t)W * H;
  if (cudaMalloc(&s->snap_beauty, np * sizeof(float4)) != cudaSuccess ||
      cudaMalloc(&s->snap_samples, np * 4) != cudaSuccess) {
    cudaGetLastError();
    return fail(ER_ERR_OOM, "snapshot buffers");
  }
  if (!s->snap_event) ER_CUDA(cudaEventCreateWithFlags(&s->snap_event, cudaEventDisableTiming));
  if (!s->snap_stream) ER_CUDA(cudaStreamCreateWithFlags(&s->snap_stream, cudaStreamNonBlocking));
  s->snap_w = W;
  s->snap_h = H;
  return ER_OK;
}

er_status check_opts(er_scene* s, const er_render_opts* o) {
  if (!o) return fail(ER_ERR_INVALID_ARG, "NULL argument");
  if (o->spp < 0 || o->sample_begin < 0 || o->max_depth < 0 || o->max_depth > 64 || o->spp_per_wave < 0)
    return fail(ER_ERR_INVALID_ARG, "render options out of range");
  // sample indices are int32 on the device: the last one must fit
  if ((int64_t)o->sample_begin + o->spp > INT32_MAX)
    return fail(ER_ERR_INVALID_ARG, "sample_begin + spp exceeds INT32_MAX");
  if (!s) return fail(ER_ERR_INVALID_ARG, "NULL argument");
  ER_CUDA(cudaSetDevice(s->device));
  return ER_OK;
}

}  // namespace

void free_wave(er_scene* s) {
  for (Wave** pw : {&s->wave, &s->wave2}) {
    if (!*pw) continue;
    for (void* p : (*pw)->mem) cudaFree(p);
    delete *pw;
    *pw = nullptr;
  }
}

void free_film(er_scene* s) {
  Film& F = s->film;
  cudaFree(F.beauty);
  for (int k = 0; k < 3; k++) cudaFree(F.aov[k]);
  cudaFree(F.sum);
  cudaFree(F.samples);
  cudaFree(F.pathcount);
  F = Film();
}

er_status render_paths_device(er_scene* s, const er_render_opts* o, float* d_rad, int32_t* d_b, bool grad_wave,
                              int64_t* launches) {
  er_render_opts oo = *o;
  oo.flags &= ~(uint32_t)(ER_RENDER_AOV | ER_RENDER_SNAPSHOTS);
  return run(s, &oo, d_rad, d_b, launches, grad_wave);
}

// The gradient wavefront: the same waves as run(), with the gradient
// variants of raygen and shade and a final per-path resolve in place of the
// accumulation.
er_status render_backward_device(er_scene* s, const er_render_opts* o, const GradArgs& G, int64_t* launches) {
  const int32_t W = s->camera.x_res, H = s->camera.y_res;
  const int32_t npix = W * H;
  const int32_t max_depth = o->max_depth > 0 ? o->max_depth : 5;
  int32_t sw = o->spp_per_wave > 0 ? o->spp_per_wave : default_spp_per_wave(o->spp, npix);
  sw = std::min(sw, std::max(1, o->spp));
  er_status st = ensure_wave(s, (int64_t)sw * npix, false, true);
  if (st != ER_OK) return st;
  // waves alternate between two pipelines as in run(); the gradients are
  // atomic sums, so the waves need no order between them
  const bool two = o->spp > sw;
  if (two) {
    if ((st = ensure_wave2(s, true)) != ER_OK) return st;
    ER_CUDA(cudaEventRecord(s->ev_fork, s->stream));
    ER_CUDA(cudaStreamWaitEvent(s->stream2, s->ev_fork, 0));
  }
  WaveParams P;
  P.W = W; P.H = H; P.npix = npix; P.max_depth = max_depth;
  P.k0 = (uint32_t)o->seed; P.k1 = (uint32_t)(o->seed >> 32);
  P.flags = o->flags & ER_RENDER_ENV_ALIAS;
  const int g_tr[2] = {grid_for(k_trace<false, false, false>, kTravBlock, s->num_sms),
                       grid_for(k_trace<true, false, false>, kTravBlock, s->num_sms)};
  const int g_sh = grid_for(k_shade<false, true>, 128, s->num_sms);
  const BatchView NB;
  int32_t k = 0;
  for (int32_t s0 = 0; s0 < o->spp; s0 += sw, k++) {
    const bool alt = two && (k & 1);
    WaveView& w = alt ? s->wave2->v : s->wave->v;
    cudaStream_t strm = alt ? s->stream2 : s->stream;
    const int32_t cur = std::min(sw, o->spp - s0);
    P.spp_wave = cur;
    P.sample_base = o->sample_begin + s0;
    const int32_t n = cur * npix;
    k_raygen<false, true><<<(n + 255) / 256, 256, 0, strm>>>(s->dev, w, P, n, NB, G);
    for (int32_t b = 0; b <= max_depth; b++) {
      if (s->dev.use_q8)
        k_trace<true, false, false><<<g_tr[1], kTravBlock, 0, strm>>>(s->dev, w, b, s->err_word, NB, 7u);
      else
        k_trace<false, false, false><<<g_tr[0], kTravBlock, 0, strm>>>(s->dev, w, b, s->err_word, NB, 7u);
      if (b == max_depth) break;
      k_shade<false, true><<<g_sh, 128, 0, strm>>>(s->dev, w, P, b, NB, G);
    }
    k_resolve_grad<<<(n + 255) / 256, 256, 0, strm>>>(w, n, G);
    ER_CUDA(cudaGetLastError());
    *launches += 2 * max_depth + 3;  // raygen, max_depth + 1 traces, max_depth shades, resolve
  }
  if (two) {
    ER_CUDA(cudaEventRecord(s->ev_acc[0], s->stream2));
    ER_CUDA(cudaStreamWaitEvent(s->stream, s->ev_acc[0], 0));
  }
  return ER_OK;
}

er_status wave_create(int64_t cap, unsigned long long* stats, Wave** out) {
  Wave* ww = new Wave();
  er_status st = wave_fill(ww, cap, false, false, stats);
  if (st != ER_OK) {
    wave_destroy(ww);
    return st;
  }
  *out = ww;
  return ER_OK;
}

void wave_destroy(Wave* w) {
  if (!w) return;
  for (void* p : w->mem) cudaFree(p);
  delete w;
}

er_status film_clear(const Film& F, cudaStream_t stream) {
  int32_t npix = F.w * F.h;
  if (npix <= 0) return ER_OK;
  k_film_clear<<<(npix + 255) / 256, 256, 0, stream>>>(F, npix);
  ER_CUDA(cudaGetLastError());
  return ER_OK;
}

// The batch's launch sequence: per wave raygen, max_depth + 1 traversal
// launches (three each in a split schedule), max_depth shade launches and
// one accumulate launch.  Slices of one job across waves are accumulated in
// sample order, so each job's film equals a single-scene render's.
er_status batch_launch(const DevScene& S, Wave* wv, const BatchSeg* d_segs, const BatchJobDev* d_jobs,
                       const std::vector<BatchWave>& waves, const BatchSchedule& sch, int num_sms, uint32_t* err,
                       cudaStream_t stream, int64_t* launches, const BatchPair* pair) {
  // resident blocks per SM
  const int occ_tr[2] = {blocks_per_sm((const void*)k_trace<false, false, true>, kTravBlock),
                         blocks_per_sm((const void*)k_trace<true, false, true>, kTravBlock)};
  const int occ_sh = blocks_per_sm((const void*)k_shade<true>, 128);
  const int q8 = S.use_q8 ? 1 : 0;
  const int tb = sch.trace_blocks_per_sm > 0 ? std::min(sch.trace_blocks_per_sm, occ_tr[q8]) : occ_tr[q8];
  const int sb = sch.shade_blocks_per_sm > 0 ? std::min(sch.shade_blocks_per_sm, occ_sh) : occ_sh;
  const int g_tr = tb * num_sms, g_sh = sb * num_sms;
  if (launches) *launches = 0;
  if (waves.empty()) return ER_OK;  // (also: occupancy queries done before any stream capture)
  const WaveParams P0{};
  int64_t nl = 0;
  // two pipelines: wave k on (pair->w2, pair->s2) when k is odd
  const bool two = pair && pair->w2 && waves.size() >= 2;
  if (two) {
    ER_CUDA(cudaEventRecord(pair->ev_fork, stream));
    ER_CUDA(cudaStreamWaitEvent(pair->s2, pair->ev_fork, 0));
  }
  for (size_t k = 0; k < waves.size(); k++) {
    const BatchWave& bw = waves[k];
    const bool alt = two && (k & 1);
    const Wave* wk = alt ? pair->w2 : wv;
    const WaveView& w = wk->v;
    cudaStream_t strm = alt ? pair->s2 : stream;
    auto trace = [&](int32_t b, const BatchView& B, uint32_t phases) {
      if (q8) k_trace<true, false, true><<<g_tr, kTravBlock, 0, strm>>>(S, w, b, err, B, phases);
      else k_trace<false, false, true><<<g_tr, kTravBlock, 0, strm>>>(S, w, b, err, B, phases);
      nl++;
    };
    if (bw.n_paths > wk->cap) return fail(ER_ERR_INVALID_ARG, "batch wave larger than its buffers");
    BatchView B;
    B.segs = d_segs + bw.seg_begin;
    B.jobs = d_jobs;
    B.n_segs = bw.n_segs;
    B.n_acc = bw.n_acc;
    const int32_t n = bw.n_paths;
    k_raygen<true><<<(n + 255) / 256, 256, 0, strm>>>(S, w, P0, n, B, GradArgs{});
    nl++;
    for (int32_t b = 0; b <= bw.max_depth; b++) {
      if (sch.split_trace) {
        trace(b, B, 1u);
        trace(b, B, 2u);
        trace(b, B, 4u);
      } else {
        trace(b, B, 7u);
      }
      if (b == bw.max_depth) break;
      k_shade<true><<<g_sh, 128, 0, strm>>>(S, w, P0, b, B, GradArgs{});
      nl++;
    }
    // a job's slices accumulate in wave order
    if (two && k > 0) ER_CUDA(cudaStreamWaitEvent(strm, pair->ev_acc[(k - 1) & 1], 0));
    k_accumulate<true><<<(bw.n_acc + 127) / 128, 128, 0, strm>>>(w, P0, Film(), 0, B);
    nl++;
    if (two) ER_CUDA(cudaEventRecord(pair->ev_acc[k & 1], strm));
  }
  if (two) {
    ER_CUDA(cudaEventRecord(pair->ev_join, pair->s2));
    ER_CUDA(cudaStreamWaitEvent(stream, pair->ev_join, 0));
    ER_CUDA(cudaStreamWaitEvent(stream, pair->ev_acc[(waves.size() - 1) & 1], 0));
  }
  ER_CUDA(cudaGetLastError());
  if (launches) *launches = nl;
  return ER_OK;
}

}  // namespace er

using namespace er;

namespace er {
namespace {

// Queues the film copies on the scene's stream (the caller synchronises).
er_status film_read_async(er_scene* s, uint32_t flags, float* beauty, float* normal, float* tangent,
                          float* bitangent, uint32_t* samples, uint32_t* pathcount) {
  Film& F = s->film;
  if (!F.beauty) return fail(ER_ERR_INVALID_ARG, "nothing rendered yet");
  bool dev = flags & ER_RENDER_DEVICE_OUT;
  size_t np = (size_t)F.w * F.h;
  er_status st;
  if ((st = copy_out(s, dev, beauty, F.beauty, np * sizeof(float4))) != ER_OK) return st;
  float* aovs[3] = {normal, tangent, bitangent};
  for (int k = 0; k < 3; k++) {
    if (!aovs[k]) continue;
    if (!F.aov_on) return fail(ER_ERR_INVALID_ARG, "AOV passes were not rendered");
    if ((st = copy_out(s, dev, aovs[k], F.aov[k], np * sizeof(float4))) != ER_OK) return st;
  }
  if ((st = copy_out(s, dev, samples, F.samples, np * sizeof(uint32_t))) != ER_OK) return st;
  return copy_out(s, dev, pathcount, F.pathcount, np * sizeof(uint32_t));
}

}  // namespace

er_status render_eval_device(er_scene* s, const er_render_opts* o, const GradArgs& G, float* beauty,
                             uint32_t* samples, uint32_t* pathcount) {
  const bool fp64 = o->flags & ER_RENDER_ACCUM_FP64;
  er_status st = ensure_film(s, false, fp64, true);
  if (st != ER_OK) return st;
  er_render_opts oo = *o;
  oo.flags &= ER_RENDER_ENV_ALIAS | ER_RENDER_ACCUM_FP64;
  int64_t launches = 0;
  const bool eval = G.eval_mat || G.eval_env;  // without either: er_render's own shade stage
  if ((st = run(s, &oo, nullptr, nullptr, &launches, false, eval ? &G : nullptr)) != ER_OK) return st;
  if ((st = film_read_async(s, o->flags & ER_RENDER_DEVICE_OUT, beauty, nullptr, nullptr, nullptr, samples,
                            pathcount)) != ER_OK)
    return st;
  ER_CUDA(cudaStreamSynchronize(s->stream));
  return check_device_error(s);
}

}  // namespace er

extern "C" er_status er_film_read(er_scene* s, uint32_t flags, float* beauty, float* normal, float* tangent,
                                  float* bitangent, uint32_t* samples, uint32_t* pathcount) {
  return guarded("er_film_read", [&]() -> er_status {
    if (!s) return fail(ER_ERR_INVALID_ARG, "scene is NULL");
    er_status st = film_read_async(s, flags, beauty, normal, tangent, bitangent, samples, pathcount);
    if (st != ER_OK) return st;
    ER_CUDA(cudaStreamSynchronize(s->stream));
    return ER_OK;
  });
}

extern "C" er_status er_film_read_sums(er_scene* s, uint32_t flags, double* sums, uint32_t* samples) {
  return guarded("er_film_read_sums", [&]() -> er_status {
    if (!s) return fail(ER_ERR_INVALID_ARG, "scene is NULL");
    const Film& F = s->film;
    if (!F.beauty || !F.sum || !F.sum_valid)
      return fail(ER_ERR_INVALID_ARG, "the film holds no FP64 sums (render it with ER_RENDER_ACCUM_FP64)");
    ER_CUDA(cudaSetDevice(s->device));
    const bool dev = flags & ER_RENDER_DEVICE_OUT;
    const size_t np = (size_t)F.w * F.h;
    er_status st;
    if ((st = copy_out(s, dev, sums, F.sum, np * 3 * sizeof(double))) != ER_OK) return st;
    if ((st = copy_out(s, dev, samples, F.samples, np * sizeof(uint32_t))) != ER_OK) return st;
    ER_CUDA(cudaStreamSynchronize(s->stream));
    return ER_OK;
  });
}

extern "C" er_status er_snapshot(er_scene* s, float* beauty, uint32_t* samples) {
  return guarded("er_snapshot", [&]() -> er_status {
    if (!s) return fail(ER_ERR_INVALID_ARG, "scene is NULL");
    ER_CUDA(cudaSetDevice(s->device));
    std::lock_guard<std::mutex> lk(s->snap_mu);
    if (!s->snap_valid) return fail(ER_ERR_INVALID_ARG, "no snapshot yet (render with ER_RENDER_SNAPSHOTS)");
    const size_t np = (size_t)s->snap_w * s->snap_h;
    ER_CUDA(cudaStreamWaitEvent(s->snap_stream, s->snap_event, 0));
    if (beauty) ER_CUDA(cudaMemcpyAsync(beauty, s->snap_beauty, np * sizeof(float4), cudaMemcpyDeviceToHost, s->snap_stream));
    if (samples) ER_CUDA(cudaMemcpyAsync(samples, s->snap_samples, np * 4, cudaMemcpyDeviceToHost, s->snap_stream));
    ER_CUDA(cudaStreamSynchronize(s->snap_stream));
    return ER_OK;
  });
}

extern "C" er_status er_render(er_scene* s, const er_render_opts* o, float* beauty, float* normal, float* tangent,
                               float* bitangent, uint32_t* samples, uint32_t* pathcount, er_render_stats* stats) {
  return guarded("er_render", [&]() -> er_status {
    er_status st = check_opts(s, o);
    if (st != ER_OK) return st;
    const bool aov = o->flags & ER_RENDER_AOV;
    const bool fp64 = o->flags & ER_RENDER_ACCUM_FP64;
    if ((o->flags & ER_RENDER_ENV_ALIAS) && (st = build_env_alias(s)) != ER_OK) return st;
    if ((st = build_env_lut(s)) != ER_OK) return st;
    if ((st = ensure_film(s, aov, fp64, !(o->flags & ER_RENDER_CONTINUE))) != ER_OK) return st;
    if ((o->flags & ER_RENDER_SNAPSHOTS) && (st = ensure_snapshot(s)) != ER_OK) return st;
    const bool keep = o->flags & ER_RENDER_KEEP_PATHS;
    s->kp_valid = false;
    if (keep) {
      const int64_t need = (int64_t)o->spp * s->camera.x_res * s->camera.y_res;
      if (need > s->kp_cap) {
        ER_CUDA(cudaStreamSynchronize(s->stream));
        cudaFree(s->kp_rad);
        s->kp_rad = nullptr;
        s->kp_cap = 0;
        if (cudaMalloc(&s->kp_rad, (size_t)std::max<int64_t>(need, 1) * 12) != cudaSuccess) {
          cudaGetLastError();
          return fail(ER_ERR_OOM, "kept-path radiance allocation failed");
        }
        s->kp_cap = need;
      }
    }
    // counters before the call, into page-locked memory (no blocking copy)
    unsigned long long* st0 = (unsigned long long*)(s->h_pin + 64);
    if (stats) ER_CUDA(cudaMemcpyAsync(st0, s->d_stats, 64, cudaMemcpyDeviceToHost, s->stream));
    ER_CUDA(cudaEventRecord(s->ev0, s->stream));
    int64_t launches = 0;
    if ((st = run(s, o, nullptr, nullptr, &launches)) != ER_OK) return st;
    if (keep) {
      s->kp_valid = true;
      s->kp_seed = o->seed;
      s->kp_begin = o->sample_begin;
      s->kp_spp = o->spp;
      s->kp_depth = o->max_depth > 0 ? o->max_depth : 5;
      s->kp_flags = o->flags & ER_RENDER_ENV_ALIAS;
      s->kp_version = s->version;
    }
    ER_CUDA(cudaEventRecord(s->ev1, s->stream));
    if (!(o->flags & ER_RENDER_NO_OUTPUT)) {
      uint32_t fl = o->flags & ER_RENDER_DEVICE_OUT;
      if ((st = film_read_async(s, fl, beauty, aov ? normal : nullptr, aov ? tangent : nullptr,
                                aov ? bitangent : nullptr, samples, pathcount)) != ER_OK)
        return st;
    }
    // the device error word rides on the same stream: one wait for the
    // film, the word and the call's end
    uint32_t* h_err = (uint32_t*)s->h_pin;
    ER_CUDA(cudaMemcpyAsync(h_err, s->err_word, 4, cudaMemcpyDeviceToHost, s->stream));
    ER_CUDA(cudaStreamSynchronize(s->stream));
    if (*h_err != 0 && (st = check_device_error(s)) != ER_OK) return st;
    if (stats) {
      float ms = 0;
      cudaEventElapsedTime(&ms, s->ev0, s->ev1);
      unsigned long long st1[8];
      ER_CUDA(cudaMemcpy(st1, s->d_stats, sizeof st1, cudaMemcpyDeviceToHost));
      std::memset(stats, 0, sizeof *stats);
      stats->ms = ms;
      stats->samples = (int64_t)o->spp * s->camera.x_res * s->camera.y_res;
      stats->rays_closest = (int64_t)(st1[0] - st0[0]);
      stats->rays_shadow = (int64_t)(st1[1] - st0[1]);
      stats->closest_nodes = (int64_t)(st1[2] - st0[2]);
      stats->closest_tris = (int64_t)(st1[3] - st0[3]);
      stats->shadow_nodes = (int64_t)(st1[4] - st0[4]);
      stats->shadow_tris = (int64_t)(st1[5] - st0[5]);
      stats->path_vertices = (int64_t)(st1[6] - st0[6]);
      stats->kernel_launches = launches;
      for (size_t k = 0; k < s->ev_stage.size(); k++) {
        float e = 0;
        cudaEventElapsedTime(&e, s->ev_pool[k], s->ev_pool[k + 1]);
        stats->stage_ms[s->ev_stage[k]] += e;
        stats->stage_launches[s->ev_stage[k]]++;
      }
    }
    return ER_OK;
  });
}

extern "C" er_status er_render_paths(er_scene* s, const er_render_opts* o, float* radiance, int32_t* bounces) {
  return guarded("er_render_paths", [&]() -> er_status {
    er_status st = check_opts(s, o);
    if (st != ER_OK) return st;
    if (!radiance || !bounces) return fail(ER_ERR_INVALID_ARG, "NULL output");
    size_t n = (size_t)o->spp * s->camera.x_res * s->camera.y_res;
    if (n == 0) return ER_OK;
    float* d_rad = nullptr;
    int32_t* d_b = nullptr;
    if (cudaMalloc(&d_rad, n * 3 * sizeof(float)) != cudaSuccess || cudaMalloc(&d_b, n * sizeof(int32_t)) != cudaSuccess) {
      cudaGetLastError();
      cudaFree(d_rad);
      return fail(ER_ERR_OOM, "path dump allocation failed");
    }
    er_render_opts oo = *o;
    oo.flags &= ~(uint32_t)(ER_RENDER_AOV | ER_RENDER_SNAPSHOTS);
    if (((oo.flags & ER_RENDER_ENV_ALIAS) && (st = build_env_alias(s)) != ER_OK) || (st = build_env_lut(s)) != ER_OK) {
      cudaFree(d_rad);
      cudaFree(d_b);
      return st;
    }
    st = run(s, &oo, d_rad, d_b, nullptr);
    if (st == ER_OK) {
      cudaMemcpyAsync(radiance, d_rad, n * 3 * sizeof(float), cudaMemcpyDeviceToHost, s->stream);
      cudaMemcpyAsync(bounces, d_b, n * sizeof(int32_t), cudaMemcpyDeviceToHost, s->stream);
      cudaError_t e = cudaStreamSynchronize(s->stream);
      if (e != cudaSuccess) st = cuda_fail(e, "er_render_paths");
    }
    cudaFree(d_rad);
    cudaFree(d_b);
    if (st == ER_OK) st = check_device_error(s);
    return st;
  });
}

// ------------------------------------------------------------------------
// Allocation-free rendering (er_render_noalloc).
//
// Some callers must not allocate device memory while they render: a host
// application that sizes its whole GPU budget once at start-up and forbids
// allocations afterwards (an editor's live preview pane next to its own
// renderer, a service with a fixed per-tenant memory quota), or a caller
// whose render thread may not enter the CUDA allocator at all.  For them the
// wavefront's scratch (path state and ray queues) lives in one file-scope
// __device__ array sized for ER_NOALLOC_MAX_PATHS paths per wave; the film is
// the caller's own device buffers.  The array exists on every GPU that loads
// this library, for the life of the process.

namespace er {
namespace {

constexpr int64_t kNoAllocPaths = ER_NOALLOC_MAX_PATHS;
constexpr size_t pad256(size_t b) { return (b + 255) & ~(size_t)255; }
constexpr size_t kNoAllocBytes = 2 * pad256(kNoAllocPaths * 16)      // throughput, radiance
                                 + pad256(kNoAllocPaths * 64)        // pending MIS terms
                                 + pad256(kNoAllocPaths * 2)         // visibility
                                 + pad256(kNoAllocPaths * 4)         // bounce counts
                                 + 4 * pad256(kNoAllocPaths * 16)    // two extension queues
                                 + pad256(kNoAllocPaths * 16)        // hits
                                 + 3 * pad256(kNoAllocPaths * 32)    // shadow queue (two halves)
                                 + pad256(16 * 4) + pad256(16 * 8);  // queue counters, ray counters

}  // namespace
}  // namespace er

// The scratch of er_render_noalloc (about 19 MB for 65,536 paths).
static __device__ __align__(256) unsigned char g_noalloc_scratch[er::kNoAllocBytes];

namespace er {
namespace {

std::mutex g_noalloc_lock;
unsigned char* g_noalloc_ptr[128];  // device address of the scratch, per device ordinal

// Host code must not take the address of g_noalloc_scratch directly (that is
// a host-side shadow); the device address is looked up with the device
// current.  er_scene_create refreshes it (noalloc_prepare), so the lookup,
// and with it the loading of this file's module that holds the array, happens
// while a scene is being created and not inside er_render_noalloc; a scene
// created after a cudaDeviceReset replaces the cached address of the old
// context.
er_status noalloc_lookup(int device, bool refresh, unsigned char** out) {
  std::lock_guard<std::mutex> lk(g_noalloc_lock);
  if (device < 0 || device >= 128) return fail(ER_ERR_INVALID_ARG, "device ordinal out of range");
  if (refresh || !g_noalloc_ptr[device]) {
    void* p = nullptr;
    cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
    if (e != cudaSuccess || !p) {
      g_noalloc_ptr[device] = nullptr;
      return cuda_fail(e != cudaSuccess ? e : cudaErrorInvalidSymbol, "cudaGetSymbolAddress");
    }
    g_noalloc_ptr[device] = (unsigned char*)p;
  }
  if (out) *out = g_noalloc_ptr[device];
  return ER_OK;
}

WaveView noalloc_view(unsigned char* base, unsigned long long*& stats) {
  WaveView w;
  size_t off = 0;
  auto take = [&](size_t bytes) {
    unsigned char* p = base + off;
    off += pad256(bytes);
    return p;
  };
  const int64_t N = kNoAllocPaths;
  w.aov = false;
  w.thr = (float4*)take(N * 16);
  w.light = (float4*)take(N * 16);
  w.pend = (float4*)take(N * 64);
  w.vis = (uint8_t*)take(N * 2);
  w.bounces = (int32_t*)take(N * 4);
  w.q_o[0] = (float4*)take(N * 16);
  w.q_d[0] = (float4*)take(N * 16);
  w.q_o[1] = (float4*)take(N * 16);
  w.q_d[1] = (float4*)take(N * 16);
  w.hits = (float4*)take(N * 16);
  w.s_o = (float4*)take(N * 32);
  w.s_d = (float4*)take(N * 32);
  w.s_p = (float4*)take(N * 32);
  w.counts = (int32_t*)take(16 * 4);
  stats = (unsigned long long*)take(16 * 8);
  w.stats = stats;
  w.shadow_half = N;
  return w;
}

}  // namespace

void noalloc_prepare(int device) {
  if (noalloc_lookup(device, true, nullptr) != ER_OK) cudaGetLastError();
}

}  // namespace er

extern "C" er_status er_render_noalloc(er_scene* s, const er_render_opts* o, float* beauty, uint32_t* samples,
                                       uint32_t* pathcount) {
  return guarded("er_render_noalloc", [&]() -> er_status {
    er_status st = check_opts(s, o);
    if (st != ER_OK) return st;
    if (!beauty || !samples || !pathcount) return fail(ER_ERR_INVALID_ARG, "er_render_noalloc: NULL film buffer");
    if ((uintptr_t)beauty % 16 != 0) return fail(ER_ERR_INVALID_ARG, "er_render_noalloc: beauty must be 16-byte aligned");
    if ((uintptr_t)samples % 4 != 0 || (uintptr_t)pathcount % 4 != 0)
      return fail(ER_ERR_INVALID_ARG, "er_render_noalloc: samples and pathcount must be 4-byte aligned");
    const uint32_t allowed = ER_RENDER_CONTINUE;
    if (o->flags & ~allowed)
      return fail(ER_ERR_INVALID_ARG, "er_render_noalloc: only ER_RENDER_CONTINUE is supported");
    const int32_t W = s->camera.x_res, H = s->camera.y_res;
    const int64_t npix = (int64_t)W * H;
    if (npix > kNoAllocPaths)
      return fail(ER_ERR_INVALID_ARG, "er_render_noalloc: " + std::to_string(npix) + " pixels exceed the limit of " +
                                          std::to_string(kNoAllocPaths) + " (ER_NOALLOC_MAX_PATHS)");
    unsigned char* base = nullptr;
    if ((st = noalloc_lookup(s->device, false, &base)) != ER_OK) return st;
    unsigned long long* stats = nullptr;
    WaveView w = noalloc_view(base, stats);
    Film F;
    F.w = W;
    F.h = H;
    F.beauty = (float4*)beauty;
    F.samples = samples;
    F.pathcount = pathcount;
    F.aov_on = false;
    if (!(o->flags & ER_RENDER_CONTINUE)) {
      k_film_clear<<<(unsigned)((npix + 255) / 256), 256, 0, s->stream>>>(F, (int32_t)npix);
    }
    const int32_t max_depth = o->max_depth > 0 ? o->max_depth : 5;
    int32_t sw = o->spp_per_wave > 0 ? o->spp_per_wave : (int32_t)(kNoAllocPaths / npix);
    sw = std::max(1, std::min(sw, (int32_t)(kNoAllocPaths / npix)));
    WaveParams P;
    P.W = W; P.H = H; P.npix = (int32_t)npix; P.max_depth = max_depth;
    P.k0 = (uint32_t)o->seed; P.k1 = (uint32_t)(o->seed >> 32);
    P.flags = 0;
    const int g_tr = grid_for(k_trace<false, false, false>, kTravBlock, s->num_sms);
    const int g_tr8 = grid_for(k_trace<true, false, false>, kTravBlock, s->num_sms);
    const int g_sh = grid_for(k_shade<false>, 128, s->num_sms);
    const BatchView NB;
    for (int32_t s0 = 0; s0 < o->spp; s0 += sw) {
      int32_t cur = std::min(sw, o->spp - s0);
      P.spp_wave = cur;
      P.sample_base = o->sample_begin + s0;
      int32_t n = cur * (int32_t)npix;
      k_raygen<false><<<(n + 255) / 256, 256, 0, s->stream>>>(s->dev, w, P, n, NB, GradArgs{});  // also zeroes the queue counters
      for (int32_t b = 0; b <= max_depth; b++) {
        if (s->dev.use_q8)
          k_trace<true, false, false><<<g_tr8, kTravBlock, 0, s->stream>>>(s->dev, w, b, s->err_word, NB, 7u);
        else
          k_trace<false, false, false><<<g_tr, kTravBlock, 0, s->stream>>>(s->dev, w, b, s->err_word, NB, 7u);
        if (b == max_depth) break;
        k_shade<false><<<g_sh, 128, 0, s->stream>>>(s->dev, w, P, b, NB, GradArgs{});
      }
      k_accumulate<false><<<(unsigned)((npix + 127) / 128), 128, 0, s->stream>>>(w, P, F, cur, NB);
    }
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return cuda_fail(e, "er_render_noalloc launch");
    return check_device_error(s);
  });
}
