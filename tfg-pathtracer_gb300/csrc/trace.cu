// er_trace_closest: closest-hit queries on caller rays, the parity gate for
// BVH::transverse (BVH.hpp:120-157) as throwRay uses it (kernel.cu:152-173).
#include "internal.h"
#include "traverse.cuh"

namespace er {
namespace {

template <bool Q8, bool STATS>
__global__ void __launch_bounds__(kTravBlock, kTravMinBlocks)
    k_trace_rays(DevScene S, const float* __restrict__ rays, int32_t n, int normalize, int32_t* tri, float* dist,
                 float* uv, unsigned long long* stats, int32_t* counter, uint32_t* err) {
  __shared__ int2 stk[kSmemStack * kTravBlock];
  TravStats st{0, 0, 0};
  persistent_traverse<kClosest, Q8, STATS>(
      S, n, counter, stk + threadIdx.x, st, err,
      [&](int32_t i, auto& tr) {
        const float* q = rays + 6 * (int64_t)i;
        f3 o = mk(q[0], q[1], q[2]);
        f3 d = mk(q[3], q[4], q[5]);
        if (normalize) d = xnormalize(d);  // Ray.hpp:17
        tr.init(S, o, d, mk1(0.f), 0.f);
      },
      [&](int32_t i, auto& tr) {
        tri[i] = tr.slot >= 0 ? __float_as_int(__ldg(S.tri_v + 3 * (size_t)tr.slot).w) : -1;
        if (dist) dist[i] = tr.slot >= 0 ? tr.best : 0.0f;
        if (uv) {
          uv[2 * (int64_t)i] = tr.slot >= 0 ? tr.u : 0.0f;
          uv[2 * (int64_t)i + 1] = tr.slot >= 0 ? tr.v : 0.0f;
        }
      });
  if (STATS) {
    atomicAdd(&stats[8], (unsigned long long)st.nodes);
    atomicAdd(&stats[9], (unsigned long long)st.boxes);
    atomicAdd(&stats[10], (unsigned long long)st.tris);
  }
}

template <bool Q8, bool STATS>
void launch(er_scene* s, const float* rays, int64_t n, int normalize, int32_t* tri, float* dist, float* uv) {
  const int grid = blocks_per_sm((const void*)k_trace_rays<Q8, STATS>, kTravBlock) * s->num_sms;
  int64_t need = (n + kTravBlock - 1) / kTravBlock;
  int g = (int)(need < grid ? need : grid);
  if (g < 1) g = 1;
  int32_t* counter = (int32_t*)((char*)s->err_word + 32);
  cudaMemsetAsync(counter, 0, sizeof(int32_t), s->stream);
  k_trace_rays<Q8, STATS><<<g, kTravBlock, 0, s->stream>>>(s->dev, rays, (int32_t)n, normalize, tri, dist, uv,
                                                          s->d_stats, counter, s->err_word);
}

}  // namespace
}  // namespace er

using namespace er;

extern "C" er_status er_trace_closest(er_scene* s, const float* rays, int64_t n, int32_t* tri_id, float* dist,
                                      float* uv, uint32_t flags, er_trace_stats* stats) {
  return guarded("er_trace_closest", [&]() -> er_status {
    if (!s || n < 0 || (n > 0 && (!rays || !tri_id))) return fail(ER_ERR_INVALID_ARG, "bad argument");
    if (n > 0x7FFFFFFF) return fail(ER_ERR_INVALID_ARG, "more than 2^31-1 rays in one call");
    ER_CUDA(cudaSetDevice(s->device));
    if (n == 0) return ER_OK;
    const bool dev = flags & ER_TRACE_DEVICE_PTRS;
    const bool want_stats = (flags & ER_TRACE_STATS) && stats;
    const float* d_rays = rays;
    int32_t* d_tri = tri_id;
    float *d_dist = dist, *d_uv = uv;
    std::vector<void*> tmp;
    auto cleanup = [&]() {
      for (void* p : tmp) cudaFree(p);
    };
    if (!dev) {
      void *a = nullptr, *b = nullptr, *c = nullptr, *e = nullptr;
      if (cudaMalloc(&a, (size_t)n * 6 * sizeof(float)) != cudaSuccess ||
          cudaMalloc(&b, (size_t)n * sizeof(int32_t)) != cudaSuccess ||
          (dist && cudaMalloc(&c, (size_t)n * sizeof(float)) != cudaSuccess) ||
          (uv && cudaMalloc(&e, (size_t)n * 2 * sizeof(float)) != cudaSuccess)) {
        cudaGetLastError();
        cudaFree(a); cudaFree(b); cudaFree(c); cudaFree(e);
        return fail(ER_ERR_OOM, "trace buffers");
      }
      tmp = {a, b, c, e};
      d_rays = (const float*)a;
      d_tri = (int32_t*)b;
      d_dist = (float*)c;
      d_uv = (float*)e;
      cudaMemcpyAsync(a, rays, (size_t)n * 6 * sizeof(float), cudaMemcpyHostToDevice, s->stream);
    }
    unsigned long long s0[16] = {0};
    if (want_stats) cudaMemcpyAsync(s0, s->d_stats, sizeof s0, cudaMemcpyDeviceToHost, s->stream);
    cudaEventRecord(s->ev0, s->stream);
    int norm = (flags & ER_TRACE_NORMALIZED) ? 0 : 1;
    if (s->dev.use_q8) {
      if (want_stats) launch<true, true>(s, d_rays, n, norm, d_tri, d_dist, d_uv);
      else launch<true, false>(s, d_rays, n, norm, d_tri, d_dist, d_uv);
    } else {
      if (want_stats) launch<false, true>(s, d_rays, n, norm, d_tri, d_dist, d_uv);
      else launch<false, false>(s, d_rays, n, norm, d_tri, d_dist, d_uv);
    }
    cudaEventRecord(s->ev1, s->stream);
    cudaError_t ce = cudaGetLastError();
    if (ce != cudaSuccess) {
      cleanup();
      return cuda_fail(ce, "k_trace_rays launch");
    }
    if (!dev) {
      cudaMemcpyAsync(tri_id, d_tri, (size_t)n * sizeof(int32_t), cudaMemcpyDeviceToHost, s->stream);
      if (dist) cudaMemcpyAsync(dist, d_dist, (size_t)n * sizeof(float), cudaMemcpyDeviceToHost, s->stream);
      if (uv) cudaMemcpyAsync(uv, d_uv, (size_t)n * 2 * sizeof(float), cudaMemcpyDeviceToHost, s->stream);
    }
    ce = cudaStreamSynchronize(s->stream);
    cleanup();
    if (ce != cudaSuccess) return cuda_fail(ce, "er_trace_closest");
    er_status st = check_device_error(s);
    if (st != ER_OK) return st;
    if (stats) {
      float ms = 0;
      cudaEventElapsedTime(&ms, s->ev0, s->ev1);
      stats->ms = ms;
      stats->node_visits = stats->box_tests = stats->tri_tests = 0;
      if (want_stats) {
        unsigned long long s1[16];
        cudaMemcpy(s1, s->d_stats, sizeof s1, cudaMemcpyDeviceToHost);
        stats->node_visits = (int64_t)(s1[8] - s0[8]);
        stats->box_tests = (int64_t)(s1[9] - s0[9]);
        stats->tri_tests = (int64_t)(s1[10] - s0[10]);
      }
    }
    return ER_OK;
  });
}
