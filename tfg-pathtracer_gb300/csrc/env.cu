// Alias table of the environment's EFFECTIVE texel distribution.
//
// The reference picks an environment texel with HDRI::binarySearch(cdf, r,
// w*h) (HDRI.hpp:130-162), which is not an exact inverse of the CDF: the
// texel it returns for a uniform r is what defines the sampling
// distribution, while the estimator still divides by HDRI::pdf.  The random
// numbers here take the 2^24 values k * 2^-24, k = 1..2^24, so the effective
// distribution is exactly count(texel) / 2^24 with count = number of k the
// search maps to the texel.  The counts are taken on the GPU (one search per
// k), turned into FP64 alias weights on the GPU, and paired by Vose's
// method (M. D. Vose, "A linear algorithm for generating random numbers
// with a given distribution", IEEE TSE 1991) on the host in FP64.  With a
// power-of-two texel count every weight and every update is a dyadic
// rational, so the table reproduces the counts exactly.  Sampling is O(1):
// column = mulhi(x, n) of one 32-bit random word, coin = a second word
// compared with a 32-bit threshold.
#include <cmath>
#include <vector>

#include "internal.h"
#include "shade.cuh"

namespace er {
namespace {

constexpr int64_t kGrid = (int64_t)1 << 24;

// The search's texel for each of its 2^24 inputs: a table lookup then
// returns exactly what the search returns, with one load instead of
// ~log2(w*h) dependent ones.
__global__ void k_env_lut(const float* __restrict__ cdf, int32_t n, int32_t* lut) {
  int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= kGrid) return;
  float r = (float)(k + 1) * (1.0f / 16777216.0f);  // u01 of (k << 8)
  lut[k] = hdri_search(cdf, r, n);
}

__global__ void k_env_counts(const float* __restrict__ cdf, int32_t n, uint32_t* counts) {
  int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= kGrid) return;
  float r = (float)(k + 1) * (1.0f / 16777216.0f);  // u01 of (k << 8)
  int32_t t = hdri_search(cdf, r, n);
  if (t >= 0 && t < n) atomicAdd(&counts[t], 1u);
}

// weight_i = count_i * n / 2^24 in FP64 (exact for n a power of two)
__global__ void k_env_weights(const uint32_t* counts, int32_t n, double* q) {
  int32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  q[i] = (double)counts[i] * (double)n / (double)kGrid;
}

}  // namespace

void invalidate_env_tables(er_scene* s) {
  s->env_alias_ok = false;
  s->env_lut_ok = false;
  s->dev.alias_idx = nullptr;
  s->dev.alias_thresh = nullptr;
  s->dev.env_lut = nullptr;
}

er_status build_env_lut(er_scene* s) {
  const int32_t n = s->dev.env.w * s->dev.env.h;
  if (s->env_lut_ok || n < kEnvLutMinTexels) return ER_OK;
  er_status st;
  if (!s->env_lut_buf && (st = dev_alloc(s, &s->env_lut_buf, (size_t)kGrid * 4)) != ER_OK) return st;
  k_env_lut<<<(unsigned)(kGrid / 256), 256, 0, s->stream>>>(s->dev.cdf, n, (int32_t*)s->env_lut_buf);
  ER_CUDA(cudaGetLastError());
  s->dev.env_lut = (const int32_t*)s->env_lut_buf;
  s->env_lut_ok = true;
  return ER_OK;
}

er_status build_env_alias(er_scene* s) {
  if (s->env_alias_ok) return ER_OK;
  const int32_t n = s->dev.env.w * s->dev.env.h;
  er_status st;
  if (!s->env_counts) {
    void* p = nullptr;
    if ((st = dev_alloc(s, &p, (size_t)n * 4)) != ER_OK) return st;
    s->env_counts = (const uint32_t*)p;
  }
  if (!s->env_q && (st = dev_alloc(s, &s->env_q, (size_t)n * 8)) != ER_OK) return st;
  void* d_counts = const_cast<uint32_t*>(s->env_counts);
  void* d_q = s->env_q;
  ER_CUDA(cudaMemsetAsync(d_counts, 0, (size_t)n * 4, s->stream));
  k_env_counts<<<(unsigned)(kGrid / 256), 256, 0, s->stream>>>(s->dev.cdf, n, (uint32_t*)d_counts);
  k_env_weights<<<(n + 255) / 256, 256, 0, s->stream>>>((const uint32_t*)d_counts, n, (double*)d_q);
  ER_CUDA(cudaGetLastError());
  std::vector<double> q((size_t)n);
  ER_CUDA(cudaMemcpyAsync(q.data(), d_q, (size_t)n * 8, cudaMemcpyDeviceToHost, s->stream));
  ER_CUDA(cudaStreamSynchronize(s->stream));

  // Vose: pair every light column with a heavy one, FP64 throughout.
  std::vector<int32_t> small, large, alias((size_t)n);
  std::vector<double> prob((size_t)n, 1.0);
  for (int32_t i = n - 1; i >= 0; i--) {
    alias[(size_t)i] = i;
    (q[(size_t)i] < 1.0 ? small : large).push_back(i);
  }
  while (!small.empty() && !large.empty()) {
    int32_t l = small.back();
    small.pop_back();
    int32_t g = large.back();
    prob[(size_t)l] = q[(size_t)l];
    alias[(size_t)l] = g;
    q[(size_t)g] = (q[(size_t)g] + q[(size_t)l]) - 1.0;
    if (q[(size_t)g] < 1.0) {
      large.pop_back();
      small.push_back(g);
    }
  }
  // leftovers (rounding for non-power-of-two n) keep probability 1
  std::vector<uint32_t> thresh((size_t)n);
  for (int32_t i = 0; i < n; i++) {
    double p = prob[(size_t)i];
    // accept the column itself when the 32-bit coin is below p * 2^32
    thresh[(size_t)i] = p >= 1.0 ? 0xFFFFFFFFu : (uint32_t)std::floor(p * 4294967296.0);
  }
  if (!s->env_alias_buf && (st = dev_alloc(s, &s->env_alias_buf, (size_t)n * 4)) != ER_OK) return st;
  if (!s->env_thresh_buf && (st = dev_alloc(s, &s->env_thresh_buf, (size_t)n * 4)) != ER_OK) return st;
  ER_CUDA(cudaMemcpyAsync(s->env_alias_buf, alias.data(), (size_t)n * 4, cudaMemcpyHostToDevice, s->stream));
  ER_CUDA(cudaMemcpyAsync(s->env_thresh_buf, thresh.data(), (size_t)n * 4, cudaMemcpyHostToDevice, s->stream));
  ER_CUDA(cudaStreamSynchronize(s->stream));
  s->dev.alias_idx = (const int32_t*)s->env_alias_buf;
  s->dev.alias_thresh = (const uint32_t*)s->env_thresh_buf;
  s->env_alias_ok = true;
  return ER_OK;
}

}  // namespace er

using namespace er;

extern "C" er_status er_env_search_table(er_scene* s, int32_t* table) {
  return guarded("er_env_search_table", [&]() -> er_status {
    if (!s || !table) return fail(ER_ERR_INVALID_ARG, "NULL argument");
    ER_CUDA(cudaSetDevice(s->device));
    if ((int64_t)s->dev.env.w * s->dev.env.h < kEnvLutMinTexels)
      return fail(ER_ERR_INVALID_ARG, "environment below the table threshold: sampled by the search");
    er_status st = build_env_lut(s);
    if (st != ER_OK) return st;
    ER_CUDA(cudaMemcpyAsync(table, s->env_lut_buf, (size_t)kGrid * 4, cudaMemcpyDeviceToHost, s->stream));
    ER_CUDA(cudaStreamSynchronize(s->stream));
    return ER_OK;
  });
}

extern "C" er_status er_env_distribution(er_scene* s, uint32_t* counts, int32_t* alias, uint32_t* thresh) {
  return guarded("er_env_distribution", [&]() -> er_status {
    if (!s) return fail(ER_ERR_INVALID_ARG, "scene is NULL");
    ER_CUDA(cudaSetDevice(s->device));
    er_status st = build_env_alias(s);
    if (st != ER_OK) return st;
    const size_t n = (size_t)s->dev.env.w * s->dev.env.h;
    if (counts) ER_CUDA(cudaMemcpyAsync(counts, s->env_counts, n * 4, cudaMemcpyDeviceToHost, s->stream));
    if (alias) ER_CUDA(cudaMemcpyAsync(alias, s->dev.alias_idx, n * 4, cudaMemcpyDeviceToHost, s->stream));
    if (thresh) ER_CUDA(cudaMemcpyAsync(thresh, s->dev.alias_thresh, n * 4, cudaMemcpyDeviceToHost, s->stream));
    ER_CUDA(cudaStreamSynchronize(s->stream));
    return ER_OK;
  });
}
