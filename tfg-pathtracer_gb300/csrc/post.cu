// Post-processing of a film on the GPU: the operations of the reference's
// PostProcessing.cpp (applyExposure :3-6, basicBlur bloom :132-211,
// reinhardTonemap :35-39, acesTonemap :41-52, clampPixels :30-33, applysRGB
// :54-57, flipX :19-28 / flipY :8-17) and its LDR output step (main.cpp:150-158:
// clamp, fastPow(v, 1/2.2) * 255), one thread per pixel, in that order.
// The arithmetic follows the reference's types: double where its
// expressions hold a double literal (ACES, sRGB, the bloom threshold sum),
// float elsewhere.
//
// Defined where the reference reads uninitialised memory: basicBlur leaves
// the alpha of below-threshold pixels and the blur of the border pixels
// (within radius/2 of an edge) unset; here they are 0.
#include <cmath>
#include <vector>

#include "internal.h"

namespace er {
namespace {

struct PostParams {
  int32_t w, h;
  float exposure;
  int32_t tonemap, clamp01, srgb, flip_x, flip_y;
  float threshold, power;
  int32_t blur;  // basicBlur's blurSize; 0 = no bloom
};

__device__ __forceinline__ float clampr(float a, float b, float c) { return a < b ? b : a > c ? c : a; }

// Ankerl's fastPow as the reference's output step uses it (high word only).
__device__ __forceinline__ double fast_pow_d(double a, double b) {
  long long bits = __double_as_longlong(a);
  int32_t hi = (int32_t)(bits >> 32);
  hi = (int32_t)(b * (double)(hi - 1072632447) + 1072632447);
  return __longlong_as_double((long long)((unsigned long long)(uint32_t)hi << 32));
}

// exposure, and the bloom threshold image (basicBlur's thresholdMatrix)
__global__ void k_post_pre(const float4* in, float4* img, float4* thr, PostParams P) {
  int32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= P.w * P.h) return;
  float4 v = in[i];
  v.x *= P.exposure; v.y *= P.exposure; v.z *= P.exposure; v.w *= P.exposure;
  img[i] = v;
  if (P.blur > 0) {
    float s = 0.f;
    s = (float)((double)s + (double)v.x / 3.0);
    s = (float)((double)s + (double)v.y / 3.0);
    s = (float)((double)s + (double)v.z / 3.0);
    thr[i] = s < P.threshold ? make_float4(0.f, 0.f, 0.f, 0.f) : v;
  }
}

// img += blur(thr) * power over the interior pixels
__global__ void k_post_bloom(float4* img, const float4* thr, const float* kern, PostParams P) {
  int32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= P.w * P.h) return;
  const int32_t x = i % P.w, y = i / P.w, b = P.blur, ks = 2 * b + 1;
  if (x < b || x >= P.w - b || y < b || y >= P.h - b) return;
  float4 s = make_float4(0.f, 0.f, 0.f, 0.f);
  for (int32_t ii = 0; ii < ks; ii++) {
    for (int32_t jj = 0; jj < ks; jj++) {
      const float4 t = thr[(x - b + ii) + (y - b + jj) * P.w];
      const float k = __ldg(kern + ii + jj * ks);
      s.x = __fadd_rn(s.x, __fmul_rn(t.x, k));
      s.y = __fadd_rn(s.y, __fmul_rn(t.y, k));
      s.z = __fadd_rn(s.z, __fmul_rn(t.z, k));
      s.w = __fadd_rn(s.w, __fmul_rn(t.w, k));
    }
  }
  float4 v = img[i];
  v.x = __fadd_rn(v.x, __fmul_rn(s.x, P.power));
  v.y = __fadd_rn(v.y, __fmul_rn(s.y, P.power));
  v.z = __fadd_rn(v.z, __fmul_rn(s.z, P.power));
  v.w = __fadd_rn(v.w, __fmul_rn(s.w, P.power));
  img[i] = v;
}

__device__ __forceinline__ float post_channel(float x, const PostParams& P) {
  if (P.tonemap == ER_TONEMAP_REINHARD) {
    x = __fdiv_rn(x, __fadd_rn(1.0f, x));
  } else if (P.tonemap == ER_TONEMAP_ACES) {
    const float a = 2.51f, b = 0.03f, c = 2.43f, d = 0.59f, e = 0.14f;
    const double xd = (double)x;
    const double num = xd * 0.6 * ((double)__fmul_rn(a, x) * 0.6 + (double)b);
    const double den = xd * 0.6 * ((double)__fmul_rn(c, x) * 0.6 + (double)d) + (double)e;
    x = clampr((float)(num / den), 0.0f, 1.0f);
  }
  if (P.clamp01) x = clampr(x, 0.0f, 1.0f);
  if (P.srgb) x = (float)pow((double)x, 1.0 / 2.2);
  return x;
}

__device__ __forceinline__ uint8_t ldr_channel(float v) {
  v = clampr(v, 0.0f, 1.0f);
  double e = fast_pow_d((double)v, 1.0 / 2.2) * 255.0;
  if (!(e >= 0.0 && e < 256.0)) e = 0.0;  // NaN: 0
  return (uint8_t)(int32_t)e;
}

// tone map, clamp, sRGB, flips; float and / or LDR output
__global__ void k_post_finish(const float4* img, float4* out, uchar4* ldr, PostParams P) {
  int32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= P.w * P.h) return;
  int32_t x = i % P.w, y = i / P.w;
  const int32_t sx = P.flip_x ? P.w - 1 - x : x, sy = P.flip_y ? P.h - 1 - y : y;
  float4 v = img[sx + sy * P.w];
  v = make_float4(post_channel(v.x, P), post_channel(v.y, P), post_channel(v.z, P), post_channel(v.w, P));
  if (out) out[i] = v;
  if (ldr) ldr[i] = make_uchar4(ldr_channel(v.x), ldr_channel(v.y), ldr_channel(v.z), ldr_channel(v.w));
}

}  // namespace
}  // namespace er

using namespace er;

extern "C" er_status er_postprocess(const float* rgba_in, int32_t width, int32_t height, const er_post_opts* opts,
                                    float* rgba_out, uint8_t* ldr_out, uint32_t flags) {
  return guarded("er_postprocess", [&]() -> er_status {
    if (!rgba_in || width <= 0 || height <= 0 || (!rgba_out && !ldr_out))
      return fail(ER_ERR_INVALID_ARG, "bad post-processing arguments");
    if ((int64_t)width * height > ((int64_t)1 << 28)) return fail(ER_ERR_INVALID_ARG, "image too large");
    er_post_opts o{};
    o.exposure = 1.0f;
    if (opts) o = *opts;
    if (o.tonemap < ER_TONEMAP_NONE || o.tonemap > ER_TONEMAP_ACES) return fail(ER_ERR_INVALID_ARG, "tonemap");
    if (o.bloom_power != 0.0f && !(o.bloom_radius >= 0.0f && o.bloom_radius <= 256.0f))
      return fail(ER_ERR_INVALID_ARG, "bloom radius out of range");
    int dev = 0;
    ER_CUDA(cudaGetDevice(&dev));
    const bool devp = flags & ER_RENDER_DEVICE_OUT;
    const size_t n = (size_t)width * height;
    PostParams P;
    P.w = width;
    P.h = height;
    P.exposure = o.exposure;
    P.tonemap = o.tonemap;
    P.clamp01 = o.clamp != 0;
    P.srgb = o.srgb != 0;
    P.flip_x = o.flip_x != 0;
    P.flip_y = o.flip_y != 0;
    P.threshold = o.bloom_threshold;
    P.power = o.bloom_power;
    P.blur = o.bloom_power != 0.0f ? (int32_t)(o.bloom_radius / 2) : 0;
    // basicBlur's kernel (PostProcessing.cpp:143-153), built on the host
    const int32_t ks = 2 * P.blur + 1;
    std::vector<float> kern(P.blur > 0 ? (size_t)ks * ks : 1, 0.0f);
    if (P.blur > 0) {
      const float sd = o.bloom_radius;
      const float kernelSize = (float)ks;
      for (int32_t x = 0; x < ks; x++)
        for (int32_t y = 0; y < ks; y++) {
          float t1 = (float)(1.0 / ((2.0 * (double)3.14159265358979323846f) * (double)(sd * sd)));
          float tx = (float)(x - (int32_t)(kernelSize / 2.0));
          float ty = (float)(y - (int32_t)(kernelSize / 2.0));
          float t2 = (float)(-(double)(tx * tx + ty * ty) / (2.0 * (double)sd * (double)sd));
          kern[(size_t)(x + y * ks)] = t1 * std::exp(t2);
        }
    }
    struct Buf {
      std::vector<void*> p;
      ~Buf() {
        for (void* q : p) cudaFree(q);
      }
      er_status get(void** out, size_t bytes) {
        cudaError_t e = cudaMalloc(out, std::max<size_t>(bytes, 16));
        if (e != cudaSuccess) {
          cudaGetLastError();
          return fail(ER_ERR_OOM, "post-processing buffers");
        }
        p.push_back(*out);
        return ER_OK;
      }
    } B;
    er_status st;
    const float4* d_in = (const float4*)rgba_in;
    float4 *img, *thr = nullptr, *d_out = nullptr;
    uchar4* d_ldr = nullptr;
    float* d_kern = nullptr;
    if (!devp) {
      void* p;
      if ((st = B.get(&p, n * 16)) != ER_OK) return st;
      ER_CUDA(cudaMemcpy(p, rgba_in, n * 16, cudaMemcpyHostToDevice));
      d_in = (const float4*)p;
    }
    if ((st = B.get((void**)&img, n * 16)) != ER_OK) return st;
    if (P.blur > 0) {
      if ((st = B.get((void**)&thr, n * 16)) != ER_OK) return st;
      if ((st = B.get((void**)&d_kern, kern.size() * 4)) != ER_OK) return st;
      ER_CUDA(cudaMemcpy(d_kern, kern.data(), kern.size() * 4, cudaMemcpyHostToDevice));
    }
    if (rgba_out) {
      if (devp) d_out = (float4*)rgba_out;
      else if ((st = B.get((void**)&d_out, n * 16)) != ER_OK) return st;
    }
    if (ldr_out) {
      if (devp) d_ldr = (uchar4*)ldr_out;
      else if ((st = B.get((void**)&d_ldr, n * 4)) != ER_OK) return st;
    }
    const unsigned blocks = (unsigned)((n + 255) / 256);
    k_post_pre<<<blocks, 256>>>(d_in, img, thr, P);
    if (P.blur > 0) k_post_bloom<<<blocks, 256>>>(img, thr, d_kern, P);
    k_post_finish<<<blocks, 256>>>(img, d_out, d_ldr, P);
    ER_CUDA(cudaGetLastError());
    if (!devp) {
      if (rgba_out) ER_CUDA(cudaMemcpy(rgba_out, d_out, n * 16, cudaMemcpyDeviceToHost));
      if (ldr_out) ER_CUDA(cudaMemcpy(ldr_out, d_ldr, n * 4, cudaMemcpyDeviceToHost));
    }
    ER_CUDA(cudaDeviceSynchronize());
    (void)dev;
    return ER_OK;
  });
}
