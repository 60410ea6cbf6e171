// er_device_bandwidth: the L2 and HBM bandwidth ceilings of the running GPU,
// measured by streaming kernels of this library (a measurement aid for the
// traversal and shading rooflines; no counterpart in the reference).
//
// L2 read: a buffer small enough to stay resident in L2 is read `reps`
// times by a grid that fills every SM, 16 bytes per load, loads cached in L2
// only (ld.global.cg), so no load is served by L1 after the first pass; the
// loaded words are folded into one value per thread that is stored, so no
// load can be dropped.  HBM copy: a buffer far larger than L2 copied to
// another, counted as read + written bytes (as a STREAM copy is).
#include <vector>

#include "internal.h"

namespace er {
namespace {

__global__ void k_l2_read(const uint4* __restrict__ buf, int64_t n16, int32_t passes, uint32_t* sink) {
  uint32_t acc = 0;
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  for (int32_t p = 0; p < passes; p++)
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n16; i += stride) {
      uint4 v = __ldcg(buf + i);
      acc ^= v.x ^ v.y ^ v.z ^ v.w;
    }
  sink[blockIdx.x * blockDim.x + threadIdx.x] = acc;
}

__global__ void k_copy(const uint4* __restrict__ a, uint4* __restrict__ b, int64_t n16) {
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n16; i += stride) b[i] = __ldcs(a + i);
}

__global__ void k_fill(uint4* b, int64_t n16) {
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n16; i += stride)
    b[i] = make_uint4((uint32_t)i, (uint32_t)(i >> 32), 0x9e3779b9u, 7u);
}

}  // namespace
}  // namespace er

using namespace er;

extern "C" er_status er_device_bandwidth(int32_t device, int32_t kind, int64_t bytes, int32_t reps, double* gbps) {
  return guarded("er_device_bandwidth", [&]() -> er_status {
    if (!gbps || reps < 1 || reps > 100000 || bytes < (1 << 20) || (kind != ER_BW_L2_READ && kind != ER_BW_HBM_COPY))
      return fail(ER_ERR_INVALID_ARG, "er_device_bandwidth: bad argument");
    if (kind == ER_BW_L2_READ && bytes > ((int64_t)64 << 20))
      return fail(ER_ERR_INVALID_ARG, "er_device_bandwidth: an L2 read buffer holds at most 64 MiB");
    if (bytes > ((int64_t)32 << 30)) return fail(ER_ERR_INVALID_ARG, "er_device_bandwidth: at most 32 GiB");
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) {
      cudaGetLastError();
      return fail(ER_ERR_NO_DEVICE, "no CUDA device visible");
    }
    if (device < 0 || device >= ndev) return fail(ER_ERR_INVALID_ARG, "device ordinal out of range");
    ER_CUDA(cudaSetDevice(device));
    cudaDeviceProp prop;
    ER_CUDA(cudaGetDeviceProperties(&prop, device));
    const int64_t n16 = bytes / 16;
    const int block = 256;
    const int grid = prop.multiProcessorCount * (prop.maxThreadsPerMultiProcessor / block);
    cudaStream_t st = nullptr;
    ER_CUDA(cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking));
    uint4 *a = nullptr, *b = nullptr;
    uint32_t* sink = nullptr;
    cudaEvent_t e0 = nullptr, e1 = nullptr;
    auto cleanup = [&]() {
      cudaFree(a);
      cudaFree(b);
      cudaFree(sink);
      if (e0) cudaEventDestroy(e0);
      if (e1) cudaEventDestroy(e1);
      cudaStreamDestroy(st);
    };
    cudaError_t e = cudaMalloc(&a, (size_t)n16 * 16);
    if (e == cudaSuccess && kind == ER_BW_HBM_COPY) e = cudaMalloc(&b, (size_t)n16 * 16);
    if (e == cudaSuccess) e = cudaMalloc(&sink, (size_t)grid * block * 4);
    if (e != cudaSuccess) {
      cudaGetLastError();
      cleanup();
      return fail(ER_ERR_OOM, "er_device_bandwidth: buffers");
    }
    cudaEventCreate(&e0);
    cudaEventCreate(&e1);
    k_fill<<<grid, block, 0, st>>>(a, n16);
    float ms = 0;
    if (kind == ER_BW_L2_READ) {
      k_l2_read<<<grid, block, 0, st>>>(a, n16, 2, sink);  // brings the buffer into L2
      cudaEventRecord(e0, st);
      k_l2_read<<<grid, block, 0, st>>>(a, n16, reps, sink);
      cudaEventRecord(e1, st);
    } else {
      k_copy<<<grid, block, 0, st>>>(a, b, n16);
      cudaEventRecord(e0, st);
      for (int32_t r = 0; r < reps; r++) k_copy<<<grid, block, 0, st>>>(a, b, n16);
      cudaEventRecord(e1, st);
    }
    e = cudaEventSynchronize(e1);
    if (e == cudaSuccess) e = cudaGetLastError();
    if (e == cudaSuccess) e = cudaEventElapsedTime(&ms, e0, e1);
    cleanup();
    if (e != cudaSuccess) return cuda_fail(e, "er_device_bandwidth");
    const double moved = (double)n16 * 16 * reps * (kind == ER_BW_HBM_COPY ? 2.0 : 1.0);
    *gbps = moved / (ms * 1e-3) / 1e9;
    return ER_OK;
  });
}
