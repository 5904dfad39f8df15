// xr_probe.cu -- measured L2 read bandwidth of the current device, the
// denominator of the DRR kernel's gather roofline (its voxel cells are read
// from L1/L2, not from HBM).  No counterpart in xReg.
//
// A buffer well inside the L2 (129 MB on GB300) is read once to make it
// resident, then read `reps` more times by a grid of one block per SM times the
// resident blocks, each thread keeping eight independent 16-byte L2 loads
// (ld.global.cg: cached in L2, not in L1) in flight.  The time of those reads
// (CUDA events on an internal stream) gives bytes / second.
#include "xr_internal.h"

namespace xr {
namespace {

constexpr int kProbeThreads = 512;
constexpr int kProbeUnroll = 8;

__device__ __forceinline__ float4 ld_cg(const float4* p) {
  float4 v;
  asm volatile("ld.global.cg.v4.f32 {%0,%1,%2,%3}, [%4];" : "=f"(v.x), "=f"(v.y), "=f"(v.z), "=f"(v.w) : "l"(p));
  return v;
}

// Reads n16 16-byte words reps times; the sum is stored only when it equals a
// value it can never take (keeps the loads live without a write per thread).
__global__ void __launch_bounds__(kProbeThreads) l2_read_kernel(const float4* __restrict__ buf, int64_t n16,
                                                               int reps, float* sink) {
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  float acc = 0.0f;
  for (int r = 0; r < reps; ++r) {
    int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    for (; i + (kProbeUnroll - 1) * stride < n16; i += kProbeUnroll * stride) {
      float4 v[kProbeUnroll];
#pragma unroll
      for (int k = 0; k < kProbeUnroll; ++k) v[k] = ld_cg(buf + i + k * stride);
#pragma unroll
      for (int k = 0; k < kProbeUnroll; ++k) acc += (v[k].x + v[k].y) + (v[k].z + v[k].w);
    }
    for (; i < n16; i += stride) {
      const float4 v = ld_cg(buf + i);
      acc += (v.x + v.y) + (v.z + v.w);
    }
  }
  if (acc == -1.0f) sink[0] = acc;  // the buffer holds zeros: never true
}

}  // namespace
}  // namespace xr

using namespace xr;

extern "C" XR_API xr_status xr_measure_l2_read_bandwidth(int32_t device, int64_t bytes, int32_t reps,
                                                         double* gbs) {
  if (!gbs || bytes < (1 << 20) || reps < 1) return fail(XR_ERR_INVALID_ARG, "measure_l2: bad argument");
  int dev = device;
  if (dev < 0 && cudaGetDevice(&dev) != cudaSuccess) return fail(XR_ERR_CUDA, "measure_l2: no current device");
  int prev = 0;
  XR_CUDA_TRY(cudaGetDevice(&prev));
  XR_CUDA_TRY(cudaSetDevice(dev));
  int l2 = 0, sms = 0, per_sm = 0;
  cudaError_t e = cudaDeviceGetAttribute(&l2, cudaDevAttrL2CacheSize, dev);
  if (e == cudaSuccess) e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  if (e == cudaSuccess) e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, l2_read_kernel, kProbeThreads, 0);
  if (e != cudaSuccess) { cudaSetDevice(prev); return cuda_fail(e, "measure_l2: device attributes"); }
  if (bytes > (int64_t)l2 / 2) {
    cudaSetDevice(prev);
    return fail(XR_ERR_INVALID_ARG, "measure_l2: the buffer must fit in half of the L2 (" + std::to_string(l2) +
                                        " bytes)");
  }
  const int64_t n16 = bytes / 16;
  void* buf = nullptr;
  float* sink = nullptr;
  cudaStream_t s = nullptr;
  cudaEvent_t t0 = nullptr, t1 = nullptr;
  float ms = 0.0f;
  e = cudaMalloc(&buf, (size_t)n16 * 16);
  if (e == cudaSuccess) e = cudaMalloc(&sink, sizeof(float));
  if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking);
  if (e == cudaSuccess) e = cudaEventCreate(&t0);
  if (e == cudaSuccess) e = cudaEventCreate(&t1);
  if (e == cudaSuccess) e = cudaMemsetAsync(buf, 0, (size_t)n16 * 16, s);
  const int blocks = sms * (per_sm > 0 ? per_sm : 1);
  if (e == cudaSuccess) {
    l2_read_kernel<<<blocks, kProbeThreads, 0, s>>>(static_cast<const float4*>(buf), n16, 2, sink);  // resident
    e = cudaEventRecord(t0, s);
  }
  if (e == cudaSuccess) {
    l2_read_kernel<<<blocks, kProbeThreads, 0, s>>>(static_cast<const float4*>(buf), n16, reps, sink);
    e = cudaGetLastError();
  }
  if (e == cudaSuccess) e = cudaEventRecord(t1, s);
  if (e == cudaSuccess) e = cudaEventSynchronize(t1);
  if (e == cudaSuccess) e = cudaEventElapsedTime(&ms, t0, t1);
  if (t0) cudaEventDestroy(t0);
  if (t1) cudaEventDestroy(t1);
  if (s) cudaStreamDestroy(s);
  if (buf) cudaFree(buf);
  if (sink) cudaFree(sink);
  cudaSetDevice(prev);
  if (e != cudaSuccess) return cuda_fail(e, "measure_l2");
  *gbs = (double)n16 * 16.0 * reps / (ms * 1.0e-3) / 1.0e9;
  return XR_OK;
}
