// xr_noalloc.cu -- grad-NCC of a batch of moving images against one fixed image
// with no device allocation at all, for callers that cannot allocate.
//
// Some hosts cannot call cudaMalloc on the path that evaluates the metric: a
// registration step running inside a CUDA-graph-driven or real-time loop where
// allocation would synchronise the device or fragment a pool the host manages,
// an embedding application whose memory is owned by another allocator, or a
// plugin that is only handed device pointers.  This entry point takes the fixed
// image, the moving images and the output as device pointers and keeps every
// intermediate (fixed-image gradients, their zero-mean copies, statistics and
// per-block moment partials) in one file-scope __device__ array of fixed size
// (kScratchBytes below).  Every GPU that loads the library holds that array until
// the process exits.
//
// Rules for callers:
//   * sizes beyond the array are rejected with XR_ERR_INVALID_ARG and a message
//     giving the bytes needed;
//   * the first call on a device looks up the array's device address with
//     cudaGetSymbolAddress (once per device, with that device current); make
//     that first call before any stream capture.  The address is kept for the
//     life of the process: after cudaDeviceReset (or anything else that tears
//     down and recreates the device's primary context) the array is a new one
//     and this library must not be called on that device again;
//   * at most 65535 moving images per call;
//   * all calls share the one array: two calls whose work overlaps on the GPU
//     (different streams, or different host threads) race and give wrong values.
//     Calls serialised on one stream are fine.  Each call overwrites everything
//     it reads later, and the statistics words are cleared at the start of
//     every call.
#include "xr_gradtile.cuh"
#include "xr_internal.h"

#include <mutex>

namespace xr {
namespace {

constexpr size_t kScratchBytes = size_t(16) << 20;  // 16 MiB

static __device__ __align__(256) unsigned char g_scratch[kScratchBytes];

constexpr int kMaxDevices = 64;
std::mutex g_addr_mu;
void* g_addr[kMaxDevices] = {};

// Device address of g_scratch for the current device (looked up once per device).
cudaError_t scratch_address(int dev, unsigned char** out) {
  if (dev < 0 || dev >= kMaxDevices) return cudaErrorInvalidDevice;
  std::lock_guard<std::mutex> lk(g_addr_mu);
  if (!g_addr[dev]) {
    void* p = nullptr;
    cudaError_t e = cudaGetSymbolAddress(&p, g_scratch);
    if (e != cudaSuccess) return e;
    g_addr[dev] = p;
  }
  *out = static_cast<unsigned char*>(g_addr[dev]);
  return cudaSuccess;
}

// stats layout (doubles): [0..2] gx sum / sum of squared deviations / count,
// [3..5] gy likewise, [6] sum of zero-mean gx, [8] sum of zero-mean gy
// (launch_sum_f writes slots k and k+2).
__global__ void zero_mean_from_stats_kernel(const float* __restrict__ g, int64_t n, const double* __restrict__ st,
                                            float* __restrict__ out) {
  const float mean = (float)(st[0] / st[2]);
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
    out[i] = g[i] - mean;
}

// One block per image, as the allocating path's grad_finalize_kernel (the same
// reduction and similarity), the fixed side's standard deviations (clamped at
// 1e-6) and zero-mean sums read from the statistics words.
__global__ void finalize_from_stats_kernel(const double* __restrict__ partials, int nblk,
                                           const double* __restrict__ st, float* __restrict__ sims) {
  __shared__ double red[6 * (gt::kFinalizeThreads / 32)];
  const double n = st[2];
  FixedNCC fx{nullptr, sqrt(st[1] / (n - 1.0)), st[6]}, fy{nullptr, sqrt(st[4] / (n - 1.0)), st[8]};
  if (fx.sd < 1.0e-6) fx.sd = 1.0e-6;
  if (fy.sd < 1.0e-6) fy.sd = 1.0e-6;
  const float sim = gt::grad_finalize_image<false>(partials + (int64_t)blockIdx.x * nblk * 6, nblk, n, fx, fy, red);
  if (threadIdx.x == 0) sims[blockIdx.x] = sim;
}

size_t align256(size_t b) { return (b + 255) & ~size_t(255); }

}  // namespace
}  // namespace xr

using namespace xr;

extern "C" XR_API xr_status xr_grad_ncc_noalloc(const float* d_fixed, const float* d_moving, int64_t rows,
                                                int64_t cols, int64_t num_moving, int32_t smooth_ksize,
                                                float* d_sims, void* cuda_stream) {
  if (!d_fixed || !d_moving || !d_sims) return fail(XR_ERR_INVALID_ARG, "xr_grad_ncc_noalloc: NULL pointer");
  if (rows < 8 || cols < 8) return fail(XR_ERR_INVALID_ARG, "xr_grad_ncc_noalloc: images must be at least 8x8");
  if (num_moving < 1) return fail(XR_ERR_INVALID_ARG, "xr_grad_ncc_noalloc: num_moving must be >= 1");
  if (smooth_ksize != 0 && smooth_ksize != 3 && smooth_ksize != 5)
    return fail(XR_ERR_UNSUPPORTED, "xr_grad_ncc_noalloc: smoothing kernel must be 0, 3 or 5");
  if (rows > (1 << 20) || cols > (1 << 20))
    return fail(XR_ERR_INVALID_ARG, "xr_grad_ncc_noalloc: size out of range");
  if (num_moving > 65535)  // one grid row of the moments launch per moving image
    return fail(XR_ERR_INVALID_ARG, "xr_grad_ncc_noalloc: at most 65535 moving images per call (got " +
                                        std::to_string(num_moving) + ")");
  cudaStream_t s = static_cast<cudaStream_t>(cuda_stream);
  int nblk = 0;
  XR_CUDA_TRY(launch_grad_moments(nullptr, (int)rows, (int)cols, 0, smooth_ksize, nullptr, nullptr, nullptr, nullptr,
                                  s, &nblk));
  const int64_t npix = rows * cols;
  const size_t img_b = align256((size_t)npix * 4);
  const size_t stats_b = 256;
  const size_t part_b = align256((size_t)num_moving * (size_t)nblk * 6 * 8);
  const size_t need = stats_b + 4 * img_b + part_b;
  if (need > kScratchBytes)
    return fail(XR_ERR_INVALID_ARG, "xr_grad_ncc_noalloc: needs " + std::to_string(need) +
                                        " bytes of scratch, more than the fixed " + std::to_string(kScratchBytes) +
                                        " (fewer moving images per call, or smaller images)");
  int dev = 0;
  XR_CUDA_TRY(cudaGetDevice(&dev));
  unsigned char* base = nullptr;
  XR_CUDA_TRY(scratch_address(dev, &base));
  double* stats = reinterpret_cast<double*>(base);
  float* gx = reinterpret_cast<float*>(base + stats_b);
  float* gy = reinterpret_cast<float*>(base + stats_b + img_b);
  float* fhx = reinterpret_cast<float*>(base + stats_b + 2 * img_b);
  float* fhy = reinterpret_cast<float*>(base + stats_b + 3 * img_b);
  double* partials = reinterpret_cast<double*>(base + stats_b + 4 * img_b);

  XR_CUDA_TRY(cudaMemsetAsync(stats, 0, stats_b, s));
  // fixed image: blur + Sobel, statistics and zero-mean copies, all on the device
  XR_CUDA_TRY(launch_grad_images(d_fixed, (int)rows, (int)cols, 1, smooth_ksize, gx, gy, s));
  XR_CUDA_TRY(launch_image_stats(gx, npix, nullptr, stats + 0, s));
  XR_CUDA_TRY(launch_image_stats(gy, npix, nullptr, stats + 3, s));
  const int zb = (int)((npix + 255) / 256 < 4096 ? (npix + 255) / 256 : 4096);
  zero_mean_from_stats_kernel<<<zb, 256, 0, s>>>(gx, npix, stats + 0, fhx);
  zero_mean_from_stats_kernel<<<zb, 256, 0, s>>>(gy, npix, stats + 3, fhy);
  XR_CUDA_TRY(cudaGetLastError());
  XR_CUDA_TRY(launch_sum_f(fhx, npix, nullptr, stats + 6, s));
  XR_CUDA_TRY(launch_sum_f(fhy, npix, nullptr, stats + 8, s));
  // moving images: fused blur + Sobel + moments, then the double combine
  XR_CUDA_TRY(launch_grad_moments(d_moving, (int)rows, (int)cols, num_moving, smooth_ksize, fhx, fhy, nullptr,
                                  partials, s, nullptr));
  finalize_from_stats_kernel<<<(unsigned)num_moving, gt::kFinalizeThreads, 0, s>>>(partials, nblk, stats, d_sims);
  XR_CUDA_TRY(cudaGetLastError());
  return XR_OK;
}
