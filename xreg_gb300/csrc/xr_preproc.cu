// xr_preproc.cu -- data preparation either side of the hot path, on the device:
//
// * HU -> linear attenuation (HUToLinAttFilter::GenerateData,
//   lib/image/xregHUToLinAtt.cpp:45-69): mu = max(hu * (mu_w - mu_a) 1e-3 + mu_w - mu_lower, 0)
//   in double, stored as float; mu_w = 0.02683, mu_a = 0.02485e-4 /mm, hu_lower = -1000.
// * Fixed-image downsampling for a coarser registration level (DownsampleProjData
//   -> DownsampleImage, lib/image/xregProjData.cpp:40-53,
//   lib/itk/xregITKResampleUtils.h:51-131): for factor < 1, a discrete Gaussian
//   (ITK DiscreteGaussianImageFilter, variance (0.5/factor)^2 in pixels, maximum
//   error 0.01, kernel width at most 32, edge pixels replicated) along x then y
//   in double; then resampling onto floor(n * factor + 0.5) pixels with the
//   same origin and spacing / factor, i.e. output pixel i reads the smoothed
//   image at continuous index i / factor with bilinear interpolation (a
//   neighbour past the last pixel gets no weight).
//
// The discrete Gaussian kernel is Lindeberg's discrete analogue
// T(k, t) = exp(-t) I_k(t) (t = variance, I_k the modified Bessel function),
// taken out from the centre until its two-sided sum reaches 1 - max_error and
// normalised to sum 1 — the construction ITK's GaussianOperator follows.  Here
// I_k is summed from its power series in double.
#include "xr_internal.h"

#include <cmath>
#include <vector>

namespace xr {
namespace {

__global__ void hu_to_mu_kernel(const float* __restrict__ hu, int64_t n, float* __restrict__ mu) {
  const double mu_w = 0.02683 * 1.0, mu_a = 0.02485 * 0.0001, hu_lower = -1000.0;
  const double hu_scale = (mu_w - mu_a) * 1.0e-3;
  const double mu_lower = (hu_lower * hu_scale) + mu_w;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    const double v = ((double)hu[i] * hu_scale) + mu_w - mu_lower;
    mu[i] = (float)(v > 0.0 ? v : 0.0);
  }
}

constexpr int kMaxTaps = 32;

struct GaussKernel {
  int radius;
  double c[kMaxTaps + 1];
};

// Separable pass along x (dir 0) or y (dir 1), edges replicated.
template <typename TIn>
__global__ void gauss_pass_kernel(const TIn* __restrict__ in, int rows, int cols, int dir, GaussKernel k,
                                  double* __restrict__ out) {
  const int64_t n = (int64_t)rows * cols;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    const int r = (int)(i / cols), c = (int)(i - (int64_t)r * cols);
    double s = k.c[0] * (double)in[i];
    for (int t = 1; t <= k.radius; ++t) {
      int a, b;
      if (dir == 0) {
        a = max(c - t, 0); b = min(c + t, cols - 1);
        s += k.c[t] * ((double)in[(int64_t)r * cols + a] + (double)in[(int64_t)r * cols + b]);
      } else {
        a = max(r - t, 0); b = min(r + t, rows - 1);
        s += k.c[t] * ((double)in[(int64_t)a * cols + c] + (double)in[(int64_t)b * cols + c]);
      }
    }
    out[i] = s;
  }
}

__global__ void resample_kernel(const double* __restrict__ in, int rows, int cols, double factor, int orows,
                                int ocols, float* __restrict__ out) {
  const int64_t n = (int64_t)orows * ocols;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    const int r = (int)(i / ocols), c = (int)(i - (int64_t)r * ocols);
    const double y = r / factor, x = c / factor;
    if (x > cols - 0.5 || y > rows - 0.5) { out[i] = 0.0f; continue; }
    int x0 = (int)floor(x), y0 = (int)floor(y);
    double fx = x - x0, fy = y - y0;
    int x1 = x0 + 1, y1 = y0 + 1;
    if (x1 > cols - 1) { x1 = x0; fx = 0.0; }
    if (y1 > rows - 1) { y1 = y0; fy = 0.0; }
    if (x0 > cols - 1) x0 = x1 = cols - 1;
    if (y0 > rows - 1) y0 = y1 = rows - 1;
    const double v00 = in[(int64_t)y0 * cols + x0], v01 = in[(int64_t)y0 * cols + x1];
    const double v10 = in[(int64_t)y1 * cols + x0], v11 = in[(int64_t)y1 * cols + x1];
    const double a = v00 + (v01 - v00) * fx, b = v10 + (v11 - v10) * fx;
    out[i] = (float)(a + (b - a) * fy);
  }
}

// exp(-t) I_k(t) from the power series of I_k.
double scaled_bessel_i(int k, double t) {
  double term = 1.0;
  for (int j = 1; j <= k; ++j) term *= (0.5 * t) / j;  // (t/2)^k / k!
  double sum = term;
  const double q = 0.25 * t * t;
  for (int m = 1; m < 500; ++m) {
    term *= q / ((double)m * (double)(m + k));
    sum += term;
    if (term < 1e-18 * sum) break;
  }
  return std::exp(-t) * sum;
}

}  // namespace

// Discrete Gaussian taps c[0..radius] (normalised so c0 + 2 sum c_k = 1).
int discrete_gaussian_taps(double variance, double max_error, int max_width, double* out) {
  std::vector<double> c;
  const double cap = 1.0 - max_error;
  c.push_back(scaled_bessel_i(0, variance));
  double sum = c[0];
  for (int k = 1; sum < cap; ++k) {
    c.push_back(scaled_bessel_i(k, variance));
    sum += 2.0 * c.back();
    if ((int)c.size() > max_width || (int)c.size() > kMaxTaps) break;  // one-sided length limit
  }
  for (double& v : c) v /= sum;
  for (size_t i = 0; i < c.size(); ++i) out[i] = c[i];
  return (int)c.size() - 1;
}

}  // namespace xr

using namespace xr;

extern "C" XR_API xr_status xr_hu_to_lin_att(const float* d_hu, int64_t n, float* d_mu, void* stream) {
  if (!d_hu || !d_mu || n < 0) return fail(XR_ERR_INVALID_ARG, "xr_hu_to_lin_att: bad argument");
  if (n == 0) return XR_OK;
  hu_to_mu_kernel<<<(unsigned)std::min<int64_t>((n + 255) / 256, 8192), 256, 0, static_cast<cudaStream_t>(stream)>>>(
      d_hu, n, d_mu);
  XR_CUDA_TRY(cudaGetLastError());
  return XR_OK;
}

extern "C" XR_API xr_status xr_downsample_image_size(int64_t rows, int64_t cols, double factor, int64_t* out_rows,
                                                    int64_t* out_cols) {
  if (!out_rows || !out_cols || rows < 1 || cols < 1 || !(factor > 0.0) || factor > 1.0)
    return fail(XR_ERR_INVALID_ARG, "xr_downsample_image_size: need rows, cols >= 1 and 0 < factor <= 1");
  *out_rows = (int64_t)((double)rows * factor + 0.5);
  *out_cols = (int64_t)((double)cols * factor + 0.5);
  if (*out_rows < 1 || *out_cols < 1) return fail(XR_ERR_INVALID_ARG, "xr_downsample_image_size: empty result");
  return XR_OK;
}

extern "C" XR_API xr_status xr_downsample_image(const float* d_src, int64_t rows, int64_t cols, double factor,
                                               double* d_scratch, float* d_dst, void* stream) {
  int64_t orows = 0, ocols = 0;
  xr_status st = xr_downsample_image_size(rows, cols, factor, &orows, &ocols);
  if (st != XR_OK) return st;
  if (!d_src || !d_dst || !d_scratch) return fail(XR_ERR_INVALID_ARG, "xr_downsample_image: NULL pointer");
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  const int64_t n = rows * cols;
  const unsigned blocks = (unsigned)std::min<int64_t>((n + 255) / 256, 8192);
  double* a = d_scratch;
  double* b = d_scratch + n;
  if (factor < 1.0) {
    GaussKernel k{};
    const double sigma = 0.5 / factor;
    k.radius = discrete_gaussian_taps(sigma * sigma, 0.01, 32, k.c);
    gauss_pass_kernel<float><<<blocks, 256, 0, s>>>(d_src, (int)rows, (int)cols, 0, k, a);
    gauss_pass_kernel<double><<<blocks, 256, 0, s>>>(a, (int)rows, (int)cols, 1, k, b);
  } else {
    GaussKernel k{};
    k.radius = 0;
    k.c[0] = 1.0;
    gauss_pass_kernel<float><<<blocks, 256, 0, s>>>(d_src, (int)rows, (int)cols, 0, k, b);
  }
  const unsigned ob = (unsigned)std::min<int64_t>((orows * ocols + 255) / 256, 8192);
  resample_kernel<<<ob, 256, 0, s>>>(b, (int)rows, (int)cols, factor, (int)orows, (int)ocols, d_dst);
  XR_CUDA_TRY(cudaGetLastError());
  return XR_OK;
}
