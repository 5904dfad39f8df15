// xr_preproc.cu -- data preparation either side of the hot path, on the device:
//
// * HU -> linear attenuation (HUToLinAttFilter::GenerateData,
//   lib/image/xregHUToLinAtt.cpp:45-69): mu = max(hu * (mu_w - mu_a) 1e-3 + mu_w - mu_lower, 0)
//   in double, stored as float; mu_w = 0.02683, mu_a = 0.02485e-4 /mm, hu_lower = -1000.
// * Fixed-image downsampling for a coarser registration level (DownsampleProjData
//   -> DownsampleImage, lib/image/xregProjData.cpp:40-53,
//   lib/itk/xregITKResampleUtils.h:51-131,183-187): for factor < 1, a discrete
//   Gaussian (ITK DiscreteGaussianImageFilter, variance (0.5/factor)^2 in pixels,
//   maximum error 0.01, kernel width at most 32, edge pixels replicated) along x
//   then y in double, rounded to the float image type; then resampling onto
//   floor(n * factor + 0.5) pixels with the same origin and spacing / factor, so
//   output pixel i reads the smoothed image at continuous index i / factor.  The
//   interpolator is DownsampleImage's default, the cubic B-spline (ITK
//   BSplineInterpolateImageFunction, order 3): coefficients by Unser's recursive
//   prefilter (pole sqrt(3) - 2, gain 6, mirror boundaries, causal start summed
//   to a 1e-10 horizon), along x then y in double; evaluation with the 4 x 4
//   cubic B-spline weights around floor(x) - 1, indices mirrored at 0 and n - 1;
//   points outside [-0.5, n - 0.5) get 0.
// * Projection pre-processing (ProjPreProc, lib/image/xregProjPreProc.cpp:31-139):
//   boundary crop (CropImage2DBoundary, lib/itk/xregITKCropPadUtils.h:89-114) and
//   the log remap (ImageIntensLogTransFilter::GenerateData,
//   lib/image/xregImageIntensLogTrans.cpp:52-146 with UseMaxIntensityAsI0):
//   I0 = max of the image smoothed by a discrete Gaussian of variance 2;
//   out = -log(x / I0) for x > 1e-6, else -log(min_pos / I0) with min_pos the
//   smallest value above 1e-6, all in float.
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
    // explicitly rounded (no fused multiply-add): the same operations as the oracle
    double s = __dmul_rn(k.c[0], (double)in[i]);
    for (int t = 1; t <= k.radius; ++t) {
      int a, b;
      if (dir == 0) {
        a = max(c - t, 0); b = min(c + t, cols - 1);
        s = __dadd_rn(s, __dmul_rn(k.c[t], __dadd_rn((double)in[(int64_t)r * cols + a], (double)in[(int64_t)r * cols + b])));
      } else {
        a = max(r - t, 0); b = min(r + t, rows - 1);
        s = __dadd_rn(s, __dmul_rn(k.c[t], __dadd_rn((double)in[(int64_t)a * cols + c], (double)in[(int64_t)b * cols + c])));
      }
    }
    out[i] = s;
  }
}

// Second smoothing pass result rounded to the float image type, widened back
// to double as the B-spline prefilter's input.
__global__ void round_to_float_kernel(double* __restrict__ v, int64_t n) {
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
    v[i] = (double)(float)v[i];
}

__global__ void widen_kernel(const float* __restrict__ in, int64_t n, double* __restrict__ out) {
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
    out[i] = (double)in[i];
}

// Cubic B-spline prefilter of `count` lines of `len` samples in place: line l
// starts at c + l * line_stride, samples `stride` apart.  One thread per line.
// z = the pole, gain = (1 - z)(1 - 1/z), horizon = terms of the causal start.
__global__ void bspline_prefilter_kernel(double* __restrict__ c, int count, int len, int64_t line_stride,
                                         int64_t stride, double z, double gain, int horizon) {
  const int l = blockIdx.x * blockDim.x + threadIdx.x;
  if (l >= count || len < 2) return;
  double* v = c + (int64_t)l * line_stride;
  for (int n = 0; n < len; ++n) v[n * stride] = __dmul_rn(v[n * stride], gain);
  // causal initialisation (mirror boundaries)
  {
    double zn = z, sum;
    if (horizon < len) {
      sum = v[0];
      for (int n = 1; n < horizon; ++n) {
        sum = __dadd_rn(sum, __dmul_rn(zn, v[n * stride]));
        zn = __dmul_rn(zn, z);
      }
      v[0] = sum;
    } else {
      const double iz = __ddiv_rn(1.0, z);
      double z2n = pow(z, (double)(len - 1));
      sum = __dadd_rn(v[0], __dmul_rn(z2n, v[(int64_t)(len - 1) * stride]));
      z2n = __dmul_rn(z2n, __dmul_rn(z2n, iz));
      for (int n = 1; n <= len - 2; ++n) {
        sum = __dadd_rn(sum, __dmul_rn(__dadd_rn(zn, z2n), v[n * stride]));
        zn = __dmul_rn(zn, z);
        z2n = __dmul_rn(z2n, iz);
      }
      v[0] = __ddiv_rn(sum, __dsub_rn(1.0, __dmul_rn(zn, zn)));
    }
  }
  for (int n = 1; n < len; ++n) v[n * stride] = __dadd_rn(v[n * stride], __dmul_rn(z, v[(n - 1) * stride]));
  // anti-causal initialisation and recursion
  {
    const int64_t a = (int64_t)(len - 1) * stride, b = (int64_t)(len - 2) * stride;
    v[a] = __dmul_rn(__ddiv_rn(z, __dsub_rn(__dmul_rn(z, z), 1.0)), __dadd_rn(__dmul_rn(z, v[b]), v[a]));
  }
  for (int n = len - 2; n >= 0; --n) v[n * stride] = __dmul_rn(z, __dsub_rn(v[(n + 1) * stride], v[n * stride]));
}

__device__ __forceinline__ int mirror_index(int k, int n) {
  if (n == 1) return 0;
  if (k < 0) k = -k;
  if (k > n - 1) k = (n - 1) - (k - (n - 1));
  return k;
}

__device__ __forceinline__ void cubic_weights(double x, int i1, double w[4]) {
  const double t = __dsub_rn(x, (double)i1);
  w[3] = __dmul_rn(__dmul_rn(__dmul_rn(1.0 / 6.0, t), t), t);
  w[0] = __dsub_rn(__dadd_rn(1.0 / 6.0, __dmul_rn(__dmul_rn(0.5, t), __dsub_rn(t, 1.0))), w[3]);
  w[2] = __dsub_rn(__dadd_rn(t, w[0]), __dmul_rn(2.0, w[3]));
  w[1] = __dsub_rn(__dsub_rn(__dsub_rn(1.0, w[0]), w[2]), w[3]);
}

// Output pixel (r, c) = cubic B-spline of the coefficients at (c / factor, r / factor).
__global__ void bspline_resample_kernel(const double* __restrict__ coef, int rows, int cols, double factor,
                                        int orows, int ocols, float* __restrict__ out) {
  const int64_t n = (int64_t)orows * ocols;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    const int r = (int)(i / ocols), c = (int)(i - (int64_t)r * ocols);
    const double x = __ddiv_rn((double)c, factor), y = __ddiv_rn((double)r, factor);
    if (!(x >= -0.5 && x < cols - 0.5 && y >= -0.5 && y < rows - 0.5)) { out[i] = 0.0f; continue; }
    const int x1 = (int)floorf((float)x), y1 = (int)floorf((float)y);  // index of weight 1
    double wx[4], wy[4];
    cubic_weights(x, x1, wx);
    cubic_weights(y, y1, wy);
    int ix[4], iy[4];
#pragma unroll
    for (int k = 0; k < 4; ++k) {
      ix[k] = mirror_index(x1 - 1 + k, cols);
      iy[k] = mirror_index(y1 - 1 + k, rows);
    }
    double acc = 0.0;
#pragma unroll
    for (int b = 0; b < 4; ++b)
#pragma unroll
      for (int a = 0; a < 4; ++a)
        acc = __dadd_rn(acc, __dmul_rn(__dmul_rn(wx[a], wy[b]), coef[(int64_t)iy[b] * cols + ix[a]]));
    out[i] = (float)acc;
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

// Discrete Gaussian taps c[0..radius] (normalised so c0 + 2 sum c_k = 1):
// e^{-t} I_0(t), e^{-t} I_1(t), then the Bessel recurrence
// c_k = c_{k-2} - 2 (k - 1) c_{k-1} / t until the two-sided sum reaches
// 1 - max_error or max_width one-sided taps.
int discrete_gaussian_taps(double variance, double max_error, int max_width, double* out) {
  std::vector<double> c;
  const double cap = 1.0 - max_error;
  c.push_back(scaled_bessel_i(0, variance));
  double sum = c[0];
  c.push_back(scaled_bessel_i(1, variance));
  sum += 2.0 * c[1];
  for (int k = 2; sum < cap && (int)c.size() < kMaxTaps + 1; ++k) {
    c.push_back(c[k - 2] - 2.0 * (k - 1) * c[k - 1] / variance);
    sum += 2.0 * c.back();
    if ((int)c.size() > max_width) break;  // one-sided length limit
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

static unsigned grid_for(int64_t n) { return (unsigned)std::min<int64_t>((n + 255) / 256, 8192); }

// Cubic B-spline coefficients of a rows x cols double image in place: along x
// (one thread per row), then along y (one thread per column).
static cudaError_t bspline_coefficients(double* c, int64_t rows, int64_t cols, cudaStream_t s) {
  const double z = std::sqrt(3.0) - 2.0;
  const double gain = (1.0 - z) * (1.0 - 1.0 / z);
  const int horizon = (int)std::ceil(std::log(1.0e-10) / std::log(std::fabs(z)));
  bspline_prefilter_kernel<<<(unsigned)((rows + 127) / 128), 128, 0, s>>>(c, (int)rows, (int)cols, cols, 1, z, gain,
                                                                          horizon);
  bspline_prefilter_kernel<<<(unsigned)((cols + 127) / 128), 128, 0, s>>>(c, (int)cols, (int)rows, 1, cols, z, gain,
                                                                          horizon);
  return cudaGetLastError();
}

extern "C" XR_API xr_status xr_downsample_image(const float* d_src, int64_t rows, int64_t cols, double factor,
                                               double* d_scratch, float* d_dst, void* stream) {
  int64_t orows = 0, ocols = 0;
  xr_status st = xr_downsample_image_size(rows, cols, factor, &orows, &ocols);
  if (st != XR_OK) return st;
  if (!d_src || !d_dst || !d_scratch) return fail(XR_ERR_INVALID_ARG, "xr_downsample_image: NULL pointer");
  if (rows > (1 << 20) || cols > (1 << 20)) return fail(XR_ERR_INVALID_ARG, "xr_downsample_image: image too large");
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  const int64_t n = rows * cols;
  double* a = d_scratch;
  double* b = d_scratch + n;
  if (factor < 1.0) {
    GaussKernel k{};
    const double sigma = 0.5 / factor;
    k.radius = discrete_gaussian_taps(sigma * sigma, 0.01, 32, k.c);
    gauss_pass_kernel<float><<<grid_for(n), 256, 0, s>>>(d_src, (int)rows, (int)cols, 0, k, a);
    gauss_pass_kernel<double><<<grid_for(n), 256, 0, s>>>(a, (int)rows, (int)cols, 1, k, b);
    round_to_float_kernel<<<grid_for(n), 256, 0, s>>>(b, n);
  } else {
    widen_kernel<<<grid_for(n), 256, 0, s>>>(d_src, n, b);
  }
  XR_CUDA_TRY(bspline_coefficients(b, rows, cols, s));
  bspline_resample_kernel<<<grid_for(orows * ocols), 256, 0, s>>>(b, (int)rows, (int)cols, factor, (int)orows,
                                                                  (int)ocols, d_dst);
  XR_CUDA_TRY(cudaGetLastError());
  return XR_OK;
}

extern "C" XR_API xr_status xr_camera_crop_boundary(const xr_camera_desc* src, int64_t width, xr_camera_desc* out) {
  if (!src || !out) return fail(XR_ERR_INVALID_ARG, "xr_camera_crop_boundary: NULL argument");
  if (width < 0 || src->num_det_rows - 2 * width < 2 || src->num_det_cols - 2 * width < 2)
    return fail(XR_ERR_INVALID_ARG, "xr_camera_crop_boundary: the crop leaves fewer than 2 rows or columns");
  // UpdateCameraModelFor2DROI in float: the principal point moves by the crop,
  // and CameraModel::setup(K, E, ...) derives the focal length again from K
  // (FocalLenFromIntrins, xregPerspectiveXform.cpp:186-190)
  xr_camera_desc d = *src;
  float K[9];
  for (int i = 0; i < 9; ++i) K[i] = (float)src->intrins[i];
  K[2] -= (float)width;
  K[5] -= (float)width;
  for (int i = 0; i < 9; ++i) d.intrins[i] = K[i];
  for (int i = 0; i < 16; ++i) d.extrins[i] = (float)src->extrins[i];
  const float rs = (float)src->det_row_spacing, cs = (float)src->det_col_spacing;
  d.det_row_spacing = rs;
  d.det_col_spacing = cs;
  d.focal_len = (std::fabs(K[0] * cs) + std::fabs(K[4] * ((rs < 0) ? cs : rs))) / 2.0f;
  d.num_det_rows = src->num_det_rows - 2 * width;
  d.num_det_cols = src->num_det_cols - 2 * width;
  *out = d;
  return XR_OK;
}

namespace xr {
namespace {

__global__ void crop_kernel(const float* __restrict__ in, int cols, int width, int orows, int ocols,
                            float* __restrict__ out) {
  const int64_t n = (int64_t)orows * ocols;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    const int r = (int)(i / ocols), c = (int)(i - (int64_t)r * ocols);
    out[i] = in[(int64_t)(r + width) * cols + (c + width)];
  }
}

constexpr int kRedBlocks = 512;
constexpr float kLogEps = 1.0e-6f;

// Second Gaussian pass (along y) rounded to float, reduced to its maximum, and
// the smallest source value above 1e-6; per-block partials.
__global__ void log_remap_stats_kernel(const double* __restrict__ a, const float* __restrict__ src, int rows,
                                       int cols, GaussKernel k, float* __restrict__ part_max,
                                       float* __restrict__ part_min) {
  const int64_t n = (int64_t)rows * cols;
  float mx = -INFINITY, mn = INFINITY;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    const int r = (int)(i / cols), c = (int)(i - (int64_t)r * cols);
    double s = __dmul_rn(k.c[0], a[i]);
    for (int t = 1; t <= k.radius; ++t) {
      const int lo = max(r - t, 0), hi = min(r + t, rows - 1);
      s = __dadd_rn(s, __dmul_rn(k.c[t], __dadd_rn(a[(int64_t)lo * cols + c], a[(int64_t)hi * cols + c])));
    }
    mx = fmaxf(mx, (float)s);
    const float x = src[i];
    if (x > kLogEps) mn = fminf(mn, x);
  }
  __shared__ float smx[32], smn[32];
  for (int o = 16; o > 0; o >>= 1) {
    mx = fmaxf(mx, __shfl_down_sync(0xffffffffu, mx, o));
    mn = fminf(mn, __shfl_down_sync(0xffffffffu, mn, o));
  }
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  if (lane == 0) { smx[w] = mx; smn[w] = mn; }
  __syncthreads();
  if (threadIdx.x == 0) {
    for (int j = 1; j < (int)(blockDim.x >> 5); ++j) { mx = fmaxf(mx, smx[j]); mn = fminf(mn, smn[j]); }
    part_max[blockIdx.x] = mx;
    part_min[blockIdx.x] = mn;
  }
}

// scal[0] = I0, scal[1] = -log(min_pos / I0) (min_pos 0 when no value exceeds 1e-6).
__global__ void log_remap_finalize_kernel(const float* __restrict__ part_max, const float* __restrict__ part_min,
                                          int nblk, int use_max, float i0, float* __restrict__ scal) {
  if (threadIdx.x != 0 || blockIdx.x != 0) return;
  float mx = -INFINITY, mn = INFINITY;
  for (int j = 0; j < nblk; ++j) { mx = fmaxf(mx, part_max[j]); mn = fminf(mn, part_min[j]); }
  const float I0 = use_max ? mx : i0;
  const float min_pos = (mn == INFINITY) ? 0.0f : mn;
  scal[0] = I0;
  scal[1] = -logf(__fdiv_rn(min_pos, I0));
}

__global__ void log_remap_kernel(const float* __restrict__ src, int64_t n, const float* __restrict__ scal,
                                 float* __restrict__ out) {
  const float I0 = scal[0], out_max = scal[1];
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    const float x = src[i];
    out[i] = (x > kLogEps) ? -logf(__fdiv_rn(x, I0)) : out_max;
  }
}

}  // namespace
}  // namespace xr

extern "C" XR_API xr_status xr_crop_image_boundary(const float* d_src, int64_t rows, int64_t cols, int64_t width,
                                                  float* d_dst, void* stream) {
  if (!d_src || !d_dst) return fail(XR_ERR_INVALID_ARG, "xr_crop_image_boundary: NULL pointer");
  if (width < 0 || rows - 2 * width < 1 || cols - 2 * width < 1 || rows > (1 << 30) || cols > (1 << 30))
    return fail(XR_ERR_INVALID_ARG, "xr_crop_image_boundary: the crop leaves no pixels");
  const int64_t orows = rows - 2 * width, ocols = cols - 2 * width;
  crop_kernel<<<grid_for(orows * ocols), 256, 0, static_cast<cudaStream_t>(stream)>>>(
      d_src, (int)cols, (int)width, (int)orows, (int)ocols, d_dst);
  XR_CUDA_TRY(cudaGetLastError());
  return XR_OK;
}

extern "C" XR_API xr_status xr_log_remap(const float* d_src, int64_t rows, int64_t cols, int32_t use_max_as_i0,
                                        float i0, double* d_scratch, float* d_dst, void* stream) {
  if (!d_src || !d_dst || !d_scratch) return fail(XR_ERR_INVALID_ARG, "xr_log_remap: NULL pointer");
  if (rows < 1 || cols < 1 || rows > (1 << 20) || cols > (1 << 20))
    return fail(XR_ERR_INVALID_ARG, "xr_log_remap: bad image size");
  if (!use_max_as_i0 && !(i0 > 0.0f)) return fail(XR_ERR_INVALID_ARG, "xr_log_remap: I0 must be positive");
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  const int64_t n = rows * cols;
  double* a = d_scratch;
  float* part_max = reinterpret_cast<float*>(d_scratch + n);
  float* part_min = part_max + kRedBlocks;
  float* scal = part_min + kRedBlocks;
  GaussKernel k{};
  k.radius = discrete_gaussian_taps(2.0, 0.01, 32, k.c);
  gauss_pass_kernel<float><<<grid_for(n), 256, 0, s>>>(d_src, (int)rows, (int)cols, 0, k, a);
  const int nblk = (int)std::min<int64_t>((n + 255) / 256, kRedBlocks);
  log_remap_stats_kernel<<<nblk, 256, 0, s>>>(a, d_src, (int)rows, (int)cols, k, part_max, part_min);
  log_remap_finalize_kernel<<<1, 32, 0, s>>>(part_max, part_min, nblk, use_max_as_i0, i0, scal);
  log_remap_kernel<<<grid_for(n), 256, 0, s>>>(d_src, n, scal, d_dst);
  XR_CUDA_TRY(cudaGetLastError());
  return XR_OK;
}
