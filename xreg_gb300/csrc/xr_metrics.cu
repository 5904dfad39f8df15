// xr_metrics.cu -- 2D similarity metric kernels.
//
// NCC (xregImgSimMetric2DNCCCPU.cpp:53-63,164-209): per moving image the sums
// S_m, S_mm, S_mf (f = zero-mean fixed image) are accumulated per thread in
// compensated (Kahan) float, reduced per block in double, and combined per image
// in double:  mean_m = S_m/n, var_m = (S_mm - n mean_m^2)/(n-1), sd = max(1e-6, sqrt),
// cov = S_mf - mean_m * sum(f), ncc = cov / (n sd_f sd_m), sim = (1 - ncc)/2.
//
// Gradient images (xregImgSimMetric2DGradImgCPU.cpp:48-65,86-101): 5x5 Gaussian
// with OpenCV's fixed sigma-0 kernel [1 4 6 4 1]/16 (3x3: [1 2 1]/4), then 3x3
// Sobel in x and y, BORDER_REFLECT_101 everywhere.  A block stages a 32x32 tile
// plus halo in shared memory; the blurred tile is computed over the
// reflect-extended input, which equals the reflect-extended blurred image because
// the kernels are symmetric.
//
// Patch NCC (xregImgSimMetric2DPatchNCCCPU.cpp:205-287,558-619): one thread per
// patch centre, two-pass mean / sample std dev over the (2r+1)^2 window from a
// shared-memory tile, score 1 - sum((m - mu_m)/sd_m * fhat), unit weights, mean
// over patches.  The fixed side (per-patch mean and 1/(sd n)) is pre-computed once.
#include "xr_cmaes_core.h"
#include "xr_gradtile.cuh"

#include <cfloat>

namespace xr {
namespace {

constexpr int kT = 32;          // output tile edge for gradient kernels
using gt::kThreads;

using gt::FF;
using gt::ff_add;
using gt::ff_prod;
using gt::ff_shfl_down;
using gt::reflect101;
using gt::warp_sum_d;
using gt::ncc_sim_from_moments;

struct Kahan {
  float s = 0.0f, c = 0.0f;
  __device__ __forceinline__ void add(float x) {
    const float y = x - c;
    const float t = s + y;
    c = (t - s) - y;
    s = t;
  }
  __device__ __forceinline__ double value() const { return (double)s - (double)c; }
  __device__ __forceinline__ FF ff() const { return FF{s, -c}; }
};

// Block-wide sum of K float-float values per thread, returned in double by
// thread 0 (the other threads get undefined values).
template <int K>
__device__ __forceinline__ void block_sum_ff(FF (&v)[K], double (&out)[K], FF* red /* [K][32] */) {
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
#pragma unroll
  for (int k = 0; k < K; ++k) {
    FF w = v[k];
    for (int o = 16; o > 0; o >>= 1) w = ff_add(w, ff_shfl_down(w, o));
    if (lane == 0) red[k * 32 + warp] = w;
  }
  __syncthreads();
  if (warp == 0) {
#pragma unroll
    for (int k = 0; k < K; ++k) {
      FF w = (lane < nw) ? red[k * 32 + lane] : FF{0.0f, 0.0f};
      for (int o = 16; o > 0; o >>= 1) w = ff_add(w, ff_shfl_down(w, o));
      out[k] = (double)w.hi + (double)w.lo;
    }
  }
}

// Block-wide sum of K doubles per thread over all warps; result valid in thread 0.
template <int K>
__device__ __forceinline__ void block_sum_d(double (&v)[K], double* red /* [K][32] */) {
  gt::block_sum_d<K>(v, red, (int)(blockDim.x >> 5));
}

// ------------------------------------------------------------------ setup --
__global__ void image_sum_kernel(const float* __restrict__ img, int64_t n, const uint8_t* __restrict__ mask,
                                 double* __restrict__ out) {
  __shared__ double red[2 * 32];
  double v[2] = {0.0, 0.0};
  for (int64_t i = threadIdx.x; i < n; i += blockDim.x)
    if (!mask || mask[i]) { v[0] += (double)img[i]; v[1] += 1.0; }
  block_sum_d<2>(v, red);
  if (threadIdx.x == 0) { out[0] = v[0]; out[2] = v[1]; }
}

__global__ void image_var_kernel(const float* __restrict__ img, int64_t n, const uint8_t* __restrict__ mask,
                                 double* __restrict__ out) {
  __shared__ double red[1 * 32];
  const double mean = out[0] / out[2];
  double v[1] = {0.0};
  for (int64_t i = threadIdx.x; i < n; i += blockDim.x)
    if (!mask || mask[i]) { const double d = (double)img[i] - mean; v[0] += d * d; }
  block_sum_d<1>(v, red);
  if (threadIdx.x == 0) out[1] = v[0];
}

__global__ void sub_scalar_kernel(const float* __restrict__ in, int64_t n, float value, float* __restrict__ out) {
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
    out[i] = in[i] - value;
}

// ---------------------------------------------------------------- NCC -----
__global__ void __launch_bounds__(kThreads) ncc_moments_kernel(const float* __restrict__ mov, int64_t npix,
                                                               const float* __restrict__ fhat,
                                                               const uint8_t* __restrict__ mask,
                                                               double* __restrict__ partials) {
  __shared__ FF red[3 * 32];
  const int64_t img = blockIdx.y;
  const float* m = mov + img * npix;
  Kahan s0, s1, s2;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < npix; i += (int64_t)gridDim.x * blockDim.x) {
    if (mask && !mask[i]) continue;
    const float x = m[i];
    s0.add(x);
    s1.add(x * x);
    s2.add(x * fhat[i]);
  }
  FF f[3] = {s0.ff(), s1.ff(), s2.ff()};
  double v[3];
  block_sum_ff<3>(f, v, red);
  if (threadIdx.x == 0) {
    double* o = partials + (img * gridDim.x + blockIdx.x) * 3;
    o[0] = v[0]; o[1] = v[1]; o[2] = v[2];
  }
}

// One block per image (as grad_finalize_kernel).
__global__ void ncc_finalize_kernel(const double* __restrict__ partials, int nblk, int64_t nimgs, double n,
                                    FixedNCC fx, float* __restrict__ sims) {
  __shared__ double red[3 * 32];
  const int64_t img = blockIdx.x;
  double a[3] = {0, 0, 0};
  const double* p = partials + img * nblk * 3;
  for (int k = threadIdx.x; k < nblk; k += blockDim.x) {
    a[0] += p[3 * k];
    a[1] += p[3 * k + 1];
    a[2] += p[3 * k + 2];
  }
  block_sum_d<3>(a, red);
  if (threadIdx.x == 0) sims[img] = (float)ncc_sim_from_moments(a[0], a[1], a[2], n, fx);
}

// ------------------------------------------------------ gradient images ---
// Stages rows [y0-H, y0+kT+H) x cols [x0-H, x0+kT+H) of an image (reflected at
// the borders), blurs with radius KR and applies Sobel on the kT x kT tile.
template <int KR>
struct GradTile {
  static constexpr int H = KR + 1;            // total halo
  static constexpr int WI = kT + 2 * H;       // staged input edge
  static constexpr int WB = kT + 2;           // blurred region edge
  float in[WI][WI + 1];
  float hb[WI][WB + 1];
  float bl[WB][WB + 1];

  __device__ void load(const float* __restrict__ img, int rows, int cols, int y0, int x0) {
    for (int i = threadIdx.x; i < WI * WI; i += blockDim.x) {
      const int r = i / WI, c = i - r * WI;
      // Rows/cols past the last tile pixel only feed pixels that are skipped;
      // clamping before the reflection keeps every read inside the image.
      const int gr = reflect101(min(y0 - H + r, rows - 1 + H), rows);
      const int gc = reflect101(min(x0 - H + c, cols - 1 + H), cols);
      in[r][c] = img[(int64_t)gr * cols + gc];
    }
    __syncthreads();
  }

  __device__ void blur() {
    if constexpr (KR == 0) {
      for (int i = threadIdx.x; i < WB * WB; i += blockDim.x) {
        const int r = i / WB, c = i - r * WB;
        bl[r][c] = in[r][c];
      }
      __syncthreads();
    } else {
    // horizontal pass over all staged rows, blurred columns [x0-1, x0+kT+1)
    for (int i = threadIdx.x; i < WI * WB; i += blockDim.x) {
      const int r = i / WB, c = i - r * WB;
      float s;
      if (KR == 2) {
        s = 0.0625f * in[r][c] + 0.25f * in[r][c + 1] + 0.375f * in[r][c + 2] + 0.25f * in[r][c + 3] +
            0.0625f * in[r][c + 4];
      } else {
        s = 0.25f * in[r][c] + 0.5f * in[r][c + 1] + 0.25f * in[r][c + 2];
      }
      hb[r][c] = s;
    }
    __syncthreads();
    for (int i = threadIdx.x; i < WB * WB; i += blockDim.x) {
      const int r = i / WB, c = i - r * WB;
      float s;
      if (KR == 2) {
        s = 0.0625f * hb[r][c] + 0.25f * hb[r + 1][c] + 0.375f * hb[r + 2][c] + 0.25f * hb[r + 3][c] +
            0.0625f * hb[r + 4][c];
      } else {
        s = 0.25f * hb[r][c] + 0.5f * hb[r + 1][c] + 0.25f * hb[r + 2][c];
      }
      bl[r][c] = s;
    }
    __syncthreads();
    }
  }

  // Sobel at tile pixel (ty, tx) in [0, kT).
  __device__ __forceinline__ void sobel(int ty, int tx, float& gx, float& gy) const {
    const int r = ty + 1, c = tx + 1;
    const float a = bl[r - 1][c - 1], b = bl[r - 1][c], cc = bl[r - 1][c + 1];
    const float d = bl[r][c - 1], f = bl[r][c + 1];
    const float g = bl[r + 1][c - 1], h = bl[r + 1][c], ii = bl[r + 1][c + 1];
    gx = ((cc - a) + 2.0f * (f - d)) + (ii - g);
    gy = ((g - a) + 2.0f * (h - b)) + (ii - cc);
  }
};

template <int KR>
__global__ void __launch_bounds__(kThreads) grad_images_kernel(const float* __restrict__ imgs, int rows, int cols,
                                                               float* __restrict__ gx, float* __restrict__ gy) {
  __shared__ GradTile<KR> t;
  const int tiles_x = (cols + kT - 1) / kT;
  const int y0 = (blockIdx.x / tiles_x) * kT, x0 = (blockIdx.x % tiles_x) * kT;
  const int64_t npix = (int64_t)rows * cols;
  const int64_t img = blockIdx.y;
  t.load(imgs + img * npix, rows, cols, y0, x0);
  t.blur();
  for (int i = threadIdx.x; i < kT * kT; i += blockDim.x) {
    const int ty = i / kT, tx = i - ty * kT;
    if (y0 + ty >= rows || x0 + tx >= cols) continue;
    float a, b;
    t.sobel(ty, tx, a, b);
    const int64_t o = img * npix + (int64_t)(y0 + ty) * cols + x0 + tx;
    gx[o] = a;
    gy[o] = b;
  }
}

// Moments of the moving gradients, one 32 x 64-pixel tile per block
// (gt::grad_tile_moments, shared with the fused evaluation kernel).
using gt::kGH;
using gt::kGW;

template <int KR>
__global__ void __launch_bounds__(kThreads) grad_moments_kernel(const float* __restrict__ imgs, int rows, int cols,
                                                                const float* __restrict__ fhx,
                                                                const float* __restrict__ fhy,
                                                                const uint8_t* __restrict__ mask,
                                                                double* __restrict__ partials) {
  __shared__ gt::GradTileSmem<KR> sm;
  const int tiles_x = (cols + kGW - 1) / kGW;
  const int y0 = (blockIdx.x / tiles_x) * kGH, x0 = (blockIdx.x % tiles_x) * kGW;
  const int64_t img = blockIdx.y;
  double v[6];
  gt::grad_tile_moments<KR, false>(imgs + img * (int64_t)rows * cols, rows, cols, y0, x0, fhx, fhy, mask, sm, v);
  if (threadIdx.x == 0) {
    double* o = partials + (img * gridDim.x + blockIdx.x) * 6;
#pragma unroll
    for (int k = 0; k < 6; ++k) o[k] = v[k];
  }
}

// One block of 128 threads per image: the tile partials combined in double
// (gt::grad_finalize_image, shared with the fused evaluation kernel).
__global__ void grad_finalize_kernel(const double* __restrict__ partials, int nblk, int64_t nimgs, double n,
                                     FixedNCC fx, FixedNCC fy, float* __restrict__ sims) {
  __shared__ double red[6 * (gt::kFinalizeThreads / 32)];
  const int64_t img = blockIdx.x;
  const float v = gt::grad_finalize_image<false>(partials + img * nblk * 6, nblk, n, fx, fy, red);
  if (threadIdx.x == 0) sims[img] = v;
}

// Batched grad-NCC over many jobs' images (launch_grad_multi): one block per
// 32x64 tile, grid-stride; the counters of FusedJob::cnt (images, then poses)
// chain the per-image combine and the mean over views behind the tiles.
// A device CMA-ES job's update from its lambda values (the float means over
// views, widened to double as the host step does) by a whole block: the stages
// of cma::update (cmaes_UpdateDistribution, then cmaes_TestForTermination),
// the ranks, recombination sums and covariance entries one per thread.
__device__ __noinline__ void cma_update_block(void* state, const float* vals, CmaReport* report) {
  __shared__ double scal[3];
  const cma::View s = cma::view(state);
  const int n = s.h->n, lam = s.h->lam, mu = s.h->mu, nt = blockDim.x, tid = threadIdx.x;
  for (int k = tid; k < lam; k += nt) s.fv[k] = (double)__ldcg(vals + k);
  __syncthreads();
  for (int k = tid; k < lam; k += nt) cma::rank(s, k);
  __syncthreads();
  if (tid == 0) cma::keep_best(s);
  __syncthreads();
  for (int t = tid; t < 2 * n; t += nt) cma::recombine(s, t);
  __syncthreads();
  if (tid == 0) cma::paths(s, scal);
  __syncthreads();
  for (int t = tid; t < mu * n; t += nt) cma::steps(s, t);
  __syncthreads();
  for (int e = tid; e < n * (n + 1) / 2; e += nt) cma::covariance(s, e, scal);
  __syncthreads();
  if (tid == 0) cma::step_size(s, scal);
  for (int e = tid; e < n * n; e += nt) cma::eig_cb(s, e);
  __syncthreads();
  for (int e = tid; e < n * (n + 1) / 2; e += nt) cma::eig_btcb(s, e);
  __syncthreads();
  const int pairs = cma::rr_pairs(n), rounds = cma::rr_rounds(n);
  for (int sweep = 0; sweep < cma::kMaxSweeps; ++sweep) {
    if (tid == 0) s.h->rotated = 0;
    __syncthreads();
    for (int r = 0; r < rounds; ++r) {
      for (int i = tid; i < pairs; i += nt) cma::rot_params(n, s.A, r, i, s.rot, &s.h->rotated);
      __syncthreads();
      for (int e = tid; e < pairs * n; e += nt) cma::rot_cols(n, s.A, s.V, r, e / n, s.rot, e % n);
      __syncthreads();
      for (int e = tid; e < pairs * n; e += nt) cma::rot_rows(n, s.A, r, e / n, s.rot, e % n);
      __syncthreads();
    }
    const int rotated = *(volatile int32_t*)&s.h->rotated;
    __syncthreads();  // every thread has read the flag before the next sweep clears it
    if (!rotated) break;
  }
  for (int e = tid; e < n * n; e += nt) cma::eig_bv(s, e);
  __syncthreads();
  for (int e = tid; e < n * n; e += nt) s.B[e] = s.T[e];
  __syncthreads();
  if (tid == 0) {
    cma::finish(s);
    if (report) {
      report->reason = s.h->reason;
      double r = 0.0, t = 0.0;
      for (int i = 0; i < n; ++i) {
        const double sd = s.h->sigma * sqrt(s.C[i * n + i]);
        if (i < 3) r = fmax(r, sd);
        else t = fmax(t, sd);
      }
      report->sd_rot = r;
      report->sd_trans = t;
    }
  }
  __syncthreads();
}

__global__ void cma_update_kernel(const CmaUpdateJob* __restrict__ jobs) {
  cma_update_block(jobs[blockIdx.x].cma, jobs[blockIdx.x].vals, jobs[blockIdx.x].report);
}

// The last tile of an image combines its moments (FP64); the last view of a
// pose, the mean over views; the last pose of a job with a device optimizer,
// the optimizer's update (the whole block).  Out of line so the tile loop keeps
// the register budget of the per-view moments kernel (40 registers, 6 blocks
// per SM, where the inlined FP64 combine took 80 and 3).
__device__ __noinline__ void grad_multi_finish(const FusedJob& J, const FusedView& V, int64_t k, int mt, int64_t nimg,
                                               double* dred, int* job_done) {
  __threadfence();
  const float sim = gt::grad_finalize_image<true>(V.partials + k * mt * 6, mt, V.n_used, V.fx, V.fy, dred);
  if (threadIdx.x == 0) {
    int done = 0;
    V.sims[k] = sim;
    __threadfence();
    unsigned int* cp = J.cnt + nimg * mt + nimg + k;
    if (atomicAdd(cp, 1u) + 1u == (unsigned int)J.nviews) {  // every view of this pose
      *cp = 0u;
      __threadfence();
      float sum = 0.0f;
      for (int w = 0; w < J.nviews; ++w) sum += __ldcg(J.views[w].sims + k);
      J.out[k] = sum / (float)J.nviews;  // ImgSimMetric2DCombineMean (as gt::combine_mean)
      if (J.cma) {  // the job's last pose: its optimizer's update by this block
        __threadfence();
        unsigned int* cj = J.cnt + nimg * mt + nimg + J.pop;
        if (atomicAdd(cj, 1u) + 1u == (unsigned int)J.pop) {
          *cj = 0u;
          done = 1;
        }
      }
    }
    *job_done = done;
  }
  __syncthreads();
  if (*job_done) {
    __threadfence();
    cma_update_block(J.cma, J.out, J.report);
  }
}

__global__ void __launch_bounds__(kThreads, 6) grad_multi_kernel(const FusedJob* __restrict__ jobs, int njobs,
                                                                 long long total) {
  __shared__ gt::GradTileSmem<2> sm;
  __shared__ double dred[6 * (gt::kFinalizeThreads / 32)];
  __shared__ int s_last, s_job_done;
  for (long long t = blockIdx.x; t < total; t += gridDim.x) {
    int j = 0;
    while (j + 1 < njobs && jobs[j + 1].tile_begin <= t) ++j;
    const FusedJob& J = jobs[j];
    const int rows = J.d.p.rows, cols = J.d.p.cols, mt = J.mt_x * J.mt_y;
    const long long local = t - J.tile_begin;
    const int64_t img = local / mt;  // projection: view-major (view * pop + pose)
    const int M = (int)(local - img * mt);
    const int64_t nimg = (int64_t)J.nviews * J.pop, v = img / J.pop, k = img - v * J.pop;
    const FusedView& V = J.views[v];
    double vals[6];
    gt::grad_tile_moments<2, false>(J.d.p.out + img * (int64_t)rows * cols, rows, cols, (M / J.mt_x) * kGH,
                                    (M % J.mt_x) * kGW, V.fhx, V.fhy, V.mask, sm, vals);
    if (threadIdx.x == 0) {
      double* o = V.partials + (k * mt + M) * 6;
#pragma unroll
      for (int q = 0; q < 6; ++q) o[q] = vals[q];
      __threadfence();
      unsigned int* ci = J.cnt + nimg * mt + img;
      s_last = atomicAdd(ci, 1u) + 1u == (unsigned int)mt;
      if (s_last) *ci = 0u;
    }
    __syncthreads();
    if (s_last) grad_multi_finish(J, V, k, mt, nimg, dred, &s_job_done);  // every tile of this image is in
    __syncthreads();
  }
}

// ------------------------------------------------------------ patch NCC ---
constexpr int kPC = 16;  // patch centres per tile edge

// Per-patch statistics of a fixed image (ComputePatchMeanStdDev,
// xregImgSimMetric2DPatchNCCCPU.cpp:558-619, in double): pixels that count are
// all of them, or the masked-in ones when use_mask_stats; the mean is divided
// and the variance formed only when more than one pixel counts; sd >= 1e-6.
// mean / scale = 1 / (sd n) give the scaled fixed patch (f - mean) scale.
// wvar (optional): the squared sd used as a patch weight (with the mask when
// there is one, xregImgSimMetric2DPatchNCCCPU.cpp:402-411); ucount (optional):
// masked-in pixels of the patch.
__device__ void patch_stats_d(const float* __restrict__ img, int cols, int r0, int c0, int d,
                              const uint8_t* __restrict__ mask, int use_mask, double* mu_out, double* sd_out,
                              int* n_out) {
  int n = 0;
  double s = 0;
  for (int r = 0; r < d; ++r)
    for (int c = 0; c < d; ++c) {
      const int64_t i = (int64_t)(r0 + r) * cols + c0 + c;
      if (!use_mask || !mask || mask[i]) { s += img[i]; ++n; }
    }
  double var = 0;
  if (n > 1) {
    s /= (double)n;
    for (int r = 0; r < d; ++r)
      for (int c = 0; c < d; ++c) {
        const int64_t i = (int64_t)(r0 + r) * cols + c0 + c;
        if (!use_mask || !mask || mask[i]) { const double t = img[i] - s; var += t * t; }
      }
    var /= (double)(n - 1);
  }
  double sd = sqrt(var);
  if (sd < 1.0e-6) sd = 1.0e-6;
  *mu_out = s;
  *sd_out = sd;
  *n_out = n;
}

__global__ void patch_fixed_stats_kernel(const float* __restrict__ img, int cols, int radius, int stride, int ncr,
                                         int ncc, const uint8_t* __restrict__ mask, int use_mask_stats,
                                         float* __restrict__ mean, float* __restrict__ scale,
                                         float* __restrict__ wvar, int* __restrict__ ucount) {
  const int64_t p = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= (int64_t)ncr * ncc) return;
  const int pr = (int)(p / ncc), pc = (int)(p - (int64_t)pr * ncc);
  const int r0 = pr * stride, c0 = pc * stride, d = 2 * radius + 1;
  double mu, sd;
  int n;
  patch_stats_d(img, cols, r0, c0, d, mask, use_mask_stats, &mu, &sd, &n);
  if (mean) {
    mean[p] = (float)mu;
    scale[p] = (float)(1.0 / (sd * (double)n));
  }
  if (wvar) {
    if (mask && !use_mask_stats) patch_stats_d(img, cols, r0, c0, d, mask, 1, &mu, &sd, &n);
    wvar[p] = (float)(sd * sd);
  }
  if (ucount) {
    int k = 0;
    for (int r = 0; r < d; ++r)
      for (int c = 0; c < d; ++c) k += (!mask || mask[(int64_t)(r0 + r) * cols + c0 + c]) ? 1 : 0;
    ucount[p] = k;
  }
}

// Shared-memory layout for one tile of kPC x (kPC rb) patch centres (columns x
// rows; dynamic): rb = patches scored per thread, stacked in a column.
struct PatchLayout {
  int Wr, Wc;    // patch-window region (moving gradient / fixed tiles)
  int WIr, WIc;  // staged input
  int WBr, WBc;  // blurred
  size_t fbytes;  // float part
  size_t bytes;   // plus the Wr x Wc mask tile
  __host__ __device__ static PatchLayout make(int radius, int stride, int grad, int kr, int rb) {
    PatchLayout L;
    L.Wc = (kPC - 1) * stride + 2 * radius + 1;
    L.Wr = (kPC * rb - 1) * stride + 2 * radius + 1;
    L.WBc = grad ? L.Wc + 2 : L.Wc;
    L.WBr = grad ? L.Wr + 2 : L.Wr;
    L.WIc = grad ? L.WBc + 2 * kr : L.Wc;
    L.WIr = grad ? L.WBr + 2 * kr : L.Wr;
    const size_t w = (size_t)L.Wr * L.Wc;
    const size_t fl = grad ? ((size_t)L.WIr * L.WIc + (size_t)L.WIr * L.WBc + (size_t)L.WBr * L.WBc + 4 * w)
                           : ((size_t)L.WIr * L.WIc + w);
    L.fbytes = fl * sizeof(float);
    L.bytes = L.fbytes + ((w + 15) & ~(size_t)15);
    return L;
  }
};

// Score 1 - sum over masked-in pixels of (m - mu_m) / sd_m * (f - fmean) fscale,
// moving statistics over all pixels (masked-in ones when use_mask_stats); the
// unmasked case is the plain patch NCC.  *var = sd_m^2.
__device__ __forceinline__ float patch_score(const float* __restrict__ m, const float* __restrict__ f,
                                             const uint8_t* __restrict__ mk, int W, int r0, int c0, int d,
                                             float fmean, float fscale, int use_mask_stats, int mask_in_sums) {
  float s = 0.0f;
  int n = 0;
  for (int r = 0; r < d; ++r)
    for (int c = 0; c < d; ++c)
      if (!use_mask_stats || !mk || mk[(r0 + r) * W + c0 + c]) { s += m[(r0 + r) * W + c0 + c]; ++n; }
  const float mu = n > 1 ? s / (float)n : s;
  float v = 0.0f, cov = 0.0f;
  for (int r = 0; r < d; ++r)
    for (int c = 0; c < d; ++c) {
      const int i = (r0 + r) * W + c0 + c;
      const float dm = m[i] - mu;
      if (!use_mask_stats || !mk || mk[i]) v = fmaf(dm, dm, v);
      if (!mk || !mask_in_sums || mk[i]) cov = fmaf(dm, f[i] - fmean, cov);
    }
  float sd = n > 1 ? sqrtf(v / (float)(n - 1)) : 0.0f;
  sd = fmaxf(sd, 1.0e-6f);
  return 1.0f - (cov / sd) * fscale;
}

// Sample variance (sd clamped at 1e-6, squared) of a d x d window with row pitch P.
__device__ __forceinline__ float patch_var(const float* __restrict__ m, int P, int r0, int c0, int d) {
  float s = 0.0f;
  for (int r = 0; r < d; ++r)
    for (int c = 0; c < d; ++c) s += m[(r0 + r) * P + c0 + c];
  const float n = (float)(d * d);
  const float mu = s / n;
  float v = 0.0f;
  for (int r = 0; r < d; ++r)
    for (int c = 0; c < d; ++c) {
      const float dm = m[(r0 + r) * P + c0 + c] - mu;
      v = fmaf(dm, dm, v);
    }
  const float sd = fmaxf(sqrtf(v / (n - 1.0f)), 1.0e-6f);
  return sd * sd;
}

// RB vertically adjacent unmasked patches of one thread (tile-local rows
// lr RB .. lr RB + RB - 1, column c0): each moving / fixed value is read once
// from shared memory for every patch whose window holds it.  Per patch the
// operations and their order are those of patch_score without a mask (sum in
// row-major order, mean, then variance and covariance in row-major order), so
// each score has the same bits.  DC / SC > 0: the patch edge and stride known
// at compile time (xReg's default 11 x 11, stride 1): each row's columns unroll
// (no loop control or address arithmetic per element).
template <int RB, int DC, int SC>
__device__ __forceinline__ void patch_scores_rows(const float* __restrict__ m, const float* __restrict__ f, int Wc,
                                                  int rbase, int c0, int d_rt, int stride_rt,
                                                  const float (&fmean)[RB], const float (&fscale)[RB],
                                                  float (&score)[RB]) {
  const int d = DC > 0 ? DC : d_rt;
  const int stride = SC > 0 ? SC : stride_rt;
  const int span = (RB - 1) * stride + d;
  constexpr int kUnroll = DC > 0 ? DC : 1;  // the columns of a patch row (the rows stay a loop: registers)
  float acc[RB], v[RB], cov[RB];
#pragma unroll
  for (int j = 0; j < RB; ++j) { acc[j] = 0.0f; v[j] = 0.0f; cov[j] = 0.0f; }
#pragma unroll 1
  for (int rr = 0; rr < span; ++rr) {
    bool in[RB];
#pragma unroll
    for (int j = 0; j < RB; ++j) in[j] = rr >= j * stride && rr < j * stride + d;
    const float* row = m + (rbase + rr) * Wc + c0;
#pragma unroll kUnroll
    for (int c = 0; c < d; ++c) {
      const float x = row[c];
#pragma unroll
      for (int j = 0; j < RB; ++j)
        if (in[j]) acc[j] += x;
    }
  }
  const float n = (float)(d * d);
  float mu[RB];
#pragma unroll
  for (int j = 0; j < RB; ++j) mu[j] = d * d > 1 ? acc[j] / n : acc[j];
#pragma unroll 1
  for (int rr = 0; rr < span; ++rr) {
    bool in[RB];
#pragma unroll
    for (int j = 0; j < RB; ++j) in[j] = rr >= j * stride && rr < j * stride + d;
    const int o = (rbase + rr) * Wc + c0;
#pragma unroll kUnroll
    for (int c = 0; c < d; ++c) {
      const float x = m[o + c], fx = f[o + c];
#pragma unroll
      for (int j = 0; j < RB; ++j)
        if (in[j]) {
          const float dm = x - mu[j];
          v[j] = fmaf(dm, dm, v[j]);
          cov[j] = fmaf(dm, fx - fmean[j], cov[j]);
        }
    }
  }
#pragma unroll
  for (int j = 0; j < RB; ++j) {
    float sd = d * d > 1 ? sqrtf(v[j] / (n - 1.0f)) : 0.0f;
    sd = fmaxf(sd, 1.0e-6f);
    score[j] = 1.0f - (cov[j] / sd) * fscale[j];
  }
}

// PASS 0: per image and direction, the sum over used patches with an unmasked
// centre of count x moving-patch variance (the normaliser of variance weights).
// PASS 1: per image and direction, the sum over used patches of
// count x weight x score (weight 1 when not weighting in the combine).
template <int GRAD, int KR, int PASS, int RB, int DC = 0, int SC = 0>
__global__ void __launch_bounds__(kThreads) patch_ncc_kernel(const float* __restrict__ imgs, int rows, int cols,
                                                             int radius, int stride, int ncr, int ncc,
                                                             PatchFixed px, PatchFixed py, PatchRun run,
                                                             double* __restrict__ partials) {
  extern __shared__ float sm[];
  __shared__ FF red[2 * 32];
  const PatchLayout L = PatchLayout::make(radius, stride, GRAD, KR, RB);
  const int Wr = L.Wr, Wc = L.Wc, WIr = L.WIr, WIc = L.WIc, WBr = L.WBr, WBc = L.WBc;
  const int WW = Wr * Wc;
  float* s_in = sm;                              // WIr x WIc
  float* s_hb = s_in + WIr * WIc;                // WIr x WBc (GRAD)
  float* s_bl = s_hb + WIr * WBc;                // WBr x WBc (GRAD)
  float* s_mx = GRAD ? s_bl + WBr * WBc : s_in;  // Wr x Wc moving (gx or raw)
  float* s_my = s_mx + WW;                       // Wr x Wc moving gy
  float* s_fx = GRAD ? s_my + WW : s_in + WIr * WIc;  // Wr x Wc fixed (gx or raw)
  float* s_fy = s_fx + WW;
  uint8_t* s_mk = reinterpret_cast<uint8_t*>(reinterpret_cast<char*>(sm) + L.fbytes);  // Wr x Wc mask

  const int tiles_x = (ncc + kPC - 1) / kPC;
  const int tpr = blockIdx.x / tiles_x, tpc = blockIdx.x - tpr * tiles_x;
  const int pr0 = tpr * kPC * RB, pc0 = tpc * kPC;
  const int y0 = pr0 * stride, x0 = pc0 * stride;  // top-left pixel of the window region
  const int64_t npix = (int64_t)rows * cols;
  const int64_t img = blockIdx.y;
  const float* src = imgs + img * npix;
  const int H = GRAD ? (KR + 1) : 0;
  const uint8_t* mk = run.mask ? s_mk : nullptr;

  for (int i = threadIdx.x; i < WIr * WIc; i += blockDim.x) {
    const int r = i / WIc, c = i - r * WIc;
    const int gr = reflect101(min(y0 - H + r, rows - 1 + H), rows);
    const int gc = reflect101(min(x0 - H + c, cols - 1 + H), cols);
    s_in[i] = src[(int64_t)gr * cols + gc];
  }
  for (int i = threadIdx.x; i < WW; i += blockDim.x) {
    const int r = i / Wc, c = i - r * Wc;
    const int gr = min(y0 + r, rows - 1), gc = min(x0 + c, cols - 1);
    if (PASS == 1) {
      s_fx[i] = px.img[(int64_t)gr * cols + gc];
      if (GRAD) s_fy[i] = py.img[(int64_t)gr * cols + gc];
    }
    if (run.mask) s_mk[i] = run.mask[(int64_t)gr * cols + gc];
  }
  __syncthreads();
  const bool need_grads = GRAD && (PASS == 1 || run.mvar == 2);
  if (need_grads) {
    if (KR == 0) {
      for (int i = threadIdx.x; i < WBr * WBc; i += blockDim.x) {
        const int r = i / WBc, c = i - r * WBc;
        s_bl[i] = s_in[r * WIc + c];
      }
    } else {
      for (int i = threadIdx.x; i < WIr * WBc; i += blockDim.x) {
        const int r = i / WBc, c = i - r * WBc;
        const float* q = s_in + r * WIc + c;
        s_hb[i] = (KR == 2) ? (0.0625f * q[0] + 0.25f * q[1] + 0.375f * q[2] + 0.25f * q[3] + 0.0625f * q[4])
                            : (0.25f * q[0] + 0.5f * q[1] + 0.25f * q[2]);
      }
      __syncthreads();
      for (int i = threadIdx.x; i < WBr * WBc; i += blockDim.x) {
        const int r = i / WBc, c = i - r * WBc;
        const float* q = s_hb + r * WBc + c;
        s_bl[i] = (KR == 2) ? (0.0625f * q[0] + 0.25f * q[WBc] + 0.375f * q[2 * WBc] + 0.25f * q[3 * WBc] +
                               0.0625f * q[4 * WBc])
                            : (0.25f * q[0] + 0.5f * q[WBc] + 0.25f * q[2 * WBc]);
      }
    }
    __syncthreads();
    for (int i = threadIdx.x; i < WW; i += blockDim.x) {
      const int r = i / Wc + 1, c = i % Wc + 1;
      const float* q = s_bl;
      const float a = q[(r - 1) * WBc + c - 1], b = q[(r - 1) * WBc + c], cc = q[(r - 1) * WBc + c + 1];
      const float d = q[r * WBc + c - 1], f = q[r * WBc + c + 1];
      const float g = q[(r + 1) * WBc + c - 1], h = q[(r + 1) * WBc + c], ii = q[(r + 1) * WBc + c + 1];
      s_mx[i] = ((cc - a) + 2.0f * (f - d)) + (ii - g);
      s_my[i] = ((g - a) + 2.0f * (h - b)) + (ii - cc);
    }
  }
  __syncthreads();

  FF v[2] = {FF{0.0f, 0.0f}, FF{0.0f, 0.0f}};
  const int lr = threadIdx.x / kPC, lc = threadIdx.x % kPC;
  const int pc = pc0 + lc;
  const int d = 2 * radius + 1;
  const int c0 = lc * stride;
  if (RB > 1) {
    // several unmasked patches per thread, no moving-variance weights (the
    // host picks this form only then); PASS 1 only
    if (PASS == 1 && pc < ncc) {
      int64_t pidx[RB];
      int cnt[RB];
      bool any = false;
#pragma unroll
      for (int j = 0; j < RB; ++j) {
        const int pr = pr0 + lr * RB + j;
        pidx[j] = (int64_t)pr * ncc + pc;
        cnt[j] = pr < ncr ? (run.cnt ? run.cnt[pidx[j]] : 1) : 0;
        any = any || cnt[j] > 0;
      }
      if (any) {
        const int rbase = lr * RB * stride;
        float kept[RB];  // per-patch score as xReg keeps it (0.5 (s_x + s_y) for GRAD)
#pragma unroll
        for (int j = 0; j < RB; ++j) kept[j] = 0.0f;
        for (int k = 0; k < (GRAD ? 2 : 1); ++k) {
          const PatchFixed& P = k == 0 ? px : py;
          float fm[RB], fs[RB], sc[RB], w[RB];
#pragma unroll
          for (int j = 0; j < RB; ++j) {
            fm[j] = cnt[j] > 0 ? P.mean[pidx[j]] : 0.0f;
            fs[j] = cnt[j] > 0 ? P.scale[pidx[j]] : 0.0f;
            w[j] = (cnt[j] > 0 && P.w) ? P.w[pidx[j]] : 1.0f;
          }
          patch_scores_rows<RB, DC, SC>(k == 0 ? s_mx : s_my, k == 0 ? s_fx : s_fy, Wc, rbase, c0, d, stride, fm,
                                        fs, sc);
#pragma unroll
          for (int j = 0; j < RB; ++j)
            if (cnt[j] > 0 && (!run.weighted || fabsf(w[j]) > 1.0e-6f)) {
              v[k] = ff_add(v[k], ff_prod((float)cnt[j], (run.weighted ? w[j] : 1.0f) * sc[j]));
              kept[j] += GRAD ? 0.5f * sc[j] : sc[j];
            }
        }
        if (run.scores)
#pragma unroll
          for (int j = 0; j < RB; ++j)
            if (cnt[j] > 0) run.scores[img * (int64_t)ncr * ncc + pidx[j]] = kept[j];
      }
    }
  } else {
    const int pr = pr0 + lr;
    if (pr < ncr && pc < ncc) {
      const int64_t pidx = (int64_t)pr * ncc + pc;
      const int cnt = run.cnt ? run.cnt[pidx] : 1;
      const int r0 = lr * stride;
      const bool centre = !mk || mk[(r0 + radius) * Wc + c0 + radius];
      if (cnt > 0) {
        // moving-patch variances used as weights: of the moving image itself
        // (mvar 1, shared by both directions) or of each gradient image (mvar 2)
        float var0 = 0.0f, var1 = 0.0f;
        if (run.mvar && centre) {
          if (run.mvar == 1) {
            var0 = GRAD ? patch_var(s_in + H * WIc + H, WIc, r0, c0, d) : patch_var(s_mx, Wc, r0, c0, d);
            var1 = var0;
          } else {
            var0 = patch_var(s_mx, Wc, r0, c0, d);
            if (GRAD) var1 = patch_var(s_my, Wc, r0, c0, d);
          }
        }
        if (PASS == 0) {
          v[0] = ff_prod((float)cnt, var0);
          v[1] = ff_prod((float)cnt, var1);
        } else {
          float w[2];
          for (int k = 0; k < 2; ++k) {
            const PatchFixed& P = k == 0 ? px : py;
            if (run.mvar) {
              float vk = k == 0 ? var0 : var1;
              if (run.normalize) {
                const float S = (float)run.mvar_sum[img * 2 + k];
                vk = S > 1.0e-6f ? vk / S : 0.0f;
              }
              w[k] = vk;
            } else {
              w[k] = P.w ? P.w[pidx] : 1.0f;
            }
          }
          float kept = 0.0f;  // per-patch score as xReg keeps it (0.5 (s_x + s_y) for GRAD)
          if (!run.weighted || fabsf(w[0]) > 1.0e-6f) {
            const float sc = patch_score(s_mx, s_fx, mk, Wc, r0, c0, d, px.mean[pidx], px.scale[pidx],
                                         run.use_mask_stats, run.mask_in_sums);
            v[0] = ff_prod((float)cnt, (run.weighted ? w[0] : 1.0f) * sc);
            kept += GRAD ? 0.5f * sc : sc;
          }
          if (GRAD && (!run.weighted || fabsf(w[1]) > 1.0e-6f)) {
            const float sc = patch_score(s_my, s_fy, mk, Wc, r0, c0, d, py.mean[pidx], py.scale[pidx],
                                         run.use_mask_stats, run.mask_in_sums);
            v[1] = ff_prod((float)cnt, (run.weighted ? w[1] : 1.0f) * sc);
            kept += 0.5f * sc;
          }
          if (run.scores) run.scores[img * (int64_t)ncr * ncc + pidx] = kept;
        }
      }
    }
  }
  double t[2];
  block_sum_ff<2>(v, t, red);
  if (threadIdx.x == 0) {
    double* o = partials + (img * gridDim.x + blockIdx.x) * 2;
    o[0] = t[0];
    o[1] = t[1];
  }
}

// Per image (one block each): the two sums over the blocks' partials.
__device__ __forceinline__ void patch_partials_sum(const double* __restrict__ p, int nblk, double (&v)[2],
                                                   double* red) {
  v[0] = 0.0;
  v[1] = 0.0;
  for (int k = threadIdx.x; k < nblk; k += blockDim.x) {
    v[0] += p[2 * k];
    v[1] += p[2 * k + 1];
  }
  block_sum_d<2>(v, red);
}

__global__ void patch_sum_partials_kernel(const double* __restrict__ partials, int nblk, double* __restrict__ out) {
  __shared__ double red[2 * 32];
  const int64_t img = blockIdx.x;
  double v[2];
  patch_partials_sum(partials + img * nblk * 2, nblk, v, red);
  if (threadIdx.x == 0) {
    out[img * 2] = v[0];
    out[img * 2 + 1] = v[1];
  }
}

// Value per image: sum / denominator per direction; FLT_MAX where normalised
// moving variances sum to at most 1e-6; patch grad-NCC 0.5 (s_x + s_y) in float.
__global__ void patch_finalize_kernel(const double* __restrict__ partials, int nblk, double den_x, double den_y,
                                      int grad, int mvar, int normalize, const double* __restrict__ mvar_sum,
                                      float* __restrict__ sims) {
  __shared__ double red[2 * 32];
  const int64_t img = blockIdx.x;
  double v[2];
  patch_partials_sum(partials + img * nblk * 2, nblk, v, red);
  if (threadIdx.x != 0) return;
  const bool chk = mvar && normalize;
  if (chk && mvar == 1 && !((float)mvar_sum[img * 2] > 1.0e-6f)) {
    sims[img] = FLT_MAX;
    return;
  }
  const float sx = (chk && !((float)mvar_sum[img * 2] > 1.0e-6f)) ? FLT_MAX : (float)(v[0] / den_x);
  if (grad) {
    const float sy = (chk && !((float)mvar_sum[img * 2 + 1] > 1.0e-6f)) ? FLT_MAX : (float)(v[1] / den_y);
    sims[img] = 0.5f * (sx + sy);
  } else {
    sims[img] = sx;
  }
}

// cnt[idx[k]] += 1 for k < n (patch multiplicities of a drawn subset).
__global__ void patch_scatter_counts_kernel(const int32_t* __restrict__ idx, int64_t n, int32_t* __restrict__ cnt) {
  const int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (k < n) atomicAdd(cnt + idx[k], 1);
}

struct ViewPtrs {
  const float* p[16];
};

__global__ void combine_mean_kernel(ViewPtrs vp, int nviews, int64_t pop, float* __restrict__ out) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= pop) return;
  out[i] = gt::combine_mean(vp.p, nviews, i, false);
}

template <typename K>
cudaError_t set_smem(K kern, size_t bytes) {
  // above the default 48 KB the kernel must opt in; the kernels' own static
  // shared memory counts against the same 48 KB, so opt in with room to spare
  if (bytes > 40 * 1024) return cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bytes);
  return cudaSuccess;
}

}  // namespace

cudaError_t launch_image_stats(const float* img, int64_t npix, const uint8_t* mask, double* d_out, cudaStream_t s) {
  image_sum_kernel<<<1, 1024, 0, s>>>(img, npix, mask, d_out);
  image_var_kernel<<<1, 1024, 0, s>>>(img, npix, mask, d_out);
  return cudaGetLastError();
}

cudaError_t launch_sum_f(const float* in, int64_t n, const uint8_t* mask, double* d_out, cudaStream_t s) {
  image_sum_kernel<<<1, 1024, 0, s>>>(in, n, mask, d_out);
  return cudaGetLastError();
}

cudaError_t launch_sub_scalar(const float* in, int64_t n, double value, float* out, cudaStream_t s) {
  const int blocks = (int)((n + 255) / 256 < 4096 ? (n + 255) / 256 : 4096);
  sub_scalar_kernel<<<blocks > 0 ? blocks : 1, 256, 0, s>>>(in, n, (float)value, out);
  return cudaGetLastError();
}

cudaError_t launch_ncc_moments(const float* mov, int64_t npix, int64_t nimgs, const float* fhat,
                               const uint8_t* mask, double* partials, int nblk, cudaStream_t s) {
  if (nimgs <= 0) return cudaSuccess;
  const dim3 grid(nblk, (unsigned)nimgs);
  ncc_moments_kernel<<<grid, kThreads, 0, s>>>(mov, npix, fhat, mask, partials);
  return cudaGetLastError();
}

cudaError_t launch_ncc_finalize(const double* partials, int nblk, int64_t nimgs, int64_t n_used, FixedNCC fx,
                                float* sims, cudaStream_t s) {
  if (nimgs <= 0) return cudaSuccess;
  ncc_finalize_kernel<<<(unsigned)nimgs, 128, 0, s>>>(partials, nblk, nimgs, (double)n_used, fx, sims);
  return cudaGetLastError();
}

cudaError_t launch_grad_images(const float* img, int rows, int cols, int64_t nimgs, int smooth_ksize, float* gx,
                               float* gy, cudaStream_t s) {
  const int tiles = ((rows + kT - 1) / kT) * ((cols + kT - 1) / kT);
  const dim3 grid(tiles, (unsigned)nimgs);
  switch (smooth_ksize) {
    case 0: grad_images_kernel<0><<<grid, kThreads, 0, s>>>(img, rows, cols, gx, gy); break;
    case 3: grad_images_kernel<1><<<grid, kThreads, 0, s>>>(img, rows, cols, gx, gy); break;
    case 5: grad_images_kernel<2><<<grid, kThreads, 0, s>>>(img, rows, cols, gx, gy); break;
    default: return cudaErrorInvalidValue;
  }
  return cudaGetLastError();
}

cudaError_t launch_grad_moments(const float* mov, int rows, int cols, int64_t nimgs, int smooth_ksize,
                                const float* fhat_x, const float* fhat_y, const uint8_t* mask, double* partials,
                                cudaStream_t s, int* nblk_out) {
  const int tiles = ((rows + kGH - 1) / kGH) * ((cols + kGW - 1) / kGW);
  if (nblk_out) *nblk_out = tiles;
  if (nimgs <= 0 || !partials) return cudaSuccess;
  const dim3 grid(tiles, (unsigned)nimgs);
  switch (smooth_ksize) {
    case 0: grad_moments_kernel<0><<<grid, kThreads, 0, s>>>(mov, rows, cols, fhat_x, fhat_y, mask, partials); break;
    case 3: grad_moments_kernel<1><<<grid, kThreads, 0, s>>>(mov, rows, cols, fhat_x, fhat_y, mask, partials); break;
    case 5: grad_moments_kernel<2><<<grid, kThreads, 0, s>>>(mov, rows, cols, fhat_x, fhat_y, mask, partials); break;
    default: return cudaErrorInvalidValue;
  }
  return cudaGetLastError();
}

cudaError_t launch_grad_multi(const FusedJob* d_jobs, int njobs, long long total, cudaStream_t s) {
  if (total <= 0) return cudaSuccess;
  int dev = 0, sms = 0, per_sm = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e == cudaSuccess) e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  if (e == cudaSuccess) e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, grad_multi_kernel, kThreads, 0);
  if (e != cudaSuccess) return e;
  const long long cap = (long long)sms * (per_sm > 0 ? per_sm : 1);
  grad_multi_kernel<<<(unsigned)(total < cap ? total : cap), kThreads, 0, s>>>(d_jobs, njobs, total);
  return cudaGetLastError();
}

cudaError_t launch_cma_updates(const CmaUpdateJob* d_jobs, int njobs, cudaStream_t s) {
  if (njobs <= 0) return cudaSuccess;
  cma_update_kernel<<<(unsigned)njobs, 128, 0, s>>>(d_jobs);
  return cudaGetLastError();
}

cudaError_t launch_grad_finalize(const double* partials, int nblk, int64_t nimgs, int64_t n_used, FixedNCC fx,
                                 FixedNCC fy, float* sims, cudaStream_t s) {
  if (nimgs <= 0) return cudaSuccess;
  grad_finalize_kernel<<<(unsigned)nimgs, 128, 0, s>>>(partials, nblk, nimgs, (double)n_used, fx, fy, sims);
  return cudaGetLastError();
}

cudaError_t launch_patch_fixed_stats(const float* img, int rows, int cols, int radius, int stride, int ncr, int ncc,
                                     const uint8_t* mask, int use_mask_stats, float* mean, float* scale, float* wvar,
                                     int* ucount, cudaStream_t s) {
  (void)rows;
  const int64_t n = (int64_t)ncr * ncc;
  if (n <= 0) return cudaSuccess;
  patch_fixed_stats_kernel<<<(unsigned)((n + 127) / 128), 128, 0, s>>>(img, cols, radius, stride, ncr, ncc, mask,
                                                                       use_mask_stats, mean, scale, wvar, ucount);
  return cudaGetLastError();
}

// Patches scored per thread: four stacked in a column when no mask and no
// moving-variance weight is involved and the taller tile fits, else one.
constexpr int kPatchRows = 4;
static int patch_rb(int radius, int stride, int grad, int kr, const PatchRun& run) {
  if (run.mask || run.mvar) return 1;
  return PatchLayout::make(radius, stride, grad, kr, kPatchRows).bytes <= 112 * 1024 ? kPatchRows : 1;
}

static int patch_tiles(int ncr, int ncc, int rb) {
  return ((ncr + kPC * rb - 1) / (kPC * rb)) * ((ncc + kPC - 1) / kPC);
}

int patch_ncc_max_blocks(int ncr, int ncc) { return patch_tiles(ncr, ncc, 1); }

cudaError_t launch_patch_ncc(const float* mov, int rows, int cols, int64_t nimgs, int grad, int smooth_ksize,
                             int radius, int stride, int ncr, int ncc, PatchFixed px, PatchFixed py, PatchRun run,
                             int pass, double* partials, cudaStream_t s, int* nblk_out) {
  const int kr = smooth_ksize == 5 ? 2 : (smooth_ksize == 3 ? 1 : 0);
  if (smooth_ksize != 0 && smooth_ksize != 3 && smooth_ksize != 5) return cudaErrorInvalidValue;
  const int rb = patch_rb(radius, stride, grad, kr, run);
  const int tiles = patch_tiles(ncr, ncc, rb);
  if (nblk_out) *nblk_out = tiles;
  if (nimgs <= 0 || !partials) return cudaSuccess;
  if (rb > 1 && pass != 1) return cudaErrorInvalidValue;
  const PatchLayout L = PatchLayout::make(radius, stride, grad, kr, rb);
  if (L.bytes > 200 * 1024) return cudaErrorInvalidValue;
  const dim3 grid(tiles, (unsigned)nimgs);
  cudaError_t e = cudaSuccess;
#define XR_PATCH_R4_11_1 kPatchRows, 11, 1  // xReg's default patches: 11 x 11, stride 1
#define XR_PATCH_LAUNCH(G, K, P, ...)                                                                        \
  e = set_smem(patch_ncc_kernel<G, K, P, __VA_ARGS__>, L.bytes);                                            \
  if (e != cudaSuccess) return e;                                                                            \
  patch_ncc_kernel<G, K, P, __VA_ARGS__><<<grid, kThreads, L.bytes, s>>>(mov, rows, cols, radius, stride, ncr, ncc, \
                                                                         px, py, run, partials);
#define XR_PATCH_PASS(G, K)                                   \
  if (rb > 1 && radius == 5 && stride == 1) {                 \
    XR_PATCH_LAUNCH(G, K, 1, XR_PATCH_R4_11_1)                \
  } else if (rb > 1) {                                        \
    XR_PATCH_LAUNCH(G, K, 1, kPatchRows)                      \
  } else if (pass == 0) {                                     \
    XR_PATCH_LAUNCH(G, K, 0, 1)                               \
  } else {                                                    \
    XR_PATCH_LAUNCH(G, K, 1, 1)                               \
  }
  if (!grad) {
    XR_PATCH_PASS(0, 0)
  } else if (kr == 0) {
    XR_PATCH_PASS(1, 0)
  } else if (kr == 1) {
    XR_PATCH_PASS(1, 1)
  } else {
    XR_PATCH_PASS(1, 2)
  }
#undef XR_PATCH_PASS
#undef XR_PATCH_LAUNCH
#undef XR_PATCH_R4_11_1
  return cudaGetLastError();
}

cudaError_t launch_patch_sum_partials(const double* partials, int nblk, int64_t nimgs, double* out, cudaStream_t s) {
  if (nimgs <= 0) return cudaSuccess;
  patch_sum_partials_kernel<<<(unsigned)nimgs, 256, 0, s>>>(partials, nblk, out);
  return cudaGetLastError();
}

cudaError_t launch_patch_finalize(const double* partials, int nblk, int64_t nimgs, double den_x, double den_y,
                                  int grad, int mvar, int normalize, const double* mvar_sum, float* sims,
                                  cudaStream_t s) {
  if (nimgs <= 0) return cudaSuccess;
  patch_finalize_kernel<<<(unsigned)nimgs, 256, 0, s>>>(partials, nblk, den_x, den_y, grad, mvar, normalize,
                                                       mvar_sum, sims);
  return cudaGetLastError();
}

cudaError_t launch_patch_scatter_counts(const int32_t* idx, int64_t n, int32_t* cnt, cudaStream_t s) {
  if (n <= 0) return cudaSuccess;
  patch_scatter_counts_kernel<<<(unsigned)((n + 127) / 128), 128, 0, s>>>(idx, n, cnt);
  return cudaGetLastError();
}

cudaError_t launch_combine_mean(const float* const* view_sims, int nviews, int64_t pop, float* out, cudaStream_t s) {
  if (nviews < 1 || nviews > 16) return cudaErrorInvalidValue;
  ViewPtrs vp;
  for (int v = 0; v < 16; ++v) vp.p[v] = v < nviews ? view_sims[v] : nullptr;
  combine_mean_kernel<<<(unsigned)((pop + 127) / 128), 128, 0, s>>>(vp, nviews, pop, out);
  return cudaGetLastError();
}

}  // namespace xr
