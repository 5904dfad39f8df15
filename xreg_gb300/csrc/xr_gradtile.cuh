// xr_gradtile.cuh -- device code shared by the split grad-NCC metric kernels
// (xr_metrics.cu) and the fused evaluation kernel (xr_raycast.cu): compensated
// reductions, the moments of one 32 x 64-pixel tile of a moving image's
// gradients, and the per-image FP64 combine.  Both paths run exactly this code
// on the same tiles, so their similarity values are identical bit for bit.
//
// Gradients (xregImgSimMetric2DGradImgCPU.cpp:48-65,86-101): OpenCV's sigma-0
// Gaussian [1 4 6 4 1]/16 (or [1 2 1]/4), then the 3x3 Sobel in x and y, with
// BORDER_REFLECT_101; NCC of each direction (xregImgSimMetric2DNCCCPU.cpp:
// 53-63,164-209), sim = 0.5 (s_x + s_y) (xregImgSimMetric2DGradNCCCPU.cpp:51-65).
#pragma once

#include "xr_internal.h"

namespace xr {
namespace gt {

constexpr int kThreads = 256;                     // block size of every tile kernel
constexpr int kGW = 32;                           // tile columns = threads across
constexpr int kGR = 8;                            // rows per thread
constexpr int kGH = kGR * (kThreads / kGW);       // tile rows (64)
constexpr int kFinalizeThreads = 128;             // threads of the per-image combine

__device__ __forceinline__ int reflect101(int i, int n) {
  if (i < 0) i = -i;
  if (i >= n) i = 2 * (n - 1) - i;
  return i;
}

// A float-float value hi + lo (about 48 significant bits).
struct FF {
  float hi, lo;
};

// Knuth's two-sum on the FP32 pipe for float-float values: this GPU's FP64 pipe
// is slow enough that block reductions in double kept it 82 % busy and bounded
// the grad-NCC moment kernel.  Explicit _rn intrinsics keep every step unfused.
__device__ __forceinline__ FF ff_add(FF a, FF b) {
  const float s = __fadd_rn(a.hi, b.hi);
  const float bb = __fsub_rn(s, a.hi);
  float e = __fadd_rn(__fsub_rn(a.hi, __fsub_rn(s, bb)), __fsub_rn(b.hi, bb));  // s + e = a.hi + b.hi exactly
  e = __fadd_rn(e, __fadd_rn(a.lo, b.lo));
  const float hi = __fadd_rn(s, e);
  return FF{hi, __fsub_rn(e, __fsub_rn(hi, s))};
}

// a b exactly as a float-float (the rounding error of the product from one fma).
__device__ __forceinline__ FF ff_prod(float a, float b) {
  const float p = __fmul_rn(a, b);
  return FF{p, fmaf(a, b, -p)};
}

__device__ __forceinline__ FF ff_shfl_down(FF v, int o) {
  return FF{__shfl_down_sync(0xffffffffu, v.hi, o), __shfl_down_sync(0xffffffffu, v.lo, o)};
}

// Blur and Sobel arithmetic with every rounding explicit (no contraction), so
// the shared-memory and the register forms of the tile give the same bits.
__device__ __forceinline__ float blur5(float a, float b, float c, float d, float e) {
  return __fadd_rn(__fadd_rn(__fadd_rn(__fadd_rn(__fmul_rn(0.0625f, a), __fmul_rn(0.25f, b)), __fmul_rn(0.375f, c)),
                             __fmul_rn(0.25f, d)),
                   __fmul_rn(0.0625f, e));
}
__device__ __forceinline__ float blur3(float a, float b, float c) {
  return __fadd_rn(__fadd_rn(__fmul_rn(0.25f, a), __fmul_rn(0.5f, b)), __fmul_rn(0.25f, c));
}
// Sobel at the centre of the blurred 3x3 neighbourhood a0 b0 c0 / a1 . c1 / a2 b2 c2
__device__ __forceinline__ void sobel3(float a0, float b0, float c0, float a1, float c1, float a2, float b2, float c2,
                                       float& gx, float& gy) {
  gx = __fadd_rn(__fadd_rn(__fsub_rn(c0, a0), __fmul_rn(2.0f, __fsub_rn(c1, a1))), __fsub_rn(c2, a2));
  gy = __fadd_rn(__fadd_rn(__fsub_rn(a2, a0), __fmul_rn(2.0f, __fsub_rn(b2, b0))), __fsub_rn(c2, c0));
}
// One pixel's contribution to the six moments.
__device__ __forceinline__ void moments_add(float (&m)[6], float gx, float gy, float fx, float fy) {
  m[0] = __fadd_rn(m[0], gx);
  m[1] = __fmaf_rn(gx, gx, m[1]);
  m[2] = __fmaf_rn(gx, fx, m[2]);
  m[3] = __fadd_rn(m[3], gy);
  m[4] = __fmaf_rn(gy, gy, m[4]);
  m[5] = __fmaf_rn(gy, fy, m[5]);
}

__device__ __forceinline__ double warp_sum_d(double v) {
  for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
  return v;
}

// Block-wide sum of K doubles per thread over the first nw warps (the others
// must hold zeros); result valid in thread 0.
template <int K>
__device__ __forceinline__ void block_sum_d(double (&v)[K], double* red /* [K][32] */, int nw) {
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
#pragma unroll
  for (int k = 0; k < K; ++k) {
    const double w = warp_sum_d(v[k]);
    if (lane == 0 && warp < nw) red[k * 32 + warp] = w;
  }
  __syncthreads();
  if (warp == 0) {
#pragma unroll
    for (int k = 0; k < K; ++k) {
      double w = (lane < nw) ? red[k * 32 + lane] : 0.0;
      w = warp_sum_d(w);
      v[k] = w;
    }
  }
}

__device__ __forceinline__ double ncc_sim_from_moments(double sm, double smm, double smf, double n,
                                                       const FixedNCC& fx) {
  const double mean = sm / n;
  double var = (smm - n * mean * mean) / (n - 1.0);
  if (var < 0.0) var = 0.0;
  double sd = sqrt(var);
  if (sd < 1.0e-6) sd = 1.0e-6;
  const double cov = smf - mean * fx.sum_fhat;
  const double ncc = cov / (n * fx.sd * sd);
  return (1.0 - ncc) * 0.5;
}

// Shared memory of one tile: the horizontally blurred rows, blurred in place
// down the columns (the vertical pass reads every input before it writes).
template <int KR>
struct GradTileSmem {
  static constexpr int H = KR + 1;                // halo: blur radius + Sobel
  static constexpr int WI = kGW + 2 * H, HI = kGH + 2 * H;
  static constexpr int WB = kGW + 2, HB = kGH + 2;
  float hb[HI][WB + 1];
  FF red[6 * (kThreads / 32)];
};

// The tile's six moments from every thread's partial sums: plain float within
// a warp (256 pixels), float-float across the warps (red: [6][8]); v valid in
// thread 0.
__device__ __forceinline__ void tile_moments_reduce(const float (&m)[6], FF* red, double (&v)[6]) {
  constexpr int kWarps = kThreads / 32;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
#pragma unroll
  for (int k = 0; k < 6; ++k) {
    float w = m[k];
    for (int o = 16; o > 0; o >>= 1) w = __fadd_rn(w, __shfl_down_sync(0xffffffffu, w, o));
    if (lane == 0) red[k * kWarps + warp] = FF{w, 0.0f};
  }
  __syncthreads();
  if (warp == 0) {
#pragma unroll
    for (int k = 0; k < 6; ++k) {
      FF w = (lane < kWarps) ? red[k * kWarps + lane] : FF{0.0f, 0.0f};
      for (int o = 16; o > 0; o >>= 1) w = ff_add(w, ff_shfl_down(w, o));
      v[k] = (double)w.hi + (double)w.lo;
    }
  }
  __syncthreads();  // red (and the tile's shared memory) is reused by the caller's next tile
}

// Image pixel (row, col) of a tile's input; CG reads through L2 only (pixels
// written earlier in the same kernel by other blocks).
template <bool CG>
__device__ __forceinline__ float tile_px(const float* __restrict__ src, int cols, int gr, int gc) {
  const float* p = src + (int64_t)gr * cols + gc;
  return CG ? __ldcg(p) : __ldg(p);
}

// Moments of the moving gradients over the 32 x 64-pixel tile at (y0, x0),
// 256 threads: each thread owns one column and eight consecutive rows, so the
// Sobel stencil slides down the column; sums are plain float per thread (8
// terms) and per warp (256 pixels), float-float across the warps.  v (valid in
// thread 0): S_gx, S_gx^2, S_gx fx, S_gy, S_gy^2, S_gy fy.
template <int KR, bool CG>
__device__ void grad_tile_moments(const float* __restrict__ src, int rows, int cols, int y0, int x0,
                                  const float* __restrict__ fhx, const float* __restrict__ fhy,
                                  const uint8_t* __restrict__ mask, GradTileSmem<KR>& sm, double (&v)[6]) {
  using S = GradTileSmem<KR>;
  constexpr int H = S::H, HI = S::HI, WB = S::WB, HB = S::HB;
  const int tx = threadIdx.x % kGW, ty = threadIdx.x / kGW;
  // Rows / cols past the last tile pixel only feed pixels that are skipped;
  // clamping before the reflection keeps every read inside the image.
  const bool interior = y0 >= H && x0 >= H && y0 + kGH + H <= rows && x0 + kGW + H <= cols;
  auto in = [&](int r, int c) -> float {
    int gr = y0 - H + r, gc = x0 - H + c;
    if (!interior) {
      gr = reflect101(min(gr, rows - 1 + H), rows);
      gc = reflect101(min(gc, cols - 1 + H), cols);
    }
    return tile_px<CG>(src, cols, gr, gc);
  };
  if constexpr (KR == 0) {
    for (int i = threadIdx.x; i < HB * WB; i += kThreads) {
      const int r = i / WB, c = i - r * WB;
      sm.hb[r][c] = in(r, c);
    }
  } else {
    // horizontal pass over all input rows, blurred columns [x0-1, x0+kGW+1)
    for (int i = threadIdx.x; i < HI * WB; i += kThreads) {
      const int r = i / WB, c = i - r * WB;
      sm.hb[r][c] = (KR == 2) ? blur5(in(r, c), in(r, c + 1), in(r, c + 2), in(r, c + 3), in(r, c + 4))
                              : blur3(in(r, c), in(r, c + 1), in(r, c + 2));
    }
    __syncthreads();
    // vertical pass in place: WB columns x 4 chunks of rows, every output of a
    // chunk computed before the barrier, written after it
    constexpr int kChunks = 4, kCh = (HB + kChunks - 1) / kChunks;
    const int c = threadIdx.x % WB, j = threadIdx.x / WB;
    float o[kCh];
    if (j < kChunks) {
#pragma unroll
      for (int k = 0; k < kCh; ++k) {
        const int r = j * kCh + k;
        if (r < HB)
          o[k] = (KR == 2) ? blur5(sm.hb[r][c], sm.hb[r + 1][c], sm.hb[r + 2][c], sm.hb[r + 3][c], sm.hb[r + 4][c])
                           : blur3(sm.hb[r][c], sm.hb[r + 1][c], sm.hb[r + 2][c]);
      }
    }
    __syncthreads();
    if (j < kChunks) {
#pragma unroll
      for (int k = 0; k < kCh; ++k) {
        const int r = j * kCh + k;
        if (r < HB) sm.hb[r][c] = o[k];
      }
    }
  }
  __syncthreads();
  const auto& bl = sm.hb;  // blurred region [HB][WB]
  float m[6] = {0.0f, 0.0f, 0.0f, 0.0f, 0.0f, 0.0f};
  const int gxc = x0 + tx;
  if (gxc < cols) {
    const int rb = ty * kGR;  // first output row (tile-local); blurred rows rb .. rb + kGR + 1
    float a0 = bl[rb][tx], b0 = bl[rb][tx + 1], c0 = bl[rb][tx + 2];
    float a1 = bl[rb + 1][tx], b1 = bl[rb + 1][tx + 1], c1 = bl[rb + 1][tx + 2];
#pragma unroll
    for (int k = 0; k < kGR; ++k) {
      const float a2 = bl[rb + k + 2][tx], b2 = bl[rb + k + 2][tx + 1], c2 = bl[rb + k + 2][tx + 2];
      const int gyr = y0 + rb + k;
      if (gyr < rows) {
        const int64_t pix = (int64_t)gyr * cols + gxc;
        if (!mask || mask[pix]) {
          float gx, gy;
          sobel3(a0, b0, c0, a1, c1, a2, b2, c2, gx, gy);
          moments_add(m, gx, gy, fhx[pix], fhy[pix]);
        }
      }
      a0 = a1; b0 = b1; c0 = c1;
      a1 = a2; b1 = b2; c1 = c2;
    }
  }
  tile_moments_reduce(m, sm.red, v);
}

// The same moments with the 5x5 blur (KR = 2) computed in registers, without
// the tile's shared-memory rows: each thread streams down its rows (plus the
// halo), keeping the last five horizontally blurred rows and the last three
// blurred rows of the three columns its Sobel stencil reads; reads go through
// L2 only.  Every value comes from the same operations as in
// grad_tile_moments, so the moments are identical bit for bit; red: [6][8].
__device__ inline void grad_tile_moments_regs5(const float* __restrict__ src, int rows, int cols, int y0, int x0,
                                               const float* __restrict__ fhx, const float* __restrict__ fhy,
                                               const uint8_t* __restrict__ mask, FF* red, double (&v)[6]) {
  constexpr int H = 3;
  const int tx = threadIdx.x % kGW, ty = threadIdx.x / kGW;
  const bool interior = y0 >= H && x0 >= H && y0 + kGH + H <= rows && x0 + kGW + H <= cols;
  auto in = [&](int r, int c) -> float {  // tile input coordinates, as grad_tile_moments
    int gr = y0 - H + r, gc = x0 - H + c;
    if (!interior) {
      gr = reflect101(min(gr, rows - 1 + H), rows);
      gc = reflect101(min(gc, cols - 1 + H), cols);
    }
    return __ldcg(src + (int64_t)gr * cols + gc);
  };
  float m[6] = {0.0f, 0.0f, 0.0f, 0.0f, 0.0f, 0.0f};
  const int gxc = x0 + tx;
  if (gxc < cols) {
    const int rb = ty * kGR;
    // horizontally blurred rows r-4 .. r and blurred rows q-2 .. q of columns
    // tx .. tx + 2 (zero until filled: the first iterations shift them in)
    float h[5][3] = {}, b[3][3] = {};
#pragma unroll 1
    for (int r = 0; r < kGR + 6; ++r) {
#pragma unroll
      for (int i = 0; i < 4; ++i)
#pragma unroll
        for (int j = 0; j < 3; ++j) h[i][j] = h[i + 1][j];
#pragma unroll
      for (int j = 0; j < 3; ++j)
        h[4][j] = blur5(in(rb + r, tx + j), in(rb + r, tx + j + 1), in(rb + r, tx + j + 2), in(rb + r, tx + j + 3),
                        in(rb + r, tx + j + 4));
      if (r >= 4) {  // blurred row rb + r - 4
#pragma unroll
        for (int j = 0; j < 3; ++j) {
          b[0][j] = b[1][j];
          b[1][j] = b[2][j];
          b[2][j] = blur5(h[0][j], h[1][j], h[2][j], h[3][j], h[4][j]);
        }
        if (r >= 6) {  // output row rb + r - 6 from blurred rows r - 6 .. r - 4
          const int gyr = y0 + rb + r - 6;
          if (gyr < rows) {
            const int64_t pix = (int64_t)gyr * cols + gxc;
            if (!mask || mask[pix]) {
              float gx, gy;
              sobel3(b[0][0], b[0][1], b[0][2], b[1][0], b[1][2], b[2][0], b[2][1], b[2][2], gx, gy);
              moments_add(m, gx, gy, fhx[pix], fhy[pix]);
            }
          }
        }
      }
    }
  }
  tile_moments_reduce(m, red, v);
}

// Per-image combine: the tile partials (nblk x 6 doubles, read through L2 when
// CG) summed by the first kFinalizeThreads threads with that stride, then
// across their warps; the similarity value (valid in thread 0).
template <bool CG>
__device__ float grad_finalize_image(const double* __restrict__ p, int nblk, double n, const FixedNCC& fx,
                                     const FixedNCC& fy, double* red /* [6][4] */) {
  constexpr int kW = kFinalizeThreads / 32;
  double a[6] = {0, 0, 0, 0, 0, 0};
  if (threadIdx.x < kFinalizeThreads)
    for (int k = threadIdx.x; k < nblk; k += kFinalizeThreads)
      for (int j = 0; j < 6; ++j) a[j] = __dadd_rn(a[j], CG ? __ldcg(p + 6 * k + j) : p[6 * k + j]);
  {
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
#pragma unroll
    for (int k = 0; k < 6; ++k) {
      const double w = warp_sum_d(a[k]);
      if (lane == 0 && warp < kW) red[k * kW + warp] = w;
    }
    __syncthreads();
    if (warp == 0) {
#pragma unroll
      for (int k = 0; k < 6; ++k) a[k] = warp_sum_d((lane < kW) ? red[k * kW + lane] : 0.0);
    }
  }
  float out = 0.0f;
  if (threadIdx.x == 0) {
    const double sx = ncc_sim_from_moments(a[0], a[1], a[2], n, fx);
    const double sy = ncc_sim_from_moments(a[3], a[4], a[5], n, fy);
    // 0.5 * (float(s_x) + float(s_y)) as in ImgSimMetric2DGradNCCCPU::compute
    out = 0.5f * ((float)sx + (float)sy);
  }
  __syncthreads();  // red is reused
  return out;
}

// Mean over views of one candidate's values (ImgSimMetric2DCombineMean,
// xregImgSimMetric2DCombine.cpp:79-96).
__device__ __forceinline__ float combine_mean(const float* const* view_sims, int nviews, int64_t i, bool cg) {
  float s = 0.0f;
  for (int v = 0; v < nviews; ++v) s += cg ? __ldcg(view_sims[v] + i) : view_sims[v][i];
  return s / (float)nviews;
}

}  // namespace gt
}  // namespace xr
