// xr_raycast.cu -- line-integral DRR kernels (one thread per detector ray).
//
// Semantics follow RayCasterLineIntCPU (xregRayCastLineIntCPU.cpp:106-290):
//   * ray from the pinhole to the detector pixel, clipped against the index
//     box [0, n-1]^3 with the segment-limited slab test
//     (xregSpatialPrimitives.cpp:176-221);
//   * if the clipped parameter interval is longer than 2e-3, both ends move
//     1e-3 inward (segment-parameter units, xregRayCastLineIntCPU.cpp:233-236);
//   * floor(len_mm / step) + 1 samples, positions advanced by repeated addition
//     of the step vector (:253-277);
//   * software trilinear interpolation with ITK's boundary rule (a neighbour
//     past the last index keeps no weight), never texture filtering;
//   * ray sum (or max) times the step in mm (:279); replace / accumulate /
//     background images as in RayCasterCPU::pre_compute (xregRayCastBaseCPU.cpp:128-158).
//
// The per-ray geometry (direction, slab test, nudge, step count, start point,
// step vector) uses explicitly rounded float intrinsics in the same order as the
// CPU oracle, so sample counts are bit-identical.  The interpolation and the sum
// use ordinary float arithmetic (FMA allowed).
#include "xr_internal.h"

#include <cfloat>

namespace xr {
namespace {

template <int VT>
struct Vox;
template <>
struct Vox<XR_VOXEL_F32> {
  __device__ __forceinline__ static float ld(const void* b, int i) {
    return __ldg(static_cast<const float*>(b) + i);
  }
};
template <>
struct Vox<XR_VOXEL_F16> {
  __device__ __forceinline__ static float ld(const void* b, int i) {
    return __half2float(__ldg(static_cast<const __half*>(b) + i));
  }
};
template <>
struct Vox<XR_VOXEL_BF16> {
  __device__ __forceinline__ static float ld(const void* b, int i) {
    return __bfloat162float(__ldg(static_cast<const __nv_bfloat16*>(b) + i));
  }
};

constexpr int kTileX = 16;
constexpr int kTileY = 16;
constexpr int kThreads = 256;

template <int VT, int KERNEL>
__global__ void __launch_bounds__(kThreads) drr_kernel(const DrrParams p, const int64_t proj_base) {
  // 16 x 16 pixels per block; each warp covers an 8 x 4 patch so the 32 rays of
  // a warp stay close together inside the volume.
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int col = blockIdx.x * kTileX + (warp & 1) * 8 + (lane & 7);
  const int row = blockIdx.y * kTileY + (warp >> 1) * 4 + (lane >> 3);
  const int64_t proj = proj_base + blockIdx.z;
  const bool active = (col < p.cols) && (row < p.rows);

  float sum = (KERNEL == XR_LINE_INT_MAX) ? -FLT_MAX : 0.0f;
  unsigned long long ns = 0;
  if (active) {
    const ProjGeom& g = p.geo[proj];
    const float fc = (float)col, fr = (float)row;
    float dir[3], v[3], src[3];
#pragma unroll
    for (int k = 0; k < 3; ++k) {
      src[k] = g.src[k];
      dir[k] = __fadd_rn(__fadd_rn(g.d0[k], __fmul_rn(fc, g.dc[k])), __fmul_rn(fr, g.dr[k]));
      v[k] = __fadd_rn(__fadd_rn(g.e0[k], __fmul_rn(fc, g.ec[k])), __fmul_rn(fr, g.er[k]));
    }
    const float maxb[3] = {(float)(p.vol.nx - 1), (float)(p.vol.ny - 1), (float)(p.vol.nz - 1)};
    bool hit = true;
    float t0 = 0.0f, t1 = 1.0f;
#pragma unroll
    for (int k = 0; k < 3; ++k) {
      if (!hit) break;
      if ((double)fabsf(dir[k]) > 1.0e-8) {
        const float inv = __frcp_rn(dir[k]);
        float ta = __fmul_rn(__fsub_rn(0.0f, src[k]), inv);
        float tb = __fmul_rn(__fsub_rn(maxb[k], src[k]), inv);
        if (tb < ta) { const float tmp = ta; ta = tb; tb = tmp; }
        t0 = (t0 < ta) ? ta : t0;
        t1 = (tb < t1) ? tb : t1;
        if (t0 > t1) hit = false;
      } else if (src[k] < 0.0f || src[k] > maxb[k]) {
        hit = false;
      }
    }
    if (hit && (__fsub_rn(t1, t0) > 2.0e-3f)) {
      t0 = __fadd_rn(t0, 1.0e-3f);
      t1 = __fsub_rn(t1, 1.0e-3f);
      float px = __fadd_rn(src[0], __fmul_rn(t0, dir[0]));
      float py = __fadd_rn(src[1], __fmul_rn(t0, dir[1]));
      float pz = __fadd_rn(src[2], __fmul_rn(t0, dir[2]));
      const float lc = __fsqrt_rn(__fadd_rn(__fadd_rn(__fmul_rn(v[0], v[0]), __fmul_rn(v[1], v[1])),
                                            __fmul_rn(v[2], v[2])));
      const float len = __fmul_rn(__fsub_rn(t1, t0), lc);
      unsigned long long nsteps = (unsigned long long)__fdiv_rn(len, p.step);
      if (!(nsteps <= p.max_steps)) {
        // A ray longer than the volume diagonal allows can only come from a
        // non-finite or degenerate pose: count it and leave the pixel unsampled
        // rather than loop for an unbounded time.
        atomicAdd(p.err_counter, 1u);
        nsteps = 0;
        hit = false;
      }
      const float sc = __fdiv_rn(p.step, lc);
      const float sx = __fmul_rn(dir[0], sc), sy = __fmul_rn(dir[1], sc), sz = __fmul_rn(dir[2], sc);

      const int nx = p.vol.nx, ny = p.vol.ny, nz = p.vol.nz;
      const int sy_ = nx, sz_ = nx * ny;
      const float bx = maxb[0], by = maxb[1], bz = maxb[2];
      const void* vox = p.vol.voxels;
      for (unsigned long long s = 0; hit && s <= nsteps; ++s) {
        const float x = fminf(fmaxf(px, 0.0f), bx);
        const float y = fminf(fmaxf(py, 0.0f), by);
        const float z = fminf(fmaxf(pz, 0.0f), bz);
        const int ix = min(__float2int_rd(x), nx - 2);
        const int iy = min(__float2int_rd(y), ny - 2);
        const int iz = min(__float2int_rd(z), nz - 2);
        const float fx = x - (float)ix, fy = y - (float)iy, fz = z - (float)iz;
        const int b = (iz * ny + iy) * nx + ix;
        const float v000 = Vox<VT>::ld(vox, b), v100 = Vox<VT>::ld(vox, b + 1);
        const float v010 = Vox<VT>::ld(vox, b + sy_), v110 = Vox<VT>::ld(vox, b + sy_ + 1);
        const float v001 = Vox<VT>::ld(vox, b + sz_), v101 = Vox<VT>::ld(vox, b + sz_ + 1);
        const float v011 = Vox<VT>::ld(vox, b + sz_ + sy_), v111 = Vox<VT>::ld(vox, b + sz_ + sy_ + 1);
        // Weighted form w0*a + w1*b rather than a + (b - a)*w: with non-negative
        // attenuation every term is >= 0, so the relative error stays at a few
        // ulps even where a ray grazes the body edge and the value is tiny.
        const float gx = 1.0f - fx, gy = 1.0f - fy, gz = 1.0f - fz;
        const float a00 = fmaf(v100, fx, v000 * gx);
        const float a10 = fmaf(v110, fx, v010 * gx);
        const float a01 = fmaf(v101, fx, v001 * gx);
        const float a11 = fmaf(v111, fx, v011 * gx);
        const float b0 = fmaf(a10, fy, a00 * gy);
        const float b1 = fmaf(a11, fy, a01 * gy);
        const float val = fmaf(b1, fz, b0 * gz);
        if (KERNEL == XR_LINE_INT_MAX) sum = (sum < val) ? val : sum;
        else sum = __fadd_rn(sum, val);
        px = __fadd_rn(px, sx);
        py = __fadd_rn(py, sy);
        pz = __fadd_rn(pz, sz);
      }
      if (hit) {
        sum = __fmul_rn(sum, p.step);
        if (VT != XR_VOXEL_F32) sum = __fmul_rn(sum, p.vol.inv_scale);
        ns = nsteps + 1;
      }
    }
    // aa_sum = 0 + sum (xregRayCastLineIntCPU.cpp:189,282), then the store rule.
    const float aa = __fadd_rn(0.0f, sum);
    const int64_t npix = (int64_t)p.rows * p.cols;
    const int64_t pix = (int64_t)row * p.cols + col;
    const int64_t oidx = proj * npix + pix;
    float prev;
    if (p.bg_projs) prev = p.bg_projs[(int64_t)p.cam_idx[proj] * npix + pix];
    else if (p.store == XR_PROJ_STORE_REPLACE) prev = p.default_bg;
    else prev = p.out[oidx];
    p.out[oidx] = (KERNEL == XR_LINE_INT_MAX) ? ((prev < aa) ? aa : prev) : __fadd_rn(prev, aa);
  }
  if (p.sample_counter) {
    for (int o = 16; o > 0; o >>= 1) ns += __shfl_down_sync(0xffffffffu, ns, o);
    if (lane == 0 && ns) atomicAdd(p.sample_counter, ns);
  }
}

template <int VT, int KERNEL>
cudaError_t launch_t(const DrrParams& p, cudaStream_t s) {
  const dim3 block(kThreads);
  const int64_t max_z = 65535;
  for (int64_t base = 0; base < p.num_projs; base += max_z) {
    const int64_t n = (p.num_projs - base) < max_z ? (p.num_projs - base) : max_z;
    const dim3 grid((p.cols + kTileX - 1) / kTileX, (p.rows + kTileY - 1) / kTileY, (unsigned)n);
    drr_kernel<VT, KERNEL><<<grid, block, 0, s>>>(p, base);
  }
  return cudaGetLastError();
}

}  // namespace

cudaError_t launch_drr(const DrrParams& p, cudaStream_t s) {
  if (p.num_projs <= 0) return cudaSuccess;
  const bool mx = p.kernel_id == XR_LINE_INT_MAX;
  switch (p.vol.voxel_type) {
    case XR_VOXEL_F32:
      return mx ? launch_t<XR_VOXEL_F32, XR_LINE_INT_MAX>(p, s) : launch_t<XR_VOXEL_F32, XR_LINE_INT_SUM>(p, s);
    case XR_VOXEL_F16:
      return mx ? launch_t<XR_VOXEL_F16, XR_LINE_INT_MAX>(p, s) : launch_t<XR_VOXEL_F16, XR_LINE_INT_SUM>(p, s);
    case XR_VOXEL_BF16:
      return mx ? launch_t<XR_VOXEL_BF16, XR_LINE_INT_MAX>(p, s) : launch_t<XR_VOXEL_BF16, XR_LINE_INT_SUM>(p, s);
    default:
      return cudaErrorInvalidValue;
  }
}

}  // namespace xr
