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
// The per-ray geometry (detector point, slab test, nudge, step count, start
// point, step vector) is xReg's own float arithmetic in Eigen's evaluation order
// (xf::ray_setup, xr_xfloat.h), so sample counts and sample positions are the
// reference's, bit for bit.  The interpolation and the sum use ordinary float
// arithmetic.
//
// Volume layouts (same values, same arithmetic, bit-identical results):
//   LINEAR  voxels x-fastest; a sample issues 8 scalar loads.
//   CELL8   for every trilinear cell (ix, iy, iz) in [0, n-2]^3 the 8 corner
//           values are stored contiguously as z-pairs (v000 v001 v100 v101 v010
//           v011 v110 v111, vxyz), so each pair the packed FP32 blend needs is
//           one 64-bit register: one 16-byte load per sample for FP16/BF16, two
//           for FP32, or one 32-byte load for FP32 (the 256-bit read, layout 2).
//           It spends 8x the voxel bytes of HBM to cut L1 requests per sample
//           from 8 to 1-2; the linear kernel is bound by exactly those requests.
//           Cells are numbered z fastest, then x, then y (VolView::cs).
#include "xr_internal.h"
#include "xr_gradtile.cuh"

#include <algorithm>
#include <atomic>
#include <cmath>
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
  // 8 corners of cell c (CELL8 layout)
  __device__ __forceinline__ static void cell(const void* b, int c, float v[8]) {
    const float4* p = static_cast<const float4*>(b) + 2 * (size_t)c;
    const float4 lo = __ldg(p), hi = __ldg(p + 1);
    v[0] = lo.x; v[1] = lo.y; v[2] = lo.z; v[3] = lo.w;
    v[4] = hi.x; v[5] = hi.y; v[6] = hi.z; v[7] = hi.w;
  }
  // The same 32-byte cell with one 256-bit load (sm_100+ .v8 form); cells are
  // 32-byte aligned because the buffer is and every cell is 32 bytes.
  __device__ __forceinline__ static void cell_wide(const void* b, int c, float v[8]) {
    const float* p = static_cast<const float*>(b) + 8 * (size_t)c;
    asm("ld.global.nc.v8.f32 {%0,%1,%2,%3,%4,%5,%6,%7}, [%8];"
        : "=f"(v[0]), "=f"(v[1]), "=f"(v[2]), "=f"(v[3]), "=f"(v[4]), "=f"(v[5]), "=f"(v[6]), "=f"(v[7])
        : "l"(p));
  }
  // cell_wide when pred is true; otherwise v is left unwritten (no memory request).
  __device__ __forceinline__ static void cell_wide_if(const void* b, int c, bool pred, float v[8]) {
    const float* p = static_cast<const float*>(b) + 8 * (size_t)c;
    asm volatile(
        "{\n\t.reg .pred q;\n\tsetp.ne.u32 q, %9, 0;\n\t"
        "@q ld.global.nc.v8.f32 {%0,%1,%2,%3,%4,%5,%6,%7}, [%8];\n\t}"
        : "+f"(v[0]), "+f"(v[1]), "+f"(v[2]), "+f"(v[3]), "+f"(v[4]), "+f"(v[5]), "+f"(v[6]), "+f"(v[7])
        : "l"(p), "r"((unsigned)pred));
  }
};
// FP16 volumes are blended on their half2 words (interp8_h16 below), so their
// corners are read as raw 16-bit values and never widened.
template <>
struct Vox<XR_VOXEL_F16> {
  __device__ __forceinline__ static unsigned int ld16(const void* b, int i) {
    return __ldg(static_cast<const unsigned short*>(b) + i);
  }
  // the 4 z-pair words of cell c (CELL8 layout)
  __device__ __forceinline__ static void cell_words(const void* b, int c, unsigned int w[4]) {
    const uint4 q = __ldg(static_cast<const uint4*>(b) + c);
    w[0] = q.x; w[1] = q.y; w[2] = q.z; w[3] = q.w;
  }
};
template <>
struct Vox<XR_VOXEL_BF16> {
  __device__ __forceinline__ static float ld(const void* b, int i) {
    return __bfloat162float(__ldg(static_cast<const __nv_bfloat16*>(b) + i));
  }
  // A bf16 value is the upper half of the float with the same value, so each
  // packed pair widens with one shift (low) and one mask (high), exactly.
  __device__ __forceinline__ static void cell(const void* b, int c, float v[8]) {
    const uint4 q = __ldg(static_cast<const uint4*>(b) + c);
    const unsigned w[4] = {q.x, q.y, q.z, q.w};
#pragma unroll
    for (int k = 0; k < 4; ++k) {
      v[2 * k] = __uint_as_float(w[k] << 16);
      v[2 * k + 1] = __uint_as_float(w[k] & 0xffff0000u);
    }
  }
};

constexpr int kThreads = 256;
// Resident blocks per SM the DRR kernel is compiled for (caps registers at 40:
// 48 warps per SM instead of 40 at 48 registers).
constexpr int kMinBlocksPerSM = 6;
// CELL8 data read with one 256-bit load per sample (float32 volumes only).
constexpr int kLayoutCell8Wide = 2;
// Sample-loop variant 3: macro-cell empty-space skipping (sum kernel).
constexpr int kUnrollMacroSkip = 3;  // loop 2 after the macro-cell trim
constexpr int kUnrollTrim4 = 4;      // four samples per iteration after the macro-cell trim
constexpr int kUnrollPairShare = 5;  // loop 3 whose second sample of a pair reuses the first's cell
constexpr int kUnrollPacked = 6;     // loop 4 on packed FP32 pairs (float32 256-bit CELL8 reads)

// Trilinear sample at index position (px, py, pz) with ITK's boundary rule:
// the position is clamped to [0, n-1], the cell to [0, n-2], so a neighbour past
// the last index gets weight 0 (weight 1 on the last voxel).  The weighted form
// w0*a + w1*b keeps every term >= 0 for non-negative attenuation, so the
// relative error stays at a few ulps even where the value is tiny.
// Cell of a position for the CELL8 layouts, with its fractions (the clamping
// rule of sample() below).  INSIDE: the caller has shown that the position lies
// in [0, n-1) on every axis, where the clamps and the saturation change
// nothing, so they are left out (same cell, same fractions).
// ADD_FLOOR (inside only): floor(p) comes from one round-down addition: for
// 0 <= p < 2^23 the floats in [2^23, 2^24) are the integers, so p + 2^23
// rounded down is exactly 2^23 + floor(p), whose bit pattern is
// 0x4B000000 + floor(p).  No conversion instructions (the cell index is formed
// from the biased integers and the bias removed once, in wrapping 32-bit
// arithmetic), but two more FMA-pipe additions per axis: faster for float32
// cells, slower for half cells whose conversions already load that pipe.
template <bool INSIDE = false, bool ADD_FLOOR = false>
__device__ __forceinline__ int cell_of(const VolView& vol, float px, float py, float pz, float& fx, float& fy,
                                       float& fz) {
  const int nx = vol.nx, ny = vol.ny;
  if (INSIDE && ADD_FLOOR) {
    constexpr float kTwo23 = 8388608.0f;
    const float tx = __fadd_rd(px, kTwo23), ty = __fadd_rd(py, kTwo23), tz = __fadd_rd(pz, kTwo23);
    fx = __fsub_rn(px, __fsub_rn(tx, kTwo23));
    fy = __fsub_rn(py, __fsub_rn(ty, kTwo23));
    fz = __fsub_rn(pz, __fsub_rn(tz, kTwo23));
    const unsigned int sx = (unsigned int)vol.cs[0], sy = (unsigned int)vol.cs[1];
    const unsigned int bias = 0x4B000000u * (sx + sy + 1u);
    const unsigned int bx = (unsigned int)__float_as_int(tx), by = (unsigned int)__float_as_int(ty),
                       bz = (unsigned int)__float_as_int(tz);
    return (int)(bx * sx + by * sy + bz - bias);
  }
  int ix = __float2int_rd(px), iy = __float2int_rd(py), iz = __float2int_rd(pz);
  if (INSIDE) {
    fx = px - (float)ix;
    fy = py - (float)iy;
    fz = pz - (float)iz;
  } else {
    ix = max(min(ix, nx - 2), 0);
    iy = max(min(iy, ny - 2), 0);
    iz = max(min(iz, vol.nz - 2), 0);
    fx = __saturatef(px - (float)ix);
    fy = __saturatef(py - (float)iy);
    fz = __saturatef(pz - (float)iz);
  }
  return ix * vol.cs[0] + iy * vol.cs[1] + iz;
}

// Weighted-form trilinear of the 8 corners in cell order (z-pairs):
// v000 v001 v100 v101 v010 v011 v110 v111 (vxyz).
__device__ __forceinline__ float interp8(const float v[8], float fx, float fy, float fz) {
  const float gx = 1.0f - fx, gy = 1.0f - fy, gz = 1.0f - fz;
  const float a00 = fmaf(v[2], fx, v[0] * gx);
  const float a01 = fmaf(v[3], fx, v[1] * gx);
  const float a10 = fmaf(v[6], fx, v[4] * gx);
  const float a11 = fmaf(v[7], fx, v[5] * gx);
  const float b0 = fmaf(a10, fy, a00 * gy);
  const float b1 = fmaf(a11, fy, a01 * gy);
  return fmaf(b1, fz, b0 * gz);
}

// ---- packed FP32 pairs (sm_100+ f32x2): each lane rounds exactly as the
// scalar instruction with the same rounding mode, so results are bit-identical
// to the scalar code and only the instruction count changes.
__device__ __forceinline__ unsigned long long pk2(float a, float b) {
  unsigned long long r;
  asm("mov.b64 %0, {%1, %2};" : "=l"(r) : "f"(a), "f"(b));
  return r;
}
__device__ __forceinline__ void upk2(unsigned long long r, float& a, float& b) {
  asm("mov.b64 {%0, %1}, %2;" : "=f"(a), "=f"(b) : "l"(r));
}
__device__ __forceinline__ unsigned long long fma2(unsigned long long a, unsigned long long b, unsigned long long c) {
  unsigned long long d;
  asm("fma.rn.f32x2 %0, %1, %2, %3;" : "=l"(d) : "l"(a), "l"(b), "l"(c));
  return d;
}
__device__ __forceinline__ unsigned long long mul2(unsigned long long a, unsigned long long b) {
  unsigned long long d;
  asm("mul.rn.f32x2 %0, %1, %2;" : "=l"(d) : "l"(a), "l"(b));
  return d;
}
__device__ __forceinline__ unsigned long long add2(unsigned long long a, unsigned long long b) {
  unsigned long long d;
  asm("add.rn.f32x2 %0, %1, %2;" : "=l"(d) : "l"(a), "l"(b));
  return d;
}
__device__ __forceinline__ unsigned long long add2_rm(unsigned long long a, unsigned long long b) {
  unsigned long long d;
  asm("add.rm.f32x2 %0, %1, %2;" : "=l"(d) : "l"(a), "l"(b));
  return d;
}
__device__ __forceinline__ unsigned long long sub2(unsigned long long a, unsigned long long b) {
  unsigned long long d;
  asm("sub.rn.f32x2 %0, %1, %2;" : "=l"(d) : "l"(a), "l"(b));
  return d;
}
// A cell as four z-pairs of float32 values: the 32-byte float32 cell with one
// 256-bit load; a 16-byte BF16 cell with one 128-bit load, each 32-bit word
// (v_z0, v_z1) widened to a pair by a shift and a mask, exactly.
template <int VT>
__device__ __forceinline__ void cell_pairs(const void* b, int c, unsigned long long q[4]) {
  if constexpr (VT == XR_VOXEL_F32) {
    const unsigned long long* p = static_cast<const unsigned long long*>(b) + 4 * (size_t)c;
    asm("ld.global.nc.v4.b64 {%0,%1,%2,%3}, [%4];" : "=l"(q[0]), "=l"(q[1]), "=l"(q[2]), "=l"(q[3]) : "l"(p));
  } else {
    const uint4 w = __ldg(static_cast<const uint4*>(b) + c);
    const unsigned int ws[4] = {w.x, w.y, w.z, w.w};
#pragma unroll
    for (int k = 0; k < 4; ++k) {
      static_assert(VT == XR_VOXEL_BF16, "FP16 cells are blended as half2 words");
      q[k] = pk2(__uint_as_float(ws[k] << 16), __uint_as_float(ws[k] & 0xffff0000u));
    }
  }
}
// interp8 on z-pairs: q0 = (v000, v001), q1 = (v100, v101), q2 = (v010, v011),
// q3 = (v110, v111); the x and y blends run on pairs, the z blend in scalar.
__device__ __forceinline__ float interp8_pairs(const unsigned long long q[4], float fx, float fy, float fz) {
  const unsigned long long one = pk2(1.0f, 1.0f);
  const unsigned long long FX = pk2(fx, fx), FY = pk2(fy, fy);
  const unsigned long long GX = sub2(one, FX), GY = sub2(one, FY);
  const unsigned long long ay0 = fma2(q[1], FX, mul2(q[0], GX));  // (a00, a01)
  const unsigned long long ay1 = fma2(q[3], FX, mul2(q[2], GX));  // (a10, a11)
  const unsigned long long B = fma2(ay1, FY, mul2(ay0, GY));      // (b0, b1)
  float b0, b1;
  upk2(B, b0, b1);
  return fmaf(b1, fz, b0 * (1.0f - fz));
}

// ---- FP16 cells: the trilinear on the stored half2 words, with no
// conversion of the corners.  The x blend runs on the (z0, z1) pairs in half
// arithmetic (fma.rn.f16x2); the y blend is four mixed-precision fmas
// (fma.rn.f32.f16: exact products of halves added in float); the z blend is
// float.  The x and y weights are scaled by 2^15 before they are rounded to
// half, so a fraction as small as one float ulp of a position (>= 2^-24) is
// still a normal half; the stored values are below 1 (the volume's maximum is
// stored in [0.5, 1)), so the half blend cannot overflow; the volume's
// inv_scale removes the scales exactly.  Error: the half rounding of the four weights
// and of the x blend, about 1e-3 of a sample at worst, within the 2e-3 bound
// for half-precision volumes.  Every FP16 path (layouts, loops, the fused
// kernel) uses this one function, so they agree bit for bit.
__device__ __forceinline__ unsigned int h2_splat(float a) {
  unsigned int d;
  asm("cvt.rn.f16x2.f32 %0, %1, %1;" : "=r"(d) : "f"(a));
  return d;
}
__device__ __forceinline__ unsigned int h2_mul(unsigned int a, unsigned int b) {
  unsigned int d;
  asm("mul.rn.f16x2 %0, %1, %2;" : "=r"(d) : "r"(a), "r"(b));
  return d;
}
__device__ __forceinline__ unsigned int h2_fma(unsigned int a, unsigned int b, unsigned int c) {
  unsigned int d;
  asm("fma.rn.f16x2 %0, %1, %2, %3;" : "=r"(d) : "r"(a), "r"(b), "r"(c));
  return d;
}
// y blend of the half pairs a0 = (a00, a01), a1 = (a10, a11) with the half
// weights (low gy, high fy) of wy: b0 = a00 gy + a10 fy, b1 = a01 gy + a11 fy
__device__ __forceinline__ void h2_yblend(unsigned int a0, unsigned int a1, unsigned int wy, float& b0, float& b1) {
  asm("{\n\t.reg .b16 p0, p1, q0, q1, g, f;\n\t.reg .f32 t, u;\n\t"
      "mov.b32 {p0, p1}, %2;\n\tmov.b32 {q0, q1}, %3;\n\tmov.b32 {g, f}, %4;\n\t"
      "fma.rn.f32.f16 t, p0, g, %5;\n\tfma.rn.f32.f16 %0, q0, f, t;\n\t"
      "fma.rn.f32.f16 u, p1, g, %5;\n\tfma.rn.f32.f16 %1, q1, f, u;\n\t}"
      : "=f"(b0), "=f"(b1)
      : "r"(a0), "r"(a1), "r"(wy), "f"(0.0f));
}
// w: (v000, v001) (v100, v101) (v010, v011) (v110, v111), low half z = 0;
// returns the sample times 2^30
__device__ __forceinline__ float interp8_h16(const unsigned int w[4], float fx, float fy, float fz) {
  constexpr float kXs = 32768.0f, kYs = 32768.0f;
  const unsigned int FX = h2_splat(__fmul_rn(fx, kXs)), GX = h2_splat(__fmaf_rn(-fx, kXs, kXs));
  const __half2 wy = __floats2half2_rn(__fmaf_rn(-fy, kYs, kYs), __fmul_rn(fy, kYs));  // (gy, fy)
  const unsigned int A0 = h2_fma(w[1], FX, h2_mul(w[0], GX));  // (a00, a01)
  const unsigned int A1 = h2_fma(w[3], FX, h2_mul(w[2], GX));  // (a10, a11)
  float b0, b1;
  h2_yblend(A0, A1, *reinterpret_cast<const unsigned int*>(&wy), b0, b1);
  return __fmaf_rn(b1, fz, __fmul_rn(b0, __fsub_rn(1.0f, fz)));
}

// Trilinear sample at index position (px, py, pz) with ITK's boundary rule:
// the position is clamped to [0, n-1], the cell to [0, n-2], so a neighbour past
// the last index gets weight 0 (weight 1 on the last voxel).  The weighted form
// w0*a + w1*b keeps every term >= 0 for non-negative attenuation, so the
// relative error stays at a few ulps even where the value is tiny.
template <int VT, int LAYOUT, bool INSIDE = false>
__device__ __forceinline__ float sample(const VolView& vol, const void* data, float px, float py, float pz) {
  // Cell = floor(position) clamped to [0, n-2]; fraction = position - cell
  // saturated to [0, 1].  Equal to clamping the position to [0, n-1] first: below
  // 0 the cell is 0 and the fraction 0, above n-1 the cell is n-2 and the
  // fraction 1, and a NaN position reads cell 0 with fraction 0.
  float v[8], fx, fy, fz;
  [[maybe_unused]] unsigned int w[4];
  if (LAYOUT == kLayoutCell8Wide) {
    const int c = cell_of<INSIDE, true>(vol, px, py, pz, fx, fy, fz);
    if constexpr (VT == XR_VOXEL_F32) Vox<VT>::cell_wide(data, c, v);
  } else if (LAYOUT == XR_LAYOUT_CELL8) {
    const int c = cell_of<INSIDE, VT == XR_VOXEL_F32>(vol, px, py, pz, fx, fy, fz);
    if constexpr (VT == XR_VOXEL_F16) Vox<VT>::cell_words(data, c, w);
    else Vox<VT>::cell(data, c, v);
  } else {
    const int nx = vol.nx, ny = vol.ny;
    int ix = __float2int_rd(px), iy = __float2int_rd(py), iz = __float2int_rd(pz);
    if (INSIDE) {
      fx = px - (float)ix;
      fy = py - (float)iy;
      fz = pz - (float)iz;
    } else {
      ix = max(min(ix, nx - 2), 0);
      iy = max(min(iy, ny - 2), 0);
      iz = max(min(iz, vol.nz - 2), 0);
      fx = __saturatef(px - (float)ix);
      fy = __saturatef(py - (float)iy);
      fz = __saturatef(pz - (float)iz);
    }
    const int sy = nx, sz = nx * ny;
    const int b = (iz * ny + iy) * nx + ix;
    if constexpr (VT == XR_VOXEL_F16) {  // the CELL8 words, packed from 8 scalar reads
      w[0] = Vox<VT>::ld16(data, b) | (Vox<VT>::ld16(data, b + sz) << 16);
      w[1] = Vox<VT>::ld16(data, b + 1) | (Vox<VT>::ld16(data, b + sz + 1) << 16);
      w[2] = Vox<VT>::ld16(data, b + sy) | (Vox<VT>::ld16(data, b + sz + sy) << 16);
      w[3] = Vox<VT>::ld16(data, b + sy + 1) | (Vox<VT>::ld16(data, b + sz + sy + 1) << 16);
    } else {
      v[0] = Vox<VT>::ld(data, b);
      v[1] = Vox<VT>::ld(data, b + sz);
      v[2] = Vox<VT>::ld(data, b + 1);
      v[3] = Vox<VT>::ld(data, b + sz + 1);
      v[4] = Vox<VT>::ld(data, b + sy);
      v[5] = Vox<VT>::ld(data, b + sz + sy);
      v[6] = Vox<VT>::ld(data, b + sy + 1);
      v[7] = Vox<VT>::ld(data, b + sz + sy + 1);
    }
  }
  if constexpr (VT == XR_VOXEL_F16) return interp8_h16(w, fx, fy, fz);
  else return interp8(v, fx, fy, fz);
}

// Walks the macro cells of the ray p0 + k st from k = kstart towards kend
// (dir +1 forward, -1 backward) and returns the ray parameter at which it
// enters the first macro cell whose (dilated) occupancy bit is set, or +inf
// (-inf backward) when none is met before kend.  Macro cell m spans continuous
// index [8m, 8m + 8) on each axis; positions are clamped to cells as the
// sampler does.  The walk is bounded by the number of macro cells on a line.
__device__ __forceinline__ float macro_march(const VolView& v, const float p0[3], const float st[3],
                                             const float inv[3], float kstart, float kend, int dir) {
  const int nm[3] = {v.nmx, v.nmy, v.nmz};
  const int n2[3] = {v.nx - 2, v.ny - 2, v.nz - 2};
  int m[3];
#pragma unroll
  for (int a = 0; a < 3; ++a) {
    const float q = p0[a] + kstart * st[a];
    m[a] = max(min(__float2int_rd(q), n2[a]), 0) >> kMacroShift;
  }
  // inv = 1 / st, formed once per ray (a division per axis and step cost more
  // than the samples the walk saves): the boundary parameters carry a few ulps
  // of error, far inside the one-sample margin the caller leaves on each side.
  float k = kstart;
  const int cap = nm[0] + nm[1] + nm[2] + 3;
  for (int it = 0; it < cap; ++it) {
    const int idx = (m[2] * nm[1] + m[1]) * nm[0] + m[0];
    if ((__ldg(v.occ + (idx >> 5)) >> (idx & 31)) & 1u) return k;
    float best = INFINITY, knext = 0.0f;
    int ax = -1, dm = 0;
#pragma unroll
    for (int a = 0; a < 3; ++a) {
      const float d = dir > 0 ? st[a] : -st[a];
      float bound;
      int step;
      if (d > 1.0e-20f) {
        if (m[a] >= nm[a] - 1) continue;  // the last macro cell on this axis runs to the volume's end
        bound = (float)((m[a] + 1) << kMacroShift);
        step = 1;
      } else if (d < -1.0e-20f) {
        if (m[a] <= 0) continue;
        bound = (float)(m[a] << kMacroShift);
        step = -1;
      } else {
        continue;
      }
      const float kk = (bound - p0[a]) * inv[a];
      const float tt = dir > 0 ? kk : -kk;  // increases along the walk
      if (tt < best) { best = tt; knext = kk; ax = a; dm = step; }
    }
    if (ax < 0) return dir > 0 ? INFINITY : -INFINITY;  // stays in this empty macro cell
    if (dir > 0 ? (knext > kend) : (knext < kend)) return dir > 0 ? INFINITY : -INFINITY;
    if (dir > 0 ? (knext > k) : (knext < k)) k = knext;
#pragma unroll
    for (int a = 0; a < 3; ++a) m[a] += (a == ax) ? dm : 0;  // static indices: m stays in registers
  }
  return k;  // walk limit: treat the rest as occupied
}

// Loop 6: the four-sample loop of loop 4 for CELL8 cells (float32 256-bit
// reads, FP16 / BF16 128-bit reads) on rays proven inside the volume, with the
// x and y coordinates kept as one
// packed pair: position advance, the round-down floor (see cell_of) and the
// fractions of x and y are one f32x2 instruction each, the corners arrive as
// z-pairs and blend along x and y on pairs (interp8_pairs).  Same positions,
// cells, fractions and sums as loop 4, bit for bit.
template <int VT>
__device__ __forceinline__ float march_packed_inside(const VolView& vol, const void* data, float px, float py,
                                                     float pz, const float sx, const float sy, const float sz,
                                                     unsigned int n, float sum) {
  constexpr float kTwo23 = 8388608.0f;
  const unsigned long long K = pk2(kTwo23, kTwo23), S = pk2(sx, sy);
  unsigned long long P = pk2(px, py);
  const unsigned int csx = (unsigned int)vol.cs[0], csy = (unsigned int)vol.cs[1];
  const unsigned int bias = 0x4B000000u * (csx + csy + 1u);
  // cell index and fractions of the current position, then advance it
  auto locate = [&](float& fx, float& fy, float& fz) -> int {
    const unsigned long long T = add2_rm(P, K);
    const float tz = __fadd_rd(pz, kTwo23);
    const unsigned long long F = sub2(P, sub2(T, K));
    fz = __fsub_rn(pz, __fsub_rn(tz, kTwo23));
    float tx, ty;
    upk2(T, tx, ty);
    upk2(F, fx, fy);
    const unsigned int bx = (unsigned int)__float_as_int(tx), by = (unsigned int)__float_as_int(ty),
                       bz = (unsigned int)__float_as_int(tz);
    P = add2(P, S);
    pz = __fadd_rn(pz, sz);
    return (int)(bx * csx + by * csy + bz - bias);
  };
  if constexpr (VT == XR_VOXEL_F16) {  // half2 words blended as stored
    for (; n >= 4; n -= 4) {
      float f[4][3];
      unsigned int w[4][4];
#pragma unroll
      for (int k = 0; k < 4; ++k) Vox<VT>::cell_words(data, locate(f[k][0], f[k][1], f[k][2]), w[k]);
#pragma unroll
      for (int k = 0; k < 4; ++k) sum = __fadd_rn(sum, interp8_h16(w[k], f[k][0], f[k][1], f[k][2]));
    }
    for (; n > 0; --n) {
      float fx, fy, fz;
      unsigned int w[4];
      Vox<VT>::cell_words(data, locate(fx, fy, fz), w);
      sum = __fadd_rn(sum, interp8_h16(w, fx, fy, fz));
    }
  } else {
    for (; n >= 4; n -= 4) {
      float f[4][3];
      unsigned long long q[4][4];
#pragma unroll
      for (int k = 0; k < 4; ++k) cell_pairs<VT>(data, locate(f[k][0], f[k][1], f[k][2]), q[k]);
#pragma unroll
      for (int k = 0; k < 4; ++k) sum = __fadd_rn(sum, interp8_pairs(q[k], f[k][0], f[k][1], f[k][2]));
    }
    for (; n > 0; --n) {
      float fx, fy, fz;
      unsigned long long q[4];
      cell_pairs<VT>(data, locate(fx, fy, fz), q);
      sum = __fadd_rn(sum, interp8_pairs(q, fx, fy, fz));
    }
  }
  return sum;
}

// The samples of one ray from the current position on, n of them, in order
// (the sum order never changes with UNROLL).  INSIDE: every position stays in
// [0, n-1) on every axis (see sample()).
template <int VT, int KERNEL, int LAYOUT, int UNROLL, bool INSIDE>
__device__ __forceinline__ float march_samples(const DrrParams& p, const void* data, float px, float py, float pz,
                                               const float sx, const float sy, const float sz, unsigned int n,
                                               float sum) {
  if constexpr (UNROLL == kUnrollPacked && INSIDE && KERNEL == XR_LINE_INT_SUM &&
                ((VT == XR_VOXEL_F32 && LAYOUT == kLayoutCell8Wide) ||
                 (VT != XR_VOXEL_F32 && LAYOUT == XR_LAYOUT_CELL8)))
    return march_packed_inside<VT>(p.vol, data, px, py, pz, sx, sy, sz, n, sum);
  if (UNROLL == kUnrollTrim4 || UNROLL == kUnrollPacked) {  // four loads in flight per thread
    for (; n >= 4; n -= 4) {
      const float v0 = sample<VT, LAYOUT, INSIDE>(p.vol, data, px, py, pz);
      px = __fadd_rn(px, sx); py = __fadd_rn(py, sy); pz = __fadd_rn(pz, sz);
      const float v1 = sample<VT, LAYOUT, INSIDE>(p.vol, data, px, py, pz);
      px = __fadd_rn(px, sx); py = __fadd_rn(py, sy); pz = __fadd_rn(pz, sz);
      const float v2 = sample<VT, LAYOUT, INSIDE>(p.vol, data, px, py, pz);
      px = __fadd_rn(px, sx); py = __fadd_rn(py, sy); pz = __fadd_rn(pz, sz);
      const float v3 = sample<VT, LAYOUT, INSIDE>(p.vol, data, px, py, pz);
      px = __fadd_rn(px, sx); py = __fadd_rn(py, sy); pz = __fadd_rn(pz, sz);
      if (KERNEL == XR_LINE_INT_MAX) {
        sum = (sum < v0) ? v0 : sum;
        sum = (sum < v1) ? v1 : sum;
        sum = (sum < v2) ? v2 : sum;
        sum = (sum < v3) ? v3 : sum;
      } else {
        sum = __fadd_rn(__fadd_rn(__fadd_rn(__fadd_rn(sum, v0), v1), v2), v3);
      }
    }
  }
  if (UNROLL == kUnrollPairShare && LAYOUT == kLayoutCell8Wide && KERNEL == XR_LINE_INT_SUM) {
    // Two samples per iteration; at a step below the voxel size both often
    // fall in one cell, and then the second load is not issued (its lane
    // makes no memory request) and the first sample's corners are reused.
    for (; n >= 2; n -= 2) {
      float f0x, f0y, f0z, f1x, f1y, f1z;
      const int c0 = cell_of<INSIDE, true>(p.vol, px, py, pz, f0x, f0y, f0z);
      px = __fadd_rn(px, sx); py = __fadd_rn(py, sy); pz = __fadd_rn(pz, sz);
      const int c1 = cell_of<INSIDE, true>(p.vol, px, py, pz, f1x, f1y, f1z);
      px = __fadd_rn(px, sx); py = __fadd_rn(py, sy); pz = __fadd_rn(pz, sz);
      float v0[8], v1[8];
      if constexpr (VT == XR_VOXEL_F32) {
        Vox<VT>::cell_wide(data, c0, v0);
#pragma unroll
        for (int i = 0; i < 8; ++i) v1[i] = 0.0f;
        Vox<VT>::cell_wide_if(data, c1, c1 != c0, v1);
      }
      const bool same = c1 == c0;
#pragma unroll
      for (int i = 0; i < 8; ++i) v1[i] = same ? v0[i] : v1[i];
      sum = __fadd_rn(__fadd_rn(sum, interp8(v0, f0x, f0y, f0z)), interp8(v1, f1x, f1y, f1z));
    }
  }
  if (UNROLL >= 2) {  // loops 3, 4 and 5 finish with the two-sample loop
    for (; n >= 2; n -= 2) {
      const float v0 = sample<VT, LAYOUT, INSIDE>(p.vol, data, px, py, pz);
      px = __fadd_rn(px, sx); py = __fadd_rn(py, sy); pz = __fadd_rn(pz, sz);
      const float v1 = sample<VT, LAYOUT, INSIDE>(p.vol, data, px, py, pz);
      px = __fadd_rn(px, sx); py = __fadd_rn(py, sy); pz = __fadd_rn(pz, sz);
      if (KERNEL == XR_LINE_INT_MAX) {
        sum = (sum < v0) ? v0 : sum;
        sum = (sum < v1) ? v1 : sum;
      } else {
        sum = __fadd_rn(__fadd_rn(sum, v0), v1);
      }
    }
  }
  for (; n > 0; --n) {
    const float v0 = sample<VT, LAYOUT, INSIDE>(p.vol, data, px, py, pz);
    px = __fadd_rn(px, sx); py = __fadd_rn(py, sy); pz = __fadd_rn(pz, sz);
    if (KERNEL == XR_LINE_INT_MAX) sum = (sum < v0) ? v0 : sum;
    else sum = __fadd_rn(sum, v0);
  }
  return sum;
}

// Traces the ray of pixel (row, col) of projection proj and stores the result
// (the caller checks that the pixel exists).  Returns the number of samples of
// the reference step rule; *loaded receives how many of them were loaded (the
// others were proven zero and skipped).
template <int VT, int KERNEL, int LAYOUT, int UNROLL>
__device__ __forceinline__ unsigned long long trace_pixel(const DrrParams& p, const int64_t proj, const int row,
                                                          const int col, unsigned int* loaded) {
  float sum = (KERNEL == XR_LINE_INT_MAX) ? -FLT_MAX : 0.0f;
  unsigned long long ns = 0;
  *loaded = 0;
  {
    // xReg's per-ray float set-up (xf::ray_setup): clipped, nudged segment,
    // start point, step vector and the step-count quotient
    const float maxb[3] = {(float)(p.vol.nx - 1), (float)(p.vol.ny - 1), (float)(p.vol.nz - 1)};
    float st0[3], stv[3], quot;
    bool hit = xf::ray_setup(p.geo[proj], (float)col, (float)row, maxb, p.step, st0, stv, quot);
    if (hit) {
      float px = st0[0], py = st0[1], pz = st0[2];
      // num_steps = size_t(quotient) through a saturating 32-bit conversion (a
      // 64-bit one runs on the slow FP64 pipe): above 2^32 - 1 it saturates and
      // NaN gives 0, so the max_steps test (max_steps < 2^31) decides as with 64 bits
      unsigned long long nsteps = __float2uint_rz(quot);
      if (!(nsteps <= p.max_steps)) {
        // A ray longer than the volume diagonal allows can only come from a
        // non-finite or degenerate pose: count it and leave the pixel unsampled
        // rather than loop for an unbounded time.
        atomicAdd(p.err_counter, 1u);
        nsteps = 0;
        hit = false;
      }
      const float sx = stv[0], sy = stv[1], sz = stv[2];
      // reciprocal steps for the skipping bounds (never for sample positions)
      const float inv_st[3] = {1.0f / sx, 1.0f / sy, 1.0f / sz};
      const void* data = (LAYOUT != XR_LAYOUT_LINEAR) ? p.vol.cells : p.vol.voxels;
      // Samples [first, last] may touch non-zero voxels; the others interpolate
      // only zeros, so for the sum they add exactly +0 and need no load.  The
      // samples before `first` still advance the position by the same float
      // additions, so every sampled position is the one the reference uses.
      unsigned int first = 0, last = (unsigned int)nsteps;
      if (KERNEL == XR_LINE_INT_SUM && p.vol.has_support && hit) {
        float lo = 0.0f, hi = (float)nsteps;
        if (p.vol.sup_lo[0] > p.vol.sup_hi[0]) hi = -1.0f;  // all-zero volume
        const float st[3] = {sx, sy, sz}, p0[3] = {px, py, pz};
#pragma unroll
        for (int k = 0; k < 3; ++k) {
          if (fabsf(st[k]) > 1.0e-20f) {
            // reciprocal steps: a few ulps of error, inside the one-sample margins below
            float a = (p.vol.sup_lo[k] - p0[k]) * inv_st[k], b = (p.vol.sup_hi[k] - p0[k]) * inv_st[k];
            if (a > b) { const float t = a; a = b; b = t; }
            lo = fmaxf(lo, a);
            hi = fminf(hi, b);
          } else if (!(p0[k] > p.vol.sup_lo[k] && p0[k] < p.vol.sup_hi[k])) {
            hi = -1.0f;
          }
        }
        if (!(lo <= hi)) {
          last = 0;
          first = 1;  // no sample can be non-zero
        } else {
          const float f0 = floorf(lo) - 1.0f, f1 = ceilf(hi) + 1.0f;
          first = f0 > 0.0f ? (unsigned int)f0 : 0u;
          last = f1 < (float)nsteps ? (unsigned int)f1 : (unsigned int)nsteps;
        }
      }
      bool trim_ok = false;  // positions drift by less than an eighth of a voxel
      if (UNROLL >= kUnrollMacroSkip && KERNEL == XR_LINE_INT_SUM && p.vol.occ && hit && first <= last) {
        // Macro-cell trim: walk the macro grid from each end of [first, last]
        // to the first occupied macro cell; the samples before (after) it lie in
        // empty macro cells and add exactly 0.  The occupancy is dilated by one
        // trilinear cell, so a sample whose float position strays less than a
        // voxel from the exact ray still reads only zero corners; repeated
        // addition drifts by at most (last + 1) half-ulps of a coordinate below
        // 2^e, kept under a voxel by the 2^(22-e) sample limit.
        const int ebits = 32 - __clz(max(p.vol.nx, max(p.vol.ny, p.vol.nz)));
        if (ebits <= 22 && last < (1u << (22 - ebits))) {
          trim_ok = true;
          const float p0[3] = {px, py, pz}, st[3] = {sx, sy, sz};
          const float kf = macro_march(p.vol, p0, st, inv_st, (float)first, (float)last, 1);
          if (kf == INFINITY) {
            first = 1u;
            last = 0u;  // every sample is zero
          } else {
            const float f = floorf(kf) - 1.0f;
            if (f > (float)first) first = (unsigned int)f;
            const float kl = macro_march(p.vol, p0, st, inv_st, (float)last, (float)first, -1);
            if (kl == -INFINITY) {
              first = 1u;
              last = 0u;
            } else {
              const float l = ceilf(kl) + 1.0f;
              if (l < (float)last) last = (unsigned int)l;
            }
          }
        }
      }
      // Rays whose first and last loaded samples lie at least a quarter voxel
      // inside [0, n-1] on every axis keep every sample there (the segment is
      // straight and the drift stays under an eighth of a voxel), so they run
      // the sampler without clamps.
      bool inside = false;
      if (UNROLL >= kUnrollMacroSkip && trim_ok && first <= last) {
        const float p0[3] = {px, py, pz}, st[3] = {sx, sy, sz};
        inside = true;
#pragma unroll
        for (int k = 0; k < 3; ++k) {
          const float a = p0[k] + (float)first * st[k], b = p0[k] + (float)last * st[k];
          inside = inside && fminf(a, b) >= 0.25f && fmaxf(a, b) <= maxb[k] - 0.25f;
        }
      }
      if (hit) {
        // advance to sample `first` (four additions per trip: the skipped samples
        // are a large part of a trimmed ray); x and y as one packed pair, whose
        // lanes round as the scalar additions do
        unsigned int skip = first <= last ? first : last + 1u;
        {
          unsigned long long P = pk2(px, py);
          const unsigned long long S = pk2(sx, sy);
          for (; skip >= 4; skip -= 4) {
            P = add2(P, S); pz = __fadd_rn(pz, sz);
            P = add2(P, S); pz = __fadd_rn(pz, sz);
            P = add2(P, S); pz = __fadd_rn(pz, sz);
            P = add2(P, S); pz = __fadd_rn(pz, sz);
          }
          for (; skip > 0; --skip) {
            P = add2(P, S); pz = __fadd_rn(pz, sz);
          }
          upk2(P, px, py);
        }
        // samples first..last in order; the sum order never changes with UNROLL
        unsigned int n = first <= last ? last - first + 1u : 0u;
        *loaded = n;
        if (inside)
          sum = march_samples<VT, KERNEL, LAYOUT, UNROLL, true>(p, data, px, py, pz, sx, sy, sz, n, sum);
        else
          sum = march_samples<VT, KERNEL, LAYOUT, UNROLL, false>(p, data, px, py, pz, sx, sy, sz, n, sum);
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
  return ns;
}

// Loop 4 keeps four cells (32 floats) in flight per thread: capped at 48
// registers (5 blocks per SM), measured faster than 40 (small spills) or 64.
template <int VT, int KERNEL, int LAYOUT, int UNROLL>
__global__ void __launch_bounds__(kThreads,
                                  (UNROLL == kUnrollTrim4 || UNROLL == kUnrollPacked) ? kMinBlocksPerSM - 1
                                                                                       : kMinBlocksPerSM)
drr_kernel(const DrrParams p, const int64_t proj_base) {
  // Each warp covers an 8 x 4 (or, tall, 4 x 8) patch of pixels so its 32 rays
  // stay close inside the volume; a block is bw x (8 / bw) warps.  The
  // projection is the fastest grid index: blocks resident at the same time trace
  // the same detector tile for many nearby poses, whose footprints overlap in L2.
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int bw = p.block_warps_x;
  const int wl = p.warp_tall ? 2 : 3;  // log2 of the warp's width in pixels
  const int wc = 1 << wl, wr = 32 >> wl;
  const int col = blockIdx.y * (wc * bw) + (warp % bw) * wc + (lane & (wc - 1));
  const int row = blockIdx.z * ((8 / bw) * wr) + (warp / bw) * wr + (lane >> wl);
  const int64_t proj = proj_base + blockIdx.x;
  unsigned long long ns = 0;
  unsigned int nl = 0;
  if (col < p.cols && row < p.rows) ns = trace_pixel<VT, KERNEL, LAYOUT, UNROLL>(p, proj, row, col, &nl);
  if (p.sample_counter) {
    unsigned long long nlw = nl;
    for (int o = 16; o > 0; o >>= 1) {
      ns += __shfl_down_sync(0xffffffffu, ns, o);
      nlw += __shfl_down_sync(0xffffffffu, nlw, o);
    }
    if (lane == 0 && ns) atomicAdd(p.sample_counter, ns);
    if (lane == 0 && nlw && p.loaded_counter) atomicAdd(p.loaded_counter, nlw);
  }
}

// ---- brick-staged variant (layout 3: float32 CELL8 cells, sum kernel) ----
// One block traces 16x16 rays of one projection.  Their samples are taken in
// slabs of cells along the rays' dominant axis: for each slab the block copies
// the cells its rays reach there (a box from every ray's cell at the slab entry
// and an estimate of its exit, widened by one cell) into shared memory, then
// each ray takes its samples in that slab from the copy; a sample whose cell
// falls outside the box reads global memory.  Positions, cells, fractions and
// the order of the sum are those of drr_kernel (support-box skipping included,
// no macro-cell trim), so every value is identical.  The staged alternative to
// gathering through L1, measured against it; never chosen by the autotuner.
constexpr int kLayoutBrick = 3;
constexpr int kBrickCells = 1400;  // 43.75 KB of 32-byte cells
constexpr int kBrickDepth = 16;    // cells per slab along the dominant axis

// Cell and fractions of a position with drr_kernel's clamping (cell_of, not INSIDE).
__device__ __forceinline__ void cell3(const VolView& vol, const float pos[3], int c[3], float f[3]) {
  c[0] = max(min(__float2int_rd(pos[0]), vol.nx - 2), 0);
  c[1] = max(min(__float2int_rd(pos[1]), vol.ny - 2), 0);
  c[2] = max(min(__float2int_rd(pos[2]), vol.nz - 2), 0);
  f[0] = __saturatef(pos[0] - (float)c[0]);
  f[1] = __saturatef(pos[1] - (float)c[1]);
  f[2] = __saturatef(pos[2] - (float)c[2]);
}

// The ray's remaining samples k..last from global memory, in order.
__device__ __forceinline__ float brick_march_global(const VolView& vol, float pos[3], const float st[3],
                                                    unsigned int& k, unsigned int last, float sum) {
  for (; k <= last; ++k) {
    int c[3];
    float f[3], v[8];
    cell3(vol, pos, c, f);
    Vox<XR_VOXEL_F32>::cell_wide(vol.cells, c[0] * vol.cs[0] + c[1] * vol.cs[1] + c[2], v);
    sum = __fadd_rn(sum, interp8(v, f[0], f[1], f[2]));
    pos[0] = __fadd_rn(pos[0], st[0]);
    pos[1] = __fadd_rn(pos[1], st[1]);
    pos[2] = __fadd_rn(pos[2], st[2]);
  }
  return sum;
}

__global__ void __launch_bounds__(kThreads, 4) drr_brick_kernel(const DrrParams p, const int64_t proj_base) {
  __shared__ float4 s_cells[2 * kBrickCells];
  __shared__ int s_code, s_amin, s_amax, s_lo[3], s_hi[3];
  const int tid = threadIdx.x;
  const int col = blockIdx.y * 16 + (tid & 15), row = blockIdx.z * 16 + (tid >> 4);
  const int64_t proj = proj_base + blockIdx.x;
  const VolView& vol = p.vol;
  const int ncell[3] = {vol.nx - 1, vol.ny - 1, vol.nz - 1};
  const float4* cells = static_cast<const float4*>(vol.cells);
  if (tid == 0) {
    s_code = -1;
    s_amin = 0x7fffffff;
    s_amax = -1;
  }
  const bool pixel = col < p.cols && row < p.rows;
  float sum = 0.0f, pos[3] = {0.0f, 0.0f, 0.0f}, st[3] = {0.0f, 0.0f, 0.0f};
  unsigned long long ns = 0;
  unsigned int nl = 0, k = 1, last = 0;  // samples k..last remain
  if (pixel) {
    // xReg's per-ray float set-up and drr_kernel's support-box bounds
    const float maxb[3] = {(float)(vol.nx - 1), (float)(vol.ny - 1), (float)(vol.nz - 1)};
    float st0[3], quot;
    bool hit = xf::ray_setup(p.geo[proj], (float)col, (float)row, maxb, p.step, st0, st, quot);
    unsigned long long nsteps = hit ? __float2uint_rz(quot) : 0ull;
    if (hit && !(nsteps <= p.max_steps)) {
      atomicAdd(p.err_counter, 1u);
      nsteps = 0;
      hit = false;
    }
    if (hit) {
      unsigned int first = 0, lst = (unsigned int)nsteps;
      if (vol.has_support) {
        float lo = 0.0f, hi = (float)nsteps;
        if (vol.sup_lo[0] > vol.sup_hi[0]) hi = -1.0f;
#pragma unroll
        for (int a = 0; a < 3; ++a) {
          if (fabsf(st[a]) > 1.0e-20f) {
            const float inv = 1.0f / st[a];
            float u = (vol.sup_lo[a] - st0[a]) * inv, w = (vol.sup_hi[a] - st0[a]) * inv;
            if (u > w) { const float t = u; u = w; w = t; }
            lo = fmaxf(lo, u);
            hi = fminf(hi, w);
          } else if (!(st0[a] > vol.sup_lo[a] && st0[a] < vol.sup_hi[a])) {
            hi = -1.0f;
          }
        }
        if (!(lo <= hi)) {
          lst = 0;
          first = 1;
        } else {
          const float f0 = floorf(lo) - 1.0f, f1 = ceilf(hi) + 1.0f;
          first = f0 > 0.0f ? (unsigned int)f0 : 0u;
          lst = f1 < (float)nsteps ? (unsigned int)f1 : (unsigned int)nsteps;
        }
      }
      pos[0] = st0[0]; pos[1] = st0[1]; pos[2] = st0[2];
      for (unsigned int i = 0, skip = first <= lst ? first : lst + 1u; i < skip; ++i) {
        pos[0] = __fadd_rn(pos[0], st[0]);
        pos[1] = __fadd_rn(pos[1], st[1]);
        pos[2] = __fadd_rn(pos[2], st[2]);
      }
      k = first;
      last = lst;
      nl = first <= lst ? lst - first + 1u : 0u;
      ns = nsteps + 1;
    }
  }
  __syncthreads();
  // the block's axis and direction: claimed by the first ray that has samples
  int code = -1;
  if (k <= last) {
    int a = 0;
    float m = fabsf(st[0]);
    if (fabsf(st[1]) > m) { a = 1; m = fabsf(st[1]); }
    if (fabsf(st[2]) > m) { a = 2; m = fabsf(st[2]); }
    code = m > 0.0f ? 2 * a + (st[a] > 0.0f ? 1 : 0) : -1;
    if (code >= 0) atomicCAS(&s_code, -1, code);
  }
  __syncthreads();
  const int bcode = s_code, ax = bcode >> 1, dir = (bcode & 1) ? 1 : -1;
  const bool staged = k <= last && bcode >= 0 && code == bcode;
  if (k <= last && !staged) sum = brick_march_global(vol, pos, st, k, last, sum);  // another axis: global reads
  if (staged) {  // the cells of this ray's first and (about) last samples along the axis
    int c0[3], c1[3];
    float f[3];
    cell3(vol, pos, c0, f);
    const float e = (float)(last - k);
    const float pe[3] = {pos[0] + e * st[0], pos[1] + e * st[1], pos[2] + e * st[2]};
    cell3(vol, pe, c1, f);
    atomicMin(&s_amin, min(c0[ax], c1[ax]) - 1);
    atomicMax(&s_amax, max(c0[ax], c1[ax]) + 1);
  }
  __syncthreads();
  if (bcode >= 0) {
    const int amin = max(s_amin, 0), amax = min(s_amax, ncell[ax] - 1);
    int z = dir > 0 ? amin : amax;  // first cell of the slab along the axis
    for (int guard = 0; guard < 8192 && (dir > 0 ? z <= amax : z >= amin); ++guard) {
      if (tid < 3) {
        s_lo[tid] = 0x7fffffff;
        s_hi[tid] = -1;
      }
      __syncthreads();
      const int zfar = dir > 0 ? z + kBrickDepth : z - kBrickDepth;  // first cell past a full slab
      if (staged && k <= last) {
        int ce[3], cx[3];
        float f[3];
        cell3(vol, pos, ce, f);
        float m = ((float)zfar - pos[ax]) / st[ax];  // samples to the slab's far side, about
        m = fminf(fmaxf(m, 0.0f), (float)(last - k));
        const float pe[3] = {pos[0] + m * st[0], pos[1] + m * st[1], pos[2] + m * st[2]};
        cell3(vol, pe, cx, f);
#pragma unroll
        for (int a = 0; a < 3; ++a) {
          if (a == ax) continue;
          atomicMin(&s_lo[a], min(ce[a], cx[a]) - 1);
          atomicMax(&s_hi[a], max(ce[a], cx[a]) + 1);
        }
      }
      __syncthreads();
      int lo[3], hi[3], lat = 1;
#pragma unroll
      for (int a = 0; a < 3; ++a) {
        if (a == ax) continue;
        lo[a] = max(s_lo[a], 0);
        hi[a] = min(s_hi[a], ncell[a] - 1);
        lat *= hi[a] >= lo[a] ? hi[a] - lo[a] + 1 : 0;
      }
      // slab depth: the full one, thinner when the box would not fit
      int d = kBrickDepth;
      bool use = lat > 0;
      if (use && lat * d > kBrickCells) {
        d = kBrickCells / lat;
        if (d < 1) {
          d = kBrickDepth;
          use = false;  // too wide a box: this slab reads global memory
        }
      }
      lo[ax] = dir > 0 ? z : max(z - d + 1, 0);
      hi[ax] = dir > 0 ? min(z + d - 1, ncell[ax] - 1) : z;
      const int W = hi[0] - lo[0] + 1, H = hi[1] - lo[1] + 1, Dz = hi[2] - lo[2] + 1;
      if (use) {
        const int total = W * H * Dz;
        for (int i = tid; i < total; i += kThreads) {
          const int x = lo[0] + i % W, y = lo[1] + (i / W) % H, zz = lo[2] + i / (W * H);
          const int64_t c = (int64_t)x * vol.cs[0] + (int64_t)y * vol.cs[1] + zz;
          s_cells[2 * i] = __ldg(cells + 2 * c);
          s_cells[2 * i + 1] = __ldg(cells + 2 * c + 1);
        }
      }
      __syncthreads();
      const int zend = dir > 0 ? z + d : z - d;  // first cell past this slab
      if (staged) {
        for (; k <= last; ++k) {
          int c[3];
          float f[3], v[8];
          cell3(vol, pos, c, f);
          if (dir > 0 ? c[ax] >= zend : c[ax] <= zend) break;
          const bool in = use && c[0] >= lo[0] && c[0] <= hi[0] && c[1] >= lo[1] && c[1] <= hi[1] && c[2] >= lo[2] &&
                          c[2] <= hi[2];
          if (in) {
            const int i = (c[0] - lo[0]) + W * ((c[1] - lo[1]) + H * (c[2] - lo[2]));
            const float4 q0 = s_cells[2 * i], q1 = s_cells[2 * i + 1];
            v[0] = q0.x; v[1] = q0.y; v[2] = q0.z; v[3] = q0.w;
            v[4] = q1.x; v[5] = q1.y; v[6] = q1.z; v[7] = q1.w;
          } else {
            Vox<XR_VOXEL_F32>::cell_wide(vol.cells, c[0] * vol.cs[0] + c[1] * vol.cs[1] + c[2], v);
          }
          sum = __fadd_rn(sum, interp8(v, f[0], f[1], f[2]));
          pos[0] = __fadd_rn(pos[0], st[0]);
          pos[1] = __fadd_rn(pos[1], st[1]);
          pos[2] = __fadd_rn(pos[2], st[2]);
        }
      }
      __syncthreads();  // the copy is read by every ray before the next slab overwrites it
      z = zend;
    }
  }
  if (k <= last) sum = brick_march_global(vol, pos, st, k, last, sum);  // past the estimated range
  if (pixel) {
    sum = __fmul_rn(sum, p.step);
    const float aa = __fadd_rn(0.0f, sum);
    const int64_t npix = (int64_t)p.rows * p.cols;
    const int64_t pix = (int64_t)row * p.cols + col;
    const int64_t oidx = proj * npix + pix;
    float prev;
    if (p.bg_projs) prev = p.bg_projs[(int64_t)p.cam_idx[proj] * npix + pix];
    else if (p.store == XR_PROJ_STORE_REPLACE) prev = p.default_bg;
    else prev = p.out[oidx];
    p.out[oidx] = __fadd_rn(prev, aa);
  }
  if (p.sample_counter) {
    const int lane = tid & 31;
    unsigned long long nlw = nl;
    for (int o = 16; o > 0; o >>= 1) {
      ns += __shfl_down_sync(0xffffffffu, ns, o);
      nlw += __shfl_down_sync(0xffffffffu, nlw, o);
    }
    if (lane == 0 && ns) atomicAdd(p.sample_counter, ns);
    if (lane == 0 && nlw && p.loaded_counter) atomicAdd(p.loaded_counter, nlw);
  }
}

// Fused evaluation: a persistent multi-job DRR loop (every block takes the
// next (job, tile, projection) item from a global counter; projections are
// the fastest index within a job), with each job's grad-NCC (5x5 smoothing) computed inside the same launch.
// No block ever waits for another.  After a block writes a 16x16 DRR tile it
// counts the tile towards every 32x64 metric tile whose input (the tile with
// its 3-pixel blur + Sobel halo, clipped to the image) the tile overlaps; the
// block whose count completes a metric tile computes that tile's moments at
// once, reading the DRR pixels back through L2 (gt::grad_tile_moments, the
// split path's own tile code); the block that completes an image's metric
// tiles combines its partials in FP64 (gt::grad_finalize_image), and the block
// that completes a pose's views writes the mean over views.  Counters are
// zero between launches: whoever completes one resets it.  Stores are made
// visible device-wide (fence) before each count; counted data is read through
// L2 (ld.global.cg), never through the incoherent L1.
constexpr int kFusedKR = 2;  // 5x5 smoothing, xReg's default

// Metric tiles the DRR tile [r0, r1) x [c0, c1) feeds, and how many DRR tiles
// (tw x th pixels) feed each; claims (into claim[]) those whose count this
// tile completes.
__device__ __forceinline__ int fused_count_tile(const FusedJob& J, unsigned int* cnt_tile, int r0, int r1, int c0,
                                                int c1, int tw, int th, int* claim) {
  constexpr int H = kFusedKR + 1;
  const int rows = J.d.p.rows, cols = J.d.p.cols;
  int n = 0;
  const int my0 = max(0, (r0 - H) / gt::kGH - 1), my1 = min(J.mt_y - 1, (r1 - 1 + H) / gt::kGH);
  const int mx0 = max(0, (c0 - H) / gt::kGW - 1), mx1 = min(J.mt_x - 1, (c1 - 1 + H) / gt::kGW);
  for (int my = my0; my <= my1; ++my) {
    const int er0 = max(0, my * gt::kGH - H), er1 = min(rows, my * gt::kGH + gt::kGH + H);
    if (!(er0 < r1 && r0 < er1)) continue;
    for (int mx = mx0; mx <= mx1; ++mx) {
      const int ec0 = max(0, mx * gt::kGW - H), ec1 = min(cols, mx * gt::kGW + gt::kGW + H);
      if (!(ec0 < c1 && c0 < ec1)) continue;
      const unsigned int target = (unsigned int)(((er1 - 1) / th - er0 / th + 1) * ((ec1 - 1) / tw - ec0 / tw + 1));
      unsigned int* c = cnt_tile + my * J.mt_x + mx;
      if (atomicAdd(c, 1u) + 1u == target) {
        *c = 0u;  // completed: zero for the next launch
        claim[n++] = my * J.mt_x + mx;
      }
    }
  }
  return n;
}

// The metric stage of a claimed tile, out of line: its registers do not
// constrain the DRR loop's (it runs a few times per image, the loop for every
// sample).  Returns, in thread 0, whether the image is complete.
__device__ __noinline__ bool fused_metric_tile(const FusedJob& J, int64_t proj, int M, gt::FF* red) {
  const DrrParams& P = J.d.p;
  const int rows = P.rows, cols = P.cols, mt = J.mt_x * J.mt_y;
  const int64_t nimg = (int64_t)J.nviews * J.pop;
  const int64_t v = proj / J.pop, k = proj - v * J.pop;
  const FusedView& V = J.views[v];
  double vals[6];
  gt::grad_tile_moments_regs5(P.out + proj * (int64_t)rows * cols, rows, cols, (M / J.mt_x) * gt::kGH,
                              (M % J.mt_x) * gt::kGW, V.fhx, V.fhy, V.mask, red, vals);
  bool last = false;
  if (threadIdx.x == 0) {
    double* o = V.partials + (k * mt + M) * 6;
#pragma unroll
    for (int q = 0; q < 6; ++q) o[q] = vals[q];
    __threadfence();
    unsigned int* ci = J.cnt + nimg * mt + proj;
    last = atomicAdd(ci, 1u) + 1u == (unsigned int)mt;
    if (last) *ci = 0u;
  }
  return last;
}

// Every metric tile of image proj is in: its FP64 combine, then (by the block
// that completes the pose's views) the mean over views.
__device__ __noinline__ void fused_metric_image(const FusedJob& J, int64_t proj, double* red) {
  const int mt = J.mt_x * J.mt_y;
  const int64_t nimg = (int64_t)J.nviews * J.pop;
  const int64_t v = proj / J.pop, k = proj - v * J.pop;
  const FusedView& V = J.views[v];
  __threadfence();
  const float sim = gt::grad_finalize_image<true>(V.partials + k * mt * 6, mt, V.n_used, V.fx, V.fy, red);
  if (threadIdx.x == 0) {
    V.sims[k] = sim;
    __threadfence();
    unsigned int* cp = J.cnt + nimg * mt + nimg + k;
    if (atomicAdd(cp, 1u) + 1u == (unsigned int)J.nviews) {  // every view of this pose
      *cp = 0u;
      __threadfence();
      float sum = 0.0f;
      for (int w = 0; w < J.nviews; ++w) sum += __ldcg(J.views[w].sims + k);
      J.out[k] = sum / (float)J.nviews;  // ImgSimMetric2DCombineMean (as gt::combine_mean)
    }
  }
}

template <int VT, int LAYOUT, int UNROLL>
__global__ void __launch_bounds__(kThreads, kMinBlocksPerSM - 1)
eval_fused_kernel(const FusedJob* __restrict__ jobs, int njobs, long long total, unsigned long long* counter) {
  // under 1 KB of shared memory: the SM's unified L1 stays with the DRR gathers
  __shared__ long long s_item;
  __shared__ gt::FF s_red[6 * (kThreads / 32)];
  __shared__ double s_dred[6 * (gt::kFinalizeThreads / 32)];
  __shared__ int s_claim[16];
  __shared__ int s_nclaim, s_last;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  for (;;) {
    if (threadIdx.x == 0) s_item = (long long)atomicAdd(counter, 1ull);
    __syncthreads();
    const long long item = s_item;
    __syncthreads();
    if (item >= total) break;
    int j = 0;
    while (j + 1 < njobs && jobs[j + 1].d.item_begin <= item) ++j;
    const FusedJob& J = jobs[j];
    const DrrParams& P = J.d.p;
    const long long local = item - J.d.item_begin;
    const int64_t proj = (int64_t)(local % P.num_projs);
    const int tile = (int)(local / P.num_projs);
    const int ty = tile / J.d.tiles_x, tx = tile - ty * J.d.tiles_x;
    // the job's block shape (as drr_kernel): bw warps across, each warp 8x4
    // pixels (or 4x8 when tall)
    const int bw = P.block_warps_x, wl = P.warp_tall ? 2 : 3;
    const int wc = 1 << wl, wr = 32 >> wl, tw = wc * bw, th = (8 / bw) * wr;
    const int col = tx * tw + (warp % bw) * wc + (lane & (wc - 1));
    const int row = ty * th + (warp / bw) * wr + (lane >> wl);
    unsigned int nl;
    if (col < P.cols && row < P.rows) trace_pixel<VT, XR_LINE_INT_SUM, LAYOUT, UNROLL>(P, proj, row, col, &nl);
    if (!J.metric) continue;
    __threadfence();  // this block's DRR pixels, visible device-wide before they are counted
    __syncthreads();
    const int mt = J.mt_x * J.mt_y;
    if (threadIdx.x == 0)
      s_nclaim = fused_count_tile(J, J.cnt + proj * mt, ty * th, min(ty * th + th, P.rows), tx * tw,
                                  min(tx * tw + tw, P.cols), tw, th, s_claim);
    __syncthreads();
    const int nclaim = s_nclaim;
    for (int c = 0; c < nclaim; ++c) {
      __threadfence();
      const bool last = fused_metric_tile(J, proj, s_claim[c], s_red);
      if (threadIdx.x == 0) s_last = last;
      __syncthreads();
      if (s_last) fused_metric_image(J, proj, s_dred);  // every tile of this image is in
      __syncthreads();
    }
  }
}

// One launch over several jobs without a work counter: blockIdx.x numbers
// every job's (tile, projection) items in the multi-job kernel's order and
// the hardware block scheduler hands them out; each block is one tile in its
// job's block shape, as drr_kernel.  Each job runs the sample loop its caster's
// tuner chose (J.p.unroll: loop 3, 4 or, PACKED, 6), at 64 registers (4
// blocks per SM; measured 3.4% faster than 48 on an uneven set of 8 jobs).
// GROUPED: every job's items are pose groups (MultiJobDrr::pose_group); a
// separate instantiation, so the per-projection kernels keep their registers.
template <int VT, int LAYOUT, bool PACKED, bool GROUPED>
__global__ void __launch_bounds__(kThreads, kMinBlocksPerSM - 2)
drr_jobs_kernel(const MultiJobDrr* __restrict__ jobs, int njobs, long long item0) {
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const long long item = item0 + blockIdx.x;
  int lo = 0, hi = njobs - 1;  // last job whose items start at or before this one
  while (lo < hi) {
    const int mid = (lo + hi + 1) >> 1;
    if (jobs[mid].item_begin <= item) lo = mid; else hi = mid - 1;
  }
  const MultiJobDrr& J = jobs[lo];
  const long long local = item - J.item_begin;
  const long long nproj = J.p.num_projs;
  int64_t proj;
  int col, row;
  if constexpr (GROUPED) {
    // 4 consecutive projections x an 8x8-pixel tile.  When the 4 share a camera
    // and the tile's central ray meets the volume at nearly the same cells under
    // all 4 poses (late CMA-ES generations), their rays through a pixel nearly
    // coincide: each warp takes a 2x4-pixel sub-tile under all 4 poses, so its
    // lanes share cells; otherwise each pair of warps takes one projection's
    // tile.  The rays and their values are the same either way.
    const long long ngrp = (nproj + 3) / 4;
    const int64_t p0 = (int64_t)(local % ngrp) * 4;
    const int tile = (int)(local / ngrp);
    const int ty = tile / J.tiles_x, tx = tile - ty * J.tiles_x;
    bool coherent = p0 + 3 < nproj;
    if (coherent) {
      // where the tile's central ray of the first pose enters and leaves the
      // volume, in that pose's camera coordinates; the other poses' camera ->
      // index affines must put those points within a voxel of it (the
      // deviation is affine, so the segment's ends bound it along the ray)
      const ProjGeom& g0 = J.p.geo[p0];
      const float maxb[3] = {(float)(J.p.vol.nx - 1), (float)(J.p.vol.ny - 1), (float)(J.p.vol.nz - 1)};
      float st0[3], stv[3], quot;
      const int cc = min(tx * 8 + 4, J.p.cols - 1), rc = min(ty * 8 + 4, J.p.rows - 1);
      coherent = xf::ray_setup(g0, (float)cc, (float)rc, maxb, J.p.step, st0, stv, quot) && quot < 1.0e6f;
      if (coherent) {
        xf::Affine M0, Mi;
        for (int k = 0; k < 9; ++k) M0.L[k] = g0.M[k];
        for (int k = 0; k < 3; ++k) M0.t[k] = g0.M[9 + k];
        xf::inverse(M0, Mi);
        float ends[2][3], cam[2][3];
        for (int k = 0; k < 3; ++k) {
          ends[0][k] = st0[k];
          ends[1][k] = st0[k] + quot * stv[k];
        }
        xf::apply(Mi, ends[0], cam[0]);
        xf::apply(Mi, ends[1], cam[1]);
        float dev = 0.0f;
        for (int q = 1; q < 4; ++q) {
          const ProjGeom& g = J.p.geo[p0 + q];
          coherent = coherent && J.p.cam_idx[p0 + q] == J.p.cam_idx[p0];
          for (int e = 0; e < 2; ++e)
            for (int i = 0; i < 3; ++i) {
              const float v = g.M[3 * i] * cam[e][0] + g.M[3 * i + 1] * cam[e][1] + g.M[3 * i + 2] * cam[e][2] +
                              g.M[9 + i];
              dev = fmaxf(dev, fabsf(v - ends[e][i]));
            }
        }
        coherent = coherent && dev < 1.0f;
      }
    }
    int q;
    if (coherent) {
      q = lane >> 3;
      col = tx * 8 + (warp & 3) * 2 + (lane & 1);
      row = ty * 8 + (warp >> 2) * 4 + ((lane & 7) >> 1);
    } else {
      q = warp >> 1;
      col = tx * 8 + (lane & 7);
      row = ty * 8 + (warp & 1) * 4 + (lane >> 3);
    }
    proj = p0 + q;
    if (proj >= nproj) return;
  } else {
    proj = (int64_t)(local % nproj);
    const int tile = (int)(local / nproj);
    const int ty = tile / J.tiles_x, tx = tile - ty * J.tiles_x;
    const int bw = J.p.block_warps_x, wl = J.p.warp_tall ? 2 : 3;
    const int wc = 1 << wl, wr = 32 >> wl;
    col = tx * (wc * bw) + (warp % bw) * wc + (lane & (wc - 1));
    row = ty * ((8 / bw) * wr) + (warp / bw) * wr + (lane >> wl);
  }
  if (col >= J.p.cols || row >= J.p.rows) return;
  unsigned int nl;
  const int loop = J.p.unroll;
  if (loop == kUnrollMacroSkip)
    trace_pixel<VT, XR_LINE_INT_SUM, LAYOUT, kUnrollMacroSkip>(J.p, proj, row, col, &nl);
  else if (PACKED && loop == kUnrollPacked)
    trace_pixel<VT, XR_LINE_INT_SUM, LAYOUT, PACKED ? kUnrollPacked : kUnrollTrim4>(J.p, proj, row, col, &nl);
  else
    trace_pixel<VT, XR_LINE_INT_SUM, LAYOUT, kUnrollTrim4>(J.p, proj, row, col, &nl);
}

constexpr int kMaxDevices = 64;

template <int VT, int LAYOUT, int UNROLL>
cudaError_t launch_fused_t(const FusedJob* d_jobs, int njobs, long long total, unsigned long long* d_counter,
                           int* blocks_out, cudaStream_t s) {
  static std::atomic<int> cached[kMaxDevices];  // blocks per device; zero = not known yet
  int dev = 0, sms = 0, per_sm = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= kMaxDevices) return cudaErrorInvalidDevice;
  int blocks = cached[dev].load(std::memory_order_relaxed);
  if (!blocks) {
    // the kernel's shared memory is small: the smallest carve-out that holds
    // every resident block leaves the rest of the SM's unified L1 to the gathers
    cudaFuncAttributes fa{};
    int smem_sm = 0;
    cudaError_t e = cudaFuncGetAttributes(&fa, eval_fused_kernel<VT, LAYOUT, UNROLL>);
    if (e == cudaSuccess) e = cudaDeviceGetAttribute(&smem_sm, cudaDevAttrMaxSharedMemoryPerMultiprocessor, dev);
    if (e != cudaSuccess) return e;
    const double need = (double)(fa.sharedSizeBytes + 1024) * (kMinBlocksPerSM - 1);
    const int pct = std::min(100, (int)std::ceil(100.0 * need / (double)std::max(smem_sm, 1)) + 1);
    e = cudaFuncSetAttribute(eval_fused_kernel<VT, LAYOUT, UNROLL>, cudaFuncAttributePreferredSharedMemoryCarveout, pct);
    if (e != cudaSuccess) return e;
    e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    if (e != cudaSuccess) return e;
    e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, eval_fused_kernel<VT, LAYOUT, UNROLL>, kThreads, 0);
    if (e != cudaSuccess) return e;
    blocks = sms * (per_sm > 0 ? per_sm : 1);
    cached[dev].store(blocks, std::memory_order_relaxed);
  }
  *blocks_out = blocks;
  cudaError_t e = cudaMemsetAsync(d_counter, 0, sizeof(unsigned long long), s);
  if (e != cudaSuccess) return e;
  eval_fused_kernel<VT, LAYOUT, UNROLL><<<blocks, kThreads, 0, s>>>(d_jobs, njobs, total, d_counter);
  return cudaGetLastError();
}

template <int VT, int LAYOUT, bool PACKED, bool GROUPED>
cudaError_t launch_jobs_g(const MultiJobDrr* d_jobs, int njobs, long long total, cudaStream_t s) {
  static std::atomic<bool> carveout_set[kMaxDevices];
  int dev = 0;
  if (cudaGetDevice(&dev) == cudaSuccess && dev >= 0 && dev < kMaxDevices &&
      !carveout_set[dev].load(std::memory_order_relaxed)) {
    cudaFuncSetAttribute(drr_jobs_kernel<VT, LAYOUT, PACKED, GROUPED>, cudaFuncAttributePreferredSharedMemoryCarveout,
                         (int)cudaSharedmemCarveoutMaxL1);
    carveout_set[dev].store(true, std::memory_order_relaxed);
  }
  const long long max_x = 0x7fffffff;
  for (long long base = 0; base < total; base += max_x) {
    const long long n = (total - base) < max_x ? (total - base) : max_x;
    drr_jobs_kernel<VT, LAYOUT, PACKED, GROUPED><<<(unsigned)n, kThreads, 0, s>>>(d_jobs, njobs, base);
  }
  return cudaGetLastError();
}

template <int VT, int LAYOUT, bool PACKED>
cudaError_t launch_jobs_t(const MultiJobDrr* d_jobs, int njobs, long long total, bool grouped, cudaStream_t s) {
  return grouped ? launch_jobs_g<VT, LAYOUT, PACKED, true>(d_jobs, njobs, total, s)
                 : launch_jobs_g<VT, LAYOUT, PACKED, false>(d_jobs, njobs, total, s);
}

template <int VT, int KERNEL, int LAYOUT, int UNROLL>
cudaError_t launch_t(const DrrParams& p, cudaStream_t s) {
  // The kernel uses no shared memory: ask for the largest L1 (the gathers hit
  // it), once per device (a preference; setting it twice is harmless).
  static std::atomic<bool> carveout_set[kMaxDevices];
  int dev = 0;
  if (cudaGetDevice(&dev) == cudaSuccess && dev >= 0 && dev < kMaxDevices &&
      !carveout_set[dev].load(std::memory_order_relaxed)) {
    cudaFuncSetAttribute(drr_kernel<VT, KERNEL, LAYOUT, UNROLL>, cudaFuncAttributePreferredSharedMemoryCarveout,
                         (int)cudaSharedmemCarveoutMaxL1);
    carveout_set[dev].store(true, std::memory_order_relaxed);
  }
  const int bw = p.block_warps_x;
  const int wc = p.warp_tall ? 4 : 8;
  const int tx = wc * bw, ty = (8 / bw) * (32 / wc);
  const int64_t max_x = 0x7fffffff;
  for (int64_t base = 0; base < p.num_projs; base += max_x) {
    const int64_t n = (p.num_projs - base) < max_x ? (p.num_projs - base) : max_x;
    const dim3 grid((unsigned)n, (p.cols + tx - 1) / tx, (p.rows + ty - 1) / ty);
    drr_kernel<VT, KERNEL, LAYOUT, UNROLL><<<grid, kThreads, 0, s>>>(p, base);
  }
  return cudaGetLastError();
}

template <int VT, int KERNEL, int LAYOUT>
cudaError_t launch_unroll(const DrrParams& p, cudaStream_t s) {
  if (p.unroll >= kUnrollMacroSkip) {
    // the macro-cell trim exists for the sum kernel; the maximum kernel runs the
    // plain two-sample loop, which gives the same image; the shared-cell pair
    // loop exists for the 256-bit float32 CELL8 read (elsewhere loop 3 runs)
    if constexpr (KERNEL == XR_LINE_INT_SUM) {
      if (p.unroll == kUnrollTrim4) return launch_t<VT, KERNEL, LAYOUT, kUnrollTrim4>(p, s);
      if constexpr ((LAYOUT == kLayoutCell8Wide && VT == XR_VOXEL_F32) ||
                    (LAYOUT == XR_LAYOUT_CELL8 && VT != XR_VOXEL_F32))
        if (p.unroll == kUnrollPacked) return launch_t<VT, KERNEL, LAYOUT, kUnrollPacked>(p, s);
      if (p.unroll == kUnrollPacked) return launch_t<VT, KERNEL, LAYOUT, kUnrollTrim4>(p, s);
      if constexpr (LAYOUT == kLayoutCell8Wide && VT == XR_VOXEL_F32)
        if (p.unroll == kUnrollPairShare) return launch_t<VT, KERNEL, LAYOUT, kUnrollPairShare>(p, s);
      return launch_t<VT, KERNEL, LAYOUT, kUnrollMacroSkip>(p, s);
    }
    return launch_t<VT, KERNEL, LAYOUT, 2>(p, s);
  }
  return p.unroll == 2 ? launch_t<VT, KERNEL, LAYOUT, 2>(p, s) : launch_t<VT, KERNEL, LAYOUT, 1>(p, s);
}

template <int VT, int KERNEL>
cudaError_t launch_layout(const DrrParams& p, cudaStream_t s) {
  if (p.vol.layout == kLayoutCell8Wide) {
    if constexpr (VT == XR_VOXEL_F32) return launch_unroll<VT, KERNEL, kLayoutCell8Wide>(p, s);
    return cudaErrorInvalidValue;
  }
  if (p.vol.layout == XR_LAYOUT_CELL8) return launch_unroll<VT, KERNEL, XR_LAYOUT_CELL8>(p, s);
  return launch_unroll<VT, KERNEL, XR_LAYOUT_LINEAR>(p, s);
}

template <int VT>
cudaError_t launch_kernel_id(const DrrParams& p, cudaStream_t s) {
  return p.kernel_id == XR_LINE_INT_MAX ? launch_layout<VT, XR_LINE_INT_MAX>(p, s)
                                        : launch_layout<VT, XR_LINE_INT_SUM>(p, s);
}

// One thread per cell (x fastest, so the voxel reads coalesce): gathers the 8
// corners from the float32 voxels and stores them as cell number
// ix csx + iy csy + iz (z fastest).
template <int VT>
__global__ void build_cells_kernel(const float* __restrict__ vox, int nx, int ny, int nz, float scale, int32_t csx,
                                   int32_t csy, void* out) {
  const int64_t ncx = nx - 1, ncy = ny - 1, ncz = nz - 1;
  const int64_t ncell = ncx * ncy * ncz;
  for (int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; t < ncell; t += (int64_t)gridDim.x * blockDim.x) {
    const int64_t ix = t % ncx, iy = (t / ncx) % ncy, iz = t / (ncx * ncy);
    const int64_t c = ix * csx + iy * csy + iz;
    const int64_t b = (iz * ny + iy) * nx + ix, sy = nx, sz = (int64_t)nx * ny;
    // z-pairs: v000 v001 v100 v101 v010 v011 v110 v111 (vxyz)
    const float v[8] = {vox[b], vox[b + sz], vox[b + 1], vox[b + sz + 1],
                        vox[b + sy], vox[b + sz + sy], vox[b + sy + 1], vox[b + sz + sy + 1]};
    if (VT == XR_VOXEL_F32) {
      float4* o = static_cast<float4*>(out) + 2 * c;
      o[0] = make_float4(v[0], v[1], v[2], v[3]);
      o[1] = make_float4(v[4], v[5], v[6], v[7]);
    } else {
      uint4 q;
      unsigned int* w = &q.x;
      for (int k = 0; k < 4; ++k) {
        if (VT == XR_VOXEL_F16) {
          __half2 h = __floats2half2_rn(v[2 * k] * scale, v[2 * k + 1] * scale);
          w[k] = *reinterpret_cast<unsigned int*>(&h);
        } else {
          __nv_bfloat162 h = __floats2bfloat162_rn(v[2 * k] * scale, v[2 * k + 1] * scale);
          w[k] = *reinterpret_cast<unsigned int*>(&h);
        }
      }
      static_cast<uint4*>(out)[c] = q;
    }
  }
}

}  // namespace

cudaError_t launch_brick(const DrrParams& p, cudaStream_t s) {
  if (p.vol.voxel_type != XR_VOXEL_F32 || !p.vol.cells || p.kernel_id != XR_LINE_INT_SUM) return cudaErrorInvalidValue;
  static std::atomic<bool> carveout_set[kMaxDevices];
  int dev = 0;
  if (cudaGetDevice(&dev) == cudaSuccess && dev >= 0 && dev < kMaxDevices &&
      !carveout_set[dev].load(std::memory_order_relaxed)) {
    // four resident blocks of 44 KB each, the rest of the SM's unified L1 for the global reads
    cudaFuncSetAttribute(drr_brick_kernel, cudaFuncAttributePreferredSharedMemoryCarveout, 80);
    carveout_set[dev].store(true, std::memory_order_relaxed);
  }
  const int64_t max_x = 0x7fffffff;
  for (int64_t base = 0; base < p.num_projs; base += max_x) {
    const int64_t n = (p.num_projs - base) < max_x ? (p.num_projs - base) : max_x;
    const dim3 grid((unsigned)n, (p.cols + 15) / 16, (p.rows + 15) / 16);
    drr_brick_kernel<<<grid, kThreads, 0, s>>>(p, base);
  }
  return cudaGetLastError();
}

cudaError_t launch_drr(const DrrParams& p, cudaStream_t s) {
  if (p.num_projs <= 0) return cudaSuccess;
  if (p.vol.layout == kLayoutBrick) return launch_brick(p, s);
  if (!(p.block_warps_x == 1 || p.block_warps_x == 2 || p.block_warps_x == 4 || p.block_warps_x == 8))
    return cudaErrorInvalidValue;
  if (p.warp_tall != 0 && p.warp_tall != 1) return cudaErrorInvalidValue;
  if (p.vol.layout != XR_LAYOUT_LINEAR && !p.vol.cells) return cudaErrorInvalidValue;
  if (p.vol.layout == kLayoutCell8Wide && p.vol.voxel_type != XR_VOXEL_F32) return cudaErrorInvalidValue;
  switch (p.vol.voxel_type) {
    case XR_VOXEL_F32: return launch_kernel_id<XR_VOXEL_F32>(p, s);
    case XR_VOXEL_F16: return launch_kernel_id<XR_VOXEL_F16>(p, s);
    case XR_VOXEL_BF16: return launch_kernel_id<XR_VOXEL_BF16>(p, s);
    default: return cudaErrorInvalidValue;
  }
}

// Marks macro cell m occupied when any trilinear cell in it has a non-zero
// corner: voxel (x, y, z) is a corner of cells x-1..x, y-1..y, z-1..z.
// Dilated macro-cell occupancy: bit m is set when some trilinear cell with base
// index in [8m - 1, 8m + 8] on every axis has a non-zero corner, i.e. some
// non-zero voxel lies in [8m - 1, 8m + 9].
__global__ void occupancy_kernel(const float* __restrict__ vox, int nx, int ny, int nz, uint32_t* occ, int nmx,
                                 int nmy, int nmz) {
  const int64_t n = (int64_t)nx * ny * nz;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    if (vox[i] == 0.0f) continue;
    const int x = (int)(i % nx), y = (int)((i / nx) % ny), z = (int)(i / ((int64_t)nx * ny));
    const int x0 = max(x - 2, 0) >> kMacroShift, x1 = min((x + 1) >> kMacroShift, nmx - 1);
    const int y0 = max(y - 2, 0) >> kMacroShift, y1 = min((y + 1) >> kMacroShift, nmy - 1);
    const int z0 = max(z - 2, 0) >> kMacroShift, z1 = min((z + 1) >> kMacroShift, nmz - 1);
    for (int mz = z0; mz <= z1; ++mz)
      for (int my = y0; my <= y1; ++my)
        for (int mx = x0; mx <= x1; ++mx) {
          const int m = (mz * nmy + my) * nmx + mx;
          const uint32_t bit = 1u << (m & 31);
          if (!(occ[m >> 5] & bit)) atomicOr(&occ[m >> 5], bit);
        }
  }
}

__global__ void support_init_kernel(int* box) {
  if (threadIdx.x < 3) box[threadIdx.x] = 0x7fffffff;
  else if (threadIdx.x < 6) box[threadIdx.x] = -1;
}

// Index bounds of the non-zero voxels: box = (min x, min y, min z, max x, max y, max z).
__global__ void support_box_kernel(const float* __restrict__ vox, int nx, int ny, int nz, int* box) {
  int mn[3] = {0x7fffffff, 0x7fffffff, 0x7fffffff}, mx[3] = {-1, -1, -1};
  const int64_t n = (int64_t)nx * ny * nz;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    if (vox[i] != 0.0f) {
      const int x = (int)(i % nx), y = (int)((i / nx) % ny), z = (int)(i / ((int64_t)nx * ny));
      mn[0] = min(mn[0], x); mn[1] = min(mn[1], y); mn[2] = min(mn[2], z);
      mx[0] = max(mx[0], x); mx[1] = max(mx[1], y); mx[2] = max(mx[2], z);
    }
  }
  for (int k = 0; k < 3; ++k) {
    for (int o = 16; o > 0; o >>= 1) {
      mn[k] = min(mn[k], __shfl_down_sync(0xffffffffu, mn[k], o));
      mx[k] = max(mx[k], __shfl_down_sync(0xffffffffu, mx[k], o));
    }
  }
  if ((threadIdx.x & 31) == 0) {
    for (int k = 0; k < 3; ++k) {
      atomicMin(&box[k], mn[k]);
      atomicMax(&box[3 + k], mx[k]);
    }
  }
}

cudaError_t launch_build_occupancy(const float* vox_f32, int nx, int ny, int nz, uint32_t* d_occ, int nmx, int nmy,
                                   int nmz, cudaStream_t s) {
  const size_t words = ((size_t)nmx * nmy * nmz + 31) / 32;
  cudaError_t e = cudaMemsetAsync(d_occ, 0, words * sizeof(uint32_t), s);
  if (e != cudaSuccess) return e;
  occupancy_kernel<<<2048, 256, 0, s>>>(vox_f32, nx, ny, nz, d_occ, nmx, nmy, nmz);
  return cudaGetLastError();
}

cudaError_t launch_support_box(const float* vox_f32, int nx, int ny, int nz, int* d_box, cudaStream_t s) {
  support_init_kernel<<<1, 32, 0, s>>>(d_box);
  support_box_kernel<<<2048, 256, 0, s>>>(vox_f32, nx, ny, nz, d_box);
  return cudaGetLastError();
}

cudaError_t launch_eval_fused(const FusedJob* d_jobs, int njobs, long long total, int32_t voxel_type, int32_t layout,
                              int32_t unroll, unsigned long long* d_counter, int* blocks_out, cudaStream_t s) {
  *blocks_out = 0;
  if (total <= 0) return cudaSuccess;
  const bool packed = unroll == kUnrollPacked;
  switch (voxel_type * 4 + layout) {
    case XR_VOXEL_F32 * 4 + XR_LAYOUT_LINEAR:
      return launch_fused_t<XR_VOXEL_F32, XR_LAYOUT_LINEAR, kUnrollTrim4>(d_jobs, njobs, total, d_counter, blocks_out, s);
    case XR_VOXEL_F32 * 4 + kLayoutCell8Wide:
      return packed ? launch_fused_t<XR_VOXEL_F32, kLayoutCell8Wide, kUnrollPacked>(d_jobs, njobs, total, d_counter,
                                                                                   blocks_out, s)
                    : launch_fused_t<XR_VOXEL_F32, kLayoutCell8Wide, kUnrollTrim4>(d_jobs, njobs, total, d_counter,
                                                                                  blocks_out, s);
    case XR_VOXEL_F16 * 4 + XR_LAYOUT_LINEAR:
      return launch_fused_t<XR_VOXEL_F16, XR_LAYOUT_LINEAR, kUnrollTrim4>(d_jobs, njobs, total, d_counter, blocks_out, s);
    case XR_VOXEL_F16 * 4 + XR_LAYOUT_CELL8:
      return launch_fused_t<XR_VOXEL_F16, XR_LAYOUT_CELL8, kUnrollTrim4>(d_jobs, njobs, total, d_counter, blocks_out, s);
    case XR_VOXEL_BF16 * 4 + XR_LAYOUT_LINEAR:
      return launch_fused_t<XR_VOXEL_BF16, XR_LAYOUT_LINEAR, kUnrollTrim4>(d_jobs, njobs, total, d_counter, blocks_out, s);
    case XR_VOXEL_BF16 * 4 + XR_LAYOUT_CELL8:
      return packed ? launch_fused_t<XR_VOXEL_BF16, XR_LAYOUT_CELL8, kUnrollPacked>(d_jobs, njobs, total, d_counter,
                                                                                   blocks_out, s)
                    : launch_fused_t<XR_VOXEL_BF16, XR_LAYOUT_CELL8, kUnrollTrim4>(d_jobs, njobs, total, d_counter,
                                                                                  blocks_out, s);
    default:
      return cudaErrorInvalidValue;
  }
}

cudaError_t launch_drr_jobs(const MultiJobDrr* d_jobs, int njobs, long long total, int32_t voxel_type, int32_t layout,
                            bool grouped, cudaStream_t s) {
  if (total <= 0) return cudaSuccess;
  switch (voxel_type * 4 + layout) {
    case XR_VOXEL_F32 * 4 + XR_LAYOUT_LINEAR:
      return launch_jobs_t<XR_VOXEL_F32, XR_LAYOUT_LINEAR, false>(d_jobs, njobs, total, grouped, s);
    case XR_VOXEL_F32 * 4 + kLayoutCell8Wide:
      return launch_jobs_t<XR_VOXEL_F32, kLayoutCell8Wide, true>(d_jobs, njobs, total, grouped, s);
    case XR_VOXEL_F16 * 4 + XR_LAYOUT_LINEAR:
      return launch_jobs_t<XR_VOXEL_F16, XR_LAYOUT_LINEAR, false>(d_jobs, njobs, total, grouped, s);
    case XR_VOXEL_F16 * 4 + XR_LAYOUT_CELL8:
      return launch_jobs_t<XR_VOXEL_F16, XR_LAYOUT_CELL8, true>(d_jobs, njobs, total, grouped, s);
    case XR_VOXEL_BF16 * 4 + XR_LAYOUT_LINEAR:
      return launch_jobs_t<XR_VOXEL_BF16, XR_LAYOUT_LINEAR, false>(d_jobs, njobs, total, grouped, s);
    case XR_VOXEL_BF16 * 4 + XR_LAYOUT_CELL8:
      return launch_jobs_t<XR_VOXEL_BF16, XR_LAYOUT_CELL8, true>(d_jobs, njobs, total, grouped, s);
    default:
      return cudaErrorInvalidValue;
  }
}

size_t cell_layout_bytes(int64_t nx, int64_t ny, int64_t nz, int32_t voxel_type) {
  const size_t ncell = (size_t)(nx - 1) * (size_t)(ny - 1) * (size_t)(nz - 1);
  return ncell * (voxel_type == XR_VOXEL_F32 ? 32 : 16);
}

cudaError_t launch_build_cells(const float* vox_f32, int nx, int ny, int nz, int32_t voxel_type, float scale,
                               void* out, cudaStream_t s) {
  int32_t cs[2];
  cell_strides(nx, ny, nz, cs);
  switch (voxel_type) {
    case XR_VOXEL_F32:
      build_cells_kernel<XR_VOXEL_F32><<<2048, 256, 0, s>>>(vox_f32, nx, ny, nz, 1.0f, cs[0], cs[1], out);
      break;
    case XR_VOXEL_F16:
      build_cells_kernel<XR_VOXEL_F16><<<2048, 256, 0, s>>>(vox_f32, nx, ny, nz, scale, cs[0], cs[1], out);
      break;
    case XR_VOXEL_BF16:
      build_cells_kernel<XR_VOXEL_BF16><<<2048, 256, 0, s>>>(vox_f32, nx, ny, nz, scale, cs[0], cs[1], out);
      break;
    default: return cudaErrorInvalidValue;
  }
  return cudaGetLastError();
}

void cell_strides(int64_t nx, int64_t ny, int64_t nz, int32_t cs[2]) {
  (void)ny;
  const int32_t cx = (int32_t)(nx - 1), cz = (int32_t)(nz - 1);
  cs[0] = cz;       // x
  cs[1] = cz * cx;  // y
}

}  // namespace xr
