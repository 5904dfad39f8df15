// xr_xfloat.h -- xReg's float geometry, operation by operation (host and device).
//
// xReg keeps poses, camera models and the index <-> physical transform as
// Eigen float objects (CoordScalar = float, FrameTransform =
// Eigen::Transform<float,3,Affine>: xregCommon.h:44-65) and sets up every ray in
// float (xregRayCastLineIntCPU.cpp:196-259).  One sample more or less on a ray
// changes a DRR pixel by about 1/300, far outside the 1e-4 tolerance, so the
// ray caster repeats that float arithmetic exactly, in the order Eigen 3.3
// evaluates it:
//   * products and norms of fixed-size 3-element operands (Matrix3f * Vector3f,
//     the linear parts in Transform * Transform, Vector3f::norm / normalized)
//     are unrolled reductions that split a length-3 sum as 1 + 2:
//     a0 + (a1 + a2);
//   * Transform * Vector3f is the 4x4 matrix times [p; 1], a sum of columns on
//     SSE packets: ((a0 + a1) + a2) + t;
//   * a product through a runtime-sized block (Matrix4f::block(0, 0, 3, 3) * v
//     and the norm of its result, the blocks of SE3Inv) is a plain loop:
//     (a0 + a1) + a2;
//   * Matrix3f::inverse is the adjugate: cofactors, determinant from the first
//     column (fixed-size order), one division 1 / det, cofactor * (1 / det);
//   * Vector::normalized divides each component by sqrt of the squared norm;
//   * Eigen's default vectorisation on x86-64 (SSE2, 4-float packets) and no
//     multiply-add contraction (the reference's build sets no -march, so the
//     compiler has no FMA instruction to contract into).
// Device code uses explicitly rounded intrinsics; host code is compiled with
// -ffp-contract=off, so both give the same bits.
#pragma once

#include <cmath>
#include <cstdint>

#if defined(__CUDACC__)
#define XF_HD __host__ __device__ __forceinline__
#else
#define XF_HD inline
#endif

namespace xr {
namespace xf {

XF_HD float mul(float a, float b) {
#if defined(__CUDA_ARCH__)
  return __fmul_rn(a, b);
#else
  return a * b;
#endif
}
XF_HD float add(float a, float b) {
#if defined(__CUDA_ARCH__)
  return __fadd_rn(a, b);
#else
  return a + b;
#endif
}
XF_HD float sub(float a, float b) {
#if defined(__CUDA_ARCH__)
  return __fsub_rn(a, b);
#else
  return a - b;
#endif
}
XF_HD float div(float a, float b) {
#if defined(__CUDA_ARCH__)
  return __fdiv_rn(a, b);
#else
  return a / b;
#endif
}
XF_HD float sqrt(float a) {
#if defined(__CUDA_ARCH__)
  return __fsqrt_rn(a);
#else
  return std::sqrt(a);
#endif
}

// a0 b0 + (a1 b1 + a2 b2): fixed-size length-3 reduction.
XF_HD float dot_fixed(float a0, float a1, float a2, float b0, float b1, float b2) {
  return add(mul(a0, b0), add(mul(a1, b1), mul(a2, b2)));
}
// (a0 b0 + a1 b1) + a2 b2: runtime-sized length-3 reduction.
XF_HD float dot_loop(float a0, float a1, float a2, float b0, float b1, float b2) {
  return add(add(mul(a0, b0), mul(a1, b1)), mul(a2, b2));
}

// Affine 3-D transform: linear part L (row-major 3x3) and translation t.
struct Affine {
  float L[9];
  float t[3];
};

// Matrix3f::inverse (adjugate over the determinant).
XF_HD void inv3(const float m[9], float out[9]) {
  // cofactor (i, j) = m(i1, j1) m(i2, j2) - m(i1, j2) m(i2, j1), i1 = i+1, i2 = i+2 (mod 3)
  float cof[9];
  for (int i = 0; i < 3; ++i) {
    const int i1 = (i + 1) % 3, i2 = (i + 2) % 3;
    for (int j = 0; j < 3; ++j) {
      const int j1 = (j + 1) % 3, j2 = (j + 2) % 3;
      cof[i * 3 + j] = sub(mul(m[i1 * 3 + j1], m[i2 * 3 + j2]), mul(m[i1 * 3 + j2], m[i2 * 3 + j1]));
    }
  }
  const float det = dot_fixed(cof[0], cof[3], cof[6], m[0], m[3], m[6]);
  const float invdet = div(1.0f, det);
  for (int r = 0; r < 3; ++r)
    for (int c = 0; c < 3; ++c) out[r * 3 + c] = mul(cof[c * 3 + r], invdet);
}

// Transform * Vector3f.  Eigen 3.3 multiplies the 4x4 matrix by [p; 1] as a
// sum of columns on SSE packets: ((L0 p0 + L1 p1) + L2 p2) + t.
XF_HD void apply(const Affine& a, const float p[3], float out[3]) {
  float o[3];
  for (int i = 0; i < 3; ++i) o[i] = add(dot_loop(a.L[i * 3], a.L[i * 3 + 1], a.L[i * 3 + 2], p[0], p[1], p[2]), a.t[i]);
  out[0] = o[0]; out[1] = o[1]; out[2] = o[2];
}

// Transform * Transform (both affine): L = La Lb, t = La tb + ta.
XF_HD void compose(const Affine& a, const Affine& b, Affine& out) {
  Affine r;
  for (int i = 0; i < 3; ++i) {
    for (int j = 0; j < 3; ++j)
      r.L[i * 3 + j] = dot_fixed(a.L[i * 3], a.L[i * 3 + 1], a.L[i * 3 + 2], b.L[j], b.L[3 + j], b.L[6 + j]);
    r.t[i] = add(dot_fixed(a.L[i * 3], a.L[i * 3 + 1], a.L[i * 3 + 2], b.t[0], b.t[1], b.t[2]), a.t[i]);
  }
  out = r;
}

// Transform::inverse(Affine): L^-1 and -(L^-1 t) (fixed-size blocks).
XF_HD void inverse(const Affine& a, Affine& out) {
  Affine r;
  inv3(a.L, r.L);
  for (int i = 0; i < 3; ++i)
    r.t[i] = -dot_fixed(r.L[i * 3], r.L[i * 3 + 1], r.L[i * 3 + 2], a.t[0], a.t[1], a.t[2]);
  out = r;
}

// SE3Inv (xregRigidUtils.cpp:29-38): R^T and (-1 R^T) t through runtime-sized blocks.
XF_HD void se3_inv(const Affine& e, Affine& out) {
  Affine r;
  for (int i = 0; i < 3; ++i)
    for (int j = 0; j < 3; ++j) r.L[i * 3 + j] = e.L[j * 3 + i];
  for (int i = 0; i < 3; ++i) r.t[i] = -dot_loop(r.L[i * 3], r.L[i * 3 + 1], r.L[i * 3 + 2], e.t[0], e.t[1], e.t[2]);
  out = r;
}

// Camera model as xReg holds it, in float.
struct Camera {
  float K[9];           // intrins
  float E[16];          // extrins (row-major 4x4; rigid)
  float focal_len;
  int32_t frame;        // 0 focal point +z, 1 focal point -z, 2 on detector
};

// Per-projection set-up: what xReg evaluates for every ray of a projection and
// gets the same result for each (176 bytes).
struct RayFrame {
  float M[12];       // camera -> ITK index: L row-major, then t
  float pin_idx[3];  // pinhole in index coordinates (M * pinhole)
  float Ki[9];       // intrins_inv
  float dz;          // det_z_val: -focal_len (-z frame) or +focal_len
  float zadj;        // z component of z_adjust (-focal_len for the on-detector frame, else 0)
  float Ei[12];      // extrins_inv: L row-major, then t
  float pin[3];      // pinhole_pt in camera-world coordinates
  float pad[3];
};

// CameraModel::setup(K, E, ...) derived members (xregPerspectiveXform.cpp:302-334)
// and the per-projection transform xform_cam_to_itk_idx = phys_to_idx * pose
// (xregRayCastLineIntCPU.cpp:206-212).
XF_HD void ray_frame(const Camera& cam, const Affine& phys_to_idx, const Affine& pose, RayFrame& g) {
  float Ki[9];
  inv3(cam.K, Ki);
  Affine E;
  for (int i = 0; i < 3; ++i) {
    for (int j = 0; j < 3; ++j) E.L[i * 3 + j] = cam.E[i * 4 + j];
    E.t[i] = cam.E[i * 4 + 3];
  }
  Affine Ei;
  se3_inv(E, Ei);
  float pin[3];
  if (cam.frame == 2) {
    const float pz[3] = {0.0f, 0.0f, cam.focal_len};
    apply(Ei, pz, pin);
  } else {
    pin[0] = Ei.t[0]; pin[1] = Ei.t[1]; pin[2] = Ei.t[2];
  }
  Affine M;
  compose(phys_to_idx, pose, M);
  float pi[3];
  apply(M, pin, pi);
  for (int k = 0; k < 9; ++k) { g.M[k] = M.L[k]; g.Ki[k] = Ki[k]; g.Ei[k] = Ei.L[k]; }
  for (int k = 0; k < 3; ++k) {
    g.M[9 + k] = M.t[k];
    g.Ei[9 + k] = Ei.t[k];
    g.pin_idx[k] = pi[k];
    g.pin[k] = pin[k];
    g.pad[k] = 0.0f;
  }
  // ((frame == -z) ? -1 : 1) * focal_len: an exact sign change
  g.dz = cam.frame == 1 ? -cam.focal_len : cam.focal_len;
  g.zadj = cam.frame == 2 ? -cam.focal_len : 0.0f;
}

// One ray of pixel (col, row): the clipped, nudged segment in index space
// (xregRayCastLineIntCPU.cpp:196-259, RayRectIntersect
// xregSpatialPrimitives.cpp:176-221).  Returns false when the ray misses the
// box [0, maxb] or its clipped parameter interval is not longer than 2e-3;
// otherwise start, step vector and num_steps (samples = num_steps + 1; the
// float quotient is returned, the caller truncates it).
XF_HD bool ray_setup(const RayFrame& g, float col, float row, const float maxb[3], float step, float start[3],
                     float stepv[3], float& steps_quot) {
  // cam.ind_pt_to_phys_det_pt: extrins_inv ((intrins_inv (det_z [c r 1])) + z_adjust)
  const float s0 = mul(g.dz, col), s1 = mul(g.dz, row), s2 = mul(g.dz, 1.0f);
  float q[3];
  for (int i = 0; i < 3; ++i) q[i] = dot_fixed(g.Ki[i * 3], g.Ki[i * 3 + 1], g.Ki[i * 3 + 2], s0, s1, s2);
  q[0] = add(q[0], 0.0f);
  q[1] = add(q[1], 0.0f);
  q[2] = add(q[2], g.zadj);
  float det[3];
  for (int i = 0; i < 3; ++i)
    det[i] = add(dot_loop(g.Ei[i * 3], g.Ei[i * 3 + 1], g.Ei[i * 3 + 2], q[0], q[1], q[2]), g.Ei[9 + i]);
  // pinhole -> detector point in index space
  float d[3];
  for (int i = 0; i < 3; ++i) {
    const float di = add(dot_loop(g.M[i * 3], g.M[i * 3 + 1], g.M[i * 3 + 2], det[0], det[1], det[2]), g.M[9 + i]);
    d[i] = sub(di, g.pin_idx[i]);
  }
  // segment-limited slab test; |v| > 1e-8 is a double comparison in the
  // reference, and 1.0e-8f is the largest float not above 1e-8
  float t0 = 0.0f, t1 = 1.0f;
  for (int k = 0; k < 3; ++k) {
    if (fabsf(d[k]) > 1.0e-8f) {
      const float inv = div(1.0f, d[k]);
      float ta = mul(sub(0.0f, g.pin_idx[k]), inv);
      float tb = mul(sub(maxb[k], g.pin_idx[k]), inv);
      if (tb < ta) { const float tmp = ta; ta = tb; tb = tmp; }
      t0 = (t0 < ta) ? ta : t0;
      t1 = (tb < t1) ? tb : t1;
      if (t0 > t1) return false;
    } else if (g.pin_idx[k] < 0.0f || g.pin_idx[k] > maxb[k]) {
      return false;
    }
  }
  if (!(sub(t1, t0) > 2.0e-3f)) return false;
  t0 = add(t0, 1.0e-3f);
  t1 = sub(t1, 1.0e-3f);
  for (int i = 0; i < 3; ++i) start[i] = add(g.pin_idx[i], mul(t0, d[i]));
  const float dlen = sqrt(dot_fixed(d[0], d[1], d[2], d[0], d[1], d[2]));
  const float ilen = mul(sub(t1, t0), dlen);
  // (det - pinhole).normalized() * step, rotated and scaled by M's 3x3 block
  float u[3];
  for (int i = 0; i < 3; ++i) u[i] = sub(det[i], g.pin[i]);
  const float z = dot_fixed(u[0], u[1], u[2], u[0], u[1], u[2]);
  if (z > 0.0f) {
    const float n = sqrt(z);
    for (int i = 0; i < 3; ++i) u[i] = div(u[i], n);
  }
  for (int i = 0; i < 3; ++i) u[i] = mul(u[i], step);
  float w[3];
  for (int i = 0; i < 3; ++i) w[i] = dot_loop(g.M[i * 3], g.M[i * 3 + 1], g.M[i * 3 + 2], u[0], u[1], u[2]);
  const float slen = sqrt(dot_loop(w[0], w[1], w[2], w[0], w[1], w[2]));
  steps_quot = div(ilen, slen);
  const float sc = div(slen, dlen);
  for (int i = 0; i < 3; ++i) stepv[i] = mul(d[i], sc);
  return true;
}

}  // namespace xf
}  // namespace xr
