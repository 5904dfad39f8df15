// xr_geom.cu -- per-projection ray set-up in FP64 on the device.
//
// For every projection p this composes camera -> ITK index space,
//   M = (D * diag(spacing))^-1 * [pose_p] - ...     (xregRayCastLineIntCPU.cpp:207-208,
//                                                     xregITKBasicImageUtils.h:133-165)
// inverts the intrinsic matrix and the rigid extrinsic (xregPerspectiveXform.cpp:230-334),
// builds the pinhole and detector-pixel affine map (xregPerspectiveXform.cpp:401-414)
// and rounds the results to float.  Every double operation is an explicitly
// rounded intrinsic (no contraction into FMA), in a fixed order, so the float
// set-up is bit-identical to the CPU oracle's and the per-ray step counts agree.
#include "xr_internal.h"

namespace xr {
namespace {

__device__ __forceinline__ double dm(double a, double b) { return __dmul_rn(a, b); }
__device__ __forceinline__ double da(double a, double b) { return __dadd_rn(a, b); }
__device__ __forceinline__ double dsb(double a, double b) { return __dsub_rn(a, b); }

__device__ void m3_inverse(const double* a, double* out) {
  const double c00 = dsb(dm(a[4], a[8]), dm(a[5], a[7]));
  const double c01 = dsb(dm(a[5], a[6]), dm(a[3], a[8]));
  const double c02 = dsb(dm(a[3], a[7]), dm(a[4], a[6]));
  const double det = da(da(dm(a[0], c00), dm(a[1], c01)), dm(a[2], c02));
  const double id = __ddiv_rn(1.0, det);
  out[0] = dm(c00, id);
  out[1] = dm(dsb(dm(a[2], a[7]), dm(a[1], a[8])), id);
  out[2] = dm(dsb(dm(a[1], a[5]), dm(a[2], a[4])), id);
  out[3] = dm(c01, id);
  out[4] = dm(dsb(dm(a[0], a[8]), dm(a[2], a[6])), id);
  out[5] = dm(dsb(dm(a[2], a[3]), dm(a[0], a[5])), id);
  out[6] = dm(c02, id);
  out[7] = dm(dsb(dm(a[1], a[6]), dm(a[0], a[7])), id);
  out[8] = dm(dsb(dm(a[0], a[4]), dm(a[1], a[3])), id);
}

__device__ void m3_mul(const double* a, const double* b, double* out) {
  for (int i = 0; i < 3; ++i)
    for (int j = 0; j < 3; ++j)
      out[i * 3 + j] = da(da(dm(a[i * 3 + 0], b[0 * 3 + j]), dm(a[i * 3 + 1], b[1 * 3 + j])),
                          dm(a[i * 3 + 2], b[2 * 3 + j]));
}

__device__ void m3_vec(const double* a, const double* v, double* out) {
  for (int i = 0; i < 3; ++i)
    out[i] = da(da(dm(a[i * 3 + 0], v[0]), dm(a[i * 3 + 1], v[1])), dm(a[i * 3 + 2], v[2]));
}

struct VolSetup {
  double Ai[9];  // physical -> index rotation/scale
  double ti[3];  // physical -> index translation
};

__global__ void proj_geom_kernel(VolSetup vs, const xr_camera_desc* __restrict__ cams,
                                 const double* __restrict__ poses, const int32_t* __restrict__ cam_idx,
                                 int64_t num_projs, int64_t pose_stride, ProjGeom* __restrict__ out) {
  const int64_t p = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= num_projs) return;
  const xr_camera_desc cam = cams[cam_idx[p]];
  // poses are indexed modulo pose_stride: projection p uses pose (p % pose_stride),
  // which implements distribute_xforms_among_cam_models without a host copy.
  const double* pose = poses + 16 * (p % pose_stride);

  double Ki[9];
  m3_inverse(cam.intrins, Ki);
  double ER[9], Et[3];
  for (int i = 0; i < 3; ++i)
    for (int j = 0; j < 3; ++j) ER[i * 3 + j] = cam.extrins[j * 4 + i];
  {
    double t[3] = {cam.extrins[3], cam.extrins[7], cam.extrins[11]};
    m3_vec(ER, t, Et);
    Et[0] = -Et[0]; Et[1] = -Et[1]; Et[2] = -Et[2];
  }
  const double f = cam.focal_len;
  double pin[3];
  if (cam.coord_frame_type == XR_CAM_ON_DETECTOR) {
    double pz[3] = {0.0, 0.0, f}, tmp[3];
    m3_vec(ER, pz, tmp);
    pin[0] = da(tmp[0], Et[0]); pin[1] = da(tmp[1], Et[1]); pin[2] = da(tmp[2], Et[2]);
  } else {
    pin[0] = Et[0]; pin[1] = Et[1]; pin[2] = Et[2];
  }
  const double dz = (cam.coord_frame_type == XR_CAM_FOCAL_NEG_Z) ? -f : f;
  const double zadj = (cam.coord_frame_type == XR_CAM_ON_DETECTOR) ? -f : 0.0;

  double kc[3] = {dm(Ki[0], dz), dm(Ki[3], dz), dm(Ki[6], dz)};
  double kr[3] = {dm(Ki[1], dz), dm(Ki[4], dz), dm(Ki[7], dz)};
  double k0[3] = {dm(Ki[2], dz), dm(Ki[5], dz), da(dm(Ki[8], dz), zadj)};
  double dcol[3], drow[3], det0[3];
  m3_vec(ER, kc, dcol);
  m3_vec(ER, kr, drow);
  m3_vec(ER, k0, det0);
  det0[0] = da(det0[0], Et[0]); det0[1] = da(det0[1], Et[1]); det0[2] = da(det0[2], Et[2]);
  double e0[3] = {dsb(det0[0], pin[0]), dsb(det0[1], pin[1]), dsb(det0[2], pin[2])};

  double TR[9], Tt[3];
  for (int i = 0; i < 3; ++i) {
    for (int j = 0; j < 3; ++j) TR[i * 3 + j] = pose[i * 4 + j];
    Tt[i] = pose[i * 4 + 3];
  }
  double MR[9], Mt[3];
  m3_mul(vs.Ai, TR, MR);
  m3_vec(vs.Ai, Tt, Mt);
  Mt[0] = da(Mt[0], vs.ti[0]); Mt[1] = da(Mt[1], vs.ti[1]); Mt[2] = da(Mt[2], vs.ti[2]);

  double src[3], d0[3], dc[3], dr[3];
  m3_vec(MR, pin, src);
  src[0] = da(src[0], Mt[0]); src[1] = da(src[1], Mt[1]); src[2] = da(src[2], Mt[2]);
  m3_vec(MR, e0, d0);
  m3_vec(MR, dcol, dc);
  m3_vec(MR, drow, dr);

  ProjGeom g;
  for (int k = 0; k < 3; ++k) {
    g.src[k] = __double2float_rn(src[k]);
    g.d0[k] = __double2float_rn(d0[k]);
    g.dc[k] = __double2float_rn(dc[k]);
    g.dr[k] = __double2float_rn(dr[k]);
    g.e0[k] = __double2float_rn(e0[k]);
    g.ec[k] = __double2float_rn(dcol[k]);
    g.er[k] = __double2float_rn(drow[k]);
    g.pad[k] = 0.0f;
  }
  out[p] = g;
}

// Host twin of m3_inverse for the per-volume inverse (same operation order; the
// host library is compiled with -ffp-contract=off).
void m3_inverse_host(const double* a, double* out) {
  const double c00 = a[4] * a[8] - a[5] * a[7];
  const double c01 = a[5] * a[6] - a[3] * a[8];
  const double c02 = a[3] * a[7] - a[4] * a[6];
  const double det = (a[0] * c00 + a[1] * c01) + a[2] * c02;
  const double id = 1.0 / det;
  out[0] = c00 * id;
  out[1] = (a[2] * a[7] - a[1] * a[8]) * id;
  out[2] = (a[1] * a[5] - a[2] * a[4]) * id;
  out[3] = c01 * id;
  out[4] = (a[0] * a[8] - a[2] * a[6]) * id;
  out[5] = (a[2] * a[3] - a[0] * a[5]) * id;
  out[6] = c02 * id;
  out[7] = (a[1] * a[6] - a[0] * a[7]) * id;
  out[8] = (a[0] * a[4] - a[1] * a[3]) * id;
}

}  // namespace

cudaError_t launch_proj_geom(const xr_volume_desc& vol, const xr_camera_desc* d_cams,
                             const double* d_poses, const int32_t* d_cam_idx, int64_t num_projs,
                             int64_t pose_stride, ProjGeom* d_out, cudaStream_t s) {
  if (num_projs <= 0) return cudaSuccess;
  // The volume's index <-> physical inverse is per volume, evaluated once per
  // launch on the host with the same FP64 operation order as the oracle.
  VolSetup vs;
  double A[9];
  for (int i = 0; i < 3; ++i)
    for (int j = 0; j < 3; ++j) A[i * 3 + j] = vol.direction[i * 3 + j] * vol.spacing[j];
  m3_inverse_host(A, vs.Ai);
  for (int i = 0; i < 3; ++i) {
    const double t = (vs.Ai[i * 3 + 0] * vol.origin[0] + vs.Ai[i * 3 + 1] * vol.origin[1]) +
                     vs.Ai[i * 3 + 2] * vol.origin[2];
    vs.ti[i] = -t;
  }
  const int threads = 128;
  const int blocks = (int)((num_projs + threads - 1) / threads);
  proj_geom_kernel<<<blocks, threads, 0, s>>>(vs, d_cams, d_poses, d_cam_idx, num_projs,
                                              pose_stride > 0 ? pose_stride : num_projs, d_out);
  return cudaGetLastError();
}

}  // namespace xr
