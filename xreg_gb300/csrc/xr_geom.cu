// xr_geom.cu -- per-projection ray set-up on the device, in xReg's float order.
//
// For every projection p this derives what xReg recomputes for each ray of the
// projection and gets the same float result for each (xregRayCastLineIntCPU.cpp:
// 196-212, CameraModel::setup xregPerspectiveXform.cpp:302-334): the camera's
// intrins_inv and extrins_inv, its pinhole, and
//   xform_cam_to_itk_idx = itk_phys_pt_to_itk_idx_xform * xforms_cam_to_itk_phys[p]
// with the pinhole in index coordinates.  The arithmetic is xf:: (xr_xfloat.h):
// float, explicitly rounded, in Eigen's evaluation order, so per-ray step counts
// and sample positions follow the reference's float geometry bit for bit.
#include "xr_cmaes_core.h"
#include "xr_internal.h"

namespace xr {
namespace {

__global__ void proj_geom_kernel(xf::Affine phys_to_idx, const xr_camera_desc* __restrict__ cams,
                                 const double* __restrict__ poses, const int32_t* __restrict__ cam_idx,
                                 int64_t num_projs, int64_t pose_stride, ProjGeom* __restrict__ out) {
  const int64_t p = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= num_projs) return;
  const xr_camera_desc& cd = cams[cam_idx[p]];
  xf::Camera cam;
  for (int k = 0; k < 9; ++k) cam.K[k] = __double2float_rn(cd.intrins[k]);
  for (int k = 0; k < 16; ++k) cam.E[k] = __double2float_rn(cd.extrins[k]);
  cam.focal_len = __double2float_rn(cd.focal_len);
  cam.frame = cd.coord_frame_type;
  // poses are indexed modulo pose_stride: projection p uses pose (p % pose_stride),
  // which implements distribute_xforms_among_cam_models without a host copy.
  // A pose is xReg's FrameTransform: float.
  const double* pd = poses + 16 * (p % pose_stride);
  xf::Affine pose;
  for (int i = 0; i < 3; ++i) {
    for (int j = 0; j < 3; ++j) pose.L[i * 3 + j] = __double2float_rn(pd[i * 4 + j]);
    pose.t[i] = __double2float_rn(pd[i * 4 + 3]);
  }
  ProjGeom g;
  xf::ray_frame(cam, phys_to_idx, pose, g);
  out[p] = g;
}

// Candidate k of a device CMA-ES job (cmaes_SamplePopulation, then
// cmaes_ReSampleSingle while outside the bounds, xregIntensity2D3DRegiCMAES.cpp:154-191)
// and its pose.  Every view's projection of candidate k draws the same bits;
// the first view's (owner) stores the candidate, its draw count and its pose.
__device__ __noinline__ void sample_candidate(const GeomJob& J, int64_t k, bool owner, double* pose_out) {
  const cma::View s = cma::view(J.cma);
  const int n = s.h->n;
  double z[kCmaDeviceMaxDim], x[kCmaDeviceMaxDim];
  int attempt = 0;
  for (;; ++attempt) {
    cma::draw(s, (int)k, attempt, z, x);
    if (cma::inside(x, J.bounds, n)) break;
    if (attempt > kCmaMaxRedraws) {
      if (owner) J.report->sample_error = 1;
      break;
    }
  }
  pose::map(J.C, J.B, x, pose_out);
  if (owner) {
    for (int i = 0; i < n; ++i) {
      s.z[k * n + i] = z[i];
      s.pop[k * n + i] = x[i];
    }
    s.att[k] = attempt;
    for (int i = 0; i < 16; ++i) J.poses[16 * k + i] = pose_out[i];
    if (k == 0) s.h->sampled = 1;
  }
}

// One thread per projection of every job (jobs in order of `first`).
__global__ void proj_geom_jobs_kernel(const GeomJob* __restrict__ jobs, int njobs, int64_t total) {
  const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= total) return;
  int j = 0;
  while (j + 1 < njobs && jobs[j + 1].first <= t) ++j;
  const GeomJob& J = jobs[j];
  const int64_t p = t - J.first;
  const xr_camera_desc& cd = J.cams[J.cam_idx[p]];
  xf::Camera cam;
  for (int k = 0; k < 9; ++k) cam.K[k] = __double2float_rn(cd.intrins[k]);
  for (int k = 0; k < 16; ++k) cam.E[k] = __double2float_rn(cd.extrins[k]);
  cam.focal_len = __double2float_rn(cd.focal_len);
  cam.frame = cd.coord_frame_type;
  const int64_t k = p % J.pose_stride;
  double drawn[16];
  const double* pd = J.poses + 16 * k;
  if (J.cma) {
    sample_candidate(J, k, p < J.pose_stride, drawn);
    pd = drawn;
  }
  xf::Affine pose;
  for (int i = 0; i < 3; ++i) {
    for (int jj = 0; jj < 3; ++jj) pose.L[i * 3 + jj] = __double2float_rn(pd[i * 4 + jj]);
    pose.t[i] = __double2float_rn(pd[i * 4 + 3]);
  }
  ProjGeom g;
  xf::ray_frame(cam, J.p2i, pose, g);
  J.out[p] = g;
}

}  // namespace

cudaError_t launch_proj_geom_jobs(const GeomJob* d_jobs, int njobs, int64_t total, cudaStream_t s) {
  if (total <= 0) return cudaSuccess;
  const int threads = 128;
  proj_geom_jobs_kernel<<<(unsigned)((total + threads - 1) / threads), threads, 0, s>>>(d_jobs, njobs, total);
  return cudaGetLastError();
}

xf::Affine phys_to_idx_xform(const xr_volume_desc& vol) {
  // ITKImagePhysicalPointTransformsAsEigen (xregITKBasicImageUtils.h:133-165):
  // float(direction(r, c) * spacing(c)) and float(origin), then
  // FrameTransform::inverse (xregRayCastLineIntCPU.cpp:307-309)
  xf::Affine i2p;
  for (int r = 0; r < 3; ++r) {
    for (int c = 0; c < 3; ++c) i2p.L[r * 3 + c] = (float)(vol.direction[r * 3 + c] * vol.spacing[c]);
    i2p.t[r] = (float)vol.origin[r];
  }
  xf::Affine p2i;
  xf::inverse(i2p, p2i);
  return p2i;
}

cudaError_t launch_proj_geom(const xr_volume_desc& vol, const xr_camera_desc* d_cams,
                             const double* d_poses, const int32_t* d_cam_idx, int64_t num_projs,
                             int64_t pose_stride, ProjGeom* d_out, cudaStream_t s) {
  if (num_projs <= 0) return cudaSuccess;
  const xf::Affine p2i = phys_to_idx_xform(vol);
  const int threads = 128;
  const int blocks = (int)((num_projs + threads - 1) / threads);
  proj_geom_kernel<<<blocks, threads, 0, s>>>(p2i, d_cams, d_poses, d_cam_idx, num_projs,
                                              pose_stride > 0 ? pose_stride : num_projs, d_out);
  return cudaGetLastError();
}

}  // namespace xr
