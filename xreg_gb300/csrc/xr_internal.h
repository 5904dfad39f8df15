// xr_internal.h -- device data layouts and launcher declarations shared by the
// translation units of libxreg_gb300.  Not part of the public ABI.
#pragma once

#include <cuda_runtime.h>
#include <cuda_fp16.h>
#include <cuda_bf16.h>
#include <cstdint>
#include <string>

#include "xreg_gb300.h"
#include "xr_step.h"
#include "xr_xfloat.h"

namespace xr {

// Per-projection ray set-up (176 bytes): the camera's inverses and pinhole and
// the camera -> index transform, all in float as xReg holds them; every
// ray-marching kernel finishes the set-up per ray with xf::ray_setup.
using ProjGeom = xf::RayFrame;
static_assert(sizeof(ProjGeom) == 176, "ProjGeom layout");

// Volume as the kernels see it.
struct VolView {
  const void* voxels;  // F32 / F16 / BF16, x fastest
  const void* cells;   // CELL8 layout: 8 corners per trilinear cell (or nullptr)
  int32_t nx, ny, nz;
  int32_t voxel_type;
  int32_t layout;      // XR_LAYOUT_LINEAR / XR_LAYOUT_CELL8
  float inv_scale;     // multiplies the ray sum (1 for F32)
  // CELL8 cell order, z fastest: cell (ix, iy, iz) is number ix cs[0] + iy cs[1] + iz
  int32_t cs[2];
  // Support box: every sample whose continuous index lies outside
  // (sup_lo, sup_hi) on some axis interpolates only zero voxels.  has_support 0
  // disables sample skipping; an all-zero volume has an empty box (lo > hi).
  int32_t has_support;
  float sup_lo[3], sup_hi[3];
  // Dilated macro-cell occupancy: bit m of occ is 0 when every trilinear cell
  // with base index in [8m - 1, 8m + 8] on each axis has only zero corners
  // (macro cell m spans cells [8m, 8m + 7]).  occ may be nullptr.
  const uint32_t* occ;
  int32_t nmx, nmy, nmz;
};
constexpr int kMacroShift = 3;  // macro cells of 8 x 8 x 8 trilinear cells

// Launch parameters of a DRR kernel.
struct DrrParams {
  VolView vol;
  const ProjGeom* geo;    // [num_projs]
  const int32_t* cam_idx; // [num_projs]
  const float* bg_projs;  // [num_cams][rows*cols] or nullptr
  float* out;             // [num_projs][rows][cols]
  unsigned long long* sample_counter;  // nullptr = no counting
  unsigned long long* loaded_counter;  // samples loaded (not skipped as provably zero); with sample_counter
  unsigned int* err_counter;          // rays whose step count exceeded max_steps
  unsigned long long max_steps;       // guard against non-finite / absurd poses
  int64_t num_projs;
  int32_t rows, cols;
  float step;
  float default_bg;
  int32_t kernel_id;      // XR_LINE_INT_SUM / MAX
  int32_t store;          // XR_PROJ_STORE_REPLACE / ACCUM
  int32_t block_warps_x;  // warps across a block (1, 2, 4, 8)
  int32_t warp_tall;      // 0: each warp covers 8x4 pixels (cols x rows); 1: 4x8
  int32_t unroll;         // sample loop 1..5 (xr_rc_set_launch_config)
};

// ---- launchers (xr_geom.cu) ----
// ITK physical -> index transform of a volume in xReg's float arithmetic.
xf::Affine phys_to_idx_xform(const xr_volume_desc& vol);
// One thread per projection: camera inverses and the camera -> index transform
// phys_to_idx * pose in xReg's float order (xf::ray_frame).
cudaError_t launch_proj_geom(const xr_volume_desc& vol, const xr_camera_desc* d_cams,
                             const double* d_poses, const int32_t* d_cam_idx, int64_t num_projs,
                             int64_t pose_stride_projs, ProjGeom* d_out, cudaStream_t s);

// ---- launchers (xr_raycast.cu) ----
cudaError_t launch_drr(const DrrParams& p, cudaStream_t s);

// One job of a multi-job DRR launch: its parameters (sum kernel; any store
// rule; p.block_warps_x and p.warp_tall give its tile shape as for
// drr_kernel), where its work items start, and its tile grid.
struct MultiJobDrr {
  DrrParams p;
  long long item_begin;  // items of this job: [item_begin, item_begin + items())
  int32_t tiles_x, tiles_y;
  // 0: one item per (tile, projection) in the job's block shape; 4: one item per
  // (8x8-pixel tile, group of 4 consecutive projections), mapped to threads by
  // how close the group's rays are (drr_jobs_kernel)
  int32_t pose_group;
  __host__ __device__ long long items() const {
    const long long units = pose_group ? (p.num_projs + pose_group - 1) / pose_group : p.num_projs;
    return units * tiles_x * tiles_y;
  }
};
// One launch whose grid covers the (tile, projection) items of jobs sharing a
// voxel type and layout (no work counter: one block per item); each job runs
// its own sample loop, p.unroll 3, 4 or 6 (6 with the cell layouts only).
// grouped: every job's pose_group is 4 (otherwise every job's is 0).
cudaError_t launch_drr_jobs(const MultiJobDrr* d_jobs, int njobs, long long total_items, int32_t voxel_type,
                            int32_t layout, bool grouped, cudaStream_t s);
// Macro-cell occupancy bitmask of a volume (see VolView::occ); d_occ holds
// ceil(nmx * nmy * nmz / 32) words and is cleared here.
cudaError_t launch_build_occupancy(const float* vox_f32, int nx, int ny, int nz, uint32_t* d_occ, int nmx, int nmy,
                                   int nmz, cudaStream_t s);
// Index bounds of the non-zero voxels into d_box[6] (min xyz, max xyz; max < min if none).
cudaError_t launch_support_box(const float* vox_f32, int nx, int ny, int nz, int* d_box, cudaStream_t s);
// Bytes of the CELL8 copy of a volume, and the kernel that builds it from
// float32 voxels (cells numbered z fastest, then x, then y: VolView::cs).
size_t cell_layout_bytes(int64_t nx, int64_t ny, int64_t nz, int32_t voxel_type);
cudaError_t launch_build_cells(const float* vox_f32, int nx, int ny, int nz, int32_t voxel_type, float scale,
                               void* out, cudaStream_t s);
// The x and y cell strides of that order (VolView::cs).
void cell_strides(int64_t nx, int64_t ny, int64_t nz, int32_t cs[2]);

// ---- launchers (xr_metrics.cu) ----
struct FixedNCC {           // per direction (one for NCC, x and y for grad-NCC)
  const float* fhat;        // zero-mean fixed image (float)
  double sd;                // sample std dev, clamped at 1e-6
  double sum_fhat;          // sum of fhat over used pixels (exact decomposition)
};

// ---- fused evaluation (xr_raycast.cu) ----
// One view of a job whose grad-NCC (5x5 smoothing) runs inside the evaluation
// kernel: the fixed side, the per-tile partials and the view's values.
struct FusedView {
  const float* fhx;       // zero-mean fixed gradients
  const float* fhy;
  const uint8_t* mask;    // or nullptr
  FixedNCC fx, fy;
  double n_used;
  double* partials;       // [pop][metric tiles][6]
  float* sims;            // [pop]
};
// A job of a fused evaluation launch: its DRR work items (16x16-pixel tiles,
// projection fastest), and when `metric` is 1 the grad-NCC of every image
// computed tile by tile as soon as the DRR pixels a 32x64 metric tile reads are
// written, then each image's value, then each pose's mean over views.
// Counters live in `cnt` (zero between launches; the block that completes a
// counter resets it): [nviews * pop * mt] DRR tiles done per metric tile, then
// [nviews * pop] metric tiles done per image, then [pop] views done per pose.
constexpr int kMaxFusedViews = 16;
struct FusedJob {
  MultiJobDrr d;
  int32_t metric;         // 1: grad-NCC fused behind the DRR; 0: DRR only
  int32_t nviews;
  int64_t pop;
  int32_t mt_x, mt_y;     // metric tiles across / down
  const FusedView* views; // [nviews]
  float* out;             // [pop] mean over views
  unsigned int* cnt;
  long long tile_begin;   // first metric tile of this job in a batched metric launch
  void* cma;              // CMA-ES state updated by the batched grad-NCC launch once every pose has its value
  CmaReport* report;      // where that update reports its termination code
};
// One persistent launch over the jobs of one (voxel type, layout) group.
cudaError_t launch_eval_fused(const FusedJob* d_jobs, int njobs, long long total_items, int32_t voxel_type,
                              int32_t layout, int32_t unroll, unsigned long long* d_counter, int* blocks_out,
                              cudaStream_t s);
// Grad-NCC (5x5 smoothing) of every image of the jobs with `metric` set, their
// DRRs already written: one launch over all their 32x64 tiles (the split
// path's tile code), each image's FP64 combine by the block that completes its
// tiles, each pose's mean over views by the block that completes its views,
// and (jobs with `cma`) the CMA-ES update by the block that completes the
// job's last pose.
cudaError_t launch_grad_multi(const FusedJob* d_jobs, int njobs, long long total_tiles, cudaStream_t s);
// Geometry of many ray casters' projections in one launch.
struct GeomJob {
  xf::Affine p2i;
  const xr_camera_desc* cams;
  double* poses;          // [pose_stride] read, or written when cma is set
  const int32_t* cam_idx;
  int64_t num_projs, pose_stride, first;  // first: index of this job's first projection over all jobs
  ProjGeom* out;
  // set: candidate (p % pose_stride) of the CMA-ES state `cma` is drawn here
  // (redrawn until inside `bounds`) and its pose C Exp(x) B written to poses
  void* cma;
  CmaReport* report;
  double C[16], B[16], bounds[kCmaDeviceMaxDim];
};
// CMA-ES updates of device-optimizer jobs whose values come from other
// launches (one block per job).
struct CmaUpdateJob {
  void* cma;
  const float* vals;  // [lambda]
  CmaReport* report;
};
cudaError_t launch_cma_updates(const CmaUpdateJob* d_jobs, int njobs, cudaStream_t s);
cudaError_t launch_proj_geom_jobs(const GeomJob* d_jobs, int njobs, int64_t total_projs, cudaStream_t s);

struct PatchFixed {         // per direction
  const float* img;         // fixed image (or its gradient), rows*cols
  const float* mean;        // per patch mean
  const float* scale;       // per patch 1 / (sd * n used for the statistics)
  const float* w;           // per patch weight, nullptr = 1
};

struct PatchRun {           // per compute
  const uint8_t* mask;      // image mask or nullptr
  const int32_t* cnt;       // times each patch is used, nullptr = once
  int use_mask_stats;       // statistics over masked-in pixels only
  int mask_in_sums;         // correlation sums over masked-in pixels only
  int weighted;             // weight_patch_sims_in_combine
  int mvar;                 // moving-variance weights: 0 none, 1 of the image, 2 of each gradient image
  int normalize;            // normalise moving variances by their sum
  const double* mvar_sum;   // [image][direction] sums of count x variance (pass 0), for pass 1
  float* scores;            // [image][patch] each patch's score (pass 1), nullptr = not kept
};

// Moments of moving images for (grad-)NCC: partials[img][block][k] in double.
cudaError_t launch_ncc_moments(const float* mov, int64_t npix, int64_t nimgs, const float* fhat,
                               const uint8_t* mask, double* partials, int nblk, cudaStream_t s);
cudaError_t launch_ncc_finalize(const double* partials, int nblk, int64_t nimgs, int64_t n_used,
                                FixedNCC fx, float* sims, cudaStream_t s);
cudaError_t launch_grad_moments(const float* mov, int rows, int cols, int64_t nimgs, int smooth_ksize,
                                const float* fhat_x, const float* fhat_y, const uint8_t* mask,
                                double* partials, cudaStream_t s, int* nblk_out);
cudaError_t launch_grad_finalize(const double* partials, int nblk, int64_t nimgs, int64_t n_used,
                                 FixedNCC fx, FixedNCC fy, float* sims, cudaStream_t s);
// Gradient images (blur + Sobel) of nimgs images; used for the fixed image.
cudaError_t launch_grad_images(const float* img, int rows, int cols, int64_t nimgs, int smooth_ksize,
                               float* gx, float* gy, cudaStream_t s);
// Mean / sum-of-squares of an image in double (setup); out[0]=sum, out[1]=sum of (x-mean)^2 computed
// in a second pass, out[2]=count.
cudaError_t launch_image_stats(const float* img, int64_t npix, const uint8_t* mask, double* d_out,
                               cudaStream_t s);
cudaError_t launch_sub_scalar(const float* in, int64_t n, double value, float* out, cudaStream_t s);
cudaError_t launch_sum_f(const float* in, int64_t n, const uint8_t* mask, double* d_out, cudaStream_t s);
// Per-patch statistics of a fixed image for patch NCC (mean / scale may be
// nullptr; wvar: variance weight; ucount: masked-in pixel count; both optional).
cudaError_t launch_patch_fixed_stats(const float* img, int rows, int cols, int radius, int stride, int ncr, int ncc,
                                     const uint8_t* mask, int use_mask_stats, float* mean, float* scale, float* wvar,
                                     int* ucount, cudaStream_t s);
// pass 0: moving-variance sums; pass 1: weighted score sums.  partials
// [image][block][2]; *nblk_out = the blocks per image of this launch (its tile
// shape depends on the mask and weight options), at most
// patch_ncc_max_blocks(ncr, ncc).
int patch_ncc_max_blocks(int ncr, int ncc);
cudaError_t launch_patch_ncc(const float* mov, int rows, int cols, int64_t nimgs, int grad, int smooth_ksize,
                             int radius, int stride, int ncr, int ncc, PatchFixed px, PatchFixed py, PatchRun run,
                             int pass, double* partials, cudaStream_t s, int* nblk_out);
cudaError_t launch_patch_sum_partials(const double* partials, int nblk, int64_t nimgs, double* out, cudaStream_t s);
cudaError_t launch_patch_finalize(const double* partials, int nblk, int64_t nimgs, double den_x, double den_y,
                                  int grad, int mvar, int normalize, const double* mvar_sum, float* sims,
                                  cudaStream_t s);
cudaError_t launch_patch_scatter_counts(const int32_t* idx, int64_t n, int32_t* cnt, cudaStream_t s);
// Mean over views of per-view similarity values: sims[v][pop] -> out[pop].
cudaError_t launch_combine_mean(const float* const* view_sims, int nviews, int64_t pop, float* out,
                                cudaStream_t s);

// ---- error plumbing (xr_capi.cu) ----
void set_error(const std::string& msg);
xr_status fail(xr_status code, const std::string& msg);
xr_status cuda_fail(cudaError_t e, const char* what);

}  // namespace xr

#define XR_CUDA_TRY(expr)                                                        \
  do {                                                                           \
    cudaError_t xr_e_ = (expr);                                                  \
    if (xr_e_ != cudaSuccess) return ::xr::cuda_fail(xr_e_, #expr);              \
  } while (0)
