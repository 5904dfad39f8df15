/*
 * xreg_gb300.h -- C ABI of the GB300-native line-integral DRR ray caster and 2D
 * similarity metrics.  Plain C types only (no CUDA, torch or C++ types in the
 * signatures); every entry point returns an xr_status (0 = success) and never
 * throws.  The message of the last failure on the calling thread is available
 * from xr_last_error().
 *
 * The entry points mirror xReg's operator surface so a thin C++ class (see
 * include/xreg_gb300/xreg_gb300.hpp) can stand in for xReg's RayCaster and
 * ImgSimMetric2D objects inside its registration pipeline.  Citations below are
 * paths inside the xReg project.
 *
 * Threading and ordering: each handle owns one CUDA stream (or uses the stream
 * given with xr_*_set_stream).  compute calls are asynchronous on that stream;
 * calls that return host data (xr_rc_proj, xr_rc_copy_projs_to_host,
 * xr_sm_sim_vals) synchronise the stream first.  A handle must not be used from
 * two threads at once (same rule as xReg's objects).
 */
#ifndef XREG_GB300_H_
#define XREG_GB300_H_

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#if defined(_WIN32)
#define XR_API __declspec(dllexport)
#else
#define XR_API __attribute__((visibility("default")))
#endif

/* ---------------------------------------------------------------- status -- */
typedef int32_t xr_status;
enum {
  XR_OK = 0,
  XR_ERR_INVALID_ARG = -1,    /* bad pointer, size, index or order of calls    */
  XR_ERR_CUDA = -2,           /* a CUDA runtime call failed                    */
  XR_ERR_OUT_OF_MEMORY = -3,  /* device allocation refused                     */
  XR_ERR_UNSUPPORTED = -4,    /* UnsupportedOperationException in xReg         */
  XR_ERR_NOT_ALLOCATED = -5,  /* compute before allocate_resources             */
  XR_ERR_DEVICE_CHECK = -6    /* a kernel's own bounds/timeout check tripped   */
};

/* Message of the last failing call on this thread ("" if none). */
XR_API const char* xr_last_error(void);
/* Library version string. */
XR_API const char* xr_version(void);

/* ----------------------------------------------------------- plain types -- */
/* Volume geometry in ITK conventions: n = size along index x, y, z (x fastest
 * in the voxel buffer); physical point = origin + direction * diag(spacing) * idx
 * (xregITKBasicImageUtils.h:133-165). */
typedef struct {
  int64_t n[3];
  double spacing[3];
  double origin[3];
  double direction[9]; /* row-major */
} xr_volume_desc;

/* Camera model (xregPerspectiveXform.h:108-273).  intrins is K (row-major 3x3),
 * extrins maps "world" to camera (row-major 4x4).  coord_frame_type:
 * 0 = origin at focal point, +z to detector; 1 = origin at focal point, -z to
 * detector (xReg's default); 2 = origin on detector. */
typedef struct {
  double intrins[9];
  double extrins[16];
  int64_t num_det_rows;
  int64_t num_det_cols;
  double det_row_spacing;
  double det_col_spacing;
  double focal_len;
  int32_t coord_frame_type;
  int32_t reserved;
} xr_camera_desc;

enum { XR_VOXEL_F32 = 0, XR_VOXEL_F16 = 1, XR_VOXEL_BF16 = 2 };
enum { XR_LINE_INT_SUM = 0, XR_LINE_INT_MAX = 1 };          /* RayCastLineIntKernel */
enum { XR_PROJ_STORE_REPLACE = 0, XR_PROJ_STORE_ACCUM = 1 }; /* ProjPixelStoreMethod */
enum { XR_INTERP_LINEAR = 0, XR_INTERP_NN = 1, XR_INTERP_SINC = 2, XR_INTERP_BSPLINE = 3 };
enum { XR_CAM_FOCAL_POS_Z = 0, XR_CAM_FOCAL_NEG_Z = 1, XR_CAM_ON_DETECTOR = 2 };
/* Device layouts of a volume (results are identical; speed differs):
 * LINEAR = voxels x-fastest; CELL8 = the 8 corners of every trilinear cell stored
 * together (8x the voxel bytes, one or two vector loads per sample). */
enum { XR_LAYOUT_AUTO = -1, XR_LAYOUT_LINEAR = 0, XR_LAYOUT_CELL8 = 1 };

/* ------------------------------------------------------- camera helpers -- */
/* CameraModel::setup(focal_len, nr, nc, rs, cs) with MakeNaiveIntrins
 * (xregPerspectiveXform.cpp:200-254). */
XR_API xr_status xr_camera_setup_naive(double focal_len, int64_t num_rows, int64_t num_cols,
                                       double row_spacing, double col_spacing,
                                       int32_t coord_frame_type, xr_camera_desc* out);
/* DownsampleCameraModel (xregPerspectiveXform.cpp:654-689). */
XR_API xr_status xr_camera_downsample(const xr_camera_desc* src, double ds_factor,
                                      int32_t force_even_dims, xr_camera_desc* out);

/* ------------------------------------------------------------ ray caster -- */
/* Replaces RayCasterLineIntCPU / RayCasterLineIntOCL
 * (xregRayCastLineIntCPU.h:33, xregRayCastLineIntOCL.h:36) behind the RayCaster
 * interface (xregRayCastInterface.h:43-434). */
typedef struct xr_raycaster_s* xr_raycaster;

/* device < 0 selects the current device. */
XR_API xr_status xr_rc_create(int32_t device, xr_raycaster* out);
XR_API xr_status xr_rc_destroy(xr_raycaster rc);
/* Use a caller-owned cudaStream_t (passed as void*); NULL restores the handle's own stream. */
XR_API xr_status xr_rc_set_stream(xr_raycaster rc, void* cuda_stream);
XR_API xr_status xr_rc_synchronize(xr_raycaster rc);

/* RayCaster::set_volumes (xregRayCastInterface.cpp:38-43).  Voxels are float32 on
 * the host; they are copied to the device now and stored as voxel_type
 * (XR_VOXEL_F16 / BF16 store scale * mu and undo the scale after the ray sum;
 * scale <= 0 picks a power of two automatically (BF16: 1).  FP16 always
 * stores max|mu| scaled into [0.5, 1) by a power of two, which its blend's
 * scaled weights need, and does not use scale; it refuses non-finite voxels
 * and a nonzero maximum below 2^-90 with XR_ERR_INVALID_ARG). */
XR_API xr_status xr_rc_set_volumes(xr_raycaster rc, int32_t num_vols, const xr_volume_desc* descs,
                                   const float* const* host_voxels, int32_t voxel_type, float scale);
/* Same, with float32 voxels already in device memory (copied, not borrowed). */
XR_API xr_status xr_rc_set_volumes_device(xr_raycaster rc, int32_t num_vols, const xr_volume_desc* descs,
                                          const float* const* device_voxels, int32_t voxel_type, float scale);
/* RayCaster::set_camera_models (xregRayCastInterface.cpp:55-59). */
XR_API xr_status xr_rc_set_camera_models(xr_raycaster rc, int32_t num_cams, const xr_camera_desc* cams);
/* RayCaster::set_num_projs (xregRayCastInterface.cpp:124-132). */
XR_API xr_status xr_rc_set_num_projs(xr_raycaster rc, int64_t num_projs);
XR_API xr_status xr_rc_num_projs(xr_raycaster rc, int64_t* out);
/* RayCaster::set_ray_step_size (default 1, xregRayCastInterface.h:390). */
XR_API xr_status xr_rc_set_ray_step_size(xr_raycaster rc, float step_mm);
/* RayCaster::set_interp_method; only XR_INTERP_LINEAR is implemented (as in
 * RayCasterOCL, xregRayCastBaseOCL.cpp:338-341); others give XR_ERR_UNSUPPORTED at compute. */
XR_API xr_status xr_rc_set_interp_method(xr_raycaster rc, int32_t method);
/* use_proj_store_replace_method / use_proj_store_accum_method (xregRayCastInterface.cpp:262-280). */
XR_API xr_status xr_rc_set_proj_store_method(xr_raycaster rc, int32_t method);
/* set_default_bg_pixel_val (xregRayCastInterface.cpp:343-346). */
XR_API xr_status xr_rc_set_default_bg_pixel_val(xr_raycaster rc, float bg);
/* RayCastLineIntParamInterface::set_kernel_id (xregRayCastInterface.h:575-591). */
XR_API xr_status xr_rc_set_kernel_id(xr_raycaster rc, int32_t kernel_id);
/* set_bg_projs: one host image per camera model (rows*cols floats each), copied;
 * use_bg_projs toggles their use (xregRayCastInterface.cpp:303-333). */
XR_API xr_status xr_rc_set_bg_projs(xr_raycaster rc, const float* const* host_imgs, int32_t use_bg_projs);
XR_API xr_status xr_rc_set_use_bg_projs(xr_raycaster rc, int32_t use_bg_projs);
/* set_xforms_cam_to_itk_phys: also sets num_projs (xregRayCastInterface.cpp:168-172).
 * xforms: row-major 4x4 doubles, camera -> ITK physical. */
XR_API xr_status xr_rc_set_xforms_cam_to_itk_phys(xr_raycaster rc, int64_t num_xforms, const double* xforms);
/* distribute_xforms_among_cam_models (xregRayCastInterface.cpp:97-114): projection
 * (cam * num_xforms + i) gets xform i and camera cam; requires
 * num_xforms * num_cams == num_projs. */
XR_API xr_status xr_rc_distribute_xforms_among_cam_models(xr_raycaster rc, int64_t num_xforms,
                                                          const double* xforms);
/* Same, with the xforms already in device memory (num_xforms * 16 doubles). */
XR_API xr_status xr_rc_distribute_xforms_device(xr_raycaster rc, int64_t num_xforms, const double* d_xforms);
/* set_camera_model_proj_associations (xregRayCastInterface.cpp:73-80). */
XR_API xr_status xr_rc_set_camera_model_proj_associations(xr_raycaster rc, int64_t n, const int32_t* cam_idx);
/* camera_model_proj_associations / set_proj_cam_model (xregRayCastInterface.cpp:78-87):
 * the camera of every projection (*count = num_projs), and one projection's camera. */
XR_API xr_status xr_rc_camera_model_proj_associations(xr_raycaster rc, int64_t cap, int32_t* cam_idx, int64_t* count);
XR_API xr_status xr_rc_set_proj_cam_model(xr_raycaster rc, int64_t proj_idx, int32_t cam_idx);
/* xforms_cam_to_itk_phys (xregRayCastInterface.cpp:182-198): every projection's
 * pose (row-major 4x4 each; *count = num_projs, 0 before any pose is set);
 * poses given on the device are copied back first. */
XR_API xr_status xr_rc_xforms_cam_to_itk_phys(xr_raycaster rc, int64_t cap, double* xforms, int64_t* count);
/* pre_multiply_all_xforms / post_multiply_all_xforms
 * (xregRayCastInterface.cpp:235-261): every pose becomes pre * pose, or
 * pose * post (in double; xReg's FrameTransform is float). */
XR_API xr_status xr_rc_pre_multiply_all_xforms(xr_raycaster rc, const double* pre_xform);
XR_API xr_status xr_rc_post_multiply_all_xforms(xr_raycaster rc, const double* post_xform);
/* num_vols, num_camera_models (xregRayCastInterface.h:93-98). */
XR_API xr_status xr_rc_num_vols(xr_raycaster rc, int32_t* out);
XR_API xr_status xr_rc_num_camera_models(xr_raycaster rc, int32_t* out);
/* xform_img_center_to_itk_phys (xregRayCastInterface.cpp:200-224): translation
 * by the ITK physical point of the volume's continuous index size / 2.
 * xform_cam_wrt_carm_center_of_rot (:226-233): translation by -focal_len / 2
 * along z.  Row-major 4x4 outputs. */
XR_API xr_status xr_rc_xform_img_center_to_itk_phys(xr_raycaster rc, int32_t vol_idx, double* out);
XR_API xr_status xr_rc_xform_cam_wrt_carm_center_of_rot(xr_raycaster rc, int32_t cam_idx, double* out);
/* RayCaster::allocate_resources + RayCasterCPU::allocate_resources
 * (xregRayCastInterface.cpp:248-260, xregRayCastBaseCPU.cpp:50-88). */
XR_API xr_status xr_rc_allocate_resources(xr_raycaster rc);
/* max_num_projs_possible (xregRayCastInterface.h:296): from free device memory. */
XR_API xr_status xr_rc_max_num_projs_possible(xr_raycaster rc, int64_t* out);
/* RayCasterLineIntCPU::compute (xregRayCastLineIntCPU.cpp:294-349); asynchronous. */
XR_API xr_status xr_rc_compute(xr_raycaster rc, int32_t vol_idx);
/* proj(idx) as a host copy (xregRayCastBaseCPU.cpp:90-117); synchronises. */
XR_API xr_status xr_rc_proj(xr_raycaster rc, int64_t proj_idx, float* host_dst);
/* raw_host_pixel_buf analogue: copies all num_projs images; synchronises. */
XR_API xr_status xr_rc_copy_projs_to_host(xr_raycaster rc, float* host_dst);
/* to_cuda_buf(): device address of the projection buffer (view-major, row-major
 * images, num_projs * rows * cols floats), valid until the next allocate_resources. */
XR_API xr_status xr_rc_device_pixel_buf(xr_raycaster rc, float** out);
/* use_other_proj_buf (xregRayCastInterface.h:320): this caster writes its images
 * into the device buffer of `other` (same detector size, enough allocated
 * projections), e.g. several objects accumulated into one DRR with the
 * accumulate store method; NULL restores its own buffer.  A destroyed `other`
 * is detected at the next compute. */
XR_API xr_status xr_rc_use_other_proj_buf(xr_raycaster rc, xr_raycaster other);
/* use_external_host_pixel_buf (xregRayCastInterface.h:287): after every compute
 * the images are copied into host_buf (num_projs images, row-major), on the
 * caster's stream; read it after xr_rc_synchronize.  NULL stops the copies. */
XR_API xr_status xr_rc_use_external_host_pixel_buf(xr_raycaster rc, float* host_buf);
/* Exact number of trilinear samples the last compute took (algorithmic-bytes
 * accounting); synchronises. */
XR_API xr_status xr_rc_last_num_samples(xr_raycaster rc, uint64_t* out);
/* How many of those samples the kernel loaded: the rest lie in cells whose
 * eight corners are zero and were skipped (they add exactly +0); synchronises.
 * No counterpart in xReg (it loads every sample). */
XR_API xr_status xr_rc_last_num_loaded_samples(xr_raycaster rc, uint64_t* out);
/* Enables (1) or disables (0) per-compute sample counting (default off). */
XR_API xr_status xr_rc_set_count_samples(xr_raycaster rc, int32_t enable);
/* Launch configuration of the DRR kernel: volume layout (XR_LAYOUT_LINEAR,
 * XR_LAYOUT_CELL8, 2 = the float32 CELL8 copy read with one 256-bit load, or
 * 3 = brick-staged: 16x16 rays per block, each slab of cells along the rays'
 * axis copied to shared memory and sampled from there; float32 volumes and the
 * sum kernel; identical values, measured 3-4x slower than the gather, never
 * autotuned; block shape and loop are ignored), warps
 * across a 256-thread block (1, 2, 4 or 8; each warp covers 8x4 pixels) and
 * the sample loop: 1 or 2 samples per iteration, or 3 / 4 = 2 / 4 per iteration
 * after each ray is trimmed to its first and last occupied macro cell (sum
 * kernel with empty-space skipping on; otherwise 3 and 4 run as 2), or 5 = 3
 * with the second sample of a pair reusing the first's corners when both lie in
 * one cell (256-bit float32 CELL8 read; elsewhere 5 runs as 3), or 6 = 4 on
 * packed FP32 pairs (float32 256-bit or FP16 / BF16 CELL8 reads; elsewhere 6
 * runs as 4).  layout
 * XR_LAYOUT_AUTO (the default) lets
 * the autotuner time the candidates on the first compute of each shape (volume
 * size, voxel type, detector, projection count) and cache the fastest for the
 * process.  No xReg counterpart (xReg's OpenCL caster has a fixed NDRange). */
XR_API xr_status xr_rc_set_launch_config(xr_raycaster rc, int32_t layout, int32_t block_warps_x, int32_t unroll);
/* The configuration the last compute used. */
XR_API xr_status xr_rc_get_launch_config(xr_raycaster rc, int32_t* layout, int32_t* block_warps_x, int32_t* unroll);
/* As xr_rc_set_launch_config with the warp shape too: warp_rows 4 = each warp
 * covers 8x4 pixels (what xr_rc_set_launch_config sets), 8 = 4x8.  The
 * autotuner also times 4x8 warps for its fastest layout and loop. */
XR_API xr_status xr_rc_set_launch_config_ex(xr_raycaster rc, int32_t layout, int32_t block_warps_x, int32_t unroll,
                                            int32_t warp_rows);
XR_API xr_status xr_rc_get_launch_config_ex(xr_raycaster rc, int32_t* layout, int32_t* block_warps_x,
                                            int32_t* unroll, int32_t* warp_rows);
/* Whether set_volumes also builds the CELL8 copy (default 1).  Set before set_volumes. */
XR_API xr_status xr_rc_set_build_cell_layout(xr_raycaster rc, int32_t enable);
/* Empty-space skipping for the line-integral sum (default 1): samples whose
 * trilinear cell lies outside the bounding box of the volume's non-zero voxels
 * add exactly zero, so they are not loaded; positions still advance by the same
 * float additions, so the DRR is bit-identical with skipping on or off and equal
 * to xReg's sample-by-sample sum.  Loop variant 3 also trims each ray's leading
 * and trailing samples that lie in empty macro cells (8x8x8 trilinear cells with
 * no non-zero corner within one cell), with the same guarantee.  The max kernel
 * never skips. */
XR_API xr_status xr_rc_set_empty_space_skipping(xr_raycaster rc, int32_t enable);

/* ------------------------------------------------------ similarity metric -- */
/* Replaces ImgSimMetric2D{NCC,GradNCC,PatchNCC,PatchGradNCC}{CPU,OCL}
 * (xregImgSimMetric2D.h:42-159). */
typedef struct xr_simmetric_s* xr_simmetric;
enum { XR_SIM_NCC = 0, XR_SIM_GRAD_NCC = 1, XR_SIM_PATCH_NCC = 2, XR_SIM_PATCH_GRAD_NCC = 3 };

XR_API xr_status xr_sm_create(int32_t kind, int32_t device, xr_simmetric* out);
XR_API xr_status xr_sm_destroy(xr_simmetric sm);
XR_API xr_status xr_sm_set_stream(xr_simmetric sm, void* cuda_stream);
/* set_fixed_image (xregImgSimMetric2D.h:69): host float image, copied. */
XR_API xr_status xr_sm_set_fixed_image(xr_simmetric sm, const float* host_img, int64_t rows, int64_t cols);
/* set_mask (xregImgSimMetric2D.h:130): host uint8 image (nonzero = use), NULL clears.
 * NCC / grad-NCC: only masked-in pixels enter the statistics.  Patch metrics: the
 * mask weights the patches and limits each patch's correlation sum, as the
 * xr_patch_options below say. */
XR_API xr_status xr_sm_set_mask(xr_simmetric sm, const uint8_t* host_mask);
/* set_num_moving_images (xregImgSimMetric2D.h:93). */
XR_API xr_status xr_sm_set_num_moving_images(xr_simmetric sm, int64_t n);
/* fixed_image, mask, num_pix_per_proj (xregImgSimMetric2D.h:72,132,139) and the
 * moving-image count: the fixed image as set (rows, cols; up to cap values), the
 * mask (*has_mask = 0 when none) and rows * cols. */
XR_API xr_status xr_sm_fixed_image(xr_simmetric sm, int64_t cap, float* out, int64_t* rows, int64_t* cols);
XR_API xr_status xr_sm_mask(xr_simmetric sm, int64_t cap, uint8_t* out, int32_t* has_mask);
XR_API xr_status xr_sm_num_pix_per_proj(xr_simmetric sm, int64_t* out);
XR_API xr_status xr_sm_num_moving_images(xr_simmetric sm, int64_t* out);
/* set_mov_imgs_buf_from_ray_caster (xregImgSimMetric2DCPU.cpp:43-72): the moving
 * images are read in place from the ray caster's device buffer at proj_offset. */
XR_API xr_status xr_sm_set_mov_imgs_buf_from_ray_caster(xr_simmetric sm, xr_raycaster rc, int64_t proj_offset);
/* set_mov_imgs_host_buf (xregImgSimMetric2D.h:122): num_moving_images host
 * images, copied to the device at every compute (the buffer must stay valid). */
XR_API xr_status xr_sm_set_mov_imgs_host_buf(xr_simmetric sm, const float* host_imgs);
/* set_mov_imgs_host_buf analogue for device memory (xregImgSimMetric2DCPU.cpp:74-88). */
XR_API xr_status xr_sm_set_mov_imgs_device_buf(xr_simmetric sm, const float* d_imgs, int64_t proj_offset);
/* ImgSimMetric2DGradImgParamInterface::set_smooth_img_before_sobel_kernel_radius
 * (default 5 = 5x5 Gaussian; 0 = no smoothing; 3 = 3x3). */
XR_API xr_status xr_sm_set_smooth_img_before_sobel_kernel_radius(xr_simmetric sm, int32_t r);
/* ImgSimMetric2DPatchCommon::set_patch_radius / set_patch_stride (defaults 5 and 1). */
XR_API xr_status xr_sm_set_patch_radius(xr_simmetric sm, int32_t r);
XR_API xr_status xr_sm_set_patch_stride(xr_simmetric sm, int32_t s);
/* Options of the patch metrics, xReg's defaults in brackets:
 * ImgSimMetric2DPatchCommon (xregImgSimMetric2DPatchCommon.h:140-180),
 * ImgSimMetric2DPatchNCCCPU (xregImgSimMetric2DPatchNCCCPU.h:92-94),
 * ImgSimMetric2DPatchGradNCCCPU (xregImgSimMetric2DPatchGradNCCCPU.h:100-104).
 * Patch weights (xregImgSimMetric2DPatchCommon.cpp:306-410): the weight image
 * (user-set, or the fixed-image patch variances) at each patch centre, zero at
 * masked centres when use_mask_for_weighting; else, with a mask and
 * use_mask_for_weighting, the patch's unmasked fraction; normalised to sum 1
 * when normalize_weights_as_prob; otherwise 1.  Moving-image patch variances
 * replace the weight per image (0 at masked centres, normalised; a total at or
 * below 1e-6 gives the value FLT_MAX).  Per patch (xregImgSimMetric2DPatchNCCCPU.cpp:200-287):
 * statistics over all pixels (over masked-in pixels when
 * use_mask_for_patch_stats), correlation sum over masked-in pixels, score
 * 1 - sum; a patch whose weight is at or below 1e-6 is left out when
 * weight_patch_sims_in_combine.  Value: sum of weight x score over the patches
 * used, divided by the patch count (compute_mean_of_patch_sims) or by the sum of
 * their weights (weight_patch_sims_in_combine).  Random subsets
 * (xregImgSimMetric2DPatchCommon.cpp:412-493): each compute draws
 * num_rand_patches patches with probability proportional to the weights,
 * rejecting those closer than rand_patch_min_pixels_sep to one already drawn;
 * xReg seeds that draw from std::random_device, here from rand_seed. */
typedef struct {
  int32_t use_mask_for_weighting;                /* [1] */
  int32_t use_mask_for_patch_stats;              /* [0] */
  int32_t normalize_weights_as_prob;             /* [1] */
  int32_t weight_patch_sims_in_combine;          /* [1] */
  int32_t compute_mean_of_patch_sims;            /* [0] */
  int32_t use_fixed_img_patch_variances_as_wgts; /* [0] */
  int32_t use_mov_img_patch_variances_as_wgts;   /* [0] */
  int32_t use_variances_in_grad_imgs_as_wgts;    /* [0] patch grad-NCC: variances of the gradient images */
  int32_t choose_rand_patches;                   /* [0] */
  int32_t mask_only_for_weights;                 /* [0] 1 = the OpenCL metric's rule
                                                    (xregImgSimMetric2DPatchNCCOCL.cpp:240): the mask
                                                    weights patches but every pixel enters the sums */
  int32_t save_all_per_patch_scores;             /* [0] keep every patch's score (xr_sm_patch_scores) */
  int32_t reserved0;                             /* 0 */
  int64_t num_rand_patches;                      /* [100] */
  double rand_patch_min_pixels_sep;              /* [-1] = sqrt(2) radius; 0 = no check */
  uint64_t rand_seed;
} xr_patch_options;
/* xReg's defaults. */
XR_API xr_status xr_patch_options_default(xr_patch_options* out);
/* Takes effect at the next allocate_resources. */
XR_API xr_status xr_sm_set_patch_options(xr_simmetric sm, const xr_patch_options* o);
XR_API xr_status xr_sm_get_patch_options(xr_simmetric sm, xr_patch_options* o);
/* set_wgt_img (xregImgSimMetric2DPatchCommon.h): host float image of the fixed
 * image's size, read at patch centres; NULL clears.  Takes effect at the next
 * allocate_resources. */
XR_API xr_status xr_sm_set_patch_wgt_img(xr_simmetric sm, const float* host_img);
/* Patches the last compute used, in draw order (row-major patch-centre grid
 * indices); *count receives the number, at most cap are written. */
XR_API xr_status xr_sm_patch_indices_used(xr_simmetric sm, int64_t cap, int64_t* idx, int64_t* count);
/* ImgSimMetric2DPatchCommon::sim_vals_for_each_patch (xregImgSimMetric2DPatchCommon.h:91,
 * filled by xregImgSimMetric2DPatchNCCCPU.cpp:172-180,247-250 and
 * xregImgSimMetric2DPatchGradNCCCPU.cpp:226-240) for moving image img of the last
 * compute, with save_all_per_patch_scores set before allocate_resources: *count =
 * the number of patches in use (all, num_rand_patches, or the set_patches_to_use
 * list); entry i is the score 1 - sum of the i-th patch in use (grid order, draw
 * order or list order), 0.5 (s_x + s_y) for patch grad-NCC (0 for a direction
 * left out by a weight at or below 1e-6); patches left out are 0; every entry
 * is FLT_MAX when the image's value is FLT_MAX. */
XR_API xr_status xr_sm_patch_scores(xr_simmetric sm, int64_t img, int64_t cap, float* out, int64_t* count);
/* ImgSimMetric2DPatchCommon::set_patches_to_use / reset_patches_to_use
 * (xregImgSimMetric2DPatchCommon.cpp:231-241): the patches to use, by grid
 * index, repeats counted (the value sums weight x score over the list and, with
 * weight_patch_sims_in_combine, divides by the list's weights); it takes the
 * place of the grid and of random draws.  n = 0 resets.  Takes effect at the
 * next allocate_resources, which checks the indices against the grid. */
XR_API xr_status xr_sm_set_patches_to_use(xr_simmetric sm, int64_t n, const int64_t* idx);
/* allocate_resources (xregImgSimMetric2D.h:81): fixed-image statistics, gradients
 * and patch statistics are computed once here and stay on the device. */
XR_API xr_status xr_sm_allocate_resources(xr_simmetric sm);
/* compute() (xregImgSimMetric2D.h:88); asynchronous. */
XR_API xr_status xr_sm_compute(xr_simmetric sm);
/* sim_vals() (xregImgSimMetric2D.h:105-112): copies num_moving_images floats; synchronises. */
XR_API xr_status xr_sm_sim_vals(xr_simmetric sm, float* host_dst);
/* Device address of the float[num_moving_images] similarity values. */
XR_API xr_status xr_sm_device_sim_vals(xr_simmetric sm, float** out);

/* ------------------------------------------- population objective (fused) -- */
/* One registration objective: a ray caster (one volume, num_views camera models)
 * and one metric per view, evaluated for a population of candidate poses.  This
 * is Intensity2D3DRegi::obj_fn (xregIntensity2D3DRegi.cpp:571-742) restricted to
 * one object: DRR per (view, pose), metric per view, mean over views
 * (ImgSimMetric2DCombineMean, xregImgSimMetric2DCombine.cpp:79-96). The fused
 * path keeps the DRRs in on-chip/L2 memory and never hands them to the host. */
typedef struct xr_objective_s* xr_objective;

/* The ray caster must have its volume and num_views camera models set; metrics
 * must have their fixed images set (one per view, all XR_SIM_NCC or all
 * XR_SIM_GRAD_NCC or all XR_SIM_PATCH_GRAD_NCC).  max_pop is the largest population. */
XR_API xr_status xr_obj_create(xr_raycaster rc, int32_t vol_idx, int32_t num_views, const xr_simmetric* metrics,
                               int64_t max_pop, xr_objective* out);
XR_API xr_status xr_obj_destroy(xr_objective obj);
/* Evaluates pop poses (row-major 4x4 doubles, camera -> ITK physical, the same
 * pose for every view, like distribute_xforms_among_cam_models) and writes pop
 * floats: the mean over views of each view's metric.  host pointers; synchronises. */
XR_API xr_status xr_obj_eval(xr_objective obj, int64_t pop, const double* host_xforms, float* host_sims);
/* Same with device pointers; asynchronous on the ray caster's stream. */
XR_API xr_status xr_obj_eval_device(xr_objective obj, int64_t pop, const double* d_xforms, float* d_sims);
/* Evaluation path of an objective: 0 (default) = split: the DRR launch, then
 * each metric's launches, replayed as a CUDA graph; 1 = fused: one persistent
 * kernel traces every DRR tile and, as soon as the DRR pixels a metric tile
 * reads are written, computes that tile's grad-NCC moments, then each image's
 * value and each pose's mean over views (grad-NCC with 5x5 smoothing; other
 * metrics keep the split path).  Both give identical values; split measured
 * faster on GB300 (the fused kernel's per-tile barriers and metric reads cost
 * more than the DRR's trip through L2/HBM saves).
 * No counterpart in xReg (its ray caster and metrics are separate passes,
 * xregRayCastLineIntOCL.cpp:39-117 then xregImgSimMetric2DGradImgOCL.cpp:41-163). */
XR_API xr_status xr_obj_set_fused(xr_objective obj, int32_t enable);

/* -------------------------------------------------- allocation-free metric -- */
/* Grad-NCC of num_moving moving images (device, rows*cols floats each, back to
 * back) against a fixed image (device), written to d_sims (device, num_moving
 * floats), asynchronously on cuda_stream, without allocating any device memory.
 * It is for callers that cannot call cudaMalloc on this path: hosts whose device
 * memory belongs to another allocator, or that hand the library only device
 * pointers.  Every intermediate lives in one fixed 16 MiB array inside the
 * library (held on each GPU that loads it until the process exits); requests
 * that need more, or more than 65535 moving images, are refused with
 * XR_ERR_INVALID_ARG.  The first call on a device looks up that array's address
 * (once per device, kept for the life of the process); make it before any
 * stream capture, and do not call this function on a device again after
 * cudaDeviceReset or anything else that recreates its primary context (the
 * kept address is then stale).  Calls share the array, so calls that overlap
 * on the GPU race: keep them on one stream.  smooth_ksize is 5, 3 or 0 as for
 * XR_SIM_GRAD_NCC; no mask.
 * No counterpart in the reference (xReg's metrics always allocate their buffers). */
XR_API xr_status xr_grad_ncc_noalloc(const float* d_fixed, const float* d_moving, int64_t rows, int64_t cols,
                                     int64_t num_moving, int32_t smooth_ksize, float* d_sims, void* cuda_stream);

/* ---------------------------------------------------------- diagnostics -- */
/* Measured L2 read bandwidth of a device (device < 0: the current one), in
 * GB/s: a buffer of `bytes` (at most half the L2) made resident, then read
 * `reps` times with 16-byte L2-cached loads from every SM.  It is the
 * denominator of the DRR kernel's gather roofline.  No counterpart in xReg. */
XR_API xr_status xr_measure_l2_read_bandwidth(int32_t device, int64_t bytes, int32_t reps, double* gbs);

#ifdef __cplusplus
}
#endif

#endif
