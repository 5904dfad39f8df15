/*
 * xreg_gb300_regi.h -- C ABI of the registration side: the CMA-ES population
 * optimizer that drives the population objective (xreg_gb300.h, xr_obj_*).
 * Plain C types, xr_status returns, xr_last_error() for messages.
 * Citations are paths inside the xReg project.
 */
#ifndef XREG_GB300_REGI_H_
#define XREG_GB300_REGI_H_

#include "xreg_gb300.h"

#ifdef __cplusplus
extern "C" {
#endif

/* CMA-ES state (double precision, on the host or attached to a device).  Replaces the vendored cmaes.c calls in
 * Intensity2D3DRegiCMAES::run (xregIntensity2D3DRegiCMAES.cpp:122-224):
 * cmaes_init, cmaes_SamplePopulation, cmaes_ReSampleSingle,
 * cmaes_UpdateDistribution, cmaes_TestForTermination, cmaes_GetPtr("xmean"/"xbestever"). */
typedef struct xr_cmaes_s* xr_cmaes;

/* cmaes_init (third_party/cmaes/cmaes_interface.h): dim parameters starting at
 * xstart with per-coordinate initial standard deviations; lambda candidates per
 * generation; seed 0 is a valid fixed seed (xReg's 0 means "seed from the clock";
 * pass your own seed to reproduce a run). */
XR_API xr_status xr_cmaes_create(int32_t dim, const double* xstart, const double* stddevs, int32_t lambda,
                                 uint64_t seed, xr_cmaes* out);
XR_API xr_status xr_cmaes_destroy(xr_cmaes e);
/* stopTolFun / stopTolX / stopMaxIter (xregIntensity2D3DRegiCMAES.cpp:124-126). */
XR_API xr_status xr_cmaes_set_stop(xr_cmaes e, double tol_fun, double tol_x, int64_t max_iter);
/* cmaes_SamplePopulation: writes lambda x dim candidates. */
XR_API xr_status xr_cmaes_sample_population(xr_cmaes e, double* pop);
/* cmaes_ReSampleSingle: redraws candidate k (bounds rejection, xregIntensity2D3DRegiCMAES.cpp:162-191)
 * and writes it into row k of pop. */
XR_API xr_status xr_cmaes_resample_single(xr_cmaes e, int32_t k, double* pop);
/* cmaes_UpdateDistribution with the lambda objective values of the last sample. */
XR_API xr_status xr_cmaes_update_distribution(xr_cmaes e, const double* fvals);
/* cmaes_TestForTermination: *reason = 0 continue, 1 function-value range below
 * tol_fun, 2 step sizes below tol_x, 3 iteration limit, 4 numerical failure. */
XR_API xr_status xr_cmaes_test_termination(xr_cmaes e, int32_t* reason);
/* Candidates per generation (lambda). */
XR_API xr_status xr_cmaes_lambda(xr_cmaes e, int32_t* lambda);
/* Current mean, best candidate seen and its value, step size, generation count
 * (any pointer may be NULL). */
XR_API xr_status xr_cmaes_get(xr_cmaes e, double* mean, double* best_x, double* best_f, double* sigma,
                              int64_t* generation);
/* Moves the state to device memory (device < 0: the current one; at most 8
 * parameters).  While attached, xr_regi_jobset_step draws each generation's
 * candidates inside its geometry launch and runs the update inside its metric
 * launch, with the same bits as the host methods: one source for both
 * (counter-based normals, one rounding per operation, the transcendental
 * functions as series of our own).  sample_population, resample_single,
 * update_distribution and set_stop refuse while attached; get,
 * test_termination and export_state read the device copy.  No counterpart in
 * xReg (its optimizer runs on the host between evaluations). */
XR_API xr_status xr_cmaes_attach_device(xr_cmaes e, int32_t device);
/* Brings an attached state back to host memory (no-op when on the host). */
XR_API xr_status xr_cmaes_detach_device(xr_cmaes e);
/* Size of the whole state block, and a copy of it (parameters, distribution,
 * eigenbasis, last population with its draws and values, history). */
XR_API xr_status xr_cmaes_state_bytes(xr_cmaes e, int64_t* bytes);
XR_API xr_status xr_cmaes_export_state(xr_cmaes e, void* out, int64_t bytes);

/* Bound-constrained derivative-free trust-region optimizer for a final level, in
 * place of NLopt's LN_BOBYQA (Intensity2D3DRegiBOBYQA, xregIntensity2D3DRegiBOBYQA.cpp:28-39;
 * Intensity2D3DRegiNLOptInterface::run, xregIntensity2D3DRegiNLOptInterface.cpp:83-188):
 * Powell's BOBYQA method -- a full quadratic model through 2n+1 interpolation
 * points, changed by the least Frobenius norm of its Hessian change as each new
 * point replaces one, box- and ball-constrained trust-region steps, geometry
 * steps, rho shrunk to rho_end -- with at most 2n+1 + max_iter evaluations as
 * xReg caps NLopt.  The first ask is the 2n+1 initial points; each later ask
 * is one point (or `points` of them after xr_dfo_set_batch); tell takes their
 * values in the same order.  rho is in the units of the coordinate with the
 * widest bounds; the others are scaled by their widths. */
typedef struct xr_dfo_s* xr_dfo;
XR_API xr_status xr_dfo_create(int32_t dim, const double* x0, const double* lower, const double* upper,
                               double rho_beg, double rho_end, int64_t max_iter, xr_dfo* out);
XR_API xr_status xr_dfo_destroy(xr_dfo d);
/* Points per ask after the initial set (1 <= points <= 2*dim+2; default 1):
 * the trust-region step and points-1 geometry steps of the farthest
 * interpolation points, to evaluate together; max_iter then counts asks.
 * Before the first tell. */
XR_API xr_status xr_dfo_set_batch(xr_dfo d, int32_t points);
/* Writes the points to evaluate (rows of dim doubles) into pts, room for
 * 2*dim+2 rows; *count = rows.  Refused once the optimizer has stopped. */
XR_API xr_status xr_dfo_ask(xr_dfo d, double* pts, int32_t* count);
/* Values of the last asked points, in order (not finite = worse than every finite value). */
XR_API xr_status xr_dfo_tell(xr_dfo d, const double* fvals);
/* *reason: 0 continue, 2 rho reached rho_end, 3 evaluation limit. */
XR_API xr_status xr_dfo_test_termination(xr_dfo d, int32_t* reason);
XR_API xr_status xr_dfo_get(xr_dfo d, double* best_x, double* best_f, double* rho, int64_t* iterations);
/* Objective values told so far. */
XR_API xr_status xr_dfo_evaluations(xr_dfo d, int64_t* evaluations);

/* ------------------------------------------------ one registration level -- */
/* The level loop of Intensity2D3DRegiCMAES::run (xregIntensity2D3DRegiCMAES.cpp:76-247)
 * or of the trust-region level in NLopt LN_BOBYQA's place
 * (xregIntensity2D3DRegiNLOptInterface.cpp:83-188), run natively over a population
 * objective (every population / batch of points is one xr_obj_eval).  Offsets x
 * are SE(3) Lie-algebra vectors [w (rad), v (mm)] (SE3OptVarsLieAlg,
 * xregSE3OptVars.cpp:128-137) and a candidate pose is
 * centre * ExpSE3(x) * centre^-1 * start_pose (centre: a rigid frame at the volume
 * centre, xregIntensity2D3DRegi.cpp:1028-1099); 4x4 row-major doubles. */
enum { XR_REGI_CMAES = 0, XR_REGI_DFO = 1 };
typedef struct {
  int32_t optimizer;   /* XR_REGI_CMAES or XR_REGI_DFO */
  int32_t lambda;      /* CMA-ES population */
  double sigma[6];     /* CMA-ES initial standard deviations */
  double bounds[6];    /* half-widths of the box: CMA-ES redraws candidates outside (0 = unbounded);
                          the trust region needs all six */
  int64_t max_iters;
  double tol_fun, tol_x;    /* CMA-ES stopping tolerances */
  double rho_beg, rho_end;  /* trust-region radii (mm-scaled, as xr_dfo_create) */
  uint64_t seed;            /* CMA-ES random stream */
} xr_regi_level_params;
XR_API xr_status xr_regi_level_params_default(int32_t optimizer, xr_regi_level_params* out);
/* best_pose: the pose of the best offset found; best_value, iterations (CMA-ES
 * generations / trust-region iterations) and stop_reason (xr_cmaes_test_termination
 * or xr_dfo_test_termination codes) may be NULL. */
XR_API xr_status xr_regi_run_level(xr_objective obj, const double* centre, const double* start_pose,
                                   const xr_regi_level_params* params, double* best_pose, double* best_value,
                                   int64_t* iterations, int32_t* stop_reason);

/* ---------------------------------------------------- data preparation -- */
/* HUToLinAttFilter (lib/image/xregHUToLinAtt.cpp:45-69): device float HU ->
 * device float attenuation (1/mm), mu_water 0.02683, mu_air 0.02485e-4,
 * hu_lower -1000, computed in double; asynchronous on cuda_stream. */
XR_API xr_status xr_hu_to_lin_att(const float* d_hu, int64_t n, float* d_mu, void* cuda_stream);
/* Output size of DownsampleImage: floor(n * factor + 0.5) per axis, 0 < factor <= 1. */
XR_API xr_status xr_downsample_image_size(int64_t rows, int64_t cols, double factor, int64_t* out_rows,
                                          int64_t* out_cols);
/* DownsampleProjData's image part (lib/image/xregProjData.cpp:40-53 ->
 * DownsampleImage, lib/itk/xregITKResampleUtils.h:51-131,183-187): discrete
 * Gaussian of variance (0.5/factor)^2 pixels (max error 0.01, replicated edges,
 * rounded to float) when factor < 1, then cubic B-spline resampling (the default
 * interpolator: mirror-boundary prefilter, 4 x 4 weights) at continuous index
 * i / factor onto the xr_downsample_image_size grid; points outside
 * [-0.5, n - 0.5) are 0.  d_scratch: 2 * rows * cols doubles.  The camera model
 * of the level comes from xr_camera_downsample.  Asynchronous. */
XR_API xr_status xr_downsample_image(const float* d_src, int64_t rows, int64_t cols, double factor,
                                     double* d_scratch, float* d_dst, void* cuda_stream);
/* ProjPreProc (lib/image/xregProjPreProc.cpp:31-139), boundary crop:
 * CropBoundaryPixels (lib/image/xregProjData.cpp:543-567) ->
 * UpdateCameraModelFor2DROI (lib/transforms/xregPerspectiveXform.cpp:482-503):
 * the principal point moves by -width on both axes, width pixels go from
 * every side. */
XR_API xr_status xr_camera_crop_boundary(const xr_camera_desc* src, int64_t width, xr_camera_desc* out);
/* CropImage2DBoundary (lib/itk/xregITKCropPadUtils.h:89-114): d_dst receives the
 * (rows - 2 width) x (cols - 2 width) interior.  Asynchronous. */
XR_API xr_status xr_crop_image_boundary(const float* d_src, int64_t rows, int64_t cols, int64_t width,
                                        float* d_dst, void* cuda_stream);
/* ProjPreProc's log remap, ImageIntensLogTransFilter (lib/image/xregImageIntensLogTrans.cpp:52-146):
 * use_max_as_i0 1 (ProjPreProc's setting) takes I0 = maximum of the image
 * smoothed by a discrete Gaussian of variance 2 pixels, else I0 = i0;
 * out = -log(x / I0) for x > 1e-6, else -log(min_pos / I0) with min_pos the
 * smallest value above 1e-6; float arithmetic.  d_scratch: rows * cols + 1025
 * doubles.  Asynchronous. */
XR_API xr_status xr_log_remap(const float* d_src, int64_t rows, int64_t cols, int32_t use_max_as_i0, float i0,
                              double* d_scratch, float* d_dst, void* cuda_stream);

/* Job set: evaluates one population for each of several registrations (each an
 * xr_objective with its own volume, cameras, fixed images and population size)
 * with ONE DRR launch over all their (tile, projection) work items (each job
 * in its autotuned block shape and sample loop), followed by one batched
 * grad-NCC launch over every job's images.  This is the multi-job batching of many
 * concurrent Intensity2D3DRegiCMAES runs (each calls obj_fn per iteration,
 * xregIntensity2D3DRegi.cpp:571-742); xReg itself has no counterpart and runs
 * them one after another.  Values are identical to evaluating each objective
 * alone.  Objectives passed in one call must be distinct and live on the job
 * set's device; any subset may be passed on any call (continuous batching). */
typedef struct xr_jobset_s* xr_jobset;
XR_API xr_status xr_jobset_create(int32_t device, xr_jobset* out);
XR_API xr_status xr_jobset_destroy(xr_jobset js);
XR_API xr_status xr_jobset_set_stream(xr_jobset js, void* cuda_stream);
/* pops[i] poses (row-major 4x4 doubles, camera -> ITK physical) for objs[i]
 * from host memory, values to host memory; synchronises. */
XR_API xr_status xr_jobset_eval(xr_jobset js, int32_t num_jobs, const xr_objective* objs, const int64_t* pops,
                                const double* const* host_xforms, float* const* host_sims);
/* Same with device pointers; asynchronous on the job set's stream. */
XR_API xr_status xr_jobset_eval_device(xr_jobset js, int32_t num_jobs, const xr_objective* objs,
                                       const int64_t* pops, const double* const* d_xforms, float* const* d_sims);
/* Work items of the last step's DRR launches and blocks of the largest one
 * (one block per item on the split path; the device-filling grid of the fused
 * kernel). */
XR_API xr_status xr_jobset_last_launch(xr_jobset js, int64_t* work_items, int32_t* blocks);
/* Evaluation path of a job set.  0 (default): one geometry launch for every
 * job, one DRR launch per (voxel type, layout) group, one batched
 * grad-NCC launch over every job's images (with the per-image FP64 combine and
 * the mean over views): three launches for jobs of one voxel type.  1: one
 * geometry launch and one fused DRR + grad-NCC launch per group.  Jobs with
 * other metrics run their metric launches after the DRR either way.  Values
 * identical either way.  No counterpart in xReg. */
XR_API xr_status xr_jobset_set_fused(xr_jobset js, int32_t enable);
/* DRR work items of the split step.  Mode 0 (default): one item per (tile,
 * projection) in each job's autotuned block shape.  Mode 2: every job's items
 * are (8x8-pixel tile, 4 consecutive projections), each block mapping the 4
 * poses' rays to threads by how close they are: a 2x4-pixel sub-tile under all
 * 4 poses per warp when the tile's central ray enters and leaves the volume
 * within a voxel under all 4 poses (the lanes share cells), one projection per
 * pair of warps otherwise.  Mode 1: grouped items only for jobs whose next
 * poses lie within a voxel of each other -- host poses whose volume corners
 * move less than the smallest spacing between them; a device optimizer's
 * sampling distribution (3 sigma sqrt(C_ii) after its last update) that does.
 * Identical values in every mode.  No counterpart in xReg. */
XR_API xr_status xr_jobset_set_pose_groups(xr_jobset js, int32_t mode);
/* Jobs of the last step that ran pose-grouped DRR items. */
XR_API xr_status xr_jobset_last_pose_grouped(xr_jobset js, int32_t* jobs);
/* Kernel launches the last step issued (not counting the autotuner's timed
 * launches on a shape's first fused step). */
XR_API xr_status xr_jobset_last_kernel_launches(xr_jobset js, int32_t* launches);

/* One generation of several registrations in one call: for each job the loop
 * body of Intensity2D3DRegiCMAES::run (xregIntensity2D3DRegiCMAES.cpp:154-226:
 * sample, redraw candidates outside the bounds, evaluate, update, test for
 * termination) or of the trust-region level (ask, evaluate, tell, test), with
 * every job's population evaluated by ONE xr_jobset_eval.  The optimizer state
 * lives in the caller's xr_cmaes / xr_dfo handle, which advances here; the
 * offsets x map to poses  centre * ExpSE3(x) * centre^-1 * start_pose  as in
 * xr_regi_run_level.  stop[i] receives job i's termination reason (0 = keep
 * going; xr_cmaes_test_termination / xr_dfo_test_termination codes). */
typedef struct {
  xr_objective obj;
  int32_t optimizer;   /* XR_REGI_CMAES (opt is an xr_cmaes) or XR_REGI_DFO (an xr_dfo) */
  int32_t reserved;    /* 0 */
  void* opt;
  double centre[16];
  double start_pose[16];
  double bounds[6];    /* CMA-ES: |x_i| <= bounds[i] (0 = unbounded) */
} xr_regi_step_job;
XR_API xr_status xr_regi_jobset_step(xr_jobset js, int32_t num_jobs, const xr_regi_step_job* jobs, int32_t* stop,
                                     int32_t* evaluated /* [num_jobs] poses evaluated per job, or NULL */);

/* The pose of each parameter vector x (an se(3) tangent: 3 rotation, 3
 * translation) in a registration level: pose = C * Exp(x) * C^-1 * start_pose,
 * C the centre of rotation frame (Intensity2D3DRegiCMAES::run's
 * SE3OptVarsLieAlg x centre-of-rotation composition, xregIntensity2D3DRegiCMAES.cpp).
 * xs [n, 6], poses [n, 16] row-major; the map every level driver here uses. */
XR_API xr_status xr_regi_pose_map(const double* centre, const double* start_pose, int64_t n, const double* xs,
                                  double* poses);

#ifdef __cplusplus
}
#endif

#endif
