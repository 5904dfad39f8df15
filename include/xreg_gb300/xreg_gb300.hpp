// xreg_gb300.hpp -- header-only C++ host classes over the C ABI (xreg_gb300.h)
// with the method names of xReg's RayCaster (lib/ray_cast/xregRayCastInterface.h)
// and ImgSimMetric2D (lib/regi/sim_metrics_2d/xregImgSimMetric2D.h).  Errors come
// back as xreg_gb300::Error (status + message); nothing else is thrown.  The
// classes hold plain arrays instead of ITK/Eigen types; the adapter that derives
// from xreg::RayCaster inside an xReg build converts at its boundary.
#ifndef XREG_GB300_HPP_
#define XREG_GB300_HPP_

#include <array>
#include <cstdint>
#include <stdexcept>
#include <string>
#include <utility>
#include <vector>

#include "../xreg_gb300.h"
#include "../xreg_gb300_io.h"

namespace xreg_gb300 {

class Error : public std::runtime_error {
 public:
  Error(xr_status s, const std::string& m) : std::runtime_error(m), status(s) {}
  xr_status status;
};

class UnsupportedOperationException : public Error {
 public:
  using Error::Error;
};

inline void check(xr_status s) {
  if (s == XR_OK) return;
  const std::string msg = xr_last_error();
  if (s == XR_ERR_UNSUPPORTED) throw UnsupportedOperationException(s, msg);
  throw Error(s, msg);
}

using Mat4 = std::array<double, 16>;  // row-major 4x4

struct CameraModel {
  xr_camera_desc desc{};
  void setup(double focal_len, int64_t nr, int64_t nc, double rs, double cs,
             int32_t frame = XR_CAM_FOCAL_NEG_Z) {
    check(xr_camera_setup_naive(focal_len, nr, nc, rs, cs, frame, &desc));
  }
  int64_t num_det_rows() const { return desc.num_det_rows; }
  int64_t num_det_cols() const { return desc.num_det_cols; }
};

inline CameraModel DownsampleCameraModel(const CameraModel& src, double ds, bool force_even_dims = false) {
  CameraModel d;
  check(xr_camera_downsample(&src.desc, ds, force_even_dims ? 1 : 0, &d.desc));
  return d;
}

struct Volume {
  xr_volume_desc desc{};
  const float* voxels = nullptr;  // host, x fastest; borrowed until set_volumes returns
};

class RayCasterLineIntCUDA {
 public:
  explicit RayCasterLineIntCUDA(int device = -1) { check(xr_rc_create(device, &h_)); }
  ~RayCasterLineIntCUDA() { xr_rc_destroy(h_); }
  RayCasterLineIntCUDA(const RayCasterLineIntCUDA&) = delete;
  RayCasterLineIntCUDA& operator=(const RayCasterLineIntCUDA&) = delete;

  xr_raycaster handle() const { return h_; }

  void set_volume(const Volume& v, int32_t voxel_type = XR_VOXEL_F32) { set_volumes({v}, voxel_type); }
  void set_volumes(const std::vector<Volume>& vols, int32_t voxel_type = XR_VOXEL_F32, float scale = 0.0f) {
    std::vector<xr_volume_desc> d;
    std::vector<const float*> p;
    for (const auto& v : vols) { d.push_back(v.desc); p.push_back(v.voxels); }
    check(xr_rc_set_volumes(h_, (int32_t)vols.size(), d.data(), p.data(), voxel_type, scale));
  }
  void set_camera_model(const CameraModel& c) { set_camera_models({c}); }
  void set_camera_models(const std::vector<CameraModel>& cams) {
    std::vector<xr_camera_desc> d;
    for (const auto& c : cams) d.push_back(c.desc);
    check(xr_rc_set_camera_models(h_, (int32_t)d.size(), d.data()));
    num_cams_ = d.size();
    if (!d.empty()) { rows_ = d[0].num_det_rows; cols_ = d[0].num_det_cols; }
  }
  size_t num_camera_models() const { return num_cams_; }
  void set_num_projs(int64_t n) { check(xr_rc_set_num_projs(h_, n)); }
  int64_t num_projs() const { int64_t n = 0; check(xr_rc_num_projs(h_, &n)); return n; }
  void set_ray_step_size(float s) { check(xr_rc_set_ray_step_size(h_, s)); }
  void set_interp_method(int32_t m) { check(xr_rc_set_interp_method(h_, m)); }
  void use_linear_interp() { set_interp_method(XR_INTERP_LINEAR); }
  void use_proj_store_replace_method() { check(xr_rc_set_proj_store_method(h_, XR_PROJ_STORE_REPLACE)); }
  void use_proj_store_accum_method() { check(xr_rc_set_proj_store_method(h_, XR_PROJ_STORE_ACCUM)); }
  void set_default_bg_pixel_val(float v) { check(xr_rc_set_default_bg_pixel_val(h_, v)); }
  void set_kernel_id(int32_t k) { check(xr_rc_set_kernel_id(h_, k)); }
  void set_bg_projs(const std::vector<const float*>& imgs, bool use = true) {
    check(xr_rc_set_bg_projs(h_, imgs.data(), use ? 1 : 0));
  }
  void set_use_bg_projs(bool use) { check(xr_rc_set_use_bg_projs(h_, use ? 1 : 0)); }
  void set_xforms_cam_to_itk_phys(const std::vector<Mat4>& x) {
    check(xr_rc_set_xforms_cam_to_itk_phys(h_, (int64_t)x.size(), x.empty() ? nullptr : x[0].data()));
  }
  void distribute_xforms_among_cam_models(const std::vector<Mat4>& x) {
    check(xr_rc_distribute_xforms_among_cam_models(h_, (int64_t)x.size(), x.empty() ? nullptr : x[0].data()));
  }
  void distribute_xform_among_cam_models(const Mat4& x) { distribute_xforms_among_cam_models({x}); }
  void set_camera_model_proj_associations(const std::vector<int32_t>& a) {
    check(xr_rc_set_camera_model_proj_associations(h_, (int64_t)a.size(), a.data()));
  }
  std::vector<int32_t> camera_model_proj_associations() const {
    int64_t n = 0;
    check(xr_rc_camera_model_proj_associations(h_, 0, nullptr, &n));
    std::vector<int32_t> out((size_t)n);
    check(xr_rc_camera_model_proj_associations(h_, n, out.data(), &n));
    return out;
  }
  void set_proj_cam_model(int64_t proj_idx, int32_t cam_idx) { check(xr_rc_set_proj_cam_model(h_, proj_idx, cam_idx)); }
  std::vector<Mat4> xforms_cam_to_itk_phys() const {
    int64_t n = 0;
    check(xr_rc_xforms_cam_to_itk_phys(h_, 0, nullptr, &n));
    std::vector<Mat4> out((size_t)n);
    check(xr_rc_xforms_cam_to_itk_phys(h_, n, n ? out[0].data() : nullptr, &n));
    return out;
  }
  void pre_multiply_all_xforms(const Mat4& m) { check(xr_rc_pre_multiply_all_xforms(h_, m.data())); }
  void post_multiply_all_xforms(const Mat4& m) { check(xr_rc_post_multiply_all_xforms(h_, m.data())); }
  int32_t num_vols() const { int32_t n = 0; check(xr_rc_num_vols(h_, &n)); return n; }
  Mat4 xform_img_center_to_itk_phys(int32_t vol_idx = 0) const {
    Mat4 m{};
    check(xr_rc_xform_img_center_to_itk_phys(h_, vol_idx, m.data()));
    return m;
  }
  Mat4 xform_cam_wrt_carm_center_of_rot(int32_t cam_idx = 0) const {
    Mat4 m{};
    check(xr_rc_xform_cam_wrt_carm_center_of_rot(h_, cam_idx, m.data()));
    return m;
  }
  void allocate_resources() { check(xr_rc_allocate_resources(h_)); }
  int64_t max_num_projs_possible() const { int64_t n = 0; check(xr_rc_max_num_projs_possible(h_, &n)); return n; }
  void compute(int32_t vol_idx = 0) { check(xr_rc_compute(h_, vol_idx)); }
  // proj(idx): host copy (xReg returns a shallow view invalidated by the next compute)
  std::vector<float> proj(int64_t idx) const {
    std::vector<float> out((size_t)(rows_ * cols_));
    check(xr_rc_proj(h_, idx, out.data()));
    return out;
  }
  std::vector<float> raw_host_pixel_buf() const {
    std::vector<float> out((size_t)(rows_ * cols_ * num_projs()));
    check(xr_rc_copy_projs_to_host(h_, out.data()));
    return out;
  }
  float* to_cuda_buf() const { float* p = nullptr; check(xr_rc_device_pixel_buf(h_, &p)); return p; }
  // RayCaster::use_other_proj_buf (as RayCasterOCL: this caster writes into the
  // other's device buffer) / use_external_host_pixel_buf
  void use_other_proj_buf(RayCasterLineIntCUDA* other) { check(xr_rc_use_other_proj_buf(h_, other ? other->h_ : nullptr)); }
  void use_external_host_pixel_buf(float* buf) { check(xr_rc_use_external_host_pixel_buf(h_, buf)); }

 private:
  xr_raycaster h_ = nullptr;
  size_t num_cams_ = 0;
  int64_t rows_ = 0, cols_ = 0;
};

class ImgSimMetric2DCUDA {
 public:
  explicit ImgSimMetric2DCUDA(int32_t kind, int device = -1) { check(xr_sm_create(kind, device, &h_)); }
  virtual ~ImgSimMetric2DCUDA() { xr_sm_destroy(h_); }
  ImgSimMetric2DCUDA(const ImgSimMetric2DCUDA&) = delete;
  ImgSimMetric2DCUDA& operator=(const ImgSimMetric2DCUDA&) = delete;

  xr_simmetric handle() const { return h_; }
  void set_fixed_image(const float* img, int64_t rows, int64_t cols) {
    check(xr_sm_set_fixed_image(h_, img, rows, cols));
  }
  void set_mask(const uint8_t* mask) { check(xr_sm_set_mask(h_, mask)); }
  void set_num_moving_images(int64_t n) { check(xr_sm_set_num_moving_images(h_, n)); n_ = n; }
  int64_t num_moving_images() const { return n_; }
  int64_t num_pix_per_proj() const { int64_t n = 0; check(xr_sm_num_pix_per_proj(h_, &n)); return n; }
  // fixed_image / mask (xregImgSimMetric2D.h:72,132): host copies (rows * cols values; empty mask = none)
  std::vector<float> fixed_image() const {
    int64_t r = 0, c = 0;
    check(xr_sm_fixed_image(h_, 0, nullptr, &r, &c));
    std::vector<float> out((size_t)(r * c));
    check(xr_sm_fixed_image(h_, r * c, out.data(), &r, &c));
    return out;
  }
  std::vector<uint8_t> mask() const {
    std::vector<uint8_t> out((size_t)num_pix_per_proj());
    int32_t has = 0;
    check(xr_sm_mask(h_, (int64_t)out.size(), out.data(), &has));
    if (!has) out.clear();
    return out;
  }
  void set_mov_imgs_buf_from_ray_caster(RayCasterLineIntCUDA* rc, int64_t proj_offset = 0) {
    check(xr_sm_set_mov_imgs_buf_from_ray_caster(h_, rc->handle(), proj_offset));
  }
  void set_mov_imgs_host_buf(const float* imgs) { check(xr_sm_set_mov_imgs_host_buf(h_, imgs)); }
  void allocate_resources() { check(xr_sm_allocate_resources(h_)); }
  void compute() { check(xr_sm_compute(h_)); }
  std::vector<float> sim_vals() const {
    std::vector<float> out((size_t)n_);
    check(xr_sm_sim_vals(h_, out.data()));
    return out;
  }
  float sim_val(int64_t i) const { return sim_vals().at((size_t)i); }

 protected:
  xr_simmetric h_ = nullptr;
  int64_t n_ = 0;
};

struct ImgSimMetric2DNCCCUDA : ImgSimMetric2DCUDA {
  explicit ImgSimMetric2DNCCCUDA(int device = -1) : ImgSimMetric2DCUDA(XR_SIM_NCC, device) {}
};

// ImgSimMetric2DPatchCommon (xregImgSimMetric2DPatchCommon.h) setters over xr_patch_options.
class ImgSimMetric2DPatchCUDA : public ImgSimMetric2DCUDA {
 public:
  ImgSimMetric2DPatchCUDA(int32_t kind, int device) : ImgSimMetric2DCUDA(kind, device) {}
  void set_patch_radius(int32_t r) { check(xr_sm_set_patch_radius(h_, r)); }
  void set_patch_stride(int32_t s) { check(xr_sm_set_patch_stride(h_, s)); }
  void set_wgt_img(const float* img) { check(xr_sm_set_patch_wgt_img(h_, img)); }
  void set_use_mask_for_weighting(bool v) { set([&](xr_patch_options& o) { o.use_mask_for_weighting = v; }); }
  void set_use_mask_for_patch_stats(bool v) { set([&](xr_patch_options& o) { o.use_mask_for_patch_stats = v; }); }
  void set_normalize_weights_as_prob(bool v) { set([&](xr_patch_options& o) { o.normalize_weights_as_prob = v; }); }
  void set_weight_patch_sims_in_combine(bool v) {
    set([&](xr_patch_options& o) { o.weight_patch_sims_in_combine = v; });
  }
  void set_compute_mean_of_patch_sims(bool v) { set([&](xr_patch_options& o) { o.compute_mean_of_patch_sims = v; }); }
  // the OpenCL patch metrics' rule: the mask only weights the patches
  void set_mask_only_for_weights(bool v) { set([&](xr_patch_options& o) { o.mask_only_for_weights = v; }); }
  // ImgSimMetric2DPatchCommon::set_save_all_per_patch_scores (xregImgSimMetric2DPatchCommon.h:93)
  void set_save_all_per_patch_scores(bool v) { set([&](xr_patch_options& o) { o.save_all_per_patch_scores = v; }); }
  void set_use_fixed_img_patch_variances_as_wgts(bool v) {
    set([&](xr_patch_options& o) { o.use_fixed_img_patch_variances_as_wgts = v; });
  }
  void set_use_mov_img_patch_variances_as_wgts(bool v) {
    set([&](xr_patch_options& o) { o.use_mov_img_patch_variances_as_wgts = v; });
  }
  // random patch subsets; xReg seeds the draw from std::random_device, here from seed
  void set_choose_rand_patches(bool v, int64_t num = 100, double min_sep = -1.0, uint64_t seed = 0) {
    set([&](xr_patch_options& o) {
      o.choose_rand_patches = v;
      o.num_rand_patches = num;
      o.rand_patch_min_pixels_sep = min_sep;
      o.rand_seed = seed;
    });
  }
  std::vector<int64_t> patch_indices_used() const {
    int64_t n = 0;
    check(xr_sm_patch_indices_used(h_, 0, nullptr, &n));
    std::vector<int64_t> out((size_t)n);
    check(xr_sm_patch_indices_used(h_, n, out.data(), &n));
    return out;
  }
  // set_patches_to_use / reset_patches_to_use (xregImgSimMetric2DPatchCommon.h:121-123)
  void set_patches_to_use(const std::vector<int64_t>& idx) {
    check(xr_sm_set_patches_to_use(h_, (int64_t)idx.size(), idx.empty() ? nullptr : idx.data()));
  }
  void reset_patches_to_use() { check(xr_sm_set_patches_to_use(h_, 0, nullptr)); }
  // sim_vals_for_each_patch (xregImgSimMetric2DPatchCommon.h:91), indexed [patch][moving image]
  std::vector<std::vector<float>> sim_vals_for_each_patch(int64_t num_mov_imgs) const {
    int64_t n = 0;
    check(xr_sm_patch_scores(h_, 0, 0, nullptr, &n));
    std::vector<std::vector<float>> out((size_t)n, std::vector<float>((size_t)num_mov_imgs));
    std::vector<float> one((size_t)n);
    for (int64_t m = 0; m < num_mov_imgs; ++m) {
      check(xr_sm_patch_scores(h_, m, n, one.data(), &n));
      for (int64_t p = 0; p < n; ++p) out[(size_t)p][(size_t)m] = one[(size_t)p];
    }
    return out;
  }

 protected:
  template <typename F>
  void set(F f) {
    xr_patch_options o;
    check(xr_sm_get_patch_options(h_, &o));
    f(o);
    check(xr_sm_set_patch_options(h_, &o));
  }
};

struct ImgSimMetric2DPatchNCCCUDA : ImgSimMetric2DPatchCUDA {
  explicit ImgSimMetric2DPatchNCCCUDA(int device = -1) : ImgSimMetric2DPatchCUDA(XR_SIM_PATCH_NCC, device) {}
};

struct ImgSimMetric2DGradNCCCUDA : ImgSimMetric2DCUDA {
  explicit ImgSimMetric2DGradNCCCUDA(int device = -1) : ImgSimMetric2DCUDA(XR_SIM_GRAD_NCC, device) {}
  void set_smooth_img_before_sobel_kernel_radius(int32_t r) {
    check(xr_sm_set_smooth_img_before_sobel_kernel_radius(h_, r));
  }
};

struct ImgSimMetric2DPatchGradNCCCUDA : ImgSimMetric2DPatchCUDA {
  explicit ImgSimMetric2DPatchGradNCCCUDA(int device = -1) : ImgSimMetric2DPatchCUDA(XR_SIM_PATCH_GRAD_NCC, device) {}
  void set_smooth_img_before_sobel_kernel_radius(int32_t r) {
    check(xr_sm_set_smooth_img_before_sobel_kernel_radius(h_, r));
  }
  // ImgSimMetric2DPatchGradNCCCPU::set_use_variances_in_grad_imgs_as_wgts
  void set_use_variances_in_grad_imgs_as_wgts(bool v) { set([&](xr_patch_options& o) { o.use_variances_in_grad_imgs_as_wgts = v; }); }
};

// Intensity2D3DRegi::obj_fn for one object over a population of poses.
class PopulationObjective {
 public:
  PopulationObjective(RayCasterLineIntCUDA& rc, const std::vector<ImgSimMetric2DCUDA*>& metrics, int64_t max_pop,
                      int32_t vol_idx = 0) {
    std::vector<xr_simmetric> hs;
    for (auto* m : metrics) hs.push_back(m->handle());
    check(xr_obj_create(rc.handle(), vol_idx, (int32_t)hs.size(), hs.data(), max_pop, &h_));
  }
  ~PopulationObjective() { xr_obj_destroy(h_); }
  PopulationObjective(const PopulationObjective&) = delete;
  PopulationObjective& operator=(const PopulationObjective&) = delete;
  std::vector<float> operator()(const std::vector<Mat4>& poses) {
    std::vector<float> out(poses.size());
    check(xr_obj_eval(h_, (int64_t)poses.size(), poses.empty() ? nullptr : poses[0].data(), out.data()));
    return out;
  }
  // the fused DRR + grad-NCC kernel instead of the split launches (identical values)
  void set_fused(bool enable) { check(xr_obj_set_fused(h_, enable ? 1 : 0)); }
  xr_objective handle() const { return h_; }

 private:
  xr_objective h_ = nullptr;
};

// SimpleRayCasterWrapperFn (xregRayCastInterface.h:552-573, xregRayCastInterface.cpp:456-533):
// one projection per camera of every volume in vols_to_proj (all volumes when
// empty) at cam_world_to_vols[i], the first replacing and the rest accumulating,
// optionally about intermediate frames; the ray caster's projection count and
// camera associations are restored afterwards.
struct SimpleRayCasterWrapperFn {
  RayCasterLineIntCUDA* ray_caster = nullptr;
  std::vector<Mat4> cam_world_to_vols;
  std::vector<Mat4> inter_frames;
  std::vector<bool> inter_frames_wrt_vol;
  std::vector<Mat4> ref_frames_cam_world_to_vol;
  std::vector<int32_t> vols_to_proj;
  std::vector<std::vector<float>> projs;

  static Mat4 mul(const Mat4& a, const Mat4& b) {
    Mat4 t{};
    for (int i = 0; i < 4; ++i)
      for (int j = 0; j < 4; ++j) {
        double v = 0.0;
        for (int k = 0; k < 4; ++k) v += a[(size_t)(i * 4 + k)] * b[(size_t)(k * 4 + j)];
        t[(size_t)(i * 4 + j)] = v;
      }
    return t;
  }
  static Mat4 affine_inverse(const Mat4& m) {  // [A t; 0 1]^-1 = [A^-1, -A^-1 t]
    const double a = m[0], b = m[1], c = m[2], d = m[4], e = m[5], f = m[6], g = m[8], h = m[9], k = m[10];
    const double A = e * k - f * h, B = -(d * k - f * g), C = d * h - e * g;
    const double det = a * A + b * B + c * C;
    if (det == 0.0) throw Error(XR_ERR_INVALID_ARG, "SimpleRayCasterWrapperFn: singular intermediate frame");
    const double inv[9] = {A / det, -(b * k - c * h) / det, (b * f - c * e) / det,
                           B / det, (a * k - c * g) / det, -(a * f - c * d) / det,
                           C / det, -(a * h - b * g) / det, (a * e - b * d) / det};
    Mat4 t{};
    for (int i = 0; i < 3; ++i) {
      for (int j = 0; j < 3; ++j) t[(size_t)(i * 4 + j)] = inv[i * 3 + j];
      t[(size_t)(i * 4 + 3)] = -(inv[i * 3] * m[3] + inv[i * 3 + 1] * m[7] + inv[i * 3 + 2] * m[11]);
    }
    t[15] = 1.0;
    return t;
  }

  void operator()() {
    RayCasterLineIntCUDA& rc = *ray_caster;
    const bool listed = !vols_to_proj.empty();
    const size_t nv = listed ? vols_to_proj.size() : (size_t)rc.num_vols();
    if (cam_world_to_vols.size() != nv) throw Error(XR_ERR_INVALID_ARG, "SimpleRayCasterWrapperFn: one pose per volume");
    const bool inter = !inter_frames.empty();
    if (inter && (inter_frames.size() != nv || inter_frames_wrt_vol.size() != nv || ref_frames_cam_world_to_vol.size() != nv))
      throw Error(XR_ERR_INVALID_ARG, "SimpleRayCasterWrapperFn: one intermediate frame per volume");
    const int64_t num_cams = (int64_t)rc.num_camera_models();
    const int64_t prev_num_projs = rc.num_projs();
    const std::vector<int32_t> cam_assocs = rc.camera_model_proj_associations();
    rc.set_num_projs(num_cams);
    for (size_t v = 0; v < nv; ++v) {
      if (v == 0) rc.use_proj_store_replace_method();
      else rc.use_proj_store_accum_method();
      rc.distribute_xform_among_cam_models(cam_world_to_vols[v]);
      if (inter) {
        if (inter_frames_wrt_vol[v]) {
          rc.pre_multiply_all_xforms(inter_frames[v]);
          rc.post_multiply_all_xforms(mul(affine_inverse(inter_frames[v]), ref_frames_cam_world_to_vol[v]));
        } else {
          rc.pre_multiply_all_xforms(mul(ref_frames_cam_world_to_vol[v], inter_frames[v]));
          rc.post_multiply_all_xforms(affine_inverse(inter_frames[v]));
        }
      }
      rc.compute(listed ? vols_to_proj[v] : (int32_t)v);
    }
    projs.assign((size_t)num_cams, {});
    for (int64_t c = 0; c < num_cams; ++c) projs[(size_t)c] = rc.proj(c);
    rc.set_num_projs(prev_num_projs);
    if ((int64_t)cam_assocs.size() == prev_num_projs && prev_num_projs > 0) rc.set_camera_model_proj_associations(cam_assocs);
  }
};

// Poses on disk (lib/itk/xregITKIOUtils.h:46-57), ITK text transform files.
inline Mat4 ReadITKAffineTransformFromFile(const std::string& path) {
  Mat4 m{};
  check(xr_itk_affine_transform_read(path.c_str(), m.data()));
  return m;
}
inline Mat4 ReadSlicerAffineTransformFromFile(const std::string& path) {
  Mat4 m{};
  check(xr_itk_slicer_affine_transform_read(path.c_str(), m.data()));
  return m;
}
inline void WriteITKAffineTransform(const std::string& path, const Mat4& xform) {
  check(xr_itk_affine_transform_write(path.c_str(), xform.data()));
}

}  // namespace xreg_gb300

#endif
