// xr_capi.cu -- the extern "C" boundary: handles, validation, device buffers,
// stream ordering and CUDA-graph capture of the population objective.
// Nothing here throws across the ABI; every entry point returns an xr_status.
#include "xr_internal.h"
#include "xr_posespread.h"
#include "xreg_gb300_regi.h"

#include <algorithm>
#include <cfloat>
#include <cmath>
#include <cstring>
#include <memory>
#include <mutex>
#include <new>
#include <random>
#include <unordered_map>
#include <string>
#include <vector>

namespace xr {

static thread_local std::string g_last_error;

void set_error(const std::string& msg) { g_last_error = msg; }

xr_status fail(xr_status code, const std::string& msg) {
  g_last_error = msg;
  return code;
}

xr_status cuda_fail(cudaError_t e, const char* what) {
  g_last_error = std::string(what) + ": " + cudaGetErrorName(e) + " (" + cudaGetErrorString(e) + ")";
  return e == cudaErrorMemoryAllocation ? XR_ERR_OUT_OF_MEMORY : XR_ERR_CUDA;
}

namespace {

// Owning device allocation.
struct DevBuf {
  void* p = nullptr;
  size_t bytes = 0;
  DevBuf() = default;
  DevBuf(const DevBuf&) = delete;
  DevBuf& operator=(const DevBuf&) = delete;
  ~DevBuf() { release(); }
  void release() {
    if (p) cudaFree(p);
    p = nullptr;
    bytes = 0;
  }
  // Grows (never shrinks) to at least n bytes; contents are not preserved.
  cudaError_t reserve(size_t n) {
    if (n <= bytes && p) return cudaSuccess;
    release();
    if (n == 0) n = 16;
    cudaError_t e = cudaMalloc(&p, n);
    if (e != cudaSuccess) { p = nullptr; return e; }
    bytes = n;
    return cudaSuccess;
  }
  template <typename T>
  T* as() const { return static_cast<T*>(p); }
};

struct DeviceGuard {
  int prev = -1;
  explicit DeviceGuard(int dev) {
    if (dev >= 0) {
      cudaGetDevice(&prev);
      if (prev != dev) cudaSetDevice(dev);
      else prev = -1;
    }
  }
  ~DeviceGuard() { if (prev >= 0) cudaSetDevice(prev); }
};

__global__ void convert_voxels_kernel(const float* __restrict__ in, int64_t n, float scale, int vt, void* out) {
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    const float v = in[i] * scale;
    if (vt == XR_VOXEL_F16) static_cast<__half*>(out)[i] = __float2half_rn(v);
    else static_cast<__nv_bfloat16*>(out)[i] = __float2bfloat16_rn(v);
  }
}

__global__ void max_abs_kernel(const float* __restrict__ in, int64_t n, unsigned int* out) {
  unsigned int m = 0;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    const float a = fabsf(in[i]);
    if (a == a) m = max(m, __float_as_uint(a));
  }
  for (int o = 16; o > 0; o >>= 1) m = max(m, __shfl_down_sync(0xffffffffu, m, o));
  if ((threadIdx.x & 31) == 0) atomicMax(out, m);
}

__global__ void cam_idx_distribute_kernel(int32_t* out, int64_t n, int64_t per_cam) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) out[i] = (int32_t)(i / per_cam);
}

// Live-handle registry: handles that refer to other handles (a metric bound to
// a ray caster, an objective over both) store the peer's id and look it up
// before every use, so destroying handles in any order never dereferences a
// freed object.
std::mutex g_reg_mu;
std::unordered_map<const void*, uint64_t> g_live;
uint64_t g_next_id = 1;

uint64_t reg_add(const void* p) {
  std::lock_guard<std::mutex> lk(g_reg_mu);
  const uint64_t id = g_next_id++;
  g_live[p] = id;
  return id;
}

void reg_remove(const void* p) {
  std::lock_guard<std::mutex> lk(g_reg_mu);
  g_live.erase(p);
}

bool reg_alive(const void* p, uint64_t id) {
  if (!p) return false;
  std::lock_guard<std::mutex> lk(g_reg_mu);
  auto it = g_live.find(p);
  return it != g_live.end() && it->second == id;
}

bool reg_contains(const void* p) {
  std::lock_guard<std::mutex> lk(g_reg_mu);
  return g_live.count(p) != 0;
}

bool finite_all(const double* v, int64_t n) {
  for (int64_t i = 0; i < n; ++i)
    if (!std::isfinite(v[i])) return false;
  return true;
}

}  // namespace
}  // namespace xr

using namespace xr;

// ===================================================================== handles
struct xr_raycaster_s {
  uint64_t id = 0;
  int device = 0;
  cudaStream_t own_stream = nullptr;
  cudaStream_t ext_stream = nullptr;
  bool has_ext_stream = false;

  struct Vol {
    xr_volume_desc desc;
    DevBuf voxels;
    DevBuf cells;            // CELL8 copy (empty when not built)
    int32_t type = XR_VOXEL_F32;
    float inv_scale = 1.0f;
    int32_t cs[2] = {0, 0};     // CELL8 cell strides (VolView::cs)
    bool has_support = false;   // support box of the non-zero voxels (empty-space skipping)
    float sup_lo[3] = {0, 0, 0}, sup_hi[3] = {0, 0, 0};
    DevBuf occ;                 // macro-cell occupancy bitmask
    int32_t nmx = 0, nmy = 0, nmz = 0;
  };
  bool skip_empty = true;
  bool build_cells = true;
  int32_t cfg_layout = XR_LAYOUT_AUTO, cfg_bw = 2, cfg_unroll = 1, cfg_warp_rows = 4;  // requested
  int32_t last_layout = -1, last_bw = 0, last_unroll = 0, last_warp_rows = 0;          // used by the last compute
  std::vector<std::unique_ptr<Vol>> vols;
  std::vector<xr_camera_desc> cams;
  DevBuf d_cams;
  bool cams_dirty = true;

  int64_t num_projs = 0;
  int64_t capacity = 0;   // projections allocated
  float step = 1.0f;
  int32_t interp = XR_INTERP_LINEAR;
  int32_t store = XR_PROJ_STORE_REPLACE;
  float default_bg = 0.0f;
  int32_t kernel_id = XR_LINE_INT_SUM;
  DevBuf d_bg;
  bool has_bg = false;
  bool use_bg = false;

  std::vector<double> xforms;      // pose_count * 16
  int64_t pose_count = 0;          // projection p uses pose (p % pose_count)
  bool xforms_dirty = true;
  bool xforms_on_device = false;   // last set through a device pointer
  std::vector<int32_t> cam_idx;    // num_projs
  bool cam_idx_dirty = true;

  DevBuf d_xforms, d_cam_idx, d_geo, d_proj, d_counters;
  xr_raycaster other = nullptr;    // use_other_proj_buf: writes into this caster's buffer
  uint64_t other_id = 0;
  float* ext_host = nullptr;       // use_external_host_pixel_buf: copy of the images after each compute
  bool allocated = false;
  bool count_samples = false;
  uint64_t generation = 1;         // bumps on every change that affects launches

  cudaStream_t stream() const { return has_ext_stream ? ext_stream : own_stream; }
  int64_t rows() const { return cams.empty() ? 0 : cams[0].num_det_rows; }
  int64_t cols() const { return cams.empty() ? 0 : cams[0].num_det_cols; }
};

struct xr_simmetric_s {
  uint64_t id = 0;
  int32_t kind = XR_SIM_NCC;
  int device = 0;
  cudaStream_t own_stream = nullptr;
  cudaStream_t ext_stream = nullptr;
  bool has_ext_stream = false;

  int64_t rows = 0, cols = 0;
  DevBuf d_fixed;
  bool has_fixed = false;
  DevBuf d_mask;
  bool has_mask = false;
  int64_t num_mov = 0;
  xr_raycaster rc = nullptr;       // bound ray caster (checked with rc_id before use)
  uint64_t rc_id = 0;
  const float* mov_dev = nullptr;
  const float* mov_host = nullptr; // set_mov_imgs_host_buf: copied to d_mov_stage at each compute
  DevBuf d_mov_stage;
  int64_t proj_offset = 0;
  int32_t smooth_ksize = 5;
  int32_t patch_radius = 5;
  int32_t patch_stride = 1;

  bool allocated = false;
  int64_t capacity = 0;            // moving images the partials buffer holds
  int64_t n_used = 0;              // pixels used by NCC (mask count or all)
  FixedNCC fx{}, fy{};
  DevBuf d_fhat_x, d_fhat_y, d_gx, d_gy, d_pmean_x, d_pscale_x, d_pmean_y, d_pscale_y;
  DevBuf d_partials, d_sims, d_scratch;
  int nblk = 0;
  int ncr = 0, ncc = 0;            // patch centre grid
  uint64_t generation = 1;
  // patch metrics: options, weights and patch subsets
  xr_patch_options popt{};
  std::vector<uint8_t> h_mask;     // host copy of the mask (patch weights)
  std::vector<float> wgt_img;      // user weight image (rows * cols) or empty
  DevBuf d_pw_x, d_pw_y, d_pcnt, d_pidx, d_mvar_sum;
  DevBuf d_pscores;                // [image][patch] scores (save_all_per_patch_scores)
  bool has_pw = false;             // per-patch weights on the device (else 1)
  std::vector<double> w_x, w_y;    // static patch weights per direction
  std::vector<double> w_draw;      // weights the random subsets are drawn with
  double tot_w_x = 0, tot_w_y = 0; // sums of the weights of the patches in use
  int64_t nused = 0;               // patches in use (with multiplicity)
  int mvar_mode = 0;               // moving-variance weights (PatchRun::mvar)
  std::mt19937 rng;
  std::vector<int32_t> last_idx;   // the patches in use when listed (the last draw, or user_idx)
  std::vector<int32_t> user_idx;   // set_patches_to_use (empty = not set)

  // The bound ray caster if it is still alive; forgets it otherwise.
  xr_raycaster live_rc() {
    if (rc && !reg_alive(rc, rc_id)) { rc = nullptr; rc_id = 0; }
    return rc;
  }
  cudaStream_t stream() {
    if (has_ext_stream) return ext_stream;
    if (xr_raycaster r = live_rc()) return r->stream();
    return own_stream;
  }
};

// Device descriptors and work counter of a fused evaluation step (see
// fused_enqueue), owned by each objective and job set.
struct FusedWork {
  DevBuf d_desc, d_counter, d_report;  // d_report: CmaReport per job of a device-optimizer step
  std::vector<unsigned char> h_desc;  // staging: pageable, consumed by the copy call itself
  int blocks = 0;
  long long items = 0;
  int launches = 0;                   // kernel launches of the last step
  int pose_grouped = 0;               // jobs of the last step with pose-grouped DRR items
};

struct xr_objective_s {
  xr_raycaster rc = nullptr;
  uint64_t rc_id = 0;
  int32_t vol_idx = 0;
  std::vector<xr_simmetric> metrics;
  std::vector<uint64_t> metric_ids;
  bool peers_alive() const {
    if (!reg_alive(rc, rc_id)) return false;
    for (size_t i = 0; i < metrics.size(); ++i)
      if (!reg_alive(metrics[i], metric_ids[i])) return false;
    return true;
  }
  int64_t max_pop = 0;
  uint64_t id = 0;
  DevBuf d_poses, d_sims;
  // fused evaluation: mode (1 fused, 0 split DRR and metric launches), its
  // counters (zero between launches) and descriptors
  int32_t fused = 0;
  // spread of the next population of an attached device optimizer (from the last step's report; < 0 unknown)
  double next_sd_rot = -1.0, next_sd_trans = -1.0;
  const void* next_sd_state = nullptr;  // the device state those figures belong to
  DevBuf d_fcnt;
  size_t fcnt_words = 0;
  FusedWork fw;
  // captured launch sequence
  cudaGraphExec_t graph_exec = nullptr;
  int64_t graph_pop = -1;
  uint64_t graph_rc_gen = 0;
  std::vector<uint64_t> graph_sm_gen;
  cudaStream_t graph_stream = nullptr;
  ~xr_objective_s() {
    if (graph_exec) cudaGraphExecDestroy(graph_exec);
  }
};

// ===================================================================== misc
extern "C" XR_API const char* xr_last_error(void) { return g_last_error.c_str(); }
extern "C" XR_API const char* xr_version(void) { return "xreg_gb300 0.1.0 (sm_103a)"; }

#define XR_CHECK_ARG(cond, msg) \
  do {                          \
    if (!(cond)) return fail(XR_ERR_INVALID_ARG, msg); \
  } while (0)

// ============================================================ camera helpers
extern "C" XR_API xr_status xr_camera_setup_naive(double f, int64_t nr, int64_t nc, double rs, double cs,
                                                  int32_t frame, xr_camera_desc* out) {
  XR_CHECK_ARG(out, "xr_camera_setup_naive: out is NULL");
  XR_CHECK_ARG(f > 1.0e-8, "xr_camera_setup_naive: focal length must be > 1e-8");
  XR_CHECK_ARG(nr > 0 && nc > 0, "xr_camera_setup_naive: rows and cols must be positive");
  XR_CHECK_ARG(rs > 1.0e-8 && cs > 1.0e-8, "xr_camera_setup_naive: spacings must be > 1e-8");
  XR_CHECK_ARG(frame >= 0 && frame <= 2, "xr_camera_setup_naive: bad coord_frame_type");
  // xReg's CameraModel holds float members (CoordScalar): the arguments are
  // floats there, and MakeNaiveIntrins divides in float.
  const float ff = (float)f, frs = (float)rs, fcs = (float)cs;
  std::memset(out, 0, sizeof(*out));
  out->coord_frame_type = frame;
  out->focal_len = ff;
  out->num_det_rows = nr;
  out->num_det_cols = nc;
  out->det_row_spacing = frs;
  out->det_col_spacing = fcs;
  float K[9] = {ff / fcs, 0, 0, 0, ff / frs, 0, 0, 0, 1};
  if (frame == XR_CAM_FOCAL_NEG_Z) { K[0] = -K[0]; K[4] = -K[4]; }
  K[2] = (float)((double)(nc - 1) * 0.5);
  K[5] = (float)((double)(nr - 1) * 0.5);
  for (int i = 0; i < 9; ++i) out->intrins[i] = K[i];
  for (int i = 0; i < 16; ++i) out->extrins[i] = (i % 5 == 0) ? 1.0 : 0.0;
  return XR_OK;
}

extern "C" XR_API xr_status xr_camera_downsample(const xr_camera_desc* src, double ds, int32_t force_even,
                                                 xr_camera_desc* dst) {
  XR_CHECK_ARG(src && dst, "xr_camera_downsample: NULL argument");
  XR_CHECK_ARG(ds > 0.0, "xr_camera_downsample: factor must be positive");
  // float arithmetic throughout, as CameraModel holds its members
  const float fds = (float)ds;
  xr_camera_desc d = *src;
  float K[9];
  for (int i = 0; i < 9; ++i) K[i] = (float)src->intrins[i];
  K[0] *= fds; K[4] *= fds; K[2] *= fds; K[5] *= fds;
  // lround(num_det_rows * ds_factor): the count converts to float first
  long nr = std::lround((float)src->num_det_rows * fds);
  long nc = std::lround((float)src->num_det_cols * fds);
  if (force_even) { if (nr % 2) --nr; if (nc % 2) --nc; }
  XR_CHECK_ARG(nr > 0 && nc > 0, "xr_camera_downsample: result has no pixels");
  for (int i = 0; i < 9; ++i) d.intrins[i] = K[i];
  for (int i = 0; i < 16; ++i) d.extrins[i] = (float)src->extrins[i];
  d.num_det_rows = nr;
  d.num_det_cols = nc;
  const float rs = (float)src->det_row_spacing / fds, cs = (float)src->det_col_spacing / fds;
  d.det_row_spacing = rs;
  d.det_col_spacing = cs;
  // FocalLenFromIntrins (xregPerspectiveXform.cpp:186-190)
  d.focal_len = (std::fabs(K[0] * cs) + std::fabs(K[4] * ((rs < 0) ? cs : rs))) / 2.0f;
  *dst = d;
  return XR_OK;
}

// ================================================================ ray caster
extern "C" XR_API xr_status xr_rc_create(int32_t device, xr_raycaster* out) {
  XR_CHECK_ARG(out, "xr_rc_create: out is NULL");
  *out = nullptr;
  int dev = device;
  if (dev < 0) XR_CUDA_TRY(cudaGetDevice(&dev));
  int ndev = 0;
  XR_CUDA_TRY(cudaGetDeviceCount(&ndev));
  XR_CHECK_ARG(dev < ndev, "xr_rc_create: no such device");
  DeviceGuard g(dev);
  auto* rc = new (std::nothrow) xr_raycaster_s();
  if (!rc) return fail(XR_ERR_OUT_OF_MEMORY, "xr_rc_create: host allocation failed");
  rc->device = dev;
  rc->id = reg_add(rc);
  cudaError_t e = cudaStreamCreateWithFlags(&rc->own_stream, cudaStreamNonBlocking);
  if (e != cudaSuccess) { reg_remove(rc); delete rc; return cuda_fail(e, "cudaStreamCreateWithFlags"); }
  e = rc->d_counters.reserve(64);
  if (e != cudaSuccess) {
    cudaStreamDestroy(rc->own_stream);
    reg_remove(rc);
    delete rc;
    return cuda_fail(e, "cudaMalloc");
  }
  cudaMemset(rc->d_counters.p, 0, 64);
  *out = rc;
  return XR_OK;
}

extern "C" XR_API xr_status xr_rc_destroy(xr_raycaster rc) {
  if (!rc) return XR_OK;
  reg_remove(rc);
  DeviceGuard g(rc->device);
  cudaStreamSynchronize(rc->stream());
  cudaStreamDestroy(rc->own_stream);
  delete rc;
  return XR_OK;
}

extern "C" XR_API xr_status xr_rc_set_stream(xr_raycaster rc, void* s) {
  XR_CHECK_ARG(rc, "xr_rc_set_stream: NULL handle");
  rc->ext_stream = static_cast<cudaStream_t>(s);
  rc->has_ext_stream = s != nullptr;
  rc->generation++;
  return XR_OK;
}

extern "C" XR_API xr_status xr_rc_synchronize(xr_raycaster rc) {
  XR_CHECK_ARG(rc, "xr_rc_synchronize: NULL handle");
  DeviceGuard g(rc->device);
  XR_CUDA_TRY(cudaStreamSynchronize(rc->stream()));
  unsigned int err = 0;
  XR_CUDA_TRY(cudaMemcpy(&err, rc->d_counters.as<char>() + 8, sizeof(err), cudaMemcpyDeviceToHost));
  if (err) {
    cudaMemset(rc->d_counters.as<char>() + 8, 0, sizeof(err));
    return fail(XR_ERR_DEVICE_CHECK, "ray caster: " + std::to_string(err) +
                                         " rays exceeded the step-count guard (non-finite or degenerate pose)");
  }
  return XR_OK;
}

// Support box of a volume's non-zero voxels for empty-space skipping: in
// continuous index coordinates every sample outside (min - 1 - m, max + 1 + m)
// on some axis interpolates only zero voxels.  The margin m = 0.5 voxel covers
// the drift of positions advanced by repeated float addition.
static xr_status vol_support(xr_raycaster rc, xr_raycaster_s::Vol& v, const float* vox_f32, cudaStream_t s) {
  int* d_box = reinterpret_cast<int*>(rc->d_counters.as<char>() + 32);
  XR_CUDA_TRY(launch_support_box(vox_f32, (int)v.desc.n[0], (int)v.desc.n[1], (int)v.desc.n[2], d_box, s));
  int box[6];
  XR_CUDA_TRY(cudaMemcpyAsync(box, d_box, sizeof(box), cudaMemcpyDeviceToHost, s));
  XR_CUDA_TRY(cudaStreamSynchronize(s));
  v.nmx = (int32_t)(((v.desc.n[0] - 1) + (1 << kMacroShift) - 1) >> kMacroShift);
  v.nmy = (int32_t)(((v.desc.n[1] - 1) + (1 << kMacroShift) - 1) >> kMacroShift);
  v.nmz = (int32_t)(((v.desc.n[2] - 1) + (1 << kMacroShift) - 1) >> kMacroShift);
  const size_t words = ((size_t)v.nmx * v.nmy * v.nmz + 31) / 32;
  XR_CUDA_TRY(v.occ.reserve(words * 4));
  XR_CUDA_TRY(launch_build_occupancy(vox_f32, (int)v.desc.n[0], (int)v.desc.n[1], (int)v.desc.n[2],
                                     v.occ.as<uint32_t>(), v.nmx, v.nmy, v.nmz, s));
  v.has_support = true;
  if (box[3] < box[0]) {  // no non-zero voxel
    for (int k = 0; k < 3; ++k) { v.sup_lo[k] = 1.0f; v.sup_hi[k] = 0.0f; }
  } else {
    for (int k = 0; k < 3; ++k) {
      v.sup_lo[k] = (float)box[k] - 1.5f;
      v.sup_hi[k] = (float)box[3 + k] + 1.5f;
    }
  }
  return XR_OK;
}

static xr_status rc_set_volumes_impl(xr_raycaster rc, int32_t n, const xr_volume_desc* descs,
                                     const float* const* voxels, int32_t vt, float scale, bool on_device) {
  XR_CHECK_ARG(rc && descs && voxels && n > 0, "set_volumes: NULL argument or no volumes");
  XR_CHECK_ARG(vt == XR_VOXEL_F32 || vt == XR_VOXEL_F16 || vt == XR_VOXEL_BF16, "set_volumes: bad voxel type");
  DeviceGuard g(rc->device);
  cudaStream_t s = rc->stream();
  std::vector<std::unique_ptr<xr_raycaster_s::Vol>> vols;
  for (int32_t i = 0; i < n; ++i) {
    const xr_volume_desc& d = descs[i];
    XR_CHECK_ARG(voxels[i], "set_volumes: NULL voxel pointer");
    XR_CHECK_ARG(d.n[0] >= 2 && d.n[1] >= 2 && d.n[2] >= 2, "set_volumes: every dimension must be >= 2");
    const int64_t nv = d.n[0] * d.n[1] * d.n[2];
    XR_CHECK_ARG(nv < (int64_t(1) << 31), "set_volumes: volumes above 2^31 voxels are not supported");
    XR_CHECK_ARG(d.spacing[0] > 0 && d.spacing[1] > 0 && d.spacing[2] > 0, "set_volumes: spacing must be > 0");
    XR_CHECK_ARG(finite_all(d.spacing, 3) && finite_all(d.origin, 3) && finite_all(d.direction, 9),
                 "set_volumes: non-finite geometry");
    auto v = std::make_unique<xr_raycaster_s::Vol>();
    v->desc = d;
    v->type = vt;
    cell_strides(d.n[0], d.n[1], d.n[2], v->cs);
    const size_t esz = vt == XR_VOXEL_F32 ? 4 : 2;
    XR_CUDA_TRY(v->voxels.reserve((size_t)nv * esz));
    if (vt == XR_VOXEL_F32) {
      XR_CUDA_TRY(cudaMemcpyAsync(v->voxels.p, voxels[i], (size_t)nv * 4,
                                  on_device ? cudaMemcpyDeviceToDevice : cudaMemcpyHostToDevice, s));
      v->inv_scale = 1.0f;
      if (rc->build_cells) {
        XR_CUDA_TRY(v->cells.reserve(cell_layout_bytes(d.n[0], d.n[1], d.n[2], vt)));
        XR_CUDA_TRY(launch_build_cells(v->voxels.as<float>(), (int)d.n[0], (int)d.n[1], (int)d.n[2], vt, 1.0f,
                                       v->cells.p, s));
      }
      xr_status st = vol_support(rc, *v, v->voxels.as<float>(), s);
      if (st != XR_OK) return st;
    } else {
      DevBuf tmp;
      const float* src = voxels[i];
      if (!on_device) {
        XR_CUDA_TRY(tmp.reserve((size_t)nv * 4));
        XR_CUDA_TRY(cudaMemcpyAsync(tmp.p, voxels[i], (size_t)nv * 4, cudaMemcpyHostToDevice, s));
        src = tmp.as<float>();
      }
      float sc = scale > 0.0f ? scale : 1.0f;
      if (vt == XR_VOXEL_F16) {
        // The half2 blend multiplies stored values by x weights scaled by 2^15
        // (so that fractions down to 2^-24 stay normal halves) and the y blend
        // by 2^15 more; stored values below 1 keep the blend below 2^15.  So
        // FP16 always stores the maximum in [0.5, 1) (a given scale is not used).
        XR_CUDA_TRY(cudaMemsetAsync(rc->d_counters.as<char>() + 16, 0, 4, s));
        max_abs_kernel<<<1024, 256, 0, s>>>(src, nv, reinterpret_cast<unsigned int*>(rc->d_counters.as<char>() + 16));
        XR_CUDA_TRY(cudaGetLastError());
        unsigned int bits = 0;
        XR_CUDA_TRY(cudaMemcpyAsync(&bits, rc->d_counters.as<char>() + 16, 4, cudaMemcpyDeviceToHost, s));
        XR_CUDA_TRY(cudaStreamSynchronize(s));
        float mx;
        std::memcpy(&mx, &bits, 4);
        XR_CHECK_ARG(std::isfinite(mx), "set_volumes: non-finite voxel");
        // the scale (at most 2^90) and its inverse times 2^-30 stay normal floats
        XR_CHECK_ARG(mx == 0.0f || mx >= 0x1p-90f, "set_volumes: FP16 volume maximum below 2^-90");
        sc = mx > 0.0f ? (float)std::ldexp(1.0, (int)std::floor(std::log2(1.0 / (double)mx))) : 1.0f;
        v->inv_scale = (float)(1.0 / ((double)sc * 32768.0 * 32768.0));
      } else {
        v->inv_scale = 1.0f / sc;
      }
      convert_voxels_kernel<<<2048, 256, 0, s>>>(src, nv, sc, vt, v->voxels.p);
      XR_CUDA_TRY(cudaGetLastError());
      if (rc->build_cells) {
        XR_CUDA_TRY(v->cells.reserve(cell_layout_bytes(d.n[0], d.n[1], d.n[2], vt)));
        XR_CUDA_TRY(launch_build_cells(src, (int)d.n[0], (int)d.n[1], (int)d.n[2], vt, sc, v->cells.p, s));
      }
      xr_status st = vol_support(rc, *v, src, s);
      if (st != XR_OK) return st;
      XR_CUDA_TRY(cudaStreamSynchronize(s));  // tmp is released at scope exit
    }
    vols.push_back(std::move(v));
  }
  XR_CUDA_TRY(cudaStreamSynchronize(s));
  rc->vols = std::move(vols);
  rc->generation++;
  return XR_OK;
}

extern "C" XR_API xr_status xr_rc_set_volumes(xr_raycaster rc, int32_t n, const xr_volume_desc* descs,
                                              const float* const* host_voxels, int32_t vt, float scale) {
  return rc_set_volumes_impl(rc, n, descs, host_voxels, vt, scale, false);
}

extern "C" XR_API xr_status xr_rc_set_volumes_device(xr_raycaster rc, int32_t n, const xr_volume_desc* descs,
                                                     const float* const* dev_voxels, int32_t vt, float scale) {
  return rc_set_volumes_impl(rc, n, descs, dev_voxels, vt, scale, true);
}

extern "C" XR_API xr_status xr_rc_set_camera_models(xr_raycaster rc, int32_t n, const xr_camera_desc* cams) {
  XR_CHECK_ARG(rc && cams && n > 0, "set_camera_models: NULL argument or no cameras");
  for (int32_t i = 0; i < n; ++i) {
    XR_CHECK_ARG(cams[i].num_det_rows > 0 && cams[i].num_det_cols > 0, "set_camera_models: empty detector");
    XR_CHECK_ARG(cams[i].coord_frame_type >= 0 && cams[i].coord_frame_type <= 2, "set_camera_models: bad frame");
    XR_CHECK_ARG(finite_all(cams[i].intrins, 9) && finite_all(cams[i].extrins, 16), "set_camera_models: non-finite");
    XR_CHECK_ARG(cams[i].num_det_rows < (1 << 30) && cams[i].num_det_cols < (1 << 30), "set_camera_models: too big");
  }
  rc->cams.assign(cams, cams + n);
  rc->cams_dirty = true;
  rc->generation++;
  return XR_OK;
}

extern "C" XR_API xr_status xr_rc_set_num_projs(xr_raycaster rc, int64_t n) {
  XR_CHECK_ARG(rc && n > 0, "set_num_projs: NULL handle or non-positive count");
  XR_CHECK_ARG(!rc->allocated || n <= rc->capacity,
               "set_num_projs: more projections than allocate_resources reserved; call allocate_resources again");
  if (n != rc->num_projs) {
    rc->num_projs = n;
    rc->cam_idx.resize((size_t)n, 0);
    rc->cam_idx_dirty = true;
    rc->generation++;
  }
  return XR_OK;
}

extern "C" XR_API xr_status xr_rc_num_projs(xr_raycaster rc, int64_t* out) {
  XR_CHECK_ARG(rc && out, "num_projs: NULL argument");
  *out = rc->num_projs;
  return XR_OK;
}

extern "C" XR_API xr_status xr_rc_set_ray_step_size(xr_raycaster rc, float step) {
  XR_CHECK_ARG(rc && step > 0.0f && std::isfinite(step), "set_ray_step_size: step must be positive and finite");
  rc->step = step;
  rc->generation++;
  return XR_OK;
}

extern "C" XR_API xr_status xr_rc_set_interp_method(xr_raycaster rc, int32_t m) {
  XR_CHECK_ARG(rc && m >= 0 && m <= 3, "set_interp_method: bad method");
  rc->interp = m;
  return XR_OK;
}

extern "C" XR_API xr_status xr_rc_set_proj_store_method(xr_raycaster rc, int32_t m) {
  XR_CHECK_ARG(rc && (m == XR_PROJ_STORE_REPLACE || m == XR_PROJ_STORE_ACCUM), "set_proj_store_method: bad method");
  rc->store = m;
  rc->generation++;
  return XR_OK;
}

extern "C" XR_API xr_status xr_rc_set_default_bg_pixel_val(xr_raycaster rc, float bg) {
  XR_CHECK_ARG(rc, "set_default_bg_pixel_val: NULL handle");
  rc->default_bg = bg;
  rc->generation++;
  return XR_OK;
}

extern "C" XR_API xr_status xr_rc_set_kernel_id(xr_raycaster rc, int32_t k) {
  XR_CHECK_ARG(rc && (k == XR_LINE_INT_SUM || k == XR_LINE_INT_MAX), "set_kernel_id: bad kernel id");
  rc->kernel_id = k;
  rc->generation++;
  return XR_OK;
}

extern "C" XR_API xr_status xr_rc_set_bg_projs(xr_raycaster rc, const float* const* imgs, int32_t use) {
  XR_CHECK_ARG(rc && imgs, "set_bg_projs: NULL argument");
  XR_CHECK_ARG(!rc->cams.empty(), "set_bg_projs: set the camera models first");
  DeviceGuard g(rc->device);
  const size_t npix = (size_t)(rc->rows() * rc->cols());
  XR_CUDA_TRY(rc->d_bg.reserve(npix * 4 * rc->cams.size()));
  for (size_t c = 0; c < rc->cams.size(); ++c) {
    XR_CHECK_ARG(imgs[c], "set_bg_projs: NULL image");
    XR_CUDA_TRY(cudaMemcpyAsync(rc->d_bg.as<float>() + c * npix, imgs[c], npix * 4, cudaMemcpyHostToDevice,
                                rc->stream()));
  }
  XR_CUDA_TRY(cudaStreamSynchronize(rc->stream()));
  rc->has_bg = true;
  rc->use_bg = use != 0;
  rc->generation++;
  return XR_OK;
}

extern "C" XR_API xr_status xr_rc_set_use_bg_projs(xr_raycaster rc, int32_t use) {
  XR_CHECK_ARG(rc, "set_use_bg_projs: NULL handle");
  XR_CHECK_ARG(!use || rc->has_bg, "set_use_bg_projs: no background projections were set");
  rc->use_bg = use != 0;
  rc->generation++;
  return XR_OK;
}

extern "C" XR_API xr_status xr_rc_set_xforms_cam_to_itk_phys(xr_raycaster rc, int64_t n, const double* xf) {
  XR_CHECK_ARG(rc && xf && n > 0, "set_xforms_cam_to_itk_phys: NULL argument");
  XR_CHECK_ARG(finite_all(xf, 16 * n), "set_xforms_cam_to_itk_phys: non-finite transform");
  xr_status st = xr_rc_set_num_projs(rc, n);
  if (st != XR_OK) return st;
  rc->xforms.assign(xf, xf + 16 * n);
  rc->pose_count = n;
  rc->xforms_dirty = true;
  rc->xforms_on_device = false;
  return XR_OK;
}

extern "C" XR_API xr_status xr_rc_distribute_xforms_among_cam_models(xr_raycaster rc, int64_t n, const double* xf) {
  XR_CHECK_ARG(rc && xf && n > 0, "distribute_xforms_among_cam_models: NULL argument");
  XR_CHECK_ARG(!rc->cams.empty(), "distribute_xforms_among_cam_models: no camera models");
  XR_CHECK_ARG(n * (int64_t)rc->cams.size() == rc->num_projs,
               "distribute_xforms_among_cam_models: num_xforms * num_cams must equal num_projs");
  XR_CHECK_ARG(finite_all(xf, 16 * n), "distribute_xforms_among_cam_models: non-finite transform");
  rc->xforms.assign(xf, xf + 16 * n);
  rc->pose_count = n;
  rc->xforms_dirty = true;
  rc->xforms_on_device = false;
  for (int64_t p = 0; p < rc->num_projs; ++p) {
    const int32_t c = (int32_t)(p / n);
    if (rc->cam_idx[(size_t)p] != c) { rc->cam_idx[(size_t)p] = c; rc->cam_idx_dirty = true; }
  }
  return XR_OK;
}

namespace {
// FrameTransform * FrameTransform in float, Eigen's order (xf::compose); the
// result is stored back as double.
void frame_mul_f32(const double* a, const double* b, double* out) {
  xf::Affine fa, fb, r;
  for (int i = 0; i < 3; ++i) {
    for (int j = 0; j < 3; ++j) {
      fa.L[i * 3 + j] = (float)a[i * 4 + j];
      fb.L[i * 3 + j] = (float)b[i * 4 + j];
    }
    fa.t[i] = (float)a[i * 4 + 3];
    fb.t[i] = (float)b[i * 4 + 3];
  }
  xf::compose(fa, fb, r);
  for (int i = 0; i < 3; ++i) {
    for (int j = 0; j < 3; ++j) out[i * 4 + j] = r.L[i * 3 + j];
    out[i * 4 + 3] = r.t[i];
    out[12 + i] = 0.0;
  }
  out[15] = 1.0;
}
}  // namespace

// The poses on the host, current (copied back when they were given on the device).
static xr_status rc_host_xforms(xr_raycaster rc, const char* fn) {
  if (rc->pose_count <= 0) return fail(XR_ERR_INVALID_ARG, std::string(fn) + ": no projection transforms were set");
  if (rc->xforms_on_device) {
    DeviceGuard g(rc->device);
    rc->xforms.resize((size_t)rc->pose_count * 16);
    XR_CUDA_TRY(cudaMemcpyAsync(rc->xforms.data(), rc->d_xforms.p, (size_t)rc->pose_count * 16 * 8,
                                cudaMemcpyDeviceToHost, rc->stream()));
    XR_CUDA_TRY(cudaStreamSynchronize(rc->stream()));
    rc->xforms_on_device = false;
  }
  return XR_OK;
}

// RayCaster::pre_multiply_all_xforms / post_multiply_all_xforms
// (xregRayCastInterface.cpp:235-261): FrameTransform products, in float as xReg
// computes them.
static xr_status rc_multiply_all(xr_raycaster rc, const double* m, bool pre, const char* fn) {
  XR_CHECK_ARG(rc && m, std::string(fn) + ": NULL argument");
  XR_CHECK_ARG(finite_all(m, 16), std::string(fn) + ": non-finite transform");
  xr_status st = rc_host_xforms(rc, fn);
  if (st != XR_OK) return st;
  for (int64_t k = 0; k < rc->pose_count; ++k) {
    double* x = rc->xforms.data() + 16 * k;
    if (pre) frame_mul_f32(m, x, x);
    else frame_mul_f32(x, m, x);
  }
  rc->xforms_dirty = true;
  return XR_OK;
}

extern "C" XR_API xr_status xr_rc_pre_multiply_all_xforms(xr_raycaster rc, const double* pre_xform) {
  return rc_multiply_all(rc, pre_xform, true, "pre_multiply_all_xforms");
}

extern "C" XR_API xr_status xr_rc_post_multiply_all_xforms(xr_raycaster rc, const double* post_xform) {
  return rc_multiply_all(rc, post_xform, false, "post_multiply_all_xforms");
}

extern "C" XR_API xr_status xr_rc_xforms_cam_to_itk_phys(xr_raycaster rc, int64_t cap, double* out, int64_t* count) {
  XR_CHECK_ARG(rc && count && (out || cap == 0), "xforms_cam_to_itk_phys: NULL argument");
  *count = rc->pose_count > 0 ? rc->num_projs : 0;
  if (cap <= 0 || *count == 0) return XR_OK;
  xr_status st = rc_host_xforms(rc, "xforms_cam_to_itk_phys");
  if (st != XR_OK) return st;
  for (int64_t p = 0; p < std::min(cap, *count); ++p)
    std::memcpy(out + 16 * p, rc->xforms.data() + 16 * (p % rc->pose_count), 16 * sizeof(double));
  return XR_OK;
}

extern "C" XR_API xr_status xr_rc_camera_model_proj_associations(xr_raycaster rc, int64_t cap, int32_t* out,
                                                                int64_t* count) {
  XR_CHECK_ARG(rc && count && (out || cap == 0), "camera_model_proj_associations: NULL argument");
  *count = (int64_t)rc->cam_idx.size();
  for (int64_t p = 0; p < std::min(cap, *count); ++p) out[p] = rc->cam_idx[(size_t)p];
  return XR_OK;
}

extern "C" XR_API xr_status xr_rc_set_proj_cam_model(xr_raycaster rc, int64_t proj_idx, int32_t cam_idx) {
  XR_CHECK_ARG(rc, "set_proj_cam_model: NULL handle");
  XR_CHECK_ARG(proj_idx >= 0 && proj_idx < (int64_t)rc->cam_idx.size(), "set_proj_cam_model: bad projection");
  XR_CHECK_ARG(cam_idx >= 0 && cam_idx < (int32_t)rc->cams.size(), "set_proj_cam_model: bad camera");
  rc->cam_idx[(size_t)proj_idx] = cam_idx;
  rc->cam_idx_dirty = true;
  return XR_OK;
}

extern "C" XR_API xr_status xr_rc_num_vols(xr_raycaster rc, int32_t* out) {
  XR_CHECK_ARG(rc && out, "num_vols: NULL argument");
  *out = (int32_t)rc->vols.size();
  return XR_OK;
}

extern "C" XR_API xr_status xr_rc_num_camera_models(xr_raycaster rc, int32_t* out) {
  XR_CHECK_ARG(rc && out, "num_camera_models: NULL argument");
  *out = (int32_t)rc->cams.size();
  return XR_OK;
}

extern "C" XR_API xr_status xr_rc_xform_img_center_to_itk_phys(xr_raycaster rc, int32_t vol_idx, double* out) {
  XR_CHECK_ARG(rc && out, "xform_img_center_to_itk_phys: NULL argument");
  XR_CHECK_ARG(vol_idx >= 0 && vol_idx < (int32_t)rc->vols.size(), "xform_img_center_to_itk_phys: bad volume index");
  const xr_volume_desc& d = rc->vols[(size_t)vol_idx]->desc;
  double c[3];
  for (int i = 0; i < 3; ++i) {
    // continuous index size / 2 (not (size - 1) / 2) to ITK physical coordinates
    double v = d.origin[i];
    for (int k = 0; k < 3; ++k) v += d.direction[i * 3 + k] * d.spacing[k] * ((double)d.n[k] / 2.0);
    c[i] = v;
  }
  for (int i = 0; i < 16; ++i) out[i] = (i % 5 == 0) ? 1.0 : 0.0;
  out[3] = c[0];
  out[7] = c[1];
  out[11] = c[2];
  return XR_OK;
}

extern "C" XR_API xr_status xr_rc_xform_cam_wrt_carm_center_of_rot(xr_raycaster rc, int32_t cam_idx, double* out) {
  XR_CHECK_ARG(rc && out, "xform_cam_wrt_carm_center_of_rot: NULL argument");
  XR_CHECK_ARG(cam_idx >= 0 && cam_idx < (int32_t)rc->cams.size(), "xform_cam_wrt_carm_center_of_rot: bad camera");
  for (int i = 0; i < 16; ++i) out[i] = (i % 5 == 0) ? 1.0 : 0.0;
  out[11] = -rc->cams[(size_t)cam_idx].focal_len / 2.0;
  return XR_OK;
}

extern "C" XR_API xr_status xr_rc_set_camera_model_proj_associations(xr_raycaster rc, int64_t n, const int32_t* ci) {
  XR_CHECK_ARG(rc && ci, "set_camera_model_proj_associations: NULL argument");
  XR_CHECK_ARG(n == rc->num_projs, "set_camera_model_proj_associations: size must equal num_projs");
  for (int64_t i = 0; i < n; ++i)
    XR_CHECK_ARG(ci[i] >= 0 && ci[i] < (int32_t)rc->cams.size(), "set_camera_model_proj_associations: bad camera");
  rc->cam_idx.assign(ci, ci + n);
  rc->cam_idx_dirty = true;
  return XR_OK;
}

extern "C" XR_API xr_status xr_rc_allocate_resources(xr_raycaster rc) {
  XR_CHECK_ARG(rc, "allocate_resources: NULL handle");
  XR_CHECK_ARG(rc->num_projs > 0, "allocate_resources: num_projs is 0");
  XR_CHECK_ARG(!rc->cams.empty(), "allocate_resources: no camera models");
  for (size_t c = 1; c < rc->cams.size(); ++c) {
    if (rc->cams[c].num_det_rows != rc->rows()) return fail(XR_ERR_INVALID_ARG, "Inconsistent number rows in camera model images!");
    if (rc->cams[c].num_det_cols != rc->cols()) return fail(XR_ERR_INVALID_ARG, "Inconsistent number columns in camera model images!");
  }
  DeviceGuard g(rc->device);
  const size_t n = (size_t)rc->num_projs;
  XR_CUDA_TRY(rc->d_proj.reserve(n * (size_t)(rc->rows() * rc->cols()) * 4));
  XR_CUDA_TRY(rc->d_geo.reserve(n * sizeof(ProjGeom)));
  XR_CUDA_TRY(rc->d_cam_idx.reserve(n * 4));
  XR_CUDA_TRY(rc->d_xforms.reserve(n * 16 * 8));
  XR_CUDA_TRY(rc->d_cams.reserve(rc->cams.size() * sizeof(xr_camera_desc)));
  rc->capacity = rc->num_projs;
  rc->cams_dirty = rc->cam_idx_dirty = rc->xforms_dirty = true;
  if (rc->xforms_on_device) rc->xforms_dirty = false;  // device-side poses already live in d_xforms? re-set required
  rc->allocated = true;
  rc->generation++;
  return XR_OK;
}

extern "C" XR_API xr_status xr_rc_max_num_projs_possible(xr_raycaster rc, int64_t* out) {
  XR_CHECK_ARG(rc && out, "max_num_projs_possible: NULL argument");
  XR_CHECK_ARG(!rc->cams.empty(), "max_num_projs_possible: no camera models");
  DeviceGuard g(rc->device);
  size_t fr = 0, tot = 0;
  XR_CUDA_TRY(cudaMemGetInfo(&fr, &tot));
  const double per = (double)(rc->rows() * rc->cols()) * 4.0 + sizeof(ProjGeom) + 16 * 8 + 4;
  *out = (int64_t)(0.9 * (double)fr / per);
  return XR_OK;
}

extern "C" XR_API xr_status xr_rc_set_count_samples(xr_raycaster rc, int32_t enable) {
  XR_CHECK_ARG(rc, "set_count_samples: NULL handle");
  rc->count_samples = enable != 0;
  rc->generation++;
  return XR_OK;
}

// ------------------------------------------------------------- autotuner
// Candidates differ only in speed (layout, block shape, unroll give bit-identical
// results), so the fastest measured one is cached per shape for the process.
namespace {
struct TuneKey {
  int64_t nx, ny, nz, rows, cols, projs_pow2;
  int32_t vt, kernel, has_cells;
  bool operator==(const TuneKey& o) const {
    return nx == o.nx && ny == o.ny && nz == o.nz && rows == o.rows && cols == o.cols &&
           projs_pow2 == o.projs_pow2 && vt == o.vt && kernel == o.kernel && has_cells == o.has_cells;
  }
};
struct TuneKeyHash {
  size_t operator()(const TuneKey& k) const {
    size_t h = 1469598103934665603ull;
    const int64_t v[9] = {k.nx, k.ny, k.nz, k.rows, k.cols, k.projs_pow2, k.vt, k.kernel, k.has_cells};
    for (int64_t x : v) h = (h ^ (size_t)x) * 1099511628211ull;
    return h;
  }
};
struct TuneCfg {
  int32_t layout, bw, unroll, tall;
  float ms;
};
std::mutex g_tune_mu;
std::unordered_map<TuneKey, TuneCfg, TuneKeyHash> g_tune;

int64_t pow2_bucket(int64_t n) {
  int64_t b = 1;
  while (b < n) b <<= 1;
  return b;
}

// Times one launch configuration on the first projections of p: as many as
// give about eight waves of blocks (all of them when there are fewer).
xr_status time_config(DrrParams p, cudaStream_t s, float* ms_out) {
  int dev = 0, sms = 0;
  XR_CUDA_TRY(cudaGetDevice(&dev));
  XR_CUDA_TRY(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
  const int64_t px = (int64_t)p.rows * p.cols;  // rays per projection; 256 per block, up to 6 blocks per SM
  const int64_t waves8 = (8LL * sms * 6 * 256 + px - 1) / std::max<int64_t>(px, 1);
  p.num_projs = std::min<int64_t>(p.num_projs, std::max<int64_t>(waves8, 4));
  cudaEvent_t a, b;
  XR_CUDA_TRY(cudaEventCreate(&a));
  XR_CUDA_TRY(cudaEventCreate(&b));
  cudaError_t e = launch_drr(p, s);  // warm-up
  if (e == cudaSuccess) e = cudaEventRecord(a, s);
  for (int r = 0; r < 2 && e == cudaSuccess; ++r) e = launch_drr(p, s);
  if (e == cudaSuccess) e = cudaEventRecord(b, s);
  if (e == cudaSuccess) e = cudaEventSynchronize(b);
  float ms = 0.0f;
  if (e == cudaSuccess) e = cudaEventElapsedTime(&ms, a, b);
  cudaEventDestroy(a);
  cudaEventDestroy(b);
  if (e != cudaSuccess) return cuda_fail(e, "autotune launch");
  *ms_out = ms * 0.5f;
  return XR_OK;
}
}  // namespace

static TuneKey tune_key(xr_raycaster rc, const xr_raycaster_s::Vol& vol, const DrrParams& p) {
  return TuneKey{vol.desc.n[0], vol.desc.n[1], vol.desc.n[2], rc->rows(), rc->cols(), pow2_bucket(p.num_projs),
                 vol.type, p.kernel_id, (vol.cells.p != nullptr ? 1 : 0) | (p.vol.occ ? 2 : 0)};
}

// Whether rc_choose_config decides without timing launches (a configuration
// fixed by the caller, or one cached for this shape).
static bool rc_config_cached(xr_raycaster rc, const xr_raycaster_s::Vol& vol, const DrrParams& p) {
  if (rc->cfg_layout != XR_LAYOUT_AUTO) return true;
  std::lock_guard<std::mutex> lk(g_tune_mu);
  return g_tune.find(tune_key(rc, vol, p)) != g_tune.end();
}

// Picks the launch configuration for p (layout, block_warps_x, unroll, warp shape).
static xr_status rc_choose_config(xr_raycaster rc, const xr_raycaster_s::Vol& vol, DrrParams& p, cudaStream_t s) {
  const bool has_cells = vol.cells.p != nullptr;
  if (rc->cfg_layout != XR_LAYOUT_AUTO) {
    if (rc->cfg_layout != XR_LAYOUT_LINEAR && !has_cells)
      return fail(XR_ERR_INVALID_ARG, "compute: CELL8 layout requested but the volume has no cell copy");
    if (rc->cfg_layout == 2 && vol.type != XR_VOXEL_F32)
      return fail(XR_ERR_INVALID_ARG, "compute: the 256-bit CELL8 read needs a float32 volume");
    if (rc->cfg_layout == 3 && (vol.type != XR_VOXEL_F32 || p.kernel_id != XR_LINE_INT_SUM))
      return fail(XR_ERR_INVALID_ARG, "compute: the brick-staged layout needs a float32 volume and the sum kernel");
    p.vol.layout = rc->cfg_layout;
    p.block_warps_x = rc->cfg_bw;
    p.unroll = rc->cfg_unroll;
    p.warp_tall = rc->cfg_warp_rows == 8 ? 1 : 0;
    return XR_OK;
  }
  const TuneKey key = tune_key(rc, vol, p);
  {
    std::lock_guard<std::mutex> lk(g_tune_mu);
    auto it = g_tune.find(key);
    if (it != g_tune.end()) {
      p.vol.layout = it->second.layout;
      p.block_warps_x = it->second.bw;
      p.unroll = it->second.unroll;
      p.warp_tall = it->second.tall;
      return XR_OK;
    }
  }
  // default when tuning is not possible right now
  p.vol.layout = has_cells ? XR_LAYOUT_CELL8 : XR_LAYOUT_LINEAR;
  p.block_warps_x = 2;
  p.unroll = 1;
  p.warp_tall = 0;
  cudaStreamCaptureStatus cap = cudaStreamCaptureStatusNone;
  XR_CUDA_TRY(cudaStreamIsCapturing(s, &cap));
  // Tuning re-runs the kernel; it needs a stream that is not being captured and an
  // output that the final launch overwrites (replace mode, no background images).
  if (cap != cudaStreamCaptureStatusNone || p.store != XR_PROJ_STORE_REPLACE || p.bg_projs) return XR_OK;
  DrrParams t = p;
  t.sample_counter = nullptr;
  TuneCfg best{p.vol.layout, p.block_warps_x, p.unroll, 0, 1e30f};
  // layout 2 = CELL8 read with one 256-bit load per sample (float32 only)
  const int32_t layouts[3] = {XR_LAYOUT_LINEAR, XR_LAYOUT_CELL8, 2};
  const int32_t bws[3] = {1, 2, 4};
  // loops 3 and 4 = 2 and 4 samples per iteration after the macro-cell trim (sum
  // kernel); 5 = loop 3 whose pairs share one load when both samples fall in one
  // cell (256-bit float32 CELL8 read), 6 = loop 4 on packed FP32 pairs (256-bit
  // float32 or 128-bit half CELL8 reads)
  const int32_t unrolls[6] = {1, 2, 3, 4, 5, 6};
  for (int32_t lay : layouts) {
    if (lay != XR_LAYOUT_LINEAR && !has_cells) continue;
    if (lay == 2 && vol.type != XR_VOXEL_F32) continue;
    for (int32_t bw : bws)
      for (int32_t un : unrolls) {
        if (un >= 3 && !(p.vol.occ && p.kernel_id == XR_LINE_INT_SUM)) continue;
        if (un == 5 && lay != 2) continue;
        if (un == 6 && !(lay == 2 || (lay == XR_LAYOUT_CELL8 && vol.type != XR_VOXEL_F32))) continue;
        t.vol.layout = lay;
        t.block_warps_x = bw;
        t.unroll = un;
        t.warp_tall = 0;
        float ms = 0.0f;
        xr_status st = time_config(t, s, &ms);
        if (st != XR_OK) return st;
        if (ms < best.ms) best = TuneCfg{lay, bw, un, 0, ms};
      }
  }
  // 4x8-pixel warps for the fastest layout and loop (rays of a warp span more
  // detector rows, which changes how their cells share L1 lines)
  {
    const TuneCfg wide = best;
    for (int32_t bw : bws) {
      t.vol.layout = wide.layout;
      t.block_warps_x = bw;
      t.unroll = wide.unroll;
      t.warp_tall = 1;
      float ms = 0.0f;
      xr_status st = time_config(t, s, &ms);
      if (st != XR_OK) return st;
      if (ms < best.ms) best = TuneCfg{wide.layout, bw, wide.unroll, 1, ms};
    }
  }
  {
    std::lock_guard<std::mutex> lk(g_tune_mu);
    g_tune[key] = best;
  }
  p.vol.layout = best.layout;
  p.block_warps_x = best.bw;
  p.unroll = best.unroll;
  p.warp_tall = best.tall;
  return XR_OK;
}

static xr_status rc_distribute_device_on(xr_raycaster rc, int64_t n, const double* d_xf, cudaStream_t s);

// The device buffer a caster's images go to: its own, or the one of the caster
// given to use_other_proj_buf while that one is alive; *cap = images it holds.
static float* rc_out(xr_raycaster rc, int64_t* cap) {
  if (rc->other && !reg_alive(rc->other, rc->other_id)) { rc->other = nullptr; rc->other_id = 0; }
  if (rc->other) {
    if (cap) *cap = rc->other->allocated ? rc->other->capacity : 0;
    return rc->other->d_proj.as<float>();
  }
  if (cap) *cap = rc->capacity;
  return rc->d_proj.as<float>();
}

// Fills the DRR launch parameters of a compute on stream s (uploading dirty host
// state); with `geometry` false the per-projection set-up is left to the caller
// (one launch for many ray casters, see rc_geom_job).
static xr_status rc_prepare(xr_raycaster rc, int32_t vol_idx, cudaStream_t s, DrrParams& p, bool geometry = true) {
  XR_CHECK_ARG(rc, "compute: NULL handle");
  if (!rc->allocated) return fail(XR_ERR_NOT_ALLOCATED, "compute: allocate_resources has not been called");
  if (rc->interp != XR_INTERP_LINEAR)
    return fail(XR_ERR_UNSUPPORTED, "compute: only linear interpolation is implemented (as RayCasterOCL)");
  XR_CHECK_ARG(vol_idx >= 0 && vol_idx < (int32_t)rc->vols.size(), "compute: bad volume index");
  XR_CHECK_ARG(rc->pose_count > 0, "compute: no projection transforms were set");
  XR_CHECK_ARG(!rc->use_bg || rc->has_bg, "compute: background projections requested but not set");
  const int64_t n = rc->num_projs;
  if (rc->cams_dirty) {
    XR_CUDA_TRY(cudaMemcpyAsync(rc->d_cams.p, rc->cams.data(), rc->cams.size() * sizeof(xr_camera_desc),
                                cudaMemcpyHostToDevice, s));
    rc->cams_dirty = false;
  }
  if (rc->cam_idx_dirty) {
    XR_CUDA_TRY(cudaMemcpyAsync(rc->d_cam_idx.p, rc->cam_idx.data(), (size_t)n * 4, cudaMemcpyHostToDevice, s));
    rc->cam_idx_dirty = false;
  }
  if (rc->xforms_dirty) {
    XR_CHECK_ARG(rc->pose_count <= rc->capacity, "compute: more transforms than allocated projections");
    XR_CUDA_TRY(cudaMemcpyAsync(rc->d_xforms.p, rc->xforms.data(), (size_t)rc->pose_count * 16 * 8,
                                cudaMemcpyHostToDevice, s));
    rc->xforms_dirty = false;
  }
  const auto& vol = *rc->vols[(size_t)vol_idx];
  if (geometry)
    XR_CUDA_TRY(launch_proj_geom(vol.desc, rc->d_cams.as<xr_camera_desc>(), rc->d_xforms.as<double>(),
                                 rc->d_cam_idx.as<int32_t>(), n, rc->pose_count, rc->d_geo.as<ProjGeom>(), s));
  p = DrrParams{};
  p.vol.voxels = vol.voxels.p;
  p.vol.cells = vol.cells.p;
  p.vol.nx = (int32_t)vol.desc.n[0];
  p.vol.ny = (int32_t)vol.desc.n[1];
  p.vol.nz = (int32_t)vol.desc.n[2];
  p.vol.voxel_type = vol.type;
  p.vol.inv_scale = vol.inv_scale;
  p.vol.cs[0] = vol.cs[0];
  p.vol.cs[1] = vol.cs[1];
  p.vol.has_support = (rc->skip_empty && vol.has_support) ? 1 : 0;
  p.vol.occ = rc->skip_empty ? vol.occ.as<uint32_t>() : nullptr;
  p.vol.nmx = vol.nmx;
  p.vol.nmy = vol.nmy;
  p.vol.nmz = vol.nmz;
  for (int k = 0; k < 3; ++k) {
    p.vol.sup_lo[k] = vol.sup_lo[k];
    p.vol.sup_hi[k] = vol.sup_hi[k];
  }
  p.geo = rc->d_geo.as<ProjGeom>();
  p.cam_idx = rc->d_cam_idx.as<int32_t>();
  p.bg_projs = rc->use_bg ? rc->d_bg.as<float>() : nullptr;
  {
    int64_t cap = 0;
    p.out = rc_out(rc, &cap);
    if (rc->other) {
      XR_CHECK_ARG(rc->other->rows() == rc->rows() && rc->other->cols() == rc->cols(),
                   "compute: the shared projection buffer has another detector size");
      XR_CHECK_ARG(n <= cap, "compute: more projections than the shared buffer holds");
    }
  }
  p.sample_counter = rc->count_samples ? reinterpret_cast<unsigned long long*>(rc->d_counters.p) : nullptr;
  p.loaded_counter =
      rc->count_samples ? reinterpret_cast<unsigned long long*>(rc->d_counters.as<char>() + 56) : nullptr;
  p.err_counter = reinterpret_cast<unsigned int*>(rc->d_counters.as<char>() + 8);
  {
    // Longest possible chord: the index-box diagonal scaled to mm by the largest
    // spacing; 64x margin covers scaled (non-rigid) poses.
    const double dx = (double)(vol.desc.n[0] - 1), dy = (double)(vol.desc.n[1] - 1), dz = (double)(vol.desc.n[2] - 1);
    const double sp = std::fmax(vol.desc.spacing[0], std::fmax(vol.desc.spacing[1], vol.desc.spacing[2]));
    const double ms = 64.0 * std::sqrt(dx * dx + dy * dy + dz * dz) * sp / (double)rc->step + 64.0;
    p.max_steps = (unsigned long long)std::fmin(ms, 2147483647.0);
  }
  p.num_projs = n;
  p.rows = (int32_t)rc->rows();
  p.cols = (int32_t)rc->cols();
  p.step = rc->step;
  p.default_bg = rc->default_bg;
  p.kernel_id = rc->kernel_id;
  p.store = rc->store;
  return XR_OK;
}

// Uploads dirty host state and enqueues geometry + DRR kernels on the stream.
static xr_status rc_enqueue_compute(xr_raycaster rc, int32_t vol_idx) {
  XR_CHECK_ARG(rc, "compute: NULL handle");
  cudaStream_t s = rc->stream();
  DrrParams p{};
  xr_status st = rc_prepare(rc, vol_idx, s, p);
  if (st != XR_OK) return st;
  const auto& vol = *rc->vols[(size_t)vol_idx];
  st = rc_choose_config(rc, vol, p, s);
  if (st != XR_OK) return st;
  rc->last_layout = p.vol.layout;
  rc->last_bw = p.block_warps_x;
  rc->last_unroll = p.unroll;
  rc->last_warp_rows = p.warp_tall ? 8 : 4;
  XR_CUDA_TRY(launch_drr(p, s));
  if (rc->ext_host)
    XR_CUDA_TRY(cudaMemcpyAsync(rc->ext_host, p.out, (size_t)p.num_projs * (size_t)(rc->rows() * rc->cols()) * 4,
                                cudaMemcpyDeviceToHost, s));
  return XR_OK;
}

extern "C" XR_API xr_status xr_rc_set_launch_config(xr_raycaster rc, int32_t layout, int32_t bw, int32_t unroll) {
  return xr_rc_set_launch_config_ex(rc, layout, bw, unroll, 4);
}

extern "C" XR_API xr_status xr_rc_set_launch_config_ex(xr_raycaster rc, int32_t layout, int32_t bw, int32_t unroll,
                                                      int32_t warp_rows) {
  XR_CHECK_ARG(rc, "set_launch_config: NULL handle");
  XR_CHECK_ARG(layout == XR_LAYOUT_AUTO || warp_rows == 4 || warp_rows == 8,
               "set_launch_config: warp_rows must be 4 (8x4-pixel warps) or 8 (4x8)");
  XR_CHECK_ARG(layout >= XR_LAYOUT_AUTO && layout <= 3, "set_launch_config: bad layout");
  XR_CHECK_ARG(layout == XR_LAYOUT_AUTO || bw == 1 || bw == 2 || bw == 4 || bw == 8,
               "set_launch_config: block_warps_x must be 1, 2, 4 or 8");
  XR_CHECK_ARG(layout == XR_LAYOUT_AUTO || (unroll >= 1 && unroll <= 6),
               "set_launch_config: unroll must be 1 to 6");
  rc->cfg_layout = layout;
  rc->cfg_bw = bw;
  rc->cfg_unroll = unroll;
  rc->cfg_warp_rows = warp_rows;
  rc->generation++;
  return XR_OK;
}

extern "C" XR_API xr_status xr_rc_get_launch_config(xr_raycaster rc, int32_t* layout, int32_t* bw, int32_t* unroll) {
  XR_CHECK_ARG(rc && layout && bw && unroll, "get_launch_config: NULL argument");
  *layout = rc->last_layout;
  *bw = rc->last_bw;
  *unroll = rc->last_unroll;
  return XR_OK;
}

extern "C" XR_API xr_status xr_rc_get_launch_config_ex(xr_raycaster rc, int32_t* layout, int32_t* bw, int32_t* unroll,
                                                      int32_t* warp_rows) {
  XR_CHECK_ARG(rc && layout && bw && unroll && warp_rows, "get_launch_config: NULL argument");
  *layout = rc->last_layout;
  *bw = rc->last_bw;
  *unroll = rc->last_unroll;
  *warp_rows = rc->last_warp_rows;
  return XR_OK;
}

extern "C" XR_API xr_status xr_rc_set_empty_space_skipping(xr_raycaster rc, int32_t enable) {
  XR_CHECK_ARG(rc, "set_empty_space_skipping: NULL handle");
  rc->skip_empty = enable != 0;
  rc->generation++;
  return XR_OK;
}

extern "C" XR_API xr_status xr_rc_set_build_cell_layout(xr_raycaster rc, int32_t enable) {
  XR_CHECK_ARG(rc, "set_build_cell_layout: NULL handle");
  rc->build_cells = enable != 0;
  return XR_OK;
}

extern "C" XR_API xr_status xr_rc_compute(xr_raycaster rc, int32_t vol_idx) {
  XR_CHECK_ARG(rc, "compute: NULL handle");
  DeviceGuard g(rc->device);
  if (rc->count_samples) {
    XR_CUDA_TRY(cudaMemsetAsync(rc->d_counters.p, 0, 8, rc->stream()));
    XR_CUDA_TRY(cudaMemsetAsync(rc->d_counters.as<char>() + 56, 0, 8, rc->stream()));
  }
  return rc_enqueue_compute(rc, vol_idx);
}

extern "C" XR_API xr_status xr_rc_proj(xr_raycaster rc, int64_t idx, float* dst) {
  XR_CHECK_ARG(rc && dst, "proj: NULL argument");
  XR_CHECK_ARG(rc->allocated, "proj: resources not allocated");
  XR_CHECK_ARG(idx >= 0 && idx < rc->num_projs, "proj: index out of range");
  xr_status st = xr_rc_synchronize(rc);
  if (st != XR_OK) return st;
  DeviceGuard g(rc->device);
  const size_t npix = (size_t)(rc->rows() * rc->cols());
  XR_CUDA_TRY(cudaMemcpy(dst, rc_out(rc, nullptr) + (size_t)idx * npix, npix * 4, cudaMemcpyDeviceToHost));
  return XR_OK;
}

extern "C" XR_API xr_status xr_rc_copy_projs_to_host(xr_raycaster rc, float* dst) {
  XR_CHECK_ARG(rc && dst, "copy_projs_to_host: NULL argument");
  XR_CHECK_ARG(rc->allocated, "copy_projs_to_host: resources not allocated");
  xr_status st = xr_rc_synchronize(rc);
  if (st != XR_OK) return st;
  DeviceGuard g(rc->device);
  const size_t n = (size_t)(rc->rows() * rc->cols()) * (size_t)rc->num_projs;
  XR_CUDA_TRY(cudaMemcpy(dst, rc_out(rc, nullptr), n * 4, cudaMemcpyDeviceToHost));
  return XR_OK;
}

extern "C" XR_API xr_status xr_rc_device_pixel_buf(xr_raycaster rc, float** out) {
  XR_CHECK_ARG(rc && out, "device_pixel_buf: NULL argument");
  XR_CHECK_ARG(rc->allocated, "device_pixel_buf: resources not allocated");
  *out = rc_out(rc, nullptr);
  return XR_OK;
}

extern "C" XR_API xr_status xr_rc_use_other_proj_buf(xr_raycaster rc, xr_raycaster other) {
  XR_CHECK_ARG(rc, "use_other_proj_buf: NULL handle");
  if (!other || other == rc) {
    rc->other = nullptr;
    rc->other_id = 0;
  } else {
    XR_CHECK_ARG(reg_contains(other), "use_other_proj_buf: unknown or destroyed ray caster");
    XR_CHECK_ARG(other->device == rc->device, "use_other_proj_buf: the ray casters are on different devices");
    XR_CHECK_ARG(!other->other, "use_other_proj_buf: that ray caster itself writes into another's buffer");
    rc->other = other;
    rc->other_id = other->id;
  }
  rc->generation++;
  return XR_OK;
}

extern "C" XR_API xr_status xr_rc_use_external_host_pixel_buf(xr_raycaster rc, float* host_buf) {
  XR_CHECK_ARG(rc, "use_external_host_pixel_buf: NULL handle");
  rc->ext_host = host_buf;
  rc->generation++;
  return XR_OK;
}

extern "C" XR_API xr_status xr_rc_last_num_samples(xr_raycaster rc, uint64_t* out) {
  XR_CHECK_ARG(rc && out, "last_num_samples: NULL argument");
  XR_CHECK_ARG(rc->count_samples, "last_num_samples: counting is disabled (xr_rc_set_count_samples)");
  xr_status st = xr_rc_synchronize(rc);
  if (st != XR_OK) return st;
  DeviceGuard g(rc->device);
  unsigned long long v = 0;
  XR_CUDA_TRY(cudaMemcpy(&v, rc->d_counters.p, 8, cudaMemcpyDeviceToHost));
  *out = v;
  return XR_OK;
}

extern "C" XR_API xr_status xr_rc_last_num_loaded_samples(xr_raycaster rc, uint64_t* out) {
  XR_CHECK_ARG(rc && out, "last_num_loaded_samples: NULL argument");
  XR_CHECK_ARG(rc->count_samples, "last_num_loaded_samples: counting is disabled (xr_rc_set_count_samples)");
  xr_status st = xr_rc_synchronize(rc);
  if (st != XR_OK) return st;
  DeviceGuard g(rc->device);
  unsigned long long v = 0;
  XR_CUDA_TRY(cudaMemcpy(&v, rc->d_counters.as<char>() + 56, 8, cudaMemcpyDeviceToHost));
  *out = v;
  return XR_OK;
}

extern "C" XR_API xr_status xr_rc_distribute_xforms_device(xr_raycaster rc, int64_t n, const double* d_xf) {
  XR_CHECK_ARG(rc && d_xf, "distribute_xforms_device: NULL argument");
  DeviceGuard g(rc->device);
  return rc_distribute_device_on(rc, n, d_xf, rc->stream());
}

// distribute_xforms_among_cam_models with device poses, enqueued on stream s;
// d_xf NULL: the poses are written into the caster's transforms by a later
// launch on s (a device optimizer's sampling).
static xr_status rc_distribute_device_on(xr_raycaster rc, int64_t n, const double* d_xf, cudaStream_t s) {
  XR_CHECK_ARG(rc && n > 0, "distribute_xforms_device: NULL argument");
  XR_CHECK_ARG(!rc->cams.empty(), "distribute_xforms_device: no camera models");
  XR_CHECK_ARG(rc->allocated, "distribute_xforms_device: allocate_resources first");
  XR_CHECK_ARG(n * (int64_t)rc->cams.size() == rc->num_projs,
               "distribute_xforms_device: num_xforms * num_cams must equal num_projs");
  if (d_xf) XR_CUDA_TRY(cudaMemcpyAsync(rc->d_xforms.p, d_xf, (size_t)n * 16 * 8, cudaMemcpyDeviceToDevice, s));
  rc->pose_count = n;
  rc->xforms_dirty = false;
  rc->xforms_on_device = true;
  bool changed = false;
  for (int64_t p = 0; p < rc->num_projs; ++p) {
    const int32_t c = (int32_t)(p / n);
    if (rc->cam_idx[(size_t)p] != c) { rc->cam_idx[(size_t)p] = c; changed = true; }
  }
  if (changed || rc->cam_idx_dirty) {
    cam_idx_distribute_kernel<<<(unsigned)((rc->num_projs + 255) / 256), 256, 0, s>>>(
        rc->d_cam_idx.as<int32_t>(), rc->num_projs, n);
    XR_CUDA_TRY(cudaGetLastError());
    rc->cam_idx_dirty = false;
  }
  return XR_OK;
}

// ======================================================== similarity metric
extern "C" XR_API xr_status xr_sm_create(int32_t kind, int32_t device, xr_simmetric* out) {
  XR_CHECK_ARG(out, "xr_sm_create: out is NULL");
  *out = nullptr;
  XR_CHECK_ARG(kind >= XR_SIM_NCC && kind <= XR_SIM_PATCH_GRAD_NCC, "xr_sm_create: unknown metric kind");
  int dev = device;
  if (dev < 0) XR_CUDA_TRY(cudaGetDevice(&dev));
  DeviceGuard g(dev);
  auto* sm = new (std::nothrow) xr_simmetric_s();
  if (!sm) return fail(XR_ERR_OUT_OF_MEMORY, "xr_sm_create: host allocation failed");
  sm->kind = kind;
  sm->device = dev;
  xr_patch_options_default(&sm->popt);
  cudaError_t e = cudaStreamCreateWithFlags(&sm->own_stream, cudaStreamNonBlocking);
  if (e != cudaSuccess) { delete sm; return cuda_fail(e, "cudaStreamCreateWithFlags"); }
  sm->id = reg_add(sm);
  *out = sm;
  return XR_OK;
}

extern "C" XR_API xr_status xr_sm_destroy(xr_simmetric sm) {
  if (!sm) return XR_OK;
  reg_remove(sm);
  DeviceGuard g(sm->device);
  cudaStreamSynchronize(sm->stream());
  cudaStreamDestroy(sm->own_stream);
  delete sm;
  return XR_OK;
}

extern "C" XR_API xr_status xr_sm_set_stream(xr_simmetric sm, void* s) {
  XR_CHECK_ARG(sm, "xr_sm_set_stream: NULL handle");
  sm->ext_stream = static_cast<cudaStream_t>(s);
  sm->has_ext_stream = s != nullptr;
  sm->generation++;
  return XR_OK;
}

extern "C" XR_API xr_status xr_sm_set_fixed_image(xr_simmetric sm, const float* img, int64_t rows, int64_t cols) {
  XR_CHECK_ARG(sm && img, "set_fixed_image: NULL argument");
  XR_CHECK_ARG(rows >= 2 && cols >= 2 && rows < (1 << 28) && cols < (1 << 28), "set_fixed_image: bad size");
  DeviceGuard g(sm->device);
  const size_t n = (size_t)(rows * cols);
  XR_CUDA_TRY(sm->d_fixed.reserve(n * 4));
  XR_CUDA_TRY(cudaMemcpy(sm->d_fixed.p, img, n * 4, cudaMemcpyHostToDevice));
  if (sm->rows != rows || sm->cols != cols) {
    sm->has_mask = false;
    sm->d_mask.release();
    sm->h_mask.clear();
    sm->wgt_img.clear();
  }
  sm->rows = rows;
  sm->cols = cols;
  sm->has_fixed = true;
  sm->allocated = false;
  sm->generation++;
  return XR_OK;
}

extern "C" XR_API xr_status xr_sm_set_mask(xr_simmetric sm, const uint8_t* mask) {
  XR_CHECK_ARG(sm, "set_mask: NULL handle");
  if (!mask) {
    sm->has_mask = false;
    sm->h_mask.clear();
    sm->allocated = false;
    sm->generation++;
    return XR_OK;
  }
  XR_CHECK_ARG(sm->has_fixed, "set_mask: set the fixed image first");
  DeviceGuard g(sm->device);
  const size_t n = (size_t)(sm->rows * sm->cols);
  XR_CUDA_TRY(sm->d_mask.reserve(n));
  XR_CUDA_TRY(cudaMemcpy(sm->d_mask.p, mask, n, cudaMemcpyHostToDevice));
  sm->h_mask.assign(mask, mask + n);
  sm->has_mask = true;
  sm->allocated = false;
  sm->generation++;
  return XR_OK;
}

extern "C" XR_API xr_status xr_sm_fixed_image(xr_simmetric sm, int64_t cap, float* out, int64_t* rows, int64_t* cols) {
  XR_CHECK_ARG(sm && rows && cols && (out || cap == 0), "fixed_image: NULL argument");
  XR_CHECK_ARG(sm->has_fixed, "fixed_image: no fixed image");
  *rows = sm->rows;
  *cols = sm->cols;
  const int64_t n = std::min<int64_t>(cap, sm->rows * sm->cols);
  if (n <= 0) return XR_OK;
  DeviceGuard g(sm->device);
  XR_CUDA_TRY(cudaMemcpy(out, sm->d_fixed.p, (size_t)n * 4, cudaMemcpyDeviceToHost));
  return XR_OK;
}

extern "C" XR_API xr_status xr_sm_mask(xr_simmetric sm, int64_t cap, uint8_t* out, int32_t* has_mask) {
  XR_CHECK_ARG(sm && has_mask && (out || cap == 0), "mask: NULL argument");
  *has_mask = sm->has_mask ? 1 : 0;
  const int64_t n = sm->has_mask ? std::min<int64_t>(cap, (int64_t)sm->h_mask.size()) : 0;
  if (n > 0) std::memcpy(out, sm->h_mask.data(), (size_t)n);
  return XR_OK;
}

extern "C" XR_API xr_status xr_sm_num_pix_per_proj(xr_simmetric sm, int64_t* out) {
  XR_CHECK_ARG(sm && out, "num_pix_per_proj: NULL argument");
  *out = sm->rows * sm->cols;
  return XR_OK;
}

extern "C" XR_API xr_status xr_sm_num_moving_images(xr_simmetric sm, int64_t* out) {
  XR_CHECK_ARG(sm && out, "num_moving_images: NULL argument");
  *out = sm->num_mov;
  return XR_OK;
}

extern "C" XR_API xr_status xr_sm_set_num_moving_images(xr_simmetric sm, int64_t n) {
  XR_CHECK_ARG(sm && n > 0, "set_num_moving_images: NULL handle or non-positive count");
  XR_CHECK_ARG(!sm->allocated || n <= sm->capacity,
               "set_num_moving_images: more images than allocate_resources reserved; allocate again");
  if (n != sm->num_mov) { sm->num_mov = n; sm->generation++; }
  return XR_OK;
}

extern "C" XR_API xr_status xr_sm_set_mov_imgs_buf_from_ray_caster(xr_simmetric sm, xr_raycaster rc, int64_t off) {
  XR_CHECK_ARG(sm && rc && off >= 0, "set_mov_imgs_buf_from_ray_caster: NULL argument or negative offset");
  sm->rc = rc;
  sm->rc_id = rc->id;
  sm->mov_dev = nullptr;
  sm->mov_host = nullptr;
  sm->proj_offset = off;
  sm->generation++;
  return XR_OK;
}

extern "C" XR_API xr_status xr_sm_set_mov_imgs_host_buf(xr_simmetric sm, const float* h) {
  XR_CHECK_ARG(sm && h, "set_mov_imgs_host_buf: NULL argument");
  sm->rc = nullptr;
  sm->rc_id = 0;
  sm->mov_dev = nullptr;
  sm->mov_host = h;
  sm->proj_offset = 0;
  sm->generation++;
  return XR_OK;
}

extern "C" XR_API xr_status xr_sm_set_mov_imgs_device_buf(xr_simmetric sm, const float* d, int64_t off) {
  XR_CHECK_ARG(sm && d && off >= 0, "set_mov_imgs_device_buf: NULL argument or negative offset");
  sm->rc = nullptr;
  sm->rc_id = 0;
  sm->mov_host = nullptr;
  sm->mov_dev = d;
  sm->proj_offset = off;
  sm->generation++;
  return XR_OK;
}

extern "C" XR_API xr_status xr_sm_set_smooth_img_before_sobel_kernel_radius(xr_simmetric sm, int32_t r) {
  XR_CHECK_ARG(sm, "set_smooth_img_before_sobel_kernel_radius: NULL handle");
  if (r != 0 && r != 3 && r != 5)
    return fail(XR_ERR_UNSUPPORTED, "set_smooth_img_before_sobel_kernel_radius: only 0, 3 and 5 are implemented");
  sm->smooth_ksize = r;
  sm->allocated = false;
  sm->generation++;
  return XR_OK;
}

extern "C" XR_API xr_status xr_sm_set_patch_radius(xr_simmetric sm, int32_t r) {
  XR_CHECK_ARG(sm && r > 0 && r <= 16, "set_patch_radius: radius must be in [1, 16]");
  sm->patch_radius = r;
  sm->allocated = false;
  sm->generation++;
  return XR_OK;
}

extern "C" XR_API xr_status xr_sm_set_patch_stride(xr_simmetric sm, int32_t s) {
  XR_CHECK_ARG(sm && s > 0 && s <= 4, "set_patch_stride: stride must be in [1, 4]");
  sm->patch_stride = s;
  sm->allocated = false;
  sm->generation++;
  return XR_OK;
}

extern "C" XR_API xr_status xr_patch_options_default(xr_patch_options* o) {
  XR_CHECK_ARG(o, "xr_patch_options_default: NULL argument");
  *o = xr_patch_options{};
  o->use_mask_for_weighting = 1;
  o->use_mask_for_patch_stats = 0;
  o->normalize_weights_as_prob = 1;
  o->weight_patch_sims_in_combine = 1;
  o->compute_mean_of_patch_sims = 0;
  o->num_rand_patches = 100;
  o->rand_patch_min_pixels_sep = -1.0;
  o->rand_seed = 0;
  return XR_OK;
}

extern "C" XR_API xr_status xr_sm_set_patch_options(xr_simmetric sm, const xr_patch_options* o) {
  XR_CHECK_ARG(sm && o, "set_patch_options: NULL argument");
  XR_CHECK_ARG(sm->kind == XR_SIM_PATCH_NCC || sm->kind == XR_SIM_PATCH_GRAD_NCC,
               "set_patch_options: not a patch metric");
  XR_CHECK_ARG(!(o->use_fixed_img_patch_variances_as_wgts && o->use_mov_img_patch_variances_as_wgts),
               "set_patch_options: fixed and moving patch variances cannot both be the weights");
  XR_CHECK_ARG(!o->choose_rand_patches || o->num_rand_patches > 0,
               "set_patch_options: num_rand_patches must be positive");
  XR_CHECK_ARG(!(o->mask_only_for_weights && o->use_mask_for_patch_stats),
               "set_patch_options: masked statistics need the mask inside the patches");
  sm->popt = *o;
  sm->rng.seed((std::mt19937::result_type)o->rand_seed);
  sm->allocated = false;
  sm->generation++;
  return XR_OK;
}

extern "C" XR_API xr_status xr_sm_get_patch_options(xr_simmetric sm, xr_patch_options* o) {
  XR_CHECK_ARG(sm && o, "get_patch_options: NULL argument");
  *o = sm->popt;
  return XR_OK;
}

extern "C" XR_API xr_status xr_sm_set_patch_wgt_img(xr_simmetric sm, const float* img) {
  XR_CHECK_ARG(sm, "set_patch_wgt_img: NULL handle");
  if (!img) {
    sm->wgt_img.clear();
  } else {
    XR_CHECK_ARG(sm->has_fixed, "set_patch_wgt_img: set the fixed image first");
    sm->wgt_img.assign(img, img + sm->rows * sm->cols);
  }
  sm->allocated = false;
  sm->generation++;
  return XR_OK;
}

extern "C" XR_API xr_status xr_sm_set_patches_to_use(xr_simmetric sm, int64_t n, const int64_t* idx) {
  XR_CHECK_ARG(sm && (idx || n == 0), "set_patches_to_use: NULL argument");
  XR_CHECK_ARG(sm->kind == XR_SIM_PATCH_NCC || sm->kind == XR_SIM_PATCH_GRAD_NCC,
               "set_patches_to_use: not a patch metric");
  XR_CHECK_ARG(n >= 0 && n <= INT32_MAX, "set_patches_to_use: bad count");
  std::vector<int32_t> v((size_t)n);
  for (int64_t k = 0; k < n; ++k) {
    XR_CHECK_ARG(idx[k] >= 0 && idx[k] <= INT32_MAX, "set_patches_to_use: patch index out of range");
    v[(size_t)k] = (int32_t)idx[k];
  }
  sm->user_idx.swap(v);
  sm->allocated = false;
  sm->generation++;
  return XR_OK;
}

extern "C" XR_API xr_status xr_sm_patch_scores(xr_simmetric sm, int64_t img, int64_t cap, float* out, int64_t* count) {
  XR_CHECK_ARG(sm && count && (out || cap == 0), "patch_scores: NULL argument");
  XR_CHECK_ARG(sm->kind == XR_SIM_PATCH_NCC || sm->kind == XR_SIM_PATCH_GRAD_NCC, "patch_scores: not a patch metric");
  XR_CHECK_ARG(sm->allocated && sm->popt.save_all_per_patch_scores,
               "patch_scores: set save_all_per_patch_scores before allocate_resources");
  XR_CHECK_ARG(img >= 0 && img < sm->num_mov, "patch_scores: bad moving image index");
  const int64_t np = (int64_t)sm->ncr * sm->ncc;
  const bool listed = !sm->user_idx.empty() || sm->popt.choose_rand_patches;
  const int64_t used = listed ? (int64_t)sm->last_idx.size() : np;
  *count = used;  // xReg sizes the list by num_patches(): the patches in use
  if (cap <= 0) return XR_OK;
  DeviceGuard g(sm->device);
  cudaStream_t s = sm->stream();
  std::vector<float> all((size_t)np);
  float sim = 0.0f;
  XR_CUDA_TRY(cudaMemcpyAsync(all.data(), sm->d_pscores.as<float>() + img * np, (size_t)np * 4,
                              cudaMemcpyDeviceToHost, s));
  XR_CUDA_TRY(cudaMemcpyAsync(&sim, sm->d_sims.as<float>() + img, 4, cudaMemcpyDeviceToHost, s));
  XR_CUDA_TRY(cudaStreamSynchronize(s));
  const int64_t n = std::min<int64_t>(cap, used);
  if (sim == FLT_MAX) {  // flat moving image: xReg marks every patch
    for (int64_t i = 0; i < n; ++i) out[i] = FLT_MAX;
    return XR_OK;
  }
  // xReg keeps the scores in the order of the patches in use
  for (int64_t i = 0; i < n; ++i) out[i] = all[(size_t)(listed ? (int64_t)sm->last_idx[(size_t)i] : i)];
  return XR_OK;
}

extern "C" XR_API xr_status xr_sm_patch_indices_used(xr_simmetric sm, int64_t cap, int64_t* idx, int64_t* count) {
  XR_CHECK_ARG(sm && count && (idx || cap == 0), "patch_indices_used: NULL argument");
  XR_CHECK_ARG(sm->kind == XR_SIM_PATCH_NCC || sm->kind == XR_SIM_PATCH_GRAD_NCC,
               "patch_indices_used: not a patch metric");
  if (!sm->user_idx.empty() || sm->popt.choose_rand_patches) {
    *count = (int64_t)sm->last_idx.size();
    for (int64_t k = 0; k < std::min<int64_t>(cap, *count); ++k) idx[k] = sm->last_idx[(size_t)k];
  } else {
    *count = (int64_t)sm->ncr * sm->ncc;
    for (int64_t k = 0; k < std::min<int64_t>(cap, *count); ++k) idx[k] = k;
  }
  return XR_OK;
}

// Zero-mean fixed image and its statistics for one NCC direction.
static xr_status sm_prepare_ncc_fixed(xr_simmetric sm, const float* img, DevBuf& fhat, FixedNCC& fx,
                                      cudaStream_t s) {
  const int64_t n = sm->rows * sm->cols;
  const uint8_t* mask = sm->has_mask ? sm->d_mask.as<uint8_t>() : nullptr;
  XR_CUDA_TRY(sm->d_scratch.reserve(64));
  double h[3];
  XR_CUDA_TRY(launch_image_stats(img, n, mask, sm->d_scratch.as<double>(), s));
  XR_CUDA_TRY(cudaMemcpyAsync(h, sm->d_scratch.p, 24, cudaMemcpyDeviceToHost, s));
  XR_CUDA_TRY(cudaStreamSynchronize(s));
  const double cnt = h[2];
  if (!(cnt >= 2.0)) return fail(XR_ERR_INVALID_ARG, "allocate_resources: fewer than 2 usable pixels");
  const double mean = h[0] / cnt;
  double sd = std::sqrt(h[1] / (cnt - 1.0));
  if (sd < 1.0e-6) sd = 1.0e-6;
  XR_CUDA_TRY(fhat.reserve((size_t)n * 4));
  XR_CUDA_TRY(launch_sub_scalar(img, n, mean, fhat.as<float>(), s));
  XR_CUDA_TRY(launch_sum_f(fhat.as<float>(), n, mask, sm->d_scratch.as<double>(), s));
  XR_CUDA_TRY(cudaMemcpyAsync(h, sm->d_scratch.p, 24, cudaMemcpyDeviceToHost, s));
  XR_CUDA_TRY(cudaStreamSynchronize(s));
  fx.fhat = fhat.as<float>();
  fx.sd = sd;
  fx.sum_fhat = h[0];
  sm->n_used = (int64_t)cnt;
  return XR_OK;
}

// compute_weights (xregImgSimMetric2DPatchCommon.cpp:306-410): the weight image
// at each patch centre (zero at masked centres when the mask weights), else the
// unmasked fraction of the patch when the mask weights, normalised to sum 1;
// otherwise 1.  wimg: weight image values at the patch centres, or nullptr.
static bool patch_weights(const xr_simmetric_s* sm, const std::vector<float>* wimg, const std::vector<int>& ucount,
                          std::vector<double>& w) {
  const int64_t np = (int64_t)sm->ncr * sm->ncc;
  const int d = 2 * sm->patch_radius + 1;
  const bool use_img = wimg != nullptr;
  const bool use_mask = sm->popt.use_mask_for_weighting && sm->has_mask;
  w.assign((size_t)np, 1.0);
  if (!use_img && !use_mask) return false;
  for (int64_t p = 0; p < np; ++p) {
    const int64_t cr = sm->patch_radius + (p / sm->ncc) * sm->patch_stride;
    const int64_t cc = sm->patch_radius + (p % sm->ncc) * sm->patch_stride;
    if (use_img) {
      double v = (*wimg)[(size_t)p];
      if (use_mask && !sm->h_mask[(size_t)(cr * sm->cols + cc)]) v = 0.0;
      w[(size_t)p] = v;
    } else {
      w[(size_t)p] = (double)ucount[(size_t)p] / (double)(d * d);
    }
  }
  if (sm->popt.normalize_weights_as_prob) {
    double t = 0;
    for (double v : w) t += v;
    for (double& v : w) v /= t;
  }
  return true;
}

// Fixed side of a patch metric: per-patch statistics of the fixed image (or its
// gradients), the static patch weights and what the moving-variance weights need.
static xr_status sm_prepare_patches(xr_simmetric sm, cudaStream_t s) {
  const xr_patch_options& o = sm->popt;
  const bool grad = sm->kind == XR_SIM_PATCH_GRAD_NCC;
  const int rows = (int)sm->rows, cols = (int)sm->cols;
  const int64_t np = (int64_t)sm->ncr * sm->ncc;
  const uint8_t* dmask = sm->has_mask ? sm->d_mask.as<uint8_t>() : nullptr;
  const int ums = o.use_mask_for_patch_stats ? 1 : 0;
  // fixed-variance weights of each direction's own image (patch NCC, or patch
  // grad-NCC with gradient-image variances), or of the fixed image for both
  const bool fv_dir = o.use_fixed_img_patch_variances_as_wgts && (!grad || o.use_variances_in_grad_imgs_as_wgts);
  const bool fv_img = o.use_fixed_img_patch_variances_as_wgts && grad && !o.use_variances_in_grad_imgs_as_wgts;
  const bool want_ucount = o.use_mask_for_weighting && sm->has_mask;
  DevBuf wv_x, wv_y, wv_img, ucnt;
  const float* img_x = grad ? sm->d_gx.as<float>() : sm->d_fixed.as<float>();
  XR_CUDA_TRY(sm->d_pmean_x.reserve((size_t)np * 4));
  XR_CUDA_TRY(sm->d_pscale_x.reserve((size_t)np * 4));
  if (fv_dir) XR_CUDA_TRY(wv_x.reserve((size_t)np * 4));
  XR_CUDA_TRY(launch_patch_fixed_stats(img_x, rows, cols, sm->patch_radius, sm->patch_stride, sm->ncr, sm->ncc,
                                       dmask, ums, sm->d_pmean_x.as<float>(), sm->d_pscale_x.as<float>(),
                                       fv_dir ? wv_x.as<float>() : nullptr, nullptr, s));
  if (grad) {
    XR_CUDA_TRY(sm->d_pmean_y.reserve((size_t)np * 4));
    XR_CUDA_TRY(sm->d_pscale_y.reserve((size_t)np * 4));
    if (fv_dir) XR_CUDA_TRY(wv_y.reserve((size_t)np * 4));
    XR_CUDA_TRY(launch_patch_fixed_stats(sm->d_gy.as<float>(), rows, cols, sm->patch_radius, sm->patch_stride,
                                         sm->ncr, sm->ncc, dmask, ums, sm->d_pmean_y.as<float>(),
                                         sm->d_pscale_y.as<float>(), fv_dir ? wv_y.as<float>() : nullptr, nullptr,
                                         s));
  }
  if (fv_img) {
    XR_CUDA_TRY(wv_img.reserve((size_t)np * 4));
    XR_CUDA_TRY(launch_patch_fixed_stats(sm->d_fixed.as<float>(), rows, cols, sm->patch_radius, sm->patch_stride,
                                         sm->ncr, sm->ncc, dmask, dmask ? 1 : 0, nullptr, nullptr,
                                         wv_img.as<float>(), nullptr, s));
  }
  if (want_ucount) {
    XR_CUDA_TRY(ucnt.reserve((size_t)np * 4));
    XR_CUDA_TRY(launch_patch_fixed_stats(sm->d_fixed.as<float>(), rows, cols, sm->patch_radius, sm->patch_stride,
                                         sm->ncr, sm->ncc, dmask, 0, nullptr, nullptr, nullptr, ucnt.as<int>(), s));
  }
  std::vector<float> h_wv_x, h_wv_y, h_wv_img, h_user;
  std::vector<int> h_ucnt;
  auto fetch = [&](DevBuf& b, auto& v) -> cudaError_t {
    v.resize((size_t)np);
    return cudaMemcpyAsync(v.data(), b.p, (size_t)np * sizeof(v[0]), cudaMemcpyDeviceToHost, s);
  };
  if (fv_dir) { XR_CUDA_TRY(fetch(wv_x, h_wv_x)); if (grad) XR_CUDA_TRY(fetch(wv_y, h_wv_y)); }
  if (fv_img) XR_CUDA_TRY(fetch(wv_img, h_wv_img));
  if (want_ucount) XR_CUDA_TRY(fetch(ucnt, h_ucnt));
  XR_CUDA_TRY(cudaStreamSynchronize(s));
  if (!sm->wgt_img.empty()) {
    h_user.resize((size_t)np);
    for (int64_t p = 0; p < np; ++p) {
      const int64_t cr = sm->patch_radius + (p / sm->ncc) * sm->patch_stride;
      const int64_t cc = sm->patch_radius + (p % sm->ncc) * sm->patch_stride;
      h_user[(size_t)p] = sm->wgt_img[(size_t)(cr * sm->cols + cc)];
    }
  }
  const std::vector<float>* user = sm->wgt_img.empty() ? nullptr : &h_user;
  bool any = false;
  if (fv_dir) {
    any |= patch_weights(sm, &h_wv_x, h_ucnt, sm->w_x);
    if (grad) any |= patch_weights(sm, &h_wv_y, h_ucnt, sm->w_y);
  } else if (fv_img) {
    any |= patch_weights(sm, &h_wv_img, h_ucnt, sm->w_x);
    sm->w_y = sm->w_x;
  } else {
    any |= patch_weights(sm, user, h_ucnt, sm->w_x);
    sm->w_y = sm->w_x;
  }
  if (!grad) sm->w_y = sm->w_x;
  // random subsets are drawn with the metric's own weights (patch grad-NCC: the
  // ones its mask / weight image give, ImgSimMetric2DPatchGradNCCCPU::compute)
  if (grad && (fv_dir || fv_img)) patch_weights(sm, user, h_ucnt, sm->w_draw);
  else sm->w_draw = sm->w_x;
  sm->has_pw = any;
  if (any) {
    std::vector<float> f((size_t)np);
    for (int64_t p = 0; p < np; ++p) f[(size_t)p] = (float)sm->w_x[(size_t)p];
    XR_CUDA_TRY(sm->d_pw_x.reserve((size_t)np * 4));
    XR_CUDA_TRY(cudaMemcpy(sm->d_pw_x.p, f.data(), (size_t)np * 4, cudaMemcpyHostToDevice));
    for (int64_t p = 0; p < np; ++p) f[(size_t)p] = (float)sm->w_y[(size_t)p];
    XR_CUDA_TRY(sm->d_pw_y.reserve((size_t)np * 4));
    XR_CUDA_TRY(cudaMemcpy(sm->d_pw_y.p, f.data(), (size_t)np * 4, cudaMemcpyHostToDevice));
  }
  sm->mvar_mode = o.use_mov_img_patch_variances_as_wgts ? ((grad && o.use_variances_in_grad_imgs_as_wgts) ? 2 : 1) : 0;
  if (!sm->user_idx.empty()) {
    // set_patches_to_use: this list, duplicates counted, instead of the grid or a draw
    for (int32_t i : sm->user_idx)
      XR_CHECK_ARG(i >= 0 && i < np, "allocate_resources: a patch given to set_patches_to_use is outside the grid");
    XR_CUDA_TRY(sm->d_pcnt.reserve((size_t)np * 4));
    XR_CUDA_TRY(sm->d_pidx.reserve(sm->user_idx.size() * 4));
    sm->last_idx = sm->user_idx;
    sm->tot_w_x = 0;
    sm->tot_w_y = 0;
    for (int32_t i : sm->last_idx) { sm->tot_w_x += sm->w_x[(size_t)i]; sm->tot_w_y += sm->w_y[(size_t)i]; }
    sm->nused = (int64_t)sm->last_idx.size();
    XR_CUDA_TRY(cudaMemcpyAsync(sm->d_pidx.p, sm->last_idx.data(), sm->last_idx.size() * 4, cudaMemcpyHostToDevice,
                                s));
    XR_CUDA_TRY(cudaMemsetAsync(sm->d_pcnt.p, 0, (size_t)np * 4, s));
    XR_CUDA_TRY(launch_patch_scatter_counts(sm->d_pidx.as<int32_t>(), sm->nused, sm->d_pcnt.as<int32_t>(), s));
    XR_CUDA_TRY(cudaStreamSynchronize(s));  // last_idx's host copy is reused by the next prepare
  } else if (o.choose_rand_patches) {
    XR_CHECK_ARG(o.num_rand_patches < np, "allocate_resources: num_rand_patches must be below the patch count");
    double t = 0;
    for (double v : sm->w_draw) t += v;
    XR_CHECK_ARG(t > 0.0, "allocate_resources: random patches need a positive total weight");
    XR_CUDA_TRY(sm->d_pcnt.reserve((size_t)np * 4));
    XR_CUDA_TRY(sm->d_pidx.reserve((size_t)o.num_rand_patches * 4));
  } else {
    sm->tot_w_x = 0;
    sm->tot_w_y = 0;
    for (int64_t p = 0; p < np; ++p) { sm->tot_w_x += sm->w_x[(size_t)p]; sm->tot_w_y += sm->w_y[(size_t)p]; }
    sm->nused = np;
  }
  return XR_OK;
}

// patch_indices_to_use (xregImgSimMetric2DPatchCommon.cpp:412-493): draws
// num_rand_patches patch indices with probability proportional to the weights,
// rejecting candidates closer than the minimum separation to an accepted one;
// then uploads their multiplicities.
static xr_status sm_draw_patches(xr_simmetric sm, cudaStream_t s) {
  const xr_patch_options& o = sm->popt;
  std::discrete_distribution<size_t> dist(sm->w_draw.begin(), sm->w_draw.end());
  const double r = (double)sm->patch_radius;
  const double min_sep = o.rand_patch_min_pixels_sep < 0 ? std::sqrt(2.0 * r * r) : o.rand_patch_min_pixels_sep;
  const bool check = min_sep > 1.0e-8;
  std::vector<std::pair<double, double>> centres;
  sm->last_idx.clear();
  const int64_t limit = 1000 * o.num_rand_patches + 100000;
  for (int64_t attempts = 0; (int64_t)sm->last_idx.size() < o.num_rand_patches; ++attempts) {
    if (attempts >= limit) return fail(XR_ERR_INVALID_ARG, "compute: could not place the random patches apart");
    const size_t cand = dist(sm->rng);
    if (check) {
      const double cr = r + (double)((int64_t)cand / sm->ncc) * sm->patch_stride;
      const double cc = r + (double)((int64_t)cand % sm->ncc) * sm->patch_stride;
      bool ok = true;
      for (const auto& e : centres)
        if (std::sqrt((e.first - cr) * (e.first - cr) + (e.second - cc) * (e.second - cc)) < min_sep) {
          ok = false;
          break;
        }
      if (!ok) continue;
      centres.emplace_back(cr, cc);
    }
    sm->last_idx.push_back((int32_t)cand);
  }
  sm->tot_w_x = 0;
  sm->tot_w_y = 0;
  for (int32_t i : sm->last_idx) { sm->tot_w_x += sm->w_x[(size_t)i]; sm->tot_w_y += sm->w_y[(size_t)i]; }
  sm->nused = (int64_t)sm->last_idx.size();
  const size_t np = (size_t)sm->ncr * (size_t)sm->ncc;
  XR_CUDA_TRY(cudaMemcpyAsync(sm->d_pidx.p, sm->last_idx.data(), sm->last_idx.size() * 4, cudaMemcpyHostToDevice, s));
  XR_CUDA_TRY(cudaMemsetAsync(sm->d_pcnt.p, 0, np * 4, s));
  XR_CUDA_TRY(launch_patch_scatter_counts(sm->d_pidx.as<int32_t>(), (int64_t)sm->last_idx.size(),
                                          sm->d_pcnt.as<int32_t>(), s));
  return XR_OK;
}

extern "C" XR_API xr_status xr_sm_allocate_resources(xr_simmetric sm) {
  XR_CHECK_ARG(sm, "allocate_resources: NULL handle");
  XR_CHECK_ARG(sm->has_fixed, "allocate_resources: no fixed image");
  XR_CHECK_ARG(sm->num_mov > 0, "allocate_resources: num_moving_images is 0");
  XR_CHECK_ARG(sm->live_rc() || sm->mov_dev || sm->mov_host, "allocate_resources: no moving image buffer");
  DeviceGuard g(sm->device);
  cudaStream_t s = sm->stream();
  const int64_t n = sm->rows * sm->cols;
  const int rows = (int)sm->rows, cols = (int)sm->cols;
  sm->capacity = sm->num_mov;
  if (sm->kind == XR_SIM_NCC) {
    xr_status st = sm_prepare_ncc_fixed(sm, sm->d_fixed.as<float>(), sm->d_fhat_x, sm->fx, s);
    if (st != XR_OK) return st;
    sm->nblk = (int)std::min<int64_t>(128, (n + 255) / 256);
    XR_CUDA_TRY(sm->d_partials.reserve((size_t)sm->capacity * sm->nblk * 3 * 8));
  } else if (sm->kind == XR_SIM_GRAD_NCC) {
    XR_CHECK_ARG(rows >= 8 && cols >= 8, "allocate_resources: gradient metrics need images of at least 8x8");
    XR_CUDA_TRY(sm->d_gx.reserve((size_t)n * 4));
    XR_CUDA_TRY(sm->d_gy.reserve((size_t)n * 4));
    XR_CUDA_TRY(launch_grad_images(sm->d_fixed.as<float>(), rows, cols, 1, sm->smooth_ksize, sm->d_gx.as<float>(),
                                   sm->d_gy.as<float>(), s));
    xr_status st = sm_prepare_ncc_fixed(sm, sm->d_gx.as<float>(), sm->d_fhat_x, sm->fx, s);
    if (st != XR_OK) return st;
    st = sm_prepare_ncc_fixed(sm, sm->d_gy.as<float>(), sm->d_fhat_y, sm->fy, s);
    if (st != XR_OK) return st;
    XR_CUDA_TRY(launch_grad_moments(nullptr, rows, cols, 0, sm->smooth_ksize, nullptr, nullptr, nullptr, nullptr, s,
                                    &sm->nblk));
    XR_CUDA_TRY(sm->d_partials.reserve((size_t)sm->capacity * sm->nblk * 6 * 8));
  } else {
    const int d = 2 * sm->patch_radius + 1;
    XR_CHECK_ARG(d <= rows && d <= cols, "allocate_resources: patch larger than the image");
    const int grad = sm->kind == XR_SIM_PATCH_GRAD_NCC;
    XR_CHECK_ARG(!grad || (rows >= 8 && cols >= 8), "allocate_resources: gradient metrics need images of at least 8x8");
    sm->ncr = (rows - 1 - 2 * sm->patch_radius) / sm->patch_stride + 1;
    sm->ncc = (cols - 1 - 2 * sm->patch_radius) / sm->patch_stride + 1;
    if (grad) {
      XR_CUDA_TRY(sm->d_gx.reserve((size_t)n * 4));
      XR_CUDA_TRY(sm->d_gy.reserve((size_t)n * 4));
      XR_CUDA_TRY(launch_grad_images(sm->d_fixed.as<float>(), rows, cols, 1, sm->smooth_ksize,
                                     sm->d_gx.as<float>(), sm->d_gy.as<float>(), s));
    }
    xr_status st = sm_prepare_patches(sm, s);
    if (st != XR_OK) return st;
    PatchFixed px{}, py{};
    sm->nblk = patch_ncc_max_blocks(sm->ncr, sm->ncc);
    XR_CUDA_TRY(sm->d_partials.reserve((size_t)sm->capacity * sm->nblk * 2 * 8));
    if (sm->popt.save_all_per_patch_scores)
      XR_CUDA_TRY(sm->d_pscores.reserve((size_t)sm->capacity * (size_t)sm->ncr * (size_t)sm->ncc * 4));
    if (sm->mvar_mode) XR_CUDA_TRY(sm->d_mvar_sum.reserve((size_t)sm->capacity * 2 * 8));
  }
  XR_CUDA_TRY(sm->d_sims.reserve((size_t)sm->capacity * 4));
  XR_CUDA_TRY(cudaStreamSynchronize(s));
  sm->allocated = true;
  sm->generation++;
  return XR_OK;
}

static xr_status sm_enqueue_compute_on(xr_simmetric sm, cudaStream_t s);

static xr_status sm_enqueue_compute(xr_simmetric sm) {
  XR_CHECK_ARG(sm, "compute: NULL handle");
  return sm_enqueue_compute_on(sm, sm->stream());
}

// Enqueues the metric's kernels on stream s.
static xr_status sm_enqueue_compute_on(xr_simmetric sm, cudaStream_t s) {
  XR_CHECK_ARG(sm, "compute: NULL handle");
  if (!sm->allocated) return fail(XR_ERR_NOT_ALLOCATED, "compute: allocate_resources has not been called");
  const int64_t npix = sm->rows * sm->cols;
  const float* mov = nullptr;
  if (xr_raycaster rc = sm->live_rc()) {
    XR_CHECK_ARG(rc->allocated, "compute: the bound ray caster has no buffer");
    XR_CHECK_ARG(rc->rows() == sm->rows && rc->cols() == sm->cols,
                 "compute: ray caster image size differs from the fixed image");
    int64_t cap = 0;
    const float* buf = rc_out(rc, &cap);
    XR_CHECK_ARG(sm->proj_offset + sm->num_mov <= cap, "compute: moving images run past the ray caster's buffer");
    mov = buf + sm->proj_offset * npix;
  } else if (sm->mov_host) {
    // ImgSimMetric2DCPU::set_mov_imgs_host_buf: the host images go to the device first
    XR_CUDA_TRY(sm->d_mov_stage.reserve((size_t)(sm->num_mov * npix) * 4));
    XR_CUDA_TRY(cudaMemcpyAsync(sm->d_mov_stage.p, sm->mov_host, (size_t)(sm->num_mov * npix) * 4,
                                cudaMemcpyHostToDevice, s));
    mov = sm->d_mov_stage.as<float>();
  } else {
    XR_CHECK_ARG(sm->mov_dev, "compute: no moving image buffer (was the bound ray caster destroyed?)");
    mov = sm->mov_dev + sm->proj_offset * npix;
  }
  const int rows = (int)sm->rows, cols = (int)sm->cols;
  const uint8_t* mask = sm->has_mask ? sm->d_mask.as<uint8_t>() : nullptr;
  switch (sm->kind) {
    case XR_SIM_NCC:
      XR_CUDA_TRY(launch_ncc_moments(mov, npix, sm->num_mov, sm->fx.fhat, mask, sm->d_partials.as<double>(),
                                     sm->nblk, s));
      XR_CUDA_TRY(launch_ncc_finalize(sm->d_partials.as<double>(), sm->nblk, sm->num_mov, sm->n_used, sm->fx,
                                      sm->d_sims.as<float>(), s));
      break;
    case XR_SIM_GRAD_NCC:
      XR_CUDA_TRY(launch_grad_moments(mov, rows, cols, sm->num_mov, sm->smooth_ksize, sm->fx.fhat, sm->fy.fhat, mask,
                                      sm->d_partials.as<double>(), s, nullptr));
      XR_CUDA_TRY(launch_grad_finalize(sm->d_partials.as<double>(), sm->nblk, sm->num_mov, sm->n_used, sm->fx,
                                       sm->fy, sm->d_sims.as<float>(), s));
      break;
    default: {
      const int grad = sm->kind == XR_SIM_PATCH_GRAD_NCC;
      const xr_patch_options& o = sm->popt;
      PatchFixed px{grad ? sm->d_gx.as<float>() : sm->d_fixed.as<float>(), sm->d_pmean_x.as<float>(),
                    sm->d_pscale_x.as<float>(), sm->has_pw ? sm->d_pw_x.as<float>() : nullptr};
      PatchFixed py{sm->d_gy.as<float>(), sm->d_pmean_y.as<float>(), sm->d_pscale_y.as<float>(),
                    sm->has_pw ? sm->d_pw_y.as<float>() : nullptr};
      PatchRun run{mask, nullptr, o.use_mask_for_patch_stats ? 1 : 0, o.mask_only_for_weights ? 0 : 1,
                   o.weight_patch_sims_in_combine ? 1 : 0,
                   sm->mvar_mode, o.normalize_weights_as_prob ? 1 : 0,
                   sm->mvar_mode ? sm->d_mvar_sum.as<double>() : nullptr};
      if (!sm->user_idx.empty()) {
        run.cnt = sm->d_pcnt.as<int32_t>();  // set_patches_to_use: counted at allocate_resources
      } else if (o.choose_rand_patches) {
        xr_status st = sm_draw_patches(sm, s);
        if (st != XR_OK) return st;
        run.cnt = sm->d_pcnt.as<int32_t>();
      }
      if (o.save_all_per_patch_scores) {
        XR_CUDA_TRY(cudaMemsetAsync(sm->d_pscores.p, 0,
                                    (size_t)sm->num_mov * (size_t)sm->ncr * (size_t)sm->ncc * 4, s));
        run.scores = sm->d_pscores.as<float>();
      }
      if (sm->mvar_mode) {
        int nblk0 = 0;
        XR_CUDA_TRY(launch_patch_ncc(mov, rows, cols, sm->num_mov, grad, sm->smooth_ksize, sm->patch_radius,
                                     sm->patch_stride, sm->ncr, sm->ncc, px, py, run, 0,
                                     sm->d_partials.as<double>(), s, &nblk0));
        XR_CHECK_ARG(nblk0 <= sm->nblk, "compute: patch partials exceed their buffer");
        XR_CUDA_TRY(launch_patch_sum_partials(sm->d_partials.as<double>(), nblk0, sm->num_mov,
                                              sm->d_mvar_sum.as<double>(), s));
      }
      int nblk = 0;
      XR_CUDA_TRY(launch_patch_ncc(mov, rows, cols, sm->num_mov, grad, sm->smooth_ksize, sm->patch_radius,
                                   sm->patch_stride, sm->ncr, sm->ncc, px, py, run, 1, sm->d_partials.as<double>(),
                                   s, &nblk));
      XR_CHECK_ARG(nblk <= sm->nblk, "compute: patch partials exceed their buffer");
      const double den_x = o.compute_mean_of_patch_sims ? (double)sm->nused
                                                        : (o.weight_patch_sims_in_combine ? sm->tot_w_x : 1.0);
      const double den_y = o.compute_mean_of_patch_sims ? (double)sm->nused
                                                        : (o.weight_patch_sims_in_combine ? sm->tot_w_y : 1.0);
      XR_CUDA_TRY(launch_patch_finalize(sm->d_partials.as<double>(), nblk, sm->num_mov, den_x, den_y, grad,
                                        sm->mvar_mode, o.normalize_weights_as_prob ? 1 : 0,
                                        sm->mvar_mode ? sm->d_mvar_sum.as<double>() : nullptr,
                                        sm->d_sims.as<float>(), s));
      break;
    }
  }
  return XR_OK;
}

extern "C" XR_API xr_status xr_sm_compute(xr_simmetric sm) {
  XR_CHECK_ARG(sm, "compute: NULL handle");
  DeviceGuard g(sm->device);
  // A metric reading a ray caster's buffer on another stream waits for it.
  xr_raycaster brc = sm->live_rc();
  if (brc && sm->stream() != brc->stream()) {
    cudaEvent_t ev;
    XR_CUDA_TRY(cudaEventCreateWithFlags(&ev, cudaEventDisableTiming));
    cudaEventRecord(ev, brc->stream());
    cudaStreamWaitEvent(sm->stream(), ev, 0);
    cudaEventDestroy(ev);
  }
  return sm_enqueue_compute(sm);
}

extern "C" XR_API xr_status xr_sm_sim_vals(xr_simmetric sm, float* dst) {
  XR_CHECK_ARG(sm && dst, "sim_vals: NULL argument");
  XR_CHECK_ARG(sm->allocated, "sim_vals: resources not allocated");
  DeviceGuard g(sm->device);
  XR_CUDA_TRY(cudaStreamSynchronize(sm->stream()));
  if (xr_raycaster brc2 = sm->live_rc()) {
    xr_status st = xr_rc_synchronize(brc2);
    if (st != XR_OK) return st;
  }
  XR_CUDA_TRY(cudaMemcpy(dst, sm->d_sims.p, (size_t)sm->num_mov * 4, cudaMemcpyDeviceToHost));
  return XR_OK;
}

extern "C" XR_API xr_status xr_sm_device_sim_vals(xr_simmetric sm, float** out) {
  XR_CHECK_ARG(sm && out, "device_sim_vals: NULL argument");
  XR_CHECK_ARG(sm->allocated, "device_sim_vals: resources not allocated");
  *out = sm->d_sims.as<float>();
  return XR_OK;
}

// ======================================================= population objective
extern "C" XR_API xr_status xr_obj_create(xr_raycaster rc, int32_t vol_idx, int32_t nviews, const xr_simmetric* ms,
                                          int64_t max_pop, xr_objective* out) {
  XR_CHECK_ARG(out, "xr_obj_create: out is NULL");
  *out = nullptr;
  XR_CHECK_ARG(rc && ms && nviews > 0 && nviews <= 16 && max_pop > 0, "xr_obj_create: bad argument");
  XR_CHECK_ARG((int32_t)rc->cams.size() == nviews, "xr_obj_create: the ray caster needs one camera model per view");
  XR_CHECK_ARG(vol_idx >= 0 && vol_idx < (int32_t)rc->vols.size(), "xr_obj_create: bad volume index");
  for (int32_t v = 0; v < nviews; ++v) {
    XR_CHECK_ARG(ms[v] && ms[v]->has_fixed, "xr_obj_create: every view needs a metric with a fixed image");
    XR_CHECK_ARG(ms[v]->rows == rc->rows() && ms[v]->cols == rc->cols(),
                 "xr_obj_create: fixed image size differs from the detector");
  }
  DeviceGuard g(rc->device);
  auto* obj = new (std::nothrow) xr_objective_s();
  if (!obj) return fail(XR_ERR_OUT_OF_MEMORY, "xr_obj_create: host allocation failed");
  obj->rc = rc;
  obj->rc_id = rc->id;
  obj->vol_idx = vol_idx;
  obj->metrics.assign(ms, ms + nviews);
  for (int32_t v = 0; v < nviews; ++v) obj->metric_ids.push_back(ms[v]->id);
  obj->max_pop = max_pop;
  std::unique_ptr<xr_objective_s> guard(obj);
  // ray caster: views * max_pop projections, poses distributed over cameras
  xr_status st = xr_rc_set_num_projs(rc, (int64_t)nviews * max_pop);
  if (st == XR_ERR_INVALID_ARG && rc->allocated) {
    rc->allocated = false;
    st = xr_rc_set_num_projs(rc, (int64_t)nviews * max_pop);
  }
  if (st != XR_OK) return st;
  st = xr_rc_allocate_resources(rc);
  if (st != XR_OK) return st;
  for (int32_t v = 0; v < nviews; ++v) {
    xr_simmetric m = ms[v];
    m->allocated = false;
    if ((st = xr_sm_set_num_moving_images(m, max_pop)) != XR_OK) return st;
    if ((st = xr_sm_set_mov_imgs_buf_from_ray_caster(m, rc, (int64_t)v * max_pop)) != XR_OK) return st;
    m->has_ext_stream = false;  // metrics follow the ray caster's stream inside the objective
    if ((st = xr_sm_allocate_resources(m)) != XR_OK) return st;
  }
  XR_CUDA_TRY(obj->d_poses.reserve((size_t)max_pop * 16 * 8));
  XR_CUDA_TRY(obj->d_sims.reserve((size_t)max_pop * 4));
  obj->id = reg_add(obj);
  *out = guard.release();
  return XR_OK;
}

extern "C" XR_API xr_status xr_obj_destroy(xr_objective obj) {
  if (!obj) return XR_OK;
  reg_remove(obj);
  if (reg_alive(obj->rc, obj->rc_id)) {
    DeviceGuard g(obj->rc->device);
    cudaStreamSynchronize(obj->rc->stream());
    delete obj;
  } else {
    // the ray caster (and its stream) is gone; wait for all device work instead
    cudaDeviceSynchronize();
    delete obj;
  }
  return XR_OK;
}

// ======================================================= fused evaluation
// Whether an objective's metric can run inside the fused evaluation kernel:
// every view grad-NCC with the default 5x5 smoothing, reading its images from
// the objective's ray caster.
static bool obj_metric_fusable(xr_objective obj) {
  for (xr_simmetric m : obj->metrics) {
    if (m->kind != XR_SIM_GRAD_NCC || m->smooth_ksize != 5 || !m->allocated) return false;
    if (m->rows != obj->rc->rows() || m->cols != obj->rc->cols()) return false;
  }
  return true;
}

static size_t align16(size_t n) { return (n + 15) & ~(size_t)15; }

// Kernel launches of one metric compute (sm_enqueue_compute_on).
static int metric_launches(const xr_simmetric_s* m) {
  if (m->kind == XR_SIM_NCC || m->kind == XR_SIM_GRAD_NCC) return 2;
  return 2 + (m->mvar_mode ? 2 : 0) + (m->popt.choose_rand_patches ? 1 : 0);
}

// One evaluation step of n objectives: per job the poses are copied in, then
// ONE geometry launch covers every job's projections; then
//   fused: ONE persistent launch per (voxel type, layout) group traces every
//     DRR tile and computes the grad-NCC of each image behind it
//     (eval_fused_kernel), each job in its autotuned block shape;
//   split: ONE DRR launch per group whose grid covers every job's tiles
//     (drr_jobs_kernel, each job in its autotuned block shape and loop), then
//     ONE batched grad-NCC launch over every job's images
//     (grad_multi_kernel, with the per-image combine and the mean over views).
// Objectives whose metrics are not grad-NCC with 5x5 smoothing get their own
// metric launches afterwards.  Values are copied to sims[i].  Everything is
// ordered on stream s.  Both ways give identical values.
static xr_status step_enqueue(FusedWork& fw, int device, int32_t n, const xr_objective* objs, const int64_t* pops,
                              const double* const* xforms, bool host_in, float* const* sims, bool host_out,
                              cudaStream_t s, bool fused, const CmaStepJob* cma = nullptr, int pose_group = 0) {
  XR_CHECK_ARG(objs && pops && xforms && sims && n > 0, "evaluation: NULL argument or no jobs");
  auto dev_opt = [&](int32_t i) { return cma != nullptr && cma[i].state != nullptr; };
  bool any_dev = false;
  for (int32_t i = 0; i < n; ++i) any_dev = any_dev || dev_opt(i);
  if (any_dev) {
    XR_CUDA_TRY(fw.d_report.reserve((size_t)n * sizeof(CmaReport)));
    XR_CUDA_TRY(cudaMemsetAsync(fw.d_report.p, 0, (size_t)n * sizeof(CmaReport), s));
  }
  CmaReport* d_report = any_dev ? fw.d_report.as<CmaReport>() : nullptr;
  std::vector<CmaUpdateJob> cu;  // device optimizers whose update has a launch of its own
  // how far a job's poses spread, in voxels at the volume (nearby poses: pose-grouped DRR items)
  auto pose_spread_vox = [&](int32_t i, const xr_raycaster_s::Vol& vol, int64_t pop) -> double {
    if (dev_opt(i)) {  // the distribution the device optimizer samples next
      const xr_objective obj = objs[i];
      if (obj->next_sd_state != cma[i].state || !(obj->next_sd_rot >= 0.0)) return INFINITY;
      return sampled_spread_voxels(vol.desc, obj->next_sd_rot, obj->next_sd_trans);
    }
    if (!host_in || pop < 2) return INFINITY;
    return pose_spread_voxels(vol.desc, xforms[i], pop);
  };
  std::vector<GeomJob> gj;
  std::vector<FusedJob> fj;
  std::vector<std::vector<FusedView>> fv((size_t)n);
  std::vector<int32_t> key;
  int64_t first = 0;
  int tuning_launches = 0;  // a shape's first step: geometry for the autotuner's timed launches
  for (int32_t i = 0; i < n; ++i) {
    xr_objective obj = objs[i];
    XR_CHECK_ARG(obj && reg_contains(obj), "evaluation: unknown or destroyed objective");
    XR_CHECK_ARG(obj->peers_alive(), "evaluation: a ray caster or metric of an objective was destroyed");
    XR_CHECK_ARG(obj->rc->device == device, "evaluation: objective lives on another device");
    for (int32_t k = 0; k < i; ++k) XR_CHECK_ARG(objs[k] != obj, "evaluation: an objective is listed twice");
    const int64_t pop = pops[i];
    XR_CHECK_ARG(pop > 0 && pop <= obj->max_pop, "evaluation: population outside [1, max_pop]");
    const bool dopt = dev_opt(i);
    if (dopt) {  // candidates drawn on the device by the geometry launch
      XR_CHECK_ARG(cma[i].lam == pop && cma[i].dim >= 1 && cma[i].dim <= kCmaDeviceMaxDim,
                   "evaluation: a device optimizer's population must be its lambda");
    } else {
      XR_CHECK_ARG(xforms[i] && sims[i], "evaluation: NULL pose or value pointer");
      if (host_in) XR_CHECK_ARG(finite_all(xforms[i], 16 * pop), "evaluation: non-finite transform");
      if (xforms[i] != obj->d_poses.as<double>())
        XR_CUDA_TRY(cudaMemcpyAsync(obj->d_poses.p, xforms[i], (size_t)pop * 16 * 8,
                                    host_in ? cudaMemcpyHostToDevice : cudaMemcpyDeviceToDevice, s));
    }
    xr_raycaster rc = obj->rc;
    const int32_t nv = (int32_t)obj->metrics.size();
    xr_status st = xr_rc_set_num_projs(rc, (int64_t)nv * pop);
    if (st != XR_OK) return st;
    if ((st = rc_distribute_device_on(rc, pop, dopt ? nullptr : obj->d_poses.as<double>(), s)) != XR_OK) return st;
    rc->store = XR_PROJ_STORE_REPLACE;  // use_proj_store_replace_method (xregIntensity2D3DRegi.cpp:598)
    FusedJob J{};
    if ((st = rc_prepare(rc, obj->vol_idx, s, J.d.p, false)) != XR_OK) return st;
    XR_CHECK_ARG(J.d.p.kernel_id == XR_LINE_INT_SUM, "evaluation: the fused step uses the line-integral sum kernel");
    const auto& vol = *rc->vols[(size_t)obj->vol_idx];
    // the ray caster's autotuned layout and block shape; the fused kernel runs
    // the four-sample loop (packed pairs where the tuner chose them); without
    // the macro-cell trim, or with a configuration fixed by the caller that the
    // fused kernel lacks, float32 volumes read their cell copy with one 256-bit
    // load and half volumes with one 128-bit load
    DrrParams& P = J.d.p;
    const bool cells = vol.cells.p != nullptr;
    const int32_t wide = cells ? (vol.type == XR_VOXEL_F32 ? 2 : XR_LAYOUT_CELL8) : XR_LAYOUT_LINEAR;
    // each job in its autotuned block shape and sample loop: the DRR job
    // kernel runs loop 3 (for the tuner's 1 to 3), 4 (4, 5) or the packed 6,
    // the fused kernel loop 4 or 6
    if (!rc_config_cached(rc, vol, P)) {  // the tuner times real launches: this caster's geometry first
      XR_CUDA_TRY(launch_proj_geom(vol.desc, rc->d_cams.as<xr_camera_desc>(), rc->d_xforms.as<double>(),
                                   rc->d_cam_idx.as<int32_t>(), rc->num_projs, rc->pose_count,
                                   rc->d_geo.as<ProjGeom>(), s));
      ++tuning_launches;
    }
    if ((st = rc_choose_config(rc, vol, P, s)) != XR_OK) return st;
    P.unroll = (P.unroll == 6 && cells) ? 6 : (!fused && P.unroll <= 3 ? 3 : 4);
    P.vol.layout = wide;
    const int wc = P.warp_tall ? 4 : 8, tw = wc * P.block_warps_x, th = (8 / P.block_warps_x) * (32 / wc);
    J.d.tiles_x = (int32_t)((P.cols + tw - 1) / tw);
    J.d.tiles_y = (int32_t)((P.rows + th - 1) / th);
    J.d.pose_group = 0;
    // items of 4 projections x 8x8 pixels: every job (mode 2) or those whose poses lie within a voxel (mode 1)
    if (!fused && (pose_group == 2 || (pose_group == 1 && pose_spread_vox(i, vol, pop) < 1.0))) {
      J.d.pose_group = 4;
      J.d.tiles_x = (int32_t)((P.cols + 7) / 8);
      J.d.tiles_y = (int32_t)((P.rows + 7) / 8);
    }
    rc->last_layout = P.vol.layout;
    rc->last_bw = P.block_warps_x;
    rc->last_unroll = P.unroll;
    rc->last_warp_rows = P.warp_tall ? 8 : 4;
    GeomJob G{};
    G.p2i = phys_to_idx_xform(vol.desc);
    G.cams = rc->d_cams.as<xr_camera_desc>();
    G.poses = rc->d_xforms.as<double>();
    G.cam_idx = rc->d_cam_idx.as<int32_t>();
    G.num_projs = rc->num_projs;
    G.pose_stride = rc->pose_count;
    G.first = first;
    G.out = rc->d_geo.as<ProjGeom>();
    if (dopt) {
      G.cma = cma[i].state;
      G.report = d_report + i;
      std::memcpy(G.C, cma[i].C, sizeof(G.C));
      std::memcpy(G.B, cma[i].B, sizeof(G.B));
      std::memcpy(G.bounds, cma[i].bounds, sizeof(G.bounds));
    }
    first += rc->num_projs;
    gj.push_back(G);
    // the metric behind the DRR
    const int rows = (int)rc->rows(), cols = (int)rc->cols();
    J.nviews = nv;
    J.pop = pop;
    J.mt_x = (cols + 31) / 32;
    J.mt_y = (rows + 63) / 64;
    J.out = obj->d_sims.as<float>();
    J.metric = obj_metric_fusable(obj) ? 1 : 0;
    for (int32_t v = 0; v < nv; ++v) {
      xr_simmetric m = obj->metrics[(size_t)v];
      m->num_mov = pop;
      m->rc = rc;
      m->rc_id = rc->id;
      m->proj_offset = (int64_t)v * pop;
      if (J.metric) {
        XR_CHECK_ARG(m->nblk == J.mt_x * J.mt_y && m->capacity >= pop, "evaluation: metric buffers do not fit");
        FusedView V{};
        V.fhx = m->fx.fhat;
        V.fhy = m->fy.fhat;
        V.mask = m->has_mask ? m->d_mask.as<uint8_t>() : nullptr;
        V.fx = m->fx;
        V.fy = m->fy;
        V.n_used = (double)m->n_used;
        V.partials = m->d_partials.as<double>();
        V.sims = m->d_sims.as<float>();
        fv[(size_t)i].push_back(V);
      }
    }
    if (dopt) {
      J.report = d_report + i;
      if (!fused && J.metric) J.cma = cma[i].state;  // updated by the batched grad-NCC launch
      else cu.push_back(CmaUpdateJob{cma[i].state, obj->d_sims.as<float>(), d_report + i});
    }
    if (J.metric) {
      // per metric tile, per image, per pose, and one for the job (its optimizer's update)
      const size_t words = (size_t)obj->max_pop * nv * (size_t)(J.mt_x * J.mt_y + 1) + (size_t)obj->max_pop + 1;
      if (obj->fcnt_words < words) {
        XR_CUDA_TRY(obj->d_fcnt.reserve(words * 4));
        XR_CUDA_TRY(cudaMemsetAsync(obj->d_fcnt.p, 0, words * 4, s));
        obj->fcnt_words = words;
      }
      J.cnt = obj->d_fcnt.as<unsigned int>();
    }
    fj.push_back(J);
    // one launch per (voxel type, layout, pose-grouped or not): the DRR job kernel
    // runs each job's loop, the fused kernel the group's first job's (every loop
    // gives the same bits)
    key.push_back((vol.type * 4 + J.d.p.vol.layout) * 2 + (J.d.pose_group ? 1 : 0));
  }
  // jobs ordered by group; item numbering restarts in each group
  std::vector<int32_t> keys(key);
  std::sort(keys.begin(), keys.end());
  keys.erase(std::unique(keys.begin(), keys.end()), keys.end());
  std::vector<int32_t> order;
  std::vector<std::pair<size_t, size_t>> ranges;
  std::vector<long long> group_items;
  for (int32_t k : keys) {
    const size_t b = order.size();
    long long items = 0;
    for (int32_t i = 0; i < n; ++i)
      if (key[(size_t)i] == k) {
        fj[(size_t)i].d.item_begin = items;
        items += fj[(size_t)i].d.items();
        order.push_back(i);
      }
    ranges.emplace_back(b, order.size());
    group_items.push_back(items);
  }
  // metric tiles of the batched grad-NCC launch, in group order
  long long total_tiles = 0;
  for (int32_t r : order) {
    FusedJob& J = fj[(size_t)r];
    J.tile_begin = total_tiles;
    if (J.metric) total_tiles += (long long)J.nviews * J.pop * J.mt_x * J.mt_y;
  }
  // one descriptor upload: geometry jobs, jobs (group order), their DRR part
  // alone (drr_jobs_kernel's array), views
  const size_t off_f = align16(gj.size() * sizeof(GeomJob));
  const size_t off_m = off_f + align16(fj.size() * sizeof(FusedJob));
  const size_t off_v = off_m + align16(fj.size() * sizeof(MultiJobDrr));
  size_t nviews_total = 0;
  for (auto& v : fv) nviews_total += v.size();
  const size_t off_u = off_v + align16(nviews_total * sizeof(FusedView));
  const size_t bytes = off_u + cu.size() * sizeof(CmaUpdateJob) + 16;
  XR_CUDA_TRY(fw.d_desc.reserve(bytes));
  XR_CUDA_TRY(fw.d_counter.reserve(256));
  fw.h_desc.assign(bytes, 0);
  unsigned char* h = fw.h_desc.data();
  unsigned char* d = fw.d_desc.as<unsigned char>();
  std::memcpy(h, gj.data(), gj.size() * sizeof(GeomJob));
  size_t vpos = 0;
  for (size_t r = 0; r < order.size(); ++r) {
    FusedJob J = fj[(size_t)order[r]];
    const auto& views = fv[(size_t)order[r]];
    J.views = views.empty() ? nullptr : reinterpret_cast<const FusedView*>(d + off_v + vpos * sizeof(FusedView));
    if (!views.empty()) std::memcpy(h + off_v + vpos * sizeof(FusedView), views.data(), views.size() * sizeof(FusedView));
    vpos += views.size();
    std::memcpy(h + off_f + r * sizeof(FusedJob), &J, sizeof(FusedJob));
    std::memcpy(h + off_m + r * sizeof(MultiJobDrr), &J.d, sizeof(MultiJobDrr));
  }
  if (!cu.empty()) std::memcpy(h + off_u, cu.data(), cu.size() * sizeof(CmaUpdateJob));
  XR_CUDA_TRY(cudaMemcpyAsync(fw.d_desc.p, h, bytes, cudaMemcpyHostToDevice, s));
  XR_CUDA_TRY(launch_proj_geom_jobs(reinterpret_cast<const GeomJob*>(d), (int)gj.size(), first, s));
  fw.launches = 1 + tuning_launches;
  fw.pose_grouped = 0;
  for (const FusedJob& f : fj) fw.pose_grouped += f.d.pose_group ? 1 : 0;
  fw.items = 0;
  fw.blocks = 0;
  for (size_t gi = 0; gi < ranges.size(); ++gi) {
    const FusedJob& f0 = fj[(size_t)order[ranges[gi].first]];
    int blocks = 0;
    if (fused)
      XR_CUDA_TRY(launch_eval_fused(reinterpret_cast<const FusedJob*>(d + off_f) + ranges[gi].first,
                                    (int)(ranges[gi].second - ranges[gi].first), group_items[gi],
                                    f0.d.p.vol.voxel_type, f0.d.p.vol.layout, f0.d.p.unroll,
                                    fw.d_counter.as<unsigned long long>(), &blocks, s));
    else {
      XR_CUDA_TRY(launch_drr_jobs(reinterpret_cast<const MultiJobDrr*>(d + off_m) + ranges[gi].first,
                                  (int)(ranges[gi].second - ranges[gi].first), group_items[gi],
                                  f0.d.p.vol.voxel_type, f0.d.p.vol.layout, f0.d.pose_group != 0, s));
      blocks = (int)std::min<long long>(group_items[gi], 0x7fffffff);
    }
    fw.items += group_items[gi];
    fw.blocks = std::max(fw.blocks, blocks);
    ++fw.launches;
  }
  if (!fused && total_tiles > 0) {
    XR_CUDA_TRY(launch_grad_multi(reinterpret_cast<const FusedJob*>(d + off_f), (int)fj.size(), total_tiles, s));
    ++fw.launches;
  }
  for (int32_t i = 0; i < n; ++i) {
    xr_objective obj = objs[i];
    xr_raycaster rc = obj->rc;
    if (rc->ext_host)
      XR_CUDA_TRY(cudaMemcpyAsync(rc->ext_host, rc_out(rc, nullptr),
                                  (size_t)rc->num_projs * (size_t)(rc->rows() * rc->cols()) * 4,
                                  cudaMemcpyDeviceToHost, s));
    if (!fj[(size_t)i].metric) {
      const int32_t nv = (int32_t)obj->metrics.size();
      const float* view_sims[16];
      for (int32_t v = 0; v < nv; ++v) {
        xr_simmetric m = obj->metrics[(size_t)v];
        xr_status st = sm_enqueue_compute_on(m, s);
        if (st != XR_OK) return st;
        view_sims[v] = m->d_sims.as<float>();
      }
      XR_CUDA_TRY(launch_combine_mean(view_sims, nv, pops[i], obj->d_sims.as<float>(), s));
      fw.launches += nv * metric_launches(obj->metrics[0]) + 1;
    }
    if (sims[i] && sims[i] != obj->d_sims.as<float>())
      XR_CUDA_TRY(cudaMemcpyAsync(sims[i], obj->d_sims.p, (size_t)pops[i] * 4,
                                  host_out ? cudaMemcpyDeviceToHost : cudaMemcpyDeviceToDevice, s));
  }
  if (!cu.empty()) {  // device optimizers whose values came from other launches
    XR_CUDA_TRY(launch_cma_updates(reinterpret_cast<const CmaUpdateJob*>(d + off_u), (int)cu.size(), s));
    ++fw.launches;
  }
  return XR_OK;
}

// Enqueues the whole objective for obj->d_poses (pop poses) on the rc stream.
static xr_status obj_enqueue(xr_objective obj, int64_t pop) {
  xr_raycaster rc = obj->rc;
  const int32_t nv = (int32_t)obj->metrics.size();
  xr_status st = xr_rc_set_num_projs(rc, (int64_t)nv * pop);
  if (st != XR_OK) return st;
  if ((st = xr_rc_distribute_xforms_device(rc, pop, obj->d_poses.as<double>())) != XR_OK) return st;
  rc->store = XR_PROJ_STORE_REPLACE;  // use_proj_store_replace_method (xregIntensity2D3DRegi.cpp:598)
  if ((st = rc_enqueue_compute(rc, obj->vol_idx)) != XR_OK) return st;
  const float* view_sims[16];
  for (int32_t v = 0; v < nv; ++v) {
    xr_simmetric m = obj->metrics[(size_t)v];
    m->num_mov = pop;
    m->rc = rc;
    m->rc_id = rc->id;
    m->proj_offset = (int64_t)v * pop;
    if ((st = sm_enqueue_compute(m)) != XR_OK) return st;
    view_sims[v] = m->d_sims.as<float>();
  }
  XR_CUDA_TRY(launch_combine_mean(view_sims, nv, pop, obj->d_sims.as<float>(), rc->stream()));
  return XR_OK;
}

static bool obj_graph_valid(xr_objective obj, int64_t pop) {
  if (!obj->graph_exec || obj->graph_pop != pop || obj->graph_rc_gen != obj->rc->generation ||
      obj->graph_stream != obj->rc->stream())
    return false;
  for (size_t v = 0; v < obj->metrics.size(); ++v)
    if (obj->graph_sm_gen[v] != obj->metrics[v]->generation) return false;
  return true;
}

static xr_status obj_run(xr_objective obj, int64_t pop) {
  xr_raycaster rc = obj->rc;
  cudaStream_t s = rc->stream();
  if (obj->fused && obj_metric_fusable(obj)) {
    const double* x = obj->d_poses.as<double>();
    float* v = obj->d_sims.as<float>();
    return step_enqueue(obj->fw, rc->device, 1, &obj, &pop, &x, false, &v, false, s, true);
  }
  // A metric that draws random patches on the host at every compute, or a copy
  // into an external host buffer, is run directly (a captured graph would replay
  // one draw; pageable copies cannot be captured).
  if (rc->ext_host) return obj_enqueue(obj, pop);
  for (xr_simmetric m : obj->metrics)
    if ((m->kind == XR_SIM_PATCH_NCC || m->kind == XR_SIM_PATCH_GRAD_NCC) && m->popt.choose_rand_patches)
      return obj_enqueue(obj, pop);
  // Host state that the captured kernels read must be current before capture;
  // a first direct run uploads it and settles generations.
  if (obj_graph_valid(obj, pop)) {
    XR_CUDA_TRY(cudaGraphLaunch(obj->graph_exec, s));
    return XR_OK;
  }
  xr_status st = obj_enqueue(obj, pop);
  if (st != XR_OK || s == nullptr) return st;  // the legacy default stream cannot be captured
  // Capture the steady-state sequence for the next calls.
  if (obj->graph_exec) { cudaGraphExecDestroy(obj->graph_exec); obj->graph_exec = nullptr; }
  cudaGraph_t graph = nullptr;
  XR_CUDA_TRY(cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal));
  st = obj_enqueue(obj, pop);
  cudaError_t ce = cudaStreamEndCapture(s, &graph);
  if (st != XR_OK) { if (graph) cudaGraphDestroy(graph); return st; }
  if (ce != cudaSuccess) { if (graph) cudaGraphDestroy(graph); return cuda_fail(ce, "cudaStreamEndCapture"); }
  ce = cudaGraphInstantiate(&obj->graph_exec, graph, 0);
  cudaGraphDestroy(graph);
  if (ce != cudaSuccess) { obj->graph_exec = nullptr; return cuda_fail(ce, "cudaGraphInstantiate"); }
  obj->graph_pop = pop;
  obj->graph_rc_gen = rc->generation;
  obj->graph_stream = s;
  obj->graph_sm_gen.resize(obj->metrics.size());
  for (size_t v = 0; v < obj->metrics.size(); ++v) obj->graph_sm_gen[v] = obj->metrics[v]->generation;
  return XR_OK;
}

extern "C" XR_API xr_status xr_obj_set_fused(xr_objective obj, int32_t enable) {
  XR_CHECK_ARG(obj, "xr_obj_set_fused: NULL handle");
  obj->fused = enable ? 1 : 0;
  return XR_OK;
}

extern "C" XR_API xr_status xr_obj_eval_device(xr_objective obj, int64_t pop, const double* d_xforms,
                                               float* d_sims) {
  XR_CHECK_ARG(obj && d_xforms && d_sims, "xr_obj_eval_device: NULL argument");
  XR_CHECK_ARG(obj->peers_alive(), "xr_obj_eval_device: a ray caster or metric of this objective was destroyed");
  XR_CHECK_ARG(pop > 0 && pop <= obj->max_pop, "xr_obj_eval_device: population outside [1, max_pop]");
  DeviceGuard g(obj->rc->device);
  cudaStream_t s = obj->rc->stream();
  XR_CUDA_TRY(cudaMemcpyAsync(obj->d_poses.p, d_xforms, (size_t)pop * 16 * 8, cudaMemcpyDeviceToDevice, s));
  xr_status st = obj_run(obj, pop);
  if (st != XR_OK) return st;
  XR_CUDA_TRY(cudaMemcpyAsync(d_sims, obj->d_sims.p, (size_t)pop * 4, cudaMemcpyDeviceToDevice, s));
  return XR_OK;
}

extern "C" XR_API xr_status xr_obj_eval(xr_objective obj, int64_t pop, const double* h_xforms, float* h_sims) {
  XR_CHECK_ARG(obj && h_xforms && h_sims, "xr_obj_eval: NULL argument");
  XR_CHECK_ARG(obj->peers_alive(), "xr_obj_eval: a ray caster or metric of this objective was destroyed");
  XR_CHECK_ARG(pop > 0 && pop <= obj->max_pop, "xr_obj_eval: population outside [1, max_pop]");
  XR_CHECK_ARG(finite_all(h_xforms, 16 * pop), "xr_obj_eval: non-finite transform");
  DeviceGuard g(obj->rc->device);
  cudaStream_t s = obj->rc->stream();
  XR_CUDA_TRY(cudaMemcpyAsync(obj->d_poses.p, h_xforms, (size_t)pop * 16 * 8, cudaMemcpyHostToDevice, s));
  xr_status st = obj_run(obj, pop);
  if (st != XR_OK) return st;
  XR_CUDA_TRY(cudaMemcpyAsync(h_sims, obj->d_sims.p, (size_t)pop * 4, cudaMemcpyDeviceToHost, s));
  return xr_rc_synchronize(obj->rc);
}

// ================================================================== job sets
// Several registration objectives evaluated in one step (step_enqueue): every
// job's poses are copied in, ONE geometry launch covers all jobs, ONE DRR
// launch per (voxel type, layout) group covers every job's (tile, projection)
// work items, ONE grad-NCC launch covers every job's images (per-image FP64
// combine and mean over views included), and the values are copied out.
// Everything is ordered on the job set's stream.
struct xr_jobset_s {
  int device = 0;
  cudaStream_t own_stream = nullptr, ext_stream = nullptr;
  bool has_ext = false;
  int blocks = 0;
  long long last_items = 0;
  unsigned int* h_err = nullptr;  // pinned: every job's step-guard flag, read with one synchronisation
  size_t h_err_cap = 0;
  CmaReport* h_report = nullptr;  // pinned: device optimizers' reports of the last step
  size_t h_report_cap = 0;
  // 0 (default): geometry, DRR and batched grad-NCC launches for every job;
  // 1: fused evaluation step
  int32_t step_mode = 0;
  // DRR items of 4 consecutive projections: 0 never, 1 for jobs whose poses
  // lie within a voxel of each other, 2 for every job
  int32_t pose_group = 0;
  FusedWork fw;
  cudaStream_t stream() const { return has_ext ? ext_stream : own_stream; }
};

extern "C" XR_API xr_status xr_jobset_create(int32_t device, xr_jobset* out) {
  XR_CHECK_ARG(out, "xr_jobset_create: out is NULL");
  *out = nullptr;
  int dev = device;
  if (dev < 0) XR_CUDA_TRY(cudaGetDevice(&dev));
  DeviceGuard g(dev);
  auto js = std::make_unique<xr_jobset_s>();
  js->device = dev;
  XR_CUDA_TRY(cudaStreamCreateWithFlags(&js->own_stream, cudaStreamNonBlocking));
  XR_CUDA_TRY(js->fw.d_counter.reserve(256));
  js->blocks = 0;  // sized per launch from the kernel's occupancy
  *out = js.release();
  return XR_OK;
}

extern "C" XR_API xr_status xr_jobset_destroy(xr_jobset js) {
  if (!js) return XR_OK;
  DeviceGuard g(js->device);
  cudaStreamSynchronize(js->stream());
  cudaStreamDestroy(js->own_stream);
  if (js->h_err) cudaFreeHost(js->h_err);
  if (js->h_report) cudaFreeHost(js->h_report);
  delete js;
  return XR_OK;
}

extern "C" XR_API xr_status xr_jobset_set_stream(xr_jobset js, void* s) {
  XR_CHECK_ARG(js, "xr_jobset_set_stream: NULL handle");
  js->ext_stream = static_cast<cudaStream_t>(s);
  js->has_ext = s != nullptr;
  return XR_OK;
}


static xr_status jobset_enqueue(xr_jobset js, int32_t n, const xr_objective* objs, const int64_t* pops,
                                const double* const* xforms, bool host_in, float* const* sims, bool host_out) {
  XR_CHECK_ARG(js && objs && pops && xforms && sims && n > 0, "xr_jobset_eval: NULL argument or no jobs");
  DeviceGuard g(js->device);
  cudaStream_t s = js->stream();
  xr_status st = step_enqueue(js->fw, js->device, n, objs, pops, xforms, host_in, sims, host_out, s,
                              js->step_mode == 1, nullptr, js->pose_group);
  js->last_items = js->fw.items;
  js->blocks = js->fw.blocks;
  return st;
}

// Waits for a step enqueued on the job set's stream (after `extra` copies of
// its own were enqueued) and turns a job's step-guard flag into an error.
static xr_status jobset_finish(xr_jobset js, int32_t n, const xr_objective* objs, const char* who) {
  if (js->h_err_cap < (size_t)n) {
    if (js->h_err) cudaFreeHost(js->h_err);
    js->h_err = nullptr;
    js->h_err_cap = 0;
    XR_CUDA_TRY(cudaMallocHost(&js->h_err, (size_t)n * sizeof(unsigned int)));
    js->h_err_cap = (size_t)n;
  }
  cudaStream_t s = js->stream();
  for (int32_t i = 0; i < n; ++i)
    XR_CUDA_TRY(cudaMemcpyAsync(js->h_err + i, objs[i]->rc->d_counters.as<char>() + 8, sizeof(unsigned int),
                                cudaMemcpyDeviceToHost, s));
  XR_CUDA_TRY(cudaStreamSynchronize(s));
  for (int32_t i = 0; i < n; ++i) {
    xr_raycaster rc = objs[i]->rc;
    if (js->h_err[i]) {
      cudaMemset(rc->d_counters.as<char>() + 8, 0, sizeof(unsigned int));
      return fail(XR_ERR_DEVICE_CHECK, std::string(who) + ": a job's rays exceeded the step-count guard");
    }
  }
  return XR_OK;
}

extern "C" XR_API xr_status xr_jobset_eval(xr_jobset js, int32_t n, const xr_objective* objs, const int64_t* pops,
                                           const double* const* host_xforms, float* const* host_sims) {
  xr_status st = jobset_enqueue(js, n, objs, pops, host_xforms, true, host_sims, true);
  if (st != XR_OK) return st;
  DeviceGuard g(js->device);
  return jobset_finish(js, n, objs, "xr_jobset_eval");
}

namespace xr {
xr_status jobset_step_cma(xr_jobset js, int32_t n, const xr_objective* objs, const int64_t* pops,
                          const double* const* host_xforms, float* const* host_sims, const CmaStepJob* cma,
                          CmaReport* reports) {
  XR_CHECK_ARG(js && objs && pops && host_xforms && host_sims && cma && reports && n > 0,
               "regi_jobset_step: NULL argument or no jobs");
  DeviceGuard g(js->device);
  cudaStream_t s = js->stream();
  bool any_dev = false;
  for (int32_t i = 0; i < n; ++i) {
    if (!cma[i].state) continue;
    any_dev = true;
    void* st_ptr = cma[i].state;
    cudaPointerAttributes pa{};
    XR_CUDA_TRY(cudaPointerGetAttributes(&pa, st_ptr));
    XR_CHECK_ARG(pa.type == cudaMemoryTypeDevice && pa.device == js->device,
                 "regi_jobset_step: a device optimizer lives on another device than the job set");
  }
  xr_status st = step_enqueue(js->fw, js->device, n, objs, pops, host_xforms, true, host_sims, true, s,
                              js->step_mode == 1, cma, js->pose_group);
  js->last_items = js->fw.items;
  js->blocks = js->fw.blocks;
  if (st != XR_OK) return st;
  if (any_dev) {
    if (js->h_report_cap < (size_t)n) {
      if (js->h_report) cudaFreeHost(js->h_report);
      js->h_report = nullptr;
      js->h_report_cap = 0;
      XR_CUDA_TRY(cudaMallocHost(&js->h_report, (size_t)n * sizeof(CmaReport)));
      js->h_report_cap = (size_t)n;
    }
    XR_CUDA_TRY(cudaMemcpyAsync(js->h_report, js->fw.d_report.p, (size_t)n * sizeof(CmaReport),
                                cudaMemcpyDeviceToHost, s));
  }
  if ((st = jobset_finish(js, n, objs, "regi_jobset_step")) != XR_OK) return st;
  for (int32_t i = 0; i < n; ++i) {
    reports[i] = any_dev ? js->h_report[i] : CmaReport{0, 0, -1.0, -1.0};
    if (cma[i].state) {
      objs[i]->next_sd_rot = reports[i].sd_rot;
      objs[i]->next_sd_trans = reports[i].sd_trans;
      objs[i]->next_sd_state = cma[i].state;
    }
  }
  return XR_OK;
}
}  // namespace xr

extern "C" XR_API xr_status xr_jobset_eval_device(xr_jobset js, int32_t n, const xr_objective* objs,
                                                  const int64_t* pops, const double* const* d_xforms,
                                                  float* const* d_sims) {
  return jobset_enqueue(js, n, objs, pops, d_xforms, false, d_sims, false);
}

extern "C" XR_API xr_status xr_jobset_set_fused(xr_jobset js, int32_t enable) {
  XR_CHECK_ARG(js, "xr_jobset_set_fused: NULL handle");
  js->step_mode = enable ? 1 : 0;
  return XR_OK;
}

extern "C" XR_API xr_status xr_jobset_set_pose_groups(xr_jobset js, int32_t mode) {
  XR_CHECK_ARG(js, "xr_jobset_set_pose_groups: NULL handle");
  XR_CHECK_ARG(mode >= 0 && mode <= 2, "xr_jobset_set_pose_groups: mode must be 0, 1 or 2");
  js->pose_group = mode;
  return XR_OK;
}

extern "C" XR_API xr_status xr_jobset_last_pose_grouped(xr_jobset js, int32_t* jobs) {
  XR_CHECK_ARG(js && jobs, "xr_jobset_last_pose_grouped: NULL argument");
  *jobs = js->fw.pose_grouped;
  return XR_OK;
}

extern "C" XR_API xr_status xr_jobset_last_kernel_launches(xr_jobset js, int32_t* launches) {
  XR_CHECK_ARG(js && launches, "xr_jobset_last_kernel_launches: NULL argument");
  *launches = js->fw.launches;
  return XR_OK;
}

extern "C" XR_API xr_status xr_jobset_last_launch(xr_jobset js, int64_t* work_items, int32_t* blocks) {
  XR_CHECK_ARG(js && work_items && blocks, "xr_jobset_last_launch: NULL argument");
  *work_items = js->last_items;
  *blocks = js->blocks;
  return XR_OK;
}
