// Drives the header-only C++ host classes (include/xreg_gb300/xreg_gb300.hpp)
// the way xReg's Intensity2D3DRegi::setup / obj_fn drive a ray caster and its
// metrics.  Reads raw inputs written by tests/test_gpu_cpp_host.py, writes the
// DRRs and similarity values for comparison with the oracle.
//   usage: host_api_check <dir>
#include <cstdio>
#include <cstdlib>
#include <fstream>
#include <iostream>
#include <string>
#include <vector>

#include "xreg_gb300/xreg_gb300.hpp"
#include "xreg_gb300/xreg_gb300_regi.hpp"

template <typename T>
static std::vector<T> read_all(const std::string& path) {
  std::ifstream f(path, std::ios::binary);
  f.seekg(0, std::ios::end);
  const size_t n = (size_t)f.tellg() / sizeof(T);
  f.seekg(0);
  std::vector<T> v(n);
  f.read(reinterpret_cast<char*>(v.data()), (std::streamsize)(n * sizeof(T)));
  return v;
}

template <typename T>
static void write_all(const std::string& path, const std::vector<T>& v) {
  std::ofstream f(path, std::ios::binary);
  f.write(reinterpret_cast<const char*>(v.data()), (std::streamsize)(v.size() * sizeof(T)));
}

int main(int argc, char** argv) {
  if (argc < 2) return 2;
  const std::string dir = argv[1];
  const auto meta = read_all<double>(dir + "/meta.f64");  // nx ny nz sp rows cols px step npose
  const int64_t nx = (int64_t)meta[0], ny = (int64_t)meta[1], nz = (int64_t)meta[2];
  const double sp = meta[3];
  const int64_t rows = (int64_t)meta[4], cols = (int64_t)meta[5];
  const double px = meta[6];
  const float step = (float)meta[7];
  const int64_t npose = (int64_t)meta[8];
  auto vox = read_all<float>(dir + "/vol.f32");
  auto poses_raw = read_all<double>(dir + "/poses.f64");
  auto fixed = read_all<float>(dir + "/fixed.f32");
  try {
    using namespace xreg_gb300;
    Volume vol;
    vol.desc.n[0] = nx; vol.desc.n[1] = ny; vol.desc.n[2] = nz;
    for (int i = 0; i < 3; ++i) { vol.desc.spacing[i] = sp; vol.desc.origin[i] = 0.0; }
    for (int i = 0; i < 9; ++i) vol.desc.direction[i] = (i % 4 == 0) ? 1.0 : 0.0;
    vol.voxels = vox.data();
    CameraModel cam;
    cam.setup(1020.0, rows, cols, px, px);
    std::vector<Mat4> poses((size_t)npose);
    for (int64_t p = 0; p < npose; ++p)
      for (int k = 0; k < 16; ++k) poses[(size_t)p][(size_t)k] = poses_raw[(size_t)(p * 16 + k)];

    // ray caster used directly (RayCaster API)
    RayCasterLineIntCUDA rc;
    rc.set_volume(vol);
    rc.set_camera_model(cam);
    rc.set_ray_step_size(step);
    rc.set_num_projs(npose);
    rc.allocate_resources();
    rc.use_proj_store_replace_method();
    rc.distribute_xforms_among_cam_models(poses);
    rc.compute(0);
    write_all(dir + "/drr.f32", rc.raw_host_pixel_buf());

    // metric reading the ray caster's buffer in place
    ImgSimMetric2DGradNCCCUDA m;
    m.set_fixed_image(fixed.data(), rows, cols);
    m.set_num_moving_images(npose);
    m.set_mov_imgs_buf_from_ray_caster(&rc, 0);
    m.allocate_resources();
    m.compute();
    write_all(dir + "/sims.f32", m.sim_vals());

    // masked patch NCC with moving-image patch variances as weights
    auto mask = read_all<uint8_t>(dir + "/mask.u8");
    ImgSimMetric2DPatchNCCCUDA pm;
    pm.set_fixed_image(fixed.data(), rows, cols);
    pm.set_mask(mask.data());
    pm.set_patch_radius(3);
    pm.set_patch_stride(2);
    pm.set_use_mov_img_patch_variances_as_wgts(true);
    pm.set_num_moving_images(npose);
    pm.set_mov_imgs_buf_from_ray_caster(&rc, 0);
    pm.allocate_resources();
    pm.compute();
    write_all(dir + "/psims.f32", pm.sim_vals());

    // the population objective over a second ray caster
    RayCasterLineIntCUDA rc2;
    rc2.set_volume(vol);
    rc2.set_camera_model(cam);
    rc2.set_ray_step_size(step);
    ImgSimMetric2DGradNCCCUDA m2;
    m2.set_fixed_image(fixed.data(), rows, cols);
    PopulationObjective obj(rc2, {&m2}, npose);
    write_all(dir + "/obj.f32", obj(poses));

    // SimpleRayCasterWrapperFn about an intermediate frame (F, R from frames.f64)
    const auto fr = read_all<double>(dir + "/frames.f64");
    Mat4 F{}, R{};
    for (int k = 0; k < 16; ++k) { F[(size_t)k] = fr[(size_t)k]; R[(size_t)k] = fr[(size_t)(16 + k)]; }
    SimpleRayCasterWrapperFn wrap;
    wrap.ray_caster = &rc2;
    wrap.cam_world_to_vols = {poses[0]};
    wrap.inter_frames = {F};
    wrap.inter_frames_wrt_vol = {true};
    wrap.ref_frames_cam_world_to_vol = {R};
    wrap();
    write_all(dir + "/wrap.f32", wrap.projs[0]);

    // a CMA-ES level run in the library, and the same level stepped one
    // generation at a time through a job set (xreg_gb300_regi.hpp)
    {
      RayCasterLineIntCUDA rc3;
      rc3.set_volume(vol);
      rc3.set_camera_model(cam);
      rc3.set_ray_step_size(step);
      ImgSimMetric2DGradNCCCUDA m3;
      m3.set_fixed_image(fixed.data(), rows, cols);
      PopulationObjective obj3(rc3, {&m3}, 8);
      xr_regi_level_params lp = DefaultLevelParams(XR_REGI_CMAES);
      lp.lambda = 8;
      lp.max_iters = 6;
      lp.seed = 11;
      Mat4 centre{};
      for (int i = 0; i < 4; ++i) centre[(size_t)(i * 5)] = 1.0;
      centre[3] = 0.5 * sp * (double)nx;
      centre[7] = 0.5 * sp * (double)ny;
      centre[11] = 0.5 * sp * (double)nz;
      const LevelResult a = RunLevel(obj3, centre, poses[0], lp);
      CMAES es(6, std::vector<double>(6, 0.0), std::vector<double>(lp.sigma, lp.sigma + 6), lp.lambda, lp.seed);
      es.set_stop(lp.tol_fun, lp.tol_x, lp.max_iters);
      JobSet js;
      int32_t reason = 0, gens = 0;
      while (reason == 0 && gens < 100) {
        const auto r = js.regi_step({StepJob(obj3, es, centre, poses[0], lp.bounds)});
        if (r.second[0] != lp.lambda) throw Error(XR_ERR_INVALID_ARG, "regi_step: wrong evaluation count");
        reason = r.first[0];
        ++gens;
      }
      // the same level with the optimizer's state on the device: sampled and
      // updated inside the step's launches, the same state block at the end
      CMAES es_dev(6, std::vector<double>(6, 0.0), std::vector<double>(lp.sigma, lp.sigma + 6), lp.lambda, lp.seed);
      es_dev.set_stop(lp.tol_fun, lp.tol_x, lp.max_iters);
      es_dev.attach_device();
      int32_t reason_dev = 0, gens_dev = 0;
      while (reason_dev == 0 && gens_dev < 100) {
        reason_dev = js.regi_step({StepJob(obj3, es_dev, centre, poses[0], lp.bounds)}).first[0];
        ++gens_dev;
      }
      if (js.last_kernel_launches() != 3) throw Error(XR_ERR_INVALID_ARG, "regi_step: expected 3 launches");
      es_dev.detach_device();
      if (gens_dev != gens || reason_dev != reason || es_dev.export_state() != es.export_state())
        throw Error(XR_ERR_INVALID_ARG, "device CMA-ES state differs from the host optimizer's");
      // again with pose-grouped DRR items for the generations whose samples lie within a voxel
      CMAES es_pg(6, std::vector<double>(6, 0.0), std::vector<double>(lp.sigma, lp.sigma + 6), lp.lambda, lp.seed);
      es_pg.set_stop(lp.tol_fun, lp.tol_x, lp.max_iters);
      es_pg.attach_device();
      js.set_pose_groups(1);
      int32_t reason_pg = 0, gens_pg = 0, grouped = 0;
      while (reason_pg == 0 && gens_pg < 100) {
        reason_pg = js.regi_step({StepJob(obj3, es_pg, centre, poses[0], lp.bounds)}).first[0];
        grouped += js.last_pose_grouped();
        ++gens_pg;
      }
      js.set_pose_groups(0);
      es_pg.detach_device();
      if (gens_pg != gens || reason_pg != reason || es_pg.export_state() != es.export_state())
        throw Error(XR_ERR_INVALID_ARG, "pose-grouped items changed the device optimizer's run");
      std::printf("pose-grouped generations: %d of %d\n", grouped, gens_pg);
      double bf = 0.0;
      int64_t g = 0;
      const Mat4 b = RegiPoseMap(centre, poses[0], es.best_x(&bf, &g))[0];
      std::vector<double> lv(a.pose.begin(), a.pose.end());
      lv.insert(lv.end(), b.begin(), b.end());
      lv.insert(lv.end(), {a.value, bf, (double)a.iterations, (double)g, (double)a.stop_reason, (double)reason});
      write_all(dir + "/levels.f64", lv);
    }

    // a pose through an ITK text transform file and back
    WriteITKAffineTransform(dir + "/pose.txt", poses[1]);
    const Mat4 back = ReadITKAffineTransformFromFile(dir + "/pose.txt");
    write_all(dir + "/pose_back.f64", std::vector<double>(back.begin(), back.end()));

    // error path: unsupported interpolation surfaces as UnsupportedOperationException
    rc.set_interp_method(XR_INTERP_SINC);
    try {
      rc.compute(0);
      std::cerr << "expected UnsupportedOperationException\n";
      return 3;
    } catch (const UnsupportedOperationException&) {
    }
  } catch (const std::exception& e) {
    std::cerr << "error: " << e.what() << "\n";
    return 1;
  }
  std::cout << "ok\n";
  return 0;
}
