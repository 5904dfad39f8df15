// xr_regi.cpp -- one registration level run natively over a population
// objective: the loop of Intensity2D3DRegiCMAES::run
// (xregIntensity2D3DRegiCMAES.cpp:76-247: sample lambda Lie-algebra offsets,
// redraw the out-of-bounds ones, evaluate the population, update, test for
// termination) or of the bound-constrained trust-region level that takes NLopt
// LN_BOBYQA's place (Intensity2D3DRegiNLOptInterface::run,
// xregIntensity2D3DRegiNLOptInterface.cpp:83-188), with every population
// evaluated in one xr_obj_eval call.
//
// A candidate offset x = [w, v] (SE3OptVarsLieAlg, xregSE3OptVars.cpp:128-137)
// maps to the pose  centre * ExpSE3(x) * centre^-1 * start  (the intermediate
// frame about the volume centre that xReg's pre/post transforms apply,
// xregIntensity2D3DRegi.cpp:1028-1099); ExpSE3 (xregRigidUtils.cpp:40-85):
// theta = |w|, R = I + a W + b W^2, t = (I + b W + c W^2) v with a = sin(theta)/theta,
// b = (1 - cos(theta))/theta^2, c = (theta - sin(theta))/theta^3 (R = I, t = v
// for theta <= 1e-14).
#include <cmath>
#include <cstring>
#include <string>
#include <vector>

#include "xr_cmaes_core.h"
#include "xr_step.h"
#include "xreg_gb300.h"
#include "xreg_gb300_regi.h"

namespace xr {
xr_status fail(xr_status code, const std::string& msg);
}  // namespace xr

namespace {

// pose(x) = C Exp(x) B with B = C^-1 start (the shared host/device map of
// xr_cmaes_core.h, so host and device candidates give the same poses)
struct PoseMap {
  double C[16], B[16];
  PoseMap(const double* centre, const double* start) {
    std::memcpy(C, centre, sizeof(C));
    double Ci[16];
    xr::pose::rigid_inverse(centre, Ci);
    xr::pose::mat_mul4(Ci, start, B);
  }
  void operator()(const double* x, double* out) const { xr::pose::map(C, B, x, out); }
};

bool finite6(const double* v) {
  for (int i = 0; i < 6; ++i)
    if (!std::isfinite(v[i])) return false;
  return true;
}

}  // namespace

using namespace xr;

extern "C" XR_API xr_status xr_regi_level_params_default(int32_t optimizer, xr_regi_level_params* out) {
  if (!out) return fail(XR_ERR_INVALID_ARG, "xr_regi_level_params_default: NULL argument");
  if (optimizer != XR_REGI_CMAES && optimizer != XR_REGI_DFO)
    return fail(XR_ERR_INVALID_ARG, "xr_regi_level_params_default: unknown optimizer");
  xr_regi_level_params p{};
  p.optimizer = optimizer;
  p.lambda = 50;
  const double deg = 3.14159265358979323846 / 180.0;
  for (int i = 0; i < 3; ++i) {
    p.sigma[i] = 10.0 * deg;
    p.sigma[i + 3] = 20.0;
  }
  if (optimizer == XR_REGI_DFO) {
    for (int i = 0; i < 3; ++i) p.bounds[i] = 2.5 * deg;
    p.bounds[3] = 5.0;
    p.bounds[4] = 5.0;
    p.bounds[5] = 10.0;
    p.max_iters = 100;
  } else {
    p.max_iters = 100;
  }
  p.tol_fun = 1.0e-6;
  p.tol_x = 1.0e-6;
  p.rho_beg = 2.0;
  p.rho_end = 0.01;
  p.seed = 0;
  *out = p;
  return XR_OK;
}

extern "C" XR_API xr_status xr_regi_run_level(xr_objective obj, const double* centre, const double* start_pose,
                                             const xr_regi_level_params* p, double* best_pose, double* best_value,
                                             int64_t* iterations, int32_t* stop_reason) {
  if (!obj || !centre || !start_pose || !p || !best_pose)
    return fail(XR_ERR_INVALID_ARG, "xr_regi_run_level: NULL argument");
  if (p->max_iters <= 0) return fail(XR_ERR_INVALID_ARG, "xr_regi_run_level: max_iters must be positive");
  const PoseMap map(centre, start_pose);
  const double zero[6] = {0, 0, 0, 0, 0, 0};
  std::vector<double> poses, pop;
  std::vector<float> sims;
  std::vector<double> f;
  double bx[6] = {0}, bf = 0.0;
  int64_t iters = 0;
  int32_t reason = 0;
  xr_status st = XR_OK;
  auto eval = [&](const double* xs, int32_t n) -> xr_status {
    poses.resize((size_t)n * 16);
    sims.resize((size_t)n);
    f.resize((size_t)n);
    for (int32_t k = 0; k < n; ++k) map(xs + (size_t)k * 6, poses.data() + (size_t)k * 16);
    xr_status e = xr_obj_eval(obj, n, poses.data(), sims.data());
    if (e != XR_OK) return e;
    for (int32_t k = 0; k < n; ++k) f[(size_t)k] = (double)sims[(size_t)k];
    return XR_OK;
  };
  if (p->optimizer == XR_REGI_CMAES) {
    if (p->lambda < 2) return fail(XR_ERR_INVALID_ARG, "xr_regi_run_level: lambda must be at least 2");
    xr_cmaes es = nullptr;
    if ((st = xr_cmaes_create(6, zero, p->sigma, p->lambda, p->seed, &es)) != XR_OK) return st;
    if ((st = xr_cmaes_set_stop(es, p->tol_fun, p->tol_x, p->max_iters)) != XR_OK) { xr_cmaes_destroy(es); return st; }
    pop.resize((size_t)p->lambda * 6);
    bool bounded = false;
    for (int i = 0; i < 6; ++i) bounded = bounded || p->bounds[i] > 0.0;
    while (st == XR_OK) {
      if ((st = xr_cmaes_sample_population(es, pop.data())) != XR_OK) break;
      // redraw candidates outside [-b, b] (xregIntensity2D3DRegiCMAES.cpp:162-191)
      for (int32_t k = 0; bounded && k < p->lambda && st == XR_OK; ++k) {
        for (int tries = 0;; ++tries) {
          bool inside = true;
          for (int i = 0; i < 6; ++i)
            if (p->bounds[i] > 0.0 && std::fabs(pop[(size_t)k * 6 + i]) > p->bounds[i]) inside = false;
          if (inside) break;
          if (tries > 100000) {
            st = fail(XR_ERR_INVALID_ARG, "xr_regi_run_level: could not sample a candidate inside the bounds");
            break;
          }
          if ((st = xr_cmaes_resample_single(es, k, pop.data())) != XR_OK) break;
        }
      }
      if (st != XR_OK) break;
      if ((st = eval(pop.data(), p->lambda)) != XR_OK) break;
      if ((st = xr_cmaes_update_distribution(es, f.data())) != XR_OK) break;
      if ((st = xr_cmaes_test_termination(es, &reason)) != XR_OK) break;
      if (reason != 0) break;
    }
    if (st == XR_OK) st = xr_cmaes_get(es, nullptr, bx, &bf, nullptr, &iters);
    xr_cmaes_destroy(es);
  } else if (p->optimizer == XR_REGI_DFO) {
    double lo[6], hi[6];
    for (int i = 0; i < 6; ++i) {
      if (!(p->bounds[i] > 0.0)) return fail(XR_ERR_INVALID_ARG, "xr_regi_run_level: the trust-region level needs bounds");
      lo[i] = -p->bounds[i];
      hi[i] = p->bounds[i];
    }
    xr_dfo d = nullptr;
    if ((st = xr_dfo_create(6, zero, lo, hi, p->rho_beg, p->rho_end, p->max_iters, &d)) != XR_OK) return st;
    pop.resize((size_t)(2 * 6 + 2) * 6);
    while (st == XR_OK) {
      int32_t n = 0;
      if ((st = xr_dfo_ask(d, pop.data(), &n)) != XR_OK) break;
      if ((st = eval(pop.data(), n)) != XR_OK) break;
      if ((st = xr_dfo_tell(d, f.data())) != XR_OK) break;
      if ((st = xr_dfo_test_termination(d, &reason)) != XR_OK) break;
      if (reason != 0) break;
    }
    if (st == XR_OK) st = xr_dfo_get(d, bx, &bf, nullptr, &iters);
    xr_dfo_destroy(d);
  } else {
    return fail(XR_ERR_INVALID_ARG, "xr_regi_run_level: unknown optimizer");
  }
  if (st != XR_OK) return st;
  if (!finite6(bx)) return fail(XR_ERR_INVALID_ARG, "xr_regi_run_level: the optimizer returned a non-finite offset");
  map(bx, best_pose);
  if (best_value) *best_value = bf;
  if (iterations) *iterations = iters;
  if (stop_reason) *stop_reason = reason;
  return XR_OK;
}

extern "C" XR_API xr_status xr_regi_pose_map(const double* centre, const double* start_pose, int64_t n,
                                             const double* xs, double* poses) {
  if (!centre || !start_pose || n < 0 || (n > 0 && (!xs || !poses)))
    return fail(XR_ERR_INVALID_ARG, "regi_pose_map: NULL argument or negative count");
  const PoseMap map(centre, start_pose);
  for (int64_t k = 0; k < n; ++k) map(xs + k * 6, poses + k * 16);
  return XR_OK;
}

extern "C" XR_API xr_status xr_regi_jobset_step(xr_jobset js, int32_t n, const xr_regi_step_job* jobs, int32_t* stop,
                                                int32_t* evaluated) {
  if (!js || !jobs || !stop || n <= 0) return fail(XR_ERR_INVALID_ARG, "regi_jobset_step: NULL argument or no job");
  std::vector<std::vector<double>> xs((size_t)n), poses((size_t)n);
  std::vector<std::vector<float>> vals((size_t)n);
  std::vector<xr_objective> objs((size_t)n);
  std::vector<int64_t> pops((size_t)n);
  std::vector<const double*> pp((size_t)n);
  std::vector<float*> vp((size_t)n);
  std::vector<CmaStepJob> cj((size_t)n);
  std::vector<CmaReport> reports((size_t)n);
  xr_status st = XR_OK;
  // sample (or ask) every host optimizer's candidates and map them to poses;
  // an optimizer attached to the device samples inside the step
  for (int32_t j = 0; j < n; ++j) {
    const xr_regi_step_job& J = jobs[j];
    if (!J.obj || !J.opt) return fail(XR_ERR_INVALID_ARG, "regi_jobset_step: job without objective or optimizer");
    objs[(size_t)j] = J.obj;
    int32_t pop = 0;
    if (J.optimizer == XR_REGI_CMAES) {
      xr_cmaes es = static_cast<xr_cmaes>(J.opt);
      int32_t lam = 0, dim = 0, dev = 0;
      void* d_state = nullptr;
      if (cmaes_device_state(es, &d_state, &lam, &dim, &dev)) {
        if (dim != 6) return fail(XR_ERR_INVALID_ARG, "regi_jobset_step: a pose optimizer has 6 parameters");
        CmaStepJob& c = cj[(size_t)j];
        const PoseMap map(J.centre, J.start_pose);
        c.state = d_state;
        std::memcpy(c.C, map.C, sizeof(c.C));
        std::memcpy(c.B, map.B, sizeof(c.B));
        for (int i = 0; i < 6; ++i) c.bounds[i] = J.bounds[i];
        c.lam = lam;
        c.dim = dim;
        pops[(size_t)j] = lam;
        continue;
      }
      if ((st = xr_cmaes_lambda(es, &lam)) != XR_OK) return st;
      pop = lam;
      xs[(size_t)j].resize((size_t)pop * 6);
      double* x = xs[(size_t)j].data();
      if ((st = xr_cmaes_sample_population(es, x)) != XR_OK) return st;
      bool bounded = false;
      for (int i = 0; i < 6; ++i) bounded = bounded || J.bounds[i] > 0.0;
      for (int32_t k = 0; bounded && k < pop; ++k) {
        for (int tries = 0;; ++tries) {
          if (cma::inside(x + (size_t)k * 6, J.bounds, 6)) break;
          if (tries > kCmaMaxRedraws)
            return fail(XR_ERR_INVALID_ARG, "regi_jobset_step: could not sample a candidate inside the bounds");
          if ((st = xr_cmaes_resample_single(es, k, x)) != XR_OK) return st;
        }
      }
    } else if (J.optimizer == XR_REGI_DFO) {
      xs[(size_t)j].resize((size_t)(2 * 6 + 2) * 6);
      if ((st = xr_dfo_ask(static_cast<xr_dfo>(J.opt), xs[(size_t)j].data(), &pop)) != XR_OK) return st;
    } else {
      return fail(XR_ERR_INVALID_ARG, "regi_jobset_step: unknown optimizer");
    }
    const PoseMap map(J.centre, J.start_pose);
    poses[(size_t)j].resize((size_t)pop * 16);
    for (int32_t k = 0; k < pop; ++k)
      map(xs[(size_t)j].data() + (size_t)k * 6, poses[(size_t)j].data() + (size_t)k * 16);
    vals[(size_t)j].resize((size_t)pop);
    pops[(size_t)j] = pop;
    pp[(size_t)j] = poses[(size_t)j].data();
    vp[(size_t)j] = vals[(size_t)j].data();
  }
  if ((st = jobset_step_cma(js, n, objs.data(), pops.data(), pp.data(), vp.data(), cj.data(), reports.data())) !=
      XR_OK)
    return st;
  // update every host optimizer and test it for termination; a device
  // optimizer was updated inside the step
  for (int32_t j = 0; j < n; ++j) {
    const xr_regi_step_job& J = jobs[j];
    int32_t reason = 0;
    if (cj[(size_t)j].state) {
      if (reports[(size_t)j].sample_error)
        return fail(XR_ERR_INVALID_ARG, "regi_jobset_step: could not sample a candidate inside the bounds");
      reason = reports[(size_t)j].reason;
    } else if (J.optimizer == XR_REGI_CMAES) {
      std::vector<double> f(vals[(size_t)j].begin(), vals[(size_t)j].end());
      xr_cmaes es = static_cast<xr_cmaes>(J.opt);
      if ((st = xr_cmaes_update_distribution(es, f.data())) != XR_OK) return st;
      if ((st = xr_cmaes_test_termination(es, &reason)) != XR_OK) return st;
    } else {
      std::vector<double> f(vals[(size_t)j].begin(), vals[(size_t)j].end());
      xr_dfo d = static_cast<xr_dfo>(J.opt);
      if ((st = xr_dfo_tell(d, f.data())) != XR_OK) return st;
      if ((st = xr_dfo_test_termination(d, &reason)) != XR_OK) return st;
    }
    stop[j] = reason;
    if (evaluated) evaluated[j] = (int32_t)pops[(size_t)j];
  }
  return XR_OK;
}
