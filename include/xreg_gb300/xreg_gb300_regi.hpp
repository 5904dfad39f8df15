// xreg_gb300_regi.hpp -- header-only C++ classes over the registration C ABI
// (xreg_gb300_regi.h): the CMA-ES and trust-region optimizers a level of
// Intensity2D3DRegiCMAES / Intensity2D3DRegiBOBYQA drives, one level run in the
// library, and job sets that evaluate (or step) many registrations with one
// DRR launch.  Errors come back as xreg_gb300::Error, as in xreg_gb300.hpp.
#ifndef XREG_GB300_REGI_HPP_
#define XREG_GB300_REGI_HPP_

#include <utility>
#include <vector>

#include "../xreg_gb300_regi.h"
#include "xreg_gb300.hpp"

namespace xreg_gb300 {

// cmaes_init / cmaes_SamplePopulation / cmaes_ReSampleSingle /
// cmaes_UpdateDistribution / cmaes_TestForTermination as
// Intensity2D3DRegiCMAES::run calls them (xregIntensity2D3DRegiCMAES.cpp:122-224).
class CMAES {
 public:
  CMAES(int32_t dim, const std::vector<double>& xstart, const std::vector<double>& stddevs, int32_t lambda,
        uint64_t seed)
      : dim_(dim) {
    if ((int32_t)xstart.size() != dim || (int32_t)stddevs.size() != dim)
      throw Error(XR_ERR_INVALID_ARG, "CMAES: xstart and stddevs need dim entries");
    check(xr_cmaes_create(dim, xstart.data(), stddevs.data(), lambda, seed, &h_));
  }
  ~CMAES() { xr_cmaes_destroy(h_); }
  CMAES(const CMAES&) = delete;
  CMAES& operator=(const CMAES&) = delete;
  void set_stop(double tol_fun, double tol_x, int64_t max_iter) { check(xr_cmaes_set_stop(h_, tol_fun, tol_x, max_iter)); }
  int32_t lambda() const {
    int32_t l = 0;
    check(xr_cmaes_lambda(h_, &l));
    return l;
  }
  // lambda x dim candidates, row-major
  std::vector<double> sample_population() {
    std::vector<double> pop((size_t)lambda() * (size_t)dim_);
    check(xr_cmaes_sample_population(h_, pop.data()));
    return pop;
  }
  void resample_single(int32_t k, std::vector<double>& pop) { check(xr_cmaes_resample_single(h_, k, pop.data())); }
  void update_distribution(const std::vector<double>& fvals) {
    if ((int32_t)fvals.size() != lambda()) throw Error(XR_ERR_INVALID_ARG, "CMAES: one value per candidate");
    check(xr_cmaes_update_distribution(h_, fvals.data()));
  }
  // 0 continue, 1 tol_fun, 2 tol_x, 3 iteration limit, 4 numerical failure
  int32_t test_for_termination() {
    int32_t r = 0;
    check(xr_cmaes_test_termination(h_, &r));
    return r;
  }
  std::vector<double> best_x(double* best_f = nullptr, int64_t* generation = nullptr) const {
    std::vector<double> x((size_t)dim_);
    check(xr_cmaes_get(h_, nullptr, x.data(), best_f, nullptr, generation));
    return x;
  }
  // The state to device memory: JobSet::regi_step then samples and updates it
  // inside the step's launches (same bits as the host methods, which refuse
  // while it is attached); detach_device brings it back.
  void attach_device(int32_t device = -1) { check(xr_cmaes_attach_device(h_, device)); }
  void detach_device() { check(xr_cmaes_detach_device(h_)); }
  // The whole state block (parameters, distribution, last population).
  std::vector<unsigned char> export_state() const {
    int64_t n = 0;
    check(xr_cmaes_state_bytes(h_, &n));
    std::vector<unsigned char> b((size_t)n);
    check(xr_cmaes_export_state(h_, b.data(), n));
    return b;
  }
  xr_cmaes handle() const { return h_; }

 private:
  int32_t dim_;
  xr_cmaes h_ = nullptr;
};

// The bound-constrained trust-region optimizer in LN_BOBYQA's level
// (xregIntensity2D3DRegiNLOptInterface.cpp:83-188): Powell's BOBYQA method,
// the 2n+1 initial points then one point per ask (set_batch for more).
class TrustRegionDFO {
 public:
  TrustRegionDFO(int32_t dim, const std::vector<double>& x0, const std::vector<double>& lower,
                 const std::vector<double>& upper, double rho_beg, double rho_end, int64_t max_iter)
      : dim_(dim) {
    if ((int32_t)x0.size() != dim || (int32_t)lower.size() != dim || (int32_t)upper.size() != dim)
      throw Error(XR_ERR_INVALID_ARG, "TrustRegionDFO: x0, lower and upper need dim entries");
    check(xr_dfo_create(dim, x0.data(), lower.data(), upper.data(), rho_beg, rho_end, max_iter, &h_));
  }
  ~TrustRegionDFO() { xr_dfo_destroy(h_); }
  TrustRegionDFO(const TrustRegionDFO&) = delete;
  TrustRegionDFO& operator=(const TrustRegionDFO&) = delete;
  // count x dim points, row-major
  std::vector<double> ask() {
    std::vector<double> pts((size_t)(2 * dim_ + 2) * (size_t)dim_);
    int32_t n = 0;
    check(xr_dfo_ask(h_, pts.data(), &n));
    pts.resize((size_t)n * (size_t)dim_);
    return pts;
  }
  void tell(const std::vector<double>& fvals) { check(xr_dfo_tell(h_, fvals.data())); }
  // points per ask after the initial set (before the first tell)
  void set_batch(int32_t points) { check(xr_dfo_set_batch(h_, points)); }
  int64_t evaluations() const {
    int64_t n = 0;
    check(xr_dfo_evaluations(h_, &n));
    return n;
  }
  // 0 continue, 2 rho reached rho_end, 3 evaluation limit
  int32_t test_for_termination() {
    int32_t r = 0;
    check(xr_dfo_test_termination(h_, &r));
    return r;
  }
  std::vector<double> best_x(double* best_f = nullptr, int64_t* iterations = nullptr) const {
    std::vector<double> x((size_t)dim_);
    check(xr_dfo_get(h_, x.data(), best_f, nullptr, iterations));
    return x;
  }
  xr_dfo handle() const { return h_; }

 private:
  int32_t dim_;
  xr_dfo h_ = nullptr;
};

// pose = centre * ExpSE3(x) * centre^-1 * start for each row x (6 values) of xs.
inline std::vector<Mat4> RegiPoseMap(const Mat4& centre, const Mat4& start, const std::vector<double>& xs) {
  if (xs.size() % 6) throw Error(XR_ERR_INVALID_ARG, "RegiPoseMap: rows of six parameters");
  std::vector<Mat4> out(xs.size() / 6);
  check(xr_regi_pose_map(centre.data(), start.data(), (int64_t)out.size(), xs.data(),
                         out.empty() ? nullptr : out[0].data()));
  return out;
}

inline xr_regi_level_params DefaultLevelParams(int32_t optimizer) {
  xr_regi_level_params p{};
  check(xr_regi_level_params_default(optimizer, &p));
  return p;
}

struct LevelResult {
  Mat4 pose{};
  double value = 0.0;
  int64_t iterations = 0;
  int32_t stop_reason = 0;
};

// One level of Intensity2D3DRegiCMAES::run (or the trust-region level) in the library.
inline LevelResult RunLevel(PopulationObjective& obj, const Mat4& centre, const Mat4& start,
                            const xr_regi_level_params& params) {
  LevelResult r;
  check(xr_regi_run_level(obj.handle(), centre.data(), start.data(), &params, r.pose.data(), &r.value,
                          &r.iterations, &r.stop_reason));
  return r;
}

// One generation of a CMA-ES level of a registration, for JobSet::regi_step.
inline xr_regi_step_job StepJob(PopulationObjective& obj, CMAES& es, const Mat4& centre, const Mat4& start,
                                const double* bounds = nullptr) {
  xr_regi_step_job j{};
  j.obj = obj.handle();
  j.optimizer = XR_REGI_CMAES;
  j.opt = es.handle();
  for (int k = 0; k < 16; ++k) { j.centre[k] = centre[(size_t)k]; j.start_pose[k] = start[(size_t)k]; }
  for (int k = 0; k < 6; ++k) j.bounds[k] = bounds ? bounds[k] : 0.0;
  return j;
}

// One iteration of a trust-region level of a registration, for JobSet::regi_step.
inline xr_regi_step_job StepJob(PopulationObjective& obj, TrustRegionDFO& d, const Mat4& centre, const Mat4& start) {
  xr_regi_step_job j{};
  j.obj = obj.handle();
  j.optimizer = XR_REGI_DFO;
  j.opt = d.handle();
  for (int k = 0; k < 16; ++k) { j.centre[k] = centre[(size_t)k]; j.start_pose[k] = start[(size_t)k]; }
  return j;
}

// Many registrations' populations in one step: geometry, DRR and grad-NCC
// launches over every job (xr_jobset_*).
class JobSet {
 public:
  explicit JobSet(int32_t device = -1) { check(xr_jobset_create(device, &h_)); }
  ~JobSet() { xr_jobset_destroy(h_); }
  JobSet(const JobSet&) = delete;
  JobSet& operator=(const JobSet&) = delete;
  void set_stream(void* cuda_stream) { check(xr_jobset_set_stream(h_, cuda_stream)); }
  // the fused DRR + grad-NCC step instead of the split one (identical values)
  void set_fused(bool enable) { check(xr_jobset_set_fused(h_, enable ? 1 : 0)); }
  // DRR items of 4 consecutive projections: 0 never, 1 tight populations, 2 every job (identical values)
  void set_pose_groups(int32_t mode) { check(xr_jobset_set_pose_groups(h_, mode)); }
  int32_t last_kernel_launches() const {
    int32_t n = 0;
    check(xr_jobset_last_kernel_launches(h_, &n));
    return n;
  }
  int32_t last_pose_grouped() const {
    int32_t n = 0;
    check(xr_jobset_last_pose_grouped(h_, &n));
    return n;
  }
  // values[i][k] for pose k of objs[i]; every objective listed at most once
  std::vector<std::vector<float>> eval(const std::vector<PopulationObjective*>& objs,
                                       const std::vector<std::vector<Mat4>>& poses) {
    if (objs.size() != poses.size()) throw Error(XR_ERR_INVALID_ARG, "JobSet::eval: one pose list per objective");
    std::vector<xr_objective> hs;
    std::vector<int64_t> pops;
    std::vector<const double*> xp;
    std::vector<std::vector<float>> out(objs.size());
    std::vector<float*> vp;
    for (size_t i = 0; i < objs.size(); ++i) {
      if (poses[i].empty()) throw Error(XR_ERR_INVALID_ARG, "JobSet::eval: an empty population");
      hs.push_back(objs[i]->handle());
      pops.push_back((int64_t)poses[i].size());
      xp.push_back(poses[i][0].data());
      out[i].resize(poses[i].size());
      vp.push_back(out[i].data());
    }
    check(xr_jobset_eval(h_, (int32_t)hs.size(), hs.data(), pops.data(), xp.data(), vp.data()));
    return out;
  }
  // One generation of every job; returns (termination code, poses evaluated) per job.
  std::pair<std::vector<int32_t>, std::vector<int32_t>> regi_step(const std::vector<xr_regi_step_job>& jobs) {
    std::vector<int32_t> stop(jobs.size()), evaluated(jobs.size());
    check(xr_regi_jobset_step(h_, (int32_t)jobs.size(), jobs.data(), stop.data(), evaluated.data()));
    return {stop, evaluated};
  }
  xr_jobset handle() const { return h_; }

 private:
  xr_jobset h_ = nullptr;
};

}  // namespace xreg_gb300

#endif
