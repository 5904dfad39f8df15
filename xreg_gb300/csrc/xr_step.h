// xr_step.h -- the interface between the registration step (xr_regi.cpp,
// xr_cmaes.cpp) and the job-set evaluation (xr_capi.cu).  Plain C++ types only.
#pragma once

#include <cstdint>

#include "xreg_gb300_regi.h"

namespace xr {

// Parameters a CMA-ES state on the device may have (the device draws keep a
// candidate in registers).
constexpr int kCmaDeviceMaxDim = 8;
// Redraws of one candidate before sampling inside the bounds is given up (as
// the host loop of xr_regi_jobset_step).
constexpr int kCmaMaxRedraws = 100000;

// A job whose CMA-ES state lives in device memory: the step's geometry launch
// draws its candidates (redrawing those outside the bounds) and maps them to
// poses, and its update runs on the device after its values.
struct CmaStepJob {
  void* state = nullptr;  // device state block (xr_cmaes_core.h layout); nullptr: poses come from the caller
  double C[16] = {};      // pose(x) = C Exp(x) B
  double B[16] = {};
  double bounds[kCmaDeviceMaxDim] = {};  // |x_i| <= bounds[i], 0 = free
  int32_t lam = 0, dim = 0;
};

// What a device-optimizer step reports per job.
struct CmaReport {
  int32_t reason;        // xr_cmaes_test_termination's code after the update
  int32_t sample_error;  // 1: a candidate stayed outside the bounds after kCmaMaxRedraws redraws
  double sd_rot, sd_trans;  // largest sigma sqrt(C_ii) of the rotation / translation parameters after the update
};

// The device state of an attached optimizer (false when its state is on the host).
bool cmaes_device_state(xr_cmaes e, void** d_state, int32_t* lambda, int32_t* dim, int32_t* device);

// One job-set step: jobs with cma[i].state == nullptr take host poses
// (host_xforms[i]) and return host values (host_sims[i]) as xr_jobset_eval;
// the others are sampled, evaluated and updated on the device, and reports[i]
// receives their outcome.  Waits for the step.
xr_status jobset_step_cma(xr_jobset js, int32_t n, const xr_objective* objs, const int64_t* pops,
                          const double* const* host_xforms, float* const* host_sims, const CmaStepJob* cma,
                          CmaReport* reports);

}  // namespace xr
