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

/* CMA-ES state (host, double precision).  Replaces the vendored cmaes.c calls in
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
/* Current mean, best candidate seen and its value, step size, generation count
 * (any pointer may be NULL). */
XR_API xr_status xr_cmaes_get(xr_cmaes e, double* mean, double* best_x, double* best_f, double* sigma,
                              int64_t* generation);

#ifdef __cplusplus
}
#endif

#endif
