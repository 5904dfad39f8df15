/*
 * cmaes_ref_shim.c -- flat C entry points over the reference's vendored CMA-ES
 * (xReg third_party/cmaes/cmaes.c, N. Hansen), compiled together with it into
 * oracle/_ref/libcmaes_ref.so.  TEST INFRASTRUCTURE ONLY: the tests use it as the
 * checker for the product's CMA-ES.  It sets the parameters the way
 * Intensity2D3DRegiCMAES::run does (xregIntensity2D3DRegiCMAES.cpp:116-127):
 * cmaes_init with the "non" parameter file, then stopTolFun / stopTolX.
 */
#include <stdlib.h>
#include <string.h>

#include "cmaes_interface.h"

void* xo_cmaes_new(int n, const double* x0, const double* sd, long seed, int lambda, double tol_fun, double tol_x,
                   double max_iter) {
  cmaes_t* t = (cmaes_t*)calloc(1, sizeof(cmaes_t));
  if (!t) return NULL;
  cmaes_init(t, n, (double*)x0, (double*)sd, seed, lambda, "non");
  t->sp.stopTolFun = tol_fun;
  t->sp.stopTolX = tol_x;
  t->sp.stopMaxIter = max_iter;
  return t;
}

void xo_cmaes_sample(void* h, double* out) {
  cmaes_t* t = (cmaes_t*)h;
  double* const* pop = cmaes_SamplePopulation(t);
  const int n = (int)cmaes_Get(t, "dimension"), lam = (int)cmaes_Get(t, "lambda");
  for (int k = 0; k < lam; ++k) memcpy(out + (size_t)k * n, pop[k], sizeof(double) * (size_t)n);
}

void xo_cmaes_update(void* h, const double* f) { cmaes_UpdateDistribution((cmaes_t*)h, f); }

int xo_cmaes_stop(void* h) { return cmaes_TestForTermination((cmaes_t*)h) != NULL; }

void xo_cmaes_mean(void* h, double* out) {
  cmaes_t* t = (cmaes_t*)h;
  const int n = (int)cmaes_Get(t, "dimension");
  memcpy(out, cmaes_GetPtr(t, "xmean"), sizeof(double) * (size_t)n);
}

double xo_cmaes_generation(void* h) { return cmaes_Get((cmaes_t*)h, "generation"); }

void xo_cmaes_free(void* h) {
  cmaes_exit((cmaes_t*)h);
  free(h);
}
