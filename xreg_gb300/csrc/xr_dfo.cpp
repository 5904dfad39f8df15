// xr_dfo.cpp -- bound-constrained, model-based derivative-free trust-region
// optimizer for the final registration level, where xReg uses NLopt's
// LN_BOBYQA (Intensity2D3DRegiBOBYQA, xregIntensity2D3DRegiBOBYQA.cpp:28-39;
// driven by Intensity2D3DRegiNLOptInterface::run,
// xregIntensity2D3DRegiNLOptInterface.cpp:83-188).
//
// In the spirit of Powell's BOBYQA ("The BOBYQA algorithm for bound constrained
// optimization without derivatives", 2009): quadratic models from 2n+1
// interpolation points around the current best point (x and x -/+ h_i e_i with
// h_i = rho * scale_i: BOBYQA's initial interpolation set; at a bound the pair
// becomes one-sided), a trust-region step of the model restricted to the box,
// a trust radius adapted by the ratio of actual to predicted reduction, and
// rho halved when neither the step nor the model points improve.  It stops when
// rho falls below rho_end or after max_iter iterations.  The model keeps the
// diagonal Hessian that 2n+1 points determine and is rebuilt every iteration.
// Unlike NLopt's serial evaluations each iteration asks for one batch (the
// previous iteration's trial step plus the 2n+1 model points), which a GPU
// evaluates in one launch.
#include <algorithm>
#include <cmath>
#include <cstring>
#include <limits>
#include <new>
#include <string>
#include <vector>

#include "xreg_gb300_regi.h"

namespace xr {
xr_status fail(xr_status code, const std::string& msg);
}
using xr::fail;

struct xr_dfo_s {
  int n = 0;
  std::vector<double> lo, hi, scale;
  std::vector<double> x;         // centre = best point so far
  double fx = std::numeric_limits<double>::infinity();
  bool have_fx = false;
  double rho = 0, rho_end = 0, delta = 0, delta_max = 0;
  int64_t iter = 0, max_iter = 0;
  std::vector<double> trial;     // trial step point (valid if has_trial)
  bool has_trial = false;
  double pred = 0;               // model-predicted reduction of the trial
  double f_at_trial_centre = 0;  // centre value when the trial was made
  std::vector<double> batch;     // last asked rows
  std::vector<double> off_a, off_b;  // offsets of the two model points per coordinate
  int stop = 0;

  double clampc(int i, double v) const { return std::min(hi[(size_t)i], std::max(lo[(size_t)i], v)); }
};

extern "C" XR_API xr_status xr_dfo_create(int32_t dim, const double* x0, const double* lower, const double* upper,
                                          double rho_beg, double rho_end, int64_t max_iter, xr_dfo* out) {
  if (!out || !x0 || !lower || !upper) return fail(XR_ERR_INVALID_ARG, "xr_dfo_create: NULL argument");
  *out = nullptr;
  if (dim < 1 || dim > 64) return fail(XR_ERR_INVALID_ARG, "xr_dfo_create: dimension must be in [1, 64]");
  if (!(rho_beg > 0) || !(rho_end > 0) || rho_end > rho_beg)
    return fail(XR_ERR_INVALID_ARG, "xr_dfo_create: need 0 < rho_end <= rho_beg");
  double smax = 0;
  for (int i = 0; i < dim; ++i) {
    if (!(upper[i] > lower[i]) || !(x0[i] >= lower[i] && x0[i] <= upper[i]))
      return fail(XR_ERR_INVALID_ARG, "xr_dfo_create: need lower < upper and x0 inside the bounds");
    smax = std::max(smax, upper[i] - lower[i]);
  }
  auto* d = new (std::nothrow) xr_dfo_s();
  if (!d) return fail(XR_ERR_OUT_OF_MEMORY, "xr_dfo_create: host allocation failed");
  d->n = dim;
  d->lo.assign(lower, lower + dim);
  d->hi.assign(upper, upper + dim);
  for (int i = 0; i < dim; ++i) d->scale.push_back((upper[i] - lower[i]) / smax);
  d->x.assign(x0, x0 + dim);
  d->rho = rho_beg;
  d->rho_end = rho_end;
  // rho and delta are measured in the units of the coordinate with the widest
  // bounds; coordinate i uses them scaled by its width / the widest width.
  d->delta = rho_beg;
  d->delta_max = 0.5 * smax;
  d->max_iter = max_iter;
  d->off_a.assign((size_t)dim, 0.0);
  d->off_b.assign((size_t)dim, 0.0);
  *out = d;
  return XR_OK;
}

extern "C" XR_API xr_status xr_dfo_destroy(xr_dfo d) {
  delete d;
  return XR_OK;
}

// Next batch: [trial step] + centre + 2 model points per coordinate.
extern "C" XR_API xr_status xr_dfo_ask(xr_dfo d, double* pts, int32_t* count) {
  if (!d || !pts || !count) return fail(XR_ERR_INVALID_ARG, "xr_dfo_ask: NULL argument");
  const int n = d->n;
  d->batch.clear();
  if (d->has_trial) d->batch.insert(d->batch.end(), d->trial.begin(), d->trial.end());
  d->batch.insert(d->batch.end(), d->x.begin(), d->x.end());
  for (int i = 0; i < n; ++i) {
    const double h = d->rho * d->scale[(size_t)i];
    const double xi = d->x[(size_t)i];
    double a = -h, b = h;
    if (xi + h > d->hi[(size_t)i]) { a = -2.0 * h; b = -h; }       // one-sided below
    else if (xi - h < d->lo[(size_t)i]) { a = h; b = 2.0 * h; }    // one-sided above
    d->off_a[(size_t)i] = d->clampc(i, xi + a) - xi;
    d->off_b[(size_t)i] = d->clampc(i, xi + b) - xi;
    for (double o : {d->off_a[(size_t)i], d->off_b[(size_t)i]}) {
      std::vector<double> p = d->x;
      p[(size_t)i] = xi + o;
      d->batch.insert(d->batch.end(), p.begin(), p.end());
    }
  }
  std::memcpy(pts, d->batch.data(), d->batch.size() * sizeof(double));
  *count = (int32_t)(d->batch.size() / (size_t)n);
  return XR_OK;
}

extern "C" XR_API xr_status xr_dfo_tell(xr_dfo d, const double* f) {
  if (!d || !f) return fail(XR_ERR_INVALID_ARG, "xr_dfo_tell: NULL argument");
  if (d->batch.empty()) return fail(XR_ERR_INVALID_ARG, "xr_dfo_tell: ask for a batch first");
  const int n = d->n;
  const int rows = (int)(d->batch.size() / (size_t)n);
  int r0 = 0;
  double f_trial = std::numeric_limits<double>::infinity();
  if (d->has_trial) f_trial = f[r0++];
  const double f0 = f[r0];
  const std::vector<double> xc = d->x;  // centre the model is built around
  // diagonal quadratic model q(t e_i) = f0 + g_i t + h_i t^2 / 2 through the
  // centre and the two points on coordinate i
  std::vector<double> g((size_t)n), hdiag((size_t)n);
  for (int i = 0; i < n; ++i) {
    const double a = d->off_a[(size_t)i], b = d->off_b[(size_t)i];
    const double da = f[r0 + 1 + 2 * i] - f0, db = f[r0 + 2 + 2 * i] - f0;
    if (a != 0.0 && b != 0.0 && a != b) {
      g[(size_t)i] = (da * b * b - db * a * a) / (a * b * (b - a));
      hdiag[(size_t)i] = 2.0 * (da * b - db * a) / (a * b * (a - b));
    } else {
      g[(size_t)i] = 0.0;
      hdiag[(size_t)i] = 0.0;
    }
  }
  // trust radius from the trial's actual / predicted reduction
  bool improved = false;
  if (d->has_trial) {
    const double actual = d->f_at_trial_centre - f_trial;
    const double ratio = d->pred > 0 ? actual / d->pred : -1.0;
    if (ratio > 0.75) d->delta = std::min(2.0 * d->delta, d->delta_max);
    else if (ratio < 0.1) d->delta = std::max(0.5 * d->delta, d->rho);
  }
  // new centre: best point of the batch (ties keep the earlier row)
  int best = r0;
  for (int r = 0; r < rows; ++r)
    if (f[r] < f[best]) best = r;
  if (!d->have_fx || f[best] < d->fx) {
    improved = d->have_fx && f[best] < d->fx - 1e-15 * std::fabs(d->fx);
    d->fx = f[best];
    d->x.assign(d->batch.begin() + (size_t)best * n, d->batch.begin() + (size_t)(best + 1) * n);
  }
  d->have_fx = true;
  if (!improved && d->iter > 0) {
    d->rho *= 0.5;
    d->delta = std::max(0.5 * d->delta, d->rho);
  }
  // trial step of the model from the (possibly moved) centre, inside the box
  std::vector<double> s((size_t)n);
  double gs = 0.0, shs = 0.0;
  for (int i = 0; i < n; ++i) {
    const double gi = g[(size_t)i] + hdiag[(size_t)i] * (d->x[(size_t)i] - xc[(size_t)i]);
    const double rad = d->delta * d->scale[(size_t)i];
    double si = (hdiag[(size_t)i] > 0.0) ? -gi / hdiag[(size_t)i] : (gi > 0 ? -rad : (gi < 0 ? rad : 0.0));
    si = std::max(-rad, std::min(rad, si));
    si = d->clampc(i, d->x[(size_t)i] + si) - d->x[(size_t)i];
    s[(size_t)i] = si;
    gs += gi * si;
    shs += hdiag[(size_t)i] * si * si;
  }
  d->pred = -(gs + 0.5 * shs);
  d->has_trial = d->pred > 0.0;
  if (d->has_trial) {
    d->trial = d->x;
    for (int i = 0; i < n; ++i) d->trial[(size_t)i] += s[(size_t)i];
    d->f_at_trial_centre = d->fx;
  }
  d->iter++;
  d->batch.clear();
  if (d->rho < d->rho_end) d->stop = 2;
  else if (d->iter >= d->max_iter) d->stop = 3;
  return XR_OK;
}

// *reason: 0 continue, 2 rho below rho_end, 3 iteration limit.
extern "C" XR_API xr_status xr_dfo_test_termination(xr_dfo d, int32_t* reason) {
  if (!d || !reason) return fail(XR_ERR_INVALID_ARG, "xr_dfo_test_termination: NULL argument");
  *reason = d->stop;
  return XR_OK;
}

extern "C" XR_API xr_status xr_dfo_get(xr_dfo d, double* best_x, double* best_f, double* rho, int64_t* iterations) {
  if (!d) return fail(XR_ERR_INVALID_ARG, "xr_dfo_get: NULL handle");
  if (best_x) std::memcpy(best_x, d->x.data(), (size_t)d->n * sizeof(double));
  if (best_f) *best_f = d->fx;
  if (rho) *rho = d->rho;
  if (iterations) *iterations = d->iter;
  return XR_OK;
}
