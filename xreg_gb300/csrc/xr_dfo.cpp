// xr_dfo.cpp -- bound-constrained derivative-free trust-region optimizer for
// the final registration level, where xReg uses NLopt's LN_BOBYQA
// (Intensity2D3DRegiBOBYQA, xregIntensity2D3DRegiBOBYQA.cpp:28-39; driven by
// Intensity2D3DRegiNLOptInterface::run, xregIntensity2D3DRegiNLOptInterface.cpp:83-188,
// at most 1 + 2n + max_iters evaluations).
//
// The method of M. J. D. Powell, "The BOBYQA algorithm for bound constrained
// optimization without derivatives" (Cambridge NA report 2009/06):
//   * a full quadratic model Q interpolating m = 2n+1 points; the first set is
//     x0 and x0 +- rho_beg e_i (one-sided at a bound, x0 + rho e_i and
//     x0 + 2 rho e_i), evaluated as one batch;
//   * each later point replaces one interpolation point, and Q changes by the
//     quadratic of least Frobenius norm of its Hessian change that
//     interpolates the new values (Powell's KKT system
//     [A Y^T; Y 0] [lambda; c; g] = [r; 0], A_ij = (y_i . y_j)^2 / 2, the
//     Hessian change sum_j lambda_j y_j y_j^T), so curvature across
//     coordinates is kept from iteration to iteration;
//   * a trust-region step minimises Q in the box and the ball (truncated
//     conjugate gradients, variables that reach a bound are fixed, as TRSBOX);
//   * the replaced point maximises |Lagrange function at the new point| times
//     a distance weight; a geometry step moves a far interpolation point to
//     where its Lagrange function is large in modulus (as ALTMOV, over the
//     lines to the other points and the Lagrange gradient, inside the box);
//   * the trust radius follows the ratio of actual to predicted reduction,
//     and rho shrinks (to rho_end, by sqrt(rho rho_end) or by 10, Powell's
//     schedule) once the steps are short and the points close.
// Differences kept on purpose: the KKT system is solved afresh (with the
// displacements rescaled to unit size) instead of updating its inverse, and
// the base point moves to every new best point; variables are scaled by their
// bound widths (rho is in the units of the widest coordinate).  One point is
// asked per iteration, as NLopt evaluates; xr_dfo_set_batch(k) asks the
// trust-region step with k-1 geometry points of the farthest interpolation
// points, which a GPU evaluates in the same launch.
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

namespace {

// Inverse of the N x N matrix a (row-major) by Gauss-Jordan elimination with
// partial pivoting; false if it is numerically singular.
bool invert(int N, std::vector<double> a, std::vector<double>& inv) {
  inv.assign((size_t)N * N, 0.0);
  for (int i = 0; i < N; ++i) inv[(size_t)i * N + i] = 1.0;
  for (int col = 0; col < N; ++col) {
    int piv = col;
    for (int r = col + 1; r < N; ++r)
      if (std::fabs(a[(size_t)r * N + col]) > std::fabs(a[(size_t)piv * N + col])) piv = r;
    const double p = a[(size_t)piv * N + col];
    if (!(std::fabs(p) > 1e-300) || !std::isfinite(p)) return false;
    if (piv != col)
      for (int k = 0; k < N; ++k) {
        std::swap(a[(size_t)piv * N + k], a[(size_t)col * N + k]);
        std::swap(inv[(size_t)piv * N + k], inv[(size_t)col * N + k]);
      }
    const double ip = 1.0 / p;
    for (int k = 0; k < N; ++k) {
      a[(size_t)col * N + k] *= ip;
      inv[(size_t)col * N + k] *= ip;
    }
    for (int r = 0; r < N; ++r) {
      if (r == col) continue;
      const double f = a[(size_t)r * N + col];
      if (f == 0.0) continue;
      for (int k = 0; k < N; ++k) {
        a[(size_t)r * N + k] -= f * a[(size_t)col * N + k];
        inv[(size_t)r * N + k] -= f * inv[(size_t)col * N + k];
      }
    }
  }
  return true;
}

double dot(const double* a, const double* b, int n) {
  double s = 0.0;
  for (int i = 0; i < n; ++i) s += a[i] * b[i];
  return s;
}

enum Kind { kInit = 0, kTrust = 1, kGeometry = 2 };

}  // namespace

struct xr_dfo_s {
  int n = 0, m = 0;
  std::vector<double> scale;  // caller coordinate = u * scale
  std::vector<double> sl, su; // bounds in u
  std::vector<double> x0;     // base point (u), kept at the best point
  std::vector<double> Y;      // m x n displacements of the interpolation points from x0
  std::vector<double> F;      // their values
  double c = 0.0;             // model Q(x0 + d) = c + g.d + d.H.d / 2
  std::vector<double> g, H;
  int kopt = 0;
  double rho = 0, rho_end = 0, delta = 0;
  int64_t nf = 0, max_eval = 0, iter = 0;
  int stop = 0;
  int batch = 1;
  bool initialised = false;
  // Lagrange functions of the current set: the inverse of the scaled KKT
  // matrix (sigma: the displacement scale it was built with)
  std::vector<double> Winv;
  double sigma = 1.0;
  // points asked and not yet told (absolute, u)
  std::vector<double> pend;
  std::vector<int> pend_kind, pend_t;
  double pred = 0.0, dnorm = 0.0;
  double fx_best = std::numeric_limits<double>::infinity();
  std::vector<double> x_best;  // u

  int N() const { return m + n + 1; }
  double* y(int t) { return Y.data() + (size_t)t * n; }

  // Q(x0 + d) - c
  double model_change(const double* d) const {
    double s = dot(g.data(), d, n);
    for (int i = 0; i < n; ++i) s += 0.5 * d[i] * dot(H.data() + (size_t)i * n, d, n);
    return s;
  }

  // inverse of the KKT matrix of the current set (displacements / sigma)
  bool factor() {
    double smax = 0.0;
    for (int t = 0; t < m; ++t) smax = std::max(smax, std::sqrt(dot(y(t), y(t), n)));
    sigma = smax > 0.0 ? smax : 1.0;
    const int NN = N();
    std::vector<double> W((size_t)NN * NN, 0.0), yh((size_t)m * n);
    for (int t = 0; t < m; ++t)
      for (int i = 0; i < n; ++i) yh[(size_t)t * n + i] = Y[(size_t)t * n + i] / sigma;
    for (int i = 0; i < m; ++i) {
      for (int j = 0; j < m; ++j) {
        const double p = dot(yh.data() + (size_t)i * n, yh.data() + (size_t)j * n, n);
        W[(size_t)i * NN + j] = 0.5 * p * p;
      }
      W[(size_t)i * NN + m] = W[(size_t)m * NN + i] = 1.0;
      for (int k = 0; k < n; ++k)
        W[(size_t)i * NN + m + 1 + k] = W[(size_t)(m + 1 + k) * NN + i] = yh[(size_t)i * n + k];
    }
    return invert(NN, W, Winv);
  }

  // Lagrange function t at x0 + d
  double lagrange(int t, const double* d) const {
    const int NN = N();
    const double* z = Winv.data() + (size_t)t * NN;  // symmetric: row t = column t
    double v = z[m];
    for (int k = 0; k < n; ++k) v += z[m + 1 + k] * d[k] / sigma;
    for (int j = 0; j < m; ++j) {
      double p = 0.0;
      for (int k = 0; k < n; ++k) p += Y[(size_t)j * n + k] * d[k];
      p /= sigma * sigma;
      v += 0.5 * z[j] * p * p;
    }
    return v;
  }

  // gradient (at x0) and Hessian of Lagrange function t
  void lagrange_derivs(int t, std::vector<double>& gl, std::vector<double>& Hl) const {
    const int NN = N();
    const double* z = Winv.data() + (size_t)t * NN;
    gl.assign((size_t)n, 0.0);
    Hl.assign((size_t)n * n, 0.0);
    for (int k = 0; k < n; ++k) gl[(size_t)k] = z[m + 1 + k] / sigma;
    const double s4 = sigma * sigma * sigma * sigma;
    for (int j = 0; j < m; ++j) {
      const double lj = z[j] / s4;
      const double* yj = Y.data() + (size_t)j * n;
      for (int a = 0; a < n; ++a)
        for (int b = 0; b < n; ++b) Hl[(size_t)a * n + b] += lj * yj[a] * yj[b];
    }
  }

  // least-Frobenius-norm model change that makes Q interpolate F
  void update_model() {
    const int NN = N();
    std::vector<double> r((size_t)m);
    for (int t = 0; t < m; ++t) r[(size_t)t] = F[(size_t)t] - (c + model_change(Y.data() + (size_t)t * n));
    std::vector<double> z((size_t)NN, 0.0);
    for (int i = 0; i < NN; ++i) {
      double s = 0.0;
      for (int t = 0; t < m; ++t) s += Winv[(size_t)i * NN + t] * r[(size_t)t];
      z[(size_t)i] = s;
    }
    c += z[(size_t)m];
    for (int k = 0; k < n; ++k) g[(size_t)k] += z[(size_t)(m + 1 + k)] / sigma;
    const double s4 = sigma * sigma * sigma * sigma;
    for (int j = 0; j < m; ++j) {
      const double lj = z[(size_t)j] / s4;
      const double* yj = Y.data() + (size_t)j * n;
      for (int a = 0; a < n; ++a)
        for (int b = 0; b < n; ++b) H[(size_t)a * n + b] += lj * yj[a] * yj[b];
    }
  }

  // moves the base point to interpolation point t (the model is re-expanded)
  void shift_to(int t) {
    std::vector<double> s(y(t), y(t) + n);
    if (dot(s.data(), s.data(), n) == 0.0) return;
    c += model_change(s.data());
    for (int a = 0; a < n; ++a) g[(size_t)a] += dot(H.data() + (size_t)a * n, s.data(), n);
    for (int j = 0; j < m; ++j)
      for (int k = 0; k < n; ++k) Y[(size_t)j * n + k] -= s[(size_t)k];
    for (int k = 0; k < n; ++k) x0[(size_t)k] += s[(size_t)k];
    for (int k = 0; k < n; ++k) Y[(size_t)t * n + k] = 0.0;  // exactly the base point
  }

  double dist_to_opt(int t) const {
    double s = 0.0;
    for (int k = 0; k < n; ++k) {
      const double v = Y[(size_t)t * n + k] - Y[(size_t)kopt * n + k];
      s += v * v;
    }
    return std::sqrt(s);
  }

  // Trust-region step from the best point (= x0): truncated conjugate
  // gradients on Q in the ball of radius delta and the box, fixing variables
  // that reach a bound.
  void trust_step(std::vector<double>& d) {
    d.assign((size_t)n, 0.0);
    std::vector<double> r(g), p((size_t)n, 0.0), Hp((size_t)n);
    std::vector<char> fixed((size_t)n, 0);
    for (int i = 0; i < n; ++i) {
      const double lo = sl[(size_t)i] - x0[(size_t)i], hi = su[(size_t)i] - x0[(size_t)i];
      if ((lo >= 0.0 && r[(size_t)i] > 0.0) || (hi <= 0.0 && r[(size_t)i] < 0.0)) fixed[(size_t)i] = 1;
    }
    bool restart = true;
    double rr_old = 0.0;
    const double g0 = std::sqrt(dot(g.data(), g.data(), n));
    for (int it = 0; it < 3 * n + 3; ++it) {
      double rr = 0.0;
      for (int i = 0; i < n; ++i)
        if (!fixed[(size_t)i]) rr += r[(size_t)i] * r[(size_t)i];
      if (rr <= 1e-24 * g0 * g0 || rr == 0.0) break;
      if (restart) {
        for (int i = 0; i < n; ++i) p[(size_t)i] = fixed[(size_t)i] ? 0.0 : -r[(size_t)i];
        restart = false;
      } else {
        const double beta = rr / rr_old;
        for (int i = 0; i < n; ++i) p[(size_t)i] = fixed[(size_t)i] ? 0.0 : -r[(size_t)i] + beta * p[(size_t)i];
      }
      rr_old = rr;
      for (int a = 0; a < n; ++a) Hp[(size_t)a] = dot(H.data() + (size_t)a * n, p.data(), n);
      const double pHp = dot(p.data(), Hp.data(), n);
      // to the ball's boundary
      const double pp = dot(p.data(), p.data(), n), dp = dot(d.data(), p.data(), n), dd = dot(d.data(), d.data(), n);
      if (pp <= 0.0) break;
      const double disc = std::max(0.0, dp * dp + pp * (delta * delta - dd));
      const double a_tr = (std::sqrt(disc) - dp) / pp;
      // to the first bound
      double a_bd = std::numeric_limits<double>::infinity();
      int ibd = -1;
      for (int i = 0; i < n; ++i) {
        if (fixed[(size_t)i] || p[(size_t)i] == 0.0) continue;
        const double lim = p[(size_t)i] > 0.0 ? su[(size_t)i] - x0[(size_t)i] - d[(size_t)i]
                                              : sl[(size_t)i] - x0[(size_t)i] - d[(size_t)i];
        const double a = std::max(0.0, lim / p[(size_t)i]);
        if (a < a_bd) { a_bd = a; ibd = i; }
      }
      const double a_cg = pHp > 0.0 ? rr / pHp : std::numeric_limits<double>::infinity();
      const double a = std::min(a_cg, std::min(a_tr, a_bd));
      if (!std::isfinite(a)) break;
      for (int i = 0; i < n; ++i) {
        d[(size_t)i] += a * p[(size_t)i];
        r[(size_t)i] += a * Hp[(size_t)i];
      }
      if (a == a_bd && ibd >= 0 && a_bd < a_tr) {
        d[(size_t)ibd] = p[(size_t)ibd] > 0.0 ? su[(size_t)ibd] - x0[(size_t)ibd] : sl[(size_t)ibd] - x0[(size_t)ibd];
        fixed[(size_t)ibd] = 1;
        restart = true;
        continue;
      }
      if (a == a_tr) break;
    }
    for (int i = 0; i < n; ++i)
      d[(size_t)i] = std::min(su[(size_t)i] - x0[(size_t)i], std::max(sl[(size_t)i] - x0[(size_t)i], d[(size_t)i]));
  }

  // Geometry step for point t: a displacement d from the best point, |d| <= rad,
  // inside the box, where |Lagrange function t| is large (along the lines to
  // the other interpolation points and along the Lagrange gradient).
  void geometry_step(int t, double rad, std::vector<double>& best_d) {
    std::vector<double> gl, Hl;
    lagrange_derivs(t, gl, Hl);
    const double l0 = lagrange(t, std::vector<double>((size_t)n, 0.0).data());
    double best = -1.0;
    best_d.assign((size_t)n, 0.0);
    auto try_line = [&](const double* v) {
      const double vv = dot(v, v, n);
      if (!(vv > 0.0)) return;
      double alo = -rad / std::sqrt(vv), ahi = rad / std::sqrt(vv);
      for (int i = 0; i < n; ++i) {
        if (v[i] == 0.0) continue;
        const double lo = (sl[(size_t)i] - x0[(size_t)i]) / v[i], hi = (su[(size_t)i] - x0[(size_t)i]) / v[i];
        alo = std::max(alo, std::min(lo, hi));
        ahi = std::min(ahi, std::max(lo, hi));
      }
      if (!(ahi > alo)) return;
      std::vector<double> Hv((size_t)n);
      for (int a = 0; a < n; ++a) Hv[(size_t)a] = dot(Hl.data() + (size_t)a * n, v, n);
      const double s1 = dot(gl.data(), v, n), s2 = dot(v, Hv.data(), n);
      double cands[3] = {alo, ahi, 0.0};
      int nc = 2;
      if (s2 != 0.0) {
        const double as = -s1 / s2;
        if (as > alo && as < ahi) cands[nc++] = as;
      }
      for (int k = 0; k < nc; ++k) {
        const double a = cands[k];
        const double val = std::fabs(l0 + a * s1 + 0.5 * a * a * s2);
        if (val > best && a != 0.0) {
          best = val;
          for (int i = 0; i < n; ++i) best_d[(size_t)i] = a * v[i];
        }
      }
    };
    for (int j = 0; j < m; ++j)
      if (j != kopt) try_line(y(j));
    try_line(gl.data());
  }

  void reduce_rho() {
    const double ratio = rho / rho_end;
    const double rnew = ratio <= 16.0 ? rho_end : (ratio <= 250.0 ? std::sqrt(ratio) * rho_end : 0.1 * rho);
    delta = std::max(0.5 * rho, rnew);
    rho = rnew;
  }

  void push(const double* ud, int kind, int t) {  // ud: displacement from x0
    for (int i = 0; i < n; ++i)
      pend.push_back(std::min(su[(size_t)i], std::max(sl[(size_t)i], x0[(size_t)i] + ud[i])));
    pend_kind.push_back(kind);
    pend_t.push_back(t);
  }

  // The next point(s) to evaluate; sets stop when rho reached rho_end with no step left.
  void propose(bool after_poor) {
    pend.clear();
    pend_kind.clear();
    pend_t.clear();
    if (nf >= max_eval) { stop = 3; return; }
    for (int guard = 0; guard < 64; ++guard) {
      // a far point after a poor step: improve the geometry first
      int far = -1;
      double dfar = 0.0;
      for (int t = 0; t < m; ++t) {
        if (t == kopt) continue;
        const double dt = dist_to_opt(t);
        if (dt > dfar) { dfar = dt; far = t; }
      }
      if (after_poor && far >= 0 && dfar > 2.0 * delta) {
        std::vector<double> d;
        geometry_step(far, std::max(std::min(0.1 * dfar, delta), rho), d);
        push(d.data(), kGeometry, far);
        return;
      }
      std::vector<double> d;
      trust_step(d);
      dnorm = std::sqrt(dot(d.data(), d.data(), n));
      if (dnorm >= 0.5 * rho) {
        pred = -model_change(d.data());
        push(d.data(), kTrust, -1);
        // optional batch: geometry points for the farthest other points
        if (batch > 1) {
          std::vector<std::pair<double, int>> order;
          for (int t = 0; t < m; ++t)
            if (t != kopt) order.emplace_back(-dist_to_opt(t), t);
          std::sort(order.begin(), order.end());
          for (int k = 0; k < (int)order.size() && (int)pend_kind.size() < batch; ++k) {
            const int t = order[(size_t)k].second;
            std::vector<double> dg;
            geometry_step(t, std::max(std::min(-0.5 * order[(size_t)k].first, delta), rho), dg);
            push(dg.data(), kGeometry, t);
          }
        }
        return;
      }
      // short step: shrink the radius; improve the geometry or refine rho
      delta = std::max(0.1 * delta, rho);
      if (delta <= 1.5 * rho) delta = rho;
      if (far >= 0 && dfar > 2.0 * delta) {
        after_poor = true;
        continue;
      }
      if (rho <= rho_end) { stop = 2; return; }
      reduce_rho();
      after_poor = false;
    }
    stop = 2;
  }

  // One evaluated point: the trust radius (a trust step), the point it
  // replaces, the model update.  Returns whether the step was poor.
  bool absorb(const double* xu, int kind, int t_fixed, double f, const std::vector<int>& reserved) {
    nf++;
    if (f < fx_best) {
      fx_best = f;
      x_best.assign(xu, xu + n);
    }
    std::vector<double> d((size_t)n);
    for (int i = 0; i < n; ++i) d[(size_t)i] = xu[i] - x0[(size_t)i];
    const double fopt = F[(size_t)kopt];
    bool poor = kind != kTrust;
    if (kind == kTrust) {
      const double ratio = pred > 0.0 ? (fopt - f) / pred : -1.0;
      if (ratio <= 0.1) delta = std::min(0.5 * delta, dnorm);
      else if (ratio <= 0.7) delta = std::max(0.5 * delta, dnorm);
      else delta = std::max(0.5 * delta, 2.0 * dnorm);
      if (delta <= 1.5 * rho) delta = rho;
      poor = ratio < 0.1;
    }
    int t = t_fixed;
    if (t < 0) {
      double best = -1.0;
      for (int j = 0; j < m; ++j) {
        if (j == kopt && !(f < fopt)) continue;
        if (std::find(reserved.begin(), reserved.end(), j) != reserved.end()) continue;
        const double dist = dist_to_opt(j) / std::max(delta, rho);
        const double w = std::max(1.0, dist * dist * dist * dist);
        const double score = std::fabs(lagrange(j, d.data())) * w;
        if (score > best) { best = score; t = j; }
      }
    }
    if (t < 0) return poor;
    const std::vector<double> Yold(Y), Winv_old(Winv);
    const double sig_old = sigma, f_old = F[(size_t)t];
    for (int k = 0; k < n; ++k) Y[(size_t)t * n + k] = d[(size_t)k];
    F[(size_t)t] = f;
    if (!factor()) {  // the new point would make the set degenerate: keep the old one
      Y = Yold;
      Winv = Winv_old;
      sigma = sig_old;
      F[(size_t)t] = f_old;
      return poor;
    }
    update_model();
    if (f < fopt) {
      kopt = t;
      shift_to(t);
      factor();
    }
    return poor;
  }
};

extern "C" XR_API xr_status xr_dfo_create(int32_t dim, const double* x0, const double* lower, const double* upper,
                                          double rho_beg, double rho_end, int64_t max_iter, xr_dfo* out) {
  if (!out || !x0 || !lower || !upper) return fail(XR_ERR_INVALID_ARG, "xr_dfo_create: NULL argument");
  *out = nullptr;
  if (dim < 1 || dim > 64) return fail(XR_ERR_INVALID_ARG, "xr_dfo_create: dimension must be in [1, 64]");
  if (!(rho_beg > 0) || !(rho_end > 0) || rho_end > rho_beg)
    return fail(XR_ERR_INVALID_ARG, "xr_dfo_create: need 0 < rho_end <= rho_beg");
  if (max_iter < 0) return fail(XR_ERR_INVALID_ARG, "xr_dfo_create: max_iter must be >= 0");
  double smax = 0;
  for (int i = 0; i < dim; ++i) {
    if (!(upper[i] > lower[i]) || !(x0[i] >= lower[i] && x0[i] <= upper[i]))
      return fail(XR_ERR_INVALID_ARG, "xr_dfo_create: need lower < upper and x0 inside the bounds");
    smax = std::max(smax, upper[i] - lower[i]);
  }
  auto* d = new (std::nothrow) xr_dfo_s();
  if (!d) return fail(XR_ERR_OUT_OF_MEMORY, "xr_dfo_create: host allocation failed");
  const int n = dim, m = 2 * dim + 1;
  d->n = n;
  d->m = m;
  for (int i = 0; i < n; ++i) {
    const double s = (upper[i] - lower[i]) / smax;
    d->scale.push_back(s);
    d->sl.push_back(lower[i] / s);
    d->su.push_back(upper[i] / s);
  }
  // BOBYQA needs room for the initial points: rho_beg <= half the narrowest width
  double wmin = std::numeric_limits<double>::infinity();
  for (int i = 0; i < n; ++i) wmin = std::min(wmin, d->su[(size_t)i] - d->sl[(size_t)i]);
  d->rho = std::min(rho_beg, 0.5 * wmin);
  d->rho_end = std::min(rho_end, d->rho);
  d->delta = d->rho;
  d->max_eval = (int64_t)m + max_iter;
  d->g.assign((size_t)n, 0.0);
  d->H.assign((size_t)n * n, 0.0);
  d->Y.assign((size_t)m * n, 0.0);
  d->F.assign((size_t)m, 0.0);
  d->x0.resize((size_t)n);
  for (int i = 0; i < n; ++i) d->x0[(size_t)i] = x0[i] / d->scale[(size_t)i];
  d->x_best = d->x0;
  // the initial set: x0, then per coordinate +-rho (one-sided at a bound)
  std::vector<double> zero((size_t)n, 0.0);
  d->push(zero.data(), kInit, 0);
  for (int i = 0; i < n; ++i) {
    const double xi = d->x0[(size_t)i], r = d->rho;
    double a = r, b = -r;
    if (xi + r > d->su[(size_t)i]) { a = -r; b = -2.0 * r; }
    else if (xi - r < d->sl[(size_t)i]) { a = r; b = 2.0 * r; }
    for (int k = 0; k < 2; ++k) {
      std::vector<double> e((size_t)n, 0.0);
      e[(size_t)i] = k == 0 ? a : b;
      d->push(e.data(), kInit, 1 + 2 * i + k);
    }
  }
  *out = d;
  return XR_OK;
}

extern "C" XR_API xr_status xr_dfo_destroy(xr_dfo d) {
  delete d;
  return XR_OK;
}

extern "C" XR_API xr_status xr_dfo_set_batch(xr_dfo d, int32_t points) {
  if (!d) return fail(XR_ERR_INVALID_ARG, "xr_dfo_set_batch: NULL handle");
  if (points < 1 || points > 2 * d->n + 2) return fail(XR_ERR_INVALID_ARG, "xr_dfo_set_batch: need 1 <= points <= 2 dim + 2");
  if (d->initialised) return fail(XR_ERR_INVALID_ARG, "xr_dfo_set_batch: set the batch before the first tell");
  d->max_eval = d->m + (d->max_eval - d->m) * points;  // max_iter iterations of `points` evaluations
  d->batch = points;
  return XR_OK;
}

extern "C" XR_API xr_status xr_dfo_ask(xr_dfo d, double* pts, int32_t* count) {
  if (!d || !pts || !count) return fail(XR_ERR_INVALID_ARG, "xr_dfo_ask: NULL argument");
  if (d->pend_kind.empty()) return fail(XR_ERR_INVALID_ARG, "xr_dfo_ask: the optimizer has stopped");
  const int n = d->n, k = (int)d->pend_kind.size();
  for (int r = 0; r < k; ++r)
    for (int i = 0; i < n; ++i) pts[(size_t)r * n + i] = d->pend[(size_t)r * n + i] * d->scale[(size_t)i];
  *count = k;
  return XR_OK;
}

extern "C" XR_API xr_status xr_dfo_tell(xr_dfo d, const double* f) {
  if (!d || !f) return fail(XR_ERR_INVALID_ARG, "xr_dfo_tell: NULL argument");
  if (d->pend_kind.empty()) return fail(XR_ERR_INVALID_ARG, "xr_dfo_tell: ask for a batch first");
  const int n = d->n, k = (int)d->pend_kind.size();
  // a value that is not finite (an empty overlap) counts as worse than every finite one
  std::vector<double> fv(f, f + k);
  double worst = -std::numeric_limits<double>::infinity();
  for (double v : d->F) worst = std::isfinite(v) ? std::max(worst, v) : worst;
  for (double v : fv) worst = std::isfinite(v) ? std::max(worst, v) : worst;
  if (!std::isfinite(worst)) worst = 0.0;
  for (double& v : fv)
    if (!std::isfinite(v)) v = worst + 1.0 + std::fabs(worst);
  f = fv.data();
  const std::vector<double> pend = d->pend;
  const std::vector<int> kinds = d->pend_kind, ts = d->pend_t;
  bool poor = false;
  if (!d->initialised) {
    for (int r = 0; r < k; ++r) {
      d->F[(size_t)ts[(size_t)r]] = f[r];
      for (int i = 0; i < n; ++i) d->Y[(size_t)ts[(size_t)r] * n + i] = pend[(size_t)r * n + i] - d->x0[(size_t)i];
      d->nf++;
      if (f[r] < d->fx_best) {
        d->fx_best = f[r];
        d->x_best.assign(pend.begin() + (size_t)r * n, pend.begin() + (size_t)(r + 1) * n);
      }
    }
    if (!d->factor()) return fail(XR_ERR_INVALID_ARG, "xr_dfo_tell: degenerate initial interpolation set");
    d->update_model();  // from the zero model: the least-norm quadratic through the set
    d->kopt = 0;
    for (int t = 1; t < d->m; ++t)
      if (d->F[(size_t)t] < d->F[(size_t)d->kopt]) d->kopt = t;
    d->shift_to(d->kopt);
    d->factor();
    d->initialised = true;
  } else {
    std::vector<int> reserved;
    for (int r = 0; r < k; ++r)
      if (kinds[(size_t)r] == kGeometry) reserved.push_back(ts[(size_t)r]);
    for (int r = 0; r < k; ++r) {
      if (kinds[(size_t)r] == kGeometry)
        reserved.erase(std::find(reserved.begin(), reserved.end(), ts[(size_t)r]));
      const bool p = d->absorb(pend.data() + (size_t)r * n, kinds[(size_t)r], ts[(size_t)r], f[r], reserved);
      if (r == 0) poor = p;
    }
    d->iter++;
  }
  d->propose(poor);
  return XR_OK;
}

// *reason: 0 continue, 2 rho reached rho_end, 3 evaluation / iteration limit.
extern "C" XR_API xr_status xr_dfo_test_termination(xr_dfo d, int32_t* reason) {
  if (!d || !reason) return fail(XR_ERR_INVALID_ARG, "xr_dfo_test_termination: NULL argument");
  *reason = d->stop;
  return XR_OK;
}

extern "C" XR_API xr_status xr_dfo_get(xr_dfo d, double* best_x, double* best_f, double* rho, int64_t* iterations) {
  if (!d) return fail(XR_ERR_INVALID_ARG, "xr_dfo_get: NULL handle");
  if (best_x)
    for (int i = 0; i < d->n; ++i) best_x[i] = d->x_best[(size_t)i] * d->scale[(size_t)i];
  if (best_f) *best_f = d->fx_best;
  if (rho) *rho = d->rho * 1.0;
  if (iterations) *iterations = d->iter;
  return XR_OK;
}

extern "C" XR_API xr_status xr_dfo_evaluations(xr_dfo d, int64_t* evaluations) {
  if (!d || !evaluations) return fail(XR_ERR_INVALID_ARG, "xr_dfo_evaluations: NULL argument");
  *evaluations = d->nf;
  return XR_OK;
}
