// xr_cmaes.cpp -- CMA-ES population optimizer (host, double precision) behind
// the C ABI, the optimizer xReg drives its population objective with
// (Intensity2D3DRegiCMAES::run, xregIntensity2D3DRegiCMAES.cpp:76-247, through
// the vendored cmaes.c interface: init / SamplePopulation / ReSampleSingle /
// UpdateDistribution / TestForTermination).
//
// Algorithm: the (mu/mu_w, lambda)-CMA-ES as published by N. Hansen ("The CMA
// Evolution Strategy: A Tutorial", 2016): log-rank weights over the best half,
// cumulative step-size adaptation, rank-one plus rank-mu covariance update with
// the h_sigma stall, eigendecomposition of C each generation (cyclic Jacobi,
// fine for the 6-parameter poses here).  Initialisation follows the convention
// of Hansen's C code that xReg calls: sigma = RMS of the per-coordinate initial
// standard deviations and C = diag(s_i^2) / sigma^2, so sigma^2 C = diag(s_i^2).
// Termination: function-value range over the recent generations below tol_fun,
// all coordinate standard deviations and evolution-path entries below tol_x,
// or the iteration limit.  Random numbers: xoshiro256** seeded by splitmix64,
// Box-Muller normals (reproducible for a given seed on one platform).
#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <deque>
#include <limits>
#include <new>
#include <numeric>
#include <string>
#include <vector>

#include "xreg_gb300_regi.h"

namespace xr {
xr_status fail(xr_status code, const std::string& msg);
}

namespace {

struct Rng {
  uint64_t s[4];
  double spare = 0.0;
  bool has_spare = false;
  explicit Rng(uint64_t seed) {
    uint64_t z = seed;
    for (int i = 0; i < 4; ++i) {
      z += 0x9e3779b97f4a7c15ull;
      uint64_t x = z;
      x = (x ^ (x >> 30)) * 0xbf58476d1ce4e5b9ull;
      x = (x ^ (x >> 27)) * 0x94d049bb133111ebull;
      s[i] = x ^ (x >> 31);
    }
  }
  static uint64_t rotl(uint64_t x, int k) { return (x << k) | (x >> (64 - k)); }
  uint64_t next() {
    const uint64_t r = rotl(s[1] * 5, 7) * 9;
    const uint64_t t = s[1] << 17;
    s[2] ^= s[0]; s[3] ^= s[1]; s[1] ^= s[2]; s[0] ^= s[3];
    s[2] ^= t;
    s[3] = rotl(s[3], 45);
    return r;
  }
  double uniform() { return (double)(next() >> 11) * (1.0 / 9007199254740992.0); }  // [0, 1)
  double normal() {
    if (has_spare) { has_spare = false; return spare; }
    double u1 = uniform();
    while (u1 <= 0.0) u1 = uniform();
    const double u2 = uniform();
    const double r = std::sqrt(-2.0 * std::log(u1));
    const double a = 6.283185307179586476925 * u2;
    spare = r * std::sin(a);
    has_spare = true;
    return r * std::cos(a);
  }
};

// Eigen-decomposition of a symmetric matrix by cyclic Jacobi rotations:
// A = V diag(d) V^T, V column-wise.
void jacobi_eig(int n, std::vector<double> A, std::vector<double>& d, std::vector<double>& V) {
  V.assign((size_t)n * n, 0.0);
  for (int i = 0; i < n; ++i) V[(size_t)i * n + i] = 1.0;
  for (int sweep = 0; sweep < 64; ++sweep) {
    double off = 0.0;
    for (int p = 0; p < n; ++p)
      for (int q = p + 1; q < n; ++q) off += A[(size_t)p * n + q] * A[(size_t)p * n + q];
    if (off < 1e-300) break;
    for (int p = 0; p < n; ++p)
      for (int q = p + 1; q < n; ++q) {
        const double apq = A[(size_t)p * n + q];
        if (std::fabs(apq) < 1e-300) continue;
        const double app = A[(size_t)p * n + p], aqq = A[(size_t)q * n + q];
        const double theta = (aqq - app) / (2.0 * apq);
        const double t = (theta >= 0 ? 1.0 : -1.0) / (std::fabs(theta) + std::sqrt(theta * theta + 1.0));
        const double c = 1.0 / std::sqrt(t * t + 1.0), s = t * c;
        for (int k = 0; k < n; ++k) {
          const double akp = A[(size_t)k * n + p], akq = A[(size_t)k * n + q];
          A[(size_t)k * n + p] = c * akp - s * akq;
          A[(size_t)k * n + q] = s * akp + c * akq;
        }
        for (int k = 0; k < n; ++k) {
          const double apk = A[(size_t)p * n + k], aqk = A[(size_t)q * n + k];
          A[(size_t)p * n + k] = c * apk - s * aqk;
          A[(size_t)q * n + k] = s * apk + c * aqk;
        }
        for (int k = 0; k < n; ++k) {
          const double vkp = V[(size_t)k * n + p], vkq = V[(size_t)k * n + q];
          V[(size_t)k * n + p] = c * vkp - s * vkq;
          V[(size_t)k * n + q] = s * vkp + c * vkq;
        }
      }
  }
  d.resize((size_t)n);
  for (int i = 0; i < n; ++i) d[(size_t)i] = A[(size_t)i * n + i];
}

}  // namespace

struct xr_cmaes_s {
  int n = 0, lambda = 0, mu = 0;
  std::vector<double> w;
  double mueff = 0, cs = 0, ds = 0, cc = 0, c1 = 0, cmu = 0, chin = 0;
  std::vector<double> m, pc, ps, C, B, D, init_sd;
  double sigma = 0;
  int64_t gen = 0;
  std::vector<double> pop, z;  // lambda x n candidates and their N(0,I) draws
  std::vector<double> best_x;
  double best_f = std::numeric_limits<double>::infinity();
  std::deque<double> hist;     // best value of recent generations
  double last_range = std::numeric_limits<double>::infinity();
  double tol_fun = 1e-12, tol_x = 1e-11;
  int64_t max_iter = 1000000;
  bool sampled = false;
  Rng rng{0};

  void draw(int k) {
    for (int i = 0; i < n; ++i) z[(size_t)k * n + i] = rng.normal();
    for (int i = 0; i < n; ++i) {
      double y = 0.0;
      for (int j = 0; j < n; ++j) y += B[(size_t)i * n + j] * D[(size_t)j] * z[(size_t)k * n + j];
      pop[(size_t)k * n + i] = m[(size_t)i] + sigma * y;
    }
  }
};

using xr::fail;

extern "C" XR_API xr_status xr_cmaes_create(int32_t dim, const double* xstart, const double* stddevs, int32_t lambda,
                                            uint64_t seed, xr_cmaes* out) {
  if (!out || !xstart || !stddevs) return fail(XR_ERR_INVALID_ARG, "xr_cmaes_create: NULL argument");
  *out = nullptr;
  if (dim < 1 || dim > 64) return fail(XR_ERR_INVALID_ARG, "xr_cmaes_create: dimension must be in [1, 64]");
  if (lambda < 2) return fail(XR_ERR_INVALID_ARG, "xr_cmaes_create: lambda must be >= 2");
  for (int i = 0; i < dim; ++i)
    if (!(stddevs[i] > 0.0) || !std::isfinite(stddevs[i]) || !std::isfinite(xstart[i]))
      return fail(XR_ERR_INVALID_ARG, "xr_cmaes_create: initial std devs must be positive and finite");
  auto* e = new (std::nothrow) xr_cmaes_s();
  if (!e) return fail(XR_ERR_OUT_OF_MEMORY, "xr_cmaes_create: host allocation failed");
  const int n = dim;
  e->n = n;
  e->lambda = lambda;
  e->mu = lambda / 2;
  e->rng = Rng(seed);
  e->w.resize((size_t)e->mu);
  double sw = 0, sw2 = 0;
  for (int i = 0; i < e->mu; ++i) {
    e->w[(size_t)i] = std::log(e->mu + 0.5) - std::log(i + 1.0);
    sw += e->w[(size_t)i];
  }
  for (double& v : e->w) { v /= sw; sw2 += v * v; }
  e->mueff = 1.0 / sw2;
  const double N = n;
  e->cs = (e->mueff + 2.0) / (N + e->mueff + 5.0);
  e->ds = 1.0 + 2.0 * std::max(0.0, std::sqrt((e->mueff - 1.0) / (N + 1.0)) - 1.0) + e->cs;
  e->cc = (4.0 + e->mueff / N) / (N + 4.0 + 2.0 * e->mueff / N);
  e->c1 = 2.0 / ((N + 1.3) * (N + 1.3) + e->mueff);
  e->cmu = std::min(1.0 - e->c1, 2.0 * (e->mueff - 2.0 + 1.0 / e->mueff) / ((N + 2.0) * (N + 2.0) + e->mueff));
  e->chin = std::sqrt(N) * (1.0 - 1.0 / (4.0 * N) + 1.0 / (21.0 * N * N));
  e->m.assign(xstart, xstart + n);
  e->init_sd.assign(stddevs, stddevs + n);
  double trace = 0;
  for (int i = 0; i < n; ++i) trace += stddevs[i] * stddevs[i];
  e->sigma = std::sqrt(trace / N);
  e->C.assign((size_t)n * n, 0.0);
  e->B.assign((size_t)n * n, 0.0);
  e->D.assign((size_t)n, 0.0);
  for (int i = 0; i < n; ++i) {
    const double s = stddevs[i] / e->sigma;
    e->C[(size_t)i * n + i] = s * s;
    e->B[(size_t)i * n + i] = 1.0;
    e->D[(size_t)i] = s;
  }
  e->pc.assign((size_t)n, 0.0);
  e->ps.assign((size_t)n, 0.0);
  e->pop.assign((size_t)lambda * n, 0.0);
  e->z.assign((size_t)lambda * n, 0.0);
  e->best_x = e->m;
  *out = e;
  return XR_OK;
}

extern "C" XR_API xr_status xr_cmaes_destroy(xr_cmaes e) {
  delete e;
  return XR_OK;
}

extern "C" XR_API xr_status xr_cmaes_set_stop(xr_cmaes e, double tol_fun, double tol_x, int64_t max_iter) {
  if (!e) return fail(XR_ERR_INVALID_ARG, "xr_cmaes_set_stop: NULL handle");
  e->tol_fun = tol_fun;
  e->tol_x = tol_x;
  e->max_iter = max_iter;
  return XR_OK;
}

extern "C" XR_API xr_status xr_cmaes_sample_population(xr_cmaes e, double* pop) {
  if (!e || !pop) return fail(XR_ERR_INVALID_ARG, "xr_cmaes_sample_population: NULL argument");
  for (int k = 0; k < e->lambda; ++k) e->draw(k);
  std::memcpy(pop, e->pop.data(), e->pop.size() * sizeof(double));
  e->sampled = true;
  return XR_OK;
}

extern "C" XR_API xr_status xr_cmaes_resample_single(xr_cmaes e, int32_t k, double* pop) {
  if (!e || !pop) return fail(XR_ERR_INVALID_ARG, "xr_cmaes_resample_single: NULL argument");
  if (!e->sampled || k < 0 || k >= e->lambda) return fail(XR_ERR_INVALID_ARG, "xr_cmaes_resample_single: bad index");
  e->draw(k);
  std::memcpy(pop + (size_t)k * e->n, e->pop.data() + (size_t)k * e->n, (size_t)e->n * sizeof(double));
  return XR_OK;
}

extern "C" XR_API xr_status xr_cmaes_update_distribution(xr_cmaes e, const double* f) {
  if (!e || !f) return fail(XR_ERR_INVALID_ARG, "xr_cmaes_update_distribution: NULL argument");
  if (!e->sampled) return fail(XR_ERR_INVALID_ARG, "xr_cmaes_update_distribution: sample a population first");
  const int n = e->n, lam = e->lambda, mu = e->mu;
  std::vector<int> idx((size_t)lam);
  std::iota(idx.begin(), idx.end(), 0);
  std::stable_sort(idx.begin(), idx.end(), [&](int a, int b) { return f[a] < f[b]; });
  if (f[idx[0]] < e->best_f) {
    e->best_f = f[idx[0]];
    e->best_x.assign(e->pop.begin() + (size_t)idx[0] * n, e->pop.begin() + (size_t)(idx[0] + 1) * n);
  }
  // recombination
  std::vector<double> mold = e->m, yw((size_t)n, 0.0), zw((size_t)n, 0.0);
  for (int i = 0; i < n; ++i) {
    double s = 0, sz = 0;
    for (int k = 0; k < mu; ++k) {
      s += e->w[(size_t)k] * e->pop[(size_t)idx[(size_t)k] * n + i];
      sz += e->w[(size_t)k] * e->z[(size_t)idx[(size_t)k] * n + i];
    }
    e->m[(size_t)i] = s;
    yw[(size_t)i] = (s - mold[(size_t)i]) / e->sigma;
    zw[(size_t)i] = sz;
  }
  // C^{-1/2} y_w = B z_w
  std::vector<double> bz((size_t)n, 0.0);
  for (int i = 0; i < n; ++i)
    for (int j = 0; j < n; ++j) bz[(size_t)i] += e->B[(size_t)i * n + j] * zw[(size_t)j];
  const double a_s = std::sqrt(e->cs * (2.0 - e->cs) * e->mueff);
  double psn = 0;
  for (int i = 0; i < n; ++i) {
    e->ps[(size_t)i] = (1.0 - e->cs) * e->ps[(size_t)i] + a_s * bz[(size_t)i];
    psn += e->ps[(size_t)i] * e->ps[(size_t)i];
  }
  psn = std::sqrt(psn);
  e->gen++;
  const double hthr = (1.4 + 2.0 / (n + 1.0)) * e->chin;
  const double hsig = (psn / std::sqrt(1.0 - std::pow(1.0 - e->cs, 2.0 * (double)e->gen)) < hthr) ? 1.0 : 0.0;
  const double a_c = std::sqrt(e->cc * (2.0 - e->cc) * e->mueff);
  for (int i = 0; i < n; ++i) e->pc[(size_t)i] = (1.0 - e->cc) * e->pc[(size_t)i] + hsig * a_c * yw[(size_t)i];
  // covariance update
  const double dh = (1.0 - hsig) * e->cc * (2.0 - e->cc);
  for (int i = 0; i < n; ++i)
    for (int j = 0; j <= i; ++j) {
      double rmu = 0;
      for (int k = 0; k < mu; ++k) {
        const int c = idx[(size_t)k];
        const double yi = (e->pop[(size_t)c * n + i] - mold[(size_t)i]) / e->sigma;
        const double yj = (e->pop[(size_t)c * n + j] - mold[(size_t)j]) / e->sigma;
        rmu += e->w[(size_t)k] * yi * yj;
      }
      const double cij = e->C[(size_t)i * n + j];
      const double v = (1.0 - e->c1 - e->cmu) * cij + e->c1 * (e->pc[(size_t)i] * e->pc[(size_t)j] + dh * cij) +
                       e->cmu * rmu;
      e->C[(size_t)i * n + j] = v;
      e->C[(size_t)j * n + i] = v;
    }
  e->sigma *= std::exp((e->cs / e->ds) * (psn / e->chin - 1.0));
  std::vector<double> d;
  jacobi_eig(n, e->C, d, e->B);
  for (int i = 0; i < n; ++i) e->D[(size_t)i] = std::sqrt(std::max(d[(size_t)i], 1e-300));
  // function-value history for the TolFun test
  e->hist.push_back(f[idx[0]]);
  const size_t hlen = 10 + (size_t)std::ceil(30.0 * n / lam);
  while (e->hist.size() > hlen) e->hist.pop_front();
  double lo = f[idx[0]], hi = f[idx[(size_t)lam - 1]];
  for (double h : e->hist) { lo = std::min(lo, h); hi = std::max(hi, h); }
  e->last_range = hi - lo;
  e->sampled = false;
  return XR_OK;
}

// stop reason: 0 continue, 1 tol_fun, 2 tol_x, 3 max_iter, 4 numerical (sigma not finite)
extern "C" XR_API xr_status xr_cmaes_test_termination(xr_cmaes e, int32_t* reason) {
  if (!e || !reason) return fail(XR_ERR_INVALID_ARG, "xr_cmaes_test_termination: NULL argument");
  *reason = 0;
  const int n = e->n;
  if (!std::isfinite(e->sigma)) { *reason = 4; return XR_OK; }
  if (e->gen >= e->max_iter) { *reason = 3; return XR_OK; }
  if (e->gen > 0 && e->last_range <= e->tol_fun) { *reason = 1; return XR_OK; }
  bool small = true;
  for (int i = 0; i < n && small; ++i)
    small = e->sigma * std::sqrt(e->C[(size_t)i * n + i]) < e->tol_x && e->sigma * std::fabs(e->pc[(size_t)i]) < e->tol_x;
  if (small && e->gen > 0) *reason = 2;
  return XR_OK;
}

extern "C" XR_API xr_status xr_cmaes_lambda(xr_cmaes e, int32_t* lambda) {
  if (!e || !lambda) return fail(XR_ERR_INVALID_ARG, "cmaes_lambda: NULL argument");
  *lambda = e->lambda;
  return XR_OK;
}

extern "C" XR_API xr_status xr_cmaes_get(xr_cmaes e, double* mean, double* best_x, double* best_f, double* sigma,
                                         int64_t* generation) {
  if (!e) return fail(XR_ERR_INVALID_ARG, "xr_cmaes_get: NULL handle");
  if (mean) std::memcpy(mean, e->m.data(), (size_t)e->n * sizeof(double));
  if (best_x) std::memcpy(best_x, e->best_x.data(), (size_t)e->n * sizeof(double));
  if (best_f) *best_f = e->best_f;
  if (sigma) *sigma = e->sigma;
  if (generation) *generation = e->gen;
  return XR_OK;
}
