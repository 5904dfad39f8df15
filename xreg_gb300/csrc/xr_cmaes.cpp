// xr_cmaes.cpp -- CMA-ES population optimizer (double precision) behind the C
// ABI, the optimizer xReg drives its population objective with
// (Intensity2D3DRegiCMAES::run, xregIntensity2D3DRegiCMAES.cpp:76-247, through
// the vendored cmaes.c interface: init / SamplePopulation / ReSampleSingle /
// UpdateDistribution / TestForTermination).
//
// Algorithm: the (mu/mu_w, lambda)-CMA-ES as published by N. Hansen ("The CMA
// Evolution Strategy: A Tutorial", 2016): log-rank weights over the best half,
// cumulative step-size adaptation, rank-one plus rank-mu covariance update with
// the h_sigma stall, eigendecomposition of C each generation (Jacobi rotations
// in round-robin order, warm-started from the last eigenbasis, so a
// generation's few sweeps run in parallel on a device block).  Initialisation follows the convention
// of Hansen's C code that xReg calls: sigma = RMS of the per-coordinate initial
// standard deviations and C = diag(s_i^2) / sigma^2, so sigma^2 C = diag(s_i^2).
// Termination: function-value range over the recent generations below tol_fun,
// all coordinate standard deviations and evolution-path entries below tol_x,
// or the iteration limit.  Sampling, update and termination are the shared
// host/device steps of xr_cmaes_core.h (counter-based normals, one rounding
// per operation): the state can move to device memory
// (xr_cmaes_attach_device), where the job-set step samples and updates it
// inside its own launches with the same bits as here.
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

#include <cuda_runtime_api.h>

#include "xr_cmaes_core.h"
#include "xr_step.h"
#include "xreg_gb300_regi.h"

namespace xr {
xr_status fail(xr_status code, const std::string& msg);
}

using xr::fail;
namespace cma = xr::cma;

struct xr_cmaes_s {
  std::vector<double> buf;  // the state block (xr_cmaes_core.h layout), 8-byte aligned
  cma::View v{};
  void* d_state = nullptr;  // device copy while attached
  int device = -1;
  size_t bytes = 0;
  bool on_device() const { return d_state != nullptr; }
  // host copy of the state; an attached state is read back from the device first
  xr_status pull() {
    if (!d_state) return XR_OK;
    int prev = 0;
    cudaGetDevice(&prev);
    cudaSetDevice(device);
    const cudaError_t e = cudaMemcpy(buf.data(), d_state, bytes, cudaMemcpyDeviceToHost);
    cudaSetDevice(prev);
    if (e != cudaSuccess) return fail(XR_ERR_CUDA, std::string("xr_cmaes: reading the device state: ") + cudaGetErrorString(e));
    v = cma::view(buf.data());
    return XR_OK;
  }
  void draw(int k, int attempt) {
    v.att[k] = attempt;
    cma::draw(v, k, attempt, v.z + (size_t)k * v.h->n, v.pop + (size_t)k * v.h->n);
  }
};

namespace {
xr_status refuse_on_device(const char* fn) {
  return fail(XR_ERR_INVALID_ARG, std::string(fn) + ": the state lives on the device (xr_cmaes_detach_device first)");
}
}  // namespace

extern "C" XR_API xr_status xr_cmaes_create(int32_t dim, const double* xstart, const double* stddevs, int32_t lambda,
                                            uint64_t seed, xr_cmaes* out) {
  if (!out || !xstart || !stddevs) return fail(XR_ERR_INVALID_ARG, "xr_cmaes_create: NULL argument");
  *out = nullptr;
  if (dim < 1 || dim > 64) return fail(XR_ERR_INVALID_ARG, "xr_cmaes_create: dimension must be in [1, 64]");
  if (lambda < 2 || lambda > (1 << 20)) return fail(XR_ERR_INVALID_ARG, "xr_cmaes_create: lambda must be in [2, 2^20]");
  for (int i = 0; i < dim; ++i)
    if (!(stddevs[i] > 0.0) || !std::isfinite(stddevs[i]) || !std::isfinite(xstart[i]))
      return fail(XR_ERR_INVALID_ARG, "xr_cmaes_create: initial std devs must be positive and finite");
  auto* e = new (std::nothrow) xr_cmaes_s();
  if (!e) return fail(XR_ERR_OUT_OF_MEMORY, "xr_cmaes_create: host allocation failed");
  const int n = dim, mu = lambda / 2;
  const int hlen = 10 + (int)std::ceil(30.0 * n / lambda);
  e->bytes = cma::state_bytes(n, lambda, mu, hlen);
  e->buf.assign((e->bytes + 7) / 8, 0.0);
  cma::Hdr& h = *reinterpret_cast<cma::Hdr*>(e->buf.data());
  h.n = n;
  h.lam = lambda;
  h.mu = mu;
  h.hlen = hlen;
  h.seed = seed;
  h.max_iter = 1000000;
  h.tol_fun = 1e-12;
  h.tol_x = 1e-11;
  h.best_f = std::numeric_limits<double>::infinity();
  h.last_range = std::numeric_limits<double>::infinity();
  cma::View& v = e->v;
  v = cma::view(e->buf.data());
  double sw = 0, sw2 = 0;
  for (int i = 0; i < mu; ++i) {
    v.w[i] = std::log(mu + 0.5) - std::log(i + 1.0);
    sw += v.w[i];
  }
  for (int i = 0; i < mu; ++i) {
    v.w[i] /= sw;
    sw2 += v.w[i] * v.w[i];
  }
  h.mueff = 1.0 / sw2;
  const double N = n;
  h.cs = (h.mueff + 2.0) / (N + h.mueff + 5.0);
  h.ds = 1.0 + 2.0 * std::max(0.0, std::sqrt((h.mueff - 1.0) / (N + 1.0)) - 1.0) + h.cs;
  h.cc = (4.0 + h.mueff / N) / (N + 4.0 + 2.0 * h.mueff / N);
  h.c1 = 2.0 / ((N + 1.3) * (N + 1.3) + h.mueff);
  h.cmu = std::min(1.0 - h.c1, 2.0 * (h.mueff - 2.0 + 1.0 / h.mueff) / ((N + 2.0) * (N + 2.0) + h.mueff));
  h.chin = std::sqrt(N) * (1.0 - 1.0 / (4.0 * N) + 1.0 / (21.0 * N * N));
  double trace = 0;
  for (int i = 0; i < n; ++i) trace += stddevs[i] * stddevs[i];
  h.sigma = std::sqrt(trace / N);
  for (int i = 0; i < n; ++i) {
    const double s = stddevs[i] / h.sigma;
    v.m[i] = xstart[i];
    v.best[i] = xstart[i];
    v.C[i * n + i] = s * s;
    v.B[i * n + i] = 1.0;
    v.D[i] = s;
  }
  *out = e;
  return XR_OK;
}

extern "C" XR_API xr_status xr_cmaes_destroy(xr_cmaes e) {
  if (e && e->d_state) {
    int prev = 0;
    cudaGetDevice(&prev);
    cudaSetDevice(e->device);
    cudaFree(e->d_state);
    cudaSetDevice(prev);
  }
  delete e;
  return XR_OK;
}

extern "C" XR_API xr_status xr_cmaes_set_stop(xr_cmaes e, double tol_fun, double tol_x, int64_t max_iter) {
  if (!e) return fail(XR_ERR_INVALID_ARG, "xr_cmaes_set_stop: NULL handle");
  if (e->on_device()) return refuse_on_device("xr_cmaes_set_stop");
  e->v.h->tol_fun = tol_fun;
  e->v.h->tol_x = tol_x;
  e->v.h->max_iter = max_iter;
  return XR_OK;
}

extern "C" XR_API xr_status xr_cmaes_sample_population(xr_cmaes e, double* pop) {
  if (!e || !pop) return fail(XR_ERR_INVALID_ARG, "xr_cmaes_sample_population: NULL argument");
  if (e->on_device()) return refuse_on_device("xr_cmaes_sample_population");
  for (int k = 0; k < e->v.h->lam; ++k) e->draw(k, 0);
  std::memcpy(pop, e->v.pop, (size_t)e->v.h->lam * e->v.h->n * sizeof(double));
  e->v.h->sampled = 1;
  return XR_OK;
}

extern "C" XR_API xr_status xr_cmaes_resample_single(xr_cmaes e, int32_t k, double* pop) {
  if (!e || !pop) return fail(XR_ERR_INVALID_ARG, "xr_cmaes_resample_single: NULL argument");
  if (e->on_device()) return refuse_on_device("xr_cmaes_resample_single");
  if (!e->v.h->sampled || k < 0 || k >= e->v.h->lam)
    return fail(XR_ERR_INVALID_ARG, "xr_cmaes_resample_single: bad index");
  if (e->v.att[k] == std::numeric_limits<int32_t>::max())
    return fail(XR_ERR_INVALID_ARG, "xr_cmaes_resample_single: too many redraws");
  e->draw(k, e->v.att[k] + 1);
  const int n = e->v.h->n;
  std::memcpy(pop + (size_t)k * n, e->v.pop + (size_t)k * n, (size_t)n * sizeof(double));
  return XR_OK;
}

extern "C" XR_API xr_status xr_cmaes_update_distribution(xr_cmaes e, const double* f) {
  if (!e || !f) return fail(XR_ERR_INVALID_ARG, "xr_cmaes_update_distribution: NULL argument");
  if (e->on_device()) return refuse_on_device("xr_cmaes_update_distribution");
  if (!e->v.h->sampled) return fail(XR_ERR_INVALID_ARG, "xr_cmaes_update_distribution: sample a population first");
  std::memcpy(e->v.fv, f, (size_t)e->v.h->lam * sizeof(double));
  cma::update(e->v);
  return XR_OK;
}

extern "C" XR_API xr_status xr_cmaes_test_termination(xr_cmaes e, int32_t* reason) {
  if (!e || !reason) return fail(XR_ERR_INVALID_ARG, "xr_cmaes_test_termination: NULL argument");
  xr_status st = e->pull();
  if (st != XR_OK) return st;
  *reason = cma::termination(e->v);
  return XR_OK;
}

extern "C" XR_API xr_status xr_cmaes_lambda(xr_cmaes e, int32_t* lambda) {
  if (!e || !lambda) return fail(XR_ERR_INVALID_ARG, "cmaes_lambda: NULL argument");
  *lambda = e->v.h->lam;
  return XR_OK;
}

extern "C" XR_API xr_status xr_cmaes_get(xr_cmaes e, double* mean, double* best_x, double* best_f, double* sigma,
                                         int64_t* generation) {
  if (!e) return fail(XR_ERR_INVALID_ARG, "xr_cmaes_get: NULL handle");
  xr_status st = e->pull();
  if (st != XR_OK) return st;
  const int n = e->v.h->n;
  if (mean) std::memcpy(mean, e->v.m, (size_t)n * sizeof(double));
  if (best_x) std::memcpy(best_x, e->v.best, (size_t)n * sizeof(double));
  if (best_f) *best_f = e->v.h->best_f;
  if (sigma) *sigma = e->v.h->sigma;
  if (generation) *generation = e->v.h->gen;
  return XR_OK;
}

extern "C" XR_API xr_status xr_cmaes_state_bytes(xr_cmaes e, int64_t* bytes) {
  if (!e || !bytes) return fail(XR_ERR_INVALID_ARG, "xr_cmaes_state_bytes: NULL argument");
  *bytes = (int64_t)e->bytes;
  return XR_OK;
}

extern "C" XR_API xr_status xr_cmaes_export_state(xr_cmaes e, void* out, int64_t bytes) {
  if (!e || !out) return fail(XR_ERR_INVALID_ARG, "xr_cmaes_export_state: NULL argument");
  if (bytes < (int64_t)e->bytes) return fail(XR_ERR_INVALID_ARG, "xr_cmaes_export_state: buffer too small");
  xr_status st = e->pull();
  if (st != XR_OK) return st;
  std::memcpy(out, e->buf.data(), e->bytes);
  return XR_OK;
}

extern "C" XR_API xr_status xr_cmaes_attach_device(xr_cmaes e, int32_t device) {
  if (!e) return fail(XR_ERR_INVALID_ARG, "xr_cmaes_attach_device: NULL handle");
  if (e->on_device()) return fail(XR_ERR_INVALID_ARG, "xr_cmaes_attach_device: already attached");
  if (e->v.h->n > xr::kCmaDeviceMaxDim)
    return fail(XR_ERR_INVALID_ARG, "xr_cmaes_attach_device: the device path takes at most 8 parameters");
  int prev = 0, dev = device;
  if (cudaGetDevice(&prev) != cudaSuccess) return fail(XR_ERR_CUDA, "xr_cmaes_attach_device: no CUDA device");
  if (dev < 0) dev = prev;
  if (cudaSetDevice(dev) != cudaSuccess) return fail(XR_ERR_INVALID_ARG, "xr_cmaes_attach_device: bad device");
  void* d = nullptr;
  cudaError_t err = cudaMalloc(&d, e->bytes);
  if (err == cudaSuccess) err = cudaMemcpy(d, e->buf.data(), e->bytes, cudaMemcpyHostToDevice);
  if (err != cudaSuccess && d) cudaFree(d);
  cudaSetDevice(prev);
  if (err != cudaSuccess) return fail(XR_ERR_CUDA, std::string("xr_cmaes_attach_device: ") + cudaGetErrorString(err));
  e->d_state = d;
  e->device = dev;
  return XR_OK;
}

extern "C" XR_API xr_status xr_cmaes_detach_device(xr_cmaes e) {
  if (!e) return fail(XR_ERR_INVALID_ARG, "xr_cmaes_detach_device: NULL handle");
  if (!e->on_device()) return XR_OK;
  xr_status st = e->pull();
  if (st != XR_OK) return st;
  int prev = 0;
  cudaGetDevice(&prev);
  cudaSetDevice(e->device);
  cudaFree(e->d_state);
  cudaSetDevice(prev);
  e->d_state = nullptr;
  e->device = -1;
  return XR_OK;
}

namespace xr {
bool cmaes_device_state(xr_cmaes e, void** d_state, int32_t* lambda, int32_t* dim, int32_t* device) {
  if (!e || !e->d_state) return false;
  *d_state = e->d_state;
  *lambda = e->v.h->lam;
  *dim = e->v.h->n;
  *device = e->device;
  return true;
}
}  // namespace xr
