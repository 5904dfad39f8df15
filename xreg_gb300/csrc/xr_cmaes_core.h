// xr_cmaes_core.h -- the CMA-ES optimizer state and its steps (sample a
// candidate, update the distribution, test for termination) and the pose map of
// a registration level, written once for the host (xr_cmaes.cpp, xr_regi.cpp)
// and the device (sampling inside the job-set geometry launch, the update
// behind the batched grad-NCC), so that both give the same bits:
//   * every floating-point operation is one IEEE double operation rounded to
//     nearest (device: the __d*_rn intrinsics, which are never contracted;
//     host: plain operators, compiled with -ffp-contract=off);
//   * the transcendental functions the optimizer needs (log and sin/cos for
//     Box-Muller normals, exp for the step-size update, sin/cos for ExpSE3)
//     are evaluated by the series below instead of either side's math library:
//     ln by 2 atanh((m-1)/(m+1)) on m in [sqrt(1/2), sqrt(2)), exp by its
//     Taylor series after a Cody-Waite reduction by ln 2, sin/cos by their
//     Taylor series after a Cody-Waite reduction by pi/2 (three-part split);
//     the coefficients are the correctly rounded doubles of 1/k! and
//     1/(2k+1), written as hex literals;
//   * random numbers are counter based: candidate k's draw number `attempt`
//     in generation g is a pure function of (seed, g, k, attempt), so the
//     candidates of a generation can be drawn in parallel and a redraw of one
//     candidate never shifts another's stream.
// The algorithm is the (mu/mu_w, lambda)-CMA-ES of N. Hansen, "The CMA
// Evolution Strategy: A Tutorial" (2016), as xReg drives it through its
// vendored cmaes.c (Intensity2D3DRegiCMAES::run,
// xregIntensity2D3DRegiCMAES.cpp:76-247); see xr_cmaes.cpp for the parameters.
#pragma once

#include <cmath>
#include <cstddef>
#include <cstdint>
#include <cstring>

#if defined(__CUDACC__)
#define XR_CMA_HD __host__ __device__ inline
#else
#define XR_CMA_HD inline
#endif

namespace xr {
namespace dm {

XR_CMA_HD double mul(double a, double b) {
#ifdef __CUDA_ARCH__
  return __dmul_rn(a, b);
#else
  return a * b;
#endif
}
XR_CMA_HD double add(double a, double b) {
#ifdef __CUDA_ARCH__
  return __dadd_rn(a, b);
#else
  return a + b;
#endif
}
XR_CMA_HD double sub(double a, double b) {
#ifdef __CUDA_ARCH__
  return __dsub_rn(a, b);
#else
  return a - b;
#endif
}
XR_CMA_HD double div(double a, double b) {
#ifdef __CUDA_ARCH__
  return __ddiv_rn(a, b);
#else
  return a / b;
#endif
}
XR_CMA_HD double sqrt(double a) {
#ifdef __CUDA_ARCH__
  return __dsqrt_rn(a);
#else
  return std::sqrt(a);
#endif
}
XR_CMA_HD double fabs(double a) { return a < 0.0 ? -a : a; }

// Cody-Waite pieces: ln 2 = kLn2Hi + kLn2Lo (kLn2Hi has 32 significant bits, so
// k * kLn2Hi is exact for |k| < 2^21); pi/2 = kPio2_1 + kPio2_2 + kPio2_3 (33
// bits each for the first two).
constexpr double kLn2Hi = 0x1.62e42fee00000p-1;
constexpr double kLn2Lo = 0x1.a39ef35793c76p-33;
constexpr double kInvLn2 = 0x1.71547652b82fep+0;
constexpr double kPio2_1 = 0x1.921fb54400000p+0;
constexpr double kPio2_2 = 0x1.0b4611a600000p-34;
constexpr double kPio2_3 = 0x1.3198a2e037073p-69;
constexpr double kTwoOverPi = 0x1.45f306dc9c883p-1;
constexpr double kTwoPi = 0x1.921fb54442d18p+2;
constexpr double kSqrtHalf = 0x1.6a09e667f3bcdp-1;

// Natural logarithm of a positive finite x.
XR_CMA_HD double ln(double x) {
  int e = 0;
  double m = frexp(x, &e);  // x = m 2^e, m in [0.5, 1): exact
  if (m < kSqrtHalf) {
    m = mul(m, 2.0);
    e -= 1;
  }
  const double s = div(sub(m, 1.0), add(m, 1.0));  // |s| <= 0.1716
  const double s2 = mul(s, s);
  // sum_k s2^k / (2k+1), k = 0..14 (the next term is below 1e-23 of the sum)
  double p = 0x1.1a7b9611a7b96p-5;        // 1/29
  p = add(0x1.2f684bda12f68p-5, mul(s2, p));  // 1/27
  p = add(0x1.47ae147ae147bp-5, mul(s2, p));  // 1/25
  p = add(0x1.642c8590b2164p-5, mul(s2, p));  // 1/23
  p = add(0x1.8618618618618p-5, mul(s2, p));  // 1/21
  p = add(0x1.af286bca1af28p-5, mul(s2, p));  // 1/19
  p = add(0x1.e1e1e1e1e1e1ep-5, mul(s2, p));  // 1/17
  p = add(0x1.1111111111111p-4, mul(s2, p));  // 1/15
  p = add(0x1.3b13b13b13b14p-4, mul(s2, p));  // 1/13
  p = add(0x1.745d1745d1746p-4, mul(s2, p));  // 1/11
  p = add(0x1.c71c71c71c71cp-4, mul(s2, p));  // 1/9
  p = add(0x1.2492492492492p-3, mul(s2, p));  // 1/7
  p = add(0x1.999999999999ap-3, mul(s2, p));  // 1/5
  p = add(0x1.5555555555555p-2, mul(s2, p));  // 1/3
  p = add(1.0, mul(s2, p));
  const double lm = mul(mul(2.0, s), p);  // 2 atanh(s) = ln(m)
  const double de = (double)e;
  return add(mul(de, kLn2Hi), add(mul(de, kLn2Lo), lm));
}

// e^y (0 below -745, +inf above 709).
XR_CMA_HD double exp(double y) {
  if (y != y) return y;
  if (y > 709.0) return mul(0x1p1000, 0x1p1000);
  if (y < -745.0) return 0.0;
  const double k = rint(mul(y, kInvLn2));
  const double r = sub(sub(y, mul(k, kLn2Hi)), mul(k, kLn2Lo));  // |r| <= 0.35
  // sum_j r^j / j!, j = 0..20
  double p = 0x1.e542ba4020225p-62;           // 1/20!
  p = add(0x1.2f49b46814157p-57, mul(r, p));  // 1/19!
  p = add(0x1.6827863b97d97p-53, mul(r, p));  // 1/18!
  p = add(0x1.952c77030ad4ap-49, mul(r, p));  // 1/17!
  p = add(0x1.ae7f3e733b81fp-45, mul(r, p));  // 1/16!
  p = add(0x1.ae7f3e733b81fp-41, mul(r, p));  // 1/15!
  p = add(0x1.93974a8c07c9dp-37, mul(r, p));  // 1/14!
  p = add(0x1.6124613a86d09p-33, mul(r, p));  // 1/13!
  p = add(0x1.1eed8eff8d898p-29, mul(r, p));  // 1/12!
  p = add(0x1.ae64567f544e4p-26, mul(r, p));  // 1/11!
  p = add(0x1.27e4fb7789f5cp-22, mul(r, p));  // 1/10!
  p = add(0x1.71de3a556c734p-19, mul(r, p));  // 1/9!
  p = add(0x1.a01a01a01a01ap-16, mul(r, p));  // 1/8!
  p = add(0x1.a01a01a01a01ap-13, mul(r, p));  // 1/7!
  p = add(0x1.6c16c16c16c17p-10, mul(r, p));  // 1/6!
  p = add(0x1.1111111111111p-7, mul(r, p));   // 1/5!
  p = add(0x1.5555555555555p-5, mul(r, p));   // 1/4!
  p = add(0x1.5555555555555p-3, mul(r, p));   // 1/3!
  p = add(0.5, mul(r, p));
  p = add(1.0, mul(r, p));
  p = add(1.0, mul(r, p));
  return ldexp(p, (int)k);
}

// sin x and cos x for |x| below about 1e6.
XR_CMA_HD void sincos(double x, double* sn, double* cs) {
  const double q = rint(mul(x, kTwoOverPi));
  const double r = sub(sub(sub(x, mul(q, kPio2_1)), mul(q, kPio2_2)), mul(q, kPio2_3));  // |r| <= pi/4
  const double r2 = mul(r, r);
  // sin r = r sum_k (-1)^k r2^k / (2k+1)!, cos r = sum_k (-1)^k r2^k / (2k)!, k = 0..10
  double ps = 0x1.71b8ef6dcf572p-66;            // 1/21!
  ps = add(-0x1.2f49b46814157p-57, mul(r2, ps));  // -1/19!
  ps = add(0x1.952c77030ad4ap-49, mul(r2, ps));   // 1/17!
  ps = add(-0x1.ae7f3e733b81fp-41, mul(r2, ps));  // -1/15!
  ps = add(0x1.6124613a86d09p-33, mul(r2, ps));   // 1/13!
  ps = add(-0x1.ae64567f544e4p-26, mul(r2, ps));  // -1/11!
  ps = add(0x1.71de3a556c734p-19, mul(r2, ps));   // 1/9!
  ps = add(-0x1.a01a01a01a01ap-13, mul(r2, ps));  // -1/7!
  ps = add(0x1.1111111111111p-7, mul(r2, ps));    // 1/5!
  ps = add(-0x1.5555555555555p-3, mul(r2, ps));   // -1/3!
  ps = add(1.0, mul(r2, ps));
  const double s = mul(r, ps);
  double pc = 0x1.e542ba4020225p-62;            // 1/20!
  pc = add(-0x1.6827863b97d97p-53, mul(r2, pc));  // -1/18!
  pc = add(0x1.ae7f3e733b81fp-45, mul(r2, pc));   // 1/16!
  pc = add(-0x1.93974a8c07c9dp-37, mul(r2, pc));  // -1/14!
  pc = add(0x1.1eed8eff8d898p-29, mul(r2, pc));   // 1/12!
  pc = add(-0x1.27e4fb7789f5cp-22, mul(r2, pc));  // -1/10!
  pc = add(0x1.a01a01a01a01ap-16, mul(r2, pc));   // 1/8!
  pc = add(-0x1.6c16c16c16c17p-10, mul(r2, pc));  // -1/6!
  pc = add(0x1.5555555555555p-5, mul(r2, pc));    // 1/4!
  pc = add(-0.5, mul(r2, pc));
  const double c = add(1.0, mul(r2, pc));
  switch ((int)((long long)q & 3)) {
    case 0: *sn = s; *cs = c; break;
    case 1: *sn = c; *cs = -s; break;
    case 2: *sn = -s; *cs = -c; break;
    default: *sn = -c; *cs = s; break;
  }
}

}  // namespace dm

namespace cma {

// Counter-based random stream: splitmix64's finaliser chained over the
// counters (S. Vigna's splitmix64; the odd multipliers separate the fields).
XR_CMA_HD uint64_t mix(uint64_t z) {
  z = (z ^ (z >> 30)) * 0xbf58476d1ce4e5b9ull;
  z = (z ^ (z >> 27)) * 0x94d049bb133111ebull;
  return z ^ (z >> 31);
}

// Two standard normals (Box-Muller) for pair `pair` of candidate k's draw
// `attempt` in generation gen.
XR_CMA_HD void normal_pair(uint64_t seed, int64_t gen, int32_t k, int32_t attempt, int32_t pair, double* z0,
                           double* z1) {
  uint64_t h = mix(seed + 0x9e3779b97f4a7c15ull);
  h = mix(h + (uint64_t)gen * 0xd1b54a32d192ed03ull);
  h = mix(h + (uint64_t)(uint32_t)k * 0xaef17502108ef2d9ull);
  h = mix(h + (uint64_t)(uint32_t)attempt * 0x9e6c63d0676a9a99ull);
  h = mix(h + (uint64_t)(uint32_t)pair * 0x8cb92ba72f3d8dd7ull);
  const uint64_t g = mix(h ^ 0x632be59bd9b4e019ull);
  const double u1 = (double)((h >> 11) + 1) * 0x1p-53;  // (0, 1]
  const double u2 = (double)(g >> 11) * 0x1p-53;        // [0, 1)
  const double r = dm::sqrt(dm::mul(-2.0, dm::ln(u1)));
  double s, c;
  dm::sincos(dm::mul(dm::kTwoPi, u2), &s, &c);
  *z0 = dm::mul(r, c);
  *z1 = dm::mul(r, s);
}

// The optimizer state: this header, then (doubles) w[mu] m[n] pc[n] ps[n]
// C[n*n] B[n*n] D[n] best[n] hist[hlen] pop[lam*n] z[lam*n] fv[lam] and the
// update's scratch A[n*n] T[n*n] V[n*n] ys[mu*n] mold[n] yw[n] zw[n] bz[n]
// rot[2n], then (int32) att[lam] idx[lam].  One contiguous block, so it moves
// between host and device memory with one copy.
struct Hdr {
  int32_t n, lam, mu, hlen;
  int32_t hcount, hhead;  // function-value history: entries stored, next slot
  int32_t sampled, reason;
  int32_t sample_error, rotated;  // rotated: the eigen sweep in progress applied a rotation
  int64_t gen, max_iter;
  uint64_t seed;
  double mueff, cs, ds, cc, c1, cmu, chin, sigma, best_f, last_range, tol_fun, tol_x;
};
static_assert(sizeof(Hdr) % 16 == 0, "state header keeps the arrays 16-byte aligned");

struct View {
  Hdr* h;
  double *w, *m, *pc, *ps, *C, *B, *D, *best, *hist, *pop, *z, *fv, *A, *T, *V, *ys, *mold, *yw, *zw, *bz, *rot;
  int32_t *att, *idx;
};

XR_CMA_HD size_t num_doubles(int n, int lam, int mu, int hlen) {
  return (size_t)mu + 3 * (size_t)n + 2 * (size_t)n * n + 2 * (size_t)n + (size_t)hlen + 2 * (size_t)lam * n +
         (size_t)lam + 3 * (size_t)n * n + (size_t)mu * n + 6 * (size_t)n;
}

XR_CMA_HD size_t state_bytes(int n, int lam, int mu, int hlen) {
  return sizeof(Hdr) + 8 * num_doubles(n, lam, mu, hlen) + 8 * (((size_t)2 * lam + 1) / 2);
}

XR_CMA_HD View view(void* base) {
  View v;
  v.h = static_cast<Hdr*>(base);
  const int n = v.h->n, lam = v.h->lam, mu = v.h->mu, hlen = v.h->hlen;
  double* d = reinterpret_cast<double*>(static_cast<unsigned char*>(base) + sizeof(Hdr));
  v.w = d; d += mu;
  v.m = d; d += n;
  v.pc = d; d += n;
  v.ps = d; d += n;
  v.C = d; d += n * n;
  v.B = d; d += n * n;
  v.D = d; d += n;
  v.best = d; d += n;
  v.hist = d; d += hlen;
  v.pop = d; d += lam * n;
  v.z = d; d += lam * n;
  v.fv = d; d += lam;
  v.A = d; d += n * n;
  v.T = d; d += n * n;
  v.V = d; d += n * n;
  v.ys = d; d += mu * n;
  v.mold = d; d += n;
  v.yw = d; d += n;
  v.zw = d; d += n;
  v.bz = d; d += n;
  v.rot = d; d += 2 * n;
  v.att = reinterpret_cast<int32_t*>(d);
  v.idx = v.att + lam;
  return v;
}

// Candidate k's draw number `attempt` of the current generation: z ~ N(0, I)
// and x = m + sigma B D z (B D z summed in column order).
XR_CMA_HD void draw(const View& s, int k, int attempt, double* z, double* x) {
  const Hdr& h = *s.h;
  const int n = h.n;
  for (int i = 0; i < n; i += 2) {
    double a, b;
    normal_pair(h.seed, h.gen, k, attempt, i / 2, &a, &b);
    z[i] = a;
    if (i + 1 < n) z[i + 1] = b;
  }
  for (int i = 0; i < n; ++i) {
    double y = 0.0;
    for (int j = 0; j < n; ++j) y = dm::add(y, dm::mul(dm::mul(s.B[i * n + j], s.D[j]), z[j]));
    x[i] = dm::add(s.m[i], dm::mul(h.sigma, y));
  }
}

// Whether x lies inside the box |x_i| <= bounds[i] (a bound <= 0 leaves x_i free).
XR_CMA_HD bool inside(const double* x, const double* bounds, int n) {
  for (int i = 0; i < n; ++i)
    if (bounds[i] > 0.0 && dm::fabs(x[i]) > bounds[i]) return false;
  return true;
}

// Order-preserving integer key of an objective value: ascending numbers (-0
// as +0), NaN after every number.
XR_CMA_HD uint64_t order_key(double v) {
  if (v != v) return ~0ull;
  if (v == 0.0) v = 0.0;
#ifdef __CUDA_ARCH__
  const uint64_t b = (uint64_t)__double_as_longlong(v);
#else
  uint64_t b;
  std::memcpy(&b, &v, sizeof(b));
#endif
  return (b >> 63) ? ~b : (b | 0x8000000000000000ull);
}

// Eigen-decomposition by Jacobi rotations in round-robin order: each round
// rotates disjoint index pairs, whose parameters all come from the matrix at
// the start of the round; the column updates of every pair come first, then
// the row updates (so a round's elements are independent of one another).
// Pair i of round r (the circle method over N = n rounded up to even; a pair
// with the index n of odd n is idle): *p < *q, false when idle.
XR_CMA_HD bool rr_pair(int n, int r, int i, int* p, int* q) {
  const int N = n + (n & 1), M = N - 1;
  int a, b;
  if (i == 0) {
    a = r;
    b = M;
  } else {
    a = (r + i) % M;
    b = (r - i + M) % M;
  }
  if (a >= n || b >= n) return false;
  *p = a < b ? a : b;
  *q = a < b ? b : a;
  return true;
}
XR_CMA_HD int rr_rounds(int n) { return n + (n & 1) - 1; }
XR_CMA_HD int rr_pairs(int n) { return (n + 1) / 2; }

// Rotation of pair i of round r from A: (c, s) into rot[2i..2i+1]; s = 0 when
// the off-diagonal entry is negligible (below 2^-56 of the two diagonal
// entries); sets *rotated when it is not.
XR_CMA_HD void rot_params(int n, const double* A, int r, int i, double* rot, int32_t* rotated) {
  int p, q;
  rot[2 * i] = 1.0;
  rot[2 * i + 1] = 0.0;
  if (!rr_pair(n, r, i, &p, &q)) return;
  const double apq = A[p * n + q], app = A[p * n + p], aqq = A[q * n + q];
  if (dm::fabs(apq) <= 1e-300 || dm::fabs(apq) <= dm::mul(0x1p-56, dm::add(dm::fabs(app), dm::fabs(aqq)))) return;
  const double theta = dm::div(dm::sub(aqq, app), dm::mul(2.0, apq));
  const double t = dm::div(theta >= 0.0 ? 1.0 : -1.0,
                           dm::add(dm::fabs(theta), dm::sqrt(dm::add(dm::mul(theta, theta), 1.0))));
  const double c = dm::div(1.0, dm::sqrt(dm::add(dm::mul(t, t), 1.0)));
  rot[2 * i] = c;
  rot[2 * i + 1] = dm::mul(t, c);
  *rotated = 1;
}

// Column update (row k of columns p, q) of pair i, in A and in the rotation
// product V.
XR_CMA_HD void rot_cols(int n, double* A, double* V, int r, int i, const double* rot, int k) {
  int p, q;
  const double c = rot[2 * i], s = rot[2 * i + 1];
  if (s == 0.0 || !rr_pair(n, r, i, &p, &q)) return;
  const double akp = A[k * n + p], akq = A[k * n + q];
  A[k * n + p] = dm::sub(dm::mul(c, akp), dm::mul(s, akq));
  A[k * n + q] = dm::add(dm::mul(s, akp), dm::mul(c, akq));
  const double vkp = V[k * n + p], vkq = V[k * n + q];
  V[k * n + p] = dm::sub(dm::mul(c, vkp), dm::mul(s, vkq));
  V[k * n + q] = dm::add(dm::mul(s, vkp), dm::mul(c, vkq));
}

// Row update (column k of rows p, q) of pair i.
XR_CMA_HD void rot_rows(int n, double* A, int r, int i, const double* rot, int k) {
  int p, q;
  const double c = rot[2 * i], s = rot[2 * i + 1];
  if (s == 0.0 || !rr_pair(n, r, i, &p, &q)) return;
  const double apk = A[p * n + k], aqk = A[q * n + k];
  A[p * n + k] = dm::sub(dm::mul(c, apk), dm::mul(s, aqk));
  A[q * n + k] = dm::add(dm::mul(s, apk), dm::mul(c, aqk));
}

// Stop reason: 0 continue, 1 tol_fun, 2 tol_x, 3 max_iter, 4 numerical (sigma not finite).
XR_CMA_HD int32_t termination(const View& s) {
  const Hdr& h = *s.h;
  const int n = h.n;
  if (!(dm::fabs(h.sigma) <= 1.7976931348623157e308)) return 4;
  if (h.gen >= h.max_iter) return 3;
  if (h.gen > 0 && h.last_range <= h.tol_fun) return 1;
  bool small = true;
  for (int i = 0; i < n && small; ++i)
    small = dm::mul(h.sigma, dm::sqrt(s.C[i * n + i])) < h.tol_x && dm::mul(h.sigma, dm::fabs(s.pc[i])) < h.tol_x;
  return (small && h.gen > 0) ? 2 : 0;
}

// One generation's update from the values in s.fv (lambda of them, for the
// candidates in s.pop / s.z): ranking, weighted recombination of the best mu,
// cumulative step-size adaptation, rank-one + rank-mu covariance update with
// the h_sigma stall, new eigen-decomposition, function-value history; the
// termination code after it goes to h.reason.  The stages below are what
// update() runs in order; the ranks, the 2n recombination sums and the
// n(n+1)/2 covariance entries are independent of one another within their
// stage (each summed in the same order wherever it runs), so a device block
// can run them in parallel with the same bits.

// Stage 1 (each k): position of candidate k in the ranking.
XR_CMA_HD void rank(const View& s, int k) {
  const int lam = s.h->lam;
  const uint64_t kk = order_key(s.fv[k]);
  int r = 0;
  for (int j = 0; j < lam; ++j) {
    const uint64_t kj = order_key(s.fv[j]);
    r += (kj < kk || (kj == kk && j < k)) ? 1 : 0;
  }
  s.idx[r] = k;
}

// Stage 2: best value so far; the old mean.
XR_CMA_HD void keep_best(const View& s) {
  Hdr& h = *s.h;
  const int n = h.n, best = s.idx[0];
  if (s.fv[best] < h.best_f) {
    h.best_f = s.fv[best];
    for (int i = 0; i < n; ++i) s.best[i] = s.pop[best * n + i];
  }
  for (int i = 0; i < n; ++i) s.mold[i] = s.m[i];
}

// Stage 3 (each t < 2n): weighted recombination of coordinate t % n of the
// candidates (t < n, the new mean and y_w) or of their draws (t >= n, z_w).
XR_CMA_HD void recombine(const View& s, int t) {
  const Hdr& h = *s.h;
  const int n = h.n, mu = h.mu, i = t % n;
  const double* src = t < n ? s.pop : s.z;
  double a = 0.0;
  for (int k = 0; k < mu; ++k) a = dm::add(a, dm::mul(s.w[k], src[s.idx[k] * n + i]));
  if (t < n) {
    s.m[i] = a;
    s.yw[i] = dm::div(dm::sub(a, s.mold[i]), h.sigma);
  } else {
    s.zw[i] = a;
  }
}

// Stage 4: evolution paths; returns in scal[0] the norm of p_sigma, in
// scal[1] the h_sigma stall factor d_h, in scal[2] 1 - c1 - cmu.
XR_CMA_HD void paths(const View& s, double* scal) {
  Hdr& h = *s.h;
  const int n = h.n;
  for (int i = 0; i < n; ++i) {  // C^{-1/2} y_w = B z_w
    double a = 0.0;
    for (int j = 0; j < n; ++j) a = dm::add(a, dm::mul(s.B[i * n + j], s.zw[j]));
    s.bz[i] = a;
  }
  const double a_s = dm::sqrt(dm::mul(dm::mul(h.cs, dm::sub(2.0, h.cs)), h.mueff));
  double psn = 0.0;
  for (int i = 0; i < n; ++i) {
    s.ps[i] = dm::add(dm::mul(dm::sub(1.0, h.cs), s.ps[i]), dm::mul(a_s, s.bz[i]));
    psn = dm::add(psn, dm::mul(s.ps[i], s.ps[i]));
  }
  psn = dm::sqrt(psn);
  h.gen += 1;
  const double hthr = dm::mul(dm::add(1.4, dm::div(2.0, dm::add((double)n, 1.0))), h.chin);
  // (1 - cs)^(2 gen) as exp(2 gen ln(1 - cs))
  const double decay = dm::exp(dm::mul(dm::mul(2.0, (double)h.gen), dm::ln(dm::sub(1.0, h.cs))));
  const double hsig = dm::div(psn, dm::sqrt(dm::sub(1.0, decay))) < hthr ? 1.0 : 0.0;
  const double a_c = dm::sqrt(dm::mul(dm::mul(h.cc, dm::sub(2.0, h.cc)), h.mueff));
  for (int i = 0; i < n; ++i)
    s.pc[i] = dm::add(dm::mul(dm::sub(1.0, h.cc), s.pc[i]), dm::mul(dm::mul(hsig, a_c), s.yw[i]));
  scal[0] = psn;
  scal[1] = dm::mul(dm::mul(dm::sub(1.0, hsig), h.cc), dm::sub(2.0, h.cc));
  scal[2] = dm::sub(dm::sub(1.0, h.c1), h.cmu);
}

// Stage 5 (each t < mu n): step (x_k - m_old) / sigma of coordinate t % n of
// the (t / n)-th best candidate.
XR_CMA_HD void steps(const View& s, int t) {
  const Hdr& h = *s.h;
  const int n = h.n, k = t / n, i = t % n;
  s.ys[t] = dm::div(dm::sub(s.pop[s.idx[k] * n + i], s.mold[i]), h.sigma);
}

// Stage 6 (each e < n(n+1)/2, the lower triangle row by row): covariance
// entry (i, j), j <= i, and its mirror.  Reads only its own old entry.
XR_CMA_HD void tri(int e, int* i, int* j) {
  int r = 0;
  while ((r + 1) * (r + 2) / 2 <= e) ++r;
  *i = r;
  *j = e - r * (r + 1) / 2;
}
XR_CMA_HD void covariance(const View& s, int e, const double* scal) {
  const Hdr& h = *s.h;
  const int n = h.n, mu = h.mu;
  int i, j;
  tri(e, &i, &j);
  double rmu = 0.0;
  for (int k = 0; k < mu; ++k) rmu = dm::add(rmu, dm::mul(dm::mul(s.w[k], s.ys[k * n + i]), s.ys[k * n + j]));
  const double cij = s.C[i * n + j];
  const double v = dm::add(dm::add(dm::mul(scal[2], cij),
                                   dm::mul(h.c1, dm::add(dm::mul(s.pc[i], s.pc[j]), dm::mul(scal[1], cij)))),
                           dm::mul(h.cmu, rmu));
  s.C[i * n + j] = v;
  s.C[j * n + i] = v;
}

// Stage 7: the step size.
XR_CMA_HD void step_size(const View& s, const double* scal) {
  Hdr& h = *s.h;
  h.sigma = dm::mul(h.sigma, dm::exp(dm::mul(dm::div(h.cs, h.ds), dm::sub(dm::div(scal[0], h.chin), 1.0))));
}

// Stage 8, the eigen-decomposition of C warm-started from the last basis B:
// (a, each e < n n) T = C B; (b, each e < n(n+1)/2) A = B^T T, lower triangle
// mirrored, and V = I; then Jacobi sweeps on A (rot_params, rot_cols,
// rot_rows per round) until a sweep rotates nothing; (c, each e < n n)
// T = B V; (d, each e < n n) B = T.
XR_CMA_HD void eig_cb(const View& s, int e) {
  const int n = s.h->n, i = e / n, j = e % n;
  double a = 0.0;
  for (int k = 0; k < n; ++k) a = dm::add(a, dm::mul(s.C[i * n + k], s.B[k * n + j]));
  s.T[e] = a;
}
XR_CMA_HD void eig_btcb(const View& s, int e) {
  const int n = s.h->n;
  int i, j;
  tri(e, &i, &j);
  double a = 0.0;
  for (int k = 0; k < n; ++k) a = dm::add(a, dm::mul(s.B[k * n + i], s.T[k * n + j]));
  s.A[i * n + j] = a;
  s.A[j * n + i] = a;
  s.V[i * n + j] = i == j ? 1.0 : 0.0;
  s.V[j * n + i] = i == j ? 1.0 : 0.0;
}
XR_CMA_HD void eig_bv(const View& s, int e) {
  const int n = s.h->n, i = e / n, j = e % n;
  double a = 0.0;
  for (int k = 0; k < n; ++k) a = dm::add(a, dm::mul(s.B[i * n + k], s.V[k * n + j]));
  s.T[e] = a;
}

// Stage 9: D from the eigenvalues, history, termination code.
XR_CMA_HD void finish(const View& s) {
  Hdr& h = *s.h;
  const int n = h.n, lam = h.lam;
  const double* f = s.fv;
  for (int i = 0; i < n; ++i) {
    const double d = s.A[i * n + i];
    s.D[i] = dm::sqrt(d > 1e-300 ? d : 1e-300);
  }
  // best value of the last hlen generations (the TolFun test's range)
  const int best = s.idx[0];
  s.hist[h.hhead] = f[best];
  h.hhead = (h.hhead + 1) % h.hlen;
  if (h.hcount < h.hlen) h.hcount += 1;
  double lo = f[best], hi = f[s.idx[lam - 1]];
  for (int i = 0; i < h.hcount; ++i) {
    lo = s.hist[i] < lo ? s.hist[i] : lo;
    hi = s.hist[i] > hi ? s.hist[i] : hi;
  }
  h.last_range = dm::sub(hi, lo);
  h.sampled = 0;
  h.reason = termination(s);
}

constexpr int kMaxSweeps = 64;

XR_CMA_HD void update(const View& s) {
  const int n = s.h->n, lam = s.h->lam, mu = s.h->mu;
  double scal[3];
  for (int k = 0; k < lam; ++k) rank(s, k);
  keep_best(s);
  for (int t = 0; t < 2 * n; ++t) recombine(s, t);
  paths(s, scal);
  for (int t = 0; t < mu * n; ++t) steps(s, t);
  for (int e = 0; e < n * (n + 1) / 2; ++e) covariance(s, e, scal);
  step_size(s, scal);
  for (int e = 0; e < n * n; ++e) eig_cb(s, e);
  for (int e = 0; e < n * (n + 1) / 2; ++e) eig_btcb(s, e);
  for (int sweep = 0; sweep < kMaxSweeps; ++sweep) {
    s.h->rotated = 0;
    for (int r = 0; r < rr_rounds(n); ++r) {
      for (int i = 0; i < rr_pairs(n); ++i) rot_params(n, s.A, r, i, s.rot, &s.h->rotated);
      for (int i = 0; i < rr_pairs(n); ++i)
        for (int k = 0; k < n; ++k) rot_cols(n, s.A, s.V, r, i, s.rot, k);
      for (int i = 0; i < rr_pairs(n); ++i)
        for (int k = 0; k < n; ++k) rot_rows(n, s.A, r, i, s.rot, k);
    }
    if (!s.h->rotated) break;
  }
  for (int e = 0; e < n * n; ++e) eig_bv(s, e);
  for (int e = 0; e < n * n; ++e) s.B[e] = s.T[e];
  finish(s);
}

}  // namespace cma

namespace pose {

// out = a b for 4 x 4 row-major matrices (each entry summed over k in order).
XR_CMA_HD void mat_mul4(const double* a, const double* b, double* out) {
  double t[16];
  for (int i = 0; i < 4; ++i)
    for (int j = 0; j < 4; ++j) {
      double s = 0.0;
      for (int k = 0; k < 4; ++k) s = dm::add(s, dm::mul(a[i * 4 + k], b[k * 4 + j]));
      t[i * 4 + j] = s;
    }
  for (int i = 0; i < 16; ++i) out[i] = t[i];
}

// ExpSE3 (xregRigidUtils.cpp:40-85) of x = [w, v]: theta = |w|,
// R = I + a W + b W^2, t = (I + b W + c W^2) v with a = sin(theta) / theta,
// b = (1 - cos(theta)) / theta^2, c = (theta - sin(theta)) / theta^3; R = I,
// t = v for theta <= 1e-14.
XR_CMA_HD void exp_se3(const double* x, double* out) {
  const double w0 = x[0], w1 = x[1], w2 = x[2];
  const double th = dm::sqrt(dm::add(dm::add(dm::mul(w0, w0), dm::mul(w1, w1)), dm::mul(w2, w2)));
  const double W[9] = {0.0, -w2, w1, w2, 0.0, -w0, -w1, w0, 0.0};
  double WW[9];
  for (int i = 0; i < 3; ++i)
    for (int j = 0; j < 3; ++j) {
      double s = 0.0;
      for (int k = 0; k < 3; ++k) s = dm::add(s, dm::mul(W[i * 3 + k], W[k * 3 + j]));
      WW[i * 3 + j] = s;
    }
  const bool big = th > 1.0e-14;
  double sn = 0.0, cs = 1.0;
  if (big) dm::sincos(th, &sn, &cs);
  const double th2 = dm::mul(th, th);
  const double a = big ? dm::div(sn, th) : 1.0;
  const double b = big ? dm::div(dm::sub(1.0, cs), th2) : 0.0;
  const double c = big ? dm::div(dm::sub(th, sn), dm::mul(th2, th)) : 0.0;
  double R[9], A[9];
  for (int i = 0; i < 9; ++i) {
    const double id = (i % 4 == 0) ? 1.0 : 0.0;
    R[i] = big ? dm::add(dm::add(id, dm::mul(a, W[i])), dm::mul(b, WW[i])) : id;
    A[i] = big ? dm::add(dm::add(id, dm::mul(b, W[i])), dm::mul(c, WW[i])) : id;
  }
  for (int i = 0; i < 16; ++i) out[i] = 0.0;
  for (int i = 0; i < 3; ++i) {
    for (int j = 0; j < 3; ++j) out[i * 4 + j] = R[i * 3 + j];
    out[i * 4 + 3] = dm::add(dm::add(dm::mul(A[i * 3 + 0], x[3]), dm::mul(A[i * 3 + 1], x[4])),
                             dm::mul(A[i * 3 + 2], x[5]));
  }
  out[15] = 1.0;
}

// Inverse of a rigid transform [R t; 0 1]: [R^T, -R^T t].
XR_CMA_HD void rigid_inverse(const double* m, double* out) {
  double t[16];
  for (int i = 0; i < 16; ++i) t[i] = 0.0;
  for (int i = 0; i < 3; ++i)
    for (int j = 0; j < 3; ++j) t[i * 4 + j] = m[j * 4 + i];
  for (int i = 0; i < 3; ++i)
    t[i * 4 + 3] = -dm::add(dm::add(dm::mul(t[i * 4 + 0], m[3]), dm::mul(t[i * 4 + 1], m[7])),
                            dm::mul(t[i * 4 + 2], m[11]));
  t[15] = 1.0;
  for (int i = 0; i < 16; ++i) out[i] = t[i];
}

// The pose of offset x in a registration level: C Exp(x) B, with B = C^-1 start.
XR_CMA_HD void map(const double* C, const double* B, const double* x, double* out) {
  double E[16], CE[16];
  exp_se3(x, E);
  mat_mul4(C, E, CE);
  mat_mul4(CE, B, out);
}

}  // namespace pose
}  // namespace xr
