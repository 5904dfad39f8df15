// xr_posespread.h -- how far a population of poses spreads over a volume, in
// voxels (host code; decides whether a job's DRR items are pose-grouped).
#pragma once

#include <algorithm>
#include <cmath>
#include <cstdint>

#include "xreg_gb300.h"

namespace xr {

// Largest displacement of a volume corner (voxel centres 0 and n-1 on each
// axis, through the volume's origin, direction and spacing) between pose 0 and
// any other pose, in units of the smallest spacing.  poses: pop row-major 4x4
// cam -> ITK-physical rigid transforms; a corner's camera coordinates are
// inverse(pose) applied to its physical point.  pop < 2 gives 0.
inline double pose_spread_voxels(const xr_volume_desc& d, const double* poses, int64_t pop) {
  const double* sp = d.spacing;
  const double vmin = std::min(sp[0], std::min(sp[1], sp[2]));
  double corners[8][3];
  for (int c = 0; c < 8; ++c)
    for (int a = 0; a < 3; ++a) {
      double s = d.origin[a];
      for (int b = 0; b < 3; ++b) s += d.direction[a * 3 + b] * (((c >> b) & 1) ? (double)(d.n[b] - 1) : 0.0) * sp[b];
      corners[c][a] = s;
    }
  // rigid inverse: R^T and -R^T t
  auto inv = [](const double* p, double* R, double* t) {
    for (int r = 0; r < 3; ++r)
      for (int c = 0; c < 3; ++c) R[r * 3 + c] = p[c * 4 + r];
    for (int r = 0; r < 3; ++r) t[r] = -(R[r * 3] * p[3] + R[r * 3 + 1] * p[7] + R[r * 3 + 2] * p[11]);
  };
  double R0[9], t0[3], best = 0.0;
  inv(poses, R0, t0);
  for (int64_t k = 1; k < pop; ++k) {
    double Rk[9], tk[3];
    inv(poses + 16 * k, Rk, tk);
    for (const auto& x : corners) {
      double d2 = 0.0;
      for (int r = 0; r < 3; ++r) {
        const double u = Rk[r * 3] * x[0] + Rk[r * 3 + 1] * x[1] + Rk[r * 3 + 2] * x[2] + tk[r];
        const double v = R0[r * 3] * x[0] + R0[r * 3 + 1] * x[1] + R0[r * 3 + 2] * x[2] + t0[r];
        d2 += (u - v) * (u - v);
      }
      best = std::max(best, std::sqrt(d2));
    }
  }
  return best / vmin;
}

// The same bound for a device CMA-ES's next population: 3 sigma of its largest
// rotation (radians) and translation (mm) standard deviations, the rotation
// acting at the volume's half diagonal, in units of the smallest spacing.
inline double sampled_spread_voxels(const xr_volume_desc& d, double sd_rot, double sd_trans) {
  const double* sp = d.spacing;
  const double vmin = std::min(sp[0], std::min(sp[1], sp[2]));
  double r2 = 0.0;
  for (int a = 0; a < 3; ++a) {
    const double h = 0.5 * (double)d.n[a] * sp[a];
    r2 += h * h;
  }
  return 3.0 * (sd_trans + sd_rot * std::sqrt(r2)) / vmin;
}

}  // namespace xr
