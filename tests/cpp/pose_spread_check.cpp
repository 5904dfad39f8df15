// Reads a volume description and poses from a binary file and prints the
// spread estimates of xr_posespread.h (checked against numpy by
// tests/test_pose_spread_cpu.py).
#include <cstdio>
#include <vector>

#include "xr_posespread.h"

int main(int argc, char** argv) {
  if (argc != 3) return 2;
  std::FILE* f = std::fopen(argv[1], "rb");
  if (!f) return 2;
  // n[3], spacing[3], origin[3], direction[9], pop, sd_rot, sd_trans, poses[pop*16] (all double)
  double head[21];
  if (std::fread(head, sizeof(double), 21, f) != 21) return 2;
  xr_volume_desc d{};
  for (int a = 0; a < 3; ++a) {
    d.n[a] = (int64_t)head[a];
    d.spacing[a] = head[3 + a];
    d.origin[a] = head[6 + a];
  }
  for (int k = 0; k < 9; ++k) d.direction[k] = head[9 + k];
  const int64_t pop = (int64_t)head[18];
  std::vector<double> poses((size_t)pop * 16);
  if (std::fread(poses.data(), sizeof(double), poses.size(), f) != poses.size()) return 2;
  std::fclose(f);
  const double out[2] = {xr::pose_spread_voxels(d, poses.data(), pop), xr::sampled_spread_voxels(d, head[19], head[20])};
  std::FILE* g = std::fopen(argv[2], "wb");
  if (!g) return 2;
  std::fwrite(out, sizeof(double), 2, g);
  std::fclose(g);
  return 0;
}
