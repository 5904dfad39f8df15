// Evaluates the host side of xr_cmaes_core.h on doubles read from a file, for
// tests/test_detmath_cpu.py:  detmath_check <mode> <in.f64> <out.f64>
//   ln, exp: one output per input; sincos: sin then cos per input;
//   normals: inputs (seed, gen, k, attempt, pair) as doubles -> two normals;
//   posemap: inputs C[16] B[16] then x[6] rows -> 16 doubles per row.
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <vector>

#include "xr_cmaes_core.h"

static std::vector<double> read_all(const char* path) {
  std::vector<double> v;
  FILE* f = std::fopen(path, "rb");
  if (!f) return v;
  double x;
  while (std::fread(&x, sizeof(double), 1, f) == 1) v.push_back(x);
  std::fclose(f);
  return v;
}

int main(int argc, char** argv) {
  if (argc != 4) return 2;
  const std::vector<double> in = read_all(argv[2]);
  std::vector<double> out;
  const char* mode = argv[1];
  if (!std::strcmp(mode, "ln")) {
    for (double x : in) out.push_back(xr::dm::ln(x));
  } else if (!std::strcmp(mode, "exp")) {
    for (double x : in) out.push_back(xr::dm::exp(x));
  } else if (!std::strcmp(mode, "sincos")) {
    for (double x : in) {
      double s, c;
      xr::dm::sincos(x, &s, &c);
      out.push_back(s);
      out.push_back(c);
    }
  } else if (!std::strcmp(mode, "normals")) {
    for (size_t i = 0; i + 5 <= in.size(); i += 5) {
      double a, b;
      xr::cma::normal_pair((uint64_t)in[i], (int64_t)in[i + 1], (int32_t)in[i + 2], (int32_t)in[i + 3],
                           (int32_t)in[i + 4], &a, &b);
      out.push_back(a);
      out.push_back(b);
    }
  } else if (!std::strcmp(mode, "posemap")) {
    if (in.size() < 32) return 3;
    for (size_t i = 32; i + 6 <= in.size(); i += 6) {
      double p[16];
      xr::pose::map(in.data(), in.data() + 16, in.data() + i, p);
      out.insert(out.end(), p, p + 16);
    }
  } else {
    return 4;
  }
  FILE* f = std::fopen(argv[3], "wb");
  if (!f) return 5;
  std::fwrite(out.data(), sizeof(double), out.size(), f);
  std::fclose(f);
  return 0;
}
