// xr_io.cpp -- poses on disk in ITK's text transform format.
//
// xReg writes a registered pose with WriteITKAffineTransform
// (lib/itk/xregITKIOUtils.cpp:226-241: an itk::AffineTransform<float, 3> with
// the pose's upper 3x3 as matrix and its last column as offset, centre 0,
// through itk::TransformFileWriter) and reads one with
// ReadITKAffineTransformFromFile (xregITKIOUtils.cpp:157-224: exactly one
// linear, non-composite transform whose class is an AffineTransform or a
// MatrixOffsetTransformBase, in double or float; the pose is its matrix and
// offset).  ReadSlicerAffineTransformFromFile (xregITKIOUtils.cpp:33-36) is the
// inverse of that.  ITK picks the file format by extension; this implements the
// text one (".txt", ".tfm"), whose layout ITK documents:
//
//   #Insight Transform File V1.0
//   #Transform 0
//   Transform: AffineTransform_float_3_3
//   Parameters: A00 A01 A02 A10 A11 A12 A20 A21 A22 T0 T1 T2
//   FixedParameters: C0 C1 C2
//
// The parameters are the matrix row by row and the translation T; the fixed
// parameters are the centre C, and the offset is T + C - A C (formed here in
// double, then rounded to float as xReg stores poses).  HDF5 (".h5",
// ".hdf5") and MATLAB (".mat") transform files need libraries that are not part
// of this build and are refused with XR_ERR_UNSUPPORTED.
#include <cctype>
#include <cerrno>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <vector>

#include "xreg_gb300.h"
#include "xreg_gb300_io.h"

namespace xr {
xr_status fail(xr_status code, const std::string& msg);
}  // namespace xr

namespace {

std::string lower_ext(const std::string& path) {
  const size_t slash = path.find_last_of("/\\");
  const size_t dot = path.find_last_of('.');
  if (dot == std::string::npos || (slash != std::string::npos && dot < slash)) return "";
  std::string e = path.substr(dot);
  for (char& c : e) c = (char)std::tolower((unsigned char)c);
  return e;
}

xr_status check_text_path(const char* fn, const std::string& path) {
  const std::string e = lower_ext(path);
  if (e == ".txt" || e == ".tfm") return XR_OK;
  if (e == ".h5" || e == ".hdf5" || e == ".mat")
    return xr::fail(XR_ERR_UNSUPPORTED, std::string(fn) + ": " + e +
                                            " transform files need a library this build does not have; use .txt or .tfm");
  return xr::fail(XR_ERR_INVALID_ARG, std::string(fn) + ": unknown transform file extension '" + e + "'");
}

std::string trim(const std::string& s) {
  size_t a = 0, b = s.size();
  while (a < b && std::isspace((unsigned char)s[a])) ++a;
  while (b > a && std::isspace((unsigned char)s[b - 1])) --b;
  return s.substr(a, b - a);
}

bool parse_numbers(const std::string& s, std::vector<double>* out) {
  out->clear();
  const char* p = s.c_str();
  for (;;) {
    while (*p && std::isspace((unsigned char)*p)) ++p;
    if (!*p) return true;
    char* end = nullptr;
    errno = 0;
    const double v = std::strtod(p, &end);
    if (end == p || errno == ERANGE) return false;
    out->push_back(v);
    p = end;
  }
}

struct TxtTransform {
  std::string cls;
  std::vector<double> params, fixed;
  bool has_params = false, has_fixed = false;
};

// Splits the file into its transforms ("Transform:" starts one).
xr_status read_transforms(const std::string& path, std::vector<TxtTransform>* out) {
  FILE* f = std::fopen(path.c_str(), "rb");
  if (!f) return xr::fail(XR_ERR_INVALID_ARG, "read_itk_affine_transform: cannot open " + path);
  std::string text;
  char buf[4096];
  size_t n;
  while ((n = std::fread(buf, 1, sizeof(buf), f)) > 0) text.append(buf, n);
  std::fclose(f);
  size_t pos = 0;
  bool header = false;
  while (pos <= text.size()) {
    size_t nl = text.find('\n', pos);
    if (nl == std::string::npos) nl = text.size();
    const std::string line = trim(text.substr(pos, nl - pos));
    pos = nl + 1;
    if (line.empty()) continue;
    if (line[0] == '#') {
      if (line.rfind("#Insight Transform File", 0) == 0) header = true;
      continue;
    }
    const size_t colon = line.find(':');
    if (colon == std::string::npos)
      return xr::fail(XR_ERR_INVALID_ARG, "read_itk_affine_transform: unexpected line '" + line + "' in " + path);
    const std::string key = trim(line.substr(0, colon)), val = trim(line.substr(colon + 1));
    if (key == "Transform") {
      out->push_back(TxtTransform{});
      out->back().cls = val;
    } else if (key == "Parameters" || key == "FixedParameters") {
      if (out->empty())
        return xr::fail(XR_ERR_INVALID_ARG, "read_itk_affine_transform: parameters before a transform in " + path);
      std::vector<double> v;
      if (!parse_numbers(val, &v))
        return xr::fail(XR_ERR_INVALID_ARG, "read_itk_affine_transform: bad number in '" + line + "'");
      if (key == "Parameters") {
        out->back().params = v;
        out->back().has_params = true;
      } else {
        out->back().fixed = v;
        out->back().has_fixed = true;
      }
    } else {
      return xr::fail(XR_ERR_INVALID_ARG, "read_itk_affine_transform: unknown key '" + key + "' in " + path);
    }
  }
  if (!header && !out->empty())
    return xr::fail(XR_ERR_INVALID_ARG, "read_itk_affine_transform: missing '#Insight Transform File' header in " + path);
  return XR_OK;
}

// 4x4 row-major inverse of an affine transform [A t; 0 1] (general A).
bool affine_inverse(const double* m, double* out) {
  const double a = m[0], b = m[1], c = m[2], d = m[4], e = m[5], f = m[6], g = m[8], h = m[9], k = m[10];
  const double A = e * k - f * h, B = -(d * k - f * g), C = d * h - e * g;
  const double det = a * A + b * B + c * C;
  if (!(std::fabs(det) > 0.0) || !std::isfinite(det)) return false;
  const double inv[9] = {A / det, -(b * k - c * h) / det, (b * f - c * e) / det,
                         B / det, (a * k - c * g) / det, -(a * f - c * d) / det,
                         C / det, -(a * h - b * g) / det, (a * e - b * d) / det};
  for (int r = 0; r < 3; ++r) {
    for (int col = 0; col < 3; ++col) out[r * 4 + col] = inv[r * 3 + col];
    out[r * 4 + 3] = -(inv[r * 3] * m[3] + inv[r * 3 + 1] * m[7] + inv[r * 3 + 2] * m[11]);
  }
  out[12] = out[13] = out[14] = 0.0;
  out[15] = 1.0;
  return true;
}

}  // namespace

using xr::fail;

extern "C" XR_API xr_status xr_itk_affine_transform_read(const char* path, double* xform) {
  if (!path || !xform) return fail(XR_ERR_INVALID_ARG, "read_itk_affine_transform: NULL argument");
  const std::string p(path);
  xr_status st = check_text_path("read_itk_affine_transform", p);
  if (st != XR_OK) return st;
  std::vector<TxtTransform> ts;
  if ((st = read_transforms(p, &ts)) != XR_OK) return st;
  if (ts.empty()) return fail(XR_ERR_INVALID_ARG, "read_itk_affine_transform: Transform file is empty!");
  if (ts.size() > 1)
    return fail(XR_ERR_INVALID_ARG, "read_itk_affine_transform: Transform file with multiple transforms is not supported!");
  const TxtTransform& t = ts[0];
  if (t.cls.find("CompositeTransform") != std::string::npos)
    return fail(XR_ERR_UNSUPPORTED, "read_itk_affine_transform: Composite transforms are not supported!");
  // the classes xReg accepts: AffineTransform and MatrixOffsetTransformBase, double or float, 3 -> 3
  // (xReg's dynamic_cast also admits MatrixOffsetTransformBase subclasses such as
  // Euler3DTransform, whose own parameterisations are not read here)
  const bool known = t.cls == "AffineTransform_double_3_3" || t.cls == "AffineTransform_float_3_3" ||
                     t.cls == "MatrixOffsetTransformBase_double_3_3" || t.cls == "MatrixOffsetTransformBase_float_3_3";
  if (!known) return fail(XR_ERR_UNSUPPORTED, "read_itk_affine_transform: Unsupported ITK transform class! (" + t.cls + ")");
  if (!t.has_params || t.params.size() != 12)
    return fail(XR_ERR_INVALID_ARG, "read_itk_affine_transform: an affine transform needs 12 parameters");
  double c[3] = {0.0, 0.0, 0.0};
  if (t.has_fixed) {
    if (t.fixed.size() != 3)
      return fail(XR_ERR_INVALID_ARG, "read_itk_affine_transform: an affine transform needs 3 fixed parameters");
    for (int i = 0; i < 3; ++i) c[i] = t.fixed[(size_t)i];
  }
  for (double v : t.params)
    if (!std::isfinite(v)) return fail(XR_ERR_INVALID_ARG, "read_itk_affine_transform: non-finite parameter");
  for (int r = 0; r < 3; ++r) {
    double off = t.params[(size_t)(9 + r)] + c[r];
    for (int k = 0; k < 3; ++k) {
      const double a = t.params[(size_t)(r * 3 + k)];
      xform[r * 4 + k] = a;
      off -= a * c[k];
    }
    xform[r * 4 + 3] = off;
  }
  // xReg casts matrix and offset to its CoordScalar, float (xregITKIOUtils.cpp:43-82)
  for (int i = 0; i < 12; ++i) xform[i] = (double)(float)xform[i];
  xform[12] = xform[13] = xform[14] = 0.0;
  xform[15] = 1.0;
  return XR_OK;
}

extern "C" XR_API xr_status xr_itk_slicer_affine_transform_read(const char* path, double* xform) {
  if (!xform) return fail(XR_ERR_INVALID_ARG, "read_slicer_affine_transform: NULL argument");
  double m[16];
  const xr_status st = xr_itk_affine_transform_read(path, m);
  if (st != XR_OK) return st;
  if (!affine_inverse(m, xform)) return fail(XR_ERR_INVALID_ARG, "read_slicer_affine_transform: singular matrix");
  return XR_OK;
}

extern "C" XR_API xr_status xr_itk_affine_transform_write(const char* path, const double* xform) {
  if (!path || !xform) return fail(XR_ERR_INVALID_ARG, "write_itk_affine_transform: NULL argument");
  const std::string p(path);
  xr_status st = check_text_path("write_itk_affine_transform", p);
  if (st != XR_OK) return st;
  for (int i = 0; i < 12; ++i)
    if (!std::isfinite(xform[i])) return fail(XR_ERR_INVALID_ARG, "write_itk_affine_transform: non-finite pose");
  FILE* f = std::fopen(p.c_str(), "wb");
  if (!f) return fail(XR_ERR_INVALID_ARG, "write_itk_affine_transform: cannot create " + p);
  // xReg's CoordScalar is float: an AffineTransform<float, 3>, centre 0, so the
  // translation parameters are the offset; 9 significant digits round-trip a float
  std::string s = "#Insight Transform File V1.0\n#Transform 0\nTransform: AffineTransform_float_3_3\nParameters:";
  char num[64];
  for (int r = 0; r < 3; ++r)
    for (int k = 0; k < 3; ++k) {
      std::snprintf(num, sizeof(num), " %.9g", (double)(float)xform[r * 4 + k]);
      s += num;
    }
  for (int r = 0; r < 3; ++r) {
    std::snprintf(num, sizeof(num), " %.9g", (double)(float)xform[r * 4 + 3]);
    s += num;
  }
  s += "\nFixedParameters: 0 0 0\n";
  const bool ok = std::fwrite(s.data(), 1, s.size(), f) == s.size();
  const bool closed = std::fclose(f) == 0;
  if (!ok || !closed) return fail(XR_ERR_INVALID_ARG, "write_itk_affine_transform: write failed for " + p);
  return XR_OK;
}
