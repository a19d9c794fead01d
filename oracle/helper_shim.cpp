// C entry points over a Helper and a DataCube implementation (test
// infrastructure), compiled twice: into oracle/_ref/libbirp_ref.so against
// the reference's own classes (oracle/build_ref.sh, where the reference tree
// is present) and by tests/test_helper_parity.py and
// tests/test_loader_parity.py against birp_cpp_gb300's, so the two are
// compared on the same inputs through ctypes.
#include <stdexcept>
#include <string>
#include <vector>

#include "DataCube.h"
#include "Helper.h"

float DateToJulianDate(int year, int month, float day);

namespace {
std::vector<std::vector<float>> mat(const float* m, int rows, int cols) {
  std::vector<std::vector<float>> out(rows, std::vector<float>(cols));
  for (int i = 0; i < rows; ++i)
    for (int j = 0; j < cols; ++j) out[i][j] = m[i * cols + j];
  return out;
}
void put(const std::vector<std::vector<float>>& m, float* out) {
  int k = 0;
  for (const auto& r : m)
    for (float v : r) out[k++] = v;
}
void put(const std::vector<float>& v, float* out) {
  for (size_t i = 0; i < v.size(); ++i) out[i] = v[i];
}
}  // namespace

extern "C" {

float h_julian(int y, int m, float d) { return DateToJulianDate(y, m, d); }
void h_gei2gse(float* out16) { put(Helper::Gei2GseTransforms(), out16); }
void h_radec_gsi(float ra, float dec, float* out3) { put(Helper::RaDecToGSI(ra, dec), out3); }
void h_radec_gse(float ra, float dec, float* out3) {
  put(Helper::RaDecGSEConversion({ra, dec}, Helper::Gei2GseTransforms()), out3);
}
void h_spherical(const float* xyz, int alt, float* out3) {
  float p[3] = {xyz[0], xyz[1], xyz[2]};
  put(alt ? Helper::XYZToSphericalAlt(p) : Helper::XYZToSpherical(p), out3);
}
void h_distance(const float* xyz, float* out2) {
  float p[3] = {xyz[0], xyz[1], xyz[2]};
  out2[0] = Helper::VectorDistance(p);
  out2[1] = Helper::VectorDistance2D(p);
}
void h_interp1(const float* x, const float* y, int n, const float* xn, int m, float* out) {
  std::vector<float> xv(x, x + n), yv(y, y + n), q(xn, xn + m);
  put(Helper::Interp1(xv, yv, q), out);
}
int h_nearest(float v, const float* x, int n) {
  std::vector<float> xv(x, x + n);
  return Helper::findNearestNeighbourIndex(v, xv);
}
int h_inverse(const float* m, int n, float* out) {
  try {
    put(Helper::GetInverse(mat(m, n, n)), out);
    return 0;
  } catch (const std::runtime_error&) {
    return 1;
  }
}
int h_det(const float* m, int rows, int cols, float* out) {
  try {
    *out = Helper::GetDeterminant(mat(m, rows, cols));
    return 0;
  } catch (const std::runtime_error&) {
    return 1;
  }
}
void h_matmul(const float* a, const float* b, int n, float* out) { put(Helper::MatrixMultiply(mat(a, n, n), mat(b, n, n)), out); }
void h_matvec(const float* a, int rows, int cols, const float* b, float* out4) {
  put(Helper::MatrixMultiply(mat(a, rows, cols), std::vector<float>(b, b + cols)), out4);
}
void h_rotate(const float* r9, const float* c3, float* out3) {
  float c[3] = {c3[0], c3[1], c3[2]};
  put(Helper::ApplyRotation(mat(r9, 3, 3), c), out3);
}
void h_two_min(const float* arr, int n, const int* mask, int nm, float* out2) {
  put(Helper::TwoMin(std::vector<float>(arr, arr + n), std::vector<int>(mask, mask + nm)), out2);
}
void h_xy_radec(float cx, float cy, const float* xs, const float* ys, const float* s1, const float* s2, int n,
                float sep, float* out2) {
  put(Helper::XYToRaDec(cx, cy, std::vector<float>(xs, xs + n), std::vector<float>(ys, ys + n),
                        std::vector<float>(s1, s1 + n), std::vector<float>(s2, s2 + n), sep),
      out2);
}
int h_explode_float(const char* s, char delim, float* out, int cap) {
  const std::vector<float> v = Helper::explode_float(s, delim);
  for (size_t i = 0; i < v.size() && (int)i < cap; ++i) out[i] = v[i];
  return (int)v.size();
}
int h_equal_distance(const float* steps, int n) { return Helper::EqualDistance(std::vector<float>(steps, steps + n)); }

}  // extern "C"

extern "C" {

// DataCube::Load of `path` through this build's DataCube: 0 with dims, the
// axes (x, y, z concatenated, at most axes_cap) and the x-fastest values (at
// most cap) copied out; 1 std::invalid_argument, 2 std::out_of_range, 3 any
// other exception, 4 too many values or slices not of the axes' shape.
int h_cube_load(const char* path, int* dims, float* axes, int axes_cap, float* vals, long cap) {
  try {
    DataCube c;
    c.Load(std::string(path), false);
    const std::vector<float>* ax[3] = {&c.coords_x, &c.coords_y, &c.coords_z};
    int o = 0;
    for (int k = 0; k < 3; ++k) {
      dims[k] = (int)ax[k]->size();
      if (o + dims[k] > axes_cap) return 4;
      for (float v : *ax[k]) axes[o++] = v;
    }
    const size_t nx = dims[0], ny = dims[1], nz = dims[2];
    if ((long)(nx * ny * nz) > cap || c.slices.size() < nz) return 4;
    size_t i = 0;
    for (size_t k = 0; k < nz; ++k) {
      if (c.slices[k].size() != ny) return 4;
      for (size_t j = 0; j < ny; ++j) {
        if (c.slices[k][j].size() != nx) return 4;
        for (size_t x = 0; x < nx; ++x) vals[i++] = c.slices[k][j][x];
      }
    }
    return 0;
  } catch (const std::out_of_range&) {
    return 2;
  } catch (const std::invalid_argument&) {
    return 1;
  } catch (...) {
    return 3;
  }
}

}  // extern "C"
