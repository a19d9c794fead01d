// Helper (see birp/Helper.h): the reference's host-side math and string
// helpers (src/Helper.cpp) with the same results in FP32, restated. Where the
// FP32 result depends on the order of operations or on float/double
// promotions (the Julian date, whose value near 2.46e6 has 0.25-day float
// resolution, and the GEI -> GSE angles), that order is the reference's.
#include "../include/birp/Helper.h"

#include <cfloat>
#include <cmath>
#include <sstream>
#include <stdexcept>

namespace {

constexpr double kPi = 3.14159265358979323846;

template <class T, class Conv>
std::vector<T> split(const std::string& s, char delim, Conv conv) {
  std::vector<T> out;
  std::istringstream in(s);
  std::string tok;
  while (std::getline(in, tok, delim))
    if (!tok.empty()) out.push_back(conv(tok));
  return out;
}

// square check shared by the determinant and the cofactors
void require_square(const std::vector<std::vector<float>>& m) {
  if (!m.empty() && m.size() != m[0].size()) throw std::runtime_error("Matrix is not quadratic");
}

// m without row r and column c
std::vector<std::vector<float>> minor_of(const std::vector<std::vector<float>>& m, size_t r, size_t c) {
  std::vector<std::vector<float>> out;
  out.reserve(m.size() - 1);
  for (size_t i = 0; i < m.size(); ++i) {
    if (i == r) continue;
    std::vector<float> row;
    row.reserve(m.size() - 1);
    for (size_t j = 0; j < m.size(); ++j)
      if (j != c) row.push_back(m[i][j]);
    out.push_back(std::move(row));
  }
  return out;
}

}  // namespace

std::vector<float> Helper::explode_float(std::string const& s, char delim) {
  return split<float>(s, delim, [](const std::string& t) { return std::stof(t); });
}

std::vector<int> Helper::explode_int(std::string const& s, char delim) {
  return split<int>(s, delim, [](const std::string& t) { return std::stoi(t); });
}

std::vector<std::string> Helper::explode_string(std::string const& s, char delim) {
  return split<std::string>(s, delim, [](const std::string& t) { return t; });
}

std::vector<std::vector<float>> Helper::MatrixMultiply(std::vector<std::vector<float>> a,
                                                       std::vector<std::vector<float>> b) {
  std::vector<std::vector<float>> out(a.size(), std::vector<float>(b.size(), 0.f));
  for (size_t i = 0; i < a.size(); ++i)
    for (size_t j = 0; j < b.size(); ++j) {
      float acc = 0.f;
      for (size_t k = 0; k < a.size(); ++k) acc = acc + a[i][k] * b[k][j];
      out[i][j] = acc;
    }
  return out;
}

std::vector<float> Helper::MatrixMultiply(std::vector<std::vector<float>> a, std::vector<float> b) {
  std::vector<float> out(4, 0.f);
  const size_t rows = std::min<size_t>(a.size(), 4);
  for (size_t r = 0; r < rows; ++r)
    for (size_t c = 0; c < a[0].size(); ++c) out[r] += a[r][c] * b[c];
  return out;
}

std::vector<std::vector<float>> Helper::MatrixScalarMultiply(std::vector<std::vector<float>> matrix, float scalar) {
  for (auto& row : matrix)
    for (float& v : row) v = v * scalar;
  return matrix;
}

std::vector<float> Helper::MatrixScalarMultiply(std::vector<float> matrix, float scalar) {
  for (float& v : matrix) v = v * scalar;
  return matrix;
}

std::vector<float> Helper::ApplyRotation(std::vector<std::vector<float>> rot, float* coords) {
  std::vector<float> out;
  out.reserve(rot.size());
  for (const auto& r : rot) out.push_back((r[0] * coords[0]) + (r[1] * coords[1]) + (r[2] * coords[2]));
  return out;
}

float Helper::GetDeterminant(const std::vector<std::vector<float>> vect) {
  require_square(vect);
  const size_t n = vect.size();
  if (n == 0) return 1.f;
  if (n == 1) return vect[0][0];
  if (n == 2) return vect[0][0] * vect[1][1] - vect[0][1] * vect[1][0];
  float det = 0.f;
  int sign = 1;
  for (size_t c = 0; c < n; ++c, sign = -sign) det = det + sign * vect[0][c] * GetDeterminant(minor_of(vect, 0, c));
  return det;
}

std::vector<std::vector<float>> Helper::GetTranspose(const std::vector<std::vector<float>> matrix1) {
  std::vector<std::vector<float>> out(matrix1[0].size(), std::vector<float>(matrix1.size()));
  for (size_t i = 0; i < matrix1.size(); ++i)
    for (size_t j = 0; j < matrix1[0].size(); ++j) out[j][i] = matrix1[i][j];
  return out;
}

std::vector<std::vector<float>> Helper::GetCofactor(const std::vector<std::vector<float>> vect) {
  require_square(vect);
  const size_t n = vect.size();
  std::vector<std::vector<float>> out(n, std::vector<float>(n));
  for (size_t i = 0; i < n; ++i)
    for (size_t j = 0; j < n; ++j) out[i][j] = ((i + j) % 2 ? -1.f : 1.f) * GetDeterminant(minor_of(vect, i, j));
  return out;
}

std::vector<std::vector<float>> Helper::GetInverse(const std::vector<std::vector<float>> vect) {
  const float det = GetDeterminant(vect);
  if (det == 0) throw std::runtime_error("Determinant is 0");
  const float d = 1.f / det;
  std::vector<std::vector<float>> out = GetTranspose(GetCofactor(vect));  // the adjugate
  for (auto& row : out)
    for (float& v : row) v *= d;
  return out;
}

float DateToJulianDate(int year, int month, float day) {
  // January and February count as months 13 and 14 of the previous year
  const bool jan_feb = month == 1 || month == 2;
  const int yp = jan_feb ? year - 1 : year;
  const int mp = jan_feb ? month + 12 : month;
  const bool julian_calendar =
      year < 1582 || (year == 1582 && month < 10) || (year == 1582 && month == 10 && day < 15);
  int b = 0;
  if (!julian_calendar) {
    const int a = (int)std::trunc(yp / 100.f);
    b = 2 - a + (int)std::trunc(a / 4.f);
  }
  // (the reference's year term for negative years uses 356.25)
  const int c = yp < 0 ? (int)std::trunc((356.25 * yp) - 0.75) : (int)std::trunc(365.25 * yp);
  const int d = (int)std::trunc(30.6001 * (mp + 1));
  return b + c + d + day + 1720994.5f;
}

std::vector<std::vector<float>> Helper::Gei2GseTransforms() {
  const float rad = kPi / 180;
  float mjd = DateToJulianDate(2024, 1, 1);
  mjd = mjd - 2400000.5f;                   // days from 1858-11-17
  const float t0 = (mjd - 51544.5f) / 36525;  // Julian centuries from J2000
  const float obliquity = 23.439f - 0.013f * t0;
  const float anomaly = 357.528 + 35999.050f * t0;
  const float mean_lon = 280.460 + 36000.772 * t0;
  const float sun_lon =
      mean_lon + (1.915 - 0.0048 * t0) * std::sin(anomaly * rad) + 0.020f * std::sin((2 * anomaly) * rad);
  const float cl = std::cos(sun_lon * rad), sl = std::sin(sun_lon * rad);
  const float ce = std::cos(obliquity * rad), se = std::sin(obliquity * rad);
  const std::vector<std::vector<float>> about_z = {{cl, sl, 0, 0}, {-sl, cl, 0, 0}, {0, 0, 1, 0}, {0, 0, 0, 1}};
  const std::vector<std::vector<float>> about_x = {{1, 0, 0, 0}, {0, ce, se, 0}, {0, -se, ce, 0}, {0, 0, 0, 1}};
  return MatrixMultiply(about_z, about_x);
}

std::vector<float> Helper::RaDecToGSI(float ra, float dec) {
  const float rad = kPi / 180;
  const float a = ra * rad, dl = dec * rad;
  const float z = std::sin(dl);
  const float yy = std::max(1 - z * z, 0.f);
  const float t = std::tan(a);
  float y = std::sqrt(yy) * t / std::sqrt(1 + t * t);
  float x = std::sqrt(std::max(1 - y * y - z * z, 0.f));
  if (90 < ra && ra < 180) {
    x = -std::abs(x);
    y = std::abs(y);
  } else if (180 < ra && ra < 270) {
    x = -std::abs(x);
    y = -std::abs(y);
  }
  return {x, y, z};
}

std::vector<float> Helper::RaDecGSEConversion(std::vector<float> ra_dec, std::vector<std::vector<float>> gei_to_gse) {
  std::vector<float> v = RaDecToGSI(ra_dec[0], ra_dec[1]);
  v.push_back(1.f);
  std::vector<float> out = MatrixMultiply(gei_to_gse, v);
  out.pop_back();
  return out;
}

std::vector<float> Helper::TwoMin(std::vector<float> arr, std::vector<int> mask) {
  int first = 0, second = 1;
  if (arr[1] < arr[0]) std::swap(first, second);
  for (int i = 2; i + 1 < (int)arr.size(); ++i) {
    if (std::find(mask.begin(), mask.end(), i) == mask.end()) continue;
    if (arr[i] < arr[first]) {
      second = first;
      first = i;
    } else if (arr[i] < arr[second]) {
      second = i;
    }
  }
  return {(float)first, (float)second};
}

std::vector<float> Helper::XYToRaDec(float ct_x, float ct_y, std::vector<float> xsky, std::vector<float> ysky,
                                     std::vector<float> sky1, std::vector<float> sky2, float skysep) {
  const float deg = 180 / kPi;
  std::vector<float> dist(xsky.size());
  for (size_t i = 0; i < xsky.size(); ++i)
    dist[i] = std::sqrt(((ct_x - xsky[i]) * (ct_x - xsky[i])) + ((ct_y - ysky[i]) * (ct_y - ysky[i])));
  const size_t near = std::min_element(dist.begin(), dist.end()) - dist.begin();
  // the two grid points nearest the target among those sharing the nearest
  // point's RA (their Dec difference) and its Dec (their RA difference)
  auto two_nearest_with = [&](const std::vector<float>& key) {
    std::vector<int> sel;
    for (size_t i = 0; i < key.size(); ++i)
      if (key[i] == key[near]) sel.push_back((int)i);
    const std::vector<float> two = TwoMin(dist, sel);
    return std::make_pair((size_t)two[0], (size_t)two[1]);
  };
  const auto [p0, p1] = two_nearest_with(sky1);
  const float diff_dec = sky2[p1] - sky2[p0];
  const float diff_x = xsky[p1] - xsky[p0], diff_y = ysky[p1] - ysky[p0];
  const auto [q0, q1] = two_nearest_with(sky2);
  float diff_ra = sky1[q1] - sky1[q0];
  const float diff_x2 = xsky[q1] - xsky[q0], diff_y2 = ysky[q1] - ysky[q0];

  const float d_ang = deg * std::atan2(diff_y, diff_x);
  const float c_ang = deg * std::atan2((ct_y - ysky[near]), (ct_x - xsky[near]));
  float ct_dec = sky2[near] + ((diff_dec / skysep) * (dist[near] * std::cos((d_ang - c_ang) / deg)));
  ct_dec = std::min(std::max(ct_dec, -90.f), 90.f);
  // an RA step across 0/360 counts as one grid step
  if (diff_ra == (skysep - 360.f)) diff_ra = skysep;
  else if (diff_ra == (360.f - skysep)) diff_ra = -1.f * skysep;
  const float d2_ang = deg * std::atan2(diff_y2, diff_x2);
  float ct_ra = sky1[near];
  if (std::cos(ct_dec / deg) != 0)
    ct_ra = sky1[near] + ((diff_ra / (1.f * skysep)) * (dist[near] * std::cos((d2_ang - c_ang) / deg)) /
                          std::cos(ct_dec / deg));
  if (ct_ra < 0) ct_ra = ct_ra + 360.f;
  else if (ct_ra > 360) ct_ra = ct_ra - 360.f;
  return {ct_ra, ct_dec};
}

int Helper::findNearestNeighbourIndex(float value, std::vector<float>& x) {
  float best = FLT_MAX;
  int idx = -1;
  for (int i = 0; i < (int)x.size(); ++i) {
    const float gap = value - x[i];
    if (gap > 0 && gap < best) {
      best = gap;
      idx = i;
    }
  }
  return idx;
}

std::vector<float> Helper::Interp1(std::vector<float>& x, std::vector<float>& y, std::vector<float> x_new) {
  // per node: the line through it and the next node (the last node reuses
  // the segment before it)
  const size_t n = x.size();
  std::vector<float> slope(n), icept(n);
  for (size_t i = 0; i + 1 < n; ++i) {
    slope[i] = (y[i + 1] - y[i]) / (x[i + 1] - x[i]);
    icept[i] = y[i] - x[i] * slope[i];
  }
  if (n >= 2) {
    slope[n - 1] = slope[n - 2];
    icept[n - 1] = icept[n - 2];
  }
  std::vector<float> out;
  out.reserve(x_new.size());
  for (float v : x_new) {
    // no node strictly below v: the reference then reads before its table;
    // here the first segment is used
    const int idx = std::max(findNearestNeighbourIndex(v, x), 0);
    out.push_back(slope[idx] * v + icept[idx]);
  }
  return out;
}

std::vector<float> Helper::XYZToSpherical(float* xyz) {
  const float x = xyz[0], y = xyz[1], z = xyz[2];
  const float r = std::sqrt(x * x + y * y + z * z);
  return {std::atan2(y, x), std::atan2(std::sqrt(x * x + y * y), z), r};
}

std::vector<float> Helper::XYZToSphericalAlt(float* xyz) {
  const float x = xyz[0], y = xyz[1], z = xyz[2];
  const float r = std::sqrt(x * x + y * y + z * z);
  return {std::atan2(z, std::sqrt(x * x + y * y)), std::atan2(y, x), r};
}

float Helper::VectorDistance(float* xyz) { return std::sqrt(xyz[0] * xyz[0] + xyz[1] * xyz[1] + xyz[2] * xyz[2]); }

float Helper::VectorDistance2D(float* xy) { return std::sqrt(xy[0] * xy[0] + xy[1] * xy[1]); }

bool Helper::EqualDistance(std::vector<float>) { return true; }
