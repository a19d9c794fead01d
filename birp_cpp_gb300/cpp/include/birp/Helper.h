// Drop-in for the reference's Helper (include/Helper.h, src/Helper.cpp): the
// small FP32 math and string helpers code written against the reference
// calls — matrix products and the 3x3 inverse of the camera pose, vector
// lengths, spherical coordinates, 1-D interpolation, and the pointing
// helpers (Julian date, GEI -> GSE rotation, RA/Dec to GEI/GSE unit vectors,
// sky-grid pixel -> RA/Dec). Same names, signatures, argument meaning and
// results, including the reference's quirks (noted per function). The GPU
// render path does not use these (it has its own FP64 pose).
#pragma once
#include <algorithm>
#include <cctype>
#include <string>
#include <vector>

class Helper {
 public:
  // in-place trims of leading / trailing white space
  static void ltrim(std::string& s) {
    s.erase(s.begin(), std::find_if(s.begin(), s.end(), [](unsigned char ch) { return !std::isspace(ch); }));
  }
  static void rtrim(std::string& s) {
    s.erase(std::find_if(s.rbegin(), s.rend(), [](unsigned char ch) { return !std::isspace(ch); }).base(), s.end());
  }
  static void trim(std::string& s) {
    rtrim(s);
    ltrim(s);
  }
  static bool ends_with(std::string const& value, std::string const& ending) {
    return ending.size() <= value.size() && std::equal(ending.rbegin(), ending.rend(), value.rbegin());
  }

  // split on delim, empty tokens dropped (std::stof / std::stoi per token)
  static std::vector<float> explode_float(std::string const& s, char delim);
  static std::vector<int> explode_int(std::string const& s, char delim);
  static std::vector<std::string> explode_string(std::string const& s, char delim);

  // a (n x n) times b: result[i][j] = sum_{k < a.size()} a[i][k] b[k][j] for
  // j < b.size() (square operands, as the reference assumes)
  static std::vector<std::vector<float>> MatrixMultiply(std::vector<std::vector<float>> a,
                                                        std::vector<std::vector<float>> b);
  // a (rows x cols, rows <= 4) times the vector b; always 4 entries (zero
  // beyond a's rows), as the reference's fixed result array
  static std::vector<float> MatrixMultiply(std::vector<std::vector<float>> a, std::vector<float> b);
  static std::vector<std::vector<float>> MatrixScalarMultiply(std::vector<std::vector<float>>, float);
  static std::vector<float> MatrixScalarMultiply(std::vector<float>, float);
  // each row of rot (first 3 entries) dotted with coords[0..2]
  static std::vector<float> ApplyRotation(std::vector<std::vector<float>> rot, float* coords);
  // cofactor inverse; std::runtime_error "Determinant is 0" when singular
  static std::vector<std::vector<float>> GetInverse(const std::vector<std::vector<float>> vect);
  // Laplace expansion along the first row; std::runtime_error "Matrix is not
  // quadratic" unless square; 1 for 0 x 0
  static float GetDeterminant(const std::vector<std::vector<float>> vect);
  static std::vector<std::vector<float>> GetTranspose(const std::vector<std::vector<float>> matrix1);
  static std::vector<std::vector<float>> GetCofactor(const std::vector<std::vector<float>> vect);

  // 4x4 GEI -> GSE rotation (Sun longitude and obliquity) for the fixed date
  // 2024-01-01 the reference uses
  static std::vector<std::vector<float>> Gei2GseTransforms();
  // unit GEI vector of right ascension / declination (degrees), with the
  // reference's quadrant rule (x < 0 for 90 < ra < 270, y < 0 for
  // 180 < ra < 270, the bounds exclusive)
  static std::vector<float> RaDecToGSI(float ra, float dec);
  // RaDecToGSI rotated by a 4x4 GEI -> GSE matrix; 3 entries
  static std::vector<float> RaDecGSEConversion(std::vector<float>, std::vector<std::vector<float>>);
  // indices (as floats) of the two smallest arr entries: entries 0 and 1,
  // then those i in [2, size-2] listed in mask
  static std::vector<float> TwoMin(std::vector<float>, std::vector<int>);
  // RA/Dec of image point (ct_x, ct_y) from a sky grid (xsky, ysky: grid
  // points in the image; sky1, sky2: their RA / Dec; skysep: grid step)
  static std::vector<float> XYToRaDec(float, float, std::vector<float>, std::vector<float>, std::vector<float>,
                                      std::vector<float>, float);
  // piecewise-linear y(x_new) from the segment whose left node is the nearest
  // node strictly below x_new (findNearestNeighbourIndex; -1 when none)
  static std::vector<float> Interp1(std::vector<float>& x, std::vector<float>& y, std::vector<float> x_new);
  static int findNearestNeighbourIndex(float value, std::vector<float>& x);
  // {phi = atan2(y, x), theta = atan2(sqrt(x^2 + y^2), z), r}
  static std::vector<float> XYZToSpherical(float*);
  // {atan2(z, sqrt(x^2 + y^2)), atan2(y, x), r}
  static std::vector<float> XYZToSphericalAlt(float*);
  static float VectorDistance(float* xyz);
  static float VectorDistance2D(float* xy);
  // the reference's check compares iterators, not the steps, so it is true
  // for every input (src/Helper.cpp:603-623); kept so callers see the same
  static bool EqualDistance(std::vector<float> steps);
};

// Julian date of (year, month, day) with the Gregorian switch on 1582-10-15,
// in the reference's float arithmetic (src/Helper.cpp:266-302).
float DateToJulianDate(int year, int month, float day);
