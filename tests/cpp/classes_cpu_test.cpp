// The C++ drop-in classes' host-only parts: the .dat loader, a cube sampled
// from a user-defined Space, and the FITS writer (no GPU is touched).
// argv[1] = output directory.
#include <cmath>
#include <cstdio>
#include <cstring>
#include <fstream>
#include <stdexcept>
#include <string>
#include <vector>

#include "birp/Camera.h"
#include "birp/Cmem.h"
#include "birp/DataCube.h"

// A user-defined Space, as the reference's tests define one (CubeFake in
// tests/Camera_test.cpp:25-29 returns 1): here an affine field, -1 outside a
// slab, as the reference's spaces mark their outside.
class AffineSpace : public Space {
 public:
  void Init() override {}
  float GetSample(float x, float y, float z) override { return z > 2.5f ? -1.f : 1.f + 0.5f * x - 0.25f * y + z; }
};

static void write_cube(const std::string& path, const std::string& dims_and_body) {
  std::ofstream f(path);
  f << "meta\n";
  for (int i = 2; i < 10; ++i) f << "#\n";
  f << dims_and_body;
}

// 0 if loading `body` succeeds, 1 on std::invalid_argument, 2 on std::out_of_range
static int load_outcome(const std::string& dir, const std::string& body, DataCube& c) {
  std::string path = dir + "/tok.dat";
  write_cube(path, body);
  try {
    c.Load(path, false);
  } catch (const std::out_of_range&) {
    return 2;
  } catch (const std::invalid_argument&) {
    return 1;
  }
  return 0;
}

// Tokens read as the reference reads them (std::stof of each white-space
// separated token): the leading number counts, trailing characters do not;
// a token without a number is invalid, an out-of-range number out_of_range.
static int loader_tokens(const std::string& dir) {
  int fails = 0;
  const std::string axes = "2 2 2\n0 1\n0 1\n0 1\n";
  DataCube c;
  fails += load_outcome(dir, axes + "+1.5 2.5abc 3e0 -4 nan inf 0x1p3 1.5E+00-2.5E+00\n", c) != 0;
  fails += !(c.slices[0][0][0] == 1.5f && c.slices[0][0][1] == 2.5f && c.slices[0][1][0] == 3.f &&
             c.slices[0][1][1] == -4.f && std::isnan(c.slices[1][0][0]) && std::isinf(c.slices[1][0][1]) &&
             c.slices[1][1][0] == 8.f && c.slices[1][1][1] == 1.5f);
  DataCube d1, d2, d3;
  fails += load_outcome(dir, axes + "1 2 3 4 5 6 7 abc\n", d1) != 1;
  fails += load_outcome(dir, axes + "1 2 3 4 5 6 7 1e400\n", d2) != 2;
  fails += load_outcome(dir, axes + "1 2 3 4 5 6 7\n", d3) != 1;  // one value short
  // the multi-threaded path (chunks split at white space): 2^21 values written
  // with 9 significant digits read back exactly
  {
    const int n = 128;
    std::string path = dir + "/big.dat";
    std::ofstream f(path);
    f << "meta\n";
    for (int i = 2; i < 10; ++i) f << "#\n";
    f << n << " " << n << " " << n << "\n";
    for (int k = 0; k < 3; ++k) {
      for (int i = 0; i < n; ++i) f << i << (i + 1 < n ? " " : "\n");
    }
    std::vector<float> want((size_t)n * n * n);
    char buf[32];
    for (size_t i = 0; i < want.size(); ++i) {
      want[i] = (float)std::sin(0.001 * (double)i) * 1e3f + (float)(i % 7);
      std::snprintf(buf, sizeof buf, "%.9g", want[i]);
      f << buf << ((i % 128 == 127) ? "\n" : "  ");
    }
    f.close();
    DataCube b;
    b.Load(path, false);
    size_t bad = 0, i = 0;
    for (int z = 0; z < n; ++z)
      for (int y = 0; y < n; ++y)
        for (int x = 0; x < n; ++x, ++i) bad += std::memcmp(&b.slices[z][y][x], &want[i], 4) != 0;
    fails += bad != 0;
  }
  return fails;
}

int main(int argc, char** argv) {
  std::string dir = argc > 1 ? argv[1] : ".";
  int fails = loader_tokens(dir);
  // a cube in the reference's text format, values spread over ragged lines
  {
    std::ofstream f(dir + "/t.dat");
    f << "meta\n";
    for (int i = 2; i < 10; ++i) f << "#\n";
    f << "3 2 2\n-1 0\n1\n5 6\n7.5 8.5\n1 2 3\n4 5\n6\n\n7 8 9\n10 11 12\n";
  }
  DataCube c;
  std::string path = dir + "/t.dat";
  c.Init(path, false);
  fails += !(c.size.x == 3 && c.size.y == 2 && c.size.z == 2);
  fails += !(c.coords_x[2] == 1.f && c.coords_y[1] == 6.f && c.coords_z[0] == 7.5f);
  fails += !(c.spacing[0] == 1.f && c.spacing[2] == 1.f && c.origin_coords[1] == 5.f);
  fails += !(c.slices[0][0][0] == 1.f && c.slices[0][1][2] == 6.f && c.slices[1][1][2] == 12.f);
  bool threw = false;
  try {
    DataCube bad;
    std::string missing = dir + "/missing.dat";
    bad.Load(missing, false);
  } catch (const std::invalid_argument&) {
    threw = true;
  }
  fails += !threw;
  // a user-defined Space sampled at the nodes (one and several host threads:
  // the same values), GetSample's -1 kept
  {
    AffineSpace src;
    const std::vector<double> xs = {-2, -1, 0.5, 3}, ys = {-1, 1, 2}, zs = {0, 1, 2, 3, 4};
    DataCube one, many;
    one.InitFromSpace(src, xs, ys, zs);
    many.InitFromSpace(src, xs, ys, zs, 3);
    fails += !(one.size.x == 4 && one.size.y == 3 && one.size.z == 5);
    for (size_t k = 0; k < zs.size(); ++k)
      for (size_t j = 0; j < ys.size(); ++j)
        for (size_t i = 0; i < xs.size(); ++i) {
          const float want = src.GetSample((float)xs[i], (float)ys[j], (float)zs[k]);
          fails += one.slices[k][j][i] != want;
          fails += many.slices[k][j][i] != want;
        }
    fails += one.slices[4][0][0] != -1.f;
    bool self = false;
    try {
      one.InitFromSpace(one, xs, ys, zs);
    } catch (const std::invalid_argument&) {
      self = true;
    }
    fails += !self;
  }
  // FITS output of a known image
  CMEM m;  // not initialised: no GPU use
  Camera cam(m, 1.0f, 3.0f, 4.0f);
  for (int j = 0; j < 3; ++j)
    for (int i = 0; i < 4; ++i) cam.image[j][i] = 10.f * j + i + 0.5f;
  float x = 1.5f, y = -2.f, z = 3.f;
  cam.SetPosition(x, y, z);
  cam.SetAim(7.f, 0.f, 0.f);
  fails += cam.ToFITS(dir + "/t") != 1;
  fails += cam.ToDat(dir + "/t") != 1;
  std::printf("%d failures\n", fails);
  return fails;
}
