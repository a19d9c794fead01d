// The C++ drop-in classes' host-only parts: the .dat loader and the FITS
// writer (no GPU is touched). argv[1] = output directory.
#include <cstdio>
#include <fstream>
#include <string>
#include <vector>

#include "birp/Camera.h"
#include "birp/Cmem.h"
#include "birp/DataCube.h"

int main(int argc, char** argv) {
  std::string dir = argc > 1 ? argv[1] : ".";
  int fails = 0;
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
