// C++ drop-in classes (Space / DataCube / CMEM / Camera) exercised the way the
// reference's own tests do (tests/CMEM_test.cpp, tests/DataCube_test.cpp,
// tests/Camera_test.cpp), without GTest: each CHECK failure is printed and
// the exit code is the number of failures. argv[1] = output directory.
#include <cmath>
#include <cstdio>
#include <fstream>
#include <functional>
#include <string>
#include <thread>
#include <vector>

#include "birp/Camera.h"
#include "birp/Cmem.h"
#include "birp/DataCube.h"

static int failures = 0;
#define CHECK(cond)                                                   \
  do {                                                                \
    if (!(cond)) {                                                    \
      std::printf("FAIL %s:%d: %s\n", __FILE__, __LINE__, #cond);     \
      ++failures;                                                     \
    }                                                                 \
  } while (0)

static bool near(float a, float b, float rel) { return std::fabs(a - b) <= rel * std::fabs(b) || a == b; }

static void cmem_basic() {
  CMEM* cmem = new CMEM();
  cmem->Init();
  CHECK(cmem->GetSample(8.f, 4.f, 4.f) == 0.f);
  CHECK(near(cmem->GetSample(4.f, 12.f, 10.f), 4.46853346e-06f, 2e-6f));
  CHECK(cmem->GetSample(3.f, 1.5f, 1.2f) == 0.f);
  CHECK(near(cmem->GetSample(8.f, 10.f, 10.f), 8.15947317e-07f, 2e-6f));
  CHECK(near(cmem->GetSample(8.f, -10.f, -10.f), 8.15947317e-07f, 2e-6f));
  CHECK(near(cmem->GetSample(8.f, 10.f, -10.f), 8.15947317e-07f, 2e-6f));
  delete cmem;
}

static void cmem_init_params() {
  std::vector<int> v = {400, 0, 0}, b = {0, 0, 4};
  float dipole = 0.f;
  int p1 = 1, p2 = 4, p3 = 6;
  float B = 3.f, alpha = 3.6f, beta = -1.0f;
  CMEM* cmem = new CMEM();
  cmem->Init(true, v, b, dipole, p1, p2, p3, B, alpha, beta);  // the reference test's shifted call
  CHECK(cmem->GetSample(8.f, 4.f, 4.f) == 0.f);
  CHECK(near(cmem->GetSample(12.f, 12.f, 10.f), 4.57952495e-07f, 2e-6f));
  CHECK(cmem->GetSample(3.f, 1.5f, 1.2f) == 0.f);
  CHECK(near(cmem->GetSample(12.f, 10.f, 10.f), 5.48567925e-07f, 2e-6f));
  CHECK(near(cmem->GetSample(12.f, -10.f, -10.f), 5.48567925e-07f, 2e-6f));
  delete cmem;
}

// Writes a cube in the exported-MHD text format the reference loads.
static void write_dat(const std::string& path, const std::vector<float>& xs, const std::vector<float>& ys,
                      const std::vector<float>& zs, const std::vector<float>& v) {
  std::ofstream f(path);
  f << "synthetic cube\n";
  for (int i = 2; i < 10; ++i) f << "# header line " << i << "\n";
  f << xs.size() << " " << ys.size() << " " << zs.size() << "\n";
  for (auto* ax : {&xs, &ys, &zs}) {
    for (size_t i = 0; i < ax->size(); ++i) f << (*ax)[i] << ((i % 6 == 5) ? "\n" : " ");
    f << "\n";
  }
  size_t nx = xs.size(), ny = ys.size(), nz = zs.size();
  for (size_t k = 0; k < nz; ++k) {
    for (size_t j = 0; j < ny; ++j) {
      for (size_t i = 0; i < nx; ++i) f << "  " << v[(k * ny + j) * nx + i];
      f << "\n";
    }
    f << "\n";
  }
}

static void datacube(const std::string& dir) {
  std::vector<float> xs, ys, zs, v;
  for (int i = 0; i < 11; ++i) xs.push_back(-5.f + i);
  for (int i = 0; i < 9; ++i) ys.push_back(-4.f + i);
  for (int i = 0; i < 7; ++i) zs.push_back(-3.f + i);
  for (int k = 0; k < 7; ++k)
    for (int j = 0; j < 9; ++j)
      for (int i = 0; i < 11; ++i) v.push_back(0.25f * i + 2.0f * j + 8.0f * k);
  std::string path = dir + "/cube.dat";
  write_dat(path, xs, ys, zs, v);
  DataCube* cube = new DataCube;
  cube->Init(path, false);
  CHECK(cube->size.x == 11 && cube->size.y == 9 && cube->size.z == 7);
  CHECK(cube->spacing[0] == 1.f && cube->origin_coords[2] == -3.f);
  cube->SetTrilinear(false);
  // nearest by truncation: node (6, 4, 3) at (1.7, 0.3, 0.9) -> i=6,j=4,k=3
  CHECK(cube->GetSample(1.7f, 0.3f, 0.9f) == 0.25f * 6 + 2.0f * 4 + 8.0f * 3);
  CHECK(cube->GetSample(-6.f, 0.f, 0.f) == -1.f);   // outside: -1
  CHECK(cube->GetSample(5.f, 0.f, 0.f) == -1.f);    // the last node is outside [c0, c_{n-1})
  cube->SetTrilinear(true);
  // the field is linear, so trilinear interpolation is exact
  float x = 1.7f, y = 0.3f, z = 0.9f;
  float want = 0.25f * (x + 5) + 2.0f * (y + 4) + 8.0f * (z + 3);
  CHECK(near(cube->GetSample(x, y, z), want, 1e-6f));
  delete cube;
}

static void camera_files_and_accumulation(const std::string& dir) {
  CMEM cmem;
  cmem.Init();
  float pixel_size_deg = 0.25f, fov_h = 36.f, fov_w = 36.f;
  Camera camera(cmem, pixel_size_deg, fov_h, fov_w);
  CHECK(camera.Width() == 144 && camera.Height() == 144);
  float x = 5.91813f, y = 6.74116f, z = 17.7067f;
  camera.SetPosition(x, y, z);
  camera.SetAim(7.81768f, 0, 0);
  camera.Render();
  camera.ToDat(dir + "/cmem_cli_default");
  camera.ToFITS(dir + "/cmem_cli_default");
  std::vector<std::vector<float>> once = camera.image;
  camera.Render();  // the reference accumulates
  int doubled = 0, total = 0;
  for (int j = 0; j < 144; ++j)
    for (int i = 0; i < 144; ++i) {
      ++total;
      doubled += camera.image[j][i] == once[j][i] + once[j][i];
    }
  CHECK(doubled == total);
  FILE* f = std::fopen((dir + "/cmem_cli_default.dat").c_str(), "r");
  CHECK(f != nullptr);
  if (f) std::fclose(f);
  f = std::fopen((dir + "/cmem_cli_default.fits").c_str(), "rb");
  CHECK(f != nullptr);
  if (f) {
    std::fseek(f, 0, SEEK_END);
    long n = std::ftell(f);
    CHECK(n % 2880 == 0 && n >= 2880 + 144 * 144 * 4);
    std::fclose(f);
  }
  // a cube render with explicit dims, step and CLIP mode
  std::vector<double> xs, ys, zs;
  for (int i = 0; i < 40; ++i) xs.push_back(-10 + 30.0 * i / 39);
  for (int i = 0; i < 32; ++i) ys.push_back(-15 + 30.0 * i / 31);
  for (int i = 0; i < 24; ++i) zs.push_back(-15 + 30.0 * i / 23);
  std::vector<float> vals(40 * 32 * 24, 1.0f);
  DataCube cube;
  cube.Init(xs, ys, zs, vals);
  cube.SetTrilinear(true);
  Camera cam2(cube, 16.f, 27.f, 48, 28);
  float px = -2, py = -12, pz = 16;
  cam2.SetPosition(px, py, pz);
  cam2.SetAim(10, 0, 0);
  cam2.SetStep(0.1);
  cam2.SetMarchMode(1);
  cam2.Render();
  cam2.ToDat(dir + "/cube_clip");
  float mx = 0;
  for (auto& row : cam2.image)
    for (float v : row) mx = std::fmax(mx, v);
  CHECK(mx > 0);
}

// Cameras on several threads sharing one read-only cube (the reference's
// threading model: GetSample has no side effects): the same images as one
// after another.
static void concurrent_cameras() {
  std::vector<double> xs, ys, zs;
  for (int i = 0; i < 48; ++i) xs.push_back(-10 + 30.0 * i / 47);
  for (int i = 0; i < 40; ++i) ys.push_back(-15 + 30.0 * i / 39);
  for (int i = 0; i < 36; ++i) zs.push_back(-15 + 30.0 * i / 35);
  std::vector<float> vals;
  for (int k = 0; k < 36; ++k)
    for (int j = 0; j < 40; ++j)
      for (int i = 0; i < 48; ++i) vals.push_back(1.0f + 0.01f * ((i * 7 + j * 13 + k * 29) % 97));
  DataCube cube;
  cube.Init(xs, ys, zs, vals);
  cube.SetTrilinear(true);
  const int n = 8;
  std::vector<std::vector<std::vector<float>>> seq(n), par(n);
  auto render = [&cube](int k, std::vector<std::vector<float>>& out) {
    Camera cam(cube, 20.f, 30.f, 40 + k, 30);
    float px = -2.f + k, py = -12.f, pz = 14.f - k;
    cam.SetPosition(px, py, pz);
    cam.SetAim(10.f, 0.f, 0.f);
    cam.SetMarchMode(1);
    cam.Render();
    out = cam.image;
  };
  for (int k = 0; k < n; ++k) render(k, seq[k]);
  std::vector<std::thread> ts;
  for (int k = 0; k < n; ++k) ts.emplace_back(render, k, std::ref(par[k]));
  for (auto& t : ts) t.join();
  for (int k = 0; k < n; ++k) CHECK(seq[k] == par[k]);
  float mx = 0;
  for (auto& row : seq[0])
    for (float v : row) mx = std::fmax(mx, v);
  CHECK(mx > 0);
}

// The roll extension: SetRoll(0) is the reference's pose (the same image
// bit for bit); a roll turns the image (a different one, not empty).
static void camera_roll() {
  std::vector<double> xs, ys, zs;
  for (int i = 0; i < 40; ++i) xs.push_back(-10 + 30.0 * i / 39);
  for (int i = 0; i < 32; ++i) ys.push_back(-15 + 30.0 * i / 31);
  for (int i = 0; i < 24; ++i) zs.push_back(-15 + 30.0 * i / 23);
  std::vector<float> vals;
  for (int k = 0; k < 24; ++k)
    for (int j = 0; j < 32; ++j)
      for (int i = 0; i < 40; ++i) vals.push_back(1.0f + 0.02f * ((i * 5 + j * 11 + k * 17) % 89));
  DataCube cube;
  cube.Init(xs, ys, zs, vals);
  cube.SetTrilinear(true);
  auto render = [&cube](double roll, bool set) {
    Camera cam(cube, 16.f, 27.f, 48, 28);
    float px = 1.f, py = -5.f, pz = 4.f;
    cam.SetPosition(px, py, pz);
    cam.SetAim(10.f, 0.f, 0.f);
    if (set) cam.SetRoll(roll);
    cam.Render();
    return cam.image;
  };
  const auto plain = render(0.0, false), zero = render(0.0, true), rolled = render(7.5, true);
  CHECK(plain == zero);
  CHECK(rolled != plain);
  float mx = 0;
  for (auto& row : rolled)
    for (float v : row) mx = std::fmax(mx, v);
  CHECK(mx > 0);
}

// The reference's own test space (tests/Camera_test.cpp:25-29: GetSample
// returns 1), rendered on the GPU through a cube sampled from it that holds
// every ray: each pixel is 200 samples of 1 times the scale, 2204113.13 in
// FP64 (the reference's FP32 sum gives 2204118).
class CubeFake : public Space {
 public:
  void Init() override {}
  float GetSample(float, float, float) override { return 1.f; }
};

static void user_defined_space() {
  CubeFake fake;
  const std::vector<double> ax = {-100.0, 0.0, 100.0};
  DataCube cube;
  cube.InitFromSpace(fake, ax, ax, ax, 2);
  cube.SetTrilinear(true);
  Camera cam(cube, 0.25f, 36.f, 36.f);
  float px = 1.f, py = 2.f, pz = 3.f;
  cam.SetPosition(px, py, pz);
  cam.SetAim(9.f, 0.f, 0.f);
  cam.Render();
  const float first = cam.image[0][0];
  bool same = true;
  for (auto& row : cam.image)
    for (float v : row) same = same && v == first;
  CHECK(same);
  CHECK(std::fabs(first - 2204113.13) < 0.5);
  // a Space with no GPU representation of its own is still refused by Render
  Camera direct(fake, 0.25f, 36.f, 36.f);
  bool threw = false;
  try {
    direct.Render();
  } catch (const std::invalid_argument&) {
    threw = true;
  }
  CHECK(threw);
}

int main(int argc, char** argv) {
  std::string dir = argc > 1 ? argv[1] : ".";
  cmem_basic();
  cmem_init_params();
  datacube(dir);
  camera_files_and_accumulation(dir);
  concurrent_cameras();
  camera_roll();
  user_defined_space();
  std::printf("%d failures\n", failures);
  return failures;
}
