// C entry points around the UNMODIFIED reference renderer (Camera, DataCube,
// CMEM from the reference's src/), compiled from the reference tree by
// oracle/build_ref.sh into oracle/_ref/libbirp_ref.so.
//
// Test infrastructure only: used in this container to pin the oracle
// restatement (oracle/birp_oracle.cpp) and to generate the golden fixtures
// under tests/golden/. It never runs on the product path.
#include <cstring>
#include <string>
#include <vector>

#include "Camera.h"
#include "Cmem.h"
#include "DataCube.h"
#include "Space.h"

namespace {
// Same fake as the reference's own Camera test (tests/Camera_test.cpp:25-29):
// every sample is 1.
class ConstSpace : public Space {
 public:
  void Init() override {}
  float GetSample(float, float, float) override { return 1.f; }
};
}  // namespace

extern "C" {

// Builds a DataCube by filling its public fields the way DataCube::Load
// (src/DataCube.cpp:28-138) leaves them: axis vectors, size, spacing = first
// gap |c0-c1| (GetAxisSpacing, :150-183), origin = c[0], slices[z][y][x].
void* ref_cube_new(const float* xs, int nx, const float* ys, int ny,
                   const float* zs, int nz, const float* values, int trilinear) {
  DataCube* c = new DataCube();
  c->coords_x.assign(xs, xs + nx);
  c->coords_y.assign(ys, ys + ny);
  c->coords_z.assign(zs, zs + nz);
  c->size.x = nx;
  c->size.y = ny;
  c->size.z = nz;
  c->spacing[0] = std::abs(xs[0] - xs[1]);
  c->spacing[1] = std::abs(ys[0] - ys[1]);
  c->spacing[2] = std::abs(zs[0] - zs[1]);
  c->origin_coords[0] = xs[0];
  c->origin_coords[1] = ys[0];
  c->origin_coords[2] = zs[0];
  c->slices.assign(nz, std::vector<std::vector<float>>(ny, std::vector<float>(nx)));
  for (int k = 0; k < nz; ++k)
    for (int j = 0; j < ny; ++j)
      for (int i = 0; i < nx; ++i)
        c->slices[k][j][i] = values[((size_t)k * ny + j) * nx + i];
  c->SetTrilinear(trilinear != 0);
  return static_cast<Space*>(c);
}

void* ref_cmem_new_default(void) {
  CMEM* m = new CMEM();
  m->Init();
  return static_cast<Space*>(m);
}

// The full 17-argument CMEM::Init (include/Cmem.h:21-41). v and b may be
// NULL for "not passed" (empty vector).
void* ref_cmem_new(const int* v, const int* b, float dipole, float p0, int p1,
                   int p2, int p3, float B, float alpha, float beta, float bs,
                   float A1, float A2, float ay_bs, float az_bs, float density) {
  CMEM* m = new CMEM();
  std::vector<int> vv, bb;
  if (v) vv.assign(v, v + 3);
  if (b) bb.assign(b, b + 3);
  m->Init(true, vv, bb, dipole, p0, p1, p2, p3, B, alpha, beta, bs, A1, A2,
          ay_bs, az_bs, density);
  return static_cast<Space*>(m);
}

void* ref_const_new(void) { return static_cast<Space*>(new ConstSpace()); }

// Space has no virtual destructor, so each handle is freed through its own type.
void ref_space_free(void* s, int kind) {
  Space* sp = static_cast<Space*>(s);
  if (kind == 0) delete static_cast<DataCube*>(sp);
  else if (kind == 1) delete static_cast<CMEM*>(sp);
  else delete static_cast<ConstSpace*>(sp);
}

void ref_sample(void* s, const float* xyz, int n, float* out) {
  Space* sp = static_cast<Space*>(s);
  for (int i = 0; i < n; ++i) out[i] = sp->GetSample(xyz[3 * i], xyz[3 * i + 1], xyz[3 * i + 2]);
}

// Camera(space, pixel_size_deg, fov_h, fov_w); SetPosition; SetAim; Render
// (src/Camera.cpp:29-67). Image dims are round(fov/pixel) as in the
// constructor. Writes ny*nx floats, row 0 = top, when out is non-NULL and
// *nx_io * *ny_io is large enough; always returns the dims.
int ref_render(void* s, float pixel_size_deg, float fov_h, float fov_w,
               float px, float py, float pz, float ax, float ay, float az,
               int renders, float* out, int* nx_io, int* ny_io) {
  Camera cam(*static_cast<Space*>(s), pixel_size_deg, fov_h, fov_w);
  cam.SetPosition(px, py, pz);
  cam.SetAim(ax, ay, az);
  for (int r = 0; r < renders; ++r) cam.Render();
  int ny = (int)cam.image.size();
  int nx = ny ? (int)cam.image[0].size() : 0;
  int cap = (*nx_io) * (*ny_io);
  *nx_io = nx;
  *ny_io = ny;
  if (!out || cap < nx * ny) return 1;
  for (int j = 0; j < ny; ++j) std::memcpy(out + (size_t)j * nx, cam.image[j].data(), sizeof(float) * nx);
  return 0;
}
}
