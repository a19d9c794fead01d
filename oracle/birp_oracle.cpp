// CPU oracle for the BIRP render path (Camera::Render sampling a DataCube or a
// CMEM emissivity space).
//
// TEST INFRASTRUCTURE. Only tests/, __graft_entry__.smoke() and bench.py's
// CPU-baseline / reference arm may load this library, and only as the
// checker or the timed CPU baseline. The product (birp_cpp_gb300) never calls
// it and has its own independent implementation of every step below.
//
// Two restatements of the reference, written from its behaviour:
//
//  * "ref32": the reference's own FP32 arithmetic, operation for operation,
//    including its float/double promotions, its quirks (aim.y/aim.z ignored in
//    the pose, the degrees/radians mix in Orient, the p2 bug in CMEM::Init, B
//    overwritten by the field magnitude), the per-sample scale, serial FP32
//    accumulation and the stop at the first sample < 0 (-1 out of bounds,
//    or a negative field value). Generalised only by
//    explicit image dims, sample count N and ray length L, plus an optional
//    per-cell lookup for nonuniform axes. With reference inputs it matches the
//    reference build (oracle/_ref) bit for bit; the tests check that.
//
//  * "fp64": the FP64 oracle. The same physics in double precision, with the
//    reference's float-typed inputs and constants promoted exactly, sample
//    positions t_i = (i+0.5)*dt, a correct per-cell lookup on every axis,
//    PREFIX (reference: stop at the first out-of-bounds or negative sample)
//    and CLIP (skip such samples until the first good one, stop at the next)
//    march modes. Its double-precision ray
//    direction and in-box tests are written as plain IEEE +,-,*,/,sqrt with no
//    contraction (build with -ffp-contract=off), so a GPU can reproduce them
//    bit for bit; the scale factor is applied once per ray.
//
// Reference citations are path:line within the reference project.
#include <algorithm>
#include <atomic>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <thread>
#include <vector>

#ifndef M_PI
#define M_PI 3.14159265358979323846
#endif

extern "C" {

// ---------------------------------------------------------------- types

// FP32 cube. values are x-fastest: v[(k*ny + j)*nx + i] = slices[k][j][i].
// axis_mode 0 = reference lookup (origin c[0], spacing |c[0]-c[1]|,
// src/DataCube.cpp:150-218); 1 = per-cell lookup (correct for nonuniform axes).
typedef struct {
  int nx, ny, nz;
  const float* xs;
  const float* ys;
  const float* zs;
  const float* values;
  int trilinear;
  int axis_mode;
} o32_cube;

// CMEM coefficients after CMEM::Init (src/Cmem.cpp:38-115), FP32.
typedef struct {
  float p0, p1, p2, p3, bs, A1, A2, B, alpha, beta, ay_bs, az_bs;
  float dn, ds, theta_n, theta_s, r0_lin, charlie;
  float a5, a21;
  float beta_c[4];
  float pressure_dynamic, pressure_magnetic;
} o32_cmem;

// CMEM coefficients, FP64.
typedef struct {
  double p0, p1, p2, p3, bs, A1, A2, B, alpha, beta, ay_bs, az_bs;
  double dn, ds, theta_n, theta_s, r0_lin, charlie;
  double a5, a21;
  double beta_c[4];
  double pressure_dynamic, pressure_magnetic;
} o64_cmem;

// The arguments of the 17-argument CMEM::Init (include/Cmem.h:21-41).
// has_v / has_b = 0 means "empty vector passed" (use defaults).
typedef struct {
  int has_v, v[3];
  int has_b, b[3];
  float dipole, p0;
  int p1, p2, p3;
  float B, alpha, beta, bs, A1, A2, ay_bs, az_bs, density;
} o_cmem_args;

// FP32 camera: what Camera holds (include/Camera.h:23-43), with explicit
// image dims (the reference derives them as round(fov/pixel_size)),
// ray_samples N (reference 200) and the integer ray length L passed to
// GenerateRayDistWidth (reference 44).
typedef struct {
  float pos[3];
  float aim[3];
  float fov_w, fov_h;
  int nx, ny;
  int n_samples;
  int ray_max;
  int mode;  // 0 prefix (reference), 1 clip
} o32_camera;

// FP64 cube: the FP64 copy of the grid.
typedef struct {
  int nx, ny, nz;
  const double* xs;
  const double* ys;
  const double* zs;
  const double* values;
  int trilinear;
} o64_cube;

typedef struct {
  double pos[3];
  double aim[3];
  double fov_w, fov_h;  // degrees
  int nx, ny;
  int n_samples;        // N
  double ray_length;    // L; dt = L / N
  int mode;             // 0 prefix (reference), 1 clip
  double roll;          // degrees added to the Sun-fixed roll (extension; 0 = reference)
} o64_camera;

// space kinds for the render entry points
enum { O_SPACE_CUBE = 0, O_SPACE_CMEM = 1, O_SPACE_CONST = 2 };

}  // extern "C"

namespace {

// =====================================================================
// ref32: the reference's FP32 arithmetic
// =====================================================================

// Helper::VectorDistance (src/Helper.cpp:591-594)
inline float vdist3f(const float* v) { return std::sqrt(v[0] * v[0] + v[1] * v[1] + v[2] * v[2]); }
inline float vdist2f(const float* v) { return std::sqrt(v[0] * v[0] + v[1] * v[1]); }

// Camera::PointToPlane (src/Camera.cpp:419-508); returns {xo, yo}.
void point_to_plane32(const float* obj, float plac, float prad, const float* dv,
                      const float* uv, const float* north, const float* right,
                      const float* position, float* out_xy) {
  float to_deg = 180 / M_PI;
  float snumer = (dv[0] * obj[0]) + (dv[1] * obj[1]) + (dv[2] * obj[2]) + plac;
  float sdenom = (dv[0] * uv[0]) + (dv[1] * uv[1]) + (dv[2] * uv[2]);
  float scalar = snumer / sdenom;
  float q[3] = {obj[0] - (scalar * uv[0]), obj[1] - (scalar * uv[1]), obj[2] - (scalar * uv[2])};
  float ov[3] = {q[0] - position[0], q[1] - position[1], q[2] - position[2]};
  float dp = std::sqrt((ov[0] * ov[0]) + (ov[1] * ov[1]) + (ov[2] * ov[2]));
  float ou[3] = {ov[0] / dp, ov[1] / dp, ov[2] / dp};
  dp = std::sqrt((ou[0] * ou[0]) + (ou[1] * ou[1]) + (ou[2] * ou[2]));
  float t1 = (ou[0] * north[0]) + (ou[1] * north[1]) + (ou[2] * north[2]);
  float t2 = dp * std::sqrt((north[0] * north[0]) + (north[1] * north[1]) + (north[2] * north[2]));
  float t3 = t1 / t2;
  if (t3 > 1) t3 = 1.f;
  else if (t3 < -1) t3 = -1.f;
  float apon = to_deg * std::acos(t3);
  float t4 = (ou[0] * right[0]) + (ou[1] * right[1]) + (ou[2] * right[2]);
  float t5 = dp * std::sqrt((right[0] * right[0]) + (right[1] * right[1]) + (right[2] * right[2]));
  float t6 = t4 / t5;
  if (t6 > 1) t6 = 1.f;
  else if (t6 < -1) t6 = -1.f;
  float apor = to_deg * std::acos(t6);
  float soy = 1.f, sox = 1.f;
  if (apor > 90) sox = -1.f;
  float oo[3] = {obj[0] - position[0], obj[1] - position[1], obj[2] - position[2]};
  float ood = std::sqrt((oo[0] * oo[0]) + (oo[1] * oo[1]) + (oo[2] * oo[2]));
  oo[0] = oo[0] / ood;
  oo[1] = oo[1] / ood;
  oo[2] = oo[2] / ood;
  (void)prad;  // angular radius (aro) is computed by the reference but unused here
  float t7 = (oo[0] * uv[0]) + (oo[1] * uv[1]) + (oo[2] * uv[2]);
  float t8 = std::sqrt((oo[0] * oo[0]) + (oo[1] * oo[1]) + (oo[2] * oo[2]));
  float t9 = t7 / t8;
  if (t9 > 1) t9 = 1.f;
  float ooa = to_deg * std::acos(t9);
  float xo = 0.f, yo = 0.f;
  if (ooa > 0.000001f) {
    xo = sox * ooa * std::sin(apon / to_deg);
    yo = soy * ooa * std::cos(apon / to_deg);
  }
  out_xy[0] = xo;
  out_xy[1] = yo;
}

// Camera::Orient (src/Camera.cpp:309-417): the Sun roll angle in degrees.
float orient32(const float* position, const float* aim) {
  float to_deg = 180.f / M_PI;
  float dv[3] = {aim[0] - position[0], aim[1] - position[1], aim[2] - position[2]};
  float distance = vdist3f(dv);
  float uv[3] = {dv[0] / distance, dv[1] / distance, dv[2] / distance};
  float phi = std::acos(uv[2]);
  float denominator = std::sin(phi);
  float theta1, theta2;
  // acos(+-1) is the double overload (int argument): degrees, as written.
  if (std::abs(denominator) < std::abs(uv[0])) {
    theta1 = (denominator * uv[0] < 0) ? std::acos(-1) * to_deg : std::acos(1) * to_deg;
  } else {
    theta1 = std::asin(uv[0] / denominator);
  }
  (void)theta1;
  if (std::abs(denominator) < std::abs(uv[1])) {
    theta2 = (denominator * uv[1] < 0) ? std::acos(-1) * to_deg : std::acos(1) * to_deg;
  } else {
    theta2 = std::asin(uv[1] / denominator);
  }
  float north[3] = {-1.f * std::cos(theta2) * std::cos(phi), -1.f * std::sin(theta2) * std::cos(phi),
                    std::sin(phi)};
  // octant sign table (src/Camera.cpp:368-392)
  const bool px = uv[0] >= 0, py = uv[1] >= 0, pz = uv[2] >= 0;
  float s0, s1;
  if (px && py && pz) { s0 = -1.f; s1 = -1.f; }
  else if (px && py && !pz) { s0 = 1.f; s1 = 1.f; }
  else if (px && !py && pz) { s0 = -1.f; s1 = 1.f; }
  else if (px && !py && !pz) { s0 = 1.f; s1 = -1.f; }
  else if (!px && py && pz) { s0 = 1.f; s1 = -1.f; }
  else if (!px && py && !pz) { s0 = -1.f; s1 = 1.f; }
  else if (!px && !py && pz) { s0 = 1.f; s1 = 1.f; }
  else { s0 = -1.f; s1 = -1.f; }
  // NaN components fall through every branch of the reference's table and
  // keep their value; only reachable with a degenerate pose.
  if (!(std::isnan(uv[0]) || std::isnan(uv[1]) || std::isnan(uv[2]))) {
    north[0] = s0 * std::abs(north[0]);
    north[1] = s1 * std::abs(north[1]);
  }
  north[2] = std::abs(north[2]);
  float right[3] = {(uv[1] * north[2]) - (uv[2] * north[1]), (uv[2] * north[0]) - (uv[0] * north[2]),
                    (uv[0] * north[1]) - (uv[1] * north[0])};
  float plac = (-1.f * dv[0] * position[0]) + (-1.f * dv[1] * position[1]) + (-1.f * dv[2] * position[2]);
  const float sun[3] = {23455.f, 0.f, 0.f};
  float p2p[2];
  point_to_plane32(sun, plac, 1, dv, uv, north, right, position, p2p);
  float angle_sun = 270 - (to_deg * std::atan2(0 - p2p[0], 0 - p2p[1]));
  if (angle_sun > 360) angle_sun = angle_sun - 360;
  else if (angle_sun < 0) angle_sun = angle_sun + 360;
  return angle_sun;
}

// Helper::MatrixMultiply (src/Helper.cpp:70-98) for 3x3.
void matmul32(const float a[3][3], const float b[3][3], float r[3][3]) {
  for (int i = 0; i < 3; ++i)
    for (int j = 0; j < 3; ++j) {
      float value = 0.0f;
      for (int k = 0; k < 3; ++k) value = value + (a[i][k] * b[k][j]);
      r[i][j] = value;
    }
}

inline float det2f(float a, float b, float c, float d) { return a * d - b * c; }

// Helper::GetDeterminant for 3x3 (src/Helper.cpp:150-191): cofactor expansion
// along row 0, accumulated as result + sign*v[0][i]*minor.
float det3f(const float v[3][3]) {
  float result = 0;
  int sign = 1;
  for (int i = 0; i < 3; ++i) {
    float s[2][2];
    for (int m = 1; m < 3; ++m) {
      int z = 0;
      for (int n = 0; n < 3; ++n)
        if (n != i) s[m - 1][z++] = v[m][n];
    }
    result = result + sign * v[0][i] * det2f(s[0][0], s[0][1], s[1][0], s[1][1]);
    sign = -sign;
  }
  return result;
}

// Helper::GetInverse (src/Helper.cpp:241-264) via GetCofactor (:207-239) and
// GetTranspose. Returns false where the reference throws (determinant 0).
bool inverse32(const float v[3][3], float r[3][3]) {
  if (det3f(v) == 0) return false;
  float d = 1.f / det3f(v);
  float cof[3][3];
  for (int i = 0; i < 3; ++i)
    for (int j = 0; j < 3; ++j) {
      float s[2][2];
      int p = 0;
      for (int x = 0; x < 3; ++x) {
        if (x == i) continue;
        int q = 0;
        for (int y = 0; y < 3; ++y) {
          if (y == j) continue;
          s[p][q++] = v[x][y];
        }
        ++p;
      }
      cof[i][j] = std::pow(-1, i + j) * det2f(s[0][0], s[0][1], s[1][0], s[1][1]);
    }
  for (int i = 0; i < 3; ++i)
    for (int j = 0; j < 3; ++j) r[i][j] = cof[j][i] * d;
  return true;
}

// Pose part of Camera::Integrate (src/Camera.cpp:85-135): R^-1 of
// Rz(180-angle_sun) Rx(phi) Rz(theta). Only aim.x enters theta/phi.
bool pose32(const float* position, const float* aim, float rinv[3][3]) {
  float to_rad = M_PI / 180.f;
  float angle_sun = orient32(position, aim);
  float asc = 180.f - angle_sun;
  float x_diff = aim[0] - position[0];
  float theta = (2 * M_PI) - std::atan2(x_diff, position[1]);
  float hyp = std::sqrt(x_diff * x_diff + position[1] * position[1]);
  float phi = std::atan2(hyp, position[2]);
  float rz[3][3] = {{std::cos(theta), -std::sin(theta), 0}, {std::sin(theta), std::cos(theta), 0}, {0, 0, 1}};
  float rx[3][3] = {{1, 0, 0}, {0, std::cos(phi), -std::sin(phi)}, {0, std::sin(phi), std::cos(phi)}};
  float rz2[3][3] = {{std::cos(asc * to_rad), -std::sin(asc * to_rad), 0},
                     {std::sin(asc * to_rad), std::cos(asc * to_rad), 0},
                     {0, 0, 1}};
  float r1[3][3], r2[3][3];
  matmul32(rz2, rx, r1);
  matmul32(r1, rz, r2);
  return inverse32(r2, rinv);
}

// DataCube::GetSample (src/DataCube.cpp:203-277), FP32. Returns -1 out of
// bounds. axis_mode 1 replaces the affine index by a per-cell lookup.
int upper_cell_f(const float* c, int n, float x) {
  // largest k in [0, n-2] with c[k] <= x (caller guarantees c[0] <= x < c[n-1])
  int lo = 0, hi = n - 1;
  while (hi - lo > 1) {
    int mid = (lo + hi) / 2;
    if (c[mid] <= x) lo = mid;
    else hi = mid;
  }
  return lo;
}

float cube32_sample(const o32_cube* c, float x, float y, float z) {
  const float* V = c->values;
  const size_t sx = 1, sy = (size_t)c->nx, sz = (size_t)c->nx * c->ny;
  if (c->axis_mode == 0) {
    float spx = std::abs(c->xs[0] - c->xs[1]);
    float spy = std::abs(c->ys[0] - c->ys[1]);
    float spz = std::abs(c->zs[0] - c->zs[1]);
    float x_ing = x - c->xs[0];
    float x_idx = (x_ing / spx);
    float y_ing = y - c->ys[0];
    float y_idx = (y_ing / spy);
    float z_ing = z - c->zs[0];
    float z_idx = (z_ing / spz);
    if ((0 > x_ing || x_idx + 1 >= c->nx) || (0 > y_ing || y_idx + 1 >= c->ny) ||
        (0 > z_ing || z_idx + 1 >= c->nz))
      return -1.f;
    if (c->trilinear) {
      int z0 = std::floor(z_idx), z1 = std::ceil(z_idx);
      int y0 = std::floor(y_idx), y1 = std::ceil(y_idx);
      int x0 = std::floor(x_idx), x1 = std::ceil(x_idx);
      float s000 = V[z0 * sz + y0 * sy + x0 * sx], s001 = V[z0 * sz + y0 * sy + x1 * sx];
      float s010 = V[z0 * sz + y1 * sy + x0 * sx], s011 = V[z0 * sz + y1 * sy + x1 * sx];
      float s100 = V[z1 * sz + y0 * sy + x0 * sx], s101 = V[z1 * sz + y0 * sy + x1 * sx];
      float s110 = V[z1 * sz + y1 * sy + x0 * sx], s111 = V[z1 * sz + y1 * sy + x1 * sx];
      float xf = x_idx - (int)x_idx, yf = y_idx - (int)y_idx, zf = z_idx - (int)z_idx;
      float lx1 = std::lerp(s000, s001, xf), lx2 = std::lerp(s010, s011, xf);
      float hx1 = std::lerp(s100, s101, xf), hx2 = std::lerp(s110, s111, xf);
      float ly = std::lerp(lx1, lx2, yf), hy = std::lerp(hx1, hx2, yf);
      return std::lerp(ly, hy, zf);
    }
    return V[(int)z_idx * sz + (int)y_idx * sy + (int)x_idx * sx];
  }
  // per-cell lookup: valid iff c[0] <= x < c[n-1]
  if (!(c->xs[0] <= x && x < c->xs[c->nx - 1]) || !(c->ys[0] <= y && y < c->ys[c->ny - 1]) ||
      !(c->zs[0] <= z && z < c->zs[c->nz - 1]))
    return -1.f;
  int kx = upper_cell_f(c->xs, c->nx, x), ky = upper_cell_f(c->ys, c->ny, y), kz = upper_cell_f(c->zs, c->nz, z);
  if (!c->trilinear) return V[kz * sz + ky * sy + kx * sx];
  float xf = (x - c->xs[kx]) / (c->xs[kx + 1] - c->xs[kx]);
  float yf = (y - c->ys[ky]) / (c->ys[ky + 1] - c->ys[ky]);
  float zf = (z - c->zs[kz]) / (c->zs[kz + 1] - c->zs[kz]);
  const float* b = V + kz * sz + ky * sy + kx;
  float lx1 = std::lerp(b[0], b[1], xf), lx2 = std::lerp(b[sy], b[sy + 1], xf);
  float hx1 = std::lerp(b[sz], b[sz + 1], xf), hx2 = std::lerp(b[sz + sy], b[sz + sy + 1], xf);
  float ly = std::lerp(lx1, lx2, yf), hy = std::lerp(hx1, hx2, yf);
  return std::lerp(ly, hy, zf);
}

// CMEM::ShueCoords / LinScaled / ShueModel / GetSample (src/Cmem.cpp:117-288), FP32.
float cmem32_sample(const o32_cmem* m, float x, float y, float z) {
  float point[3] = {x, y, z};
  float pc[2] = {y, z};
  float r = vdist3f(point);
  float theta = (x != 0) ? std::acos(x / r) : 0;
  float phi = (y != 0) ? std::acos(y / vdist2f(pc)) : 0;
  // LinScaled (:188-222)
  float phi_n = std::acos((std::cos(theta) * std::cos(m->theta_n)) +
                          (std::sin(theta) * std::sin(m->theta_n) * std::cos(phi - M_PI / 2)));
  float phi_s = std::acos((std::cos(theta) * std::cos(m->theta_s)) +
                          (std::sin(theta) * std::sin(m->theta_s) * std::cos(phi - (3 * M_PI / 2))));
  float sin_phi = std::sin(phi);
  float f = std::pow(std::cos(theta / 2) + m->a5 * std::sin(2 * theta) * (1 - std::exp(-theta)),
                     (m->p1 * (m->beta_c[0] + m->beta_c[1] * std::cos(phi) + m->beta_c[3] * (sin_phi * sin_phi))));
  float q = m->p2 * m->charlie * std::exp(m->p3 * m->dn * (std::pow(phi_n, m->a21))) +
            m->p2 * m->charlie * std::exp(m->p3 * m->ds * (std::pow(phi_s, m->a21)));
  float r_mp = m->p0 * m->r0_lin * f + q;
  // ShueModel (:280-288)
  float ry = m->bs * std::pow((2 / (1 + std::cos(theta))), m->ay_bs);
  float rz = m->bs * std::pow((2 / (1 + std::cos(theta))), m->az_bs);
  float a1 = rz * std::cos(phi), a2 = ry * std::sin(phi);
  float r_bs = (ry * rz) / std::sqrt((a1 * a1) + (a2 * a2));
  float thickness = 0.05f;
  float half = thickness / 2;
  if (r < r_mp - half) return 0;
  if (r >= r_mp - half && r <= r_mp + half) {
    float norm = (r - (r_mp - half)) / (r_mp + half);
    float h = theta / 2, s = std::sin(theta);
    float b1 = m->A1 * (std::exp(-m->B * (h * h * h * h))) * std::pow(r / 10, (-m->alpha - (m->beta * (s * s))));
    return std::lerp(0.f, b1, norm);
  }
  if (r > r_mp + half && r < r_bs - half) {
    float h = theta / 2, s = std::sin(theta);
    return m->A1 * (std::exp(-m->B * (h * h * h * h))) * std::pow(r / 10, (-m->alpha - (m->beta * (s * s))));
  }
  if (r >= r_bs - half && r <= r_bs + half) {
    float h = theta / 2, s = std::sin(theta);
    double d10 = r / 10;
    float norm = (r - (r_bs - half)) / (r_bs + half);
    float b1 = m->A1 * (std::exp(-m->B * (h * h * h * h))) * std::pow(r / 10, (-m->alpha - (m->beta * (s * s))));
    float b2 = m->A2 * (1 / (d10 * d10 * d10));
    return std::lerp(b1, b2, norm);
  }
  double d10 = r / 10;
  return m->A2 * (1 / (d10 * d10 * d10));
}

// CMEM::Init + CalcDynamicPressure + CalcMagneticPressure + CalcInitialAlpha
// + DefineLinearCoeffs (src/Cmem.cpp:38-115, 250-325), FP32.
const float kLinA[22] = {12.544f, -0.194f, 0.305f,  0.0573f, 2.178f,  0.0571f, -0.999f, 16.473f,
                         0.00152f, 0.382f, 0.0431f, -0.00763f, -0.210f, 0.0405f, -4.430f, -0.636f,
                         -2.600f,  0.832f, -5.328f, 1.103f,  -0.907f, 1.450f};

void cmem32_init(const o_cmem_args* g, o32_cmem* m) {
  float v[3], b[3];
  if (!g->has_v) { v[0] = 400; v[1] = 0; v[2] = 0; }
  else { v[0] = g->v[0]; v[1] = g->v[1]; v[2] = g->v[2]; }
  if (!g->has_b) { b[0] = 0; b[1] = 0; b[2] = 5; }
  else { b[0] = g->b[0]; b[1] = g->b[1]; b[2] = g->b[2]; }
  float dipole = g->dipole;
  float B = g->B;
  m->alpha = g->alpha;
  m->beta = g->beta;
  m->p0 = g->p0 == 0 ? 0.786300004f : g->p0;
  m->p1 = g->p1 == 0 ? 1.f : g->p1;
  m->p2 = g->p2 == 0 ? 3.f : g->p3;  // reference bug kept (src/Cmem.cpp:90)
  m->p3 = g->p3 == 0 ? 4.f : g->p3;
  m->bs = g->bs == 0 ? 12.64f : g->bs;
  m->A1 = g->A1 == 0 ? 7.2e-06f : g->A1;
  m->A2 = g->A2 == 0 ? 3.5e-06f : g->A2;
  float density = g->density == 0 ? 5 : g->density;
  // CalcDynamicPressure (:292-304)
  float proton_mass = 0.00000000000000000000000000167f;
  float vms = vdist3f(v) * 1000;
  float n = density * 1000000;
  m->pressure_dynamic = 0.5f * proton_mass * n * (vms * vms) * 1000000000;
  // CalcMagneticPressure (:308-318): overwrites B with |b| in tesla
  B = vdist3f(b) * 0.000000001;
  float mu0 = 4 * M_PI * 0.0000001;
  m->pressure_magnetic = (B * B) / (2 * mu0) * 1000000000;
  m->B = B;
  // CalcInitialAlpha (:320-325) when the flaring parameters are "NULL" (0)
  float init_alpha = (0.58f - 0.010 * b[2]) * (1 + 0.010f * m->pressure_dynamic) + 0.2f;
  m->ay_bs = (g->ay_bs == 0) ? init_alpha : g->ay_bs;
  m->az_bs = (g->az_bs == 0) ? init_alpha : g->az_bs;
  // DefineLinearCoeffs (:250-276)
  const float* a = kLinA;
  m->beta_c[0] = a[6] + a[7] * ((std::exp(a[8] * b[2]) - 1) / (std::exp(a[9] * b[2]) + 1));
  m->beta_c[1] = a[10];
  m->beta_c[2] = a[11] + a[12] * dipole;
  m->beta_c[3] = a[13];
  float pt = m->pressure_dynamic + m->pressure_magnetic;
  m->charlie = a[14] * std::pow(pt, a[15]);
  m->dn = a[16] + a[17] * dipole + a[18] * (dipole * dipole);
  m->ds = a[16] - a[17] * dipole + a[18] * (dipole * dipole);
  m->theta_n = a[19] + a[20] * dipole;
  m->theta_s = a[19] - a[20] * dipole;
  m->r0_lin = a[0] * std::pow(m->pressure_dynamic + m->pressure_magnetic, a[1]) *
              (1 + a[2] * ((std::exp(a[3] * b[2]) - 1) / (std::exp(a[4] * b[2]) + 1)));
  m->a5 = a[5];
  m->a21 = a[21];
}

// =====================================================================
// fp64: the FP64 oracle
// =====================================================================

inline double vdist3d(const double* v) { return std::sqrt(v[0] * v[0] + v[1] * v[1] + v[2] * v[2]); }

double orient64(const double* position, const double* aim) {
  const double to_deg = 180.0 / M_PI;
  double dv[3] = {aim[0] - position[0], aim[1] - position[1], aim[2] - position[2]};
  double distance = vdist3d(dv);
  double uv[3] = {dv[0] / distance, dv[1] / distance, dv[2] / distance};
  double phi = std::acos(uv[2]);
  double den = std::sin(phi);
  double theta2;
  if (std::abs(den) < std::abs(uv[1])) theta2 = (den * uv[1] < 0) ? std::acos(-1.0) * to_deg : 0.0;
  else theta2 = std::asin(uv[1] / den);
  double north[3] = {-std::cos(theta2) * std::cos(phi), -std::sin(theta2) * std::cos(phi), std::sin(phi)};
  const bool px = uv[0] >= 0, py = uv[1] >= 0, pz = uv[2] >= 0;
  double s0, s1;
  if (px && py && pz) { s0 = -1; s1 = -1; }
  else if (px && py && !pz) { s0 = 1; s1 = 1; }
  else if (px && !py && pz) { s0 = -1; s1 = 1; }
  else if (px && !py && !pz) { s0 = 1; s1 = -1; }
  else if (!px && py && pz) { s0 = 1; s1 = -1; }
  else if (!px && py && !pz) { s0 = -1; s1 = 1; }
  else if (!px && !py && pz) { s0 = 1; s1 = 1; }
  else { s0 = -1; s1 = -1; }
  north[0] = s0 * std::abs(north[0]);
  north[1] = s1 * std::abs(north[1]);
  north[2] = std::abs(north[2]);
  double right[3] = {uv[1] * north[2] - uv[2] * north[1], uv[2] * north[0] - uv[0] * north[2],
                     uv[0] * north[1] - uv[1] * north[0]};
  double plac = (-dv[0] * position[0]) + (-dv[1] * position[1]) + (-dv[2] * position[2]);
  // PointToPlane of the Sun at (23455, 0, 0)
  const double obj[3] = {23455.0, 0.0, 0.0};
  double snumer = dv[0] * obj[0] + dv[1] * obj[1] + dv[2] * obj[2] + plac;
  double sdenom = dv[0] * uv[0] + dv[1] * uv[1] + dv[2] * uv[2];
  double scalar = snumer / sdenom;
  double ov[3] = {obj[0] - scalar * uv[0] - position[0], obj[1] - scalar * uv[1] - position[1],
                  obj[2] - scalar * uv[2] - position[2]};
  double dp = vdist3d(ov);
  double ou[3] = {ov[0] / dp, ov[1] / dp, ov[2] / dp};
  dp = vdist3d(ou);
  double t3 = (ou[0] * north[0] + ou[1] * north[1] + ou[2] * north[2]) / (dp * vdist3d(north));
  t3 = std::min(1.0, std::max(-1.0, t3));
  double apon = to_deg * std::acos(t3);
  double t6 = (ou[0] * right[0] + ou[1] * right[1] + ou[2] * right[2]) / (dp * vdist3d(right));
  t6 = std::min(1.0, std::max(-1.0, t6));
  double apor = to_deg * std::acos(t6);
  double sox = apor > 90 ? -1.0 : 1.0;
  double oo[3] = {obj[0] - position[0], obj[1] - position[1], obj[2] - position[2]};
  double ood = vdist3d(oo);
  oo[0] /= ood;
  oo[1] /= ood;
  oo[2] /= ood;
  double t9 = (oo[0] * uv[0] + oo[1] * uv[1] + oo[2] * uv[2]) / vdist3d(oo);
  if (t9 > 1) t9 = 1.0;
  double ooa = to_deg * std::acos(t9);
  double xo = 0, yo = 0;
  if (ooa > (double)0.000001f) {
    xo = sox * ooa * std::sin(apon / to_deg);
    yo = ooa * std::cos(apon / to_deg);
  }
  double angle_sun = 270.0 - to_deg * std::atan2(-xo, -yo);
  if (angle_sun > 360) angle_sun -= 360;
  else if (angle_sun < 0) angle_sun += 360;
  return angle_sun;
}

double det3d(const double v[3][3]) {
  double result = 0;
  double sign = 1;
  for (int i = 0; i < 3; ++i) {
    double s[2][2];
    for (int m = 1; m < 3; ++m) {
      int z = 0;
      for (int n = 0; n < 3; ++n)
        if (n != i) s[m - 1][z++] = v[m][n];
    }
    result = result + sign * v[0][i] * (s[0][0] * s[1][1] - s[0][1] * s[1][0]);
    sign = -sign;
  }
  return result;
}

// R^-1 (cofactor inverse, as the reference) in double. rinv[r][c].
bool pose64(const double* position, const double* aim, double roll, double rinv[3][3]) {
  const double to_rad = M_PI / 180.0;
  double asc = 180.0 - (orient64(position, aim) + roll);
  double x_diff = aim[0] - position[0];
  double theta = 2 * M_PI - std::atan2(x_diff, position[1]);
  double hyp = std::sqrt(x_diff * x_diff + position[1] * position[1]);
  double phi = std::atan2(hyp, position[2]);
  double rz[3][3] = {{std::cos(theta), -std::sin(theta), 0}, {std::sin(theta), std::cos(theta), 0}, {0, 0, 1}};
  double rx[3][3] = {{1, 0, 0}, {0, std::cos(phi), -std::sin(phi)}, {0, std::sin(phi), std::cos(phi)}};
  double rz2[3][3] = {{std::cos(asc * to_rad), -std::sin(asc * to_rad), 0},
                      {std::sin(asc * to_rad), std::cos(asc * to_rad), 0},
                      {0, 0, 1}};
  double r1[3][3], r2[3][3];
  for (int i = 0; i < 3; ++i)
    for (int j = 0; j < 3; ++j) {
      double v = 0;
      for (int k = 0; k < 3; ++k) v += rz2[i][k] * rx[k][j];
      r1[i][j] = v;
    }
  for (int i = 0; i < 3; ++i)
    for (int j = 0; j < 3; ++j) {
      double v = 0;
      for (int k = 0; k < 3; ++k) v += r1[i][k] * rz[k][j];
      r2[i][j] = v;
    }
  double det = det3d(r2);
  if (det == 0) return false;
  double d = 1.0 / det;
  for (int i = 0; i < 3; ++i)
    for (int j = 0; j < 3; ++j) {
      // cofactor of r2[j][i]
      int r0 = (j == 0) ? 1 : 0, rr1 = (j == 2) ? 1 : 2;
      int c0 = (i == 0) ? 1 : 0, c1 = (i == 2) ? 1 : 2;
      double minor = r2[r0][c0] * r2[rr1][c1] - r2[r0][c1] * r2[rr1][c0];
      double sgn = ((i + j) & 1) ? -1.0 : 1.0;
      rinv[i][j] = sgn * minor * d;
    }
  return true;
}

// Per-camera ray frame for the FP64 oracle: the exact double operations the
// GPU reproduces.
struct Frame64 {
  double rinv[3][3];
  double tfx, tfy, aspect;
  double pos[3];
  double dt;
  double K;  // per-sample scale of src/Camera.cpp:201 with ray_width = dt
};

bool frame64(const o64_camera* c, Frame64* f) {
  if (!pose64(c->pos, c->aim, c->roll, f->rinv)) return false;
  const double to_rad = M_PI / 180.0;
  f->aspect = (double)c->nx / (double)c->ny;
  f->tfx = std::tan(to_rad * (c->fov_w / 2.0));
  f->tfy = std::tan(to_rad * (c->fov_h / 2.0));
  for (int a = 0; a < 3; ++a) f->pos[a] = c->pos[a];
  f->dt = c->ray_length / (double)c->n_samples;
  f->K = ((f->dt * (100000.0 * 6378.1)) / (4.0 / M_PI)) / 10000.0;
  return true;
}

// Ray direction of pixel (column i, row j): d = normalize(R^-1 (sx, sy, -1)),
// computed as (sx*R[:,0] - R[:,2]) + sy*R[:,1], then * (1/sqrt(|w|^2)).
void ray_dir64(const Frame64& f, int nx, int ny, int i, int j, double d[3]) {
  double dx = ((double)i + 0.5) / (double)nx;
  double sx = ((2.0 * dx) - 1.0) * f.tfx * f.aspect;
  double dy = ((double)j + 0.5) / (double)ny;
  double sy = (1.0 - (2.0 * dy)) * f.tfy;
  double w[3];
  for (int r = 0; r < 3; ++r) {
    double A = sx * f.rinv[r][0] - f.rinv[r][2];
    double B = sy * f.rinv[r][1];
    w[r] = A + B;
  }
  double n2 = (w[0] * w[0] + w[1] * w[1]) + w[2] * w[2];
  double inv = 1.0 / std::sqrt(n2);
  for (int r = 0; r < 3; ++r) d[r] = w[r] * inv;
}

inline double sample_t64(double dt, int i) { return ((double)i + 0.5) * dt; }

int upper_cell_d(const double* c, int n, double x) {
  int lo = 0, hi = n - 1;
  while (hi - lo > 1) {
    int mid = (lo + hi) / 2;
    if (c[mid] <= x) lo = mid;
    else hi = mid;
  }
  return lo;
}

inline bool in_axis64(const double* c, int n, double x) { return c[0] <= x && x < c[n - 1]; }

double cube64_sample(const o64_cube* c, const double* p) {
  int kx = upper_cell_d(c->xs, c->nx, p[0]);
  int ky = upper_cell_d(c->ys, c->ny, p[1]);
  int kz = upper_cell_d(c->zs, c->nz, p[2]);
  const size_t sy = (size_t)c->nx, sz = (size_t)c->nx * c->ny;
  const double* b = c->values + kz * sz + ky * sy + kx;
  if (!c->trilinear) return b[0];
  double xf = (p[0] - c->xs[kx]) / (c->xs[kx + 1] - c->xs[kx]);
  double yf = (p[1] - c->ys[ky]) / (c->ys[ky + 1] - c->ys[ky]);
  double zf = (p[2] - c->zs[kz]) / (c->zs[kz + 1] - c->zs[kz]);
  double lx1 = std::lerp(b[0], b[1], xf), lx2 = std::lerp(b[sy], b[sy + 1], xf);
  double hx1 = std::lerp(b[sz], b[sz + 1], xf), hx2 = std::lerp(b[sz + sy], b[sz + sy + 1], xf);
  double ly = std::lerp(lx1, lx2, yf), hy = std::lerp(hx1, hx2, yf);
  return std::lerp(ly, hy, zf);
}

void cmem64_init(const o_cmem_args* g, o64_cmem* m) {
  double v[3], b[3];
  if (!g->has_v) { v[0] = 400; v[1] = 0; v[2] = 0; }
  else { v[0] = g->v[0]; v[1] = g->v[1]; v[2] = g->v[2]; }
  if (!g->has_b) { b[0] = 0; b[1] = 0; b[2] = 5; }
  else { b[0] = g->b[0]; b[1] = g->b[1]; b[2] = g->b[2]; }
  double dipole = g->dipole;
  m->alpha = g->alpha;
  m->beta = g->beta;
  m->p0 = g->p0 == 0 ? (double)0.786300004f : (double)g->p0;
  m->p1 = g->p1 == 0 ? 1.0 : (double)g->p1;
  m->p2 = g->p2 == 0 ? 3.0 : (double)g->p3;  // reference bug kept
  m->p3 = g->p3 == 0 ? 4.0 : (double)g->p3;
  m->bs = g->bs == 0 ? (double)12.64f : (double)g->bs;
  m->A1 = g->A1 == 0 ? (double)7.2e-06f : (double)g->A1;
  m->A2 = g->A2 == 0 ? (double)3.5e-06f : (double)g->A2;
  double density = g->density == 0 ? 5.0 : (double)g->density;
  double proton_mass = (double)0.00000000000000000000000000167f;
  double vms = vdist3d(v) * 1000;
  double n = density * 1000000;
  m->pressure_dynamic = 0.5 * proton_mass * n * (vms * vms) * 1e9;
  m->B = vdist3d(b) * 1e-9;
  double mu0 = 4 * M_PI * 1e-7;
  m->pressure_magnetic = (m->B * m->B) / (2 * mu0) * 1e9;
  double init_alpha = ((double)0.58f - 0.010 * b[2]) * (1 + (double)0.010f * m->pressure_dynamic) + (double)0.2f;
  m->ay_bs = (g->ay_bs == 0) ? init_alpha : (double)g->ay_bs;
  m->az_bs = (g->az_bs == 0) ? init_alpha : (double)g->az_bs;
  double a[22];
  for (int i = 0; i < 22; ++i) a[i] = kLinA[i];
  m->beta_c[0] = a[6] + a[7] * ((std::exp(a[8] * b[2]) - 1) / (std::exp(a[9] * b[2]) + 1));
  m->beta_c[1] = a[10];
  m->beta_c[2] = a[11] + a[12] * dipole;
  m->beta_c[3] = a[13];
  double pt = m->pressure_dynamic + m->pressure_magnetic;
  m->charlie = a[14] * std::pow(pt, a[15]);
  m->dn = a[16] + a[17] * dipole + a[18] * (dipole * dipole);
  m->ds = a[16] - a[17] * dipole + a[18] * (dipole * dipole);
  m->theta_n = a[19] + a[20] * dipole;
  m->theta_s = a[19] - a[20] * dipole;
  m->r0_lin = a[0] * std::pow(pt, a[1]) * (1 + a[2] * ((std::exp(a[3] * b[2]) - 1) / (std::exp(a[4] * b[2]) + 1)));
  m->a5 = a[5];
  m->a21 = a[21];
}

// CMEM boundary radii at direction (theta, phi), FP64.
void cmem64_radii(const o64_cmem* m, double theta, double phi, double* r_mp, double* r_bs) {
  double phi_n = std::acos(std::cos(theta) * std::cos(m->theta_n) +
                           std::sin(theta) * std::sin(m->theta_n) * std::cos(phi - M_PI / 2));
  double phi_s = std::acos(std::cos(theta) * std::cos(m->theta_s) +
                           std::sin(theta) * std::sin(m->theta_s) * std::cos(phi - 3 * M_PI / 2));
  double sp = std::sin(phi);
  double f = std::pow(std::cos(theta / 2) + m->a5 * std::sin(2 * theta) * (1 - std::exp(-theta)),
                      m->p1 * (m->beta_c[0] + m->beta_c[1] * std::cos(phi) + m->beta_c[3] * (sp * sp)));
  double q = m->p2 * m->charlie * std::exp(m->p3 * m->dn * std::pow(phi_n, m->a21)) +
             m->p2 * m->charlie * std::exp(m->p3 * m->ds * std::pow(phi_s, m->a21));
  *r_mp = m->p0 * m->r0_lin * f + q;
  double base = 2 / (1 + std::cos(theta));
  double ry = m->bs * std::pow(base, m->ay_bs);
  double rz = m->bs * std::pow(base, m->az_bs);
  double a1 = rz * std::cos(phi), a2 = ry * std::sin(phi);
  *r_bs = (ry * rz) / std::sqrt(a1 * a1 + a2 * a2);
}

double cmem64_sample(const o64_cmem* m, const double* p) {
  double x = p[0], y = p[1], z = p[2];
  double r = std::sqrt(x * x + y * y + z * z);
  double theta = (x != 0) ? std::acos(x / r) : 0.0;
  double phi = (y != 0) ? std::acos(y / std::sqrt(y * y + z * z)) : 0.0;
  double r_mp, r_bs;
  cmem64_radii(m, theta, phi, &r_mp, &r_bs);
  const double half = (double)(0.05f / 2);
  double h = theta / 2, s = std::sin(theta);
  double sheath = m->A1 * std::exp(-m->B * (h * h * h * h)) * std::pow(r / 10, -m->alpha - m->beta * (s * s));
  double d10 = r / 10;
  double outer = m->A2 * (1 / (d10 * d10 * d10));
  // the reference's shell tests, verbatim in structure (a NaN radius falls
  // through to the last shell, as in src/Cmem.cpp:135-176)
  if (r < r_mp - half) return 0.0;
  if (r >= r_mp - half && r <= r_mp + half) return std::lerp(0.0, sheath, (r - (r_mp - half)) / (r_mp + half));
  if (r > r_mp + half && r < r_bs - half) return sheath;
  if (r >= r_bs - half && r <= r_bs + half) return std::lerp(sheath, outer, (r - (r_bs - half)) / (r_bs + half));
  return outer;
}

// In-box sample range of one ray: [a, b) with every sample in it inside the
// box and samples a-1, b outside (or the ends of [0, N)). The box is convex and
// each axis test is monotone in i, so the in-box samples are contiguous.
void ray_range64(const o64_cube* c, const Frame64& f, int N, const double* d, int* a_out, int* b_out) {
  const double* ax[3] = {c->xs, c->ys, c->zs};
  const int n[3] = {c->nx, c->ny, c->nz};
  int a = -1, b = N;
  for (int i = 0; i < N; ++i) {
    double t = sample_t64(f.dt, i);
    bool in = true;
    for (int k = 0; k < 3; ++k) {
      double p = f.pos[k] + d[k] * t;
      if (!in_axis64(ax[k], n[k], p)) { in = false; break; }
    }
    if (in && a < 0) a = i;
    if (!in && a >= 0) { b = i; break; }
  }
  if (a < 0) { a = N; b = N; }
  *a_out = a;
  *b_out = b;
}

struct Job64 {
  const o64_cube* cube;
  const o64_cmem* cmem;
  int kind;
  const o64_camera* cam;
  Frame64 f;
};

double render_pixel64(const Job64& J, int i, int j) {
  const o64_camera* c = J.cam;
  double d[3];
  ray_dir64(J.f, c->nx, c->ny, i, j, d);
  const int N = c->n_samples;
  double sum = 0.0;
  if (J.kind == O_SPACE_CUBE) {
    const o64_cube* cb = J.cube;
    const double* ax[3] = {cb->xs, cb->ys, cb->zs};
    const int n[3] = {cb->nx, cb->ny, cb->nz};
    bool started = false;
    for (int s = 0; s < N; ++s) {
      double t = sample_t64(J.f.dt, s);
      double p[3];
      bool in = true;
      for (int k = 0; k < 3; ++k) {
        p[k] = J.f.pos[k] + d[k] * t;
        if (!in_axis64(ax[k], n[k], p[k])) in = false;
      }
      // a negative value ends the run as an out-of-bounds sample does: the
      // reference stops at the first scaled sample < 0 (src/Camera.cpp:205-209),
      // its -1 outside the box and negative field values alike
      const double v = in ? cube64_sample(cb, p) : -1.0;
      if (v < 0.0) {  // (a NaN value is summed, as in the reference)
        if (c->mode == 0) break;       // PREFIX: stop at the first bad sample
        if (started) break;            // CLIP: the run ends at the first bad sample after it starts
        continue;
      }
      started = true;
      sum += v;
    }
  } else {
    for (int s = 0; s < N; ++s) {
      double t = sample_t64(J.f.dt, s);
      double p[3] = {J.f.pos[0] + d[0] * t, J.f.pos[1] + d[1] * t, J.f.pos[2] + d[2] * t};
      sum += (J.kind == O_SPACE_CMEM) ? cmem64_sample(J.cmem, p) : 1.0;
    }
  }
  return sum * J.f.K;
}

template <class F>
void parallel_for(int n, int threads, F fn) {
  if (threads <= 1 || n < 2) {
    for (int i = 0; i < n; ++i) fn(i);
    return;
  }
  std::atomic<int> next{0};
  std::vector<std::thread> ts;
  int nt = std::min(threads, n);
  for (int t = 0; t < nt; ++t)
    ts.emplace_back([&]() {
      for (;;) {
        int i = next.fetch_add(1);
        if (i >= n) break;
        fn(i);
      }
    });
  for (auto& t : ts) t.join();
}

// ref32 render of one pixel (src/Camera.cpp:140-229), accumulating onto *px.
struct Job32 {
  const o32_cube* cube;
  const o32_cmem* cmem;
  int kind;
  const o32_camera* cam;
  float rinv[3][3];
  std::vector<float> ray_dist;
  float ray_width;
  float tan_x, tan_y, aspect;
};

inline float space32_sample(const Job32& J, float x, float y, float z) {
  if (J.kind == O_SPACE_CUBE) return cube32_sample(J.cube, x, y, z);
  if (J.kind == O_SPACE_CMEM) return cmem32_sample(J.cmem, x, y, z);
  return 1.f;
}

void render_pixel32(const Job32& J, int i, int j, float* px) {
  const o32_camera* c = J.cam;
  float device_x = (i + 0.5f) / (c->nx);
  float device_y = (j + 0.5f) / (c->ny);
  float to_rad = M_PI / 180.f;
  float screen_x = ((2 * device_x) - 1) * std::tan(to_rad * (c->fov_w / 2)) * J.aspect;
  float screen_y = (1 - (2 * device_y)) * std::tan(to_rad * (c->fov_h / 2));
  float sv[3] = {screen_x, screen_y, -1};
  float nd = vdist3f(sv);
  float su[3] = {screen_x / nd, screen_y / nd, -1 / nd};
  float w[3];
  for (int r = 0; r < 3; ++r) w[r] = (J.rinv[r][0] * su[0]) + (J.rinv[r][1] * su[1]) + (J.rinv[r][2] * su[2]);
  float wd = vdist3f(w);
  float wu[3] = {w[0] / wd, w[1] / wd, w[2] / wd};
  bool started = false;
  for (int k = 0; k < c->n_samples; ++k) {
    float t = J.ray_dist[k];
    float x = wu[0] * t + c->pos[0];
    float y = wu[1] * t + c->pos[1];
    float z = wu[2] * t + c->pos[2];
    float s = space32_sample(J, x, y, z);
    s = (s * J.ray_width * (1000 * 100 * 6378.1) / (4 / M_PI)) / 10000;
    if (s < 0) {
      if (c->mode == 0 || started) break;
      continue;
    }
    started = true;
    *px = *px + s;
  }
}

}  // namespace

extern "C" {

int oracle_version(void) { return 1; }

// ---------------- FP32 (reference-exact) entry points

void oracle_cmem32_init(const o_cmem_args* g, o32_cmem* out) { cmem32_init(g, out); }

void oracle_cmem32_sample(const o32_cmem* m, const float* xyz, int n, float* out) {
  for (int i = 0; i < n; ++i) out[i] = cmem32_sample(m, xyz[3 * i], xyz[3 * i + 1], xyz[3 * i + 2]);
}

void oracle_cube32_sample(const o32_cube* c, const float* xyz, int n, float* out) {
  for (int i = 0; i < n; ++i) out[i] = cube32_sample(c, xyz[3 * i], xyz[3 * i + 1], xyz[3 * i + 2]);
}

float oracle_orient32(const float* pos, const float* aim) { return orient32(pos, aim); }

// Renders into out[ny*nx] (row 0 = top), accumulating like Camera::Render
// (the image is not cleared). Returns 0, or 4 where the reference throws on a
// singular rotation.
int oracle_render32(int kind, const o32_cube* cube, const o32_cmem* cmem, const o32_camera* cam,
                    float* out, int threads) {
  Job32 J;
  J.cube = cube;
  J.cmem = cmem;
  J.kind = kind;
  J.cam = cam;
  if (!pose32(cam->pos, cam->aim, J.rinv)) return 4;
  // GenerateRayDistWidth (src/Camera.cpp:69-81)
  for (int k = 0; k < cam->n_samples; ++k) J.ray_dist.push_back(cam->ray_max * ((k + 0.5f) / cam->n_samples));
  J.ray_width = cam->n_samples > 1 ? J.ray_dist[1] - J.ray_dist[0] : 0.f;
  J.aspect = (float)cam->nx / (float)cam->ny;
  parallel_for(cam->ny, threads, [&](int j) {
    for (int i = 0; i < cam->nx; ++i) render_pixel32(J, i, j, out + (size_t)j * cam->nx + i);
  });
  return 0;
}

// Renders the listed pixels only (for timing a bounded sample of a large
// image); out[k] receives pixel (pi[k], pj[k]) starting from 0.
int oracle_render32_pixels(int kind, const o32_cube* cube, const o32_cmem* cmem, const o32_camera* cam,
                           const int* pi, const int* pj, int n, float* out, int threads) {
  Job32 J;
  J.cube = cube;
  J.cmem = cmem;
  J.kind = kind;
  J.cam = cam;
  if (!pose32(cam->pos, cam->aim, J.rinv)) return 4;
  for (int k = 0; k < cam->n_samples; ++k) J.ray_dist.push_back(cam->ray_max * ((k + 0.5f) / cam->n_samples));
  J.ray_width = cam->n_samples > 1 ? J.ray_dist[1] - J.ray_dist[0] : 0.f;
  J.aspect = (float)cam->nx / (float)cam->ny;
  int chunks = (n + 63) / 64;
  parallel_for(chunks, threads, [&](int ch) {
    for (int k = ch * 64; k < std::min(n, ch * 64 + 64); ++k) {
      out[k] = 0.f;
      render_pixel32(J, pi[k], pj[k], out + k);
    }
  });
  return 0;
}

// ---------------- FP64 oracle entry points

void oracle_cmem64_init(const o_cmem_args* g, o64_cmem* out) { cmem64_init(g, out); }

void oracle_cmem64_sample(const o64_cmem* m, const double* xyz, int n, double* out) {
  for (int i = 0; i < n; ++i) out[i] = cmem64_sample(m, xyz + 3 * i);
}

void oracle_cmem64_radii(const o64_cmem* m, double theta, double phi, double* r_mp, double* r_bs) {
  cmem64_radii(m, theta, phi, r_mp, r_bs);
}

// Samples the FP64 cube; out-of-box points give -1.
void oracle_cube64_sample(const o64_cube* c, const double* xyz, int n, double* out) {
  for (int i = 0; i < n; ++i) {
    const double* p = xyz + 3 * i;
    bool in = in_axis64(c->xs, c->nx, p[0]) && in_axis64(c->ys, c->ny, p[1]) && in_axis64(c->zs, c->nz, p[2]);
    out[i] = in ? cube64_sample(c, p) : -1.0;
  }
}

// Pose of the FP64 oracle: R^-1 (row-major 9), tan(fov_w/2), tan(fov_h/2),
// aspect, dt, K. Returns 4 for a singular rotation.
int oracle_frame64(const o64_camera* cam, double* rinv9, double* tfx, double* tfy, double* aspect,
                   double* dt, double* K, double* angle_sun) {
  Frame64 f;
  if (!frame64(cam, &f)) return 4;
  for (int r = 0; r < 3; ++r)
    for (int c = 0; c < 3; ++c) rinv9[3 * r + c] = f.rinv[r][c];
  *tfx = f.tfx;
  *tfy = f.tfy;
  *aspect = f.aspect;
  *dt = f.dt;
  *K = f.K;
  *angle_sun = orient64(cam->pos, cam->aim);
  return 0;
}

void oracle_ray_dir64(const o64_camera* cam, int i, int j, double* d) {
  Frame64 f;
  frame64(cam, &f);
  ray_dir64(f, cam->nx, cam->ny, i, j, d);
}

// In-box sample range [a, b) of pixel (i, j) against a cube.
int oracle_ray_range64(const o64_cube* cube, const o64_camera* cam, int i, int j, int* a, int* b) {
  Frame64 f;
  if (!frame64(cam, &f)) return 4;
  double d[3];
  ray_dir64(f, cam->nx, cam->ny, i, j, d);
  ray_range64(cube, f, cam->n_samples, d, a, b);
  return 0;
}

int oracle_render64(int kind, const o64_cube* cube, const o64_cmem* cmem, const o64_camera* cam,
                    double* out, int threads) {
  Job64 J{cube, cmem, kind, cam, {}};
  if (!frame64(cam, &J.f)) return 4;
  parallel_for(cam->ny, threads, [&](int j) {
    for (int i = 0; i < cam->nx; ++i) out[(size_t)j * cam->nx + i] = render_pixel64(J, i, j);
  });
  return 0;
}

int oracle_render64_pixels(int kind, const o64_cube* cube, const o64_cmem* cmem, const o64_camera* cam,
                           const int* pi, const int* pj, int n, double* out, int threads) {
  Job64 J{cube, cmem, kind, cam, {}};
  if (!frame64(cam, &J.f)) return 4;
  int chunks = (n + 31) / 32;
  parallel_for(chunks, threads, [&](int ch) {
    for (int k = ch * 32; k < std::min(n, ch * 32 + 32); ++k) out[k] = render_pixel64(J, pi[k], pj[k]);
  });
  return 0;
}

}  // extern "C"
