// C ABI of the GB300 BIRP render path (include/birp_gb300.h): device context,
// cube upload, CMEM set-up, the per-camera FP64 frame, the plain per-call
// render and the graph-replayed batch.
#include <algorithm>
#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <mutex>
#include <numeric>
#include <string>
#include <thread>
#include <vector>

#include <unistd.h>

#include "../../include/birp_gb300.h"
#include "birp_host.h"
#include "birp_internal.h"

using namespace birp;

namespace birp {

Context g_ctx;
static thread_local std::string t_err;

birp_status fail(birp_status s, const char* fmt, ...) {
  char buf[512];
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(buf, sizeof buf, fmt, ap);
  va_end(ap);
  t_err = buf;
  return s;
}

birp_status ok() {
  t_err.clear();
  return BIRP_OK;
}

// ---------------------------------------------------------------- FP64 frame
//
// The FP64 oracle's camera frame, operation for operation (these steps must
// stay alike: the kernels reproduce the oracle's FP64 ray directions and
// in-box tests bit for bit from this frame). Follows Camera::Orient,
// PointToPlane and the pose part of Camera::Integrate
// (src/Camera.cpp:85-135, 309-508) in double precision.

static inline double norm3(const double* v) { return std::sqrt(v[0] * v[0] + v[1] * v[1] + v[2] * v[2]); }

double sun_roll_deg(const double* pos, const double* aim) {
  const double to_deg = 180.0 / M_PI;
  double dv[3] = {aim[0] - pos[0], aim[1] - pos[1], aim[2] - pos[2]};
  double dist = norm3(dv);
  double u[3] = {dv[0] / dist, dv[1] / dist, dv[2] / dist};
  double phi = std::acos(u[2]);
  double den = std::sin(phi);
  double th2;
  // the reference's mixed units: the clamped branch is in degrees
  if (std::abs(den) < std::abs(u[1])) th2 = (den * u[1] < 0) ? std::acos(-1.0) * to_deg : 0.0;
  else th2 = std::asin(u[1] / den);
  double nrt[3] = {-std::cos(th2) * std::cos(phi), -std::sin(th2) * std::cos(phi), std::sin(phi)};
  // octant sign table (src/Camera.cpp:368-392)
  const bool gx = u[0] >= 0, gy = u[1] >= 0, gz = u[2] >= 0;
  static const double kSign[8][2] = {
      // index = (!gx)*4 + (!gy)*2 + (!gz)
      {-1, -1}, {1, 1}, {-1, 1}, {1, -1}, {1, -1}, {-1, 1}, {1, 1}, {-1, -1}};
  const int oct = (!gx) * 4 + (!gy) * 2 + (!gz);
  nrt[0] = kSign[oct][0] * std::abs(nrt[0]);
  nrt[1] = kSign[oct][1] * std::abs(nrt[1]);
  nrt[2] = std::abs(nrt[2]);
  double rgt[3] = {u[1] * nrt[2] - u[2] * nrt[1], u[2] * nrt[0] - u[0] * nrt[2], u[0] * nrt[1] - u[1] * nrt[0]};
  double plac = (-dv[0] * pos[0]) + (-dv[1] * pos[1]) + (-dv[2] * pos[2]);
  // projection of the Sun at (23455, 0, 0) onto the image plane
  const double sun[3] = {23455.0, 0.0, 0.0};
  double sn = dv[0] * sun[0] + dv[1] * sun[1] + dv[2] * sun[2] + plac;
  double sd = dv[0] * u[0] + dv[1] * u[1] + dv[2] * u[2];
  double sc = sn / sd;
  double ov[3] = {sun[0] - sc * u[0] - pos[0], sun[1] - sc * u[1] - pos[1], sun[2] - sc * u[2] - pos[2]};
  double dp = norm3(ov);
  double ou[3] = {ov[0] / dp, ov[1] / dp, ov[2] / dp};
  dp = norm3(ou);
  double c_n = (ou[0] * nrt[0] + ou[1] * nrt[1] + ou[2] * nrt[2]) / (dp * norm3(nrt));
  c_n = std::min(1.0, std::max(-1.0, c_n));
  double apon = to_deg * std::acos(c_n);
  double c_r = (ou[0] * rgt[0] + ou[1] * rgt[1] + ou[2] * rgt[2]) / (dp * norm3(rgt));
  c_r = std::min(1.0, std::max(-1.0, c_r));
  double apor = to_deg * std::acos(c_r);
  double sox = apor > 90 ? -1.0 : 1.0;
  double oo[3] = {sun[0] - pos[0], sun[1] - pos[1], sun[2] - pos[2]};
  double ood = norm3(oo);
  oo[0] /= ood;
  oo[1] /= ood;
  oo[2] /= ood;
  double c_o = (oo[0] * u[0] + oo[1] * u[1] + oo[2] * u[2]) / norm3(oo);
  if (c_o > 1) c_o = 1.0;
  double ooa = to_deg * std::acos(c_o);
  double xo = 0, yo = 0;
  if (ooa > (double)0.000001f) {
    xo = sox * ooa * std::sin(apon / to_deg);
    yo = ooa * std::cos(apon / to_deg);
  }
  double roll = 270.0 - to_deg * std::atan2(-xo, -yo);
  if (roll > 360) roll -= 360;
  else if (roll < 0) roll += 360;
  return roll;
}

birp_status camera_frame(const birp_camera& c, Frame& f) {
  const double to_rad = M_PI / 180.0;
  f.angle_sun = sun_roll_deg(c.pos, c.aim);
  // the caller's roll offset adds to the Sun-fixed roll (0: exactly the
  // reference's angle)
  double asc = 180.0 - (f.angle_sun + c.roll_deg);
  double xd = c.aim[0] - c.pos[0];
  double theta = 2 * M_PI - std::atan2(xd, c.pos[1]);
  double hyp = std::sqrt(xd * xd + c.pos[1] * c.pos[1]);
  double phi = std::atan2(hyp, c.pos[2]);
  const double rz[3][3] = {{std::cos(theta), -std::sin(theta), 0}, {std::sin(theta), std::cos(theta), 0}, {0, 0, 1}};
  const double rx[3][3] = {{1, 0, 0}, {0, std::cos(phi), -std::sin(phi)}, {0, std::sin(phi), std::cos(phi)}};
  const double rs[3][3] = {{std::cos(asc * to_rad), -std::sin(asc * to_rad), 0},
                           {std::sin(asc * to_rad), std::cos(asc * to_rad), 0},
                           {0, 0, 1}};
  double m1[3][3], m2[3][3];
  for (int i = 0; i < 3; ++i)
    for (int j = 0; j < 3; ++j) {
      double acc = 0;
      for (int k = 0; k < 3; ++k) acc += rs[i][k] * rx[k][j];
      m1[i][j] = acc;
    }
  for (int i = 0; i < 3; ++i)
    for (int j = 0; j < 3; ++j) {
      double acc = 0;
      for (int k = 0; k < 3; ++k) acc += m1[i][k] * rz[k][j];
      m2[i][j] = acc;
    }
  // determinant by cofactor expansion along row 0, as Helper::GetDeterminant
  double det = 0, sg = 1;
  for (int i = 0; i < 3; ++i) {
    int a0 = (i == 0) ? 1 : 0, a1 = (i == 2) ? 1 : 2;
    det = det + sg * m2[0][i] * (m2[1][a0] * m2[2][a1] - m2[1][a1] * m2[2][a0]);
    sg = -sg;
  }
  if (det == 0) return fail(BIRP_ERR_SINGULAR, "camera rotation is singular (determinant 0)");
  double dinv = 1.0 / det;
  // R^-1 = transpose(cofactors) / det
  for (int i = 0; i < 3; ++i)
    for (int j = 0; j < 3; ++j) {
      int r0 = (j == 0) ? 1 : 0, r1 = (j == 2) ? 1 : 2;
      int c0 = (i == 0) ? 1 : 0, c1 = (i == 2) ? 1 : 2;
      double minor = m2[r0][c0] * m2[r1][c1] - m2[r0][c1] * m2[r1][c0];
      double sgn = ((i + j) & 1) ? -1.0 : 1.0;
      f.rinv[i][j] = sgn * minor * dinv;
    }
  f.aspect = (double)c.nx / (double)c.ny;
  f.tfx = std::tan(to_rad * (c.fov_w_deg / 2.0));
  f.tfy = std::tan(to_rad * (c.fov_h_deg / 2.0));
  f.dt = c.ray_length / (double)c.n_samples;
  f.K = ((f.dt * (100000.0 * 6378.1)) / (4.0 / M_PI)) / 10000.0;
  return BIRP_OK;
}

birp_status validate_camera(const birp_camera* c) {
  if (!c) return fail(BIRP_ERR_INVALID, "camera is NULL");
  for (int k = 0; k < 3; ++k)
    if (!std::isfinite(c->pos[k]) || !std::isfinite(c->aim[k]))
      return fail(BIRP_ERR_INVALID, "camera position/aim must be finite");
  if (!(c->nx >= 1 && c->ny >= 1) || (int64_t)c->nx * c->ny > (int64_t)1 << 30)
    return fail(BIRP_ERR_INVALID, "image dims %d x %d out of range", c->nx, c->ny);
  if (!(c->fov_w_deg > 0 && c->fov_w_deg < 180 && c->fov_h_deg > 0 && c->fov_h_deg < 180))
    return fail(BIRP_ERR_INVALID, "field of view must lie in (0, 180) degrees");
  if (!(c->n_samples >= 1 && c->n_samples <= (1 << 22)))
    return fail(BIRP_ERR_INVALID, "n_samples %d out of range [1, 2^22]", c->n_samples);
  if (!(c->ray_length > 0 && std::isfinite(c->ray_length)))
    return fail(BIRP_ERR_INVALID, "ray_length must be positive");
  if (c->march != BIRP_MARCH_PREFIX && c->march != BIRP_MARCH_CLIP)
    return fail(BIRP_ERR_INVALID, "march must be PREFIX or CLIP");
  if (!(c->segments == 0 || c->segments == 1 || c->segments == 2 || c->segments == 4 || c->segments == 8))
    return fail(BIRP_ERR_INVALID, "segments must be 0, 1, 2, 4 or 8");
  auto pow2 = [](int v) { return v > 0 && (v & (v - 1)) == 0; };
  if (c->warp_rays_x < 0 || (c->warp_rays_x > 0 && !pow2(c->warp_rays_x)) || c->tile_warps_x < 0 ||
      (c->tile_warps_x > 0 && !pow2(c->tile_warps_x)) || c->tile_warps_x > 4)
    return fail(BIRP_ERR_INVALID, "warp_rays_x and tile_warps_x must be 0 or powers of two (tile_warps_x <= 4)");
  return BIRP_OK;
}

namespace {
int log2_of(int v) {
  int l = 0;
  while ((1 << l) < v) ++l;
  return l;
}
}  // namespace

// Tile shape: lanes per ray, warp-block width and warps across a tile, each
// explicit or else from the tuned tables (tune.cpp).
birp_status choose_shape(const birp_camera& c, int kind, bool batched, int& seg, int& wbx, int& wgx) {
  TunedShape t = tuned_shape((int64_t)c.nx * c.ny, c.n_samples, kind, c.trilinear, batched);
  seg = c.segments > 0 ? log2_of(c.segments) : t.seg_log2;
  wbx = c.warp_rays_x > 0 ? log2_of(c.warp_rays_x) : (t.wbx_l2 >= 0 && c.segments == 0 ? t.wbx_l2 : default_wbx_l2(seg));
  wgx = c.tile_warps_x > 0 ? log2_of(c.tile_warps_x) : (t.wgx_l2 >= 0 && c.segments == 0 ? t.wgx_l2 : 1);
  if (!tile_shape_ok(seg, wbx, wgx))
    return fail(BIRP_ERR_INVALID, "tile shape (%d lanes per ray, %d rays across a warp block, %d warps across a tile) "
                                  "is not one the kernels take (tiles up to 32 pixels a side)",
                1 << seg, 1 << wbx, 1 << wgx);
  return BIRP_OK;
}

birp_status build_request(const birp_cube* cube, const birp_cmem* cmem, const birp_camera& c, float* out,
                          RequestDev& r, bool batched) {
  birp_status st = validate_camera(&c);
  if (st) return st;
  if ((cube == nullptr) == (cmem == nullptr)) return fail(BIRP_ERR_INVALID, "exactly one of cube / cmem must be given");
  Frame f;
  st = camera_frame(c, f);
  if (st) return st;
  std::memset(&r, 0, sizeof r);
  for (int i = 0; i < 3; ++i)
    for (int j = 0; j < 3; ++j) r.rinv[i][j] = f.rinv[i][j];
  r.tfx = f.tfx;
  r.tfy = f.tfy;
  r.aspect = f.aspect;
  for (int k = 0; k < 3; ++k) {
    r.pos[k] = c.pos[k];
    r.pos32[k] = (float)c.pos[k];
    r.pos_hi[k] = r.pos32[k];
    r.pos_lo[k] = (float)(c.pos[k] - (double)r.pos_hi[k]);
  }
  r.dt = f.dt;
  r.dt32 = (float)f.dt;
  r.dt_hi = r.dt32;
  r.dt_lo = (float)(f.dt - (double)r.dt_hi);
  r.K = f.K;
  r.nx = c.nx;
  r.ny = c.ny;
  r.N = c.n_samples;
  r.mode = c.march;
  r.interp = c.trilinear ? 1 : 0;
  r.kind = cube ? SPACE_CUBE : SPACE_CMEM;
  if (birp_status s2 = choose_shape(c, r.kind, batched, r.seg_log2, r.wbx_l2, r.wgx_l2)) return s2;
  const int tw = tile_w(r.seg_log2, r.wbx_l2, r.wgx_l2), th = tile_h(r.seg_log2, r.wbx_l2, r.wgx_l2);
  r.tiles_x = (c.nx + tw - 1) / tw;
  int tiles_y = (c.ny + th - 1) / th;
  r.tiles = r.tiles_x * tiles_y;
  r.out = out;
  if (cube) {
    r.cube = cube->d_desc;
    r.layout = cube->layout;
    r.has_neg = cube->has_neg > 0 ? 1 : 0;
  } else {
    r.cmem = cmem->d_desc;
  }
  return BIRP_OK;
}

birp_status ensure_scratch(size_t img_floats) {
  Context& g = g_ctx;
  if (g.scratch_floats >= img_floats) return BIRP_OK;
  if (g.scratch) cudaFree(g.scratch);
  g.scratch = nullptr;
  g.scratch_floats = 0;
  size_t want = std::max(img_floats, (size_t)1 << 20);
  cudaError_t e = cudaMalloc(&g.scratch, want * sizeof(float));
  if (e != cudaSuccess) return fail(BIRP_ERR_NOMEM, "cudaMalloc(%zu B) for the image: %s", want * 4, cudaGetErrorString(e));
  g.scratch_floats = want;
  return BIRP_OK;
}

birp_status check_init() {
  if (g_ctx.device < 0) return fail(BIRP_ERR_NOT_INIT, "birp_init has not been called");
  // the current device is per host thread: a caller on another thread than
  // birp_init's is switched to the library's device
  int cur = -1;
  if (cudaGetDevice(&cur) != cudaSuccess || cur != g_ctx.device) {
    const cudaError_t e = cudaSetDevice(g_ctx.device);
    if (e != cudaSuccess) return fail(BIRP_ERR_CUDA, "cudaSetDevice(%d): %s", g_ctx.device, cudaGetErrorString(e));
  }
  return BIRP_OK;
}

cudaStream_t pick_stream(void* s) { return s ? (cudaStream_t)s : g_ctx.stream; }

bool host_direct_writes() {
  if (!g_ctx.pageable_access) return false;
  const char* v = std::getenv("BIRP_HOST_DIRECT");
  return !(v && v[0] == '0');
}

void prefault_outputs(float* const* dst, const size_t* floats, int n) {
  static const size_t page = [] {
    long p = sysconf(_SC_PAGESIZE);
    return (size_t)(p > 0 ? p : 4096) / sizeof(float);
  }();
  size_t total = 0;
  for (int i = 0; i < n; ++i) total += dst[i] ? floats[i] : 0;
  const unsigned hw = std::max(1u, std::thread::hardware_concurrency());
  // >= 128 MB per thread: when the pages are mapped already (the usual case
  // for reused buffers) the touch is ~1 store per page, cheaper than a thread
  const int nt = (int)std::min<size_t>({8, hw, total / (1u << 25) + 1});
  auto work = [&](int t) {
    for (int i = t; i < n; i += nt) {
      if (!dst[i] || !floats[i]) continue;
      volatile float* p = dst[i];
      for (size_t k = 0; k < floats[i]; k += page) p[k] = 0.f;
      p[floats[i] - 1] = 0.f;
    }
  };
  std::vector<std::thread> th;
  for (int t = 1; t < nt; ++t) th.emplace_back(work, t);
  work(0);
  for (auto& x : th) x.join();
}

void parallel_copy(float* const* dst, const float* const* src, const size_t* floats, int n) {
  size_t total = 0;
  for (int i = 0; i < n; ++i) total += dst[i] ? floats[i] : 0;
  const unsigned hw = std::max(1u, std::thread::hardware_concurrency());
  const int nt = (int)std::min<size_t>({8, hw, total / (1u << 20) + 1});  // >= 4 MB per thread
  // thread t copies the floats [t * total / nt, (t + 1) * total / nt) of the concatenation
  auto work = [&](int t) {
    const size_t lo = total * t / nt, hi = total * (t + 1) / nt;
    size_t base = 0;
    for (int i = 0; i < n && base < hi; ++i) {
      if (!dst[i]) continue;
      const size_t a = std::max(lo, base), b = std::min(hi, base + floats[i]);
      if (a < b) std::memcpy(dst[i] + (a - base), src[i] + (a - base), (b - a) * sizeof(float));
      base += floats[i];
    }
  };
  std::vector<std::thread> th;
  for (int t = 1; t < nt; ++t) th.emplace_back(work, t);
  work(0);
  for (auto& x : th) x.join();
}

}  // namespace birp

#define CK(x)                                                                                  \
  do {                                                                                         \
    cudaError_t e_ = (x);                                                                      \
    if (e_ != cudaSuccess) return fail(BIRP_ERR_CUDA, "%s: %s", #x, cudaGetErrorString(e_));   \
  } while (0)

// ============================================================== C ABI

extern "C" {

int birp_version(void) { return 10000; }

const char* birp_last_error(void) { return t_err.c_str(); }

birp_status birp_init(int device) {
  std::lock_guard<std::mutex> lk(g_ctx.mu);
  if (g_ctx.device >= 0) {
    if (g_ctx.device == device) return ok();
    return fail(BIRP_ERR_INVALID, "already initialised on device %d", g_ctx.device);
  }
  int n = 0;
  CK(cudaGetDeviceCount(&n));
  if (device < 0 || device >= n) return fail(BIRP_ERR_INVALID, "device %d not present (%d devices)", device, n);
  CK(cudaSetDevice(device));
  CK(cudaStreamCreateWithFlags(&g_ctx.stream, cudaStreamNonBlocking));
  CK(cudaMalloc(&g_ctx.stats, sizeof(KernelStats)));
  CK(cudaMemset(g_ctx.stats, 0, sizeof(KernelStats)));
  CK(cudaDeviceGetAttribute(&g_ctx.sms, cudaDevAttrMultiProcessorCount, device));
  CK(cudaDeviceGetAttribute(&g_ctx.pageable_access, cudaDevAttrPageableMemoryAccess, device));
  g_ctx.device = device;
  return ok();
}

void birp_shutdown(void) {
  std::lock_guard<std::mutex> lk(g_ctx.mu);
  if (g_ctx.device < 0) return;
  cudaSetDevice(g_ctx.device);
  cudaStreamSynchronize(g_ctx.stream);
  if (g_ctx.scratch) cudaFree(g_ctx.scratch);
  if (g_ctx.flush) cudaFree(g_ctx.flush);
  if (g_ctx.stats) cudaFree(g_ctx.stats);
  if (g_ctx.xyz_scratch) cudaFree(g_ctx.xyz_scratch);
  cudaStreamDestroy(g_ctx.stream);
  g_ctx.scratch = nullptr;
  g_ctx.scratch_floats = 0;
  g_ctx.flush = nullptr;
  g_ctx.stats = nullptr;
  g_ctx.xyz_scratch = nullptr;
  g_ctx.xyz_floats = 0;
  g_ctx.stream = nullptr;
  g_ctx.device = -1;
}

// ---------------------------------------------------------------- cube

static_assert(BIRP_CUBE_RECORDS == CUBE_RECORDS && BIRP_CUBE_COMPACT == CUBE_COMPACT && BIRP_CUBE_PAIRS == CUBE_PAIRS,
              "the kernels' layout codes are the ABI's");

birp_status birp_cube_create(const double* xs, int nx, const double* ys, int ny, const double* zs, int nz,
                             const float* values, birp_cube** out) {
  return birp_cube_create_layout(xs, nx, ys, ny, zs, nz, values, BIRP_CUBE_RECORDS, out);
}

birp_status birp_cube_create_layout(const double* xs, int nx, const double* ys, int ny, const double* zs, int nz,
                                    const float* values, int layout, birp_cube** out) {
  if (birp_status s = check_init()) return s;
  if (!out || !values || !xs || !ys || !zs) return fail(BIRP_ERR_INVALID, "NULL argument");
  if (layout != BIRP_CUBE_RECORDS && layout != BIRP_CUBE_COMPACT && layout != BIRP_CUBE_PAIRS)
    return fail(BIRP_ERR_INVALID, "unknown cube layout %d", layout);
  *out = nullptr;
  const double* axes[3] = {xs, ys, zs};
  const int n[3] = {nx, ny, nz};
  birp_cube* c = new birp_cube();
  c->layout = layout;
  for (int k = 0; k < 3; ++k) {
    birp_status s = analyze_axis(axes[k], n[k], "xyz"[k], *c, k);
    if (s) {
      delete c;
      return s;
    }
  }
  const uint64_t px = (uint64_t)nx + 2, py = (uint64_t)ny + 2, pz = (uint64_t)nz + 2;
  const uint64_t total = px * py * pz;
  if (total >= ((uint64_t)1 << 31)) {
    delete c;
    return fail(BIRP_ERR_INVALID, "cube too large (%llu padded nodes; limit 2^31)", (unsigned long long)total);
  }
  birp_status s = upload_cube(*c, values, nullptr, false);
  if (s) {
    destroy_cube_device(*c);
    delete c;
    return s;
  }
  *out = c;
  return ok();
}

birp_status birp_cube_destroy(birp_cube* cube) {
  if (!cube) return ok();
  if (g_ctx.device >= 0) cudaStreamSynchronize(g_ctx.stream);
  destroy_cube_device(*cube);
  delete cube;
  return ok();
}

birp_status birp_cube_get_info(const birp_cube* cube, birp_cube_info* info) {
  if (!cube || !info) return fail(BIRP_ERR_INVALID, "NULL argument");
  info->nx = cube->n[0];
  info->ny = cube->n[1];
  info->nz = cube->n[2];
  for (int k = 0; k < 3; ++k) info->uniform[k] = cube->uniform[k];
  info->device_bytes = cube->device_bytes;
  info->layout = cube->layout;
  return ok();
}

birp_status birp_cube_sample(const birp_cube* cube, int trilinear, const float* xyz, int n, float* out) {
  if (birp_status s = check_init()) return s;
  if (!cube || (n > 0 && (!xyz || !out)) || n < 0) return fail(BIRP_ERR_INVALID, "bad argument");
  if (n == 0) return ok();
  std::lock_guard<std::mutex> lk(g_ctx.mu);
  if (birp_status s = ensure_xyz_scratch((size_t)n * 4)) return s;
  float* d_xyz = g_ctx.xyz_scratch;
  float* d_out = d_xyz + (size_t)3 * n;
  cudaStream_t st = g_ctx.stream;
  CK(cudaMemcpyAsync(d_xyz, xyz, sizeof(float) * 3 * n, cudaMemcpyHostToDevice, st));
  CK(launch_cube_sample(cube->d_desc, trilinear, d_xyz, n, d_out, st));
  CK(cudaMemcpyAsync(out, d_out, sizeof(float) * n, cudaMemcpyDeviceToHost, st));
  CK(cudaStreamSynchronize(st));
  return ok();
}

// ---------------------------------------------------------------- CMEM

void birp_cmem_default_params(birp_cmem_params* p) {
  if (!p) return;
  std::memset(p, 0, sizeof *p);
  // CMEM::Init(true) defaults (include/Cmem.h:21-41)
  p->dipole = 0.f;
  p->p0 = 0.786300004f;
  p->p1 = 1;
  p->p2 = 3;
  p->p3 = 4;
  p->B = 2.f;
  p->alpha = 2.5f;
  p->beta = -1.6f;
  p->bs = 12.6400003f;
  p->A1 = 7.2e-06f;
  p->A2 = 3.5000000000000004e-06f;
}

birp_status birp_cmem_create(const birp_cmem_params* p, birp_cmem** out) {
  if (birp_status s = check_init()) return s;
  if (!p || !out) return fail(BIRP_ERR_INVALID, "NULL argument");
  *out = nullptr;
  birp_cmem* m = new birp_cmem();
  cmem_coefficients(*p, m->h_desc);
  cudaError_t e = cudaMalloc(&m->d_desc, sizeof(CmemDev));
  if (e != cudaSuccess) {
    delete m;
    return fail(BIRP_ERR_NOMEM, "cudaMalloc: %s", cudaGetErrorString(e));
  }
  e = cudaMemcpy(m->d_desc, &m->h_desc, sizeof(CmemDev), cudaMemcpyHostToDevice);
  if (e != cudaSuccess) {
    cudaFree(m->d_desc);
    delete m;
    return fail(BIRP_ERR_CUDA, "cudaMemcpy: %s", cudaGetErrorString(e));
  }
  *out = m;
  return ok();
}

birp_status birp_cmem_destroy(birp_cmem* m) {
  if (!m) return ok();
  if (g_ctx.device >= 0) cudaStreamSynchronize(g_ctx.stream);
  if (m->d_desc) cudaFree(m->d_desc);
  delete m;
  return ok();
}

birp_status birp_cmem_sample(const birp_cmem* m, const float* xyz, int n, float* out) {
  if (birp_status s = check_init()) return s;
  if (!m || (n > 0 && (!xyz || !out)) || n < 0) return fail(BIRP_ERR_INVALID, "bad argument");
  if (n == 0) return ok();
  std::lock_guard<std::mutex> lk(g_ctx.mu);
  if (birp_status s = ensure_xyz_scratch((size_t)n * 4)) return s;
  float* d_xyz = g_ctx.xyz_scratch;
  float* d_out = d_xyz + (size_t)3 * n;
  cudaStream_t st = g_ctx.stream;
  CK(cudaMemcpyAsync(d_xyz, xyz, sizeof(float) * 3 * n, cudaMemcpyHostToDevice, st));
  CK(launch_cmem_sample(m->d_desc, d_xyz, n, d_out, st));
  CK(cudaMemcpyAsync(out, d_out, sizeof(float) * n, cudaMemcpyDeviceToHost, st));
  CK(cudaStreamSynchronize(st));
  return ok();
}

birp_status birp_cmem_margin_check(const birp_cmem* m, int n, float* max_rel_err, float* margin) {
  if (birp_status s = check_init()) return s;
  if (!m || !max_rel_err || n <= 0) return fail(BIRP_ERR_INVALID, "bad argument");
  std::lock_guard<std::mutex> lk(g_ctx.mu);
  if (birp_status s = ensure_xyz_scratch(4)) return s;
  float* d = g_ctx.xyz_scratch;
  cudaStream_t st = g_ctx.stream;
  CK(cudaMemsetAsync(d, 0, sizeof(float), st));
  CK(launch_cmem_radii_check(m->d_desc, n, 12345ull, d, st));
  CK(cudaMemcpyAsync(max_rel_err, d, sizeof(float), cudaMemcpyDeviceToHost, st));
  CK(cudaStreamSynchronize(st));
  if (margin) *margin = m->h_desc.eps_rel;
  return ok();
}

birp_status birp_fastmath_check(int which, const float* x, const float* y, int n, float* fast, float* lib) {
  if (birp_status s = check_init()) return s;
  if (which < 0 || which > 3 || n < 0 || (n > 0 && (!x || !y || !fast || !lib)))
    return fail(BIRP_ERR_INVALID, "bad argument");
  if (n == 0) return ok();
  std::lock_guard<std::mutex> lk(g_ctx.mu);
  if (birp_status s = ensure_xyz_scratch((size_t)n * 4)) return s;
  float* dx = g_ctx.xyz_scratch;
  float *dy = dx + n, *df = dx + 2 * (size_t)n, *dl = dx + 3 * (size_t)n;
  cudaStream_t st = g_ctx.stream;
  CK(cudaMemcpyAsync(dx, x, sizeof(float) * n, cudaMemcpyHostToDevice, st));
  CK(cudaMemcpyAsync(dy, y, sizeof(float) * n, cudaMemcpyHostToDevice, st));
  CK(launch_fastmath(which, dx, dy, n, df, dl, st));
  CK(cudaMemcpyAsync(fast, df, sizeof(float) * n, cudaMemcpyDeviceToHost, st));
  CK(cudaMemcpyAsync(lib, dl, sizeof(float) * n, cudaMemcpyDeviceToHost, st));
  CK(cudaStreamSynchronize(st));
  return ok();
}

// ---------------------------------------------------------------- camera / render

void birp_camera_defaults(birp_camera* c) {
  if (!c) return;
  std::memset(c, 0, sizeof *c);
  c->pos[0] = 5.91813f;
  c->pos[1] = 6.74116f;
  c->pos[2] = 17.7067f;
  c->aim[0] = 7.81768f;
  c->fov_w_deg = 36.0;
  c->fov_h_deg = 36.0;
  c->nx = 144;
  c->ny = 144;
  c->n_samples = 200;
  c->ray_length = 44.0;
  c->trilinear = 0;
  c->march = BIRP_MARCH_PREFIX;
  c->segments = 0;
}

birp_status birp_camera_frame(const birp_camera* cam, double* rinv9, double* tan_w, double* tan_h, double* aspect,
                              double* step, double* scale, double* angle_sun) {
  if (birp_status s = validate_camera(cam)) return s;
  Frame f;
  if (birp_status s = camera_frame(*cam, f)) return s;
  if (rinv9)
    for (int i = 0; i < 9; ++i) rinv9[i] = f.rinv[i / 3][i % 3];
  if (tan_w) *tan_w = f.tfx;
  if (tan_h) *tan_h = f.tfy;
  if (aspect) *aspect = f.aspect;
  if (step) *step = f.dt;
  if (scale) *scale = f.K;
  if (angle_sun) *angle_sun = f.angle_sun;
  return ok();
}

birp_status birp_render_device(const birp_cube* cube, const birp_cmem* cmem, const birp_camera* cam,
                               float* out_device, void* stream) {
  if (birp_status s = check_init()) return s;
  if (!out_device) return fail(BIRP_ERR_INVALID, "out_device is NULL");
  RequestDev r;
  if (birp_status s = build_request(cube, cmem, *cam, out_device, r)) return s;
  CK(launch_render_plain(r, g_ctx.stats, pick_stream(stream), cmem ? &cmem->h_desc : nullptr));
  return ok();
}

birp_status birp_render(const birp_cube* cube, const birp_cmem* cmem, const birp_camera* cam, float* out_host,
                        void* stream) {
  if (birp_status s = check_init()) return s;
  if (!out_host) return fail(BIRP_ERR_INVALID, "out_host is NULL");
  if (birp_status s = validate_camera(cam)) return s;
  std::lock_guard<std::mutex> lk(g_ctx.mu);
  const size_t npx = (size_t)cam->nx * cam->ny;
  cudaStream_t st = pick_stream(stream);
  RequestDev r;
  if (host_direct_writes()) {
    // the kernel writes every pixel of the caller's image itself
    if (birp_status s = build_request(cube, cmem, *cam, out_host, r)) return s;
    prefault_outputs(&out_host, &npx, 1);
    CK(launch_render_plain(r, g_ctx.stats, st, cmem ? &cmem->h_desc : nullptr));
  } else {
    if (birp_status s = ensure_scratch(npx)) return s;
    if (birp_status s = build_request(cube, cmem, *cam, g_ctx.scratch, r)) return s;
    CK(launch_render_plain(r, g_ctx.stats, st, cmem ? &cmem->h_desc : nullptr));
    CK(cudaMemcpyAsync(out_host, g_ctx.scratch, npx * sizeof(float), cudaMemcpyDeviceToHost, st));
  }
  CK(cudaStreamSynchronize(st));
  return ok();
}

birp_status birp_time_render_device(const birp_cube* cube, const birp_cmem* cmem, const birp_camera* cam,
                                    float* out_device, int repeats, int flush_l2, float* kernel_ms) {
  if (birp_status s = check_init()) return s;
  if (!out_device || !kernel_ms || repeats < 1) return fail(BIRP_ERR_INVALID, "bad argument");
  RequestDev r;
  if (birp_status s = build_request(cube, cmem, *cam, out_device, r)) return s;
  cudaStream_t st = g_ctx.stream;
  const size_t flush_bytes = (size_t)512 << 20;  // larger than the 126 MB L2
  if (flush_l2 && !g_ctx.flush) CK(cudaMalloc(&g_ctx.flush, flush_bytes));
  cudaEvent_t e0, e1;
  CK(cudaEventCreate(&e0));
  CK(cudaEventCreate(&e1));
  float total = 0.f;
  for (int i = 0; i < repeats; ++i) {
    if (flush_l2) CK(cudaMemsetAsync(g_ctx.flush, i & 0xff, flush_bytes, st));
    CK(cudaEventRecord(e0, st));
    CK(launch_render_plain(r, g_ctx.stats, st, cmem ? &cmem->h_desc : nullptr));
    CK(cudaEventRecord(e1, st));
    CK(cudaEventSynchronize(e1));
    float ms = 0.f;
    CK(cudaEventElapsedTime(&ms, e0, e1));
    total += ms;
  }
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  *kernel_ms = total / repeats;
  return ok();
}

birp_status birp_debug_bounds(unsigned long long* status, int reset) {
  if (birp_status s = check_init()) return s;
  if (!status) return fail(BIRP_ERR_INVALID, "NULL argument");
  CK(cudaDeviceSynchronize());
  if (!read_bounds_status(status, reset != 0)) {
    *status = 0;
    return fail(BIRP_ERR_INVALID, "not a bounds-checking build (BIRP_DEBUG_BOUNDS)");
  }
  return ok();
}

birp_status birp_get_kernel_stats(birp_kernel_stats* out, int reset) {
  if (birp_status s = check_init()) return s;
  if (!out) return fail(BIRP_ERR_INVALID, "NULL argument");
  KernelStats k;
  CK(cudaDeviceSynchronize());
  CK(cudaMemcpy(&k, g_ctx.stats, sizeof k, cudaMemcpyDeviceToHost));
  out->exact_range_rays = k.exact_range_rays;
  out->exact_nearest = k.exact_nearest;
  out->exact_cmem = k.exact_cmem;
  out->items = k.items;
  out->samples = k.samples;
  out->cells = k.cells;
  if (reset) CK(cudaMemset(g_ctx.stats, 0, sizeof(KernelStats)));
  if (k.error) return fail(BIRP_ERR_DEVICE, "device check %u failed (info %u)", k.error, k.error_info);
  return ok();
}

}  // extern "C"

extern "C" {

birp_status birp_flush_l2(void) {
  if (birp_status s = check_init()) return s;
  std::lock_guard<std::mutex> lk(g_ctx.mu);
  const size_t flush_bytes = (size_t)512 << 20;
  if (!g_ctx.flush) CK(cudaMalloc(&g_ctx.flush, flush_bytes));
  static unsigned char v = 0;
  CK(cudaMemsetAsync(g_ctx.flush, ++v, flush_bytes, g_ctx.stream));
  CK(cudaStreamSynchronize(g_ctx.stream));
  return ok();
}

birp_status birp_measure_peaks(double* fp32_tflops, double* l2_read_gbs, size_t* l2_buffer_bytes) {
  if (birp_status s = check_init()) return s;
  std::lock_guard<std::mutex> lk(g_ctx.mu);
  cudaStream_t st = g_ctx.stream;
  float* sink = nullptr;
  float4* buf = nullptr;
  // L2 read rate: the largest over L2-resident buffers of 16, 32 and 64 MB
  // (where a buffer's lines sit in the two dies' L2 halves varies with the
  // allocation), read with loads that bypass L1 (a grid-stride pass gives
  // each SM the same slice in every repetition, which L1 would otherwise
  // serve), each launch reading about 2 GB, best of 3 launches per size
  const size_t max_bytes = (size_t)64 << 20;
  CK(cudaMalloc(&sink, sizeof(float)));
  CK(cudaMalloc(&buf, max_bytes));
  CK(cudaMemsetAsync(buf, 0, max_bytes, st));
  cudaEvent_t e0, e1;
  CK(cudaEventCreate(&e0));
  CK(cudaEventCreate(&e1));
  const int blocks = g_ctx.sms * 8, iters = 20000;
  float best_f = 1e30f;
  double best_gbs = 0.0;
  size_t best_bytes = 0;
  for (int rep = 0; rep < 3; ++rep) {
    float ms;
    CK(cudaEventRecord(e0, st));
    CK(launch_peak_fp32(sink, blocks, iters, st));
    CK(cudaEventRecord(e1, st));
    CK(cudaEventSynchronize(e1));
    CK(cudaEventElapsedTime(&ms, e0, e1));
    best_f = std::min(best_f, ms);
  }
  for (size_t bytes : {(size_t)16 << 20, (size_t)32 << 20, max_bytes}) {
    const int reps = (int)(((size_t)2 << 30) / bytes);
    CK(launch_peak_read(buf, bytes / 16, 1, sink, g_ctx.sms * 4, st));  // bring the buffer into L2
    for (int rep = 0; rep < 3; ++rep) {
      float ms;
      CK(cudaEventRecord(e0, st));
      CK(launch_peak_read(buf, bytes / 16, reps, sink, g_ctx.sms * 4, st));
      CK(cudaEventRecord(e1, st));
      CK(cudaEventSynchronize(e1));
      CK(cudaEventElapsedTime(&ms, e0, e1));
      const double gbs = (double)bytes * reps / (ms * 1e-3) / 1e9;
      if (gbs > best_gbs) {
        best_gbs = gbs;
        best_bytes = bytes;
      }
    }
  }
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  cudaFree(sink);
  cudaFree(buf);
  if (fp32_tflops) *fp32_tflops = 2.0 * 8 * iters * (double)blocks * 256 / (best_f * 1e-3) / 1e12;
  if (l2_read_gbs) *l2_read_gbs = best_gbs;
  if (l2_buffer_bytes) *l2_buffer_bytes = best_bytes;
  return ok();
}

}  // extern "C"
