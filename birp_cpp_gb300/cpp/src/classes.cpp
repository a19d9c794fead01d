// The reference's C++ classes (Space, DataCube, CMEM, Camera) over the GB300
// C ABI (include/birp_gb300.h). Errors come back as the reference's
// exception types: std::invalid_argument for bad input
// (src/DataCube.cpp:136), std::runtime_error for a singular pose
// (src/Helper.cpp:243) and for device errors.
#include <algorithm>
#include <cerrno>
#include <charconv>
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <fstream>
#include <mutex>
#include <sstream>
#include <stdexcept>
#include <string>
#include <system_error>
#include <thread>
#include <vector>

#include "../../../include/birp_gb300.h"
#include "../include/birp/Camera.h"
#include "../include/birp/Cmem.h"
#include "../include/birp/DataCube.h"

namespace {

void check(birp_status s) {
  if (s == BIRP_OK) return;
  std::string msg = birp_last_error();
  if (s == BIRP_ERR_INVALID) throw std::invalid_argument(msg);
  if (s == BIRP_ERR_SINGULAR) throw std::runtime_error("Determinant is 0: " + msg);
  throw std::runtime_error("birp: " + msg);
}

// The device is chosen once per process: BIRP_DEVICE (default 0). Safe to
// call from several threads (a failed first attempt is retried by the next).
void ensure_init() {
  static std::once_flag once;
  std::call_once(once, [] {
    const char* env = std::getenv("BIRP_DEVICE");
    int dev = env ? std::atoi(env) : 0;
    birp_status s = birp_init(dev);
    if (s != BIRP_OK && s != BIRP_ERR_INVALID) check(s);  // throws: call_once runs again next time
  });
}

}  // namespace

// ================================================================ DataCube

DataCube::~DataCube() {
  if (gpu) birp_cube_destroy(gpu);
}

void DataCube::Init() {}

void DataCube::Init(std::string& filename, bool debug) { Load(filename, debug); }

void DataCube::InitMeta() {
  // what InitSpacing / InitOriginCoords / InitSize leave (src/DataCube.cpp:140-197)
  size.x = (int)coords_x.size();
  size.y = (int)coords_y.size();
  size.z = (int)coords_z.size();
  const std::vector<float>* ax[3] = {&coords_x, &coords_y, &coords_z};
  for (int k = 0; k < 3; ++k) {
    spacing[k] = ax[k]->size() >= 2 ? std::abs((*ax[k])[0] - (*ax[k])[1]) : 0.f;
    origin_coords[k] = ax[k]->empty() ? 0.f : (*ax[k])[0];
  }
}

void DataCube::Init(const std::vector<double>& xs, const std::vector<double>& ys, const std::vector<double>& zs,
                    const std::vector<float>& values) {
  const size_t nx = xs.size(), ny = ys.size(), nz = zs.size();
  if (values.size() != nx * ny * nz) throw std::invalid_argument("values size != nx*ny*nz");
  coords_x.assign(xs.begin(), xs.end());
  coords_y.assign(ys.begin(), ys.end());
  coords_z.assign(zs.begin(), zs.end());
  ax64[0] = xs;
  ax64[1] = ys;
  ax64[2] = zs;
  slices.assign(nz, std::vector<std::vector<float>>(ny, std::vector<float>(nx)));
  for (size_t k = 0; k < nz; ++k)
    for (size_t j = 0; j < ny; ++j)
      std::memcpy(slices[k][j].data(), values.data() + (k * ny + j) * nx, nx * sizeof(float));
  InitMeta();
  if (gpu) {  // uploaded again on next use
    birp_cube_destroy(gpu);
    gpu = nullptr;
  }
}

void DataCube::InitFromSpace(Space& src, const std::vector<double>& xs, const std::vector<double>& ys,
                             const std::vector<double>& zs, int threads) {
  if (&src == static_cast<Space*>(this)) throw std::invalid_argument("a cube cannot be sampled from itself");
  const size_t nx = xs.size(), ny = ys.size(), nz = zs.size();
  std::vector<float> vals(nx * ny * nz);
  const int nt = (int)std::max<size_t>(1, std::min<size_t>((size_t)std::max(threads, 1), nz));
  auto slab = [&](int t) {  // z slabs t, t + nt, ...
    for (size_t k = (size_t)t; k < nz; k += (size_t)nt)
      for (size_t j = 0; j < ny; ++j)
        for (size_t i = 0; i < nx; ++i)
          vals[(k * ny + j) * nx + i] = src.GetSample((float)xs[i], (float)ys[j], (float)zs[k]);
  };
  if (nt == 1) {
    slab(0);
  } else {
    std::vector<std::thread> pool;
    for (int t = 0; t < nt; ++t) pool.emplace_back(slab, t);
    for (std::thread& th : pool) th.join();
  }
  Init(xs, ys, zs, vals);
}

namespace {

bool is_space(char c) { return c == ' ' || c == '\n' || c == '\t' || c == '\r' || c == '\v' || c == '\f'; }

// One token's value as the reference reads it (Helper::explode_float ->
// std::stof, src/Helper.cpp:25-38): its leading number, trailing characters
// ignored; 1 if it holds no number (std::invalid_argument there), 2 if the
// number is out of range (std::out_of_range there). std::from_chars reads the
// plain decimal forms; strtof with errno (what std::stof uses) decides the
// rest: a leading '+', hex, values that are zero, subnormal or beyond float.
int token_value(const char* p, const char* tok_end, float& v) {
  auto r = std::from_chars(p, tok_end, v);
  if (r.ec == std::errc() && r.ptr != p && std::isnormal(v)) return 0;
  errno = 0;
  char* q = nullptr;
  v = std::strtof(p, &q);
  if (q == p) return 1;
  return errno == ERANGE ? 2 : 0;
}

// Reads the first `count` white-space separated tokens of [p, end) into out
// on up to 32 threads: chunks split at white space, tokens counted per chunk,
// then each chunk parsed at its offset. Returns 0, or the token_value error
// (also 1 when there are fewer than `count` tokens).
int parse_tokens(const char* p, const char* end, size_t count, float* out) {
  const size_t bytes = (size_t)(end - p);
  unsigned T = std::min(32u, std::max(1u, std::thread::hardware_concurrency()));
  if (bytes < ((size_t)1 << 22)) T = 1;
  std::vector<const char*> cut(T + 1, end);
  cut[0] = p;
  for (unsigned t = 1; t < T; ++t) {
    const char* c = p + bytes / T * t;
    while (c < end && !is_space(*c)) ++c;  // a token stays in the chunk it starts in
    cut[t] = std::max(c, cut[t - 1]);
  }
  std::vector<size_t> n(T, 0), off(T + 1, 0);
  std::vector<int> err(T, 0);
  auto run = [&](auto fn) {
    std::vector<std::thread> ts;
    for (unsigned t = 1; t < T; ++t) ts.emplace_back(fn, t);
    fn(0u);
    for (auto& th : ts) th.join();
  };
  run([&](unsigned t) {
    size_t k = 0;
    bool prev_space = true;
    for (const char* c = cut[t]; c < cut[t + 1]; ++c) {
      const bool s = is_space(*c);
      k += (!s && prev_space);
      prev_space = s;
    }
    n[t] = k;
  });
  for (unsigned t = 0; t < T; ++t) off[t + 1] = off[t] + n[t];
  if (off[T] < count) return 1;
  run([&](unsigned t) {
    const char* c = cut[t];
    for (size_t i = off[t]; i < std::min(off[t + 1], count); ++i) {
      while (is_space(*c)) ++c;
      const char* e = c;
      while (e < cut[t + 1] && !is_space(*e)) ++e;
      if (int r = token_value(c, e, out[i])) {
        err[t] = r;
        return;
      }
      c = e;
    }
  });
  for (int e : err)
    if (e) return e;
  return 0;
}

void throw_token_error(int e) {
  if (e == 2) throw std::out_of_range("Datacube value out of range.");
  throw std::invalid_argument("Datacube is invalid, inaccessible, or malformed.");
}

}  // namespace

// The exported-MHD text format read by the reference (src/DataCube.cpp:28-138):
// line 10 holds the node counts "nx ny nz"; from line 11 come the x, y and z
// node coordinates, then the values with x fastest (rows of x, ny rows per
// slice, nz slices): white-space separated tokens across any line breaks, each
// read as the reference reads a token (std::stof of it). The values are
// parsed on all host threads.
void DataCube::Load(std::string filename, bool debug) {
  std::ifstream f(filename, std::ios::binary | std::ios::ate);
  if (!f) throw std::invalid_argument("Datacube is invalid, inaccessible, or malformed.");
  std::string text((size_t)f.tellg(), '\0');
  f.seekg(0);
  if (!f.read(&text[0], (std::streamsize)text.size()))
    throw std::invalid_argument("Datacube is invalid, inaccessible, or malformed.");
  // locate line 10 and the start of line 11
  size_t pos = 0;
  for (int line = 1; line < 10 && pos != std::string::npos; ++line) {
    pos = text.find('\n', pos);
    if (pos != std::string::npos) ++pos;
  }
  if (pos == std::string::npos) throw std::invalid_argument("Datacube is invalid, inaccessible, or malformed.");
  const char* p = text.c_str() + pos;
  const char* end = text.c_str() + text.size();
  char* q = nullptr;
  long dims[3];
  for (int k = 0; k < 3; ++k) {
    dims[k] = std::strtol(p, &q, 10);
    if (q == p || dims[k] < 2) throw std::invalid_argument("Datacube is invalid, inaccessible, or malformed.");
    p = q;
  }
  std::vector<double> ax[3];
  for (int k = 0; k < 3; ++k) {
    ax[k].resize(dims[k]);
    for (long i = 0; i < dims[k]; ++i) {
      while (p < end && is_space(*p)) ++p;
      const char* e = p;
      while (e < end && !is_space(*e)) ++e;
      float v;
      if (p >= end) throw_token_error(1);
      if (int r = token_value(p, e, v)) throw_token_error(r);
      ax[k][i] = v;  // the reference reads coordinates as float
      p = e;
    }
  }
  const size_t count = (size_t)dims[0] * dims[1] * dims[2];
  std::vector<float> vals(count);
  if (int r = parse_tokens(p, end, count, vals.data())) throw_token_error(r);
  Init(ax[0], ax[1], ax[2], vals);
  if (debug && size.z > 80 && size.y > 79 && size.x > 100) {
    // the reference's debug markers (src/DataCube.cpp:127-133)
    slices[80][79][50] = 1;
    for (int i = 0; i < 101; i++) slices[80][79][i] = 1;
  }
}

void DataCube::Upload() {
  ensure_init();
  if (gpu) {
    birp_cube_destroy(gpu);
    gpu = nullptr;
  }
  const size_t nx = coords_x.size(), ny = coords_y.size(), nz = coords_z.size();
  std::vector<double> xs[3];
  const std::vector<float>* f[3] = {&coords_x, &coords_y, &coords_z};
  for (int k = 0; k < 3; ++k) {
    if (ax64[k].size() == f[k]->size()) xs[k] = ax64[k];
    else xs[k].assign(f[k]->begin(), f[k]->end());
  }
  std::vector<float> flat(nx * ny * nz);
  if (slices.size() < nz) throw std::invalid_argument("slices do not match the axes");
  for (size_t k = 0; k < nz; ++k) {
    if (slices[k].size() < ny) throw std::invalid_argument("slices do not match the axes");
    for (size_t j = 0; j < ny; ++j) {
      if (slices[k][j].size() < nx) throw std::invalid_argument("slices do not match the axes");
      std::memcpy(flat.data() + (k * ny + j) * nx, slices[k][j].data(), nx * sizeof(float));
    }
  }
  check(birp_cube_create_layout(xs[0].data(), (int)nx, xs[1].data(), (int)ny, xs[2].data(), (int)nz, flat.data(),
                                layout, &gpu));
  InitMeta();
}

void DataCube::SetLayout(int l) {
  if (l != BIRP_CUBE_RECORDS && l != BIRP_CUBE_COMPACT && l != BIRP_CUBE_PAIRS)
    throw std::invalid_argument("unknown cube layout");
  if (l != layout && gpu) {  // rebuilt on next use
    birp_cube_destroy(gpu);
    gpu = nullptr;
  }
  layout = l;
}

const birp_cube* DataCube::GpuCube() {
  if (!gpu) Upload();
  return gpu;
}

void DataCube::SetTrilinear(bool option) { trilinear = option; }

void DataCube::GetSamples(const float* xyz, int n, float* out) {
  check(birp_cube_sample(GpuCube(), trilinear ? 1 : 0, xyz, n, out));
}

float DataCube::GetSample(float x, float y, float z) {
  const float p[3] = {x, y, z};
  float out = 0.f;
  GetSamples(p, 1, &out);
  return out;
}

// ================================================================ CMEM

CMEM::~CMEM() {
  if (gpu) birp_cmem_destroy(gpu);
}

void CMEM::Init() { Init(true); }

void CMEM::Init(bool, std::vector<int> v, std::vector<int> b, float dipole, float p0, int p1, int p2, int p3, float B,
                float alpha, float beta, float bs, float A1, float A2, float ay_bs, float az_bs, float density) {
  ensure_init();
  birp_cmem_params p;
  std::memset(&p, 0, sizeof p);
  p.has_v = !v.empty();
  p.has_b = !b.empty();
  for (int i = 0; i < 3; ++i) {
    p.v[i] = (p.has_v && (int)v.size() > i) ? v[i] : 0;
    p.b[i] = (p.has_b && (int)b.size() > i) ? b[i] : 0;
  }
  p.dipole = dipole;
  p.p0 = p0;
  p.p1 = p1;
  p.p2 = p2;
  p.p3 = p3;
  p.B = B;
  p.alpha = alpha;
  p.beta = beta;
  p.bs = bs;
  p.A1 = A1;
  p.A2 = A2;
  p.ay_bs = ay_bs;
  p.az_bs = az_bs;
  p.density = density;
  if (gpu) birp_cmem_destroy(gpu);
  gpu = nullptr;
  check(birp_cmem_create(&p, &gpu));
}

void CMEM::GetSamples(const float* xyz, int n, float* out) {
  if (!gpu) Init();
  check(birp_cmem_sample(gpu, xyz, n, out));
}

float CMEM::GetSample(float x, float y, float z) {
  const float p[3] = {x, y, z};
  float out = 0.f;
  GetSamples(p, 1, &out);
  return out;
}

// ================================================================ Camera

Camera::Camera(Space& cube, float pixel_size_degrees, float plot_fov_h, float plot_fov_w)
    : dataCube(&cube), fov_x(plot_fov_w), fov_y(plot_fov_h), pixel_size_deg(pixel_size_degrees) {
  // image dims as src/Camera.cpp:38-39
  image_dimension_y = (int)std::round(plot_fov_h / pixel_size_deg);
  image_dimension_x = (int)std::round(plot_fov_w / pixel_size_deg);
  image.assign(image_dimension_y, std::vector<float>(image_dimension_x, 0.f));
}

Camera::Camera(Space& cube, float plot_fov_h, float plot_fov_w, int nx, int ny)
    : dataCube(&cube), image_dimension_x(nx), image_dimension_y(ny), fov_x(plot_fov_w), fov_y(plot_fov_h),
      pixel_size_deg(plot_fov_w / (float)nx) {
  image.assign(image_dimension_y, std::vector<float>(image_dimension_x, 0.f));
}

Camera::~Camera() {}

void Camera::SetPosition(float& x, float& y, float& z) {
  position.x = x;
  position.y = y;
  position.z = z;
}

void Camera::SetAim(float x, float y, float z) {
  aim.x = x;
  aim.y = y;
  aim.z = z;
}

void Camera::SetSamples(int n, double length) {
  ray_samples = n;
  ray_length = length;
}

void Camera::SetStep(double step, double length) {
  if (!(step > 0)) throw std::invalid_argument("step must be positive");
  ray_samples = (int)std::lround(length / step);
  ray_length = length;
}

void Camera::SetMarchMode(int mode) { march = mode; }

void Camera::SetSegments(int lanes) { segments = lanes; }

void Camera::SetRoll(double degrees) { roll_deg = degrees; }

birp_camera Camera::Describe() const {
  birp_camera c;
  std::memset(&c, 0, sizeof c);
  c.pos[0] = position.x;
  c.pos[1] = position.y;
  c.pos[2] = position.z;
  c.aim[0] = aim.x;
  c.aim[1] = aim.y;
  c.aim[2] = aim.z;
  c.fov_w_deg = fov_x;
  c.fov_h_deg = fov_y;
  c.nx = image_dimension_x;
  c.ny = image_dimension_y;
  c.n_samples = ray_samples;
  c.ray_length = ray_length;
  c.trilinear = dataCube->Trilinear() ? 1 : 0;
  c.march = march;
  c.segments = segments;
  c.roll_deg = roll_deg;
  return c;
}

namespace {

// the GPU source of a Space: exactly one of cube / cmem
void gpu_source(Space* s, const birp_cube*& cube, const birp_cmem*& cmem) {
  cube = s->GpuCube();
  cmem = cube ? nullptr : s->GpuCmem();
  if (!cube && !cmem)
    throw std::invalid_argument(
        "this Space has no GPU representation (DataCube or CMEM); DataCube::InitFromSpace samples it onto a grid");
}

// the reference accumulates into image (src/Camera.cpp:223)
void accumulate(std::vector<std::vector<float>>& image, const float* out, int nx, int ny) {
  for (int j = 0; j < ny; ++j)
    for (int i = 0; i < nx; ++i) image[j][i] = image[j][i] + out[(size_t)j * nx + i];
}

}  // namespace

void Camera::Render() {
  ensure_init();
  const birp_camera c = Describe();
  const birp_cube* cube;
  const birp_cmem* cmem;
  gpu_source(dataCube, cube, cmem);
  std::vector<float> out((size_t)c.nx * c.ny);
  check(birp_render(cube, cmem, &c, out.data(), nullptr));
  accumulate(image, out.data(), c.nx, c.ny);
}

void RenderBatch(const std::vector<Camera*>& cameras) {
  ensure_init();
  if (cameras.empty()) return;
  std::vector<birp_request> reqs(cameras.size());
  std::vector<std::vector<float>> outs(cameras.size());
  std::vector<float*> ptrs(cameras.size());
  int64_t pixels = 0;
  for (size_t i = 0; i < cameras.size(); ++i) {
    reqs[i].cam = cameras[i]->Describe();
    gpu_source(cameras[i]->dataCube, reqs[i].cube, reqs[i].cmem);
    outs[i].resize((size_t)reqs[i].cam.nx * reqs[i].cam.ny);
    ptrs[i] = outs[i].data();
    pixels += (int64_t)outs[i].size();
  }
  birp_batch* b = nullptr;
  check(birp_batch_create((int)cameras.size(), pixels, &b));
  const birp_status st = birp_batch_render(b, reqs.data(), (int)reqs.size(), ptrs.data());
  birp_batch_destroy(b);
  check(st);
  for (size_t i = 0; i < cameras.size(); ++i)
    accumulate(cameras[i]->image, outs[i].data(), reqs[i].cam.nx, reqs[i].cam.ny);
}

int Camera::ToDat(std::string filename) {
  std::ofstream outfile(filename + ".dat");
  for (int j = 0; j < image_dimension_y; ++j) {
    for (int i = 0; i < image_dimension_x; ++i) {
      outfile << std::to_string(image[j][i]);
      outfile << ",";
    }
    outfile << "\n";
  }
  return 1;
}

namespace {

// One 80-character FITS header card.
std::string card(const std::string& key, const std::string& value, const std::string& comment = "") {
  char buf[96];
  std::string k = key;
  for (char& ch : k) ch = (char)std::toupper((unsigned char)ch);
  std::snprintf(buf, sizeof buf, "%-8.8s= %20s", k.c_str(), value.c_str());
  std::string s = buf;
  if (!comment.empty()) s += " / " + comment;
  s.resize(80, ' ');
  return s;
}

std::string fnum(double v) {
  char b[32];
  std::snprintf(b, sizeof b, "%.9G", v);
  return b;
}

}  // namespace

// A single-image FITS file (primary HDU, BITPIX -32, big-endian float32)
// with the reference's cards (src/Camera.cpp:263-286): CRVAL1/CDELT1,
// CRVAL2/CDELT2 in degrees, POS_X..AIM_Z and the RHO record. Rows are
// written from image row 0 (the top), like the reference's raster.
int Camera::ToFITS(std::string filename) {
  std::string hdr;
  hdr += card("SIMPLE", "T", "conforms to FITS standard");
  hdr += card("BITPIX", "-32", "IEEE single precision");
  hdr += card("NAXIS", "2");
  hdr += card("NAXIS1", std::to_string(image_dimension_x));
  hdr += card("NAXIS2", std::to_string(image_dimension_y));
  hdr += card("CRVAL1", fnum(-(fov_x / 2)), "[deg]");
  hdr += card("CDELT1", fnum(pixel_size_deg), "[deg]");
  hdr += card("CRVAL2", fnum(-(fov_y / 2)), "[deg]");
  hdr += card("CDELT2", fnum(pixel_size_deg), "[deg]");
  hdr += card("POS_X", fnum(position.x), "[float]");
  hdr += card("POS_Y", fnum(position.y), "[float]");
  hdr += card("POS_Z", fnum(position.z), "[float]");
  hdr += card("AIM_X", fnum(aim.x), "[float]");
  hdr += card("AIM_Y", fnum(aim.y), "[float]");
  hdr += card("AIM_Z", fnum(aim.z), "[float]");
  hdr += card("RHO", "'0       '", "[t] comment");
  std::string endc = "END";
  endc.resize(80, ' ');
  hdr += endc;
  hdr.resize((hdr.size() + 2879) / 2880 * 2880, ' ');
  std::vector<unsigned char> data;
  data.reserve((size_t)image_dimension_x * image_dimension_y * 4);
  for (int j = 0; j < image_dimension_y; ++j)
    for (int i = 0; i < image_dimension_x; ++i) {
      uint32_t u;
      std::memcpy(&u, &image[j][i], 4);
      for (int s = 24; s >= 0; s -= 8) data.push_back((unsigned char)(u >> s));
    }
  data.resize((data.size() + 2879) / 2880 * 2880, 0);
  std::ofstream f(filename + ".fits", std::ios::binary | std::ios::trunc);
  f.write(hdr.data(), (std::streamsize)hdr.size());
  f.write(reinterpret_cast<const char*>(data.data()), (std::streamsize)data.size());
  return 1;
}
