// Host-side internals shared by the C ABI translation units.
#pragma once
#include <cuda_runtime.h>

#include <cstdint>
#include <mutex>
#include <vector>

#include "../../include/birp_gb300.h"
#include "birp_internal.h"

// Opaque handle types of the C ABI.
struct birp_cube {
  int n[3] = {0, 0, 0};
  std::vector<double> c[3];     // host copies of the axes
  int uniform[3] = {0, 0, 0};
  double inv_h[3] = {0, 0, 0};  // uniform axes: 1 / spacing
  double min_gap[3] = {0, 0, 0};
  birp::CubeDev h_desc{};       // host copy of the device descriptor
  birp::CubeDev* d_desc = nullptr;
  float4* d_vals = nullptr;     // cell records (birp_internal.h)
  double* d_c64 = nullptr;      // 3 axes, concatenated
  float4* d_lut = nullptr;
  float2* d_cells = nullptr;    // walk tables (up and down) of the 3 axes, concatenated
  int layout = BIRP_CUBE_RECORDS;
  float* d_grid = nullptr;      // compact layout: padded node values
  float2* d_pairs = nullptr;    // pairs layout: padded {value, z-slope} per node
  float4* d_walk4 = nullptr;    // compact and pairs layouts: walk tables with inverse widths
  float2* d_nodes_ff = nullptr; // node coordinates as float pairs, 3 axes concatenated
  int has_neg = -1;             // a value below zero (-1: not yet known)
  uint8_t* d_negflag = nullptr; // its negative-value flags (CubeDev::negflag)
  size_t device_bytes = 0;
  cudaStream_t alloc_stream = nullptr;  // non-null: stream-ordered (pool) allocations
};

struct birp_cmem {
  birp::CmemDev h_desc{};
  birp::CmemDev* d_desc = nullptr;
};

namespace birp {

// Library context: one device per process.
struct Context {
  int device = -1;
  int sms = 0;
  cudaStream_t stream = nullptr;
  KernelStats* stats = nullptr;
  float* scratch = nullptr;      // image buffer of birp_render
  size_t scratch_floats = 0;
  float* xyz_scratch = nullptr;  // point-sample buffers
  size_t xyz_floats = 0;
  void* flush = nullptr;         // L2 flush buffer (timing)
  int pageable_access = 0;       // kernels may write pageable host memory
  std::mutex mu;
};
extern Context g_ctx;

// True when render outputs in host memory are written by the kernels
// directly (the device reads and writes pageable host memory coherently,
// e.g. over NVLink-C2C); BIRP_HOST_DIRECT=0 in the environment turns it off.
bool host_direct_writes();
// memcpy of many (dst, src, bytes) pieces on up to 8 host threads.
void parallel_copy(float* const* dst, const float* const* src, const size_t* floats, int n);
// Writes one float per host page of each output image (on up to 8 threads)
// so the pages are mapped before a kernel writes them: a device fault on an
// unmapped page of pageable memory is far slower than a host write. Only for
// outputs the kernel then overwrites whole.
void prefault_outputs(float* const* dst, const size_t* floats, int n);

// FP64 camera frame (see camera_frame in capi.cu).
struct Frame {
  double rinv[3][3];
  double tfx, tfy, aspect, dt, K, angle_sun;
};

birp_status fail(birp_status s, const char* fmt, ...);
birp_status ok();
birp_status check_init();
birp_status validate_camera(const birp_camera* c);
birp_status camera_frame(const birp_camera& c, Frame& f);
// batched: the request is rendered inside a batch (lanes-per-ray table)
birp_status build_request(const birp_cube* cube, const birp_cmem* cmem, const birp_camera& c, float* out,
                          RequestDev& r, bool batched = false);
cudaStream_t pick_stream(void* s);

// cube.cu
birp_status analyze_axis(const double* c, int n, char name, birp_cube& cube, int k);
// builds the device form of cube.layout (cube.n, cube.c, ... already set)
birp_status upload_cube(birp_cube& cube, const float* values, cudaStream_t stream, bool stream_alloc);
// estimate of the device bytes a cube of these dims will hold
size_t cube_device_bytes(const birp_cube& cube);
// whether any of the n values is below zero (a NaN is not)
bool any_negative(const float* v, size_t n);
void destroy_cube_device(birp_cube& cube);
birp_status ensure_xyz_scratch(size_t floats);

// cmem_host.cpp
void cmem_coefficients(const birp_cmem_params& p, CmemDev& m);

// tune.cpp: tile shape from the committed tuning tables (-1: the default for
// the lanes per ray)
struct TunedShape {
  int seg_log2, wbx_l2, wgx_l2;
};
TunedShape tuned_shape(int64_t pixels, int n_samples, int kind, int trilinear, bool batched);

}  // namespace birp
