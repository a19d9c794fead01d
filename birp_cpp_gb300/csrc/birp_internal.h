// Internal host/device structures of the GB300 render path.
//
// Data layout in HBM (one cube):
//  * values: one 32-byte record per cell holding the 8 coefficients of its
//    trilinear polynomial f = c0 + c1 x + c2 y + c3 z + c4 xy + c5 xz + c6 yz
//    + c7 xyz in the cell's local coordinates (x, y, z) = p - (lower node)
//    (physical units, so a ray's step along an axis is the same in every
//    cell), computed in FP64 from the FP32 corner values and stored FP32 as
//    {c0, c3, c1, c5 | c2, c6, c4, c7} (the pairs the march's packed FP32x2
//    FMAs take: {c0, c3}, {c1, c5}, {c2, c6}, {c4, c7}); c0 is the value of the cell's lower
//    corner (node k). Records are x fastest for cells -1..n-1 on every axis:
//    one guard cell each side whose outside corners repeat the edge node and
//    whose coefficients along that axis are exactly 0, so a cell index that
//    FP32 rounding puts one step outside [0, n-2] still reads in-bounds
//    memory and interpolates continuously.
//  * per-axis walk tables: float2 {base, exit plane} per cell -1..n-1, one
//    table for rays moving up (exit plane c_{k+1}) and one, stored in reverse
//    cell order, for rays moving down (exit plane c_k), so a ray always walks
//    its table forward. The guard cells' exit planes are +inf / -inf, which
//    ends the walk at the box edge.
//  * compact layout (a cube-creation option for memory-bound uses such as
//    serving many cubes under a byte budget): instead of the records, the
//    FP32 node values with one guard node each side ((nx+2)(ny+2)(nz+2),
//    about 1x the input), the march forming a cell's coefficients from its
//    8 corners in FP32, and float4 walk tables {base, exit plane, 1/width, 0}
//    (1/width = 0 at guard cells).
//  * pairs layout (the middle ground: about 2x the input, near the records
//    layout's speed): the same padded grid, each node a float2 {v, s} of its
//    value and the slope of its z-edge, s = (v(k+1) - v(k)) / (z(k+1) - z(k))
//    computed in FP64 (0 on the guard cells along z), so a cell's 4 z-edges
//    {c + s z} are 4 8-byte loads whose differences along x and y give its 8
//    coefficients; float4 walk tables as in the compact layout.
//  * per-axis index tables (LUT) for nonuniform axes: float4 bins of width at
//    most the smallest cell, each holding one piecewise-linear index map.
//  * FP64 axis coordinates, read only by the exact (FP64) decisions.
#pragma once
#include <cstdint>
#include <cuda_runtime.h>

namespace birp {

constexpr int kMaxLutBins = 1 << 16;  // per axis

// One axis of a cube.
struct AxisDev {
  int n;            // nodes
  int uniform;      // 1: idx = (x - c0) * inv_h (affine); 0: LUT
  float c0;         // first node (FP32)
  float inv_h;      // 1 / spacing (uniform)
  float lut_x0;     // LUT origin (FP32 of c[0])
  float lut_inv_w;  // 1 / bin width
  int lut_n;        // bins
  int lut_off;      // offset of this axis' bins in CubeDev::lut
  double c_first;   // c[0]  (FP64)
  double c_last;    // c[n-1] (FP64)
  const double* c64;  // n FP64 node coordinates (device)
};

struct CubeDev {
  AxisDev ax[3];
  const float4* rec;    // cell records, 2 float4 each (see above)
  uint32_t cx;          // records along x: nx + 1
  uint32_t cxy;         // records per z slab: (nx + 1) * (ny + 1)
  int all_uniform;
  const float4* lut;    // concatenated LUT bins (nullptr if all uniform)
  // walk tables (see above): walk_up[k] + j and walk_dn[k] - j are cell j's
  // entries, j in [-1, n-1]
  const float2* walk_up[3];
  const float2* walk_dn[3];
  // node coordinates of each axis as float pairs {hi, lo} (hi + lo = the
  // FP64 coordinate to ~48 bits), for the nearest-mode crossings; entries
  // -1 and n are the sentinels -inf and +inf
  const float2* nodes_ff[3];
  // compact and pairs layouts (rec == nullptr): padded node values and their
  // strides, and the float4 walk tables (same indexing as walk_up / walk_dn).
  // Node (i, j, k)'s value is grid[record_index(gx, gxy, i, j, k) << gshift]
  // (gshift 0: compact, one float per node; 1: pairs, {v, s} per node).
  int node_vals;        // 1 in the compact and pairs layouts
  int gshift;
  const float* grid;
  uint32_t gx;          // nx + 2
  uint32_t gxy;         // (nx + 2) * (ny + 2)
  const float4* walk4_up[3];
  const float4* walk4_dn[3];
  // cubes holding a value below zero (nullptr otherwise): one byte per node
  // (i, j, k), x fastest, 1 when a node in [i-1, i+2] x [j-1, j+2] x
  // [k-1, k+2] is negative, i.e. when the cell with lower node (i, j, k) or a
  // neighbour of it has a negative corner; with the largest |coordinate|, the
  // inverse of the smallest cell width and the most nodes over the three axes
  // (the bound on how far an FP32 cell index can be off)
  const uint8_t* negflag;
  float neg_cmax, neg_inv_gap;
  int neg_nmax;
  // extents of the tables above, for the bounds-checking build
  // (BIRP_DEBUG_BOUNDS): float4 of rec, floats of grid, entries of the walk
  // table allocation, entries of nodes_ff (sentinels included), LUT bins,
  // negflag bytes
  long long rec_f4, grid_n;
  int walk_n, nodes_n, lut_total;
  long long neg_n;
};

// CMEM coefficients (src/Cmem.cpp:38-115 after Init), FP32 and FP64 copies.
struct CmemDev {
  float p0r0, p1, p2c, p3dn, p3ds, a5, a21, bs, ay, az, A1, A2, B, alpha, beta;
  float bc0, bc1, bc3, cos_tn, sin_tn, cos_ts, sin_ts;
  double d_p0, d_p1, d_p2, d_p3, d_dn, d_ds, d_tn, d_ts, d_r0, d_charlie, d_a5, d_a21;
  double d_bs, d_ay, d_az, d_A1, d_A2, d_B, d_alpha, d_beta, d_bc0, d_bc1, d_bc3;
  float eps_rel;  // FP32 boundary-decision margin (relative to r)
};

// A CMEM model passed by value as a kernel parameter: the kernels that take
// one read its constants as parameter operands (no loads) for the requests
// whose model is `dev`; other requests (dev == nullptr: all) read theirs
// through RequestDev::cmem.
struct CmemParam {
  CmemDev m;
  const CmemDev* dev;
};

enum SpaceKind : int { SPACE_CUBE = 0, SPACE_CMEM = 1 };
// Device layouts of a cube (the values of BIRP_CUBE_*).
enum CubeLayout : int { CUBE_RECORDS = 0, CUBE_COMPACT = 1, CUBE_PAIRS = 2 };
enum MarchMode : int { MARCH_PREFIX = 0, MARCH_CLIP = 1 };

// One render request as the kernels see it (per camera).
struct RequestDev {
  // FP64 frame: exactly the FP64 oracle's pose (R^-1, tan(fov/2), aspect)
  double rinv[3][3];
  double tfx, tfy, aspect;
  double pos[3];
  double dt;
  double K;          // per-sample scale (src/Camera.cpp:201 with ray_width = dt)
  float pos32[3];
  float dt32;
  // pos and dt as float pairs (hi + lo, ~48-bit significands): the nearest-mode
  // walk computes its cell crossings in this float-float arithmetic
  float pos_hi[3], pos_lo[3];
  float dt_hi, dt_lo;
  int nx, ny, N;
  int mode;          // MarchMode
  int interp;        // 1 trilinear, 0 nearest
  int kind;          // SpaceKind
  int seg_log2;      // rays are split over 2^seg_log2 lanes
  int wbx_l2;        // a warp marches 2^wbx_l2 rays across
  int wgx_l2;        // 2^wgx_l2 of the CTA's 4 warps sit across the tile
  int tiles_x;       // tiles along x for this request's tile shape
  int tiles;         // total tiles
  int layout;        // cube: CUBE_RECORDS, CUBE_COMPACT or CUBE_PAIRS
  int has_neg;       // cube: 1 when it holds a value below zero (it carries flags)
  const CubeDev* cube;   // device pointer (kind == SPACE_CUBE)
  const CmemDev* cmem;   // device pointer (kind == SPACE_CMEM)
  float* out;            // ny*nx floats, row 0 = top
};

// Status/counters the kernels report (device memory, read by the host).
struct KernelStats {
  unsigned long long exact_range_rays;   // rays whose in-box range needed FP64
  unsigned long long exact_nearest;      // nearest-mode samples decided in FP64
  unsigned long long exact_cmem;         // CMEM samples decided in FP64
  unsigned long long items;              // work items rendered (persistent kernel)
  unsigned long long samples;            // ray-samples evaluated
  unsigned long long cells;              // cell segments integrated (cell-space march)
  unsigned int error;                    // nonzero: a device-side consistency check failed
  unsigned int error_info;
};

// Work item table of a batch: request r owns items [first[r], first[r+1]).
// The pointers are fixed for the life of a batch object (so a captured CUDA
// graph stays valid); the sizes of each launch are read from device memory.
struct BatchDev {
  const RequestDev* reqs;
  const int* first;        // n_reqs + 1 prefix sums of tiles, in launch order
  const int* order;        // request index of each launch position (largest work first)
  const int* hdr;          // {n_reqs, total_items}
  unsigned int* counter;   // work queue head (zeroed before each launch)
  KernelStats* stats;
};

// Host-side launch helpers (render.cu).
// cmem_host: the host copy of req's CMEM model (CMEM requests), passed to the
// kernel as a parameter
cudaError_t launch_render_plain(const RequestDev& req, KernelStats* stats, cudaStream_t stream,
                                const CmemDev* cmem_host = nullptr);
// Persistent-kernel classes: trilinear cube requests in the records layout
// (fewer registers, more resident warps than the general kernel), the same in
// the compact and in the pairs layout, CMEM requests, nearest-mode cube
// requests (any layout), trilinear requests of cubes holding a negative value
// (any layout; FP64 sums next to negative nodes), and the general kernel that
// renders any request (used where one launch must take a mix, see
// birp_batch_render_noalloc).
enum BatchClass : int {
  BATCH_CUBE_TRI = 0,
  BATCH_ANY = 1,
  BATCH_CUBE_TRI_COMPACT = 2,
  BATCH_CMEM = 3,
  BATCH_CUBE_NEAREST = 4,
  BATCH_CUBE_SIGNED = 5,  // trilinear cubes holding a negative value, any layout
  BATCH_CUBE_TRI_PAIRS = 6,
  BATCH_CLASSES = 7
};
// model: the CMEM model the CMEM class kernel takes as a parameter (nullptr:
// none, every request reads its model through its pointer)
cudaError_t launch_render_batch(const BatchDev& b, int grid, cudaStream_t stream, int cls = BATCH_ANY,
                                const CmemParam* model = nullptr);
// The persistent kernel of class cls (its launch's function, for finding its
// node in a captured graph).
const void* render_batch_function(int cls);
int persistent_grid(int cls);
cudaError_t launch_cube_fill(const float* src_xfast, int nx, int ny, int nz, float* dst, cudaStream_t stream);
// node values (x fastest; device memory or pinned host memory the device
// reads) into the interior of the padded grid
cudaError_t launch_cube_pad_copy(const float* src, int nx, int ny, int nz, float* dst, cudaStream_t stream);
cudaError_t launch_cube_negflags(const float* padded, int nx, int ny, int nz, uint8_t* flags, cudaStream_t stream);
// bounds-checking build: the first out-of-range access (code << 48 | index),
// 0 if none, optionally reset; other builds: always 0, returns false
bool read_bounds_status(unsigned long long* status, bool reset);
cudaError_t launch_cube_records(const float* padded, int nx, int ny, int nz, const double* cx64, const double* cy64,
                                const double* cz64, float4* rec, cudaStream_t stream);
// the pairs layout's {value, z-slope} per padded node (padded: the guard-filled
// scalar grid; cz64: the FP64 z coordinates)
cudaError_t launch_cube_pairs(const float* padded, int nx, int ny, int nz, const double* cz64, float2* pairs,
                              cudaStream_t stream);
cudaError_t launch_cube_sample(const CubeDev* cube, int trilinear, const float* xyz, int n, float* out,
                               cudaStream_t stream);
cudaError_t launch_cmem_sample(const CmemDev* cmem, const float* xyz, int n, float* out, cudaStream_t stream);
cudaError_t launch_cmem_radii_check(const CmemDev* cmem, int n, unsigned long long seed, float* max_err,
                                    cudaStream_t stream);
cudaError_t launch_peak_fp32(float* sink, int blocks, int iters, cudaStream_t stream);
// the CMEM kernel's fast functions beside CUDA's (see birp_fastmath_check)
cudaError_t launch_fastmath(int which, const float* x, const float* y, int n, float* fast, float* lib,
                            cudaStream_t stream);
cudaError_t launch_peak_read(const float4* buf, size_t n4, int reps, float* sink, int blocks, cudaStream_t stream);
// Pixel tile of a request's tile shape (lanes per ray 2^seg_log2, warp-block
// width 2^wbx_l2 rays, 2^wgx_l2 warps across the tile), whether the kernels
// take that shape, and the default warp-block width for seg_log2.
int tile_w(int seg_log2, int wbx_l2, int wgx_l2);
int tile_h(int seg_log2, int wbx_l2, int wgx_l2);
bool tile_shape_ok(int seg_log2, int wbx_l2, int wgx_l2);
int default_wbx_l2(int seg_log2);

}  // namespace birp
