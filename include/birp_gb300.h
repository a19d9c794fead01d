/*
 * C ABI of the GB300 BIRP render path.
 *
 * The render path of the reference (Zach-Clare/birp_cpp) is Camera::Render
 * sampling a Space (a gridded DataCube or the analytic CMEM model). Each entry
 * point below names the reference interface it replaces. Conventions:
 *   - every call returns a birp_status; birp_last_error() gives a message
 *     (per calling thread); no C++ exception crosses this boundary;
 *   - handles are opaque; the caller owns the arrays it passes in and out;
 *   - images are float, ny rows of nx, row 0 = top (as Camera::image);
 *   - a "stream" argument is a cudaStream_t passed as void*; NULL selects the
 *     library's own stream;
 *   - the GPU computes in FP32 with FP64 used for the per-camera pose and for
 *     every decision that must agree exactly with the FP64 oracle.
 */
#ifndef BIRP_GB300_H
#define BIRP_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef enum {
  BIRP_OK = 0,
  BIRP_ERR_INVALID = 1,   /* bad argument; reference: std::invalid_argument (src/DataCube.cpp:136) */
  BIRP_ERR_CUDA = 2,      /* a CUDA call failed */
  BIRP_ERR_NOMEM = 3,     /* device or pinned allocation failed, or over a memory budget */
  BIRP_ERR_SINGULAR = 4,  /* rotation not invertible; reference: std::runtime_error (src/Helper.cpp:243) */
  BIRP_ERR_NOT_INIT = 5,  /* birp_init not called */
  BIRP_ERR_TIMEOUT = 6,   /* a wait ran out of time */
  BIRP_ERR_BUSY = 7,      /* queue full */
  BIRP_ERR_DEVICE = 8     /* a device-side consistency check failed */
} birp_status;

typedef struct birp_cube birp_cube;
typedef struct birp_cmem birp_cmem;

/* Library version (major*10000 + minor*100 + patch). */
int birp_version(void);

/* Selects the CUDA device and creates the library's stream. No reference
 * counterpart (the reference is CPU-only); called once before anything else. */
birp_status birp_init(int device);
/* Frees the library's device state. Handles must be destroyed first. */
void birp_shutdown(void);
/* Message of the last failing call on this thread ("" if none). */
const char* birp_last_error(void);

/* ---------------------------------------------------------------- DataCube */

/* Builds a cube resident in GPU memory from axis node coordinates (strictly
 * increasing, >= 2 nodes each) and values x-fastest:
 * values[(k*ny + j)*nx + i] = slices[k][j][i].
 * Replaces DataCube::Load filling coords_x/y/z, size, spacing, origin_coords
 * and slices (src/DataCube.cpp:28-197, include/DataCube.h:30-42). Nonuniform
 * axes are sampled with a per-cell lookup (the reference's EqualDistance check
 * never fires, src/Helper.cpp:616, so it treats every axis as uniform). */
birp_status birp_cube_create(const double* xs, int nx, const double* ys, int ny, const double* zs, int nz,
                             const float* values, birp_cube** out);
/* Device layouts of a cube (no reference counterpart: the reference keeps
 * nested std::vectors on the host).
 *   RECORDS: one 32-byte record of trilinear coefficients per cell, about 8x
 *            the FP32 values; the fastest to render (the default).
 *   PAIRS:   per node its FP32 value and the slope of its z-edge, plus a guard
 *            layer, about 2x; the kernels form a cell's coefficients from its
 *            4 z-edges (6 differences, 7 products). About 1.2x the records
 *            layout's render time at a quarter of its memory.
 *   COMPACT: the FP32 node values plus a guard layer, about 1x; the kernels
 *            form each cell's coefficients from its 8 corners. For holding
 *            the most cubes under a memory budget (birp_server_config). */
enum { BIRP_CUBE_RECORDS = 0, BIRP_CUBE_COMPACT = 1, BIRP_CUBE_PAIRS = 2 };
/* birp_cube_create with an explicit layout. */
birp_status birp_cube_create_layout(const double* xs, int nx, const double* ys, int ny, const double* zs, int nz,
                                    const float* values, int layout, birp_cube** out);
birp_status birp_cube_destroy(birp_cube* cube);

typedef struct {
  int nx, ny, nz;
  int uniform[3];          /* 1 where the axis is uniform (affine index) */
  size_t device_bytes;     /* GPU memory held by the cube */
  int layout;              /* BIRP_CUBE_RECORDS, BIRP_CUBE_COMPACT or BIRP_CUBE_PAIRS */
} birp_cube_info;
birp_status birp_cube_get_info(const birp_cube* cube, birp_cube_info* info);

/* Samples the cube at n points (xyz interleaved, host arrays); -1 outside the
 * box [c0, c_{n-1}) on any axis. Replaces DataCube::GetSample
 * (src/DataCube.cpp:203-277) with SetTrilinear (:199). */
birp_status birp_cube_sample(const birp_cube* cube, int trilinear, const float* xyz, int n, float* out);

/* ---------------------------------------------------------------- CMEM */

/* The arguments of CMEM::Init (include/Cmem.h:21-41); has_v/has_b = 0 means
 * an empty vector (defaults). 0 means "unset" for the scalar parameters, as
 * in the reference. */
typedef struct {
  int has_v, v[3];
  int has_b, b[3];
  float dipole, p0;
  int p1, p2, p3;
  float B, alpha, beta, bs, A1, A2, ay_bs, az_bs, density;
} birp_cmem_params;

/* Fills the reference's default arguments (CMEM::Init() -> Init(true)). */
void birp_cmem_default_params(birp_cmem_params* p);
/* Runs CMEM::Init's coefficient setup on the host in FP64 (src/Cmem.cpp:38-115,
 * 250-325, including its p2 quirk at :90) and uploads the coefficients. */
birp_status birp_cmem_create(const birp_cmem_params* p, birp_cmem** out);
birp_status birp_cmem_destroy(birp_cmem* cmem);
/* CMEM::GetSample (src/Cmem.cpp:117-186) at n points on the GPU (host arrays). */
birp_status birp_cmem_sample(const birp_cmem* cmem, const float* xyz, int n, float* out);

/* ---------------------------------------------------------------- Camera */

typedef enum { BIRP_MARCH_PREFIX = 0, BIRP_MARCH_CLIP = 1 } birp_march;

/* What Camera holds (include/Camera.h:23-43): position, aim (only aim[0]
 * enters the pose, as in src/Camera.cpp:92-98), field of view in degrees, with
 * explicit image dims (the reference uses round(fov / pixel_size_deg),
 * src/Camera.cpp:38-39), samples per ray (reference 200) and ray length in
 * Earth radii (reference 44): sample i sits at t = (i + 0.5) * ray_length /
 * n_samples. PREFIX stops a ray at its first sample below zero: out of the
 * box, or a negative cube value (the reference, src/Camera.cpp:205-209);
 * CLIP skips such samples up to the first good one and stops at the next.
 * segments: lanes per ray (1, 2, 4, 8), 0 = tuned choice. roll_deg: a roll
 * about the view axis in degrees, added to the Sun-fixed roll angle of
 * Camera::Orient (src/Camera.cpp:309-417); 0 (the default) is the
 * reference's pose exactly (an extension: the reference has no roll input).
 * warp_rays_x, tile_warps_x: the kernels' tile shape, a power of two each
 * (0 = tuned choice): rays across the block of rays one warp marches (of its
 * 32 / segments), and warps across a pixel tile (of 4, so 1, 2 or 4); tiles
 * are at most 32 pixels on a side. The image is the same for every shape
 * (lanes per ray change only the order of the sum). */
typedef struct {
  double pos[3];
  double aim[3];
  double fov_w_deg, fov_h_deg;
  int nx, ny;
  int n_samples;
  double ray_length;
  int trilinear;
  int march;
  int segments;
  double roll_deg;
  int warp_rays_x;
  int tile_warps_x;
} birp_camera;

/* Fills the reference's CLI defaults (src/main.cpp:37-63): pos
 * (5.91813, 6.74116, 17.7067), aim (7.81768, 0, 0), 36 x 36 degrees at 0.25
 * degree pixels (144 x 144), 200 samples over 44 Re, nearest, PREFIX. */
void birp_camera_defaults(birp_camera* cam);

/* Renders one image of a cube (cmem == NULL) or of CMEM (cube == NULL) into a
 * HOST array of ny*nx floats; returns when the image is in out_host.
 * Replaces Camera::Render (src/Camera.cpp:63-233) — except that the output is
 * overwritten, where the reference adds to Camera::image. Where the device
 * accesses pageable host memory coherently (cudaDevAttrPageableMemoryAccess,
 * e.g. Grace over NVLink-C2C) the kernel writes out_host itself; otherwise
 * the image is copied back. BIRP_HOST_DIRECT=0 in the environment forces the
 * copy. */
birp_status birp_render(const birp_cube* cube, const birp_cmem* cmem, const birp_camera* cam, float* out_host,
                        void* stream);
/* Same, into DEVICE memory, asynchronous on the stream. */
birp_status birp_render_device(const birp_cube* cube, const birp_cmem* cmem, const birp_camera* cam,
                               float* out_device, void* stream);

/* The FP64 frame of a camera as the kernels use it: R^-1 (row-major 9),
 * tan(fov_w/2), tan(fov_h/2), aspect nx/ny, step, per-sample scale
 * (src/Camera.cpp:201) and the Sun roll angle of Camera::Orient
 * (src/Camera.cpp:309-417), all FP64. */
birp_status birp_camera_frame(const birp_camera* cam, double* rinv9, double* tan_w, double* tan_h,
                              double* aspect, double* step, double* scale, double* angle_sun);

/* ---------------------------------------------------------------- batches */

/* A batch renders many requests (any mix of cubes, CMEM, image sizes, steps)
 * in ONE launch of a persistent kernel, replayed from a CUDA graph. Replaces
 * the reference's one-render-per-cube loop (src/main.cpp:242-264). */
typedef struct {
  const birp_cube* cube;   /* exactly one of cube / cmem */
  const birp_cmem* cmem;
  birp_camera cam;
} birp_request;

typedef struct birp_batch birp_batch;

/* max_requests and max_pixels bound one launch; the batch owns device and
 * pinned host buffers of that size. */
birp_status birp_batch_create(int max_requests, int64_t max_pixels, birp_batch** out);
birp_status birp_batch_destroy(birp_batch* b);
/* Starts rendering n requests on the batch's stream and returns. */
birp_status birp_batch_submit(birp_batch* b, const birp_request* reqs, int n);
/* Waits for the submitted requests; images land in the batch's pinned host
 * buffer (birp_batch_image). */
birp_status birp_batch_wait(birp_batch* b);
/* Pointer to request i's image in the pinned host buffer, valid until the
 * next submit (NULL after a birp_batch_render that wrote the caller's
 * buffers directly). */
const float* birp_batch_image(const birp_batch* b, int i);
/* submit + wait, with each image in outs[i] (host arrays of ny*nx floats):
 * written by the kernel itself where the device accesses pageable host
 * memory (as birp_render), else copied from the pinned buffer on several
 * host threads. */
birp_status birp_batch_render(birp_batch* b, const birp_request* reqs, int n, float* const* outs);
/* Renders n requests (n <= 256) like birp_batch_submit but allocates nothing,
 * for callers that cannot call cudaMalloc on their render path (code running
 * inside another framework's operator, where that framework owns the device
 * memory; loops that must not allocate). The caller passes the requests and
 * one DEVICE output buffer of ny*nx floats per request; the only other device
 * memory used is a 70 KB array inside this library (held on every GPU that
 * loads it), set up by the first call on each device (make that first call
 * before any stream capture). Runs on the library's device (birp_init), as
 * the other entry points, from any host thread. Asynchronous on `stream`
 * (NULL: the library's stream). A stream that is capturing is refused with
 * BIRP_ERR_INVALID: the request table is copied from a host array that the
 * next call overwrites. Every call shares the device array, so calls whose
 * work overlaps on the GPU race: order them on one stream. More than 256
 * requests, or a NULL output, is BIRP_ERR_INVALID; n = 0 does nothing. No
 * counterpart in the reference. */
birp_status birp_batch_render_noalloc(const birp_request* reqs, int n, float* const* outs_device, void* stream);

/* Device time of the batch's last launch in ms (CUDA events around the
 * graph: H2D of descriptors, kernel, D2H of the images). */
birp_status birp_batch_last_ms(const birp_batch* b, float* kernel_ms, float* total_ms);

/* Bytes each launch of the batch copies host -> device: its request
 * descriptors and work tables (fixed by the batch's max_requests). */
birp_status birp_batch_upload_bytes(const birp_batch* b, size_t* bytes);

/* The library built with BIRP_DEBUG_BOUNDS (libbirp_gb300_debug.so) checks
 * every table access of the render kernels; the first out-of-range one is
 * recorded (code << 48 | index; codes: 1 index table, 2 node value, 3
 * negative-value flag, 4 box plane, 5 walk table, 6 cell record, 7 padded
 * grid, 8 node plane, 9 nearest value) and redirected to a valid element.
 * Gives that status (0: none) and resets it when `reset`; in other builds
 * *status = 0 and BIRP_ERR_INVALID. No counterpart in the reference. */
birp_status birp_debug_bounds(unsigned long long* status, int reset);

/* ---------------------------------------------------------------- serving */

/* A continuous-batching server: requests are admitted as they arrive; a
 * scheduler thread groups pending requests into batches, launches them on
 * `slots` concurrent streams as slots and cube memory free up, and keeps
 * cubes resident in GPU memory under a byte budget with LRU eviction and
 * re-upload from host (pinned) copies. */
typedef struct birp_server birp_server;

typedef struct {
  int64_t cube_budget_bytes;   /* GPU bytes the resident cubes may hold */
  int slots;                   /* batches in flight */
  int max_batch_requests;
  int64_t max_batch_pixels;
  int max_queue;               /* pending requests before submit returns BIRP_ERR_BUSY */
  double max_wait_ms;          /* batching window: launch when this old or the batch is full */
  int cube_layout;             /* device layout of the server's cubes (BIRP_CUBE_*) */
  /* Promotion of popular cubes to a faster layout: promoted_layout
   * (BIRP_CUBE_RECORDS or BIRP_CUBE_PAIRS, faster than cube_layout) and the
   * part of cube_budget_bytes the promoted cubes may hold (0 = none). When
   * no upload is waiting, the most-requested resident cube (at least 16
   * requests) whose promoted copy fits that share is rebuilt in
   * promoted_layout from its host copy and takes the other copy's place;
   * that copy is freed once no batch in flight uses it. No counterpart in the
   * reference. */
  int promoted_layout;
  int64_t promoted_budget_bytes;
  int uploaders;               /* cube uploads in parallel (1..8; one stream each) */
} birp_server_config;

typedef struct {
  int64_t ticket;
  birp_status status;
  double latency_ms;           /* submit -> image in host memory */
  double queue_ms;             /* submit -> launch */
} birp_result;

typedef struct {
  int64_t submitted, completed, rejected, batches;
  int64_t cube_uploads, cube_evictions, cube_hits;
  int64_t resident_bytes;
  int64_t cube_promotions;     /* compact cubes rebuilt in the records layout */
  int64_t promoted_bytes;      /* GPU bytes the promoted cubes hold now */
} birp_server_stats;

void birp_server_default_config(birp_server_config* c);
birp_status birp_server_create(const birp_server_config* c, birp_server** out);
birp_status birp_server_destroy(birp_server* s);
/* Registers a cube whose values stay in HOST memory (copied into pinned
 * memory); it is uploaded on first use and may be evicted. */
birp_status birp_server_add_cube(birp_server* s, const double* xs, int nx, const double* ys, int ny,
                                 const double* zs, int nz, const float* values, int* cube_id);
birp_status birp_server_add_cmem(birp_server* s, const birp_cmem_params* p, int* source_id);
/* Queues one render of source_id; the image is written to out_host
 * (ny*nx floats) before the ticket completes. */
birp_status birp_server_submit(birp_server* s, int source_id, const birp_camera* cam, float* out_host,
                               int64_t* ticket);
/* Waits for a ticket (timeout_ms < 0: no limit). */
birp_status birp_server_wait(birp_server* s, int64_t ticket, double timeout_ms, birp_result* res);
birp_status birp_server_get_stats(const birp_server* s, birp_server_stats* st);

/* ---------------------------------------------------------------- telemetry */

typedef struct {
  uint64_t exact_range_rays;   /* rays whose in-box range was decided in FP64 */
  uint64_t exact_nearest;      /* nearest-mode samples decided in FP64 */
  uint64_t exact_cmem;         /* CMEM samples decided in FP64 */
  uint64_t items;              /* tiles rendered by the persistent kernel */
  uint64_t samples;            /* ray-samples evaluated (the roofline's unit) */
  uint64_t cells;              /* cell segments integrated by the trilinear march */
} birp_kernel_stats;

/* Reads (and optionally clears) the kernels' counters. */
birp_status birp_get_kernel_stats(birp_kernel_stats* st, int reset);

/* Timing of one plain render on the library stream with CUDA events: the
 * render kernel alone (kernel_ms) — used by the benchmark for the roofline. */
birp_status birp_time_render_device(const birp_cube* cube, const birp_cmem* cmem, const birp_camera* cam,
                                    float* out_device, int repeats, int flush_l2, float* kernel_ms);

/* Writes a 512 MB buffer (larger than L2) on the library stream and waits:
 * run between timed renders so each starts with a cold L2. */
birp_status birp_flush_l2(void);

/* Roofline denominators measured on this GPU: FP32 FMA throughput (TFLOP/s,
 * FMA = 2 flops) and the read bandwidth of an L2-resident buffer (GB/s; loads
 * that bypass L1, the best over 16, 32 and 64 MB buffers, whose size is
 * returned in l2_buffer_bytes). Any output may be NULL. No counterpart in the
 * reference. */
birp_status birp_measure_peaks(double* fp32_tflops, double* l2_read_gbs, size_t* l2_buffer_bytes);

/* Largest FP32 error of the CMEM boundary radii against FP64 over n
 * directions, relative to (|r| + 5 Re), where the radius is under 100 Re (a
 * self-check of the margin the kernels use; margin receives that margin). */
birp_status birp_cmem_margin_check(const birp_cmem* cmem, int n, float* max_rel_err, float* margin);

/* The CMEM kernel's fast functions evaluated on the GPU beside CUDA's own at
 * the same n FP32 arguments (host arrays): which = 0 its atan2 for y >= 0
 * (atan2_pos(y, x) vs atan2f(y, x)), 1 its power (pow_pos(x, y) vs powf), 2
 * its square root (sqrt_fast(x) vs sqrtf), 3 its base-2 exponential (ex2_fast
 * vs exp2f); y is ignored by 2 and 3. A self-check of the error bounds the
 * CMEM kernel relies on; no counterpart in the reference. */
birp_status birp_fastmath_check(int which, const float* x, const float* y, int n, float* fast, float* lib);

#ifdef __cplusplus
}
#endif
#endif /* BIRP_GB300_H */
