// DataCube upload: axis analysis, index tables for nonuniform axes and the
// guard-padded FP32 grid in HBM (layout in birp_internal.h). Replaces the
// state DataCube::Load / InitSpacing / InitOriginCoords / InitSize leave
// behind (src/DataCube.cpp:28-197).
#include <algorithm>
#include <cmath>
#include <cstring>
#include <vector>

#include "birp_host.h"

namespace birp {

birp_status analyze_axis(const double* c, int n, char name, birp_cube& cube, int k) {
  if (n < 2) return fail(BIRP_ERR_INVALID, "axis %c needs at least 2 nodes (got %d)", name, n);
  for (int i = 0; i < n; ++i)
    if (!std::isfinite(c[i])) return fail(BIRP_ERR_INVALID, "axis %c node %d is not finite", name, i);
  double min_gap = INFINITY;
  for (int i = 1; i < n; ++i) {
    double g = c[i] - c[i - 1];
    if (!(g > 0)) return fail(BIRP_ERR_INVALID, "axis %c must be strictly increasing (node %d)", name, i);
    min_gap = std::min(min_gap, g);
  }
  const double h = (c[n - 1] - c[0]) / (n - 1);
  bool uniform = true;
  for (int i = 1; i < n && uniform; ++i) uniform = std::abs((c[i] - c[i - 1]) - h) <= 1e-6 * h;
  cube.n[k] = n;
  cube.c[k].assign(c, c + n);
  cube.uniform[k] = uniform ? 1 : 0;
  cube.inv_h[k] = 1.0 / h;
  cube.min_gap[k] = min_gap;
  const double span = c[n - 1] - c[0];
  if (span / min_gap > (double)kMaxLutBins)
    return fail(BIRP_ERR_INVALID, "axis %c: span / smallest cell = %.0f exceeds %d", name, span / min_gap,
                kMaxLutBins);
  return BIRP_OK;
}

// Index table of one axis: bins of width w = the smallest cell; bin b covers
// [c0 + b w, c0 + (b+1) w) and holds {xk, kk, s0, s1} with the continuous index
// idx(x) = kk + (x - xk) * (x < xk ? s0 : s1): xk is the one node strictly
// inside the bin (if any; else the node below the bin start), kk its index,
// s0/s1 the inverse widths of the cells left/right of it.
static void build_lut(const std::vector<double>& c, double w, std::vector<float4>& lut) {
  const int n = (int)c.size();
  const int nb = std::max(1, (int)std::ceil((c[n - 1] - c[0]) / w));
  lut.resize(nb);
  int k = 0;
  for (int b = 0; b < nb; ++b) {
    const double xb = c[0] + b * w;
    while (k < n - 2 && c[k + 1] <= xb) ++k;
    double xk, s0, s1;
    int kk;
    const double inv_k = 1.0 / (c[k + 1] - c[k]);
    if (c[k + 1] > xb && c[k + 1] < xb + w) {
      xk = c[k + 1];
      kk = k + 1;
      s0 = inv_k;
      s1 = (k + 2 <= n - 1) ? 1.0 / (c[k + 2] - c[k + 1]) : inv_k;
    } else {
      xk = c[k];
      kk = k;
      s0 = s1 = inv_k;
    }
    lut[b] = make_float4((float)xk, (float)kk, (float)s0, (float)s1);
  }
}

bool any_negative(const float* v, size_t n) {
  // sign bits first, per chunk (a loop the compiler vectorises); a chunk with
  // one set (-0.0, a negative value or a NaN) is tested exactly
  constexpr size_t kChunk = 1 << 16;
  for (size_t i0 = 0; i0 < n; i0 += kChunk) {
    const size_t i1 = std::min(n, i0 + kChunk);
    uint32_t sign = 0;
    for (size_t i = i0; i < i1; ++i) {
      uint32_t b;
      std::memcpy(&b, v + i, sizeof b);
      sign |= b;
    }
    if (sign & 0x80000000u)
      for (size_t i = i0; i < i1; ++i)
        if (v[i] < 0.f) return true;
  }
  return false;
}

birp_status ensure_xyz_scratch(size_t floats) {
  Context& g = g_ctx;
  if (g.xyz_floats >= floats) return BIRP_OK;
  if (g.xyz_scratch) cudaFree(g.xyz_scratch);
  g.xyz_scratch = nullptr;
  g.xyz_floats = 0;
  size_t want = std::max(floats, (size_t)1 << 16);
  cudaError_t e = cudaMalloc(&g.xyz_scratch, want * sizeof(float));
  if (e != cudaSuccess) return fail(BIRP_ERR_NOMEM, "cudaMalloc: %s", cudaGetErrorString(e));
  g.xyz_floats = want;
  return BIRP_OK;
}

void destroy_cube_device(birp_cube& c) {
  if (c.alloc_stream) {
    // stream-ordered pool memory: no device-wide synchronisation on release
    for (void* p : {(void*)c.d_vals, (void*)c.d_c64, (void*)c.d_lut, (void*)c.d_desc, (void*)c.d_cells,
                    (void*)c.d_grid, (void*)c.d_pairs, (void*)c.d_walk4, (void*)c.d_nodes_ff, (void*)c.d_negflag})
      if (p) cudaFreeAsync(p, c.alloc_stream);
  } else {
    for (void* p : {(void*)c.d_vals, (void*)c.d_c64, (void*)c.d_lut, (void*)c.d_desc, (void*)c.d_cells,
                    (void*)c.d_grid, (void*)c.d_pairs, (void*)c.d_walk4, (void*)c.d_nodes_ff, (void*)c.d_negflag})
      if (p) cudaFree(p);
  }
  c.d_pairs = nullptr;
  c.d_negflag = nullptr;
  c.d_nodes_ff = nullptr;
  c.d_grid = nullptr;
  c.d_walk4 = nullptr;
  c.d_cells = nullptr;
  c.d_vals = nullptr;
  c.d_c64 = nullptr;
  c.d_lut = nullptr;
  c.d_desc = nullptr;
}

#define CKU(x)                                                                                 \
  do {                                                                                         \
    cudaError_t e_ = (x);                                                                      \
    if (e_ != cudaSuccess)                                                                     \
      return fail(e_ == cudaErrorMemoryAllocation ? BIRP_ERR_NOMEM : BIRP_ERR_CUDA, "%s: %s", #x, \
                  cudaGetErrorString(e_));                                                     \
  } while (0)

template <class T>
static cudaError_t dev_alloc(T** p, size_t bytes, cudaStream_t alloc_stream) {
  return alloc_stream ? cudaMallocAsync((void**)p, bytes, alloc_stream) : cudaMalloc((void**)p, bytes);
}

birp_status upload_cube(birp_cube& c, const float* values, cudaStream_t st, bool stream_alloc) {
  const int nx = c.n[0], ny = c.n[1], nz = c.n[2];
  const size_t px = (size_t)nx + 2, py = (size_t)ny + 2, pz = (size_t)nz + 2;
  const size_t total = px * py * pz;
  const size_t nodes = (size_t)nx * ny * nz;
  if (c.has_neg < 0) c.has_neg = any_negative(values, nodes) ? 1 : 0;
  if (!st) st = g_ctx.stream;
  c.alloc_stream = stream_alloc ? st : nullptr;

  CubeDev& d = c.h_desc;
  std::memset(&d, 0, sizeof d);
  d.all_uniform = (c.uniform[0] && c.uniform[1] && c.uniform[2]) ? 1 : 0;

  // index tables for every axis when any axis is nonuniform
  std::vector<float4> lut;
  int lut_off[3] = {0, 0, 0}, lut_n[3] = {0, 0, 0};
  if (!d.all_uniform) {
    for (int k = 0; k < 3; ++k) {
      std::vector<float4> one;
      build_lut(c.c[k], c.min_gap[k], one);
      lut_off[k] = (int)lut.size();
      lut_n[k] = (int)one.size();
      lut.insert(lut.end(), one.begin(), one.end());
    }
  }

  size_t coords = (size_t)nx + ny + nz;
  // walk tables of every axis, per cell -1..n-1: the up table in cell order,
  // then the down table in reverse cell order. Guard cells take the edge node
  // as base (their coefficients along the axis are 0) and an infinite exit
  // plane, so the walk stops there. Records layout: float2 {base, exit
  // plane}; compact and pairs layouts: float4 {base, exit plane, 1/width (0
  // at guard cells), 0}. One padding entry at the end: a walk that reads one
  // entry ahead of its cell may read one past the last table's guard cell
  // (the value is never used).
  const bool compact = c.layout == BIRP_CUBE_COMPACT;
  const bool pairs = c.layout == BIRP_CUBE_PAIRS;
  const bool nodes_layout = compact || pairs;  // node values (no records)
  std::vector<float4> walk;
  walk.reserve(2 * (coords + 3) + 1);
  size_t up_off[3], dn_off[3];
  for (int k = 0; k < 3; ++k) {
    const std::vector<double>& ck = c.c[k];
    const int n = c.n[k];
    auto iw = [&](int j) { return (float)(1.0 / (ck[j + 1] - ck[j])); };
    walk.push_back(make_float4((float)ck[0], (float)ck[0], 0.f, 0.f));  // cell -1
    up_off[k] = walk.size();
    for (int j = 0; j + 1 < n; ++j) walk.push_back(make_float4((float)ck[j], (float)ck[j + 1], iw(j), 0.f));
    walk.push_back(make_float4((float)ck[n - 1], INFINITY, 0.f, 0.f));  // cell n-1
    walk.push_back(make_float4((float)ck[n - 1], (float)ck[n - 1], 0.f, 0.f));  // cell n-1
    for (int j = n - 2; j >= 0; --j) walk.push_back(make_float4((float)ck[j], (float)ck[j], iw(j), 0.f));
    dn_off[k] = walk.size() - 1;  // cell 0
    walk.push_back(make_float4((float)ck[0], -INFINITY, 0.f, 0.f));  // cell -1
  }
  walk.push_back(make_float4(0.f, 0.f, 0.f, 0.f));
  std::vector<float2> walk2;
  if (!nodes_layout) {
    walk2.reserve(walk.size());
    for (const float4& w : walk) walk2.push_back(make_float2(w.x, w.y));
  }
  const size_t records = ((size_t)nx + 1) * ((size_t)ny + 1) * ((size_t)nz + 1);
  // the padded scalar grid; records and pairs layouts: turned into records
  // (pairs), then freed (held in d_grid until then, so a failed upload
  // releases it with the rest)
  float* scalar = nullptr;
  CKU(dev_alloc(&scalar, total * sizeof(float), c.alloc_stream));
  c.d_grid = scalar;
  if (nodes_layout) {
    CKU(dev_alloc(&c.d_walk4, walk.size() * sizeof(float4), c.alloc_stream));
    if (pairs) CKU(dev_alloc(&c.d_pairs, total * sizeof(float2), c.alloc_stream));
  } else {
    CKU(dev_alloc(&c.d_cells, walk2.size() * sizeof(float2), c.alloc_stream));
    CKU(dev_alloc(&c.d_vals, records * 2 * sizeof(float4), c.alloc_stream));
    // the walk reads a record with one 32-byte load, which needs 32-byte
    // alignment (device allocations are 256-byte aligned)
    if (reinterpret_cast<uintptr_t>(c.d_vals) % 32 != 0)
      return fail(BIRP_ERR_CUDA, "cell records not 32-byte aligned");
  }
  CKU(dev_alloc(&c.d_c64, coords * sizeof(double), c.alloc_stream));
  CKU(dev_alloc(&c.d_nodes_ff, (coords + 6) * sizeof(float2), c.alloc_stream));
  if (!lut.empty()) CKU(dev_alloc(&c.d_lut, lut.size() * sizeof(float4), c.alloc_stream));
  CKU(dev_alloc(&c.d_desc, sizeof(CubeDev), c.alloc_stream));
  if (c.has_neg) CKU(dev_alloc(&c.d_negflag, nodes, c.alloc_stream));
  c.device_bytes = coords * sizeof(double) + (coords + 6) * sizeof(float2) + lut.size() * sizeof(float4) +
                   sizeof(CubeDev) + (c.has_neg ? nodes : 0) +
                   (compact ? total * sizeof(float) + walk.size() * sizeof(float4)
                    : pairs ? total * sizeof(float2) + walk.size() * sizeof(float4)
                            : records * 2 * sizeof(float4) + walk2.size() * sizeof(float2));

  // interior values from the caller's x-fastest array: pinned host memory
  // (the server's copies) is read by a kernel straight into the padded grid;
  // other (pageable) memory goes by one strided 3D copy
  cudaPointerAttributes pa{};
  const bool pinned = cudaPointerGetAttributes(&pa, values) == cudaSuccess && pa.type == cudaMemoryTypeHost;
  cudaGetLastError();  // (an unregistered pointer is not an error to keep)
  if (pinned) {
    CKU(launch_cube_pad_copy(values, nx, ny, nz, scalar, st));
  } else {
    cudaMemcpy3DParms p;
    std::memset(&p, 0, sizeof p);
    p.srcPtr = make_cudaPitchedPtr((void*)values, (size_t)nx * sizeof(float), nx, ny);
    p.dstPtr = make_cudaPitchedPtr(scalar, px * sizeof(float), px, py);
    p.dstPos = make_cudaPos(sizeof(float), 1, 1);
    p.extent = make_cudaExtent((size_t)nx * sizeof(float), ny, nz);
    p.kind = cudaMemcpyHostToDevice;
    CKU(cudaMemcpy3DAsync(&p, st));
  }
  CKU(launch_cube_fill(nullptr, nx, ny, nz, scalar, st));
  if (c.has_neg) CKU(launch_cube_negflags(scalar, nx, ny, nz, c.d_negflag, st));
  // (the host vectors below stay alive until the synchronize at the end)
  std::vector<double> all;
  all.reserve(coords);
  for (int k = 0; k < 3; ++k) all.insert(all.end(), c.c[k].begin(), c.c[k].end());
  CKU(cudaMemcpyAsync(c.d_c64, all.data(), coords * sizeof(double), cudaMemcpyHostToDevice, st));
  // node coordinates as float pairs, each axis between sentinels -inf / +inf
  // (a walk past the last plane finds no crossing)
  std::vector<float2> nodes_ff;
  nodes_ff.reserve(coords + 6);
  size_t ff_off[3];
  for (int k = 0, o = 0; k < 3; o += c.n[k], ++k) {
    nodes_ff.push_back(make_float2(-INFINITY, 0.f));
    ff_off[k] = nodes_ff.size();
    for (int i = 0; i < c.n[k]; ++i) {
      const double v = all[o + i];
      const float h = (float)v;
      nodes_ff.push_back(make_float2(h, (float)(v - (double)h)));
    }
    nodes_ff.push_back(make_float2(INFINITY, 0.f));
  }
  CKU(cudaMemcpyAsync(c.d_nodes_ff, nodes_ff.data(), nodes_ff.size() * sizeof(float2), cudaMemcpyHostToDevice, st));
  if (nodes_layout) {
    CKU(cudaMemcpyAsync(c.d_walk4, walk.data(), walk.size() * sizeof(float4), cudaMemcpyHostToDevice, st));
    if (pairs) {
      CKU(launch_cube_pairs(scalar, nx, ny, nz, c.d_c64 + nx + ny, c.d_pairs, st));
      if (c.alloc_stream) {
        c.d_grid = nullptr;
        CKU(cudaFreeAsync(scalar, st));
      }
    }
  } else {
    CKU(launch_cube_records(scalar, nx, ny, nz, c.d_c64, c.d_c64 + nx, c.d_c64 + nx + ny, c.d_vals, st));
    if (c.alloc_stream) {
      c.d_grid = nullptr;
      CKU(cudaFreeAsync(scalar, st));
    }
    CKU(cudaMemcpyAsync(c.d_cells, walk2.data(), walk2.size() * sizeof(float2), cudaMemcpyHostToDevice, st));
  }
  if (!lut.empty()) CKU(cudaMemcpyAsync(c.d_lut, lut.data(), lut.size() * sizeof(float4), cudaMemcpyHostToDevice, st));

  size_t off = 0;
  for (int k = 0; k < 3; ++k) {
    AxisDev& a = d.ax[k];
    const std::vector<double>& ck = c.c[k];
    a.n = c.n[k];
    a.uniform = c.uniform[k];
    a.c0 = (float)ck[0];
    a.inv_h = (float)c.inv_h[k];
    a.lut_x0 = (float)ck[0];
    a.lut_inv_w = (float)(1.0 / c.min_gap[k]);
    a.lut_n = lut_n[k];
    a.lut_off = lut_off[k];
    a.c_first = ck[0];
    a.c_last = ck[a.n - 1];
    a.c64 = c.d_c64 + off;
    d.nodes_ff[k] = c.d_nodes_ff + ff_off[k];
    off += a.n;
  }
  d.negflag = c.d_negflag;
  d.rec_f4 = nodes_layout ? 0 : (long long)(records * 2);
  d.grid_n = compact ? (long long)total : pairs ? 2 * (long long)total : 0;
  d.walk_n = (int)walk.size();
  d.nodes_n = (int)nodes_ff.size();
  d.lut_total = (int)lut.size();
  d.neg_n = c.has_neg ? (long long)nodes : 0;
  if (c.has_neg) {
    double cmax = 0.0, inv_gap = 0.0;
    for (int k = 0; k < 3; ++k) {
      cmax = std::max({cmax, std::abs(c.c[k].front()), std::abs(c.c[k].back())});
      inv_gap = std::max(inv_gap, 1.0 / c.min_gap[k]);
      d.neg_nmax = std::max(d.neg_nmax, c.n[k]);
    }
    d.neg_cmax = (float)cmax;
    d.neg_inv_gap = (float)inv_gap;
  }
  d.rec = c.d_vals;
  d.cx = (uint32_t)(nx + 1);
  d.cxy = (uint32_t)((nx + 1) * (ny + 1));
  d.lut = c.d_lut;
  d.node_vals = nodes_layout ? 1 : 0;
  d.gshift = pairs ? 1 : 0;
  d.grid = compact ? c.d_grid : pairs ? reinterpret_cast<const float*>(c.d_pairs) : nullptr;
  d.gx = (uint32_t)px;
  d.gxy = (uint32_t)(px * py);
  for (int k = 0; k < 3; ++k) {
    if (nodes_layout) {
      d.walk4_up[k] = c.d_walk4 + up_off[k];
      d.walk4_dn[k] = c.d_walk4 + dn_off[k];
    } else {
      d.walk_up[k] = c.d_cells + up_off[k];
      d.walk_dn[k] = c.d_cells + dn_off[k];
    }
  }
  CKU(cudaMemcpyAsync(c.d_desc, &d, sizeof d, cudaMemcpyHostToDevice, st));
  CKU(cudaStreamSynchronize(st));
  if (!compact && !c.alloc_stream) {
    c.d_grid = nullptr;
    CKU(cudaFree(scalar));
  }
  return BIRP_OK;
}

}  // namespace birp

namespace birp {
size_t cube_device_bytes(const birp_cube& c) {
  const size_t total = ((size_t)c.n[0] + 2) * ((size_t)c.n[1] + 2) * ((size_t)c.n[2] + 2);
  const size_t coords = (size_t)c.n[0] + c.n[1] + c.n[2];
  const bool all_uniform = c.uniform[0] && c.uniform[1] && c.uniform[2];
  size_t lut = 0;
  if (!all_uniform)
    for (int k = 0; k < 3; ++k)
      lut += (size_t)std::max(1.0, std::ceil((c.c[k].back() - c.c[k].front()) / c.min_gap[k])) * sizeof(float4);
  const size_t walk = 2 * (coords + 3) + 1;
  const size_t records = ((size_t)c.n[0] + 1) * ((size_t)c.n[1] + 1) * ((size_t)c.n[2] + 1);
  const size_t nodes_ff = (coords + 6) * sizeof(float2);
  const size_t layout_bytes =
      nodes_ff + (c.layout == BIRP_CUBE_COMPACT ? total * sizeof(float) + walk * sizeof(float4)
                  : c.layout == BIRP_CUBE_PAIRS ? total * sizeof(float2) + walk * sizeof(float4)
                                                : records * 2 * sizeof(float4) + walk * sizeof(float2));
  const size_t negflag = c.has_neg > 0 ? (size_t)c.n[0] * c.n[1] * c.n[2] : 0;
  return layout_bytes + coords * sizeof(double) + lut + sizeof(CubeDev) + negflag;
}
}  // namespace birp
