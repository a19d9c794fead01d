// Batched renders: many requests in one launch of the persistent kernel,
// replayed from a CUDA graph (staging copy of the descriptors, queue-head
// reset, kernel). Replaces the reference's one-render-per-cube loop
// (src/main.cpp:242-264).
#include <algorithm>
#include <cstring>
#include <vector>

#include "batch.h"

using namespace birp;

#define CKB(x)                                                                                 \
  do {                                                                                         \
    cudaError_t e_ = (x);                                                                      \
    if (e_ != cudaSuccess)                                                                     \
      return fail(e_ == cudaErrorMemoryAllocation ? BIRP_ERR_NOMEM : BIRP_ERR_CUDA, "%s: %s", #x, \
                  cudaGetErrorString(e_));                                                     \
  } while (0)

namespace birp {

static size_t align_up(size_t x, size_t a) { return (x + a - 1) / a * a; }

int request_class(const birp_request& r) {
  if (r.cmem) return BATCH_CMEM;
  if (!r.cam.trilinear) return BATCH_CUBE_NEAREST;
  if (r.cube && r.cube->has_neg > 0) return BATCH_CUBE_SIGNED;
  if (r.cube && r.cube->layout == BIRP_CUBE_COMPACT) return BATCH_CUBE_TRI_COMPACT;
  if (r.cube && r.cube->layout == BIRP_CUBE_PAIRS) return BATCH_CUBE_TRI_PAIRS;
  return BATCH_CUBE_TRI;
}

static void free_batch(birp_batch* b) {
  if (!b) return;
  if (b->stream) cudaStreamSynchronize(b->stream);
  if (b->exec) cudaGraphExecDestroy(b->exec);
  if (b->graph) cudaGraphDestroy(b->graph);
  if (b->h_stage) cudaFreeHost(b->h_stage);
  if (b->h_out) cudaFreeHost(b->h_out);
  if (b->d_stage) cudaFree(b->d_stage);
  if (b->d_out) cudaFree(b->d_out);
  if (b->d_counter) cudaFree(b->d_counter);
  for (cudaEvent_t e : {b->e_start, b->e_kernel, b->e_end, b->fork})
    if (e) cudaEventDestroy(e);
  for (int c = 0; c < BATCH_CLASSES; ++c) {
    if (b->join[c]) cudaEventDestroy(b->join[c]);
    if (b->branch[c]) cudaStreamDestroy(b->branch[c]);
  }
  if (b->stream) cudaStreamDestroy(b->stream);
  delete b;
}

birp_status batch_create(int max_requests, int64_t max_pixels, birp_batch** out) {
  if (birp_status s = check_init()) return s;
  if (!out || max_requests < 1 || max_pixels < 1 || max_requests > (1 << 20))
    return fail(BIRP_ERR_INVALID, "bad batch limits");
  *out = nullptr;
  birp_batch* b = new birp_batch();
  b->max_req = max_requests;
  b->max_px = max_pixels;
  // staging block: hdr[C][4] | first[C][max+1] | order[C][max] | (16B aligned) RequestDev[max]
  size_t off = 4 * BATCH_CLASSES * sizeof(int);
  for (int c = 0; c < BATCH_CLASSES; ++c) {
    b->off_first[c] = off;
    off += (size_t)(max_requests + 1) * sizeof(int);
  }
  for (int c = 0; c < BATCH_CLASSES; ++c) {
    b->off_order[c] = off;
    off += (size_t)max_requests * sizeof(int);
  }
  b->off_reqs = align_up(off, 16);
  b->stage_bytes = b->off_reqs + (size_t)max_requests * sizeof(RequestDev);
  auto bail = [&](birp_status s) {
    free_batch(b);
    return s;
  };
  cudaError_t e;
  if ((e = cudaStreamCreateWithFlags(&b->stream, cudaStreamNonBlocking)) != cudaSuccess ||
      (e = cudaHostAlloc(&b->h_stage, b->stage_bytes, cudaHostAllocDefault)) != cudaSuccess ||
      (e = cudaMalloc(&b->d_stage, b->stage_bytes)) != cudaSuccess ||
      (e = cudaMalloc(&b->d_counter, BATCH_CLASSES * sizeof(unsigned int))) != cudaSuccess ||
      (e = cudaMalloc(&b->d_out, (size_t)max_pixels * sizeof(float))) != cudaSuccess ||
      (e = cudaHostAlloc(&b->h_out, (size_t)max_pixels * sizeof(float), cudaHostAllocDefault)) != cudaSuccess ||
      (e = cudaEventCreate(&b->e_start)) != cudaSuccess || (e = cudaEventCreate(&b->e_kernel)) != cudaSuccess ||
      (e = cudaEventCreate(&b->e_end)) != cudaSuccess ||
      (e = cudaEventCreateWithFlags(&b->fork, cudaEventDisableTiming)) != cudaSuccess)
    return bail(fail(e == cudaErrorMemoryAllocation ? BIRP_ERR_NOMEM : BIRP_ERR_CUDA, "batch allocation: %s",
                     cudaGetErrorString(e)));
  for (int c = 0; c < BATCH_CLASSES; ++c)
    if ((e = cudaStreamCreateWithFlags(&b->branch[c], cudaStreamNonBlocking)) != cudaSuccess ||
        (e = cudaEventCreateWithFlags(&b->join[c], cudaEventDisableTiming)) != cudaSuccess)
      return bail(fail(BIRP_ERR_CUDA, "batch streams: %s", cudaGetErrorString(e)));
  std::memset(b->h_stage, 0, b->stage_bytes);

  // One graph: descriptors H2D, the queue heads reset, then the kernels of
  // the six classes as parallel branches: CMEM (few but heavy requests),
  // trilinear cubes holding negative values, nearest mode, and the three
  // trilinear-cube kernels (compact, pairs and records layout). Each is a
  // persistent kernel sized to fill the GPU on its own;
  // launched side by side, the CTAs of one class take the SM slots that
  // another class's CTAs leave when its queue runs dry, so the classes of a
  // mixed batch overlap instead of each paying its tail in turn, and a class
  // with no requests (its CTAs exit at once) costs no serial launch gap.
  // Every request falls in one of these classes, so the general kernel is not
  // launched.
  BatchDev* bd = b->bd;
  for (int c = 0; c < BATCH_CLASSES; ++c) {
    bd[c].hdr = reinterpret_cast<const int*>(b->d_stage) + 4 * c;
    bd[c].first = reinterpret_cast<const int*>(b->d_stage + b->off_first[c]);
    bd[c].order = reinterpret_cast<const int*>(b->d_stage + b->off_order[c]);
    bd[c].reqs = reinterpret_cast<const RequestDev*>(b->d_stage + b->off_reqs);
    bd[c].counter = b->d_counter + c;
    bd[c].stats = g_ctx.stats;
    b->grid[c] = persistent_grid(c);
  }
  if ((e = cudaStreamBeginCapture(b->stream, cudaStreamCaptureModeThreadLocal)) != cudaSuccess)
    return bail(fail(BIRP_ERR_CUDA, "capture: %s", cudaGetErrorString(e)));
  cudaMemcpyAsync(b->d_stage, b->h_stage, b->stage_bytes, cudaMemcpyHostToDevice, b->stream);
  cudaMemsetAsync(b->d_counter, 0, BATCH_CLASSES * sizeof(unsigned int), b->stream);
  cudaEventRecord(b->fork, b->stream);
  for (int c : {BATCH_CMEM, BATCH_CUBE_SIGNED, BATCH_CUBE_NEAREST, BATCH_CUBE_TRI_COMPACT, BATCH_CUBE_TRI_PAIRS,
                BATCH_CUBE_TRI}) {
    cudaStreamWaitEvent(b->branch[c], b->fork, 0);
    launch_render_batch(bd[c], b->grid[c], b->branch[c], c);
    cudaEventRecord(b->join[c], b->branch[c]);
    cudaStreamWaitEvent(b->stream, b->join[c], 0);
  }
  e = cudaStreamEndCapture(b->stream, &b->graph);
  if (e != cudaSuccess) return bail(fail(BIRP_ERR_CUDA, "capture: %s", cudaGetErrorString(e)));
  if ((e = cudaGraphInstantiate(&b->exec, b->graph, 0)) != cudaSuccess)
    return bail(fail(BIRP_ERR_CUDA, "graph instantiate: %s", cudaGetErrorString(e)));
  // the CMEM kernel's node, whose model parameter each launch may set
  size_t n_nodes = 0;
  if ((e = cudaGraphGetNodes(b->graph, nullptr, &n_nodes)) != cudaSuccess)
    return bail(fail(BIRP_ERR_CUDA, "graph nodes: %s", cudaGetErrorString(e)));
  std::vector<cudaGraphNode_t> nodes(n_nodes);
  if ((e = cudaGraphGetNodes(b->graph, nodes.data(), &n_nodes)) != cudaSuccess)
    return bail(fail(BIRP_ERR_CUDA, "graph nodes: %s", cudaGetErrorString(e)));
  for (cudaGraphNode_t nd : nodes) {
    cudaGraphNodeType t;
    cudaKernelNodeParams kp{};
    if (cudaGraphNodeGetType(nd, &t) == cudaSuccess && t == cudaGraphNodeTypeKernel &&
        cudaGraphKernelNodeGetParams(nd, &kp) == cudaSuccess && kp.func == render_batch_function(BATCH_CMEM)) {
      b->cmem_node = nd;
      b->cmem_launch = kp;
    }
  }
  if (!b->cmem_node) return bail(fail(BIRP_ERR_CUDA, "batch graph without its CMEM kernel node"));
  *out = b;
  return ok();
}

birp_status batch_submit(birp_batch* b, const birp_request* reqs, int n, float* const* direct_outs) {
  if (birp_status s = check_init()) return s;
  if (!b || n < 0 || (n > 0 && !reqs)) return fail(BIRP_ERR_INVALID, "bad argument");
  if (n > b->max_req) return fail(BIRP_ERR_INVALID, "%d requests exceed the batch limit %d", n, b->max_req);
  if (b->pending)
    if (birp_status s = batch_wait(b)) return s;
  int* hdr = reinterpret_cast<int*>(b->h_stage);
  RequestDev* rq = reinterpret_cast<RequestDev*>(b->h_stage + b->off_reqs);
  b->offsets.assign(n, 0);
  b->npx.assign(n, 0);
  int64_t used = 0;
  std::vector<double> work(n);
  std::vector<int> members[BATCH_CLASSES];
  for (int i = 0; i < n; ++i) {
    const birp_camera& c = reqs[i].cam;
    if (birp_status s = validate_camera(&c)) return s;
    int64_t npx = (int64_t)c.nx * c.ny;
    if (used + npx > b->max_px)
      return fail(BIRP_ERR_INVALID, "batch images need more than %lld pixels", (long long)b->max_px);
    b->offsets[i] = used;
    b->npx[i] = npx;
    float* out = direct_outs ? direct_outs[i] : b->d_out + used;
    if (birp_status s = build_request(reqs[i].cube, reqs[i].cmem, c, out, rq[i], true)) return s;
    used += npx;
    work[i] = (double)npx * c.n_samples * (reqs[i].cmem ? 16.0 : 1.0);
    members[request_class(reqs[i])].push_back(i);
  }
  // per class: largest work first, so long renders start early and small
  // ones fill the tail
  for (int cls = 0; cls < BATCH_CLASSES; ++cls) {
    int* first = reinterpret_cast<int*>(b->h_stage + b->off_first[cls]);
    int* order = reinterpret_cast<int*>(b->h_stage + b->off_order[cls]);
    std::vector<int>& m = members[cls];
    std::stable_sort(m.begin(), m.end(), [&](int x, int y) { return work[x] > work[y]; });
    const int k = (int)m.size();
    first[0] = 0;
    for (int j = 0; j < k; ++j) {
      order[j] = m[j];
      first[j + 1] = first[j] + rq[m[j]].tiles;
    }
    hdr[4 * cls] = k;
    hdr[4 * cls + 1] = first[k];
  }
  // one CMEM model for every CMEM request: the CMEM kernel gets it as a
  // parameter (its constants become operands instead of loads)
  const birp_cmem* model = nullptr;
  bool one_model = true;
  for (int i = 0; i < n; ++i)
    if (reqs[i].cmem) {
      if (!model) model = reqs[i].cmem;
      else if (reqs[i].cmem != model) one_model = false;
    }
  CmemParam cp{};
  if (model && one_model) {
    cp.m = model->h_desc;
    cp.dev = model->d_desc;
  }
  if (std::memcmp(&cp, &b->cmem_model, sizeof cp) != 0) {
    cudaKernelNodeParams kp = b->cmem_launch;
    void* args[2] = {&b->bd[BATCH_CMEM], &cp};
    kp.kernelParams = args;
    kp.extra = nullptr;
    cudaError_t e = cudaGraphExecKernelNodeSetParams(b->exec, b->cmem_node, &kp);
    if (e != cudaSuccess) return fail(BIRP_ERR_CUDA, "CMEM model parameter: %s", cudaGetErrorString(e));
    b->cmem_model = cp;
  }
  b->n = n;
  b->used = used;
  b->direct = direct_outs != nullptr;
  if (b->direct) {
    std::vector<size_t> cnt(b->npx.begin(), b->npx.end());
    prefault_outputs(direct_outs, cnt.data(), n);
  }
  cudaError_t e;
  if ((e = cudaEventRecord(b->e_start, b->stream)) != cudaSuccess ||
      (e = cudaGraphLaunch(b->exec, b->stream)) != cudaSuccess ||
      (e = cudaEventRecord(b->e_kernel, b->stream)) != cudaSuccess ||
      (used > 0 && !b->direct &&
       (e = cudaMemcpyAsync(b->h_out, b->d_out, (size_t)used * sizeof(float), cudaMemcpyDeviceToHost,
                            b->stream)) != cudaSuccess) ||
      (e = cudaEventRecord(b->e_end, b->stream)) != cudaSuccess)
    return fail(BIRP_ERR_CUDA, "batch launch: %s", cudaGetErrorString(e));
  b->pending = true;
  return ok();
}

birp_status batch_wait(birp_batch* b) {
  if (!b) return fail(BIRP_ERR_INVALID, "NULL batch");
  if (!b->pending) return ok();
  cudaError_t e = cudaEventSynchronize(b->e_end);
  b->pending = false;
  if (e != cudaSuccess) return fail(BIRP_ERR_CUDA, "batch: %s", cudaGetErrorString(e));
  return ok();
}

}  // namespace birp

extern "C" {

birp_status birp_batch_create(int max_requests, int64_t max_pixels, birp_batch** out) {
  return batch_create(max_requests, max_pixels, out);
}

birp_status birp_batch_destroy(birp_batch* b) {
  free_batch(b);
  return ok();
}

birp_status birp_batch_submit(birp_batch* b, const birp_request* reqs, int n) { return batch_submit(b, reqs, n); }

birp_status birp_batch_wait(birp_batch* b) { return batch_wait(b); }

const float* birp_batch_image(const birp_batch* b, int i) {
  if (!b || i < 0 || i >= b->n || b->pending || b->direct) return nullptr;
  return b->h_out + b->offsets[i];
}

birp_status birp_batch_render(birp_batch* b, const birp_request* reqs, int n, float* const* outs) {
  if (n > 0 && !outs) return fail(BIRP_ERR_INVALID, "outs is NULL");
  bool direct = host_direct_writes() && n > 0;
  for (int i = 0; i < n && direct; ++i) direct = outs[i] != nullptr;
  if (direct) {
    // the kernel writes each image straight into the caller's buffer
    if (birp_status s = batch_submit(b, reqs, n, outs)) return s;
    return batch_wait(b);
  }
  if (birp_status s = batch_submit(b, reqs, n)) return s;
  if (birp_status s = batch_wait(b)) return s;
  std::vector<const float*> src(n);
  std::vector<size_t> cnt(n);
  for (int i = 0; i < n; ++i) {
    src[i] = b->h_out + b->offsets[i];
    cnt[i] = (size_t)b->npx[i];
  }
  parallel_copy(outs, src.data(), cnt.data(), n);
  return ok();
}

birp_status birp_batch_upload_bytes(const birp_batch* b, size_t* bytes) {
  if (!b || !bytes) return fail(BIRP_ERR_INVALID, "NULL argument");
  *bytes = b->stage_bytes;  // the one host -> device copy of the graph
  return ok();
}

birp_status birp_batch_last_ms(const birp_batch* b, float* kernel_ms, float* total_ms) {
  if (!b || b->pending) return fail(BIRP_ERR_INVALID, "no finished launch");
  float k = 0, t = 0;
  CKB(cudaEventElapsedTime(&k, b->e_start, b->e_kernel));
  CKB(cudaEventElapsedTime(&t, b->e_start, b->e_end));
  if (kernel_ms) *kernel_ms = k;
  if (total_ms) *total_ms = t;
  return ok();
}

}  // extern "C"
