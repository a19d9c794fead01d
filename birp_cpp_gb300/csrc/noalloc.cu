// Batch render that allocates nothing (birp_batch_render_noalloc).
//
// Some callers cannot call cudaMalloc on their render path: code that runs
// inside another framework's custom operator, where the framework owns all
// device memory and hands over only input/output buffers; real-time loops
// that must not allocate (an allocation can synchronise the device or fail
// under a fixed memory budget). This entry point serves them: the caller
// passes the requests and its own device output buffers, and the only other
// device memory the persistent batch kernel needs (its work-queue head and
// the request table) lives in the file-scope array below, which every GPU
// that loads this library holds until the process exits.
#include <cstring>
#include <mutex>

#include "batch.h"
#include "birp_host.h"

namespace birp {
namespace {

constexpr int kNoAllocMaxRequests = 256;
// layout: hdr[4] | first[max+1] | order[max] | pad to 16 | RequestDev[max] | queue head
constexpr size_t kOffFirst = 4 * sizeof(int);
constexpr size_t kOffOrder = kOffFirst + (kNoAllocMaxRequests + 1) * sizeof(int);
constexpr size_t kOffReqs = (kOffOrder + kNoAllocMaxRequests * sizeof(int) + 15) / 16 * 16;
constexpr size_t kOffCounter = kOffReqs + kNoAllocMaxRequests * sizeof(RequestDev);
constexpr size_t kScratchBytes = (kOffCounter + sizeof(unsigned int) + 255) / 256 * 256;
static_assert(kScratchBytes <= 70000, "the array's size as the header states it (70 KB)");

// The scratch of every call. In host code this name is only a stand-in for
// the symbol: its device address comes from cudaGetSymbolAddress.
static __device__ __align__(256) unsigned char g_noalloc_scratch[kScratchBytes];

constexpr int kMaxDevices = 64;
std::mutex g_setup_mu;
unsigned char* g_scratch_addr[kMaxDevices] = {};
int g_grid[kMaxDevices][BATCH_CLASSES] = {};  // persistent grid per kernel class

// Host staging of the request table (pageable host memory; cudaMemcpyAsync
// returns once it has been read, so the lock covers only the copy).
std::mutex g_stage_mu;
alignas(16) unsigned char g_stage[kOffCounter];

// Once per device, with that device current: the device address of the
// scratch array and the persistent grid size of each kernel class.
birp_status setup_device(int dev, unsigned char** addr, const int** grid) {
  std::lock_guard<std::mutex> lk(g_setup_mu);
  if (!g_scratch_addr[dev]) {
    void* p = nullptr;
    cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
    if (e != cudaSuccess) return fail(BIRP_ERR_CUDA, "cudaGetSymbolAddress: %s", cudaGetErrorString(e));
    g_scratch_addr[dev] = static_cast<unsigned char*>(p);
    for (int c = 0; c < BATCH_CLASSES; ++c) g_grid[dev][c] = persistent_grid(c);
  }
  *addr = g_scratch_addr[dev];
  *grid = g_grid[dev];
  return BIRP_OK;
}

}  // namespace
}  // namespace birp

using namespace birp;

extern "C" birp_status birp_batch_render_noalloc(const birp_request* reqs, int n, float* const* outs_device,
                                                 void* stream) {
  if (n < 0 || (n > 0 && (!reqs || !outs_device))) return fail(BIRP_ERR_INVALID, "bad argument");
  if (n > kNoAllocMaxRequests)
    return fail(BIRP_ERR_INVALID, "%d requests exceed the no-allocation limit of %d per call", n, kNoAllocMaxRequests);
  if (n == 0) return ok();
  // the library's device, as every other entry point: a call from a thread
  // whose current device is another GPU is switched to it (the cubes' device
  // descriptors live there)
  if (birp_status s = check_init()) return s;
  const int dev = g_ctx.device;
  if (dev >= kMaxDevices) return fail(BIRP_ERR_INVALID, "device %d out of range", dev);
  cudaStream_t st = pick_stream(stream);
  // The request table is staged in one host array and copied from there: a
  // captured copy would keep reading that array at every replay, which by
  // then holds the latest call's requests, so a capturing stream is refused.
  cudaStreamCaptureStatus cap = cudaStreamCaptureStatusNone;
  cudaError_t e = cudaStreamIsCapturing(st, &cap);
  if (e != cudaSuccess) return fail(BIRP_ERR_CUDA, "cudaStreamIsCapturing: %s", cudaGetErrorString(e));
  if (cap != cudaStreamCaptureStatusNone)
    return fail(BIRP_ERR_INVALID, "the stream is capturing: this call stages its requests in host memory that the "
                                  "next call overwrites, so it cannot be recorded into a graph");
  unsigned char* scratch = nullptr;
  const int* grid = nullptr;
  if (birp_status s = setup_device(dev, &scratch, &grid)) return s;

  std::lock_guard<std::mutex> lk(g_stage_mu);
  int* hdr = reinterpret_cast<int*>(g_stage);
  int* first = reinterpret_cast<int*>(g_stage + kOffFirst);
  int* order = reinterpret_cast<int*>(g_stage + kOffOrder);
  RequestDev* rq = reinterpret_cast<RequestDev*>(g_stage + kOffReqs);
  // one launch: a trilinear-cube kernel when every request is of its class,
  // else the general kernel
  int cls = n > 0 ? request_class(reqs[0]) : BATCH_ANY;
  for (int i = 0; i < n; ++i) {
    if (!outs_device[i]) return fail(BIRP_ERR_INVALID, "output %d is NULL", i);
    if (birp_status s = build_request(reqs[i].cube, reqs[i].cmem, reqs[i].cam, outs_device[i], rq[i], true))
      return s;
    if (request_class(reqs[i]) != cls) cls = BATCH_ANY;
  }
  // largest work first (as the allocating batch path)
  for (int i = 0; i < n; ++i) order[i] = i;
  auto work = [&](int i) { return (double)reqs[i].cam.nx * reqs[i].cam.ny * reqs[i].cam.n_samples * (reqs[i].cmem ? 16.0 : 1.0); };
  for (int i = 1; i < n; ++i)  // insertion sort, stable
    for (int j = i; j > 0 && work(order[j]) > work(order[j - 1]); --j) std::swap(order[j], order[j - 1]);
  first[0] = 0;
  for (int k = 0; k < n; ++k) first[k + 1] = first[k] + rq[order[k]].tiles;
  hdr[0] = n;
  hdr[1] = first[n];
  hdr[2] = hdr[3] = 0;

  BatchDev bd;
  bd.hdr = reinterpret_cast<const int*>(scratch);
  bd.first = reinterpret_cast<const int*>(scratch + kOffFirst);
  bd.order = reinterpret_cast<const int*>(scratch + kOffOrder);
  bd.reqs = reinterpret_cast<const RequestDev*>(scratch + kOffReqs);
  bd.counter = reinterpret_cast<unsigned int*>(scratch + kOffCounter);
  bd.stats = nullptr;
  // the queue head must start at zero; the table is overwritten whole
  if ((e = cudaMemsetAsync(scratch + kOffCounter, 0, sizeof(unsigned int), st)) != cudaSuccess ||
      (e = cudaMemcpyAsync(scratch, g_stage, kOffReqs + (size_t)n * sizeof(RequestDev), cudaMemcpyHostToDevice,
                           st)) != cudaSuccess ||
      (e = launch_render_batch(bd, grid[cls], st, cls)) != cudaSuccess)
    return fail(BIRP_ERR_CUDA, "no-allocation batch: %s", cudaGetErrorString(e));
  return ok();
}
