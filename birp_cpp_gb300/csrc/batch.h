// Batch object shared by the batch C ABI and the server.
#pragma once
#include <vector>

#include "birp_host.h"

struct birp_batch {
  int max_req = 0;
  int64_t max_px = 0;
  // staging block: hdr[C][4] | first[C][max+1] | order[C][max] | (16 B
  // aligned) RequestDev[max] for the C = BATCH_CLASSES kernel classes; class
  // c's tables describe its share of the requests
  size_t off_first[birp::BATCH_CLASSES] = {}, off_order[birp::BATCH_CLASSES] = {};
  size_t off_reqs = 0, stage_bytes = 0;
  char* h_stage = nullptr;   // pinned descriptors of the next launch
  char* d_stage = nullptr;
  unsigned int* d_counter = nullptr;  // work queue heads, one per kernel class
  float* d_out = nullptr;    // images of the launch, concatenated
  float* h_out = nullptr;    // pinned copy of the images
  std::vector<int64_t> offsets;
  std::vector<int64_t> npx;
  int n = 0;
  int64_t used = 0;
  int grid[birp::BATCH_CLASSES] = {};
  bool pending = false;
  bool direct = false;       // the last launch wrote the caller's host images itself
  cudaStream_t stream = nullptr;
  // capture-time streams and events of the graph's parallel branches (one
  // branch per kernel class)
  cudaStream_t branch[birp::BATCH_CLASSES] = {};
  cudaEvent_t fork = nullptr, join[birp::BATCH_CLASSES] = {};
  // {descriptors H2D, queue heads reset, then the kernels of the classes as
  // parallel branches}
  cudaGraph_t graph = nullptr;
  cudaGraphExec_t exec = nullptr;
  birp::BatchDev bd[birp::BATCH_CLASSES] = {};  // the kernels' work tables
  // the CMEM class kernel's node: its CMEM model parameter is set before a
  // launch whose CMEM requests share one model
  cudaGraphNode_t cmem_node = nullptr;
  cudaKernelNodeParams cmem_launch{};
  birp::CmemParam cmem_model{};  // the parameter the node holds now
  cudaEvent_t e_start = nullptr, e_kernel = nullptr, e_end = nullptr;
};

namespace birp {
// the persistent-kernel class (BatchClass) that renders a request
int request_class(const birp_request& r);
birp_status batch_create(int max_requests, int64_t max_pixels, birp_batch** out);
// direct_outs: when given, request i's image is written by the kernel into
// direct_outs[i] (host memory the device can write) and nothing is copied back
birp_status batch_submit(birp_batch* b, const birp_request* reqs, int n, float* const* direct_outs = nullptr);
birp_status batch_wait(birp_batch* b);
}  // namespace birp
