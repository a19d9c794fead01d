// Continuous-batching render server (birp_server_* in include/birp_gb300.h).
//
// Requests are admitted as they arrive. A scheduler thread forms a batch from
// the pending queue whenever a slot (a batch object with its own stream and
// CUDA graph) is free, taking requests whose source is resident. Cubes live in
// GPU memory under a byte budget; a request for a cube that is not resident
// waits while one of the uploader threads brings the cube in (evicting
// least-recently-used cubes that no in-flight batch references, re-uploading
// from the pinned host copy on that uploader's own stream, with
// stream-ordered pool allocations so neither upload nor eviction
// synchronises the device) — the other requests keep being batched
// meanwhile. With a promotion share, an idle uploader rebuilds the most
// requested cube in the faster promoted layout. Batches on different slots
// overlap on the GPU. One completion thread per slot waits for its batch,
// copies each image to the caller's buffer unless the kernels wrote it there,
// and completes the tickets.
// The reference has no counterpart: its only "many renders" path is the
// serial directory loop of src/main.cpp:242-264.
#include <algorithm>
#include <chrono>
#include <condition_variable>
#include <cstring>
#include <deque>
#include <thread>
#include <unordered_map>
#include <vector>

#include "batch.h"

using namespace birp;

namespace {

using Clock = std::chrono::steady_clock;

double ms_since(Clock::time_point t0, Clock::time_point t1) {
  return std::chrono::duration<double, std::milli>(t1 - t0).count();
}

struct Source {
  int kind = 0;  // 0 cube, 1 cmem
  std::vector<double> ax[3];
  float* h_vals = nullptr;  // pinned host copy (cubes)
  int64_t bytes = 0;        // device bytes when resident
  int has_neg = 0;          // a value below zero (the cube then carries flags)
  birp_cube* resident = nullptr;
  uint64_t last_use = 0;
  int in_use = 0;           // batches (forming or in flight) that reference it
  bool uploading = false;   // queued for or in the uploader
  birp_status upload_err = BIRP_OK;  // the last upload's failure, reported once
  birp_cmem* cmem = nullptr;
  int64_t requests = 0;       // requests submitted for it (the promotion's ranking)
  int64_t bytes_promoted = 0;  // device bytes in the promoted layout
  bool promoting = false;      // its promoted copy is being built
};

struct Req {
  int64_t ticket = 0;
  int src = 0;
  birp_camera cam{};
  float* out = nullptr;
  Clock::time_point t_submit, t_launch, t_done;
  birp_status status = BIRP_OK;
  bool done = false;
};

struct Slot {
  birp_batch* batch = nullptr;
  std::vector<Req*> reqs;
  std::vector<int> srcs;  // distinct sources pinned by this batch
  std::vector<birp_cube*> cubes;  // the device cubes its requests read
  bool busy = false;
  bool has_work = false;
  std::condition_variable cv;
  std::thread worker;
};

}  // namespace

struct birp_server {
  birp_server_config cfg{};
  std::mutex mu;
  std::condition_variable cv_sched, cv_done, cv_upload;
  std::deque<Req*> pending;
  std::deque<int> upload_q;  // sources to make resident, in request order
  std::vector<std::thread> uploaders;  // one stream each (upload_streams)
  std::unordered_map<int64_t, Req*> tickets;
  std::vector<Source> sources;
  std::vector<Slot*> slots;
  std::thread scheduler;
  bool stop = false;
  int64_t next_ticket = 1;
  uint64_t tick = 0;
  int64_t resident_bytes = 0;
  int64_t promoted_bytes = 0;  // resident cubes in the promoted layout
  // copies replaced by their promoted copy while batches in flight still
  // read them: freed when the last of those batches completes
  std::vector<std::pair<birp_cube*, int>> retired;
  std::vector<cudaStream_t> upload_streams;
  birp_server_stats st{};
};

namespace {

void finish(birp_server*, Req* r, birp_status status) {
  r->status = status;
  r->t_done = Clock::now();
  r->done = true;
}

// Frees budget for `need` more bytes by evicting least-recently-used
// resident cubes (other than source `keep`) that no batch references; called
// with the lock held. BIRP_ERR_BUSY when the budget is held by in-flight
// batches (retry later).
birp_status make_room_bytes(birp_server* s, int64_t need, int keep) {
  if (need > s->cfg.cube_budget_bytes)
    return fail(BIRP_ERR_NOMEM, "cube needs %lld B, budget is %lld B", (long long)need,
                (long long)s->cfg.cube_budget_bytes);
  while (s->resident_bytes + need > s->cfg.cube_budget_bytes) {
    int victim = -1;
    for (int i = 0; i < (int)s->sources.size(); ++i) {
      const Source& o = s->sources[i];
      if (i == keep || !o.resident || o.in_use > 0 || o.promoting) continue;
      if (victim < 0 || o.last_use < s->sources[victim].last_use) victim = i;
    }
    if (victim < 0) return BIRP_ERR_BUSY;
    Source& v = s->sources[victim];
    birp_cube* c = v.resident;
    v.resident = nullptr;
    s->resident_bytes -= (int64_t)c->device_bytes;
    if (c->layout != s->cfg.cube_layout) s->promoted_bytes -= (int64_t)c->device_bytes;
    s->st.cube_evictions++;
    destroy_cube_device(*c);  // stream-ordered release on the upload stream
    delete c;
  }
  return BIRP_OK;
}

birp_status make_room(birp_server* s, int id) { return make_room_bytes(s, s->sources[id].bytes, id); }

// A cube that batches in flight may still read is freed once the last of
// them completes (called with the lock held).
void retire_cube(birp_server* s, birp_cube* c) {
  int refs = 0;
  for (Slot* sl : s->slots)
    if (sl->busy && std::find(sl->cubes.begin(), sl->cubes.end(), c) != sl->cubes.end()) ++refs;
  if (refs == 0) {
    s->resident_bytes -= (int64_t)c->device_bytes;
    destroy_cube_device(*c);
    delete c;
  } else {
    s->retired.push_back({c, refs});
  }
}

// Promotion (promoted_budget_bytes > 0; uploader thread, lock held on entry
// and exit): the most-requested resident cube of the server's layout whose
// promoted copy fits the promotion share is rebuilt in the promoted layout
// from its host copy, with the lock released meanwhile, and takes the other
// copy's place. Returns whether it did one.
bool try_promote(birp_server* s, std::unique_lock<std::mutex>& lk, cudaStream_t stream) {
  if (s->cfg.promoted_budget_bytes <= 0) return false;
  int best = -1;
  for (int i = 0; i < (int)s->sources.size(); ++i) {
    const Source& o = s->sources[i];
    if (o.kind != 0 || !o.resident || o.resident->layout != s->cfg.cube_layout || o.uploading || o.promoting ||
        o.requests < 16 || s->promoted_bytes + o.bytes_promoted > s->cfg.promoted_budget_bytes)
      continue;
    if (best < 0 || o.requests > s->sources[best].requests) best = i;
  }
  if (best < 0) return false;
  // room for the promoted copy beside the other one until the swap
  if (make_room_bytes(s, s->sources[best].bytes_promoted, best) != BIRP_OK) return false;
  Source& src = s->sources[best];
  src.promoting = true;
  const int64_t reserved = src.bytes_promoted;
  s->resident_bytes += reserved;
  const float* vals = src.h_vals;
  const int has_neg = src.has_neg;
  std::vector<double> ax[3] = {src.ax[0], src.ax[1], src.ax[2]};
  lk.unlock();
  birp_cube* c = new birp_cube();
  c->layout = s->cfg.promoted_layout;
  c->has_neg = has_neg;
  birp_status rc = BIRP_OK;
  for (int k = 0; k < 3 && rc == BIRP_OK; ++k) rc = analyze_axis(ax[k].data(), (int)ax[k].size(), "xyz"[k], *c, k);
  if (rc == BIRP_OK) rc = upload_cube(*c, vals, stream, true);
  lk.lock();
  Source& done = s->sources[best];  // (the vector may have grown meanwhile)
  s->resident_bytes -= reserved;
  done.promoting = false;
  if (rc != BIRP_OK || !done.resident) {
    destroy_cube_device(*c);
    delete c;
    return false;
  }
  s->resident_bytes += (int64_t)c->device_bytes;
  s->promoted_bytes += (int64_t)c->device_bytes;
  done.bytes_promoted = (int64_t)c->device_bytes;
  birp_cube* old = done.resident;
  done.resident = c;  // batches formed from now on read the promoted copy
  done.bytes = (int64_t)c->device_bytes;
  retire_cube(s, old);
  s->st.cube_promotions++;
  return true;
}

// Uploader threads (`uploaders` of them, each with its own stream): each
// makes queued cubes resident one at a time, with the lock released during
// the upload itself, and wakes the scheduler; several uploads proceed at
// once.
void uploader_loop(birp_server* s, int idx) {
  cudaSetDevice(g_ctx.device);  // per host thread
  const cudaStream_t stream = s->upload_streams[idx];
  std::unique_lock<std::mutex> lk(s->mu);
  while (!s->stop) {
    if (s->upload_q.empty()) {
      // idle: promote a popular cube, else wait for work (and look again for
      // a promotion now and then)
      if (try_promote(s, lk, stream)) continue;
      if (s->cfg.promoted_budget_bytes > 0) s->cv_upload.wait_for(lk, std::chrono::milliseconds(20));
      else s->cv_upload.wait(lk);
      continue;
    }
    const int id = s->upload_q.front();
    birp_status rc = make_room(s, id);
    if (rc == BIRP_ERR_BUSY) {  // wait for a batch to finish, then retry
      s->cv_upload.wait_for(lk, std::chrono::milliseconds(1));
      continue;
    }
    s->upload_q.pop_front();
    Source& src = s->sources[id];
    if (rc == BIRP_OK) {
      birp_cube* c = new birp_cube();
      c->layout = s->cfg.cube_layout;
      c->has_neg = src.has_neg;
      const int64_t reserved = src.bytes;
      s->resident_bytes += reserved;
      const float* vals = src.h_vals;
      std::vector<double> ax[3] = {src.ax[0], src.ax[1], src.ax[2]};
      lk.unlock();
      for (int k = 0; k < 3 && rc == BIRP_OK; ++k)
        rc = analyze_axis(ax[k].data(), (int)ax[k].size(), "xyz"[k], *c, k);
      if (rc == BIRP_OK) rc = upload_cube(*c, vals, stream, true);
      lk.lock();
      Source& done = s->sources[id];  // (the vector may have grown meanwhile)
      s->resident_bytes -= reserved;
      if (rc == BIRP_OK) {
        s->resident_bytes += (int64_t)c->device_bytes;
        done.bytes = (int64_t)c->device_bytes;
        done.resident = c;
        done.last_use = ++s->tick;
        s->st.cube_uploads++;
      } else {
        destroy_cube_device(*c);
        delete c;
      }
    }
    Source& done = s->sources[id];
    done.upload_err = rc;
    done.uploading = false;
    s->cv_sched.notify_all();
  }
}

void slot_worker(birp_server* s, Slot* slot) {
  cudaSetDevice(g_ctx.device);  // per host thread
  std::unique_lock<std::mutex> lk(s->mu);
  for (;;) {
    slot->cv.wait(lk, [&] { return slot->has_work || s->stop; });
    if (!slot->has_work) return;
    lk.unlock();
    birp_status rc = batch_wait(slot->batch);
    // copy images to the callers' buffers (outside the lock) unless the
    // kernels wrote them there
    if (rc == BIRP_OK && !slot->batch->direct)
      for (size_t i = 0; i < slot->reqs.size(); ++i)
        std::memcpy(slot->reqs[i]->out, slot->batch->h_out + slot->batch->offsets[i],
                    (size_t)slot->batch->npx[i] * sizeof(float));
    lk.lock();
    for (Req* r : slot->reqs) finish(s, r, rc);
    s->st.completed += (int64_t)slot->reqs.size();
    for (int id : slot->srcs) s->sources[id].in_use--;
    // replaced cubes this batch still read: free the last reader's
    for (birp_cube* c : slot->cubes)
      for (size_t k = 0; k < s->retired.size(); ++k)
        if (s->retired[k].first == c && --s->retired[k].second == 0) {
          s->resident_bytes -= (int64_t)c->device_bytes;
          destroy_cube_device(*c);
          delete c;
          s->retired.erase(s->retired.begin() + (long)k);
          break;
        }
    slot->reqs.clear();
    slot->srcs.clear();
    slot->cubes.clear();
    slot->has_work = false;
    slot->busy = false;
    s->cv_done.notify_all();
    s->cv_sched.notify_all();
    s->cv_upload.notify_all();  // budget an uploader waits for may be free now
  }
}

void scheduler_loop(birp_server* s) {
  cudaSetDevice(g_ctx.device);  // per host thread
  std::unique_lock<std::mutex> lk(s->mu);
  const auto window = std::chrono::duration<double, std::milli>(s->cfg.max_wait_ms);
  while (!s->stop) {
    Slot* slot = nullptr;
    bool any_busy = false;
    for (Slot* sl : s->slots) {
      if (!sl->busy && !slot) slot = sl;
      any_busy |= sl->busy;
    }
    if (!slot || s->pending.empty()) {
      s->cv_sched.wait(lk);
      continue;
    }
    // batching window: while the GPU is busy, let a small batch fill up a little
    if (any_busy && (int)s->pending.size() < s->cfg.max_batch_requests) {
      auto deadline = s->pending.front()->t_submit + std::chrono::duration_cast<Clock::duration>(window);
      if (Clock::now() < deadline) {
        s->cv_sched.wait_until(lk, deadline);
        continue;
      }
    }
    // form a batch in arrival order from requests whose source is resident;
    // a request for a cube that is not resident stays pending while the
    // uploader brings the cube in
    std::vector<Req*> go;
    std::vector<int> used_srcs;
    int64_t px = 0;
    std::deque<Req*> waiting;
    std::vector<int> failed;  // sources whose upload failure this scan reports
    while (!s->pending.empty() && (int)go.size() < s->cfg.max_batch_requests) {
      Req* r = s->pending.front();
      int64_t n = (int64_t)r->cam.nx * r->cam.ny;
      if (n > s->cfg.max_batch_pixels) {  // can never fit
        s->pending.pop_front();
        fail(BIRP_ERR_INVALID, "image larger than the batch pixel limit");
        finish(s, r, BIRP_ERR_INVALID);
        s->st.completed++;
        s->cv_done.notify_all();
        continue;
      }
      Source& src = s->sources[r->src];
      if (src.kind == 0 && !src.resident) {
        s->pending.pop_front();
        if (src.upload_err != BIRP_OK) {  // the upload for it failed
          finish(s, r, src.upload_err);
          s->st.completed++;
          s->cv_done.notify_all();
          if (std::find(failed.begin(), failed.end(), r->src) == failed.end()) failed.push_back(r->src);
          continue;
        }
        if (!src.uploading) {
          src.uploading = true;
          s->upload_q.push_back(r->src);
          s->cv_upload.notify_one();
        }
        waiting.push_back(r);
        continue;
      }
      if (px + n > s->cfg.max_batch_pixels) break;
      s->pending.pop_front();
      go.push_back(r);
      px += n;
      if (std::find(used_srcs.begin(), used_srcs.end(), r->src) == used_srcs.end()) {
        used_srcs.push_back(r->src);
        src.in_use++;  // no eviction while this batch references it
        src.last_use = ++s->tick;
        if (src.kind == 0) s->st.cube_hits++;
      }
    }
    for (auto it = waiting.rbegin(); it != waiting.rend(); ++it) s->pending.push_front(*it);
    // a failure is reported to the requests pending now; later ones retry
    for (int id : failed) s->sources[id].upload_err = BIRP_OK;
    if (go.empty()) {  // every pending request waits for an upload
      s->cv_sched.wait(lk);
      continue;
    }
    slot->busy = true;
    std::vector<birp_request> reqs;
    for (Req* r : go) {
      birp_request q{};
      const Source& src = s->sources[r->src];
      q.cube = src.kind == 0 ? src.resident : nullptr;
      q.cmem = src.kind == 1 ? src.cmem : nullptr;
      q.cam = r->cam;
      reqs.push_back(q);
    }
    // where the device writes pageable host memory, the kernels write each
    // request's image straight into its caller's buffer (no copy-out)
    std::vector<float*> direct;
    if (host_direct_writes())
      for (Req* r : go) direct.push_back(r->out);
    const auto now = Clock::now();
    birp_status rc =
        batch_submit(slot->batch, reqs.data(), (int)reqs.size(), direct.empty() ? nullptr : direct.data());
    for (Req* r : go) r->t_launch = now;
    s->st.batches++;
    slot->reqs = go;
    slot->srcs = used_srcs;
    slot->cubes.clear();
    for (int id : used_srcs)
      if (s->sources[id].kind == 0) slot->cubes.push_back(s->sources[id].resident);
    if (rc != BIRP_OK) {
      for (Req* r : go) finish(s, r, rc);
      s->st.completed += (int64_t)go.size();
      for (int id : used_srcs) s->sources[id].in_use--;
      slot->reqs.clear();
      slot->srcs.clear();
      slot->cubes.clear();
      slot->busy = false;
      s->cv_done.notify_all();
      continue;
    }
    slot->has_work = true;
    slot->cv.notify_one();
  }
}

}  // namespace

extern "C" {

void birp_server_default_config(birp_server_config* c) {
  if (!c) return;
  c->cube_budget_bytes = (int64_t)60 << 30;
  c->slots = 3;
  c->max_batch_requests = 64;
  c->max_batch_pixels = (int64_t)8 << 20;
  c->max_queue = 1 << 16;
  c->max_wait_ms = 1.0;
  c->cube_layout = BIRP_CUBE_RECORDS;
  c->promoted_layout = BIRP_CUBE_RECORDS;
  c->promoted_budget_bytes = 0;
  c->uploaders = 1;
}

birp_status birp_server_create(const birp_server_config* cfg, birp_server** out) {
  if (birp_status e = check_init()) return e;
  if (!out) return fail(BIRP_ERR_INVALID, "NULL argument");
  *out = nullptr;
  birp_server_config c;
  birp_server_default_config(&c);
  if (cfg) c = *cfg;
  if (c.slots < 1 || c.slots > 16 || c.max_batch_requests < 1 || c.max_batch_pixels < 1 || c.max_queue < 1 ||
      c.cube_budget_bytes < 0 || !(c.max_wait_ms >= 0) ||
      (c.cube_layout != BIRP_CUBE_RECORDS && c.cube_layout != BIRP_CUBE_COMPACT && c.cube_layout != BIRP_CUBE_PAIRS) ||
      c.promoted_budget_bytes < 0 || c.promoted_budget_bytes > c.cube_budget_bytes || c.uploaders < 1 ||
      c.uploaders > 8 || (c.promoted_layout != BIRP_CUBE_RECORDS && c.promoted_layout != BIRP_CUBE_PAIRS) ||
      (c.promoted_budget_bytes > 0 &&
       !(c.promoted_layout == BIRP_CUBE_RECORDS ? c.cube_layout != BIRP_CUBE_RECORDS
         : c.promoted_layout == BIRP_CUBE_PAIRS  ? c.cube_layout == BIRP_CUBE_COMPACT
                                                 : false)))
    return fail(BIRP_ERR_INVALID, "bad server configuration");
  birp_server* s = new birp_server();
  s->cfg = c;
  for (int i = 0; i < c.uploaders; ++i) {
    cudaStream_t us = nullptr;
    cudaError_t e = cudaStreamCreateWithFlags(&us, cudaStreamNonBlocking);
    if (e != cudaSuccess) {
      for (cudaStream_t u : s->upload_streams) cudaStreamDestroy(u);
      delete s;
      return fail(BIRP_ERR_CUDA, "stream: %s", cudaGetErrorString(e));
    }
    s->upload_streams.push_back(us);
  }
  // keep freed cube memory in the process's pool for reuse (no release to the
  // driver between evictions); a per-process setting of this library's pool
  cudaMemPool_t pool;
  if (cudaDeviceGetDefaultMemPool(&pool, g_ctx.device) == cudaSuccess) {
    uint64_t keep = (uint64_t)c.cube_budget_bytes;
    cudaMemPoolSetAttribute(pool, cudaMemPoolAttrReleaseThreshold, &keep);
  }
  for (int i = 0; i < c.slots; ++i) {
    Slot* sl = new Slot();
    birp_status rc = batch_create(c.max_batch_requests, c.max_batch_pixels, &sl->batch);
    if (rc != BIRP_OK) {
      delete sl;
      birp_server_destroy(s);
      return rc;
    }
    s->slots.push_back(sl);
  }
  for (Slot* sl : s->slots) sl->worker = std::thread(slot_worker, s, sl);
  for (int i = 0; i < c.uploaders; ++i) s->uploaders.emplace_back(uploader_loop, s, i);
  s->scheduler = std::thread(scheduler_loop, s);
  *out = s;
  return ok();
}

birp_status birp_server_destroy(birp_server* s) {
  if (!s) return ok();
  {
    std::lock_guard<std::mutex> lk(s->mu);
    s->stop = true;
    s->cv_sched.notify_all();
    s->cv_upload.notify_all();
    for (Slot* sl : s->slots) sl->cv.notify_all();
  }
  if (s->scheduler.joinable()) s->scheduler.join();
  for (std::thread& u : s->uploaders)
    if (u.joinable()) u.join();
  for (Slot* sl : s->slots) {
    // a batch still in flight is waited for by its worker before it exits
    {
      std::unique_lock<std::mutex> lk(s->mu);
      sl->cv.notify_all();
    }
    if (sl->worker.joinable()) sl->worker.join();
    if (sl->batch) {
      batch_wait(sl->batch);
      birp_batch_destroy(sl->batch);
    }
    delete sl;
  }
  for (Req* r : s->pending) delete r;
  for (auto& kv : s->tickets)
    if (std::find(s->pending.begin(), s->pending.end(), kv.second) == s->pending.end()) delete kv.second;
  for (auto& rc : s->retired) {
    destroy_cube_device(*rc.first);
    delete rc.first;
  }
  s->retired.clear();
  for (Source& src : s->sources) {
    if (src.resident) {
      destroy_cube_device(*src.resident);
      delete src.resident;
    }
    if (src.h_vals) cudaFreeHost(src.h_vals);
    if (src.cmem) birp_cmem_destroy(src.cmem);
  }
  for (cudaStream_t u : s->upload_streams) {
    cudaStreamSynchronize(u);
    cudaStreamDestroy(u);
  }
  delete s;
  return ok();
}

birp_status birp_server_add_cube(birp_server* s, const double* xs, int nx, const double* ys, int ny,
                                 const double* zs, int nz, const float* values, int* cube_id) {
  if (!s || !cube_id || !values || !xs || !ys || !zs) return fail(BIRP_ERR_INVALID, "NULL argument");
  birp_cube probe;
  probe.layout = s->cfg.cube_layout;
  const double* axes[3] = {xs, ys, zs};
  const int n[3] = {nx, ny, nz};
  for (int k = 0; k < 3; ++k)
    if (birp_status rc = analyze_axis(axes[k], n[k], "xyz"[k], probe, k)) return rc;
  Source src;
  src.kind = 0;
  for (int k = 0; k < 3; ++k) src.ax[k].assign(axes[k], axes[k] + n[k]);
  size_t count = (size_t)nx * ny * nz;
  cudaError_t e = cudaHostAlloc(&src.h_vals, count * sizeof(float), cudaHostAllocDefault);
  if (e != cudaSuccess) return fail(BIRP_ERR_NOMEM, "pinned host copy: %s", cudaGetErrorString(e));
  std::memcpy(src.h_vals, values, count * sizeof(float));
  src.has_neg = probe.has_neg = any_negative(src.h_vals, count) ? 1 : 0;
  src.bytes = (int64_t)cube_device_bytes(probe);
  birp_cube probe_promoted = probe;
  probe_promoted.layout = s->cfg.promoted_layout;
  src.bytes_promoted = (int64_t)cube_device_bytes(probe_promoted);
  std::lock_guard<std::mutex> lk(s->mu);
  s->sources.push_back(std::move(src));
  *cube_id = (int)s->sources.size() - 1;
  return ok();
}

birp_status birp_server_add_cmem(birp_server* s, const birp_cmem_params* p, int* id) {
  if (!s || !p || !id) return fail(BIRP_ERR_INVALID, "NULL argument");
  Source src;
  src.kind = 1;
  if (birp_status rc = birp_cmem_create(p, &src.cmem)) return rc;
  std::lock_guard<std::mutex> lk(s->mu);
  s->sources.push_back(std::move(src));
  *id = (int)s->sources.size() - 1;
  return ok();
}

birp_status birp_server_submit(birp_server* s, int source_id, const birp_camera* cam, float* out_host,
                               int64_t* ticket) {
  if (!s || !cam || !out_host || !ticket) return fail(BIRP_ERR_INVALID, "NULL argument");
  if (birp_status rc = validate_camera(cam)) return rc;
  std::lock_guard<std::mutex> lk(s->mu);
  if (source_id < 0 || source_id >= (int)s->sources.size()) return fail(BIRP_ERR_INVALID, "unknown source %d", source_id);
  if ((int)s->pending.size() >= s->cfg.max_queue) {
    s->st.rejected++;
    return fail(BIRP_ERR_BUSY, "queue full (%d pending)", (int)s->pending.size());
  }
  s->sources[source_id].requests++;
  Req* r = new Req();
  r->ticket = s->next_ticket++;
  r->src = source_id;
  r->cam = *cam;
  r->out = out_host;
  r->t_submit = Clock::now();
  s->pending.push_back(r);
  s->tickets[r->ticket] = r;
  s->st.submitted++;
  *ticket = r->ticket;
  s->cv_sched.notify_all();
  return ok();
}

birp_status birp_server_wait(birp_server* s, int64_t ticket, double timeout_ms, birp_result* res) {
  if (!s) return fail(BIRP_ERR_INVALID, "NULL server");
  std::unique_lock<std::mutex> lk(s->mu);
  auto it = s->tickets.find(ticket);
  if (it == s->tickets.end()) return fail(BIRP_ERR_INVALID, "unknown ticket %lld", (long long)ticket);
  Req* r = it->second;
  if (timeout_ms < 0) {
    s->cv_done.wait(lk, [&] { return r->done; });
  } else if (!s->cv_done.wait_for(lk, std::chrono::duration<double, std::milli>(timeout_ms), [&] { return r->done; })) {
    return fail(BIRP_ERR_TIMEOUT, "ticket %lld not done after %.1f ms", (long long)ticket, timeout_ms);
  }
  if (res) {
    res->ticket = r->ticket;
    res->status = r->status;
    res->latency_ms = ms_since(r->t_submit, r->t_done);
    res->queue_ms = (r->t_launch == Clock::time_point{}) ? res->latency_ms : ms_since(r->t_submit, r->t_launch);
  }
  birp_status st = r->status;
  s->tickets.erase(it);
  delete r;
  if (st != BIRP_OK) return fail(st, "request failed (status %d)", (int)st);
  return ok();
}

birp_status birp_server_get_stats(const birp_server* s, birp_server_stats* out) {
  if (!s || !out) return fail(BIRP_ERR_INVALID, "NULL argument");
  birp_server* m = const_cast<birp_server*>(s);
  std::lock_guard<std::mutex> lk(m->mu);
  *out = m->st;
  out->resident_bytes = m->resident_bytes;
  out->promoted_bytes = m->promoted_bytes;
  return ok();
}

}  // extern "C"
