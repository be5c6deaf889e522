// Serving loop: continuous batching of render jobs and ray queries on one GPU.
//
// One scheduler thread owns the device work. Each turn it
//   1. admits pending requests in arrival order while the HBM budget and the
//      shared queue capacity allow (render: its accumulation buffer and its
//      pixels of the queues; query: its ray and result buffers); a query may
//      pass a render job that waits only for queue space;
//   2. starts admitted queries on the query stream (copy in, trace, copy out);
//   3. runs one batched iteration of all admitted render jobs (up to k samples
//      each, the ct_batch kernels with a job table built for this iteration),
//      alternating between two render streams with a queue set each, so one
//      iteration's last, nearly empty bounces overlap the next iteration's
//      first passes; an iteration is issued once its stream's previous one has
//      finished (at most two in flight), and the thread never blocks on one, so
//      queries that arrive meanwhile start at once on their own stream, which
//      runs at the device's highest priority;
//   4. retires requests whose completion events have fired, freeing their
//      device state and waking waiters.
// Jobs arriving while others are on the GPU join at the next iteration; a
// job's samples, seeds and per-pixel accumulation order do not depend on the
// other jobs, so its result equals the job rendered alone. A job takes up to
// k = min(spp, I / pixels) samples per iteration, I = min(iter_pixels,
// max_inflight_pixels), at least one, and has min(spp, S k) slot buffers, S =
// kStreams: sample i goes to slot i mod S k, so S consecutive iterations (on
// the S streams) write disjoint slots and the next one, on the same stream as
// the first, is ordered after it. The slots are added in slot order when the job
// finishes. Each slot sums its samples in sample order however the
// iterations fall, and k depends only on the job and the configuration.
#include <cuda_runtime.h>

#include <algorithm>
#include <chrono>
#include <condition_variable>
#include <cstring>
#include <deque>
#include <mutex>
#include <thread>
#include <unordered_map>
#include <vector>

#include "../../include/cudatracer.h"
#include "ct_internal.h"

using namespace ct;

namespace {

constexpr uint32_t kIterPixels = 1u << 22;  // default pixel-samples a job may take per iteration
// Render streams, each with a queue set and a job table (measured at 100 and
// 400 requests/s: 4 streams gave the same tails as 2 within noise, for two more
// queue sets).
constexpr int kStreams = 2;

enum Kind { kRender = 0, kClosest = 1, kAny = 2 };
enum State { kPending, kActive, kFinishing, kDone };

struct Request {
  uint64_t id = 0;
  Kind kind = kRender;
  State state = kPending;
  ct_status status = CT_OK;
  // render
  ct_batch_job job{};
  float* host_out = nullptr;
  uint32_t done_spp = 0;
  uint32_t k = 1;      // samples per iteration
  uint32_t slots = 1;  // slot buffers: min(spp, kStreams * k)
  int64_t last_iter = -2;  // the last iteration that took samples of this job
  cudaEvent_t ready = nullptr;  // its slot buffers are zeroed
  uint32_t waited = 0;          // render streams already ordered after `ready` (bit per stream)
  // query
  const ct_bvh* bvh = nullptr;
  const float* horg = nullptr;
  const float* hdir = nullptr;
  uint32_t n = 0;
  float tri_eps = 1e-3f;
  int32_t* hhit = nullptr;
  float* ht = nullptr;
  uint8_t* hocc = nullptr;
  // device state
  void* dmem = nullptr;
  size_t bytes = 0;
  uint32_t pixels = 0;
  cudaEvent_t ev = nullptr;
  double t_submit = 0, t_admit = 0, t_done = 0;
};

size_t request_bytes(const Request& r) {
  if (r.kind == kRender) return (size_t)r.slots * r.pixels * sizeof(float4);
  // org + dir + hit/occluded + t + counters (+ settlement records on a wide BVH), each 256-byte aligned
  auto al = [](size_t b) { return (b + 255) & ~(size_t)255; };
  return al((size_t)r.n * 16) * 2 + al((size_t)r.n * 4) * 2 + 256 +
         (rt_bvh_wide(r.bvh) ? al((size_t)r.n * kWideRecordBytes) : 0);
}

}  // namespace

struct ct_server {
  ct_ctx* ctx = nullptr;
  ct_server_config cfg{};
  int device = 0;
  std::thread th;
  std::mutex mu;
  std::condition_variable cv;       // work for the scheduler
  std::condition_variable done_cv;  // completions for waiters
  bool stop = false;
  uint64_t next_id = 1;
  std::deque<Request*> pending;                // guarded by mu
  std::unordered_map<uint64_t, Request*> all;  // guarded by mu
  ct_server_stats stats{};                     // guarded by mu
  // scheduler-thread state
  std::vector<Request*> render;     // admitted render jobs
  std::vector<Request*> finishing;  // waiting for their completion event
  size_t used_bytes = 0;
  uint32_t inflight_pixels = 0;
  std::chrono::steady_clock::time_point t0;
  DevQueues q[kStreams] = {};  // one queue set per render stream
  std::vector<std::pair<void*, size_t>> q_owned[kStreams];
  int32_t max_stack = 1;
  BatchJob* d_table[kStreams] = {};
  int32_t* d_bases[kStreams] = {};
  BatchJob* h_table[kStreams] = {};  // pinned staging
  int32_t* h_bases[kStreams] = {};
  uint32_t table_cap = 0;
  cudaEvent_t table_ev[kStreams] = {};
  int slot = 0;          // render stream, queue set and job table of the next iteration
  int64_t iter = 0;      // iterations issued
  cudaStream_t rs[kStreams] = {}, qs = nullptr, ms = nullptr;  // render, query, setup
  // the server's own memory pool for request state: freed request memory stays
  // reserved in it between requests (release threshold at its maximum) without
  // changing the device's default pool, which the host application may use
  cudaMemPool_t pool = nullptr;

  double now() const { return std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count(); }
  void loop();
  void start(Request* r);
  void start_query(Request* r);
  cudaError_t render_iteration(std::vector<Request*>& finished);
  void retire_locked();
  void free_tables();
};

// Device state of an admitted request: stream-ordered allocation on the stream
// that uses it, so freeing never waits for the whole device.
void ct_server::start(Request* r) {
  cudaStream_t st = r->kind == kRender ? ms : qs;
  cudaError_t e = cudaMallocFromPoolAsync(&r->dmem, r->bytes, pool, st);
  if (e != cudaSuccess) {
    cudaGetLastError();
    r->dmem = nullptr;
    r->status = CT_ERR_OUT_OF_MEMORY;
    return;
  }
  if (cudaEventCreateWithFlags(&r->ev, cudaEventDisableTiming) != cudaSuccess) {
    r->status = CT_ERR_CUDA;
    cudaFreeAsync(r->dmem, st);
    r->dmem = nullptr;
    return;
  }
  if (r->kind == kRender) {
    // zeroed on the setup stream; each render stream waits for `ready` before its first use
    if (cudaMemsetAsync(r->dmem, 0, r->bytes, ms) != cudaSuccess ||
        cudaEventCreateWithFlags(&r->ready, cudaEventDisableTiming) != cudaSuccess ||
        cudaEventRecord(r->ready, ms) != cudaSuccess) {
      cudaGetLastError();
      r->status = CT_ERR_CUDA;
      cudaFreeAsync(r->dmem, ms);
      r->dmem = nullptr;
    }
  } else {
    start_query(r);
  }
}

void ct_server::start_query(Request* r) {
  auto al = [](size_t b) { return (b + 255) & ~(size_t)255; };
  char* m = (char*)r->dmem;
  float4* org = (float4*)m;
  float4* dir = (float4*)(m + al((size_t)r->n * 16));
  int32_t* hit = (int32_t*)(m + 2 * al((size_t)r->n * 16));
  float* t = (float*)(m + 2 * al((size_t)r->n * 16) + al((size_t)r->n * 4));
  int* cursor = (int*)(m + 2 * al((size_t)r->n * 16) + 2 * al((size_t)r->n * 4));
  void* recs = m + 2 * al((size_t)r->n * 16) + 2 * al((size_t)r->n * 4) + 256;
  cudaError_t e = cudaMemcpyAsync(org, r->horg, (size_t)r->n * 16, cudaMemcpyHostToDevice, qs);
  if (e == cudaSuccess) e = cudaMemcpyAsync(dir, r->hdir, (size_t)r->n * 16, cudaMemcpyHostToDevice, qs);
  if (e == cudaSuccess) {
    uint32_t* err = rt_ctx_error(ctx);
    if (rt_bvh_wide(r->bvh)) {
      e = r->kind == kClosest
              ? launch_trace_wide_closest(rt_bvh_wdev(r->bvh), org, dir, hit, t, r->n, err, cursor, recs, nullptr, qs)
              : launch_trace_wide_any(rt_bvh_wdev(r->bvh), org, dir, (uint8_t*)hit, r->n, err, cursor, recs, nullptr,
                                      qs);
    } else {
      e = r->kind == kClosest
              ? launch_trace_closest(rt_bvh_dev(r->bvh), org, dir, hit, t, r->n, r->tri_eps, err, cursor, qs)
              : launch_trace_any(rt_bvh_dev(r->bvh), org, dir, (uint8_t*)hit, r->n, r->tri_eps, err, cursor, qs);
    }
  }
  if (e == cudaSuccess) {
    if (r->kind == kClosest) {
      e = cudaMemcpyAsync(r->hhit, hit, (size_t)r->n * 4, cudaMemcpyDeviceToHost, qs);
      if (e == cudaSuccess) e = cudaMemcpyAsync(r->ht, t, (size_t)r->n * 4, cudaMemcpyDeviceToHost, qs);
    } else {
      e = cudaMemcpyAsync(r->hocc, hit, (size_t)r->n, cudaMemcpyDeviceToHost, qs);
    }
  }
  const cudaError_t fe = cudaFreeAsync(r->dmem, qs);  // after the copies, in stream order
  r->dmem = nullptr;
  if (e == cudaSuccess) e = fe;
  if (e == cudaSuccess) e = cudaEventRecord(r->ev, qs);
  if (e != cudaSuccess) {
    cudaGetLastError();
    r->status = CT_ERR_CUDA;
  }
}

void ct_server::free_tables() {
  for (int k = 0; k < kStreams; k++) {
    if (d_table[k]) rt_free(ctx, d_table[k], (size_t)table_cap * sizeof(BatchJob));
    if (d_bases[k]) rt_free(ctx, d_bases[k], (size_t)(table_cap + 1) * 4);
    if (h_table[k]) cudaFreeHost(h_table[k]);
    if (h_bases[k]) cudaFreeHost(h_bases[k]);
    d_table[k] = nullptr, d_bases[k] = nullptr, h_table[k] = nullptr, h_bases[k] = nullptr;
  }
  table_cap = 0;
}

// Up to k samples of every admitted render job. `finished` receives the jobs that
// took their last one (their images are being copied out).
cudaError_t ct_server::render_iteration(std::vector<Request*>& finished) {
  // one table entry per (job, sample) taken this iteration
  uint32_t n = 0;
  for (Request* r : render) n += std::min(r->k, r->job.spp - r->done_spp);
  // the table slot is free once the iteration that used it has finished
  cudaError_t e = cudaEventSynchronize(table_ev[slot]);
  if (e != cudaSuccess) return e;
  if (n > table_cap) {
    for (int k = 0; k < kStreams; k++)  // the other tables may be in use
      if ((e = cudaStreamSynchronize(rs[k])) != cudaSuccess) return e;
    free_tables();
    const uint32_t cap = std::max<uint32_t>(64, n * 2);
    for (int k = 0; k < kStreams; k++) {
      if (rt_alloc(ctx, (size_t)cap * sizeof(BatchJob), (void**)&d_table[k]) != CT_OK ||
          rt_alloc(ctx, (size_t)(cap + 1) * 4, (void**)&d_bases[k]) != CT_OK)
        return cudaErrorMemoryAllocation;
      if ((e = cudaMallocHost((void**)&h_table[k], (size_t)cap * sizeof(BatchJob))) != cudaSuccess) return e;
      if ((e = cudaMallocHost((void**)&h_bases[k], (size_t)(cap + 1) * 4)) != cudaSuccess) return e;
    }
    table_cap = cap;
  }
  cudaStream_t st = rs[slot];
  const DevQueues& q = this->q[slot];
  BatchJob* ht = h_table[slot];
  int32_t* hb = h_bases[slot];
  int32_t base = 0, depth = 1;
  uint32_t j = 0;
  for (Request* r : render) {
    const uint32_t m = std::min(r->k, r->job.spp - r->done_spp);
    if (!(r->waited & (1u << slot))) {  // each stream's first use waits for the zero fill
      if ((e = cudaStreamWaitEvent(st, r->ready, 0)) != cudaSuccess) return e;
      r->waited |= 1u << slot;
    }
    BatchJob J;
    std::memset(&J, 0, sizeof(J));
    J.sc = rt_scene_dev(r->job.scene);
    J.bvh = rt_bvh_dev(r->job.bvh);
    J.f = rt_frame_const(&r->job.camera, &r->job.params);
    J.max_depth = r->job.params.max_depth;
    J.spp_left = 1;
    J.exact = cfg.exact_math;
    for (uint32_t s = 0; s < m; s++, j++) {
      const uint32_t i = r->done_spp + s;  // sample index
      ht[j] = J;
      ht[j].f.frame = r->job.params.frame_index + 2u * i;
      ht[j].accum = (float4*)r->dmem + (size_t)(i % r->slots) * r->pixels;
      ht[j].pix_base = base;
      hb[j] = base;
      base += (int32_t)r->pixels;
    }
    depth = std::max(depth, r->job.params.max_depth);
    max_stack = std::max(max_stack, J.bvh.stack_entries);
    r->done_spp += m;
  }
  const int64_t this_iter = iter++;
  hb[n] = base;
  if ((e = cudaMemcpyAsync(d_table[slot], ht, (size_t)n * sizeof(BatchJob), cudaMemcpyHostToDevice, st)) != cudaSuccess)
    return e;
  if ((e = cudaMemcpyAsync(d_bases[slot], hb, (size_t)(n + 1) * 4, cudaMemcpyHostToDevice, st)) != cudaSuccess) return e;
  if ((e = cudaMemsetAsync(q.counts, 0, 16 * sizeof(int32_t), st)) != cudaSuccess) return e;
  DevBatch b{d_table[slot], d_bases[slot], (int32_t)n, base, max_stack, 0, 2};  // quad BVHs
  const bool fast = math_fast_traversal(cfg.exact_math);
  const int exact_shade = math_exact_shading(cfg.exact_math);
  e = launch_batch_raygen(b, q, exact_shade, st);
  for (int pass = 0; pass < depth && e == cudaSuccess; pass++) {
    const int cur = pass & 1;
    const uint32_t path_length = pass == 0 ? 0u : (uint32_t)pass + 1u;  // Kernel.cu:306, 330
    e = launch_batch_extend(b, q, cur, fast, 128, 24, st);
    if (e == cudaSuccess) e = launch_batch_shade(b, q, cur, path_length, pass, exact_shade, 1, st);
    if (e == cudaSuccess) e = launch_batch_connect(b, q, fast, 128, st);
  }
  if (e == cudaSuccess) e = cudaEventRecord(table_ev[slot], st);
  slot = (slot + 1) % kStreams;
  std::vector<Request*> keep;
  for (Request* r : render) {
    const int64_t prev = r->last_iter;
    r->last_iter = this_iter;
    if (r->done_spp < r->job.spp) {
      keep.push_back(r);
      continue;
    }
    // samples of earlier iterations may still run on the other streams: wait for
    // their latest iterations (a job that took all its samples in this one skips it)
    if (prev >= 0)
      for (int k = 0; k < kStreams && e == cudaSuccess; k++)
        if (rs[k] != st) e = cudaStreamWaitEvent(st, table_ev[k], 0);
    // add the slot buffers in slot order, copy the image out, free in stream order
    float4* acc = (float4*)r->dmem;
    for (uint32_t s = 1; s < r->slots && e == cudaSuccess; s++)
      e = launch_fold(acc, acc + (size_t)s * r->pixels, (int)r->pixels, st);
    if (e == cudaSuccess)
      e = cudaMemcpyAsync(r->host_out, r->dmem, (size_t)r->pixels * sizeof(float4), cudaMemcpyDeviceToHost, st);
    if (e == cudaSuccess) e = cudaFreeAsync(r->dmem, st);
    if (e == cudaSuccess) e = cudaEventRecord(r->ev, st);
    inflight_pixels -= r->k * r->pixels;  // its queue space frees with this iteration's set
    finished.push_back(r);
  }
  render.swap(keep);
  return e;
}

void ct_server::retire_locked() {
  std::vector<Request*> keep;
  bool any = false;
  for (Request* r : finishing) {
    const cudaError_t qr = r->ev ? cudaEventQuery(r->ev) : cudaSuccess;
    if (qr == cudaErrorNotReady) {
      keep.push_back(r);
      continue;
    }
    if (qr != cudaSuccess && r->status == CT_OK) r->status = CT_ERR_CUDA;
    if (r->t_admit > 0 || r->bytes) {
      used_bytes -= r->bytes;
      rt_account(ctx, -(int64_t)r->bytes);
    }
    r->dmem = nullptr;
    if (r->ev) cudaEventDestroy(r->ev), r->ev = nullptr;
    if (r->ready) cudaEventDestroy(r->ready), r->ready = nullptr;
    r->t_done = now();
    r->state = kDone;
    if (r->status == CT_OK) stats.completed++;
    else stats.failed++;
    any = true;
  }
  finishing.swap(keep);
  if (any) done_cv.notify_all();
}

void ct_server::loop() {
  cudaSetDevice(device);
  std::unique_lock<std::mutex> lk(mu);
  while (true) {
    if (pending.empty() && render.empty() && finishing.empty()) {
      if (stop) break;
      cv.wait(lk, [&] { return stop || !pending.empty(); });
      continue;
    }
    // admissions in arrival order (accounting under the lock, device work outside);
    // a query may pass a render job that waits for queue space (renders keep their
    // order among themselves, and the HBM budget is taken in arrival order)
    std::vector<Request*> admitted;
    bool render_waits = false;
    for (size_t i = 0; i < pending.size();) {
      Request* r = pending[i];
      if (r->kind == kRender && render_waits) {
        i++;
        continue;
      }
      r->bytes = request_bytes(*r);
      const bool fits_budget = cfg.hbm_budget == 0 || used_bytes + r->bytes <= cfg.hbm_budget;
      const bool fits_queue = r->kind != kRender || inflight_pixels + r->k * r->pixels <= cfg.max_inflight_pixels;
      if (!fits_budget || !fits_queue) {
        if (i == 0 && render.empty() && finishing.empty() && admitted.empty()) {
          // cannot fit even with nothing else admitted
          pending.erase(pending.begin());
          r->status = CT_ERR_OUT_OF_MEMORY;
          r->bytes = 0;
          r->state = kFinishing;
          finishing.push_back(r);
          continue;
        }
        if (fits_budget && r->kind == kRender) {  // waits for queue space only
          render_waits = true;
          i++;
          continue;
        }
        break;
      }
      pending.erase(pending.begin() + (std::ptrdiff_t)i);
      if (!rt_account(ctx, (int64_t)r->bytes)) {
        r->status = CT_ERR_OUT_OF_MEMORY;
        r->bytes = 0;
        r->state = kFinishing;
        finishing.push_back(r);
        continue;
      }
      used_bytes += r->bytes;
      stats.peak_bytes = std::max<uint64_t>(stats.peak_bytes, used_bytes);
      if (r->kind == kRender) inflight_pixels += r->k * r->pixels;
      else stats.query_rays += r->n;
      r->t_admit = now();
      admitted.push_back(r);
    }
    lk.unlock();
    for (Request* r : admitted) start(r);
    std::vector<Request*> finished;
    for (Request* r : admitted) {
      if (r->status != CT_OK) {
        if (r->kind == kRender) inflight_pixels -= r->k * r->pixels;
        finished.push_back(r);
      } else if (r->kind == kRender) {
        render.push_back(r);
      } else {
        finished.push_back(r);  // completion event recorded on the query stream
      }
    }
    bool iterated = false, stream_busy = false;
    if (!render.empty()) {
      // issue the next iteration only once its stream's previous one has finished,
      // so the thread keeps admitting and starting queries in the meantime
      const cudaError_t q = cudaEventQuery(table_ev[slot]);
      stream_busy = q == cudaErrorNotReady;
      if (stream_busy) cudaGetLastError();
    }
    if (!render.empty() && !stream_busy) {
      const cudaError_t e = render_iteration(finished);
      iterated = true;
      if (e != cudaSuccess) {
        cudaGetLastError();
        // jobs still in flight give their queue space back with their failure
        for (Request* r : render) {
          r->status = CT_ERR_CUDA;
          inflight_pixels -= r->k * r->pixels;
          finished.push_back(r);
        }
        render.clear();
      }
    }
    lk.lock();
    if (iterated) stats.iterations++;
    for (Request* r : finished) r->state = kFinishing, finishing.push_back(r);
    retire_locked();
    if ((render.empty() && !finishing.empty() && pending.empty()) || stream_busy) {
      // only completions outstanding, or the render streams busy: wait briefly
      // instead of spinning (a new arrival ends the wait at once)
      const uint64_t seen = next_id;  // advances with every submission
      cv.wait_for(lk, std::chrono::microseconds(50), [&] { return stop || next_id != seen; });
    }
  }
}

extern "C" {

ct_status ct_server_create(ct_ctx* ctx, const ct_server_config* cfg, ct_server** out) {
  if (!ctx || !cfg || !out || cfg->max_inflight_pixels == 0) return rt_fail(ctx, CT_ERR_INVALID_ARGUMENT, "bad server config");
  *out = nullptr;
  if (cudaSetDevice(rt_ctx_device(ctx)) != cudaSuccess) return rt_fail(ctx, CT_ERR_CUDA, "cudaSetDevice");
  auto* s = new ct_server();
  s->ctx = ctx;
  s->cfg = *cfg;
  s->device = rt_ctx_device(ctx);
  s->t0 = std::chrono::steady_clock::now();
  ct_status st = CT_OK;
  for (int k = 0; k < kStreams && st == CT_OK; k++)
    st = rt_alloc_queues(ctx, cfg->max_inflight_pixels, s->q[k], s->q_owned[k]);
  cudaError_t e = cudaSuccess;
  // a private pool that keeps freed request memory between requests
  if (st == CT_OK) {
    cudaMemPoolProps props;
    std::memset(&props, 0, sizeof(props));
    props.allocType = cudaMemAllocationTypePinned;
    props.location.type = cudaMemLocationTypeDevice;
    props.location.id = s->device;
    e = cudaMemPoolCreate(&s->pool, &props);
    if (e == cudaSuccess) {
      uint64_t keep = ~0ull;
      e = cudaMemPoolSetAttribute(s->pool, cudaMemPoolAttrReleaseThreshold, &keep);
    }
  }
  for (int k = 0; k < kStreams && st == CT_OK && e == cudaSuccess; k++)
    e = cudaStreamCreateWithFlags(&s->rs[k], cudaStreamNonBlocking);
  // ray queries and the request set-up (zero fills) run at the device's highest stream
  // priority: their kernels are short and a query should not wait behind a render iteration
  int prio_least = 0, prio_greatest = 0;
  if (st == CT_OK && e == cudaSuccess) e = cudaDeviceGetStreamPriorityRange(&prio_least, &prio_greatest);
  if (st == CT_OK && e == cudaSuccess)
    e = cudaStreamCreateWithPriority(&s->qs, cudaStreamNonBlocking, prio_greatest);
  if (st == CT_OK && e == cudaSuccess)
    e = cudaStreamCreateWithPriority(&s->ms, cudaStreamNonBlocking, prio_greatest);
  for (int k = 0; k < kStreams && st == CT_OK && e == cudaSuccess; k++) {
    e = cudaEventCreateWithFlags(&s->table_ev[k], cudaEventDisableTiming);
    if (e == cudaSuccess) e = cudaEventRecord(s->table_ev[k], s->rs[k]);
  }
  if (st != CT_OK || e != cudaSuccess) {
    for (int k = 0; k < kStreams; k++) {
      rt_free_list(ctx, s->q_owned[k]);
      if (s->rs[k]) cudaStreamDestroy(s->rs[k]);
    }
    for (cudaStream_t x : {s->qs, s->ms})
      if (x) cudaStreamDestroy(x);
    if (s->pool) cudaMemPoolDestroy(s->pool);
    delete s;
    return st != CT_OK ? st : rt_fail(ctx, CT_ERR_CUDA, cudaGetErrorString(e));
  }
  s->th = std::thread([s] { s->loop(); });
  *out = s;
  return CT_OK;
}

ct_status ct_server_destroy(ct_server* s) {
  if (!s) return CT_ERR_INVALID_ARGUMENT;
  {
    std::lock_guard<std::mutex> g(s->mu);
    s->stop = true;
  }
  s->cv.notify_all();
  s->th.join();
  cudaSetDevice(s->device);
  cudaDeviceSynchronize();
  for (auto& kv : s->all) {
    if (kv.second->ev) cudaEventDestroy(kv.second->ev);
    if (kv.second->ready) cudaEventDestroy(kv.second->ready);
    delete kv.second;
  }
  s->free_tables();
  for (int k = 0; k < kStreams; k++) {
    if (s->table_ev[k]) cudaEventDestroy(s->table_ev[k]);
    rt_free_list(s->ctx, s->q_owned[k]);
    if (s->rs[k]) cudaStreamDestroy(s->rs[k]);
  }
  for (cudaStream_t x : {s->qs, s->ms})
    if (x) cudaStreamDestroy(x);
  if (s->pool) cudaMemPoolDestroy(s->pool);  // every request's memory was freed in stream order above
  delete s;
  return CT_OK;
}

ct_status ct_server_submit_render(ct_server* s, const ct_batch_job* job, float* host_out, uint64_t* request_id) {
  if (!s || !job || !host_out || !request_id) return CT_ERR_INVALID_ARGUMENT;
  const ct_status st = rt_check_job(s->ctx, *job);
  if (st != CT_OK) return st;
  auto* r = new Request();
  r->kind = kRender;
  r->job = *job;
  r->host_out = host_out;
  r->pixels = (uint32_t)(job->params.width * job->params.height);
  const uint32_t per_iter = std::min(s->cfg.iter_pixels ? s->cfg.iter_pixels : kIterPixels, s->cfg.max_inflight_pixels);
  r->k = std::max<uint32_t>(1, std::min<uint32_t>(job->spp, per_iter / r->pixels));
  r->slots = std::min<uint32_t>(job->spp, kStreams * r->k);
  {
    std::lock_guard<std::mutex> g(s->mu);
    r->id = s->next_id++;
    r->t_submit = s->now();
    s->all[r->id] = r;
    s->pending.push_back(r);
    s->stats.submitted++;
  }
  s->cv.notify_all();
  *request_id = r->id;
  return CT_OK;
}

ct_status ct_server_submit_query(ct_server* s, const ct_bvh* bvh, const float* host_org, const float* host_dir,
                                 uint32_t n, float tri_eps, int32_t any_hit, int32_t* host_hit, float* host_t,
                                 uint8_t* host_occluded, uint64_t* request_id) {
  if (!s || !bvh || !host_org || !host_dir || !request_id || n == 0) return CT_ERR_INVALID_ARGUMENT;
  if (any_hit ? !host_occluded : (!host_hit || !host_t)) return CT_ERR_INVALID_ARGUMENT;
  auto* r = new Request();
  r->kind = any_hit ? kAny : kClosest;
  r->bvh = bvh;
  r->horg = host_org;
  r->hdir = host_dir;
  r->n = n;
  r->tri_eps = tri_eps;
  r->hhit = host_hit;
  r->ht = host_t;
  r->hocc = host_occluded;
  {
    std::lock_guard<std::mutex> g(s->mu);
    r->id = s->next_id++;
    r->t_submit = s->now();
    s->all[r->id] = r;
    s->pending.push_back(r);
    s->stats.submitted++;
  }
  s->cv.notify_all();
  *request_id = r->id;
  return CT_OK;
}

ct_status ct_server_wait(ct_server* s, uint64_t id, double timeout_s, ct_request_info* info) {
  if (!s) return CT_ERR_INVALID_ARGUMENT;
  std::unique_lock<std::mutex> lk(s->mu);
  auto it = s->all.find(id);
  if (it == s->all.end()) return CT_ERR_INVALID_ARGUMENT;
  Request* r = it->second;
  auto done = [&] { return r->state == kDone; };
  if (timeout_s < 0) {
    s->done_cv.wait(lk, done);
  } else if (!s->done_cv.wait_for(lk, std::chrono::duration<double>(timeout_s), done)) {
    return CT_ERR_TIMEOUT;
  }
  if (info) {
    info->status = r->status;
    info->kind = (int32_t)r->kind;
    info->submit_s = r->t_submit;
    info->admit_s = r->t_admit;
    info->done_s = r->t_done;
    info->device_bytes = r->bytes;
  }
  const ct_status st = r->status;
  s->all.erase(it);
  delete r;
  return st;
}

ct_status ct_server_get_stats(ct_server* s, ct_server_stats* out) {
  if (!s || !out) return CT_ERR_INVALID_ARGUMENT;
  unsigned long long h[8] = {0};
  cudaSetDevice(s->device);
  // ray counters of the render iterations, both queue sets (current when no iteration is running)
  for (int k = 0; k < kStreams; k++) {
    unsigned long long hk[8] = {0};
    if (cudaMemcpy(hk, s->q[k].stats, sizeof(hk), cudaMemcpyDeviceToHost) != cudaSuccess) return CT_ERR_CUDA;
    for (int i = 0; i < 8; i++) h[i] += hk[i];
  }
  std::lock_guard<std::mutex> g(s->mu);
  *out = s->stats;
  out->extension_rays = h[0];
  out->shadow_rays = h[1];
  return CT_OK;
}

}  // extern "C"
