// lsb_server.cu -- the request loop: sort jobs of mixed sizes admitted by free
// HBM onto concurrent CUDA streams, small jobs batched together as they
// arrive, buffers kept resident in a memory pool, latency percentiles beside
// throughput.
//
// The reference program sorts one array per run (mpi/mpi_lsbsort.cpp:599-789)
// and has no serving path; this is the GB300-side service around the same
// sort. Scheduling is continuous: whenever a stream slot finishes, the next
// requests that fit in the memory budget are admitted, so jobs that arrive
// while others are on the GPU overlap with them.
#include <algorithm>
#include <atomic>
#include <chrono>
#include <condition_variable>
#include <cstring>
#include <deque>
#include <mutex>
#include <thread>
#include <unordered_map>
#include <vector>

#include "../../include/lsb.h"
#include "lsb_internal.h"

namespace {

using Clock = std::chrono::steady_clock;

double ms_between(Clock::time_point a, Clock::time_point b) {
  return std::chrono::duration<double, std::milli>(b - a).count();
}

struct Request {
  uint64_t id = 0;
  int64_t n = 0;
  int kind = 0;  // 0 = host buffer, 1 = generated on the device
  lsb_elem_t* host = nullptr;
  int dist = 0;
  uint64_t seed = 0;
  int keep = 0;  // generated: keep the sorted result on the device until fetched
  Clock::time_point t_submit, t_admit, t_done;
  int status = LSB_OK;
  bool done = false;
  int batch = 1;
  struct Unit* unit = nullptr;
  int64_t unit_offset = 0;  // element offset inside the unit's buffer
};

struct Unit {
  struct Server* server = nullptr;
  int slot = -1;
  std::vector<Request*> reqs;
  int64_t n_total = 0;
  lsb_elem_t* d_a = nullptr;
  lsb_elem_t* d_b = nullptr;
  void* ws = nullptr;
  int64_t* d_off = nullptr;
  size_t bytes = 0;       // charged against the budget while buffers are held
  int kept = 0;           // results still waiting to be fetched
  bool b_ws_freed = false;
  Clock::time_point t_done;
  std::atomic<int> gpu_done{0};  // set by the stream callback
  cudaEvent_t ev_start = nullptr, ev_end = nullptr;  // the unit's span on its stream
};

struct Server {
  lsb_server_config_t cfg{};
  int device = 0;
  cudaMemPool_t pool = nullptr;
  std::vector<cudaStream_t> streams;
  std::vector<int64_t*> h_off;  // pinned offsets staging, per slot
  std::vector<Unit*> running;   // per slot
  std::mutex mu;
  std::condition_variable cv_work, cv_done;
  std::deque<Request*> pending;
  std::vector<Unit*> finished;  // filled by stream callbacks
  std::unordered_map<uint64_t, Request*> reqs;
  uint64_t next_id = 1;
  size_t budget = 0, in_use = 0, peak = 0;
  bool stop = false;
  std::thread worker;
  // statistics
  std::vector<double> latencies, service;
  int64_t elements_done = 0, requests_done = 0, units_done = 0, batched_requests = 0;
  Clock::time_point t_first{}, t_last{};
  bool have_first = false;
  // device spans of finished units, ms after ref_event (the server's creation)
  cudaEvent_t ref_event = nullptr;
  std::vector<std::pair<float, float>> spans;
};

size_t unit_bytes(const lsb_server_config_t& cfg, int64_t n_total, int64_t nseg, size_t* ws_out) {
  size_t ws = 0;
  if (nseg > 1) lsb_segmented_workspace_bytes(n_total, nseg, cfg.digit_bits, &ws);
  else lsb_workspace_bytes(n_total, cfg.digit_bits, &ws);
  ws = lsb::align_up(std::max<size_t>(ws, 256), 256);
  *ws_out = ws;
  return 2u * (size_t)n_total * sizeof(lsb_elem_t) + ws + (size_t)(nseg + 1) * 8u + 1024u;
}

// Stream callback. It takes no lock and makes no CUDA call: the worker thread
// holds the server lock around CUDA calls, and a callback waiting for that
// lock while the CUDA runtime waits for the callback would deadlock. The
// worker picks the flag up (woken here, or by its 2 ms poll).
void CUDART_CB on_unit_done(void* p) {
  Unit* u = static_cast<Unit*>(p);
  u->t_done = Clock::now();
  u->gpu_done.store(1, std::memory_order_release);
  u->server->cv_work.notify_all();
}

int alloc_from_pool(Server* s, void** p, size_t bytes, cudaStream_t st) {
  if (cudaMallocFromPoolAsync(p, bytes, s->pool, st) != cudaSuccess) {
    cudaGetLastError();
    *p = nullptr;
    return LSB_ERR_NO_MEMORY;
  }
  return LSB_OK;
}

// Issues the whole job of a unit on its slot's stream (worker thread only).
int launch_unit(Server* s, Unit* u) {
  cudaStream_t st = s->streams[u->slot];
  const int64_t k = (int64_t)u->reqs.size();
  size_t ws_bytes = 0;
  unit_bytes(s->cfg, u->n_total, k, &ws_bytes);
  const size_t elems = (size_t)u->n_total * sizeof(lsb_elem_t);
  int rc = alloc_from_pool(s, (void**)&u->d_a, std::max<size_t>(elems, 16), st);
  if (rc == LSB_OK) rc = alloc_from_pool(s, (void**)&u->d_b, std::max<size_t>(elems, 16), st);
  if (rc == LSB_OK) rc = alloc_from_pool(s, &u->ws, ws_bytes, st);
  if (rc == LSB_OK && k > 1) rc = alloc_from_pool(s, (void**)&u->d_off, (size_t)(k + 1) * 8u, st);
  if (rc != LSB_OK) return rc;
  if (cudaEventCreate(&u->ev_start) != cudaSuccess || cudaEventCreate(&u->ev_end) != cudaSuccess ||
      cudaEventRecord(u->ev_start, st) != cudaSuccess)
    return LSB_ERR_CUDA;
  // inputs
  for (Request* r : u->reqs) {
    lsb_elem_t* dst = u->d_a + r->unit_offset;
    if (r->kind == 0) {
      if (r->n && cudaMemcpyAsync(dst, r->host, (size_t)r->n * sizeof(lsb_elem_t),
                                  cudaMemcpyHostToDevice, st) != cudaSuccess)
        return LSB_ERR_CUDA;
    } else if (int g = lsb_generate(dst, r->n, r->dist, r->seed, st)) {
      return g;
    }
  }
  // the sort: one request alone, or the batch as segments of one sort
  if (k == 1) {
    rc = lsb_sort_pairs(u->d_a, u->d_b, u->n_total, s->cfg.digit_bits, u->ws, ws_bytes, st);
  } else {
    int64_t* h = s->h_off[u->slot];
    h[0] = 0;
    for (int64_t i = 0; i < k; i++) h[i + 1] = h[i] + u->reqs[i]->n;
    if (cudaMemcpyAsync(u->d_off, h, (size_t)(k + 1) * 8u, cudaMemcpyHostToDevice, st) != cudaSuccess)
      return LSB_ERR_CUDA;
    lsb_tuning_t t;
    std::memset(&t, 0, sizeof t);
    t.digit_bits = s->cfg.digit_bits;
    rc = lsb_sort_segmented(u->d_a, u->d_b, u->n_total, u->d_off, k, &t, u->ws, ws_bytes, st);
  }
  if (rc != LSB_OK) return rc;
  // outputs
  for (Request* r : u->reqs)
    if (r->kind == 0 && r->n &&
        cudaMemcpyAsync(r->host, u->d_a + r->unit_offset, (size_t)r->n * sizeof(lsb_elem_t),
                        cudaMemcpyDeviceToHost, st) != cudaSuccess)
      return LSB_ERR_CUDA;
  if (cudaEventRecord(u->ev_end, st) != cudaSuccess) return LSB_ERR_CUDA;
  if (cudaLaunchHostFunc(st, on_unit_done, u) != cudaSuccess) return LSB_ERR_CUDA;
  return LSB_OK;
}

// Worker thread: completions, then admission, continuously.
void worker_loop(Server* s) {
  cudaSetDevice(s->device);
  std::unique_lock<std::mutex> lk(s->mu);
  const int64_t small = s->cfg.batch_max_elems > 0 ? s->cfg.batch_max_elems : (int64_t)1 << 22;
  for (;;) {
    s->cv_work.wait_for(lk, std::chrono::milliseconds(2), [&] {
      if (s->stop || !s->finished.empty()) return true;
      for (Unit* u : s->running)
        if (u && u->gpu_done.load(std::memory_order_acquire)) return true;
      if (s->pending.empty()) return false;
      for (Unit* u : s->running)
        if (!u) return true;
      return false;
    });
    // 1. completed units: release what is not kept, record statistics
    for (Unit* u : s->running)
      if (u && u->gpu_done.load(std::memory_order_acquire)) {
        for (Request* r : u->reqs) r->t_done = u->t_done;
        s->finished.push_back(u);
      }
    std::vector<Unit*> fin;
    fin.swap(s->finished);
    for (Unit* u : fin) {
      cudaStream_t st = s->streams[u->slot];
      lk.unlock();
      if (u->d_b) cudaFreeAsync(u->d_b, st);
      if (u->ws) cudaFreeAsync(u->ws, st);
      if (u->d_off) cudaFreeAsync(u->d_off, st);
      float t0 = 0.f, t1 = 0.f;
      const bool timed = u->ev_start && u->ev_end && u->gpu_done.load(std::memory_order_acquire) &&
                         cudaEventElapsedTime(&t0, s->ref_event, u->ev_start) == cudaSuccess &&
                         cudaEventElapsedTime(&t1, s->ref_event, u->ev_end) == cudaSuccess;
      if (u->ev_start) cudaEventDestroy(u->ev_start);
      if (u->ev_end) cudaEventDestroy(u->ev_end);
      u->ev_start = u->ev_end = nullptr;
      cudaGetLastError();
      lk.lock();
      if (timed) s->spans.emplace_back(t0, t1);
      u->b_ws_freed = true;
      s->running[u->slot] = nullptr;
      for (Request* r : u->reqs) {
        r->done = true;
        if (r->kind == 1 && r->keep) u->kept++;
        s->latencies.push_back(ms_between(r->t_submit, r->t_done));
        s->service.push_back(ms_between(r->t_admit, r->t_done));
        s->elements_done += r->n;
        s->requests_done++;
        if (u->reqs.size() > 1) s->batched_requests++;
        if (!s->have_first || r->t_submit < s->t_first) s->t_first = r->t_submit;
        s->have_first = true;
        if (r->t_done > s->t_last) s->t_last = r->t_done;
      }
      s->units_done++;
      const size_t ab = 2u * (size_t)u->n_total * sizeof(lsb_elem_t);
      if (u->kept == 0) {
        lk.unlock();
        if (u->d_a) cudaFreeAsync(u->d_a, st);
        lk.lock();
        s->in_use -= u->bytes;
        for (Request* r : u->reqs) r->unit = nullptr;
        delete u;
      } else {
        const size_t keep_bytes = ab / 2;
        s->in_use -= (u->bytes - keep_bytes);
        u->bytes = keep_bytes;
      }
    }
    if (!fin.empty()) s->cv_done.notify_all();
    if (s->stop && s->pending.empty()) {
      bool idle = true;
      for (Unit* u : s->running) idle = idle && !u;
      if (idle) break;
    }
    // 2. admission: FIFO; consecutive small requests become one batch
    for (int slot = 0; slot < (int)s->running.size() && !s->pending.empty(); slot++) {
      if (s->running[slot]) continue;
      Unit* u = new Unit();
      u->server = s;
      u->slot = slot;
      int64_t total = 0;
      size_t need = 0, ws = 0;
      while (!s->pending.empty()) {
        Request* r = s->pending.front();
        const bool batchable = r->n <= small && (u->reqs.empty() || total + r->n <= small);
        if (!u->reqs.empty() && !batchable) break;
        if ((int64_t)u->reqs.size() >= s->cfg.batch_max_requests && s->cfg.batch_max_requests > 0) break;
        const size_t b = unit_bytes(s->cfg, total + r->n, (int64_t)u->reqs.size() + 1, &ws);
        if (s->in_use + b > s->budget) break;  // wait for memory to free up
        need = b;
        r->unit_offset = total;
        total += r->n;
        u->reqs.push_back(r);
        s->pending.pop_front();
        if (r->n > small) break;  // large jobs run alone
      }
      if (u->reqs.empty()) {
        delete u;
        break;
      }
      u->n_total = total;
      u->bytes = need;
      s->in_use += need;
      s->peak = std::max(s->peak, s->in_use);
      s->running[slot] = u;
      const auto now = Clock::now();
      for (Request* r : u->reqs) {
        r->t_admit = now;
        r->unit = u;
        r->batch = (int)u->reqs.size();
      }
      lk.unlock();
      const int rc = launch_unit(s, u);
      lk.lock();
      if (rc != LSB_OK) {
        // the unit never reaches its callback: finish it here
        for (Request* r : u->reqs) {
          r->status = rc;
          r->t_done = Clock::now();
        }
        s->finished.push_back(u);
      }
    }
  }
}

}  // namespace

struct lsb_server : Server {};

extern "C" {

int lsb_server_create(const lsb_server_config_t* cfg, lsb_server_t** out) {
  if (!out) return LSB_ERR_INVALID_ARG;
  *out = nullptr;
  lsb_server* s = new lsb_server();
  if (cfg) s->cfg = *cfg;
  if (s->cfg.slots <= 0) s->cfg.slots = 4;
  if (s->cfg.digit_bits < 1 || s->cfg.digit_bits > 16) s->cfg.digit_bits = 16;
  if (cudaGetDevice(&s->device) != cudaSuccess) {
    delete s;
    return LSB_ERR_NO_DEVICE;
  }
  size_t free_b = 0, total_b = 0;
  if (cudaMemGetInfo(&free_b, &total_b) != cudaSuccess) {
    delete s;
    return LSB_ERR_CUDA;
  }
  s->budget = s->cfg.hbm_budget_bytes > 0 ? (size_t)s->cfg.hbm_budget_bytes : free_b / 10 * 8;
  cudaMemPoolProps pp;
  std::memset(&pp, 0, sizeof pp);
  pp.allocType = cudaMemAllocationTypePinned;
  pp.location.type = cudaMemLocationTypeDevice;
  pp.location.id = s->device;
  if (cudaMemPoolCreate(&s->pool, &pp) != cudaSuccess) {
    delete s;
    return LSB_ERR_CUDA;
  }
  uint64_t keep = UINT64_MAX;  // buffers stay resident in the pool between requests
  cudaMemPoolSetAttribute(s->pool, cudaMemPoolAttrReleaseThreshold, &keep);
  const int64_t maxb = s->cfg.batch_max_requests > 0 ? s->cfg.batch_max_requests : 4096;
  for (int i = 0; i < s->cfg.slots; i++) {
    cudaStream_t st;
    int64_t* h = nullptr;
    if (cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking) != cudaSuccess ||
        cudaMallocHost((void**)&h, (size_t)(maxb + 1) * 8u) != cudaSuccess) {
      delete s;
      return LSB_ERR_CUDA;
    }
    s->streams.push_back(st);
    s->h_off.push_back(h);
    s->running.push_back(nullptr);
  }
  if (s->cfg.batch_max_requests <= 0) s->cfg.batch_max_requests = (int32_t)maxb;
  if (cudaEventCreate(&s->ref_event) != cudaSuccess ||
      cudaEventRecord(s->ref_event, s->streams[0]) != cudaSuccess ||
      cudaEventSynchronize(s->ref_event) != cudaSuccess) {
    delete s;
    return LSB_ERR_CUDA;
  }
  s->worker = std::thread(worker_loop, s);
  *out = s;
  return LSB_OK;
}

static int submit(lsb_server_t* s, Request* r, uint64_t* id) {
  std::lock_guard<std::mutex> lk(s->mu);
  if (s->stop) {
    delete r;
    return LSB_ERR_INVALID_ARG;
  }
  r->id = s->next_id++;
  r->t_submit = Clock::now();
  s->reqs[r->id] = r;
  s->pending.push_back(r);
  if (id) *id = r->id;
  s->cv_work.notify_all();
  return LSB_OK;
}

int lsb_server_submit_host(lsb_server_t* s, lsb_elem_t* h_data, int64_t n, uint64_t* id) {
  if (!s || n < 0 || (n > 0 && !h_data)) return LSB_ERR_INVALID_ARG;
  if (n > LSB_MAX_ELEMENTS) return LSB_ERR_TOO_LARGE;
  Request* r = new Request();
  r->kind = 0;
  r->host = h_data;
  r->n = n;
  return submit(s, r, id);
}

int lsb_server_submit_generated(lsb_server_t* s, int64_t n, int dist, uint64_t seed, int keep_result,
                                uint64_t* id) {
  if (!s || n < 0 || dist < 0 || dist > LSB_DIST_NEARLY_SORTED) return LSB_ERR_INVALID_ARG;
  if (n > LSB_MAX_ELEMENTS) return LSB_ERR_TOO_LARGE;
  Request* r = new Request();
  r->kind = 1;
  r->n = n;
  r->dist = dist;
  r->seed = seed;
  r->keep = keep_result ? 1 : 0;
  return submit(s, r, id);
}

int lsb_server_wait(lsb_server_t* s, uint64_t id, double timeout_s, lsb_request_info_t* info) {
  if (!s) return LSB_ERR_INVALID_ARG;
  std::unique_lock<std::mutex> lk(s->mu);
  auto it = s->reqs.find(id);
  if (it == s->reqs.end()) return LSB_ERR_INVALID_ARG;
  Request* r = it->second;
  const auto deadline = Clock::now() + std::chrono::duration_cast<Clock::duration>(
                                           std::chrono::duration<double>(timeout_s));
  while (!r->done) {
    if (s->cv_done.wait_until(lk, deadline) == std::cv_status::timeout && !r->done)
      return LSB_ERR_DEVICE_TIMEOUT;
  }
  if (info) {
    std::memset(info, 0, sizeof *info);
    info->status = r->status;
    info->batch = r->batch;
    info->n = r->n;
    info->latency_ms = ms_between(r->t_submit, r->t_done);
    info->queue_ms = ms_between(r->t_submit, r->t_admit);
  }
  return r->status;
}

int lsb_server_fetch(lsb_server_t* s, uint64_t id, lsb_elem_t* h_out, int64_t n) {
  if (!s || n < 0 || (n > 0 && !h_out)) return LSB_ERR_INVALID_ARG;
  Unit* u = nullptr;
  lsb_elem_t* src = nullptr;
  cudaStream_t st = nullptr;
  {
    std::lock_guard<std::mutex> lk(s->mu);
    auto it = s->reqs.find(id);
    if (it == s->reqs.end()) return LSB_ERR_INVALID_ARG;
    Request* r = it->second;
    if (!r->done || r->kind != 1 || !r->keep || !r->unit) return LSB_ERR_INVALID_ARG;
    if (n != r->n) return LSB_ERR_INVALID_ARG;
    u = r->unit;
    src = u->d_a + r->unit_offset;
    st = s->streams[u->slot];
    r->keep = 0;
  }
  int rc = LSB_OK;
  if (n && (cudaMemcpyAsync(h_out, src, (size_t)n * sizeof(lsb_elem_t), cudaMemcpyDeviceToHost, st) !=
                cudaSuccess ||
            cudaStreamSynchronize(st) != cudaSuccess))
    rc = LSB_ERR_CUDA;
  lsb_elem_t* to_free = nullptr;
  {
    std::lock_guard<std::mutex> lk(s->mu);
    if (--u->kept == 0) {
      to_free = u->d_a;
      s->in_use -= u->bytes;
      for (Request* r : u->reqs) r->unit = nullptr;
      delete u;
    }
  }
  if (to_free) {  // CUDA calls only outside the server lock
    cudaFreeAsync(to_free, st);
    s->cv_work.notify_all();
  }
  return rc;
}

int lsb_server_device_stats(lsb_server_t* s, lsb_server_device_stats_t* out) {
  if (!s || !out) return LSB_ERR_INVALID_ARG;
  std::vector<std::pair<float, float>> sp;
  {
    std::lock_guard<std::mutex> lk(s->mu);
    sp = s->spans;
  }
  std::memset(out, 0, sizeof *out);
  out->units_timed = (int64_t)sp.size();
  if (sp.empty()) return LSB_OK;
  // union of the spans, and the most spans open at one instant (an end
  // sorts before a start at the same time)
  std::vector<std::pair<double, int>> ev;
  double sum = 0.0;
  for (auto& x : sp) {
    sum += (double)x.second - x.first;
    ev.emplace_back(x.first, +1);
    ev.emplace_back(x.second, -1);
  }
  std::sort(ev.begin(), ev.end());
  int open = 0, peak = 0;
  double busy = 0.0, since = 0.0;
  for (auto& e : ev) {
    if (e.second > 0) {
      if (open == 0) since = e.first;
      open++;
      peak = std::max(peak, open);
    } else {
      open--;
      if (open == 0) busy += e.first - since;
    }
  }
  out->busy_ms = busy;
  out->unit_ms_sum = sum;
  out->overlap = busy > 0.0 ? sum / busy : 0.0;
  out->max_concurrent = peak;
  return LSB_OK;
}

int lsb_server_stats(lsb_server_t* s, lsb_server_stats_t* out) {
  if (!s || !out) return LSB_ERR_INVALID_ARG;
  std::lock_guard<std::mutex> lk(s->mu);
  std::memset(out, 0, sizeof *out);
  out->requests_done = s->requests_done;
  out->elements_done = s->elements_done;
  out->units = s->units_done;
  out->batched_requests = s->batched_requests;
  out->peak_bytes = (int64_t)s->peak;
  out->budget_bytes = (int64_t)s->budget;
  if (!s->latencies.empty()) {
    std::vector<double> l = s->latencies, sv = s->service;
    std::sort(l.begin(), l.end());
    std::sort(sv.begin(), sv.end());
    auto pct = [](const std::vector<double>& v, double q) {
      return v[std::min(v.size() - 1, (size_t)(q * (double)(v.size() - 1) + 0.5))];
    };
    out->latency_p50_ms = pct(l, 0.50);
    out->latency_p99_ms = pct(l, 0.99);
    out->service_p50_ms = pct(sv, 0.50);
    out->service_p99_ms = pct(sv, 0.99);
    const double span = ms_between(s->t_first, s->t_last);
    out->wall_ms = span;
    out->elements_per_s = span > 0 ? (double)s->elements_done / (span / 1e3) : 0.0;
  }
  return LSB_OK;
}

int lsb_server_destroy(lsb_server_t* s) {
  if (!s) return LSB_OK;
  {
    std::lock_guard<std::mutex> lk(s->mu);
    s->stop = true;
    s->cv_work.notify_all();
  }
  if (s->worker.joinable()) s->worker.join();
  for (cudaStream_t st : s->streams) cudaStreamSynchronize(st);
  for (auto& kv : s->reqs) {
    Request* r = kv.second;
    if (r->unit && r->keep) {  // results never fetched
      Unit* u = r->unit;
      if (--u->kept == 0) {
        cudaFreeAsync(u->d_a, s->streams[u->slot]);
        for (Request* q : u->reqs) q->unit = nullptr;
        delete u;
      }
    }
  }
  for (cudaStream_t st : s->streams) {
    cudaStreamSynchronize(st);
    cudaStreamDestroy(st);
  }
  for (int64_t* h : s->h_off) cudaFreeHost(h);
  for (auto& kv : s->reqs) delete kv.second;
  if (s->pool) cudaMemPoolDestroy(s->pool);
  delete s;
  return LSB_OK;
}

}  // extern "C"
