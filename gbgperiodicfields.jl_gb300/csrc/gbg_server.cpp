// Serving loop (C ABI: gbg_server_*): resident fields, requests admitted by free device
// memory, continuous batching over stream slots, event-polled completion with deadlines.
//
// The reference has no request loop; this is the serving form built around the resident
// transfers.  One native progress thread owns every CUDA call the server makes:
//
//   submit (any thread)  -> queue (arrival order)
//   progress thread      -> retire finished slots, expire deadlines, admit the next run
//                           from the head of the queue onto a free slot, sleep briefly
//
// A run is built on its slot's stream: per request, bins from the stream-ordered pool and
// gbg_bins_build; then the batch tables (uploaded from the slot's pinned staging) and
// gbg_batch_run; then the per-request status words are copied to pinned memory and an
// event is recorded.  No call on this path synchronizes the device.
#include <algorithm>
#include <chrono>
#include <condition_variable>
#include <cstring>
#include <deque>
#include <mutex>
#include <string>
#include <thread>
#include <unordered_map>
#include <unordered_set>
#include <vector>

#include "gbg_common.cuh"

namespace {

using Clock = std::chrono::steady_clock;

double seconds_since(Clock::time_point t0, Clock::time_point t) {
  return std::chrono::duration<double>(t - t0).count();
}

// The admission rule: the longest prefix of the queue (at most max_batch requests) whose
// bytes fit in free_bytes and in which no field is scattered into twice nor gathered from
// after a scatter into it (the batch runs every gather of a run before its scatters).
int plan_run(const int32_t *kinds, const uint64_t *fields, const size_t *bytes, int n, size_t free_bytes,
             int max_batch) {
  std::unordered_set<uint64_t> written;
  size_t used = 0;
  int k = 0;
  for (; k < n && k < max_batch; ++k) {
    if (used + bytes[k] > free_bytes) break;
    if (written.count(fields[k])) break;
    if (kinds[k] == GBG_REQ_ANTERPOLATE) written.insert(fields[k]);
    used += bytes[k];
  }
  return k;
}

struct Request {
  int64_t ticket = 0;
  gbg_request r{};
  gbg_grid grid{};
  size_t bytes = 0;  // bins
  Clock::time_point submitted;
};

struct Slot {
  cudaStream_t stream = nullptr;
  cudaEvent_t done = nullptr;
  int32_t *dev_status = nullptr;   // max_batch + 1 words: per request, then the run's
  int32_t *host_status = nullptr;  // pinned copy
  void *staging = nullptr;         // pinned batch tables
  size_t staging_bytes = 0;
  bool busy = false, expired = false;
  Clock::time_point deadline;
  std::vector<Request> reqs;
  std::vector<gbg_bins> bins;
  gbg_batch batch = nullptr;
  size_t bytes = 0;
};

// Arrival-order dependencies of one field: the event of the last run that scattered into
// it and the events of the runs that gathered from it since.
struct FieldDeps {
  cudaEvent_t last_write = nullptr;
  std::vector<cudaEvent_t> reads;
};

}  // namespace

struct gbg_server_s {
  gbg_server_config cfg{};
  int device = 0;
  std::mutex mu;
  std::condition_variable cv_work, cv_done;
  std::thread worker;
  bool stop = false;
  std::string thread_error;

  std::deque<Request> queue;
  std::vector<Slot> slots;
  std::unordered_map<gbg_field, FieldDeps> deps;
  std::vector<cudaEvent_t> event_pool;
  std::unordered_map<int64_t, gbg_status> results;
  int64_t next_ticket = 1;

  size_t in_use = 0, peak = 0;
  int fault_alloc = 0, fault_deadline = 0;

  Clock::time_point t0 = Clock::now();
  int64_t submitted = 0, completed = 0, failed = 0, runs = 0, points = 0;
  bool have_first = false;
  double first_submit = 0.0, last_done = 0.0;
  std::vector<double> latencies_ms;

  int64_t in_flight_requests() const {
    int64_t n = 0;
    for (const Slot &s : slots) n += s.busy ? (int64_t)s.reqs.size() : 0;
    return n;
  }
};

namespace {

using gbg::set_error;

cudaEvent_t take_event(gbg_server_s *s) {
  if (!s->event_pool.empty()) {
    cudaEvent_t e = s->event_pool.back();
    s->event_pool.pop_back();
    return e;
  }
  cudaEvent_t e = nullptr;
  if (cudaEventCreateWithFlags(&e, cudaEventDisableTiming) != cudaSuccess) return nullptr;
  return e;
}

// Drops the dependency events that have completed (they order nothing any more).
void prune_deps(gbg_server_s *s) {
  for (auto &kv : s->deps) {
    FieldDeps &d = kv.second;
    if (d.last_write && cudaEventQuery(d.last_write) == cudaSuccess) {
      s->event_pool.push_back(d.last_write);
      d.last_write = nullptr;
    }
    auto keep = d.reads.begin();
    for (cudaEvent_t e : d.reads) {
      if (cudaEventQuery(e) == cudaSuccess) s->event_pool.push_back(e);
      else *keep++ = e;
    }
    d.reads.erase(keep, d.reads.end());
  }
}

void finish_request(gbg_server_s *s, const Request &rq, gbg_status st, Clock::time_point now) {
  s->results[rq.ticket] = st;
  if (st == GBG_OK) {
    ++s->completed;
    s->points += rq.r.npoints;
    s->latencies_ms.push_back(1e3 * std::chrono::duration<double>(now - rq.submitted).count());
  } else {
    ++s->failed;
  }
  s->last_done = seconds_since(s->t0, now);
}

void release_slot(gbg_server_s *s, Slot &sl) {
  for (gbg_bins b : sl.bins) gbg::bins_destroy_async(b, sl.stream);
  gbg::batch_destroy_async(sl.batch, sl.stream);
  sl.bins.clear();
  sl.batch = nullptr;
  s->in_use -= sl.bytes;
  sl.bytes = 0;
  sl.reqs.clear();
  sl.busy = sl.expired = false;
}

// Retires finished runs and reports runs past their deadline.
void poll_slots(gbg_server_s *s) {
  const Clock::time_point now = Clock::now();
  for (Slot &sl : s->slots) {
    if (!sl.busy) continue;
    const cudaError_t q = cudaEventQuery(sl.done);
    if (q == cudaSuccess) {
      if (!sl.expired) {
        const int32_t run_word = sl.host_status[s->cfg.max_batch];
        for (size_t i = 0; i < sl.reqs.size(); ++i) {
          const int32_t w = sl.host_status[i] | run_word;
          gbg_status st = GBG_OK;
          if (w & GBG_DEV_TIMEOUT) st = GBG_ETIMEOUT;
          else if (w & GBG_DEV_NONFINITE) st = GBG_ENONFINITE;
          finish_request(s, sl.reqs[i], st, now);
        }
      }
      release_slot(s, sl);
      s->cv_done.notify_all();
    } else if (q != cudaErrorNotReady) {
      cudaGetLastError();
      if (!sl.expired)
        for (const Request &rq : sl.reqs) finish_request(s, rq, GBG_ECUDA, now);
      s->thread_error = std::string("run failed on the device: ") + cudaGetErrorString(q);
      // the slot's memory cannot be shown idle; it is kept out of use
      sl.expired = true;
      s->cv_done.notify_all();
    } else if (!sl.expired && now >= sl.deadline) {
      for (const Request &rq : sl.reqs) finish_request(s, rq, GBG_ETIMEOUT, now);
      sl.expired = true;  // memory stays held until the event completes
      s->cv_done.notify_all();
    }
  }
}

// Orders a run on `st` after the earlier runs it depends on, and records its event as
// the fields' new last write / reader.
void order_run(gbg_server_s *s, cudaStream_t st, const std::vector<Request> &reqs, cudaEvent_t done, bool before) {
  std::unordered_set<gbg_field> reads, writes;
  for (const Request &rq : reqs) (rq.r.kind == GBG_REQ_ANTERPOLATE ? writes : reads).insert(rq.r.field);
  if (before) {
    for (gbg_field f : reads) {
      auto it = s->deps.find(f);
      if (it != s->deps.end() && it->second.last_write) cudaStreamWaitEvent(st, it->second.last_write, 0);
    }
    for (gbg_field f : writes) {
      auto it = s->deps.find(f);
      if (it == s->deps.end()) continue;
      if (it->second.last_write) cudaStreamWaitEvent(st, it->second.last_write, 0);
      for (cudaEvent_t e : it->second.reads) cudaStreamWaitEvent(st, e, 0);
    }
    return;
  }
  // after the run: one event per field role (the slot's own `done` is reused elsewhere)
  for (gbg_field f : writes) {
    FieldDeps &d = s->deps[f];
    cudaEvent_t e = take_event(s);
    if (!e) continue;
    cudaEventRecord(e, st);
    if (d.last_write) s->event_pool.push_back(d.last_write);
    d.last_write = e;
    for (cudaEvent_t r : d.reads) s->event_pool.push_back(r);
    d.reads.clear();
  }
  for (gbg_field f : reads) {
    if (writes.count(f)) continue;
    cudaEvent_t e = take_event(s);
    if (!e) continue;
    cudaEventRecord(e, st);
    s->deps[f].reads.push_back(e);
  }
  (void)done;
}

// Builds and launches one run on a free slot; returns false when nothing was admitted.
bool admit(gbg_server_s *s) {
  if (s->queue.empty()) return false;
  Slot *slot = nullptr;
  for (Slot &sl : s->slots)
    if (!sl.busy) {
      slot = &sl;
      break;
    }
  if (!slot) return false;
  const int n = (int)std::min<size_t>(s->queue.size(), (size_t)s->cfg.max_batch);
  std::vector<int32_t> kinds(n);
  std::vector<uint64_t> fields(n);
  std::vector<size_t> bytes(n);
  for (int i = 0; i < n; ++i) {
    kinds[i] = s->queue[i].r.kind;
    fields[i] = reinterpret_cast<uint64_t>(s->queue[i].r.field);
    bytes[i] = s->queue[i].bytes;
  }
  const size_t free_bytes = s->cfg.hbm_budget_bytes > s->in_use ? s->cfg.hbm_budget_bytes - s->in_use : 0;
  const int k = plan_run(kinds.data(), fields.data(), bytes.data(), n, free_bytes, s->cfg.max_batch);
  if (k == 0) return false;
  Slot &sl = *slot;
  sl.reqs.assign(s->queue.begin(), s->queue.begin() + k);
  s->queue.erase(s->queue.begin(), s->queue.begin() + k);
  const Clock::time_point now = Clock::now();
  cudaStream_t st = sl.stream;
  order_run(s, st, sl.reqs, sl.done, true);
  // per-request bins; a request whose allocation fails is reported and left out
  std::vector<Request> kept;
  std::vector<gbg_batch_item> items;
  for (const Request &rq : sl.reqs)
    if (rq.r.ready_event) cudaStreamWaitEvent(st, static_cast<cudaEvent_t>(rq.r.ready_event), 0);
  cudaMemsetAsync(sl.dev_status, 0, sizeof(int32_t) * (s->cfg.max_batch + 1), st);
  for (Request &rq : sl.reqs) {
    gbg_bins b = nullptr;
    gbg_status bst = GBG_ENOMEM;
    if (s->fault_alloc > 0) {
      --s->fault_alloc;
      set_error(GBG_ENOMEM, "injected allocation failure");
    } else {
      size_t got = 0;
      bst = gbg::bins_create_async(rq.grid, rq.r.npoints, s->cfg.brick, st, &b, &got);
      if (bst == GBG_OK) {
        sl.bytes += got;
        s->in_use += got;
      }
    }
    if (bst == GBG_OK)
      bst = gbg_bins_build(b, rq.r.pos_dtype, rq.r.positions, rq.r.npoints, sl.dev_status + kept.size(), st);
    if (bst != GBG_OK) {
      if (b) gbg::bins_destroy_async(b, st);
      finish_request(s, rq, bst, now);
      continue;
    }
    sl.bins.push_back(b);
    gbg_batch_item it{};
    it.field = rq.r.field;
    it.bins = b;
    it.scheme = rq.r.scheme;
    if (rq.r.kind == GBG_REQ_INTERPOLATE) {
      it.out = rq.r.out;
    } else {
      it.dest = rq.r.field;
      it.q = rq.r.q;
      it.alpha = rq.r.alpha;
      it.beta = rq.r.beta;
    }
    items.push_back(it);
    kept.push_back(rq);
  }
  sl.reqs.swap(kept);
  s->peak = std::max(s->peak, s->in_use);
  gbg_status bst = GBG_OK;
  if (!items.empty()) {
    bst = gbg::batch_create_async(items.data(), (int32_t)items.size(), st, sl.staging, sl.staging_bytes, &sl.batch);
    if (bst == GBG_OK) bst = gbg_batch_run(sl.batch, sl.dev_status + s->cfg.max_batch, st);
  }
  if (bst != GBG_OK) {
    // nothing of the run was launched past the bins: report and release in stream order
    for (const Request &rq : sl.reqs) finish_request(s, rq, bst, now);
    sl.reqs.clear();
  }
  cudaMemcpyAsync(sl.host_status, sl.dev_status, sizeof(int32_t) * (s->cfg.max_batch + 1), cudaMemcpyDeviceToHost,
                  st);
  order_run(s, st, sl.reqs, sl.done, false);
  cudaEventRecord(sl.done, st);
  sl.busy = true;
  sl.expired = sl.reqs.empty();
  sl.deadline = now + std::chrono::duration_cast<Clock::duration>(std::chrono::duration<double>(s->cfg.timeout_seconds));
  if (s->fault_deadline > 0) {
    --s->fault_deadline;
    sl.deadline = now;
  }
  ++s->runs;
  s->cv_done.notify_all();
  return true;
}

void worker_main(gbg_server_s *s) {
  cudaSetDevice(s->device);
  std::unique_lock<std::mutex> lk(s->mu);
  int idle = 0;
  while (true) {
    poll_slots(s);
    bool any = false;
    while (admit(s)) any = true;
    if (any) prune_deps(s);
    bool busy = false;
    for (const Slot &sl : s->slots) busy = busy || sl.busy;
    if (s->stop && s->queue.empty() && !busy) break;
    if (s->stop && !busy && !s->queue.empty()) {
      // stopping with requests that can never be admitted (budget): fail them
      const Clock::time_point now = Clock::now();
      for (const Request &rq : s->queue) finish_request(s, rq, GBG_EBUSY, now);
      s->queue.clear();
      s->cv_done.notify_all();
      continue;
    }
    if (!busy && s->queue.empty()) {
      s->cv_work.wait_for(lk, std::chrono::milliseconds(5));
      idle = 0;
    } else {
      // device work in flight: poll the events every few microseconds
      lk.unlock();
      if (++idle < 64) std::this_thread::yield();
      else std::this_thread::sleep_for(std::chrono::microseconds(20));
      lk.lock();
    }
  }
}

gbg_status check_request(const gbg_request &r, gbg_grid *grid) {
  if (r.kind != GBG_REQ_INTERPOLATE && r.kind != GBG_REQ_ANTERPOLATE) return set_error(GBG_EARG, "bad request kind");
  if (r.pos_dtype != GBG_F32 && r.pos_dtype != GBG_F64) return set_error(GBG_EARG, "bad position dtype");
  int32_t ncomp = 0, max_width = 0;
  GBG_TRY(gbg::field_info(r.field, grid, &ncomp, &max_width));
  const int w = r.scheme.stencil_width;
  if (w < 2 || w > 8 || w % 2 || r.scheme.num_powers != w)
    return set_error(GBG_EUNSUPPORTED, "served schemes have 2, 4, 6 or 8 nodes and num_powers == stencil_width");
  if (w > max_width) return set_error(GBG_EARG, "the scheme is wider than the field's ghost layer");
  if (r.npoints < 0 || r.npoints > 0x7fffffffLL) return set_error(GBG_EDIM, "point count outside 0..2^31-1");
  if (r.npoints > 0 && !r.positions) return set_error(GBG_EARG, "null positions");
  if (r.npoints > 0 && r.kind == GBG_REQ_INTERPOLATE && !r.out) return set_error(GBG_EARG, "null output");
  if (r.npoints > 0 && r.kind == GBG_REQ_ANTERPOLATE && !r.q) return set_error(GBG_EARG, "null quantities");
  return GBG_OK;
}

double percentile(std::vector<double> v, double p) {
  if (v.empty()) return 0.0;
  std::sort(v.begin(), v.end());
  const double x = p * (double)(v.size() - 1);
  const size_t i = (size_t)x;
  const double f = x - (double)i;
  return i + 1 < v.size() ? v[i] * (1.0 - f) + v[i + 1] * f : v[i];
}

}  // namespace

extern "C" {

gbg_status gbg_server_plan(const int32_t *kinds, const uint64_t *fields, const size_t *bytes, int32_t n,
                           size_t free_bytes, int32_t max_batch, int32_t *run_length) {
  gbg::clear_error();
  if (!run_length || n < 0 || (n > 0 && (!kinds || !fields || !bytes)) || max_batch < 1)
    return set_error(GBG_EARG, "bad plan arguments");
  *run_length = plan_run(kinds, fields, bytes, n, free_bytes, max_batch);
  return GBG_OK;
}

gbg_status gbg_server_create(const gbg_server_config *config, gbg_server *out) {
  gbg::clear_error();
  if (!config || !out) return set_error(GBG_EARG, "null argument");
  gbg_server_config c = *config;
  if (c.slots < 1 || c.slots > 64) return set_error(GBG_EARG, "slots must be 1..64");
  if (c.max_batch < 1 || c.max_batch > 256) return set_error(GBG_EARG, "max_batch must be 1..256");
  if (!(c.timeout_seconds > 0.0)) return set_error(GBG_EARG, "timeout_seconds must be positive");
  for (int d = 0; d < 3; ++d)
    if (c.brick[d] < 0 || c.brick[d] > 64) return set_error(GBG_EARG, "brick edges must be 0..64");
  int dev = 0;
  GBG_CUDA_TRY(cudaGetDevice(&dev));
  if (c.hbm_budget_bytes == 0) {
    size_t free_b = 0, total_b = 0;
    GBG_CUDA_TRY(cudaMemGetInfo(&free_b, &total_b));
    c.hbm_budget_bytes = free_b / 2;
  }
  auto *s = new (std::nothrow) gbg_server_s;
  if (!s) return set_error(GBG_ENOMEM, "host allocation failed");
  s->cfg = c;
  s->device = dev;
  s->slots.resize(c.slots);
  const size_t staging = gbg::batch_table_bytes(c.max_batch);
  for (Slot &sl : s->slots) {
    bool ok = cudaStreamCreateWithFlags(&sl.stream, cudaStreamNonBlocking) == cudaSuccess &&
              cudaEventCreateWithFlags(&sl.done, cudaEventDisableTiming) == cudaSuccess &&
              cudaMalloc(&sl.dev_status, sizeof(int32_t) * (c.max_batch + 1)) == cudaSuccess &&
              cudaMallocHost(&sl.host_status, sizeof(int32_t) * (c.max_batch + 1)) == cudaSuccess &&
              cudaMallocHost(&sl.staging, staging) == cudaSuccess;
    sl.staging_bytes = staging;
    if (!ok) {
      const cudaError_t e = cudaGetLastError();
      gbg_server_destroy(s);
      return set_error(GBG_ECUDA, std::string("server: creating the slots: ") + cudaGetErrorString(e));
    }
    std::memset(sl.host_status, 0, sizeof(int32_t) * (c.max_batch + 1));
  }
  s->worker = std::thread(worker_main, s);
  *out = s;
  return GBG_OK;
}

gbg_status gbg_server_submit(gbg_server s, const gbg_request *request, int64_t *ticket) {
  gbg::clear_error();
  if (!s || !request || !ticket) return set_error(GBG_EARG, "null argument");
  Request rq;
  rq.r = *request;
  GBG_TRY(check_request(rq.r, &rq.grid));
  rq.bytes = gbg::bins_bytes(rq.grid, rq.r.npoints, s->cfg.brick);
  if (rq.bytes == 0) return set_error(GBG_EUNSUPPORTED, "the request's bins cannot be planned");
  std::lock_guard<std::mutex> lk(s->mu);
  if (rq.bytes > s->cfg.hbm_budget_bytes)
    return set_error(GBG_EBUSY, "the request needs " + std::to_string(rq.bytes) +
                                    " bytes of device memory, more than the server's budget of " +
                                    std::to_string(s->cfg.hbm_budget_bytes));
  if (s->stop) return set_error(GBG_EBUSY, "the server is stopping");
  rq.ticket = s->next_ticket++;
  rq.submitted = Clock::now();
  if (!s->have_first) {
    s->have_first = true;
    s->first_submit = seconds_since(s->t0, rq.submitted);
  }
  ++s->submitted;
  s->queue.push_back(rq);
  *ticket = rq.ticket;
  s->cv_work.notify_one();
  return GBG_OK;
}

gbg_status gbg_server_wait(gbg_server s, int64_t ticket, double timeout_seconds, gbg_status *result) {
  gbg::clear_error();
  if (!s || !result) return set_error(GBG_EARG, "null argument");
  std::unique_lock<std::mutex> lk(s->mu);
  if (ticket < 1 || ticket >= s->next_ticket) return set_error(GBG_EARG, "unknown ticket");
  const auto until = Clock::now() + std::chrono::duration_cast<Clock::duration>(
                                        std::chrono::duration<double>(std::max(0.0, timeout_seconds)));
  while (true) {
    auto it = s->results.find(ticket);
    if (it != s->results.end()) {
      *result = it->second;
      s->results.erase(it);
      return GBG_OK;
    }
    bool pending = false;
    for (const Request &rq : s->queue) pending = pending || rq.ticket == ticket;
    for (const Slot &sl : s->slots)
      for (const Request &rq : sl.reqs) pending = pending || (sl.busy && !sl.expired && rq.ticket == ticket);
    if (!pending) return set_error(GBG_EARG, "ticket already waited for");
    if (s->cv_done.wait_until(lk, until) == std::cv_status::timeout && Clock::now() >= until)
      return set_error(GBG_ETIMEOUT, "the request is still pending");
  }
}

gbg_status gbg_server_drain(gbg_server s, double timeout_seconds) {
  gbg::clear_error();
  if (!s) return set_error(GBG_EARG, "null server");
  std::unique_lock<std::mutex> lk(s->mu);
  const auto until = Clock::now() + std::chrono::duration_cast<Clock::duration>(
                                        std::chrono::duration<double>(std::max(0.0, timeout_seconds)));
  while (true) {
    bool busy = !s->queue.empty();
    for (const Slot &sl : s->slots) busy = busy || sl.busy;
    if (!busy) return GBG_OK;
    if (s->cv_done.wait_until(lk, until) == std::cv_status::timeout && Clock::now() >= until)
      return set_error(GBG_ETIMEOUT, "requests still queued or in flight");
  }
}

gbg_status gbg_server_stats(gbg_server s, int32_t reset, gbg_server_counters *out) {
  gbg::clear_error();
  if (!s || !out) return set_error(GBG_EARG, "null argument");
  std::lock_guard<std::mutex> lk(s->mu);
  gbg_server_counters r{};
  r.submitted = s->submitted;
  r.completed = s->completed;
  r.failed = s->failed;
  r.queued = (int64_t)s->queue.size();
  r.in_flight = s->in_flight_requests();
  r.runs = s->runs;
  r.points = s->points;
  r.p50_ms = percentile(s->latencies_ms, 0.50);
  r.p99_ms = percentile(s->latencies_ms, 0.99);
  double sum = 0.0, mx = 0.0;
  for (double v : s->latencies_ms) {
    sum += v;
    mx = std::max(mx, v);
  }
  r.mean_ms = s->latencies_ms.empty() ? 0.0 : sum / (double)s->latencies_ms.size();
  r.max_ms = mx;
  r.first_submit_s = s->first_submit;
  r.last_done_s = s->last_done;
  r.hbm_in_use = s->in_use;
  r.hbm_peak = s->peak;
  r.hbm_budget = s->cfg.hbm_budget_bytes;
  *out = r;
  if (reset) {
    s->submitted = s->completed = s->failed = s->runs = s->points = 0;
    s->latencies_ms.clear();
    s->have_first = false;
    s->first_submit = s->last_done = 0.0;
    s->peak = s->in_use;
  }
  return GBG_OK;
}

gbg_status gbg_server_inject(gbg_server s, int32_t fault, int32_t count) {
  gbg::clear_error();
  if (!s || count < 0) return set_error(GBG_EARG, "bad argument");
  std::lock_guard<std::mutex> lk(s->mu);
  if (fault == GBG_FAULT_ALLOC) s->fault_alloc = count;
  else if (fault == GBG_FAULT_DEADLINE) s->fault_deadline = count;
  else return set_error(GBG_EARG, "unknown fault");
  return GBG_OK;
}

gbg_status gbg_server_destroy(gbg_server s) {
  gbg::clear_error();
  if (!s) return GBG_OK;
  gbg_status st = GBG_OK;
  if (s->worker.joinable()) {
    // the worker finishes the queue; bound the wait by the run deadline
    gbg_server_drain(s, std::max(1.0, 4.0 * s->cfg.timeout_seconds));
    {
      std::lock_guard<std::mutex> lk(s->mu);
      s->stop = true;
      s->cv_work.notify_all();
    }
    s->worker.join();
  }
  bool stuck = false;
  for (Slot &sl : s->slots) {
    if (sl.busy) {
      stuck = true;  // device work never finished: leave its memory alone
      continue;
    }
    if (sl.done) cudaEventDestroy(sl.done);
    if (sl.stream) cudaStreamDestroy(sl.stream);
    if (sl.dev_status) cudaFree(sl.dev_status);
    if (sl.host_status) cudaFreeHost(sl.host_status);
    if (sl.staging) cudaFreeHost(sl.staging);
  }
  if (!stuck) {
    for (auto &kv : s->deps) {
      if (kv.second.last_write) cudaEventDestroy(kv.second.last_write);
      for (cudaEvent_t e : kv.second.reads) cudaEventDestroy(e);
    }
    for (cudaEvent_t e : s->event_pool) cudaEventDestroy(e);
    delete s;
  } else {
    st = set_error(GBG_ETIMEOUT, "server: device work still in flight at destruction; its memory was not freed");
  }
  return st;
}

}  // extern "C"
