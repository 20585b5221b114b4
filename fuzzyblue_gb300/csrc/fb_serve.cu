// fb_serve.cu — request loop for precompute jobs: HBM-budget admission,
// concurrent batches on separate streams (continuous batching), and a
// device-resident LRU cache of finished tables (fb_server_* in
// include/fuzzyblue.h).
//
// One scheduler thread owns every CUDA call of the server. Each pass of its
// loop (1) collects finished batches (a host callback after each batch wakes
// it), moving their tables into the resident cache and freeing their
// temporaries; (2) while a stream is free, picks the request that leads its
// batch - on a high-priority stream the oldest cheap request, on a
// low-priority stream the oldest request of any class, an expensive one only
// while no other expensive batch runs - adds the queued
// requests of the lead's table class in arrival order while the budget
// (evicting unpinned resident tables, least recently used first) and the
// batch's estimated duration allow, and launches them as one batch build
// whose CTAs exit after a few work items, so that a cheap batch's kernels
// are dispatched ahead of a long build already running; while a long build
// has run well past its estimated duration, cheap batches keep to the
// low-priority streams beside it, and a request queued for over a second
// leads the next batch on any stream; (3) sleeps until woken.
// Requests for parameters already resident or in flight share that result.
#include <cuda_runtime.h>

#include <algorithm>
#include <atomic>
#include <chrono>
#include <condition_variable>
#include <cstring>
#include <deque>
#include <mutex>
#include <string>
#include <thread>
#include <unordered_map>
#include <vector>

#include "../../include/fuzzyblue.h"
#include "fb_internal.h"

namespace {

// Work items a CTA of a served build takes before it exits.
constexpr int kServeItemsPerCta = 2;

double now_ms() {
  using namespace std::chrono;
  return duration<double, std::milli>(steady_clock::now().time_since_epoch()).count();
}

struct Entry {
  std::string key;
  fb_atmosphere* atm = nullptr;  // set when ready
  size_t out_bytes = 0;
  int pins = 0;
  uint64_t last_use = 0;
  bool ready = false;
  std::vector<uint64_t> waiters;  // tickets completed by this entry
};

enum class State { Queued, Running, Done, Cancelled, Failed };

struct Request {
  fb_params params;
  std::string key;
  State state = State::Queued;
  double t_submit = 0, t_done = 0;
  Entry* entry = nullptr;
  bool pinned = false;
  int status = FB_OK;
  size_t need = 0;  // outputs + temporaries
};

struct Batch {
  fb_pending* pending = nullptr;
  int stream_slot = -1;
  std::vector<Entry*> entries;
  size_t bytes = 0;
  double cost = 0;      // texel-orders
  double t_launch = 0;  // ms
  bool expensive = false;  // led by a request above the cheap threshold
  bool has_callback = false;      // completion is signalled by the host callback
  std::atomic<bool> done{false};  // set by that callback as its last action
};

// Cache key: the parameter bytes with every padding and reserved field zeroed.
std::string key_of(const fb_params& p) {
  fb_params c = p;
  std::memset(c.reserved, 0, sizeof(c.reserved));
  c.raw._pad0 = 0;
  fb_density_profile* prof[3] = {&c.raw.rayleigh_density, &c.raw.mie_density, &c.raw.absorption_density};
  for (fb_density_profile* q : prof)
    for (auto& L : q->layers) std::memset(L._pad, 0, sizeof(L._pad));
  return std::string(reinterpret_cast<const char*>(&c), sizeof(c));
}

}  // namespace

struct fb_server {
  fb_builder* b = nullptr;
  fb_server_config cfg;
  std::mutex mu;
  std::condition_variable cv;       // wakes the scheduler
  std::condition_variable cv_done;  // wakes waiters
  std::thread th;
  bool stop = false;
  std::deque<uint64_t> queue;
  std::deque<uint64_t> finished;  // tickets completed or failed, not yet taken by fb_server_completed
  std::unordered_map<uint64_t, Request> reqs;
  std::unordered_map<std::string, Entry*> entries;
  std::vector<Batch*> inflight;
  std::vector<cudaStream_t> streams;
  std::vector<bool> stream_busy;
  std::vector<bool> stream_high;  // high-priority stream (cheap batches)
  size_t resident_bytes = 0, inflight_bytes = 0;
  double rate = 0;  // best texel-orders per ms seen over a finished batch (0: none yet)
  uint64_t next_ticket = 1, clock = 0;
  fb_server_stats st;
  std::vector<double> lat;
  double batched_atmospheres = 0;
};

namespace {

void complete_request(fb_server* s, uint64_t t, Entry* e) {
  auto it = s->reqs.find(t);
  if (it == s->reqs.end() || it->second.state == State::Cancelled) return;
  Request& r = it->second;
  r.state = State::Done;
  r.entry = e;
  r.pinned = true;
  e->pins++;
  e->last_use = ++s->clock;
  r.t_done = now_ms();
  s->lat.push_back(r.t_done - r.t_submit);
  s->st.completed++;
  s->finished.push_back(t);
  s->cv_done.notify_all();
}

void fail_request(fb_server* s, uint64_t t, int status) {
  auto it = s->reqs.find(t);
  if (it == s->reqs.end()) return;
  it->second.state = State::Failed;
  it->second.status = status;
  s->finished.push_back(t);
  s->cv_done.notify_all();
}

// Frees unpinned resident tables, least recently used first, until `need`
// more bytes fit in the budget (or until the entry count is within limits).
void evict(fb_server* s, size_t need, bool for_count) {
  while (true) {
    const bool over_bytes = s->resident_bytes + s->inflight_bytes + need > s->cfg.hbm_budget_bytes;
    size_t nready = 0;
    for (auto& kv : s->entries)
      if (kv.second->ready) ++nready;
    const bool over_count = for_count && nready > s->cfg.cache_entries;
    if (!over_bytes && !over_count) return;
    Entry* victim = nullptr;
    for (auto& kv : s->entries) {
      Entry* e = kv.second;
      if (e->ready && e->pins == 0 && (!victim || e->last_use < victim->last_use)) victim = e;
    }
    if (!victim) return;
    fbi::atmosphere_free(victim->atm);
    s->resident_bytes -= victim->out_bytes;
    s->entries.erase(victim->key);
    delete victim;
    s->st.evictions++;
  }
}

// Runs on a CUDA driver thread when the batch's stream reaches it. The batch
// (and with it the server) stays alive until `done` is set, so storing it is
// the callback's last access to either.
void CUDART_CB on_batch_done(void* arg) {
  auto* pair = static_cast<std::pair<fb_server*, Batch*>*>(arg);
  fb_server* s = pair->first;
  Batch* bt = pair->second;
  delete pair;
  s->cv.notify_all();
  bt->done.store(true);
}

void collect(fb_server* s) {
  for (size_t i = 0; i < s->inflight.size();) {
    Batch* bt = s->inflight[i];
    bool finished = bt->done.load();
    if (!bt->has_callback && !finished) {
      finished = cudaEventQuery(fbi::pending_event(bt->pending)) == cudaSuccess;
      if (!finished) cudaGetLastError();
    }
    if (!finished) {
      ++i;
      continue;
    }
    for (size_t k = 0; k < bt->entries.size(); ++k) {
      Entry* e = bt->entries[k];
      e->atm = fbi::pending_detach(bt->pending, (uint32_t)k);
      e->ready = true;
      s->resident_bytes += e->out_bytes;
      for (uint64_t t : e->waiters) complete_request(s, t, e);
      e->waiters.clear();
    }
    s->inflight_bytes -= bt->bytes;
    const double took = now_ms() - bt->t_launch;
    if (took > 0) s->rate = std::max(s->rate, bt->cost / took);
    fbi::pending_destroy(bt->pending);
    s->stream_busy[bt->stream_slot] = false;
    delete bt;
    s->inflight.erase(s->inflight.begin() + i);
    s->cv_done.notify_all();
  }
  evict(s, 0, true);
}

// Work of one request in texel-orders (scattering texels x orders): the
// scheduler's cost estimate.
double cost_of(const fb_params& p) {
  const fb_params_raw& r = p.raw;
  return (double)r.scattering_r_size * r.scattering_mu_size * r.scattering_mu_s_size * r.scattering_nu_size *
         std::max(1u, p.order);
}
// Requests that share a batch: the same table class (scattering sizes) and
// precision, so that a cheap request never waits for an expensive one.
bool same_class(const fb_params& a, const fb_params& b) {
  return a.raw.scattering_r_size == b.raw.scattering_r_size && a.raw.scattering_mu_size == b.raw.scattering_mu_size &&
         a.raw.scattering_mu_s_size == b.raw.scattering_mu_s_size &&
         a.raw.scattering_nu_size == b.raw.scattering_nu_size && a.precision == b.precision;
}
// Batches up to this cost (texel-orders) run on the high-priority streams.
constexpr double kCheapBatch = 1048576.0 * 8;
// Starvation guard: a batch on a low-priority stream that has run longer than
// kStarveFactor times its estimated duration (its cost at the best throughput
// seen so far) plus kStarveSlackMs holds new cheap batches off the
// high-priority streams until it finishes; they then share the low-priority
// streams with it, where the block scheduler serves kernels in launch order.
constexpr double kStarveFactor = 2.0;
constexpr double kStarveSlackMs = 20.0;
constexpr double kInitialRate = 1.0e6;  // texel-orders per ms before any batch finished
// A batch takes further requests only while its estimated duration stays
// under this: one atmosphere of the default class already fills the GPU, so
// larger batches gain little throughput while every request in them waits
// for the whole batch.
constexpr double kBatchTargetMs = 100.0;

bool low_priority_starved(const fb_server* s, double now) {
  const double rate = s->rate > 0 ? s->rate : kInitialRate;
  for (const Batch* bt : s->inflight)
    if (!s->stream_high[bt->stream_slot] && now - bt->t_launch > kStarveFactor * bt->cost / rate + kStarveSlackMs)
      return true;
  return false;
}

// Answers a queued request from a resident or in-flight result with the same
// parameters; true if there was one.
bool share_result(fb_server* s, uint64_t t, Request& r) {
  auto ex = s->entries.find(r.key);
  if (ex == s->entries.end()) return false;
  s->st.cache_hits++;
  if (ex->second->ready) complete_request(s, t, ex->second);
  else {
    r.state = State::Running;
    ex->second->waiters.push_back(t);
  }
  return true;
}

// Queue entries looked at for the request that leads a batch.
constexpr size_t kLeadScan = 4096;
// Aging: a request queued longer than this leads the next batch on any free
// stream, whatever its class. Under overload this serves the queue in
// arrival order, so that cheap requests cannot hold an expensive one back
// without bound; at moderate load no request waits that long.
constexpr double kUrgentMs = 1000.0;

// Picks a free stream and the request that leads its batch: a high-priority
// stream takes the oldest cheap request (none while a long batch is held
// back), a low-priority stream the oldest request of any class; with no
// low-priority stream at all the high-priority ones take everything. The
// oldest request, once urgent (kUrgentMs), takes any free stream.
// Drops cancelled and shared entries met on the way. `cheap_only`: the batch
// may hold cheap requests only.
bool pick_lead(fb_server* s, int& slot, uint64_t& lead, bool& cheap_only) {
  int free_high = -1, free_low = -1;
  bool any_low = false;
  for (size_t k = 0; k < s->streams.size(); ++k) {
    any_low |= !s->stream_high[k];
    if (s->stream_busy[k]) continue;
    if (s->stream_high[k]) {
      if (free_high < 0) free_high = (int)k;
    } else if (free_low < 0) {
      free_low = (int)k;
    }
  }
  if (free_high < 0 && free_low < 0) return false;
  const double now = now_ms();
  const bool high_for_all = !any_low;
  const bool hold_high = !high_for_all && low_priority_starved(s, now);
  // one expensive batch at a time: it fills the GPU alone, and a second one
  // beside it would only stretch both (they run in arrival order instead)
  bool expensive_running = false;
  for (const Batch* bt : s->inflight) expensive_running |= bt->expensive;
  size_t seen = 0;
  bool oldest = true;
  for (auto qi = s->queue.begin(); qi != s->queue.end() && seen < kLeadScan;) {
    const uint64_t t = *qi;
    auto it = s->reqs.find(t);
    if (it == s->reqs.end() || it->second.state != State::Queued) {
      qi = s->queue.erase(qi);
      continue;
    }
    if (share_result(s, t, it->second)) {
      qi = s->queue.erase(qi);
      continue;
    }
    if (oldest && now - it->second.t_submit > kUrgentMs) {
      slot = free_high >= 0 ? free_high : free_low;
      lead = t;
      cheap_only = false;
      return true;
    }
    oldest = false;
    if (free_low < 0 && hold_high) return false;
    const bool cheap = cost_of(it->second.params) <= kCheapBatch;
    if (free_high >= 0 && (high_for_all || (cheap && !hold_high))) {
      slot = free_high;
      lead = t;
      cheap_only = !high_for_all;
      return true;
    }
    if (free_low >= 0 && (cheap || high_for_all || !expensive_running)) {
      slot = free_low;
      lead = t;
      cheap_only = false;
      return true;
    }
    ++qi;
    ++seen;
  }
  return false;
}

void admit(fb_server* s) {
  int slot;
  uint64_t lead;
  bool cheap_only;
  while (pick_lead(s, slot, lead, cheap_only)) {
    // the lead request, then the queued requests of its class in arrival
    // order (shared results are settled as they are met)
    const fb_params head = s->reqs[lead].params;
    const double cost_cap = kBatchTargetMs * (s->rate > 0 ? s->rate : kInitialRate);
    Batch* bt = new Batch();
    std::vector<fb_params> params;
    size_t bytes = 0;
    double cost = 0;
    bool full = false;
    for (auto qi = s->queue.begin(); qi != s->queue.end() && params.size() < s->cfg.max_batch && !full;) {
      const uint64_t t = *qi;
      auto it = s->reqs.find(t);
      if (it == s->reqs.end() || it->second.state != State::Queued) {
        qi = s->queue.erase(qi);
        continue;
      }
      Request& r = it->second;
      if (!same_class(r.params, head) || (cheap_only && cost_of(r.params) > kCheapBatch)) {
        ++qi;
        continue;
      }
      if (share_result(s, t, r)) {  // resident or in flight: share it
        qi = s->queue.erase(qi);
        continue;
      }
      if (!params.empty() && cost + cost_of(r.params) > cost_cap) break;
      if (s->resident_bytes + s->inflight_bytes + bytes + r.need > s->cfg.hbm_budget_bytes) {
        evict(s, bytes + r.need, false);
        if (s->resident_bytes + s->inflight_bytes + bytes + r.need > s->cfg.hbm_budget_bytes) {
          full = true;
          break;
        }
      }
      Entry* e = new Entry();
      e->key = r.key;
      e->out_bytes = fbi::sizes_of(r.params).out_bytes;
      e->waiters.push_back(t);
      s->entries[r.key] = e;
      bt->entries.push_back(e);
      params.push_back(r.params);
      bytes += r.need;
      cost += cost_of(r.params);
      r.state = State::Running;
      qi = s->queue.erase(qi);
    }
    if (params.empty()) {
      delete bt;
      return;
    }
    int rc = fbi::build(s->b, s->streams[slot], params.data(), (uint32_t)params.size(), true, &bt->pending,
                        kServeItemsPerCta);
    if (rc != FB_OK) {
      for (size_t k = 0; k < bt->entries.size(); ++k) {
        Entry* e = bt->entries[k];
        for (uint64_t t : e->waiters) fail_request(s, t, rc);
        s->entries.erase(e->key);
        delete e;
      }
      delete bt;
      s->cv_done.notify_all();
      return;
    }
    bt->stream_slot = slot;
    bt->bytes = bytes;
    bt->cost = cost;
    bt->t_launch = now_ms();
    bt->expensive = cost_of(head) > kCheapBatch;
    s->stream_busy[slot] = true;
    s->inflight_bytes += bytes;
    s->inflight.push_back(bt);
    s->st.batches++;
    s->batched_atmospheres += (double)params.size();
    auto* arg = new std::pair<fb_server*, Batch*>(s, bt);
    if (cudaLaunchHostFunc(s->streams[slot], on_batch_done, arg) == cudaSuccess) {
      bt->has_callback = true;
    } else {
      cudaGetLastError();
      delete arg;  // completion is then found by polling the batch's event
    }
  }
}

void loop(fb_server* s) {
  cudaSetDevice(fbi::builder_device(s->b));
  std::unique_lock<std::mutex> g(s->mu);
  while (!s->stop || !s->inflight.empty()) {
    collect(s);
    if (!s->stop) admit(s);
    s->cv.wait_for(g, std::chrono::milliseconds(2));
  }
}

int fail_srv(int code, const char* msg) { return fbi::set_error(code, msg); }

}  // namespace

extern "C" void fb_server_config_default(fb_server_config* c) {
  if (!c) return;
  std::memset(c, 0, sizeof(*c));
  c->hbm_budget_bytes = 120ull << 30;
  c->max_batch = 64;
  c->max_inflight = 4;
  c->cache_entries = 4096;
  c->max_queue = 65536;
}

extern "C" int fb_server_create(fb_builder* b, const fb_server_config* cfg, fb_server** out) {
  if (!b || !out) return fail_srv(FB_ERR_INVALID_ARGUMENT, "NULL argument");
  *out = nullptr;
  fb_server* s = new fb_server();
  fb_server_config_default(&s->cfg);
  if (cfg) s->cfg = *cfg;
  if (s->cfg.max_batch == 0) s->cfg.max_batch = 1;
  if (s->cfg.max_inflight == 0) s->cfg.max_inflight = 1;
  std::memset(&s->st, 0, sizeof(s->st));
  if (cudaSetDevice(fbi::builder_device(b)) != cudaSuccess) {
    delete s;
    return fail_srv(FB_ERR_CUDA, "cudaSetDevice failed");
  }
  // Half the streams (at least one) at the device's highest priority for
  // cheap batches, the rest at the lowest: with CTAs that exit after a few
  // work items, the block scheduler serves a cheap request's kernels ahead of
  // an expensive build already running.
  int prio_low = 0, prio_high = 0;
  if (cudaDeviceGetStreamPriorityRange(&prio_low, &prio_high) != cudaSuccess) {
    cudaGetLastError();
    prio_low = prio_high = 0;
  }
  const uint32_t n_high = std::max(1u, s->cfg.max_inflight / 2);
  for (uint32_t k = 0; k < s->cfg.max_inflight; ++k) {
    cudaStream_t st;
    const bool high = k < n_high;
    if (cudaStreamCreateWithPriority(&st, cudaStreamNonBlocking, high ? prio_high : prio_low) != cudaSuccess) {
      for (cudaStream_t x : s->streams) cudaStreamDestroy(x);
      delete s;
      return fail_srv(FB_ERR_CUDA, "cudaStreamCreate failed");
    }
    s->streams.push_back(st);
    s->stream_busy.push_back(false);
    s->stream_high.push_back(high);
  }
  s->b = b;
  fbi::builder_ref(b);
  s->th = std::thread(loop, s);
  *out = s;
  return FB_OK;
}

extern "C" int fb_server_submit(fb_server* s, const fb_params* p, uint64_t* ticket) {
  if (!s || !p || !ticket) return fail_srv(FB_ERR_INVALID_ARGUMENT, "NULL argument");
  int rc = fb_params_validate(p);
  if (rc) return rc;
  const fbi::TableSizes z = fbi::sizes_of(*p);
  std::lock_guard<std::mutex> g(s->mu);
  if (s->stop) return fail_srv(FB_ERR_SHUTDOWN, "server is shutting down");
  if (z.out_bytes + z.tmp_bytes > s->cfg.hbm_budget_bytes) {
    s->st.rejected++;
    return fail_srv(FB_ERR_BUDGET, "request larger than the HBM budget");
  }
  if (s->queue.size() >= s->cfg.max_queue) {
    s->st.rejected++;
    return fail_srv(FB_ERR_BUDGET, "request queue is full");
  }
  const uint64_t t = s->next_ticket++;
  Request& r = s->reqs[t];
  r.params = *p;
  r.key = key_of(*p);
  r.t_submit = now_ms();
  r.need = z.out_bytes + z.tmp_bytes;
  s->st.submitted++;
  auto ex = s->entries.find(r.key);
  if (ex != s->entries.end()) {
    s->st.cache_hits++;
    if (ex->second->ready) {
      complete_request(s, t, ex->second);
      s->cv_done.notify_all();
    } else {
      r.state = State::Running;
      ex->second->waiters.push_back(t);
    }
  } else {
    s->queue.push_back(t);
    s->cv.notify_all();
  }
  *ticket = t;
  return FB_OK;
}

namespace {
int poll_locked(fb_server* s, uint64_t t, fb_atmosphere** out) {
  auto it = s->reqs.find(t);
  if (it == s->reqs.end()) return fail_srv(FB_ERR_NOT_FOUND, "unknown ticket");
  Request& r = it->second;
  switch (r.state) {
    case State::Done:
      r.entry->last_use = ++s->clock;
      if (out) *out = r.entry->atm;
      return FB_OK;
    case State::Cancelled:
      return FB_ERR_CANCELLED;
    case State::Failed:
      return r.status;
    default:
      return FB_NOT_READY;
  }
}
}  // namespace

extern "C" int fb_server_poll(fb_server* s, uint64_t t, fb_atmosphere** out) {
  if (!s) return fail_srv(FB_ERR_INVALID_ARGUMENT, "server is NULL");
  std::lock_guard<std::mutex> g(s->mu);
  return poll_locked(s, t, out);
}

extern "C" int fb_server_wait(fb_server* s, uint64_t t, uint32_t timeout_ms, fb_atmosphere** out) {
  if (!s) return fail_srv(FB_ERR_INVALID_ARGUMENT, "server is NULL");
  std::unique_lock<std::mutex> g(s->mu);
  const auto deadline = std::chrono::steady_clock::now() + std::chrono::milliseconds(timeout_ms);
  while (true) {
    int rc = poll_locked(s, t, out);
    if (rc != FB_NOT_READY) return rc;
    if (timeout_ms == UINT32_MAX) s->cv_done.wait(g);
    else if (s->cv_done.wait_until(g, deadline) == std::cv_status::timeout) return poll_locked(s, t, out);
  }
}

extern "C" int fb_server_completed(fb_server* s, uint64_t* tickets, uint32_t capacity, uint32_t timeout_ms,
                                   uint32_t* count) {
  if (!s || !count || (!tickets && capacity)) return fail_srv(FB_ERR_INVALID_ARGUMENT, "NULL argument");
  std::unique_lock<std::mutex> g(s->mu);
  if (s->finished.empty() && timeout_ms) {
    auto ready = [&] { return !s->finished.empty() || s->stop; };
    if (timeout_ms == UINT32_MAX) {
      s->cv_done.wait(g, ready);
    } else {
      s->cv_done.wait_until(g, std::chrono::steady_clock::now() + std::chrono::milliseconds(timeout_ms), ready);
    }
  }
  uint32_t n = 0;
  while (n < capacity && !s->finished.empty()) {
    tickets[n++] = s->finished.front();
    s->finished.pop_front();
  }
  *count = n;
  return FB_OK;
}

extern "C" int fb_server_release(fb_server* s, uint64_t t) {
  if (!s) return fail_srv(FB_ERR_INVALID_ARGUMENT, "server is NULL");
  std::lock_guard<std::mutex> g(s->mu);
  auto it = s->reqs.find(t);
  if (it == s->reqs.end()) return fail_srv(FB_ERR_NOT_FOUND, "unknown ticket");
  Request& r = it->second;
  if (r.state == State::Queued || r.state == State::Running) return FB_NOT_READY;
  if (r.pinned && r.entry) r.entry->pins--;
  s->reqs.erase(it);
  s->cv.notify_all();
  return FB_OK;
}

extern "C" int fb_server_cancel(fb_server* s, uint64_t t) {
  if (!s) return fail_srv(FB_ERR_INVALID_ARGUMENT, "server is NULL");
  std::lock_guard<std::mutex> g(s->mu);
  auto it = s->reqs.find(t);
  if (it == s->reqs.end()) return fail_srv(FB_ERR_NOT_FOUND, "unknown ticket");
  Request& r = it->second;
  if (r.state == State::Queued) {
    r.state = State::Cancelled;
    s->st.cancelled++;
    s->cv_done.notify_all();
    return FB_OK;
  }
  if (r.state == State::Running) return FB_NOT_READY;
  return fail_srv(FB_ERR_NOT_FOUND, "request already finished");
}

extern "C" int fb_server_get_stats(fb_server* s, fb_server_stats* out) {
  if (!s || !out) return fail_srv(FB_ERR_INVALID_ARGUMENT, "NULL argument");
  std::lock_guard<std::mutex> g(s->mu);
  fb_server_stats o = s->st;
  o.resident_bytes = s->resident_bytes;
  o.inflight_bytes = s->inflight_bytes;
  uint64_t q = 0;
  for (uint64_t t : s->queue) {
    auto it = s->reqs.find(t);
    if (it != s->reqs.end() && it->second.state == State::Queued) ++q;
  }
  o.queued = q;
  if (!s->lat.empty()) {
    std::vector<double> v = s->lat;
    std::sort(v.begin(), v.end());
    auto at = [&](double f) { return v[std::min(v.size() - 1, (size_t)(f * (v.size() - 1) + 0.5))]; };
    o.p50_ms = at(0.50);
    o.p99_ms = at(0.99);
    double sum = 0;
    for (double x : v) sum += x;
    o.mean_ms = sum / v.size();
  }
  o.mean_batch = s->st.batches ? s->batched_atmospheres / s->st.batches : 0.0;
  *out = o;
  return FB_OK;
}

extern "C" void fb_server_destroy(fb_server* s) {
  if (!s) return;
  {
    std::lock_guard<std::mutex> g(s->mu);
    s->stop = true;
    for (auto& kv : s->reqs)
      if (kv.second.state == State::Queued) kv.second.state = State::Cancelled;
    s->queue.clear();
  }
  s->cv.notify_all();
  s->cv_done.notify_all();
  if (s->th.joinable()) s->th.join();
  cudaSetDevice(fbi::builder_device(s->b));
  for (auto& kv : s->entries) {
    if (kv.second->atm) fbi::atmosphere_free(kv.second->atm);
    delete kv.second;
  }
  for (cudaStream_t st : s->streams) {
    cudaStreamSynchronize(st);
    cudaStreamDestroy(st);
  }
  fbi::builder_unref(s->b);
  delete s;
}
