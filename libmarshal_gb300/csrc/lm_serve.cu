// lm_serve.cu -- a conversion server: requests arrive one at a time, are
// admitted under an HBM budget and run in batches that start as soon as a
// lane has room (continuous batching).
//
// No reference counterpart: the reference converts one buffer per blocking
// call (src/cl_marshal.cc:561-818).  Here a worker thread owns the GPU side:
//  * admission: a request is admitted while the payload bytes of admitted,
//    unfinished requests stay within the budget (FIFO: a request that does
//    not fit waits, and so do the ones behind it).  Requests whose data is on
//    the host are staged through a device pool of the budget's size;
//  * lanes: requests are sorted by payload into three lanes (small, medium,
//    large) with up to kSlots batches in flight each; every slot has its own
//    stream (small lanes at the highest priority) and lm_batch_t, so a long
//    conversion does not hold back short ones and batches overlap;
//  * batching: when a lane has a free slot, every admitted request queued on
//    it (up to the lane's batch limits) becomes one lm_batch_run;
//  * completion: a host function enqueued after each batch stamps the time
//    and wakes the worker, which releases the budget and reports the
//    request (latency = completion - submission).
#include <algorithm>
#include <atomic>
#include <chrono>
#include <condition_variable>
#include <cstdio>
#include <cstring>
#include <deque>
#include <map>
#include <mutex>
#include <string>
#include <thread>
#include <vector>

#include "lm_internal.h"
#include "../../include/lm_marshal.h"

namespace {

using Clock = std::chrono::steady_clock;

int64_t now_ns() {
  return std::chrono::duration_cast<std::chrono::nanoseconds>(
             Clock::now().time_since_epoch())
      .count();
}

constexpr int kLanes = 3;
constexpr int kSlots = 2;
// lane by payload: <= 2 MiB, <= 64 MiB, larger
constexpr uint64_t kLaneLimit[kLanes - 1] = {2ull << 20, 64ull << 20};
// batch limits per lane: requests and payload bytes; staging arena of each
// slot's batch handle
constexpr size_t kLaneMaxReqs[kLanes] = {4096, 256, 4};
constexpr uint64_t kLaneMaxBytes[kLanes] = {1ull << 30, 4ull << 30, 8ull << 30};
constexpr uint64_t kLaneArena[kLanes] = {1ull << 30, 2ull << 30, 4ull << 30};

struct SReq {
  uint64_t ticket = 0;
  lm_request r{};
  lm_job job{};
  uint64_t bytes = 0;
  bool host = false;      // staged through the pool
  uint64_t pool_off = 0;  // host mode: where in the pool
  int64_t t_submit = 0, t_admit = 0;
  int lane = 0;
};

struct Slot {
  cudaStream_t stream = nullptr;  // batches of different slots overlap
  lm_batch_t batch = nullptr;
  std::vector<SReq> reqs;
  std::vector<lm_job> jobs;
  std::atomic<int> done{0};
  std::atomic<int64_t> t_done{0};
  bool busy = false;
  int status = 0;
  std::condition_variable *wake = nullptr;  // the server's
};

struct Lane {
  std::deque<SReq> queue;  // admitted, waiting for a slot
  Slot slots[kSlots];
};

// First-fit allocator over [0, size) with 256-byte granules.
class PoolAlloc {
 public:
  void reset(uint64_t size) {
    free_.clear();
    if (size) free_[0] = size;
  }
  bool alloc(uint64_t bytes, uint64_t *off) {
    const uint64_t need = (bytes + 255) / 256 * 256;
    for (auto it = free_.begin(); it != free_.end(); ++it) {
      if (it->second >= need) {
        *off = it->first;
        const uint64_t rest = it->second - need, at = it->first + need;
        free_.erase(it);
        if (rest) free_[at] = rest;
        return true;
      }
    }
    return false;
  }
  void release(uint64_t off, uint64_t bytes) {
    uint64_t size = (bytes + 255) / 256 * 256;
    auto next = free_.lower_bound(off);
    if (next != free_.end() && off + size == next->first) {
      size += next->second;
      next = free_.erase(next);
    }
    if (next != free_.begin()) {
      auto prev = std::prev(next);
      if (prev->first + prev->second == off) {
        prev->second += size;
        return;
      }
    }
    free_[off] = size;
  }

 private:
  std::map<uint64_t, uint64_t> free_;
};

uint64_t payload_of(const lm_request &r) {
  const long long d[4] = {r.d0, r.d1, r.d2, r.d3};
  for (int k = 0; k < 4; ++k)
    if (d[k] < 0) return 0;
  uint64_t n = 0;
  switch (r.op) {
    case LM_OP_0100: n = (uint64_t)d[0] * d[1] * d[2] * d[3]; break;
    case LM_OP_010:
    case LM_OP_100: n = (uint64_t)d[0] * d[1] * d[2]; break;
    default: n = (uint64_t)d[0] * d[1]; break;
  }
  return n * (uint64_t)r.elem_bytes;
}

}  // namespace

struct lm_serve_st {
  int device = 0;
  uint64_t budget = 0;
  // shared with the API calls, under mu
  std::mutex mu;
  std::condition_variable cv;
  std::deque<SReq> incoming;  // submitted, not yet seen by the worker
  std::vector<lm_serve_done> finished;
  uint64_t next_ticket = 1;
  bool stop = false;
  std::string error;
  lm_serve_stats stats{};
  // owned by the worker thread
  std::deque<SReq> waiting;  // seen, not admitted
  Lane lanes[kLanes];
  uint64_t inflight = 0;  // payload bytes admitted and not finished
  char *pool = nullptr;   // host staging pool (on the first host request)
  PoolAlloc palloc;
  std::vector<lm_serve_done> done_local;
  std::thread worker;

  void run();
  void launch(Lane &ln, Slot &sl);
  void finish(Slot &sl);
};

static void CUDART_CB slot_done(void *p) {
  Slot *sl = static_cast<Slot *>(p);
  sl->t_done.store(now_ns());
  sl->done.store(1);
  sl->wake->notify_one();
}

// Enqueues one batch (every CUDA call here is asynchronous).
void lm_serve_st::launch(Lane &ln, Slot &sl) {
  sl.jobs.clear();
  for (SReq &q : sl.reqs) {
    if (q.host) {
      q.job.buf = pool + q.pool_off;
      cudaMemcpyAsync(q.job.buf, q.r.src, q.bytes, cudaMemcpyHostToDevice,
                      sl.stream);
    }
    sl.jobs.push_back(q.job);
  }
  // no autotuning here: timing candidate plans would stall this thread
  sl.status = lm_batch_run(sl.batch, sl.stream, sl.jobs.data(),
                           (int)sl.jobs.size(), LM_BATCH_NO_TUNE)
                  ? 1
                  : 0;
  if (sl.status) {
    std::lock_guard<std::mutex> lk(mu);
    error = lm_last_error();
  }
  for (SReq &q : sl.reqs)
    if (q.host)
      cudaMemcpyAsync(q.r.dst, q.job.buf, q.bytes, cudaMemcpyDeviceToHost,
                      sl.stream);
  sl.done.store(0);
  sl.busy = true;
  sl.wake = &cv;
  if (cudaLaunchHostFunc(sl.stream, slot_done, &sl) != cudaSuccess) {
    // no callback: wait here so the slot still completes
    cudaStreamSynchronize(sl.stream);
    slot_done(&sl);
  }
}

void lm_serve_st::finish(Slot &sl) {
  const int64_t t = sl.t_done.load();
  for (SReq &q : sl.reqs) {
    lm_serve_done d;
    d.ticket = q.ticket;
    d.status = sl.status;
    d.latency_ns = t - q.t_submit;
    d.queue_ns = q.t_admit - q.t_submit;
    d.done_ns = t;
    done_local.push_back(d);
    inflight -= q.bytes;
    if (q.host) palloc.release(q.pool_off, q.bytes);
  }
  sl.reqs.clear();
  sl.busy = false;
}

void lm_serve_st::run() {
  cudaSetDevice(device);
  while (true) {
    bool progress = false, stopping;
    uint64_t batches = 0;
    {
      std::lock_guard<std::mutex> lk(mu);
      while (!incoming.empty()) {
        waiting.push_back(incoming.front());
        incoming.pop_front();
      }
      stopping = stop;
    }
    // completions
    for (Lane &ln : lanes)
      for (Slot &sl : ln.slots)
        if (sl.busy && sl.done.load()) {
          finish(sl);
          progress = true;
        }
    // admission, in submission order
    while (!waiting.empty()) {
      SReq &q = waiting.front();
      if (inflight + q.bytes > budget) break;
      if (q.host) {
        if (!pool) {
          if (cudaMalloc(&pool, budget) != cudaSuccess) {
            pool = nullptr;
            std::lock_guard<std::mutex> lk(mu);
            error = "cannot allocate the staging pool";
            break;
          }
          palloc.reset(budget);
        }
        if (!palloc.alloc(q.bytes, &q.pool_off)) break;  // fragmented: wait
      }
      q.t_admit = now_ns();
      inflight += q.bytes;
      lanes[q.lane].queue.push_back(q);
      waiting.pop_front();
      progress = true;
    }
    // launches: every lane with queued requests and a free slot
    for (int li = 0; li < kLanes; ++li) {
      Lane &ln = lanes[li];
      if (ln.queue.empty()) continue;
      Slot *free_slot = nullptr;
      for (Slot &sl : ln.slots)
        if (!sl.busy) {
          free_slot = &sl;
          break;
        }
      if (!free_slot) continue;
      uint64_t bytes = 0;
      while (!ln.queue.empty() && free_slot->reqs.size() < kLaneMaxReqs[li] &&
             (free_slot->reqs.empty() ||
              bytes + ln.queue.front().bytes <= kLaneMaxBytes[li])) {
        bytes += ln.queue.front().bytes;
        free_slot->reqs.push_back(ln.queue.front());
        ln.queue.pop_front();
      }
      launch(ln, *free_slot);
      batches += 1;
      progress = true;
    }
    {
      std::lock_guard<std::mutex> lk(mu);
      stats.batches += batches;
      stats.completed += done_local.size();
      stats.peak_inflight_bytes =
          std::max<unsigned long long>(stats.peak_inflight_bytes, inflight);
      finished.insert(finished.end(), done_local.begin(), done_local.end());
    }
    done_local.clear();
    if (stopping) {
      bool idle = waiting.empty();
      for (Lane &ln : lanes) {
        idle = idle && ln.queue.empty();
        for (Slot &sl : ln.slots) idle = idle && !sl.busy;
      }
      if (idle) break;
    }
    if (!progress) {
      // woken by a submission or a finished batch; the timeout bounds a
      // wake-up that raced with this check
      std::unique_lock<std::mutex> lk(mu);
      cv.wait_for(lk, std::chrono::microseconds(50),
                  [&] { return !incoming.empty() || stop; });
    }
  }
}

extern "C" {

bool lm_serve_create(lm_serve_t *out, unsigned long long budget_bytes) {
  if (!out) return lm::set_error("serve: null handle pointer");
  if (budget_bytes == 0) return lm::set_error("serve: budget must be > 0");
  lm_serve_st *s = new lm_serve_st();
  cudaGetDevice(&s->device);
  s->budget = budget_bytes;
  int lo = 0, hi = 0;
  cudaDeviceGetStreamPriorityRange(&lo, &hi);  // hi: numerically lowest
  bool ok = true;
  for (int li = 0; li < kLanes && ok; ++li) {
    const int prio = li == 0 ? hi : (li == 1 ? (lo + hi) / 2 : lo);
    for (Slot &sl : s->lanes[li].slots) {
      ok = ok &&
           cudaStreamCreateWithPriority(&sl.stream, cudaStreamNonBlocking,
                                        prio) == cudaSuccess &&
           !lm_batch_create(&sl.batch) &&
           !lm_batch_set_arena(sl.batch, kLaneArena[li]);
      if (!ok) break;
    }
  }
  if (!ok) {
    for (Lane &ln : s->lanes)
      for (Slot &sl : ln.slots) {
        if (sl.stream) cudaStreamDestroy(sl.stream);
        if (sl.batch) lm_batch_destroy(sl.batch);
      }
    delete s;
    return lm::set_error("serve: cannot create the lane streams");
  }
  s->worker = std::thread([s] { s->run(); });
  *out = s;
  return false;
}

bool lm_serve_submit(lm_serve_t s, const lm_request *req,
                     unsigned long long *ticket) {
  if (!s || !req) return lm::set_error("serve: null argument");
  const int e = req->elem_bytes;
  if (e != 1 && e != 2 && e != 4 && e != 8)
    return lm::set_error("serve: element size must be 1, 2, 4 or 8");
  if (req->op < LM_OP_0100 || req->op > LM_OP_TRANSPOSE)
    return lm::set_error("serve: unknown op");
  SReq q;
  q.r = *req;
  q.bytes = payload_of(*req);
  q.host = req->buf == nullptr;
  if (q.host && q.bytes > 0 && (!req->src || !req->dst))
    return lm::set_error("serve: a host request needs src and dst");
  if (q.bytes > s->budget)
    return lm::set_error("serve: request larger than the HBM budget");
  q.job.buf = req->buf;
  q.job.elem_bytes = e;
  q.job.op = req->op;
  q.job.d0 = req->d0;
  q.job.d1 = req->d1;
  q.job.d2 = req->d2;
  q.job.d3 = req->d3;
  q.lane = q.bytes <= kLaneLimit[0] ? 0 : (q.bytes <= kLaneLimit[1] ? 1 : 2);
  q.t_submit = now_ns();
  {
    std::lock_guard<std::mutex> lk(s->mu);
    if (s->stop) return lm::set_error("serve: server is shutting down");
    q.ticket = s->next_ticket++;
    s->incoming.push_back(q);
    s->stats.submitted += 1;
    s->stats.bytes += q.bytes;
  }
  s->cv.notify_one();
  if (ticket) *ticket = q.ticket;
  return false;
}

int lm_serve_poll(lm_serve_t s, lm_serve_done *out, int cap) {
  if (!s || cap < 0 || (cap > 0 && !out)) return -1;
  std::lock_guard<std::mutex> lk(s->mu);
  const int n = std::min<int>(cap, (int)s->finished.size());
  if (n > 0) {
    std::copy(s->finished.begin(), s->finished.begin() + n, out);
    s->finished.erase(s->finished.begin(), s->finished.begin() + n);
  }
  return n;
}

bool lm_serve_drain(lm_serve_t s, long long timeout_ms) {
  if (!s) return lm::set_error("serve: null handle");
  const int64_t t0 = now_ns();
  while (true) {
    {
      std::lock_guard<std::mutex> lk(s->mu);
      if (s->stats.completed == s->stats.submitted) {
        if (!s->error.empty()) {
          std::string m = "serve: " + s->error;
          s->error.clear();
          return lm::set_error(m.c_str());
        }
        return false;
      }
    }
    if (timeout_ms >= 0 && now_ns() - t0 > timeout_ms * 1000000ll)
      return lm::set_error("serve: drain timed out");
    std::this_thread::sleep_for(std::chrono::microseconds(50));
  }
}

bool lm_serve_stats_get(lm_serve_t s, lm_serve_stats *out) {
  if (!s || !out) return lm::set_error("serve: null argument");
  std::lock_guard<std::mutex> lk(s->mu);
  *out = s->stats;
  return false;
}

// Trace replay: request k is submitted arrival_ns[k] after the call starts
// (and, in server mode, not before requests 0..after[k] have all completed,
// so a trace may reuse buffers ring-wise); out[k] gets its completion with latency and
// queueing measured from the scheduled arrival.  With LM_SERVE_PLAIN the
// server is bypassed: every request runs alone through the per-op planner
// on one stream at its arrival (one request per launch sequence; stream
// order already keeps reused buffers safe), with the planner's default
// choice per shape (no autotuning, which would time candidates on first
// sight of a shape class).
static void wait_until(int64_t t) {
  while (now_ns() < t) std::this_thread::yield();
}

bool lm_serve_replay(lm_serve_t s, const lm_request *reqs,
                     const long long *arrival_ns, const int *after, int n,
                     unsigned flags, lm_serve_done *out) {
  if (n < 0 || (n > 0 && (!reqs || !arrival_ns || !out)))
    return lm::set_error("serve replay: bad arguments");
  const bool plain = (flags & LM_SERVE_PLAIN) != 0;
  if (!plain && !s) return lm::set_error("serve replay: null server");
  for (int k = 0; k < n; ++k)
    if (after && (after[k] >= k || after[k] < -1))
      return lm::set_error("serve replay: after[k] must be -1 or < k");
  const int64_t t0 = now_ns() + 1000000;  // 1 ms to get going
  if (plain) {
    // completion times from timing events (a host callback per request
    // would stall the stream for its round trip): request k's completion is
    // the host time of the start event plus the device time between it and
    // k's event
    cudaStream_t st;
    if (cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking) != cudaSuccess)
      return lm::set_error("serve replay: stream");
    std::vector<cudaEvent_t> ev(n + 1, nullptr);
    bool ev_ok = true;
    for (int k = 0; k <= n && ev_ok; ++k)
      ev_ok = cudaEventCreate(&ev[k]) == cudaSuccess;
    if (!ev_ok) {
      for (cudaEvent_t e : ev)
        if (e) cudaEventDestroy(e);
      cudaStreamDestroy(st);
      return lm::set_error("serve replay: events");
    }
    std::vector<int64_t> t_sub(n);
    std::vector<int> status(n, 0);
    cudaEventRecord(ev[n], st);
    cudaEventSynchronize(ev[n]);
    const int64_t t_ev = now_ns();  // the start event has executed
    for (int k = 0; k < n; ++k) {
      const lm_request &r = reqs[k];
      uint64_t T, a, B, b;
      wait_until(t0 + arrival_ns[k]);
      t_sub[k] = now_ns();
      if (!r.buf || !lm::op_as_0100(r.op, r.d0, r.d1, r.d2, r.d3, &T, &a, &B, &b))
        status[k] = 1;
      else if (lm::run_0100_planned(st, r.buf, r.elem_bytes, T, a, B, b, 0))
        status[k] = 1;
      cudaEventRecord(ev[k], st);
    }
    cudaStreamSynchronize(st);
    bool failed = false;
    for (int k = 0; k < n; ++k) {
      float ms = 0.f;
      cudaEventElapsedTime(&ms, ev[n], ev[k]);
      const int64_t arr = t0 + arrival_ns[k];
      out[k].ticket = (unsigned long long)k + 1;
      out[k].status = status[k];
      out[k].done_ns = std::max<int64_t>(t_sub[k], t_ev + (int64_t)(ms * 1e6));
      out[k].latency_ns = out[k].done_ns - arr;
      out[k].queue_ns = t_sub[k] - arr;
      failed |= status[k] != 0;
    }
    for (cudaEvent_t e : ev) cudaEventDestroy(e);
    cudaStreamDestroy(st);
    return failed ? lm::set_error("serve replay: a plain request failed")
                  : false;
  }
  std::vector<unsigned long long> ticket(n, 0);
  std::vector<char> done(n, 0);
  std::vector<lm_serve_done> got(n);
  std::map<unsigned long long, int> index;  // ticket -> request
  std::vector<lm_serve_done> buf(1024);
  auto collect = [&]() {
    const int m = lm_serve_poll(s, buf.data(), (int)buf.size());
    for (int i = 0; i < m; ++i) {
      auto it = index.find(buf[i].ticket);
      if (it == index.end()) continue;  // not ours
      got[it->second] = buf[i];
      done[it->second] = 1;
    }
    return m;
  };
  std::vector<int64_t> t_sub(n);
  int prefix = -1;  // requests 0..prefix have all completed
  for (int k = 0; k < n; ++k) {
    wait_until(t0 + arrival_ns[k]);
    if (after && after[k] >= 0)
      while (true) {
        while (prefix + 1 < k && done[prefix + 1]) ++prefix;
        if (prefix >= after[k]) break;
        if (collect() == 0) std::this_thread::yield();
      }
    t_sub[k] = now_ns();
    if (lm_serve_submit(s, &reqs[k], &ticket[k])) return true;
    index[ticket[k]] = k;
    collect();
  }
  if (lm_serve_drain(s, -1)) return true;
  while (collect() > 0) {
  }
  for (int k = 0; k < n; ++k) {
    if (!done[k]) return lm::set_error("serve replay: a completion is missing");
    const int64_t arr = t0 + arrival_ns[k];
    out[k] = got[k];
    out[k].latency_ns = got[k].done_ns - arr;
    out[k].queue_ns = (t_sub[k] - arr) + got[k].queue_ns;
  }
  return false;
}

void lm_serve_destroy(lm_serve_t s) {
  if (!s) return;
  {
    std::lock_guard<std::mutex> lk(s->mu);
    s->stop = true;
  }
  s->cv.notify_one();
  if (s->worker.joinable()) s->worker.join();
  for (Lane &ln : s->lanes)
    for (Slot &sl : ln.slots) {
      if (sl.stream) cudaStreamSynchronize(sl.stream);
      if (sl.batch) lm_batch_destroy(sl.batch);
      if (sl.stream) cudaStreamDestroy(sl.stream);
    }
  if (s->pool) cudaFree(s->pool);
  delete s;
}

}  // extern "C"
