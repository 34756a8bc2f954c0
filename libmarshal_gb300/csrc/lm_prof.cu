// lm_prof.cu -- per-kernel timing and launch counting.
//
// Counterpart of the reference's Profiling class (include/cl_profile.h:6-63),
// which wraps one cl::Event per kernel and reports its device time.  Here every
// kernel launch of the library goes through a ProfScope: it counts the launch
// and, while profiling is enabled, brackets the launch with two CUDA events on
// the launching stream.  lm_prof_collect() waits for the recorded events and
// returns per-kernel launch counts and summed device time.
#include <atomic>
#include <cstring>
#include <mutex>
#include <string>
#include <vector>

#include "lm_internal.h"
#include "../../include/lm_marshal.h"

namespace lm {

namespace {
struct Rec {
  const char *name;
  cudaEvent_t a, b;
};
std::atomic<unsigned long long> g_launches{0};
std::atomic<bool> g_enabled{false};
std::mutex g_mu;
std::vector<Rec> g_recs;
std::vector<cudaEvent_t> g_free;

cudaEvent_t take_event() {
  if (!g_free.empty()) {
    cudaEvent_t e = g_free.back();
    g_free.pop_back();
    return e;
  }
  cudaEvent_t e = nullptr;
  cudaEventCreate(&e);
  return e;
}
}  // namespace

ProfScope::ProfScope(cudaStream_t s, const char *name) : s_(s), name_(name) {
  g_launches.fetch_add(1, std::memory_order_relaxed);
  if (!g_enabled.load(std::memory_order_relaxed)) return;
  // launches recorded into a graph are not timed (their events would
  // belong to the graph, not to a run of it)
  cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
  if (cudaStreamIsCapturing(s, &cs) != cudaSuccess) {
    cudaGetLastError();  // the query's own error only
    return;
  }
  if (cs != cudaStreamCaptureStatusNone) return;  // a pending launch error
                                                  // stays for the caller
  std::lock_guard<std::mutex> lock(g_mu);
  a_ = take_event();
  b_ = take_event();
  if (a_) cudaEventRecord((cudaEvent_t)a_, s_);
}

ProfScope::~ProfScope() {
  if (!a_) return;
  cudaEventRecord((cudaEvent_t)b_, s_);
  std::lock_guard<std::mutex> lock(g_mu);
  g_recs.push_back(Rec{name_, (cudaEvent_t)a_, (cudaEvent_t)b_});
}

}  // namespace lm

using namespace lm;

extern "C" {

unsigned long long lm_launch_count(void) {
  return g_launches.load(std::memory_order_relaxed);
}

void lm_prof_enable(int on) { g_enabled.store(on != 0); }

int lm_prof_collect(lm_prof_entry *out, int cap) {
  std::vector<Rec> recs;
  {
    std::lock_guard<std::mutex> lock(g_mu);
    recs.swap(g_recs);
  }
  std::vector<lm_prof_entry> acc;
  for (const Rec &r : recs) {
    float ms = 0.f;
    if (cudaEventSynchronize(r.b) != cudaSuccess ||
        cudaEventElapsedTime(&ms, r.a, r.b) != cudaSuccess) {
      cudaGetLastError();  // leave no error behind for the next call
      ms = 0.f;
    }
    size_t i = 0;
    for (; i < acc.size(); ++i)
      if (strncmp(acc[i].name, r.name, sizeof(acc[i].name) - 1) == 0) break;
    if (i == acc.size()) {
      lm_prof_entry e;
      memset(&e, 0, sizeof(e));
      strncpy(e.name, r.name, sizeof(e.name) - 1);
      acc.push_back(e);
    }
    acc[i].launches += 1;
    acc[i].total_ms += ms;
  }
  {
    std::lock_guard<std::mutex> lock(g_mu);
    for (const Rec &r : recs) {
      g_free.push_back(r.a);
      g_free.push_back(r.b);
    }
  }
  int n = (int)acc.size();
  for (int i = 0; i < n && i < cap; ++i) out[i] = acc[i];
  return n;
}

int lm_prof_timeline(lm_prof_span *out, int cap) {
  std::vector<Rec> recs;
  {
    std::lock_guard<std::mutex> lock(g_mu);
    recs.swap(g_recs);
  }
  // the earliest start is the origin: every start event is compared with
  // the first recorded one (launches on other streams may start earlier)
  float origin = 0.f;
  std::vector<float> t0(recs.size(), 0.f), t1(recs.size(), 0.f);
  for (size_t k = 0; k < recs.size(); ++k) {
    if (cudaEventSynchronize(recs[k].b) != cudaSuccess ||
        cudaEventElapsedTime(&t0[k], recs[0].a, recs[k].a) != cudaSuccess ||
        cudaEventElapsedTime(&t1[k], recs[0].a, recs[k].b) != cudaSuccess) {
      cudaGetLastError();
      t0[k] = t1[k] = 0.f;
    }
    if (t0[k] < origin) origin = t0[k];
  }
  const int n = (int)recs.size();
  for (int k = 0; k < n && k < cap; ++k) {
    memset(&out[k], 0, sizeof(out[k]));
    strncpy(out[k].name, recs[k].name, sizeof(out[k].name) - 1);
    out[k].start_ms = t0[k] - origin;
    out[k].end_ms = t1[k] - origin;
  }
  {
    std::lock_guard<std::mutex> lock(g_mu);
    for (const Rec &r : recs) {
      g_free.push_back(r.a);
      g_free.push_back(r.b);
    }
  }
  return n;
}

}  // extern "C"
