// lm_api.cu -- host dispatch, planner and the exported C ABI.
//
// Drop-in surface (see include/marshal.h and include/lm_marshal.h):
//   gpu_aos_asta_bs_float/double, gpu_aos_asta_pttwac, gpu_soa_asta_pttwac
//       -- include/marshal.h:26-31 of the reference, same signatures;
//   lm_* -- one entry per cl_* function of include/cl_marshal.h:26-49 with
//       (cl_command_queue, cl_mem) replaced by (cudaStream_t, void *buf, int
//       elem_bytes); same argument order, same meaning, same error convention:
//       false on success, true on error (API.wiki:12,20), with the message
//       available from lm_last_error().
//
// Everything is stream ordered.  Scratch (done bits, ticket words) comes from
// the device's stream-ordered memory pool (cudaMallocAsync / cudaFreeAsync on
// the caller's stream), so concurrent calls on different streams never share
// it and repeated calls reuse pooled memory instead of allocating.
#include <atomic>
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <map>
#include <mutex>
#include <string>
#include <tuple>

#include "lm_core.cuh"
#include "lm_internal.h"
#include "../../include/lm_marshal.h"
#include "../../include/marshal.h"

namespace lm {

// ---- device info ------------------------------------------------------------

const DeviceInfo &device_info() {
  static DeviceInfo cache[64];
  static std::mutex mu;
  int dev = 0;
  cudaGetDevice(&dev);
  DeviceInfo &d = cache[dev & 63];
  if (d.device != dev) {
    std::lock_guard<std::mutex> lock(mu);
    if (d.device != dev) {
      DeviceInfo n;
      n.device = dev;
      cudaDeviceGetAttribute(&n.sms, cudaDevAttrMultiProcessorCount, dev);
      cudaDeviceGetAttribute(&n.max_smem_optin,
                             cudaDevAttrMaxSharedMemoryPerBlockOptin, dev);
      cudaDeviceGetAttribute(&n.max_smem_per_sm,
                             cudaDevAttrMaxSharedMemoryPerMultiprocessor, dev);
      cudaDeviceGetAttribute(&n.cc_major, cudaDevAttrComputeCapabilityMajor, dev);
      cudaDeviceGetAttribute(&n.cc_minor, cudaDevAttrComputeCapabilityMinor, dev);
      if (n.sms <= 0) n.sms = 1;
      if (n.max_smem_optin <= 0) n.max_smem_optin = 48 * 1024;
      d = n;
    }
  }
  return d;
}

// ---- errors -----------------------------------------------------------------

static thread_local std::string g_err;

static bool fail(const char *fmt, ...) {
  char buf[512];
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(buf, sizeof(buf), fmt, ap);
  va_end(ap);
  g_err = buf;
  if (getenv("LM_VERBOSE")) fprintf(stderr, "libmarshal_gb300: %s\n", buf);
  return true;
}

bool set_error(const char *msg) { return fail("%s", msg); }

static bool cuda_fail(cudaError_t e, const char *what) {
  return fail("%s: %s", what, cudaGetErrorString(e));
}

// ---- scratch ----------------------------------------------------------------

int prepare_launch(const void *kern, LaunchCache &c, size_t smem, int threads,
                   cudaError_t *err) {
  *err = cudaSuccess;
  int dev = 0;
  cudaGetDevice(&dev);
  const int d = dev & 7;
  const int need = (int)smem + 1;
  if (need > 48 * 1024 + 1 && c.smem_set[d].load(std::memory_order_acquire) < need) {
    if ((*err = cudaFuncSetAttribute(kern,
                                     cudaFuncAttributeMaxDynamicSharedMemorySize,
                                     (int)smem)) != cudaSuccess)
      return 0;
    int cur = c.smem_set[d].load();
    while (cur < need && !c.smem_set[d].compare_exchange_weak(cur, need)) {
    }
  }
  const uint64_t key = c.occ_key[d].load(std::memory_order_acquire);
  if (key && (key >> 16) == (uint64_t)smem) return (int)(key & 0xffff);
  int occ = 0;
  if ((*err = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, kern, threads,
                                                            smem)) != cudaSuccess)
    return 0;
  c.occ_key[d].store(((uint64_t)smem << 16) | (uint64_t)(occ & 0xffff),
                     std::memory_order_release);
  return occ;
}

void pool_keep_memory() {
  static std::atomic<bool> done[64];
  int dev = 0;
  cudaGetDevice(&dev);
  if (done[dev & 63].load(std::memory_order_acquire)) return;
  cudaMemPool_t pool;
  if (cudaDeviceGetDefaultMemPool(&pool, dev) == cudaSuccess) {
    uint64_t thr = ~0ull;  // keep freed blocks pooled between calls
    cudaMemPoolSetAttribute(pool, cudaMemPoolAttrReleaseThreshold, &thr);
  }
  done[dev & 63].store(true, std::memory_order_release);
}

struct Scratch {
  void *p = nullptr;
  cudaStream_t s = nullptr;
  ~Scratch() {
    if (p) cudaFreeAsync(p, s);
  }
};

// Like get_scratch, but a failed allocation only returns false (no error
// recorded): for plans that have a fallback.
static bool try_scratch(Scratch &sc, size_t bytes, cudaStream_t s) {
  pool_keep_memory();
  sc.s = s;
  if (cudaMallocAsync(&sc.p, bytes ? bytes : 4, s) != cudaSuccess) {
    cudaGetLastError();
    sc.p = nullptr;
    return false;
  }
  return true;
}

static bool get_scratch(Scratch &sc, size_t bytes, cudaStream_t s) {
  pool_keep_memory();
  sc.s = s;
  cudaError_t e = cudaMallocAsync(&sc.p, bytes ? bytes : 4, s);
  if (e != cudaSuccess) {
    sc.p = nullptr;
    return cuda_fail(e, "scratch allocation");
  }
  return false;
}

static bool get_zeroed(Scratch &sc, size_t bytes, cudaStream_t s) {
  pool_keep_memory();
  sc.s = s;
  cudaError_t e = cudaMallocAsync(&sc.p, bytes ? bytes : 4, s);
  if (e != cudaSuccess) {
    sc.p = nullptr;
    return cuda_fail(e, "scratch allocation");
  }
  e = cudaMemsetAsync(sc.p, 0, bytes ? bytes : 4, s);
  if (e != cudaSuccess) return cuda_fail(e, "scratch clear");
  return false;
}

// ---- persistent status word (failures of waiting kernels) ---------------

uint32_t *device_status_word() {
  static std::mutex mu;
  static uint32_t *words[64] = {nullptr};
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 64) return nullptr;
  std::lock_guard<std::mutex> lock(mu);
  if (!words[dev]) {
    void *p = nullptr;
    if (cudaMalloc(&p, 4) != cudaSuccess) return nullptr;
    if (cudaMemset(p, 0, 4) != cudaSuccess) return nullptr;
    words[dev] = (uint32_t *)p;
  }
  return words[dev];
}

// Reads and clears the status word after the stream's work has finished.
static bool check_status(cudaStream_t s, const char *what) {
  uint32_t *w = device_status_word();
  if (!w) return fail("%s: no status word", what);
  uint32_t v = 0;
  cudaError_t e = cudaMemcpyAsync(&v, w, 4, cudaMemcpyDeviceToHost, s);
  if (e == cudaSuccess) e = cudaStreamSynchronize(s);
  if (e != cudaSuccess) return cuda_fail(e, what);
  if (v != kStatusOk) {
    cudaMemsetAsync(w, 0, 4, s);
    return fail("%s: an inter-CTA wait timed out (status %u)", what, v);
  }
  return false;
}

// ---- timing (the reference's elapsed_time accumulator) ----------------------

struct OpTimer {
  unsigned long long *et;
  cudaStream_t s;
  cudaEvent_t a = nullptr, b = nullptr;
  OpTimer(unsigned long long *et_, cudaStream_t s_) : et(et_), s(s_) {
    if (et) {
      cudaEventCreate(&a);
      cudaEventCreate(&b);
      cudaEventRecord(a, s);
    }
  }
  // Adds the elapsed kernel time in ns (blocks, like Profiling::Report).
  bool finish() {
    if (!et) return false;
    cudaEventRecord(b, s);
    cudaError_t e = cudaEventSynchronize(b);
    if (e != cudaSuccess) return cuda_fail(e, "timing");
    if (check_status(s, "status")) return true;
    float ms = 0.f;
    cudaEventElapsedTime(&ms, a, b);
    *et += (unsigned long long)((double)ms * 1.0e6);
    return false;
  }
  ~OpTimer() {
    if (a) cudaEventDestroy(a);
    if (b) cudaEventDestroy(b);
  }
};

static bool valid_e(int e) { return e == 1 || e == 2 || e == 4 || e == 8; }

// Elements are moved as e-byte words, so the buffer must be e-byte aligned.
static bool misaligned(const void *buf, int e) {
  return ((uintptr_t)buf & (uintptr_t)(e - 1)) != 0;
}

// Limit for every inter-CTA wait (LM_WAIT_TIMEOUT_MS overrides, default 2 s).
static uint64_t wait_timeout_ns() {
  const char *v = getenv("LM_WAIT_TIMEOUT_MS");
  const long long ms = v ? atoll(v) : 2000;
  return (uint64_t)(ms > 0 ? ms : 2000) * 1000000ull;
}

// ---- planner ----------------------------------------------------------------

enum class Method { Auto, BS, Pttwac, Stash, TwoPass, Cycles, Staged, Resident };

TuneParams &tune_params() {
  static thread_local TuneParams p;
  return p;
}

bool &planner_beside_other_work() {
  static thread_local bool v = false;
  return v;
}

// A tuned choice: the method, and the variant of it (an index into the
// table below) in bits 8-15.
struct TuneVariant {
  Method m;
  TuneParams p;
};
static const TuneVariant kVariants[] = {
    {Method::Auto, {}},
    {Method::Staged, {16u << 10, 0}},
    {Method::Staged, {0, 0}},            // 32 KB blocks (built-in)
    {Method::Staged, {64u << 10, 0}},
    {Method::Cycles, {}},
    {Method::Stash, {0, 0}},             // the planner's CTAs per SM
    {Method::Stash, {0, 1}},
    {Method::Stash, {0, 2}},
    {Method::TwoPass, {}},
    {Method::Pttwac, {}},
};
constexpr int kNumVariants = (int)(sizeof(kVariants) / sizeof(kVariants[0]));

// Sets the thread's tuning overrides for the life of the object.
struct TuneScope {
  TuneParams saved;
  explicit TuneScope(const TuneParams &p) : saved(tune_params()) {
    tune_params() = p;
  }
  ~TuneScope() { tune_params() = saved; }
};

static bool check_launch(cudaError_t e, const char *what) {
  if (e != cudaSuccess) return cuda_fail(e, what);
  return false;
}

static bool run_pttwac_direct(cudaStream_t s, void *buf, int e, uint64_t T,
                              uint64_t a, uint64_t B, uint64_t b) {
  const size_t fb = pttwac_flag_bytes(buf, T, (uint32_t)a, (uint32_t)B,
                                      (uint32_t)b, e);
  if (fb == 0) return fail("PTTWAC: shape exceeds 2^32 units per instance");
  Scratch flags;
  if (get_zeroed(flags, fb, s)) return true;
  return check_launch(launch_pttwac0100(s, buf, e, T, (uint32_t)a,
                                        (uint32_t)B, (uint32_t)b,
                                        (uint32_t *)flags.p),
                      "PTTWAC launch");
}

// Largest-unit-first search for a two-pass split of one 100(a, B, b):
// returns a2 | a with a2*U in [128, 1024] bytes whose tile a2 x B x b fits BS.
static uint64_t split_a(uint64_t a, uint64_t B, uint64_t b, int e) {
  const uint64_t U = b * e;
  uint64_t best = 0;
  for (uint64_t d = 2; d <= a && d * U <= 1024; ++d) {
    if (a % d) continue;
    if (d * U < 128) continue;
    BsPlan p = plan_bs0100(1, (uint32_t)d, (uint32_t)B, (uint32_t)b, e);
    if (!p.feasible) continue;
    best = d;
    break;  // smallest d with a >= 128-byte unit
  }
  return best;
}

static uint64_t split_B(uint64_t a, uint64_t B, uint64_t b, int e) {
  const uint64_t U = b * e;
  for (uint64_t c = 2; c <= B && c * U <= 1024; ++c) {
    if (B % c) continue;
    if (c * U < 128) continue;
    BsPlan p = plan_bs0100(1, (uint32_t)a, (uint32_t)c, (uint32_t)b, e);
    if (!p.feasible) continue;
    return c;
  }
  return 0;
}

// 0100(T, a, B, b): [T][a][B][b] -> [T][B][a][b] with e-byte elements.
static bool do_0100(cudaStream_t s, void *buf, int e, uint64_t T, uint64_t a,
                    uint64_t B, uint64_t b, Method m) {
  if (!valid_e(e)) return fail("element size must be 1, 2, 4 or 8 (got %d)", e);
  if (T == 0 || a == 0 || B == 0 || b == 0) return false;  // empty
  if (a == 1 || B == 1) return false;                      // identity
  if (buf == nullptr) return fail("null buffer");
  if (misaligned(buf, e)) return fail("buffer must be aligned to the element size");
  if (a * B >= 0xffffffffull) return fail("a*B must be < 2^32");
  widen_units(buf, &e, &b);
  if (m == Method::Auto || m == Method::BS) {
    BsPlan p = plan_bs0100(T, (uint32_t)a, (uint32_t)B, (uint32_t)b, e);
    // a megabyte or more in fewer tile chunks (or clusters) than SMs leaves
    // most of the GPU idle: the methods below spread any shape over blocks
    const uint64_t chunks = (T + p.tiles_per_chunk - 1) / p.tiles_per_chunk;
    // (the 16-byte tile kernel sizes its own chunks to the GPU)
    const bool t010 = b == 1 && p.feasible && p.cluster == 1 &&
                      tile010_applies(buf, e, T, a, B);
    const uint64_t bytes = T * a * B * b * (uint64_t)e;
    const uint64_t ctas = chunks * (uint64_t)p.cluster;
    const uint64_t sms = (uint64_t)device_info().sms;
    bool thin = m == Method::Auto && !t010 && bytes >= (1ull << 20) &&
                ctas < sms;
    // payloads the resident form takes (from 512 KB): the on-chip plan wins
    // from half the SMs up (64 tiles of 64 x 4096 bytes in 2-CTA clusters:
    // 0.0173 vs 0.0182 ms), the resident form below (one 1000 x 1000 byte
    // tile over a 16-CTA cluster: 0.0336 vs 0.0144 ms)
    if (m == Method::Auto && !t010 && p.feasible && bytes >= (512ull << 10) &&
        !planner_beside_other_work() && !getenv("LM_NO_RESIDENT") &&
        resident0100_applies(T, a, B, b, e)) {
      // (under stream capture the resident form does not run)
      cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
      if (cudaStreamIsCapturing(s, &cs) == cudaSuccess &&
          cs == cudaStreamCaptureStatusNone)
        thin = ctas * 2 < sms;
    }
    if (p.feasible && !thin)
      return check_launch(launch_bs0100(s, buf, e, T, (uint32_t)a,
                                        (uint32_t)B, (uint32_t)b, p),
                          "BS launch");
    if (m == Method::BS)
      return fail("BS: tile of %llu bytes exceeds on-chip capacity",
                  (unsigned long long)(a * B * b * e));
  }
  const uint64_t U = b * e;
  // all cycles short (multiplicative order of a modulo a*B - 1 at most
  // kCycleMaxLen): whole-cycle moves, 2 x payload, no flags (lm_cycles.cu)
  if (m == Method::Cycles ||
      (m == Method::Auto && U >= 64 && !getenv("LM_NO_CYCLES"))) {
    const uint32_t L = cycle_order(a, B, kCycleMaxLen);
    if (L && a * B - 1 <= (1ull << 28)) {
      // leader lists are cached per shape, except under stream capture
      // (where the list is computed into per-call scratch)
      cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
      cudaStreamIsCapturing(s, &cs);
      Scratch sc;
      if (get_scratch(sc, cycle_scratch_bytes(a, B), s)) return true;
      return check_launch(
          launch_cycles100(s, buf, e, T, (uint32_t)a, (uint32_t)B,
                           (uint32_t)b, L, sc.p,
                           cs == cudaStreamCaptureStatusNone),
          "cycles launch");
    }
    if (m == Method::Cycles)
      return fail("cycles: the cycles of 100(%llu, %llu) are longer than %u",
                  (unsigned long long)a, (unsigned long long)B,
                  (unsigned)kCycleMaxLen);
  }
  // a payload that fits the shared memory of all SMs: one cooperative
  // launch at 2 x payload (not beside other work, where it would wait for
  // every SM to drain, nor under stream capture)
  if (m == Method::Resident ||
      (m == Method::Auto && !planner_beside_other_work() &&
       !getenv("LM_NO_RESIDENT"))) {
    uint32_t *status = device_status_word();
    const cudaError_t err =
        status ? launch_resident0100(s, buf, e, T, a, B, b, status,
                                     wait_timeout_ns())
               : cudaErrorNotSupported;
    if (err == cudaSuccess) return false;
    if (err != cudaErrorNotSupported) return cuda_fail(err, "resident launch");
    if (m == Method::Resident)
      return fail("resident: 0100(%llu, %llu, %llu, %llu) does not fit shared "
                  "memory (or the stream is being captured)",
                  (unsigned long long)T, (unsigned long long)a,
                  (unsigned long long)B, (unsigned long long)b);
  }
  // the stash wavefront spreads rows over all CTAs: with too few rows per
  // SM its steps are too small to keep HBM busy
  const uint64_t stash_min_rows = kStashRowsPerSm * (uint64_t)device_info().sms;
  const bool want_stash =
      m == Method::Stash ||
      (m == Method::Auto && T == 1 && U < 128 && a * B >= (1ull << 20) &&
       a >= stash_min_rows && !getenv("LM_NO_STASH"));
  if (want_stash) {
    // 100 on small units: the 3 x payload streaming plan (lm_stash.cu).
    StashPlan sp = T == 1 ? plan_stash(a, B, (uint32_t)b, e) : StashPlan();
    // very tall matrices leave each CTA short strips (a step's rows x strip
    // must fit shared memory); below 384-byte strips the staged form moves
    // units of 4 bytes and more faster (fp64 32768 x 16000: 3.06 TB/s by
    // the stash with 256-byte strips, 3.24 TB/s staged)
    if (m == Method::Auto && sp.feasible && U >= 4 && sp.g * U < 384 &&
        staged0100_applies(T, a, B, b, e))
      sp = StashPlan();
    uint32_t *status = sp.feasible ? device_status_word() : nullptr;
    if (sp.feasible && status) {
      // the stash (about half the payload) may not be available: then the
      // plans below, which need less scratch, take over
      Scratch sc;
      if (try_scratch(sc, stash_scratch_bytes(sp), s))
        return check_launch(launch_stash100(s, buf, e, a, B, (uint32_t)b, sp,
                                            sc.p, status, wait_timeout_ns()),
                            "stash launch");
      if (m == Method::Stash) return fail("stash: no scratch for this size");
    }
    if (m == Method::Stash)
      return fail("stash plan not applicable to 0100(%llu, %llu, %llu, %llu)",
                  (unsigned long long)T, (unsigned long long)a,
                  (unsigned long long)B, (unsigned long long)b);
  }
  // any shape through scratch: block transposes out of place, then a copy
  // back (4 x payload, but every access in whole sectors); falls through
  // when the scratch cannot be had
  // (units of 512 bytes and more move as whole lines in cycle following,
  // which needs no scratch and is as fast or faster)
  // (also larger units when the tiles are many and small: cycle following
  // on 18 tiles of 72 x 100 1600-byte units ran 2.3 TB/s, the staged form
  // 2.9 TB/s)
  if (m == Method::Staged ||
      (m == Method::Auto &&
       (U < kStagedMaxUnit || (T > 1 && a * B < 65536)) &&
       T * a * B * b * e >= (1ull << 20) &&
       !getenv("LM_NO_STAGED"))) {
    if (staged0100_applies(T, a, B, b, e)) {
      // the scratch copy sits at the buffer's address modulo 16, so the
      // copy back runs in aligned 16-byte vectors
      Scratch sc;
      if (try_scratch(sc, T * a * B * b * e + 16, s))
        return check_launch(
            launch_staged0100(s, buf, e, T, a, B, b,
                              (char *)sc.p + ((uintptr_t)buf & 15)),
            "staged launch");
      if (m == Method::Staged) return fail("staged: no scratch for this size");
    } else if (m == Method::Staged) {
      return fail("staged: units above 32 KB or too many blocks");
    }
  }
  if ((m == Method::Auto && U < 128) || m == Method::TwoPass) {
    // Aggregate small super-elements into >=128-byte units first so the
    // cycle-following pass moves whole cache lines.
    uint64_t a2 = split_a(a, B, b, e);
    if (a2) {
      const uint64_t a1 = a / a2;
      if (do_0100(s, buf, e, T * a1, a2, B, b, Method::BS)) return true;
      return do_0100(s, buf, e, T, a1, B, a2 * b, Method::Pttwac);
    }
    uint64_t c = split_B(a, B, b, e);
    if (c) {
      const uint64_t B1 = B / c;
      if (do_0100(s, buf, e, T, a, B1, c * b, Method::Pttwac)) return true;
      return do_0100(s, buf, e, T * B1, a, c, b, Method::BS);
    }
    if (m == Method::TwoPass) return fail("no two-pass split for this shape");
  }
  return run_pttwac_direct(s, buf, e, T, a, B, b);
}

// ---- autotuner ----------------------------------------------------------------
// Shape class = (element bytes, log2 of a, B and b, and whether the op has
// several instances).  For each class met by a tuned call the candidate plans
// are timed once on a scratch buffer of the job's size and the fastest is
// remembered; LM_TUNE_FILE names a text file that is loaded at first use and
// appended to ("e la lB lb multi method" per line).

struct TuneKey {
  int e, la, lB, lb, multi;
  bool operator<(const TuneKey &o) const {
    return std::tie(e, la, lB, lb, multi) <
           std::tie(o.e, o.la, o.lB, o.lb, o.multi);
  }
};

static int ilog2(uint64_t v) {
  int l = 0;
  while (v > 1) {
    v >>= 1;
    ++l;
  }
  return l;
}

static std::mutex g_tune_mu;
static std::map<TuneKey, int> g_tune;
static bool g_tune_loaded = false;

static void tune_load_locked() {
  if (g_tune_loaded) return;
  g_tune_loaded = true;
  const char *f = getenv("LM_TUNE_FILE");
  if (!f) return;
  FILE *fp = fopen(f, "r");
  if (!fp) return;
  // lines "v2 e log2a log2B log2b multi variant"; other lines are skipped
  char line[256];
  while (fgets(line, sizeof(line), fp)) {
    TuneKey k;
    int m;
    if (sscanf(line, "v2 %d %d %d %d %d %d", &k.e, &k.la, &k.lB, &k.lb,
               &k.multi, &m) == 6)
      g_tune[k] = m;
  }
  fclose(fp);
}

static void tune_save_locked(const TuneKey &k, int m) {
  const char *f = getenv("LM_TUNE_FILE");
  if (!f) return;
  FILE *fp = fopen(f, "a");
  if (!fp) return;
  fprintf(fp, "v2 %d %d %d %d %d %d\n", k.e, k.la, k.lB, k.lb, k.multi, m);
  fclose(fp);
}

// Whether a forced method applies to this exact shape (a tuned choice is
// shared by every shape of its class, whose factors may differ).
static bool method_applies(Method m, int e, uint64_t T, uint64_t a,
                           uint64_t B, uint64_t b) {
  switch (m) {
    case Method::Stash:
      return T == 1 && plan_stash(a, B, (uint32_t)b, e).feasible;
    case Method::TwoPass:
      return b * e < 128 && (split_a(a, B, b, e) || split_B(a, B, b, e));
    case Method::BS:
      return plan_bs0100(T, (uint32_t)a, (uint32_t)B, (uint32_t)b, e).feasible;
    case Method::Cycles:
      return cycle_order(a, B, kCycleMaxLen) != 0 && a * B - 1 <= (1ull << 28);
    case Method::Staged:
      return staged0100_applies(T, a, B, b, e);
    case Method::Resident:
      return resident0100_applies(T, a, B, b, e);
    default:
      return true;
  }
}

// The tuned variant (index into kVariants) of a shape class: every variant
// that applies is timed once on a scratch buffer of the job's shape (after
// a warm-up run), the fastest is kept, in memory and in LM_TUNE_FILE.
static int tuned_variant(cudaStream_t s, int e, uint64_t T, uint64_t a,
                         uint64_t B, uint64_t b) {
  const TuneKey key{e, ilog2(a), ilog2(B), ilog2(b), T > 1 ? 1 : 0};
  {
    std::lock_guard<std::mutex> lock(g_tune_mu);
    tune_load_locked();
    auto it = g_tune.find(key);
    if (it != g_tune.end() && it->second >= 0 && it->second < kNumVariants)
      return it->second;
  }
  const uint64_t bytes = T * a * B * b * (uint64_t)e;
  void *tmp = nullptr;
  int best = 0;
  if (cudaMallocAsync(&tmp, bytes, s) == cudaSuccess) {
    cudaEvent_t e0, e1;
    cudaEventCreate(&e0);
    cudaEventCreate(&e1);
    float best_ms = 1e30f;
    for (int i = 0; i < kNumVariants; ++i) {
      const TuneVariant &v = kVariants[i];
      if (v.m == Method::TwoPass && b * e >= 128) continue;
      TuneScope scope(v.p);
      const std::string saved = g_err;
      if (!method_applies(v.m, e, T, a, B, b) ||
          do_0100(s, tmp, e, T, a, B, b, v.m)) {  // warm-up
        g_err = saved;
        continue;
      }
      cudaEventRecord(e0, s);
      do_0100(s, tmp, e, T, a, B, b, v.m);
      cudaEventRecord(e1, s);
      cudaEventSynchronize(e1);
      float ms = 0.f;
      cudaEventElapsedTime(&ms, e0, e1);
      if (ms < best_ms) {
        best_ms = ms;
        best = i;
      }
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    cudaFreeAsync(tmp, s);
  }
  std::lock_guard<std::mutex> lock(g_tune_mu);
  g_tune[key] = best;
  tune_save_locked(key, best);
  return best;
}

bool run_0100_planned(cudaStream_t s, void *buf, int e, uint64_t T,
                      uint64_t a, uint64_t B, uint64_t b, int tune) {
  if (valid_e(e)) widen_units(buf, &e, &b);  // the tuned class is the wide one
  if (tune && valid_e(e) && T > 0 && a > 1 && B > 1 && b > 0 &&
      T * a * B * b * (uint64_t)e >= (1ull << 20)) {
    const TuneVariant &v = kVariants[tuned_variant(s, e, T, a, B, b)];
    TuneScope scope(v.p);
    if (method_applies(v.m, e, T, a, B, b))
      return do_0100(s, buf, e, T, a, B, b, v.m);
  }
  return do_0100(s, buf, e, T, a, B, b, Method::Auto);
}

static bool do_010_pttwac(cudaStream_t s, void *buf, int e, uint64_t A,
                          uint64_t a, uint64_t B, int R, int P) {
  if (!valid_e(e)) return fail("element size must be 1, 2, 4 or 8 (got %d)", e);
  if (A == 0 || a <= 1 || B <= 1) return false;
  if (buf == nullptr) return fail("null buffer");
  if (misaligned(buf, e)) return fail("buffer must be aligned to the element size");
  if (R < 1 || R > 32 || (R & (R - 1))) return fail("R must be a power of two in [1, 32]");
  if (P < 0) return fail("P must be >= 0");
  if (a * B < 0xffffffffull && pttwac010_smem_fits((uint32_t)a, (uint32_t)B, R, P))
    return check_launch(launch_pttwac010_smem(s, buf, e, A, (uint32_t)a,
                                              (uint32_t)B, R, P),
                        "010 PTTWAC launch");
  // tile larger than the shared-memory done-bit map: done bits in HBM
  return do_0100(s, buf, e, A, a, B, 1, Method::Pttwac);
}

static bool do_pad(cudaStream_t s, void *buf, int e, int64_t x, int64_t y,
                   int64_t pad, bool padding, uint64_t timeout_ns,
                   int64_t stall_block) {
  if (!valid_e(e)) return fail("element size must be 1, 2, 4 or 8 (got %d)", e);
  if (x < 0 || y < 0 || pad < x) return fail("padding needs 0 <= x <= pad, y >= 0");
  if ((y == 0 || pad == x) && stall_block < 0) return false;
  if (buf == nullptr) return fail("null buffer");
  if (misaligned(buf, e)) return fail("buffer must be aligned to the element size");
  Scratch sc, st;
  if (get_zeroed(sc, pad_scratch_bytes(x, y, pad), s)) return true;
  if (get_zeroed(st, 4, s)) return true;
  cudaError_t err =
      padding ? launch_padding(s, buf, e, x, y, pad, (uint32_t *)sc.p,
                               (uint32_t *)st.p, timeout_ns, stall_block)
              : launch_unpadding(s, buf, e, x, y, pad, (uint32_t *)sc.p,
                                 (uint32_t *)st.p, timeout_ns, stall_block);
  if (err != cudaSuccess) return cuda_fail(err, padding ? "padding" : "unpadding");
  uint32_t status = 0;
  err = cudaMemcpyAsync(&status, st.p, 4, cudaMemcpyDeviceToHost, s);
  if (err == cudaSuccess) err = cudaStreamSynchronize(s);
  if (err != cudaSuccess) return cuda_fail(err, "padding status");
  if (status != kStatusOk)
    return fail("%s: an inter-CTA wait timed out (status %u)",
                padding ? "padding" : "unpadding", status);
  return false;
}

// Staged full transposition [A*a][B*b] -> [B*b][A*a] (src/cl_marshal.cc:561-776).
static bool do_transpose(cudaStream_t s, void *buf, int e, int64_t A,
                         int64_t a, int64_t B, int64_t b, int R, int stages,
                         int variant010) {
  if (!valid_e(e)) return fail("element size must be 1, 2, 4 or 8 (got %d)", e);
  if (A <= 0 || a <= 0 || B <= 0 || b <= 0) return fail("dimensions must be positive");
  auto t010 = [&](int64_t AA, int64_t aa, int64_t BB) -> bool {
    if (variant010 == 2) return do_010_pttwac(s, buf, e, AA, aa, BB, R, 1);
    Method m = variant010 == 1 ? Method::BS : Method::Auto;
    BsPlan p = plan_bs0100(AA, (uint32_t)aa, (uint32_t)BB, 1, e);
    if (!p.feasible && variant010 == 0)
      return do_010_pttwac(s, buf, e, AA, aa, BB, R, 1);
    return do_0100(s, buf, e, AA, aa, BB, 1, m);
  };
  auto t100 = [&](int64_t AA, int64_t BB, int64_t bb) {
    return do_0100(s, buf, e, 1, AA, BB, bb, Method::Auto);
  };
  auto t0100 = [&](int64_t AA, int64_t aa, int64_t BB, int64_t bb) {
    return do_0100(s, buf, e, AA, aa, BB, bb, Method::Auto);
  };
  // Every stage code yields the same final layout, the full transpose
  // [A*a][B*b] -> [B*b][A*a]: with the 010 variant left to the library it
  // runs as one planned 100, which moves 2-4 x payload where the staged
  // sequences move 2 x payload per stage (7200 x 1800: 2.4-7.7 x faster,
  // int8 and fp16 in one launch held in shared memory).  Forced variants run
  // the reference's stages.
  if (variant010 == 0) return t100(A * a, B * b, 1);
  switch (stages) {
    case 2:  // 010(A, a, B*b) -> 100(A, B*b, a)            (:569-601)
      if (a > 1 && t010(A, a, B * b)) return true;
      return t100(A, B * b, a);
    case 22:  // 100(A*a, B, b) -> 010(B, A*a, b)           (:602-634)
      if (t100(A * a, B, b)) return true;
      return b > 1 ? t010(B, A * a, b) : false;
    case 3:  // 100(A*a,B,b) -> 010(B*A,a,b) -> 0100(B,A,b,a) (:636-677)
      if (t100(A * a, B, b)) return true;
      if (a > 1 && t010(B * A, a, b)) return true;
      return t0100(B, A, b, a);
    case 32:  // 0100(A,a,B,b) -> 010(A*B,a,b) -> 100(A,B*b,a) (:679-720)
      if (t0100(A, a, B, b)) return true;
      if (a > 1 && t010(A * B, a, b)) return true;
      return t100(A, B * b, a);
    case 4:  // 0100 -> 010 -> 100(A,B,b*a) -> 0100(B,A,b,a)  (:722-767)
      if (t0100(A, a, B, b)) return true;
      if (t010(B * A, a, b)) return true;
      if (t100(A, B, b * a)) return true;
      return t0100(B, A, b, a);
    default:  // element-wise fallback 0100(1, A*a, B*b, 1)  (:769-775)
      return t0100(1, A * a, B * b, 1);
  }
}

// ---- full transposition of an arbitrary M x N matrix ------------------------
// The reference's flow for general matrices (test/cl_unittest.cc:396-640):
// "Algorithm 5" picks the super-element sizes a | M' and b | N' as the
// largest divisors within [24, floor(sqrt(MAX_MEM))] of M' = M + pad_h and
// N' = N + pad_w, growing each dimension by one until it has such a divisor
// (the test sorts the divisors and takes the largest in range, :420-463);
// "Algorithm 3" picks the stage code (:515-617): 2 if a >= 6 and a*B*b fits
// MAX_MEM, else 22 if b >= 6 and b*A*a fits, else 3 (a <= b) or 32.  MAX_MEM
// is the reference's 48 KB of local memory in elements (12288 for 4-byte,
// 6144 for 8-byte elements, :22-28; 12288 for narrower ones here).
struct FullPlan {
  int64_t A = 0, a = 0, B = 0, b = 0, pad_h = 0, pad_w = 0;
  int stages = 0;
};

static int64_t largest_divisor_in(int64_t n, int64_t lo, int64_t hi) {
  for (int64_t d = std::min(hi, n); d >= lo; --d)
    if (n % d == 0) return d;
  return 0;
}

static FullPlan plan_full(int64_t M, int64_t N, int e) {
  const int64_t max_mem = 49152 / std::max(e, 4);
  int64_t hi = 1;
  while ((hi + 1) * (hi + 1) <= max_mem) ++hi;
  const int64_t lo = 24;
  FullPlan p;
  int64_t h = M, w = N;
  while ((p.a = largest_divisor_in(h, lo, hi)) == 0) ++h;
  while ((p.b = largest_divisor_in(w, lo, hi)) == 0) ++w;
  p.pad_h = h - M;
  p.pad_w = w - N;
  p.A = h / p.a;
  p.B = w / p.b;
  if (p.a >= 6 && p.a * p.B * p.b <= max_mem) p.stages = 2;
  else if (p.b >= 6 && p.b * p.A * p.a <= max_mem) p.stages = 22;
  else p.stages = p.a <= p.b ? 3 : 32;
  return p;
}

}  // namespace lm

using namespace lm;

// ============================================================================
// C ABI
// ============================================================================

extern "C" {

const char *lm_last_error(void) { return g_err.c_str(); }

const char *lm_version(void) { return "libmarshal_gb300 1.0 (sm_103a)"; }

void lm_marshal_finalize(void) {
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) return;
  cycle_cache_clear();
  stash_cache_clear();
  cudaMemPool_t pool;
  if (cudaDeviceGetDefaultMemPool(&pool, dev) == cudaSuccess)
    cudaMemPoolTrimTo(pool, 0);
}

// reference: cl_marshal_finalize (src/cl_marshal.cc:116-119)
void cl_marshal_finalize(void) { lm_marshal_finalize(); }

bool lm_transpose_010_bs(lm_stream_t stream, void *buf, int elem_bytes,
                         int A, int a, int B, unsigned long long *et) {
  OpTimer t(et, (cudaStream_t)stream);
  if (A < 0 || a < 0 || B < 0) return fail("dimensions must be >= 0");
  if (do_0100((cudaStream_t)stream, buf, elem_bytes, (uint64_t)A, (uint64_t)a,
              (uint64_t)B, 1, Method::BS))
    return true;
  return t.finish();
}

bool lm_transpose_010_pttwac(lm_stream_t stream, void *buf, int elem_bytes,
                             int A, int a, int B, unsigned long long *et,
                             int R, int P) {
  OpTimer t(et, (cudaStream_t)stream);
  if (A < 0 || a < 0 || B < 0) return fail("dimensions must be >= 0");
  if (do_010_pttwac((cudaStream_t)stream, buf, elem_bytes, (uint64_t)A,
                    (uint64_t)a, (uint64_t)B, R, P))
    return true;
  return t.finish();
}

bool lm_transpose_100(lm_stream_t stream, void *buf, int elem_bytes, int A,
                      int B, int b, unsigned long long *et) {
  OpTimer t(et, (cudaStream_t)stream);
  if (A < 0 || B < 0 || b < 0) return fail("dimensions must be >= 0");
  if (do_0100((cudaStream_t)stream, buf, elem_bytes, 1, (uint64_t)A,
              (uint64_t)B, (uint64_t)b, Method::Auto))
    return true;
  return t.finish();
}

bool lm_transpose_0100(lm_stream_t stream, void *buf, int elem_bytes, int A,
                       int a, int B, int b, unsigned long long *et) {
  OpTimer t(et, (cudaStream_t)stream);
  if (A < 0 || a < 0 || B < 0 || b < 0) return fail("dimensions must be >= 0");
  if (do_0100((cudaStream_t)stream, buf, elem_bytes, (uint64_t)A, (uint64_t)a,
              (uint64_t)B, (uint64_t)b, Method::Auto))
    return true;
  return t.finish();
}

bool lm_transpose_0100_method(lm_stream_t stream, void *buf, int elem_bytes,
                              int A, int a, int B, int b, int method,
                              unsigned long long *et) {
  OpTimer t(et, (cudaStream_t)stream);
  if (A < 0 || a < 0 || B < 0 || b < 0) return fail("dimensions must be >= 0");
  if (method < 0 || method > 7) return fail("method must be 0..7");
  const Method m = method == 1   ? Method::BS
                   : method == 2 ? Method::Pttwac
                   : method == 3 ? Method::Stash
                   : method == 4 ? Method::TwoPass
                   : method == 5 ? Method::Cycles
                   : method == 6 ? Method::Staged
                   : method == 7 ? Method::Resident
                                 : Method::Auto;
  if (do_0100((cudaStream_t)stream, buf, elem_bytes, (uint64_t)A, (uint64_t)a,
              (uint64_t)B, (uint64_t)b, m))
    return true;
  return t.finish();
}

bool lm_transpose(lm_stream_t stream, void *buf, int elem_bytes, int A, int a,
                  int B, int b, int R, int stages, unsigned long long *et) {
  OpTimer t(et, (cudaStream_t)stream);
  if (do_transpose((cudaStream_t)stream, buf, elem_bytes, A, a, B, b, R,
                   stages, 0))
    return true;
  return t.finish();
}

bool lm_transpose_ex(lm_stream_t stream, void *buf, int elem_bytes, int A,
                     int a, int B, int b, int R, int stages, int variant010,
                     unsigned long long *et) {
  OpTimer t(et, (cudaStream_t)stream);
  if (variant010 < 0 || variant010 > 2) return fail("variant010 must be 0, 1 or 2");
  if (do_transpose((cudaStream_t)stream, buf, elem_bytes, A, a, B, b, R,
                   stages, variant010))
    return true;
  return t.finish();
}

bool lm_full_transpose_plan(int M, int N, int elem_bytes, int *plan7,
                            long long *padded_elems) {
  if (!valid_e(elem_bytes))
    return fail("element size must be 1, 2, 4 or 8 (got %d)", elem_bytes);
  if (M <= 0 || N <= 0) return fail("full transpose: M and N must be > 0");
  const FullPlan p = plan_full(M, N, elem_bytes);
  if (plan7) {
    const int64_t v[7] = {p.A, p.a, p.B, p.b, p.pad_h, p.pad_w, p.stages};
    for (int k = 0; k < 7; ++k) plan7[k] = (int)v[k];
  }
  if (padded_elems)
    *padded_elems = (long long)((M + p.pad_h) * (int64_t)(N + p.pad_w));
  return false;
}

bool lm_full_transpose(lm_stream_t stream, void *buf, int elem_bytes, int M,
                       int N, long long capacity_elems, int variant010,
                       unsigned long long *et) {
  cudaStream_t s = (cudaStream_t)stream;
  if (!valid_e(elem_bytes))
    return fail("element size must be 1, 2, 4 or 8 (got %d)", elem_bytes);
  if (M <= 0 || N <= 0) return fail("full transpose: M and N must be > 0");
  if (variant010 < 0 || variant010 > 2)
    return fail("full transpose: variant010 must be 0, 1 or 2");
  if (buf == nullptr) return fail("null buffer");
  if (misaligned(buf, elem_bytes))
    return fail("buffer must be aligned to the element size");
  const FullPlan p = plan_full(M, N, elem_bytes);
  const int64_t need = variant010 == 0
                           ? (int64_t)M * N
                           : (M + p.pad_h) * (int64_t)(N + p.pad_w);
  if (capacity_elems < need)
    return fail("full transpose: the buffer must hold %lld elements (has %lld)",
                (long long)need, capacity_elems);
  OpTimer t(et, s);
  if (variant010 == 0) {
    // the same permutation without padding: one planned 100
    if (do_0100(s, buf, elem_bytes, 1, M, N, 1, Method::Auto)) return true;
    return t.finish();
  }
  // [M][N] -> [M][N + pad_w] -> transposed [N + pad_w][M + pad_h] (rows past
  // M were never written: their columns become rows past N) -> [N][M]
  if (p.pad_w > 0 && do_pad(s, buf, elem_bytes, N, M, N + p.pad_w, true,
                            2000000000ull, -1))
    return true;
  if (do_transpose(s, buf, elem_bytes, p.A, p.a, p.B, p.b, 1, p.stages,
                   variant010))
    return true;
  if (p.pad_h > 0 && do_pad(s, buf, elem_bytes, M, N, M + p.pad_h, false,
                            2000000000ull, -1))
    return true;
  return t.finish();
}

bool lm_aos_asta_bs(lm_stream_t stream, void *buf, int elem_bytes, int height,
                    int width, int tile_size) {
  if (tile_size <= 0 || height < 0 || width < 0 || height % tile_size)
    return fail("height must be a multiple of tile_size");
  return lm_transpose_010_bs(stream, buf, elem_bytes, height / tile_size,
                             tile_size, width, nullptr);
}

bool lm_aos_asta_pttwac(lm_stream_t stream, void *buf, int elem_bytes,
                        int height, int width, int tile_size, int R, int P) {
  if (tile_size <= 0 || height < 0 || width < 0 || height % tile_size)
    return fail("height must be a multiple of tile_size");
  return lm_transpose_010_pttwac(stream, buf, elem_bytes, height / tile_size,
                                 tile_size, width, nullptr, R, P);
}

bool lm_aos_asta(lm_stream_t stream, void *buf, int elem_bytes, int height,
                 int width, int tile_size, int R) {
  // src/cl_marshal.cc:814-818: BS, and PTTWAC only if BS reported an error.
  return lm_aos_asta_bs(stream, buf, elem_bytes, height, width, tile_size) &&
         lm_aos_asta_pttwac(stream, buf, elem_bytes, height, width, tile_size,
                            R, 1);
}

bool lm_padding(lm_stream_t stream, void *buf, int elem_bytes, int x_size,
                int y_size, int pad_size, unsigned long long *et) {
  OpTimer t(et, (cudaStream_t)stream);
  if (do_pad((cudaStream_t)stream, buf, elem_bytes, x_size, y_size, pad_size,
             true, 2000000000ull, -1))
    return true;
  return t.finish();
}

bool lm_unpadding(lm_stream_t stream, void *buf, int elem_bytes, int x_size,
                  int y_size, int pad_size, unsigned long long *et) {
  OpTimer t(et, (cudaStream_t)stream);
  if (do_pad((cudaStream_t)stream, buf, elem_bytes, x_size, y_size, pad_size,
             false, 2000000000ull, -1))
    return true;
  return t.finish();
}

// Failure-detection hook: runs padding (or unpadding) with task `stall_block`
// waiting on a flag that is never set, bounded by timeout_ns.  Must return
// true (error) with a timeout message and leave the context usable.
bool lm_debug_pad_stall(lm_stream_t stream, void *buf, int elem_bytes,
                        int x_size, int y_size, int pad_size, int unpad,
                        long long stall_block, unsigned long long timeout_ns) {
  return do_pad((cudaStream_t)stream, buf, elem_bytes, x_size, y_size,
                pad_size, unpad == 0, timeout_ns, stall_block);
}

// Failure-detection hook: the resident form of 0100(A, a, B, b) with its
// grid barrier waiting for one arrival more than there are CTAs, bounded by
// timeout_ns.  Must return true (error) with a timeout message, leave the
// buffer as it was (no CTA writes) and the context usable.
bool lm_debug_resident_stall(lm_stream_t stream, void *buf, int elem_bytes,
                             int A, int a, int B, int b,
                             unsigned long long timeout_ns) {
  cudaStream_t s = (cudaStream_t)stream;
  if (!valid_e(elem_bytes))
    return fail("element size must be 1, 2, 4 or 8 (got %d)", elem_bytes);
  if (A <= 0 || a <= 1 || B <= 1 || b <= 0) return fail("dimensions must be positive");
  if (buf == nullptr) return fail("null buffer");
  if (misaligned(buf, elem_bytes))
    return fail("buffer must be aligned to the element size");
  uint32_t *status = device_status_word();
  if (!status) return fail("resident: no status word");
  const cudaError_t err =
      launch_resident0100(s, buf, elem_bytes, (uint64_t)A, (uint64_t)a,
                          (uint64_t)B, (uint64_t)b, status, timeout_ns, 1);
  if (err == cudaErrorNotSupported)
    return fail("resident: the shape does not fit shared memory");
  if (err != cudaSuccess) return cuda_fail(err, "resident launch");
  return check_status(s, "resident");
}

// Waits for `stream` and returns (then clears) the accumulated status of
// waiting kernels on the current device: 0 = ok.
unsigned lm_device_status(lm_stream_t stream) {
  uint32_t *w = device_status_word();
  if (!w) return 0xffffffffu;
  uint32_t v = 0;
  cudaStream_t s = (cudaStream_t)stream;
  if (cudaMemcpyAsync(&v, w, 4, cudaMemcpyDeviceToHost, s) != cudaSuccess ||
      cudaStreamSynchronize(s) != cudaSuccess)
    return 0xffffffffu;
  if (v) cudaMemsetAsync(w, 0, 4, s);
  return v;
}

int lm_tune_entries(void) {
  std::lock_guard<std::mutex> lock(g_tune_mu);
  tune_load_locked();
  return (int)g_tune.size();
}

// Pins (variant >= 0) or reads (variant < 0) the tuned variant of the shape
// class of 0100(T, a, B, b) on elem_bytes elements; returns the class's
// variant afterwards, or -1 when it has none (or the arguments are bad).
int lm_tune_variant(int elem_bytes, long long T, long long a, long long B,
                    long long b, int variant) {
  if (!valid_e(elem_bytes) || T <= 0 || a <= 0 || B <= 0 || b <= 0 ||
      variant >= kNumVariants)
    return -1;
  int e = elem_bytes;
  uint64_t bb = (uint64_t)b;
  widen_units(nullptr, &e, &bb);  // the class is keyed on the wide unit
  const TuneKey key{e, ilog2((uint64_t)a), ilog2((uint64_t)B), ilog2(bb),
                    T > 1 ? 1 : 0};
  std::lock_guard<std::mutex> lock(g_tune_mu);
  tune_load_locked();
  if (variant >= 0) g_tune[key] = variant;
  auto it = g_tune.find(key);
  return it == g_tune.end() ? -1 : it->second;
}

// Planner query used by the Python API's IsFeasible(): 1 when the 0100 tile
// [a][B][b] of elem_bytes elements can be staged on chip (BS), else 0.
int lm_bs_feasible(long long T, int a, int B, int b, int elem_bytes) {
  if (!valid_e(elem_bytes) || T <= 0 || a <= 0 || B <= 0 || b <= 0) return 0;
  return plan_bs0100((uint64_t)T, (uint32_t)a, (uint32_t)B, (uint32_t)b,
                     elem_bytes).feasible ? 1 : 0;
}

// ---- reference CUDA drop-ins (include/marshal.h:26-31) ----------------------
// Same signatures; launch on the legacy default stream like the reference
// (src/marshal.cu:27-80).  `timer` is accepted and left untouched, as the
// reference kernels never write it.

bool gpu_aos_asta_bs_float(float *src, int height, int width, int tile_size,
                           clock_t *timer) {
  (void)timer;
  return lm_aos_asta_bs(nullptr, src, 4, height, width, tile_size);
}

bool gpu_aos_asta_bs_double(double *src, int height, int width, int tile_size,
                            clock_t *timer) {
  (void)timer;
  return lm_aos_asta_bs(nullptr, src, 8, height, width, tile_size);
}

bool gpu_aos_asta_pttwac(float *src, int height, int width, int tile_size,
                         clock_t *timer) {
  (void)timer;
  return lm_aos_asta_pttwac(nullptr, src, 4, height, width, tile_size, 1, 0);
}

bool gpu_soa_asta_pttwac(float *src, int height, int width, int tile_size,
                         clock_t *timer) {
  (void)timer;
  // [w][h/t][t] -> [h/t][w][t] == 100(A=w, B=h/t, b=t)
  if (tile_size <= 0 || height < 0 || width < 0 || height % tile_size)
    return fail("height must be a multiple of tile_size");
  return lm_transpose_100(nullptr, src, 4, width, height / tile_size,
                          tile_size, nullptr);
}

}  // extern "C"
