// lm_internal.h -- interface between the host dispatch (lm_api.cu) and the
// kernel launchers.  Every launcher is stream-ordered, allocates nothing
// (scratch is passed in) and returns cudaSuccess or the launch error.
#pragma once

#include <atomic>
#include <cstddef>
#include <cstdint>
#include <cuda_runtime.h>

namespace lm {

struct DeviceInfo {
  int device = -1;
  int sms = 0;
  int max_smem_optin = 0;   // bytes per CTA, opt-in maximum
  int max_smem_per_sm = 0;
  int cc_major = 0, cc_minor = 0;
};
const DeviceInfo &device_info();  // current device, cached

// Records `msg` as the calling thread's lm_last_error(); returns true.
bool set_error(const char *msg);

// Every kernel launch of the library is wrapped in a ProfScope: it counts the
// launch and, while profiling is on (lm_prof_enable), records a CUDA event
// pair around it on the launching stream (lm_prof.cu).
class ProfScope {
 public:
  ProfScope(cudaStream_t s, const char *name);
  ~ProfScope();
  ProfScope(const ProfScope &) = delete;
  ProfScope &operator=(const ProfScope &) = delete;

 private:
  cudaStream_t s_;
  const char *name_;
  void *a_ = nullptr, *b_ = nullptr;
};

// ---- 0100 by barrier-synchronised tiles in shared memory ------------------
// [T][a][B][b] -> [T][B][a][b]; elements of e bytes.  Each tile (a*B*b*e
// bytes) is staged on chip: several tiles per CTA when small, one tile per
// CTA, or one tile spread over a thread-block cluster (distributed shared
// memory) when it exceeds one CTA's shared memory.
struct BsPlan {
  bool feasible = false;
  int cluster = 1;             // CTAs per tile (1, 2, 4, 8 or 16)
  uint32_t tiles_per_chunk = 1;
  uint32_t rows_per_cta = 0;   // rows of B*b elements held by one CTA
  uint32_t pitch = 0;          // shared-memory bytes per row
  size_t smem_bytes = 0;       // per CTA
  int threads = 512;
};
BsPlan plan_bs0100(uint64_t T, uint32_t a, uint32_t B, uint32_t b, int e,
                   size_t smem_budget = 0 /*0: device maximum*/);
cudaError_t launch_bs0100(cudaStream_t s, void *buf, int e, uint64_t T,
                          uint32_t a, uint32_t B, uint32_t b,
                          const BsPlan &plan);

// ---- launch preparation cache ---------------------------------------------
// A kernel's dynamic shared-memory limit is raised only when a launch needs
// more than any before it on this device, and its occupancy is remembered
// for the last size asked: small conversions are bound by host time per
// call, and these driver queries cost about as much as the launch itself.
struct LaunchCache {
  std::atomic<int> smem_set[8];       // per device: largest limit set (+1)
  std::atomic<uint64_t> occ_key[8];   // per device: (smem << 16) | occupancy
};
// Sets the attribute if needed and returns the CTAs per SM for `threads`
// threads and `smem` dynamic bytes (0 on error, with *err set).
int prepare_launch(const void *kern, LaunchCache &c, size_t smem, int threads,
                   cudaError_t *err);

// ---- per-shape-class tuning overrides ---------------------------------------
// The autotuner (lm_api.cu, run_0100_planned) picks a method and a variant
// of it per shape class; the variant reaches the plan builders through
// these thread-local overrides, set only around the tuned call (0: the
// built-in choice).
struct TuneParams {
  uint32_t staged_block_bytes = 0;  // staged form: bytes staged per block
  int stash_per_sm = 0;             // stash plan: CTAs per SM (1 or 2)
  // staged form: square blocks of S x S units get S * staged_wide columns
  // (0 or 1: square)
  uint32_t staged_wide = 0;
};
TuneParams &tune_params();

// True on a thread while the batch executor runs planner jobs beside its
// other kernels: the planner then takes no whole-GPU cooperative form (its
// launch would wait for every SM to drain).
bool &planner_beside_other_work();

// ---- planner thresholds (the per-op planner and the batch executor) ------
// Measured on GB300 with 256 MB matrices: the staged form (4 x payload
// through scratch) beats cycle following on units below 512 bytes, ties it
// from 512 to 1023 bytes on one tile and beats it on many small tiles
// (0100(18, 72, 100, 100) of 800-byte units: 2.49 vs 1.60 TB/s); the
// stash (3 x payload) needs about 48 rows per SM to keep its wavefront fed,
// and below that the staged form is faster.
constexpr uint64_t kStagedMaxUnit = 1024;
constexpr uint64_t kStashRowsPerSm = 48;

// ---- 010 tiles with 16-byte accesses (lm_tile010.cu) ----------------------
// [T][a][B] -> [T][B][a] for a 16-byte aligned buffer whose tiles hold at
// most 32 KB and have a*e or B*e a multiple of 16 bytes.
bool tile010_applies(const void *buf, int e, uint64_t T, uint64_t a,
                     uint64_t B);
cudaError_t launch_tile010(cudaStream_t s, void *buf, int e, uint64_t T,
                           uint32_t a, uint32_t B);

// ---- 0100 by cycle following with done-bits in global memory -------------
// A instances of 100(a, B, b): units of b*e bytes; one done bit per unit.
// `flags` must hold pttwac_flag_bytes(...) zeroed bytes.
size_t pttwac_flag_bytes(const void *buf, uint64_t T, uint32_t a, uint32_t B,
                         uint32_t b, int e);
cudaError_t launch_pttwac0100(cudaStream_t s, void *buf, int e, uint64_t T,
                              uint32_t a, uint32_t B, uint32_t b,
                              uint32_t *flags);
// Queries (and so loads, where modules load lazily) every variant of the
// kernel behind launch_pttwac0100 on the current device, so that later
// launches do no first-use work.
cudaError_t pttwac_prepare();

// ---- 010 by in-tile cycle following with done-bits in shared memory ------
// [A][a][B] -> [A][B][a].  R is the spreading factor of the done-bit map
// (power of two, 1..32) and P the padding words per 32 flag words.
bool pttwac010_smem_fits(uint32_t a, uint32_t B, int R, int P);
cudaError_t launch_pttwac010_smem(cudaStream_t s, void *buf, int e,
                                  uint64_t A, uint32_t a, uint32_t B, int R,
                                  int P);

// ---- 100 for small units with 3 x payload traffic (lm_stash.cu) ---------
// K1 saves the half of the matrix that is overwritten before it is read; K2
// is a persistent wavefront over column groups with per-chunk progress
// counters and bounded waits (status word on timeout).
struct StashPlan {
  bool feasible = false;
  uint32_t g = 0, G = 0;       // units per column group, groups
  uint32_t W = 0, nchunks = 0; // rows per chunk, chunks (= CTAs)
  uint32_t pitch = 0;          // shared bytes per gathered row
  size_t smem_bytes = 0;
  int ctas_per_sm = 1;
  uint32_t margin = 0;         // steps of slack between CTAs
  uint64_t A = 0;              // rows (the row-offset table has A+1 words)
  size_t stash_bytes = 0;
};
StashPlan plan_stash(uint64_t A, uint64_t B, uint32_t b, int e);
size_t stash_scratch_bytes(const StashPlan &p);  // scratch to pass
// Byte range of that scratch that must be zero before the launch (the
// progress counters); the rest is fully written before it is read.
size_t stash_zero_offset(const StashPlan &p);
size_t stash_zero_bytes(const StashPlan &p);
// Frees the cached stash row-offset tables of the current device.
void stash_cache_clear();
cudaError_t launch_stash100(cudaStream_t s, void *buf, int e, uint64_t A,
                            uint64_t B, uint32_t b, const StashPlan &p,
                            void *scratch, uint32_t *status,
                            uint64_t timeout_ns);

// ---- whole-cycle moves (lm_cycles.cu) ----------------------------------------
// Cycles held in registers: at most this many units.
constexpr uint32_t kCycleMaxLen = 32;
// Multiplicative order of a modulo a*B - 1 (the length every cycle of a
// 100(a, B) divides), or 0 when it exceeds `limit` or a*B - 1 >= 2^32.
uint32_t cycle_order(uint64_t a, uint64_t B, uint32_t limit);
size_t cycle_scratch_bytes(uint64_t a, uint64_t B);
// Frees the cached cycle-leader lists of the current device (waits for
// their readers).
void cycle_cache_clear();
// T instances of 100(a, B, b) whose cycles have at most L <= kCycleMaxLen
// units.  `scratch` holds cycle_scratch_bytes(a, B) bytes; with may_cache
// (never while the stream is being captured) the cycle leaders come from a
// per-device cache of shapes, else they are computed into the scratch.
cudaError_t launch_cycles100(cudaStream_t s, void *buf, int e, uint64_t T,
                             uint32_t a, uint32_t B, uint32_t b, uint32_t L,
                             void *scratch, bool may_cache);

// ---- 0100 through scratch (lm_batch.cu) -------------------------------------
// The blocks of every tile transposed through shared memory into `scratch`
// (T*a*B*b*e bytes, out of place), then copied back over the buffer: 4 x
// payload traffic, any shape whose unit is at most 32 KB.
bool staged0100_applies(uint64_t T, uint64_t a, uint64_t B, uint64_t b, int e);
cudaError_t launch_staged0100(cudaStream_t s, void *buf, int e, uint64_t T,
                              uint64_t a, uint64_t B, uint64_t b,
                              void *scratch);

// ---- 0100 held whole in shared memory (lm_batch.cu) -------------------------
// Payloads that fit the shared memory of all SMs (about 30 MB on GB300): the
// staged form's blocks loaded by every CTA, a grid barrier, then written
// transposed over the buffer: one cooperative launch, 2 x payload.
// cudaErrorNotSupported when the shape does not fit or the stream is being
// captured.  A barrier wait that runs out sets `status` and skips the writes
// (`missing` > 0, a failure-detection test: the barrier waits for that many
// arrivals more than there are CTAs).
bool resident0100_applies(uint64_t T, uint64_t a, uint64_t B, uint64_t b,
                          int e);
cudaError_t launch_resident0100(cudaStream_t s, void *buf, int e, uint64_t T,
                                uint64_t a, uint64_t B, uint64_t b,
                                uint32_t *status, uint64_t timeout_ns,
                                uint32_t missing = 0);

// A 0100 moves whole units of b elements, so the same byte permutation is a
// 0100 over elements of any width w dividing the unit's b*e bytes.  Widens
// *e to the largest such w up to 8 that also divides the buffer address, and
// rescales *b (fewer, wider accesses in every kernel); b == 1 is unchanged.
inline void widen_units(const void *buf, int *e, uint64_t *b) {
  if (*b <= 1) return;
  const uint64_t U = *b * (uint64_t)*e;
  int w = 8;
  while (w > *e && (U % (uint64_t)w || (uintptr_t)buf % (uintptr_t)w)) w >>= 1;
  if (w > *e) {
    *b = U / (uint64_t)w;
    *e = w;
  }
}

// An LM_OP_* with its dimensions as the 0100(T, a, B, b) it performs; false
// for an unknown op or bad dimensions (lm_batch.cu).
bool op_as_0100(int op, long long d0, long long d1, long long d2, long long d3,
                uint64_t *T, uint64_t *a, uint64_t *B, uint64_t *b);

// The per-op planner (lm_api.cu) for one 0100; tune != 0 lets the
// autotuner pick the algorithm of this shape class.
bool run_0100_planned(cudaStream_t s, void *buf, int e, uint64_t T,
                      uint64_t a, uint64_t B, uint64_t b, int tune);

// Keeps the current device's stream-ordered pool from returning freed
// blocks to the system (scratch and arenas are reused call after call).
void pool_keep_memory();

// Per-device persistent status word that waiting kernels OR their failures
// into (allocated on first use); lm_api.cu reads and clears it.
uint32_t *device_status_word();

// ---- row padding / unpadding with bounded inter-CTA waits ----------------
// padding:   [y][x] -> [y][pad] (new columns zero)
// unpadding: [y][pad] -> [y][x], tail y*x..y*pad-1 zero.
// `scratch` must hold pad_scratch_bytes(...) zeroed bytes; `status` one
// zeroed word that the kernel sets to kStatusWaitTimeout when a wait runs
// out.  stall_block >= 0 makes that block wait on a flag nothing sets
// (failure-detection test hook).
size_t pad_scratch_bytes(uint64_t x, uint64_t y, uint64_t pad);
cudaError_t launch_padding(cudaStream_t s, void *buf, int e, uint64_t x,
                           uint64_t y, uint64_t pad, uint32_t *scratch,
                           uint32_t *status, uint64_t timeout_ns,
                           int64_t stall_block);
cudaError_t launch_unpadding(cudaStream_t s, void *buf, int e, uint64_t x,
                             uint64_t y, uint64_t pad, uint32_t *scratch,
                             uint32_t *status, uint64_t timeout_ns,
                             int64_t stall_block);

}  // namespace lm
