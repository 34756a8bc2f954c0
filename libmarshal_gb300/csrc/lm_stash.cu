// lm_stash.cu -- in-place 100 for small super-elements with 3 x payload traffic.
//
// The reference moves small super-elements by cycle following
// (_transpose_100, src/cl/cl_aos_asta.cl:352-569): for the plain transpose
// (b = 1) every step is a dependent 4-byte access.  Cycle following on
// cache-line units needs a preceding 010 pass, i.e. two full passes (4 x
// payload bytes).  This file implements a streaming alternative that moves
// 3 x payload bytes and only touches memory in >= 128-byte runs:
//
//   [A][B] units -> [B][A].  Destination rows are produced in groups of g
//   (one group = g source columns, a column strip of the source) in order
//   J = 0, 1, ...; group J's destination region D_J is the address range
//   [g*J*A, g*(J+1)*A) of the buffer.  A source unit at address x = i*B + j
//   is overwritten when its region J(x) = x / (g*A) is written and consumed
//   when its column group j / g is gathered.  Units whose region comes first
//   must be saved: for group J these are exactly the rows i < r(J) =
//   ceil(g*J*(A-1)/B) (half of the matrix over all J).
//
//   Row i is read from the stash by every group J >= J_i (the first group
//   with i < r(J)), so the stash holds one contiguous suffix per row: units
//   [J_i*g, B) of row i, at the same address modulo 16 as in the buffer.
//   K0 (k_stash_offsets) lays the suffixes out; K1 (k_stash_save) copies
//   them with 16-byte vectors (a memcpy of half the data).
//   K2 (k_stash_wave): a persistent grid; CTA c owns the source rows
//   [c*W, (c+1)*W).  For each J it gathers its rows' group-J strip (from the
//   stash for i < r(J), from the buffer otherwise) into shared memory,
//   publishes progress[c] = J+1, waits until every CTA whose rows hold
//   original data inside its destination range has gathered group J, and
//   writes its W units into each of the g destination rows.  Every wait is
//   on a CTA that never waits for a later step, so the waits end; each one
//   is also bounded by %globaltimer and reports through a status word.
#include <algorithm>
#include <cstdio>
#include <cstdlib>
#include <map>
#include <mutex>
#include <tuple>

#include "lm_core.cuh"
#include "lm_internal.h"

namespace lm {

struct StashArgs {
  char *base;
  char *stash;
  const uint64_t *roff;  // byte offset of each row's stash suffix, A+1
  uint32_t *progress;    // one counter per row chunk
  uint32_t progress_words;  // cleared by K1 before the wave starts
  uint32_t *status;
  uint64_t A, B;         // rows, columns (units)
  uint32_t b;            // elements per unit
  uint32_t e;            // bytes per element
  uint32_t g;            // units per column group
  uint32_t G;            // groups
  uint32_t W;            // rows per chunk
  uint32_t nchunks;
  uint32_t pitch;        // shared bytes per gathered row
  uint32_t gb;           // g*b elements per full strip row
  FastDiv div_gb;
  FastDiv div_b;
  uint64_t timeout_ns;
  uint32_t margin;       // stash margin k (steps of slack between CTAs)
  uint32_t tma;          // 1: gather rows with bulk copies, 0: cp.async
  uint32_t jcut;         // K1 saves the wave's first jcut steps' strips last
  // first stashed group of a row (stash_first_group) without a division:
  // i*B and g*(A-1) are < 2^32
  uint64_t gAk;          // g*A*margin
  FastDiv div_D;         // g*(A-1)
  FastDiv div_Bc, div_Wc;  // B and W (chunk of a position)
};

__device__ __forceinline__ uint64_t first_group(uint64_t i, const StashArgs &g) {
  const uint64_t lhs = i * g.B;
  return lhs < g.gAk ? 0 : (uint64_t)fdiv((uint32_t)(lhs - g.gAk), g.div_D) + 1;
}

// Bytes of one ring stage: W rows of `pitch` bytes, then W uint32 row
// offsets; rounded to 128 so every stage (a bulk-copy destination) stays
// 16-byte aligned.
__host__ __device__ __forceinline__ size_t stash_stage_bytes(uint64_t W,
                                                             uint32_t pitch) {
  return (size_t)((W * pitch + W * 4 + 127) / 128 * 128);
}

// Rows whose group-J strip is saved: r(J) = ceil((g*A*(J+k) - g*J) / B), at
// most A.  With margin k = 0 these are exactly the rows overwritten before
// they are consumed; a margin k > 0 also saves the rows overwritten within k
// steps after consumption (about k*g*A/B rows per step), so that a write of
// step J depends only on gathers of steps <= J-k: the CTAs are no longer in
// lockstep.
__host__ __device__ __forceinline__ uint64_t stash_rows(uint64_t J, uint64_t g,
                                                        uint64_t A, uint64_t B,
                                                        uint64_t k) {
  const uint64_t num = g * A * (J + k) - g * J;
  const uint64_t r = (num + B - 1) / B;
  return r < A ? r : A;
}

// First group J_i that reads row i from the stash: the smallest J with
// i < r(J), i.e. g*(A-1)*J > i*B - g*A*k.  J_i >= G: row i is not stashed.
__host__ __device__ __forceinline__ uint64_t stash_first_group(
    uint64_t i, uint64_t g, uint64_t A, uint64_t B, uint64_t k) {
  const uint64_t lhs = i * B, rhs = g * A * k;
  return lhs < rhs ? 0 : (lhs - rhs) / (g * (A - 1)) + 1;
}

// Bytes of row i's stash slot: the suffix rounded up to 16 bytes, plus 16
// so the data can start at its buffer address modulo 16.
__host__ __device__ __forceinline__ uint64_t stash_slot_bytes(
    uint64_t i, uint64_t g, uint64_t A, uint64_t B, uint64_t G, uint64_t U,
    uint64_t k) {
  const uint64_t Ji = stash_first_group(i, g, A, B, k);
  if (Ji >= G) return 0;
  return ((B - Ji * g) * U + 15) / 16 * 16 + 16;
}

// K0: per-row stash offsets, one block of 32 warps: warp w owns a contiguous
// range of rows and walks it 32 rows at a time (lane l: row base + l, so
// the table writes are coalesced), with warp-shuffle scans; a first pass
// sums each warp's range, the 32 sums are scanned, a second pass writes
// roff[i] = slot start + (buffer address of the row's suffix mod 16).
__global__ void __launch_bounds__(1024) k_stash_offsets(StashArgs sa) {
  __shared__ uint64_t warp_tot[32];
  uint64_t *roff = const_cast<uint64_t *>(sa.roff);
  const uint64_t A = sa.A, B = sa.B, g = sa.g, G = sa.G;
  const uint64_t U = (uint64_t)sa.b * sa.e;
  const uint32_t lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const uint64_t per = (A + 31) / 32;
  const uint64_t r0 = min64(A, (uint64_t)warp * per), r1 = min64(A, r0 + per);
  auto slot = [&](uint64_t Ji) -> uint64_t {
    return Ji >= G ? 0 : ((B - Ji * g) * U + 15) / 16 * 16 + 16;
  };
  uint64_t sum = 0;  // lane-private partial of this warp's range
  for (uint64_t i = r0 + lane; i < r1; i += 32) sum += slot(first_group(i, sa));
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) sum += __shfl_xor_sync(kFull, sum, o);
  if (lane == 0) warp_tot[warp] = sum;
  __syncthreads();
  if (warp == 0) {
    uint64_t w = warp_tot[lane];
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const uint64_t v = __shfl_up_sync(kFull, w, o);
      if (lane >= (uint32_t)o) w += v;
    }
    warp_tot[lane] = w;  // inclusive over warps
  }
  __syncthreads();
  uint64_t carry = warp ? warp_tot[warp - 1] : 0;
  for (uint64_t base_i = r0; base_i < r1; base_i += 32) {
    const uint64_t i = base_i + lane;
    uint64_t Ji = 0, sz = 0;
    if (i < r1) {
      Ji = first_group(i, sa);
      sz = slot(Ji);
    }
    uint64_t inc = sz;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const uint64_t v = __shfl_up_sync(kFull, inc, o);
      if (lane >= (uint32_t)o) inc += v;
    }
    if (i < r1) {
      const uintptr_t src = (uintptr_t)sa.base + (i * B + Ji * g) * U;
      roff[i] = carry + inc - sz + (src & 15);
    }
    carry += __shfl_sync(kFull, inc, 31);
  }
  if (threadIdx.x == 1023) roff[A] = warp_tot[31];
}

// K1: copy every row's stash suffix: one warp per row at a time, 16-byte
// vectors between the (equally misaligned) buffer and stash addresses, the
// ragged head and tail bytes one by one.  (Splitting the stash into equal
// contiguous ranges per warp balances the work but ran 30-60 % slower: the
// warps' streams then sit a fixed distance apart in memory, while suffixes
// of different lengths keep them staggered; this form runs at the speed of
// a plain copy of the same bytes.)  In two passes: first the part of
// each suffix that the wave reads after its first jcut steps, with
// evict-first stores, then the part those steps read (their strips, about
// 30 MB for the fp32 16384 x 12289 transposition), with evict-last stores,
// so that most of it is still in L2 when the wave starts (0.8 % faster).
constexpr int kSaveThreads = 256;
constexpr uint32_t kStashEarlySteps = 20;

// Copies n bytes from src to dst (equal addresses modulo 16) with one warp;
// last: evict-last stores under `policy`, else evict-first stores.
__device__ __forceinline__ void save_bytes(const char *src, char *dst,
                                           uint64_t n, uint32_t lane,
                                           bool last, uint64_t policy) {
  const uint64_t head = min64((16 - ((uintptr_t)src & 15)) & 15, n);
  const uint64_t nvec = (n - head) / 16;
  const uint64_t tail0 = head + nvec * 16;
  if (lane < head) dst[lane] = src[lane];
  if (lane < n - tail0) dst[tail0 + lane] = src[tail0 + lane];
  const uint4 *vs = reinterpret_cast<const uint4 *>(src + head);
  uint4 *vd = reinterpret_cast<uint4 *>(dst + head);
  for (uint64_t v = lane; v < nvec; v += 32 * 4) {
    uint4 x[4];
#pragma unroll
    for (int u = 0; u < 4; ++u)
      if (v + 32 * u < nvec) x[u] = __ldcs(vs + v + 32 * u);
#pragma unroll
    for (int u = 0; u < 4; ++u) {
      if (v + 32 * u >= nvec) continue;
      if (last) st_hint16(vd + v + 32 * u, x[u], policy);
      else __stcs(vd + v + 32 * u, x[u]);
    }
  }
}

__global__ void __launch_bounds__(kSaveThreads) k_stash_save(StashArgs g) {
  // the wave may be scheduled onto SMs as this grid's blocks drain
  asm volatile("griddepcontrol.launch_dependents;" ::: "memory");
  const uint32_t lane = threadIdx.x & 31;
  // the wave's progress counters start at zero (K2 runs after K1)
  for (uint32_t x = blockIdx.x * kSaveThreads + threadIdx.x;
       x < g.progress_words; x += gridDim.x * kSaveThreads)
    g.progress[x] = 0u;
  const uint64_t gw = ((uint64_t)blockIdx.x * kSaveThreads + threadIdx.x) >> 5;
  const uint64_t nw = ((uint64_t)gridDim.x * kSaveThreads) >> 5;
  const uint64_t U = (uint64_t)g.b * g.e;
  const uint64_t pol_last = l2_policy_evict_last();
  for (int pass = 0; pass < 2; ++pass) {
    for (uint64_t i = gw; i < g.A; i += nw) {
      const uint64_t Ji = first_group(i, g);
      if (Ji >= g.G) continue;
      const char *src = g.base + (i * g.B + Ji * g.g) * U;
      char *dst = g.stash + g.roff[i];
      const uint64_t n = (g.B - Ji * g.g) * U;
      // strips J_i .. jcut-1 of the row: its first (jcut - J_i) strips
      const uint64_t early =
          Ji < g.jcut ? min64(n, (g.jcut - Ji) * (uint64_t)g.g * U) : 0;
      if (pass == 0)
        save_bytes(src + early, dst + early, n - early, lane, false, pol_last);
      else
        save_bytes(src, dst, early, lane, true, pol_last);
    }
  }
}

// K2: the wavefront, warp-specialised.  Per CTA:
//   warps 0-3 (producers): gather step J into ring stage J % kStages (one
//     bulk copy per row of a 16-byte aligned superset of its strip, each
//     issued by the producer thread that owns the row, rowoff[] records
//     where the strip starts; or, with cp.async, all four warps copy
//     16-byte pieces); completion lands on `full`;
//   warp 4 (publisher): when stage J has landed, publishes progress = J+1;
//   warp 5 (checker): waits for the CTAs whose rows hold original data in
//     step J's destination range, then marks the stage `ready`;
//   warps 6.. (writers): write step J from the stage, then free it (`empty`,
//     which the publisher also arrives on).
// Every wait is bounded by %globaltimer; a timeout sets the status word and
// all roles stop.
constexpr int kWaveThreads = 512;
constexpr int kStages = 3;
constexpr int kProducerWarps = 4;
constexpr int kPublisherWarp = kProducerWarps;
constexpr int kCheckerWarp = kProducerWarps + 1;
constexpr int kWriterWarps = kWaveThreads / 32 - kProducerWarps - 2;
constexpr uint32_t kCheckAhead = 4;  // steps whose chunks the checker prefetches
constexpr int kMaxRowBlocks = 4;  // rows per chunk <= 128
constexpr uint32_t kStashMargin = 2;
constexpr uint32_t kMaxChunks = 1024;  // CTAs of the wave (co-resident)
constexpr uint32_t kProgStride = 32;   // one 128-byte line per progress word

template <int E>
__global__ void __launch_bounds__(kWaveThreads, 2) k_stash_wave(StashArgs g) {
  using T = typename Elem<E>::T;
  extern __shared__ __align__(128) unsigned char smem[];
  __shared__ __align__(8) uint64_t full[kStages], ready[kStages],
      empty[kStages];  // ready = dependencies satisfied
  __shared__ volatile int s_ok;
  __shared__ volatile int s_pstop;  // producers only: stop at this step
  __shared__ uint32_t seen[kMaxChunks];  // poller: last progress read
  const uint32_t ch = blockIdx.x;
  const uint64_t i0 = (uint64_t)ch * g.W;
  if (i0 >= g.A) return;
  const uint32_t Wc = (uint32_t)min64(g.W, g.A - i0);
  const uint32_t warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const uint32_t U = g.b * E;
  // stage s: rows at smem + s*stage_sz, row offsets (uint32) after the rows
  const size_t rows_sz = (size_t)g.W * g.pitch;
  const size_t stage_sz = stash_stage_bytes(g.W, g.pitch);
  auto stage = [&](uint32_t s) { return smem + s * stage_sz; };
  auto rowoff = [&](uint32_t s) {
    return reinterpret_cast<uint32_t *>(smem + s * stage_sz + rows_sz);
  };
  if (threadIdx.x == 0) {
    for (int s = 0; s < kStages; ++s) {
      mbar_init(&full[s], g.tma ? (uint32_t)kProducerWarps : kProducerWarps * 32u);
      mbar_init(&ready[s], 1);
      // freed by every writer warp and by the publisher, so a stage is not
      // refilled (its `full` barrier not completed again) before the
      // publisher has seen the step in it: a parity wait that fell a whole
      // ring behind would otherwise wait for the wrong phase
      mbar_init(&empty[s], kWriterWarps + 1);
    }
    fence_mbar_init();
    s_ok = 1;
    s_pstop = 0;
  }
  for (uint32_t c = threadIdx.x; c < kMaxChunks; c += blockDim.x) seen[c] = 0;
  // launched as a programmatic dependent of K1: everything above ran while
  // K1's last blocks were finishing; K1's writes (stash, cleared progress
  // counters) are visible after this wait (a no-op without the attribute)
  asm volatile("griddepcontrol.wait;" ::: "memory");
  __syncthreads();

  // bounded wait; false on timeout or when another role has failed
  auto wait_bar = [&](uint64_t *bar, uint32_t parity) {
    const uint64_t t0 = global_timer_ns();
    while (!mbar_try_wait(bar, parity)) {
      if (!s_ok) return false;
      if (global_timer_ns() - t0 > g.timeout_ns) {
        atomicOr(g.status, kStatusWaitTimeout);
        s_ok = 0;
        return false;
      }
    }
    return true;
  };

  if (warp < kProducerWarps) {
    // ---------------- producers ----------------
    const uint32_t pt = threadIdx.x;  // 0 .. 127
    constexpr uint32_t kP = kProducerWarps * 32;
    uint32_t issued = 0;
    // with bulk copies each producer thread owns one row of the chunk (a
    // warp issues its lanes' copies one after another, so the rows are
    // spread over the four warps): row t = 4 * lane + warp, its first
    // stashed group and stash offset
    const uint32_t my_t = lane * kProducerWarps + warp;
    const bool my_row = g.tma && my_t < Wc;
    const uint64_t my_Ji = my_row ? first_group(i0 + my_t, g) : ~0ull;
    const uint64_t my_ro = my_row ? g.roff[i0 + my_t] : 0;
    for (uint32_t J = 0; J < g.G; ++J) {
      const uint32_t s = J % kStages;
      const uint64_t col0 = (uint64_t)J * g.g;
      const uint32_t len = (uint32_t)min64(g.g, g.B - col0) * U;
      unsigned char *sb = stage(s);
      // row i's strip: from its stash suffix when J >= J_i
      auto strip = [&](uint64_t i, uint64_t Ji, uint64_t ro) -> const char * {
        return J >= Ji ? g.stash + ro + (col0 - Ji * g.g) * U
                       : g.base + (i * g.B + col0) * U;
      };
      bool stop = !s_ok;
      if (!stop && J >= kStages)
        stop = !wait_bar(&empty[s], ((J / kStages) - 1) & 1);
      // the four producer warps take the same decision: s_pstop is written
      // only before the first barrier and read only between the two
      if (stop) s_pstop = 1;
      asm volatile("bar.sync 1, %0;" ::"n"(kP) : "memory");
      const bool stop_all = s_pstop != 0;
      // bulk copies: every producer warp arrives on the stage with the
      // bytes of its rows before the second barrier, so all expected bytes
      // are counted before any copy starts
      uintptr_t my_a0 = 0;
      uint32_t my_bytes = 0;
      if (g.tma && !stop_all) {
        if (my_row) {
          const char *src = strip(i0 + my_t, my_Ji, my_ro);
          my_a0 = (uintptr_t)src & ~(uintptr_t)15;
          my_bytes = (uint32_t)((((uintptr_t)src + len + 15) & ~(uintptr_t)15) - my_a0);
          rowoff(s)[my_t] = my_t * g.pitch + (uint32_t)((uintptr_t)src - my_a0);
        }
        uint32_t bytes = my_bytes;
#pragma unroll
        for (int o = 16; o > 0; o >>= 1)
          bytes += __shfl_xor_sync(kFull, bytes, o);
        if (lane == 0) mbar_arrive_expect_tx(&full[s], bytes);
      }
      asm volatile("bar.sync 1, %0;" ::"n"(kP) : "memory");
      if (stop_all) {
        s_ok = 0;
        break;
      }
      issued = J + 1;
      if (g.tma) {
        // one bulk copy per row (16-byte aligned superset)
        if (my_bytes) {
          fence_proxy_async_smem();
          bulk_g2s(sb + (size_t)my_t * g.pitch, (const void *)my_a0, my_bytes,
                   &full[s]);
        }
      } else {
        // 16-byte chunks per row (upper bound; chunks past the strip skipped)
        const uint32_t nc = (len + 15) / 16 + 1;
        for (uint32_t w = pt; w < Wc * nc; w += kP) {
          const uint32_t t = w / nc, c = w - t * nc;
          const uint64_t i = i0 + t;
          const char *src = strip(i, first_group(i, g), g.roff[i]);
          const uintptr_t a0 = (uintptr_t)src & ~(uintptr_t)15;
          const uintptr_t a1 = ((uintptr_t)src + len + 15) & ~(uintptr_t)15;
          if (c == 0)
            rowoff(s)[t] = t * g.pitch + (uint32_t)((uintptr_t)src - a0);
          if (a0 + 16 * (uintptr_t)c < a1)
            cp_async16(sb + (size_t)t * g.pitch + 16 * c,
                       (const void *)(a0 + 16 * (uintptr_t)c));
        }
        cp_async_mbar_arrive_noinc(&full[s]);
      }
    }
    if (!s_ok) {
      // after a failure: let this CTA's copies in flight land before exiting
      if (g.tma) {
        const uint32_t j0 = issued > (uint32_t)kStages ? issued - kStages : 0;
        for (uint32_t J = j0; J < issued; ++J) {
          const uint64_t t0 = global_timer_ns();
          while (!mbar_try_wait(&full[J % kStages], (J / kStages) & 1) &&
                 global_timer_ns() - t0 < g.timeout_ns) {
          }
        }
      } else {
        asm volatile("cp.async.wait_all;" ::: "memory");
      }
    }
  } else if (warp == kPublisherWarp) {
    // ---------------- publisher: progress = steps gathered ----------------
    for (uint32_t J = 0; J < g.G; ++J) {
      const uint32_t s = J % kStages;
      const bool landed = wait_bar(&full[s], (J / kStages) & 1);
      if (!__all_sync(kFull, landed)) break;
      if (lane == 0) st_release_gpu(g.progress + kProgStride * ch, J + 1);
      if (lane == 0) mbar_arrive(&empty[s]);
    }
    // never leave another CTA waiting on this one
    if (!s_ok && lane == 0) st_release_gpu(g.progress + kProgStride * ch, g.G);
  } else if (warp == kCheckerWarp) {
    // ---------------- checker: dependencies of each step ----------------
    // The rows holding original data in step J's destination range lie in
    // chunks [first(J), last(J)] (a superset); J needs their progress >=
    // J+1-margin.  seen[] caches the last value read (progress only grows),
    // and the chunks of the next kCheckAhead steps are read along, so most
    // steps are decided from the cache.  Progress words are read with
    // gpu-scope acquire loads (each pairs with the owner's release store):
    // a relaxed read followed by a gpu-scope fence cost about 2 us per step
    // on this path.
    // positions below A*B < 2^32: 32-bit divisions by invariants
    auto first_c = [&](uint64_t J) -> uint64_t {
      return fdiv(fdiv((uint32_t)(J * g.g * g.A + i0), g.div_Bc), g.div_Wc);
    };
    auto last_c = [&](uint64_t J) -> uint64_t {
      const uint64_t c0 = J * g.g;
      const uint64_t gj = min64(g.g, g.B - c0);
      return min64(fdiv(fdiv((uint32_t)((c0 + gj - 1) * g.A + i0 + Wc - 1),
                             g.div_Bc),
                        g.div_Wc),
                   g.nchunks - 1);
    };
    bool good = true;
    for (uint32_t J = 0; J < g.G && good; ++J) {
      const uint32_t s = J % kStages;
      const uint32_t need = J + 1 > g.margin ? J + 1 - g.margin : 0u;
      if (need > 0) {
        const uint64_t cf = first_c(J), cl = last_c(J);
        const uint64_t la = last_c(min64(J + kCheckAhead, g.G - 1));
        const uint64_t t0 = global_timer_ns();
        for (uint64_t c = cf + lane; c <= la && good; c += 32) {
          if (c == ch) continue;
          if (c <= cl) {
            if (seen[c] >= need) continue;
            unsigned ns = 32;
            uint32_t v;
            while ((v = ld_acquire_gpu(g.progress + kProgStride * c)) < need) {
              if (!s_ok || global_timer_ns() - t0 > g.timeout_ns) {
                good = false;
                break;
              }
              __nanosleep(ns);
              if (ns < 256) ns <<= 1;
            }
            seen[c] = v;
          } else if (seen[c] < need + kCheckAhead) {
            seen[c] = ld_acquire_gpu(g.progress + kProgStride * c);
          }
        }
        good = __all_sync(kFull, good);
      }
      if (!good) break;
      if (J >= kStages) {
        const bool ok = wait_bar(&empty[s], ((J / kStages) - 1) & 1);
        if (!__all_sync(kFull, ok)) {
          good = false;
          break;
        }
      }
      if (lane == 0) mbar_arrive(&ready[s]);
    }
    if (!good && lane == 0) {
      atomicOr(g.status, kStatusWaitTimeout);
      s_ok = 0;
    }
  } else {
    // ---------------- writers ----------------
    const uint32_t wid = warp - kProducerWarps - 2;
    const uint32_t wb = Wc * g.b;
    T *dst = reinterpret_cast<T *>(g.base);
    for (uint32_t J = 0; J < g.G; ++J) {
      const uint32_t s = J % kStages;
      const bool go = wait_bar(&full[s], (J / kStages) & 1) &&
                      wait_bar(&ready[s], (J / kStages) & 1);
      if (!__all_sync(kFull, go)) break;
      const uint64_t col0 = (uint64_t)J * g.g;
      const uint32_t gj = (uint32_t)min64(g.g, g.B - col0);
      const unsigned char *tb = stage(s);
      const uint32_t *ro = rowoff(s);
      const uint64_t dbase = (col0 * g.A + i0) * g.b;
      const uint64_t drow = g.A * g.b;
      if (g.b == 1) {
        // each lane's rows i = lane + 32m: offsets once per step
        uint32_t rof[kMaxRowBlocks];
#pragma unroll
        for (int m = 0; m < kMaxRowBlocks; ++m) {
          const uint32_t i = lane + 32 * m;
          rof[m] = i < Wc ? ro[i] : 0u;
        }
        for (uint32_t kk = wid; kk < gj; kk += kWriterWarps) {
          T *d = dst + dbase + kk * drow;
          const uint32_t koff = kk * E;
#pragma unroll
          for (int m = 0; m < kMaxRowBlocks; ++m) {
            const uint32_t i = lane + 32 * m;
            if (i < Wc)
              __stcg(d + i, *reinterpret_cast<const T *>(tb + rof[m] + koff));
          }
        }
      } else {
        for (uint32_t kk = wid; kk < gj; kk += kWriterWarps) {
          T *d = dst + dbase + kk * drow;
          const uint32_t koff = kk * g.b * E;
          for (uint32_t rem = lane; rem < wb; rem += 32) {
            const uint32_t i = fdiv(rem, g.div_b);
            const uint32_t sub = rem - i * g.b;
            __stcg(d + rem,
                   *reinterpret_cast<const T *>(tb + ro[i] + koff + sub * E));
          }
        }
      }
      __syncwarp();
      if (lane == 0) mbar_arrive(&empty[s]);
    }
  }
  __syncthreads();
}

// --- host side ---------------------------------------------------------------

// Row pitch of a gathered strip: room for the 16-byte aligned superset a
// bulk copy fetches (at most round16(len) + 16 bytes), and an odd number of
// 16-byte words so that 8 consecutive rows start in distinct bank groups.
static uint32_t stash_pitch(uint64_t row_bytes, int e) {
  (void)e;
  uint64_t p = (row_bytes + 15) / 16 * 16 + 16;
  if (((p / 16) & 1) == 0) p += 16;
  return (uint32_t)p;
}

template <int E>
static int wave_occupancy(size_t smem) {
  auto kern = k_stash_wave<E>;
  if (cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize,
                           (int)smem) != cudaSuccess)
    return 0;
  int occ = 0;
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, kern, kWaveThreads,
                                                    smem) != cudaSuccess)
    return 0;
  return occ;
}

static int wave_occupancy_e(int e, size_t smem) {
  switch (e) {
    case 1: return wave_occupancy<1>(smem);
    case 2: return wave_occupancy<2>(smem);
    case 4: return wave_occupancy<4>(smem);
    default: return wave_occupancy<8>(smem);
  }
}

static StashPlan plan_stash_uncached(uint64_t A, uint64_t B, uint32_t b,
                                     int e);

// plan_stash with the last 16 plans of this thread kept: a plan sums every
// row's stash slot (two 64-bit divisions per row), and the planner, the
// batch router and the tuner ask for the same shapes again and again.  The
// key holds everything the plan reads: the shape, the device, the tuned
// CTAs per SM and the LM_STASH_* overrides.
StashPlan plan_stash(uint64_t A, uint64_t B, uint32_t b, int e) {
  struct Entry {
    uint64_t A = 0, B = 0;
    uint32_t b = 0;
    int e = 0, dev = -1, tuned = 0;
    long long strip = 0, per_sm = 0, margin = 0;
    bool used = false;
    StashPlan p;
  };
  static thread_local Entry cache[16];
  static thread_local uint32_t next = 0;
  const char *es = getenv("LM_STASH_STRIP");
  const char *ep = getenv("LM_STASH_PER_SM");
  const char *em = getenv("LM_STASH_MARGIN");
  Entry k;
  k.A = A, k.B = B, k.b = b, k.e = e;
  k.dev = device_info().device;
  k.tuned = tune_params().stash_per_sm;
  k.strip = es ? atoll(es) : 0;
  k.per_sm = ep ? atoll(ep) : 0;
  k.margin = em ? atoll(em) : 0;
  for (const Entry &c : cache)
    if (c.used && c.A == k.A && c.B == k.B && c.b == k.b && c.e == k.e &&
        c.dev == k.dev && c.tuned == k.tuned && c.strip == k.strip &&
        c.per_sm == k.per_sm && c.margin == k.margin)
      return c.p;
  k.used = true;
  k.p = plan_stash_uncached(A, B, b, e);
  cache[next++ % 16] = k;
  return k.p;
}

static StashPlan plan_stash_uncached(uint64_t A, uint64_t B, uint32_t b,
                                     int e) {
  StashPlan p;
  if (e != 1 && e != 2 && e != 4 && e != 8) return p;
  if (A < 2 || B < 2 || b == 0) return p;
  const uint64_t U = (uint64_t)b * e;
  const DeviceInfo &di = device_info();
  const uint64_t max_smem = (uint64_t)di.max_smem_optin - 1024;
  // Strip per step: the largest (1024 bytes down to 128, in steps of 128)
  // that keeps a CTA's step at most kStepBytes and three ring stages within
  // shared memory, two CTAs per SM first.  Longer steps amortise each step's
  // handshakes; the sweep on both directions of the fp32 16384 x 12289
  // transposition and on fp64 peaked near
  // 32-40 KB per step.  LM_STASH_STRIP / LM_STASH_PER_SM force a choice.
  const char *es = getenv("LM_STASH_STRIP");
  const char *ep = getenv("LM_STASH_PER_SM");
  const char *em = getenv("LM_STASH_MARGIN");
  const uint32_t margin =
      em && atoi(em) > 0 && atoi(em) < 64 ? (uint32_t)atoi(em) : kStashMargin;
  const int tuned = tune_params().stash_per_sm;
  const int per_sms[2] = {tuned == 1 || (!tuned && ep && atoi(ep) == 1) ? 1 : 2,
                          1};
  constexpr uint64_t kStepBytes = 40 * 1024;
  // rows per chunk rounded up so that every chunk's piece of an output row
  // starts on a 32-byte sector (W*U a multiple of 32), where that keeps 95 %
  // of the CTAs: a sector is then written by one CTA, not two at different
  // times (fp32 16384 x 12289: 56 rows instead of 54, wave 3.5 us faster)
  uint64_t walign = 32;
  for (uint64_t u = U; u % 2 == 0 && walign > 1; u /= 2) walign /= 2;
  auto try_plan = [&](uint64_t strip, int per_sm) -> bool {
    const uint64_t ctas = (uint64_t)di.sms * per_sm;
    uint64_t W = (A + ctas - 1) / ctas;
    const uint64_t Wal = (W + walign - 1) / walign * walign;
    if ((A + Wal - 1) / Wal * 100 >= ctas * 95) W = Wal;
    uint64_t g = std::max<uint64_t>(1, strip / U);
    if (g > B) g = B;
    const uint64_t G = (B + g - 1) / g;
    const uint32_t pitch = stash_pitch(g * U, e);
    const uint64_t smem = (uint64_t)kStages * stash_stage_bytes(W, pitch);
    const uint64_t nch = (A + W - 1) / W;
    if (smem > max_smem / per_sm || W * g * b >= 0xffffffffull ||
        g * b >= 0xffffffffull || G > 65535 || W > 32u * kMaxRowBlocks ||
        nch > kMaxChunks ||
        (uint64_t)wave_occupancy_e(e, (size_t)smem) * di.sms < nch)
      return false;
    p.feasible = true;
    p.g = (uint32_t)g;
    p.G = (uint32_t)G;
    p.W = (uint32_t)W;
    p.nchunks = (uint32_t)nch;
    p.pitch = pitch;
    p.smem_bytes = (size_t)smem;
    p.ctas_per_sm = per_sm;
    p.margin = margin;
    p.A = A;
    uint64_t total = 0;
    for (uint64_t i = 0; i < A; ++i)
      total += stash_slot_bytes(i, g, A, B, G, U, margin);
    p.stash_bytes = (size_t)total;
    return true;
  };
  if (es && atoll(es) > 0) {
    for (int per_sm : per_sms)
      if (try_plan((uint64_t)atoll(es), per_sm)) return p;
    return p;
  }
  // the largest strip under the step cap
  auto best_for = [&](int per_sm) -> bool {
    const uint64_t W = (A + (uint64_t)di.sms * per_sm - 1) / ((uint64_t)di.sms * per_sm);
    for (uint64_t strip = 1024; strip >= 128; strip -= 128) {
      if (W * strip > kStepBytes && strip > 128) continue;
      if (try_plan(strip, per_sm)) return true;
    }
    return false;
  };
  if (tuned == 2 && best_for(2)) return p;  // the tuned variant, if it fits
  if (per_sms[0] == 2 && !tuned) {
    StashPlan p2;
    if (best_for(2)) p2 = p;
    // two CTAs per SM with strips below 896 bytes: one CTA per SM with
    // 896- or 1024-byte strips instead, where they fit (twice the rows per
    // step, past the step cap; 12289 x 16384 fp32: 0.411 ms with one CTA
    // and 896-byte strips, 0.431 ms with two and 768-byte strips)
    if (!p2.feasible || (uint64_t)p2.g * U < 896)
      for (uint64_t strip = 1024; strip >= 896; strip -= 128)
        if (try_plan(strip, 1)) return p;
    if (p2.feasible) {
      p = p2;
      return p;
    }
  }
  best_for(1);
  return p;
}

static size_t align256(size_t v) { return (v + 255) / 256 * 256; }

size_t stash_zero_offset(const StashPlan &p) {
  return align256(p.stash_bytes) + align256((size_t)(p.A + 1) * 8);
}

size_t stash_zero_bytes(const StashPlan &p) {
  return (size_t)p.nchunks * 4 * kProgStride;
}

size_t stash_scratch_bytes(const StashPlan &p) {
  // stash + row offsets (A+1) + progress counters + status
  return p.stash_bytes + 256 + (size_t)(p.A + 1) * 8 + 256 +
         (size_t)p.nchunks * 4 * kProgStride + 256 + 4;
}

// The row-offset table depends only on the shape, the plan and the buffer
// address modulo 16: tables computed outside stream capture are kept per
// device (the first kRoffEntries shapes, kRoffBytes in all, until
// lm_marshal_finalize) and reused; a call on another stream waits for the
// producing kernel.
constexpr int kRoffEntries = 16;
constexpr size_t kRoffBytes = 64ull << 20;
struct RoffEntry {
  void *mem = nullptr;
  size_t bytes = 0;
  cudaEvent_t ready = nullptr;
};
using RoffKey = std::tuple<int, uint64_t, uint64_t, uint32_t, uint32_t,
                           uint32_t, uint32_t, uint32_t>;
static std::mutex g_roff_mu;
static std::map<RoffKey, RoffEntry> g_roff;

static cudaError_t launch_offsets(cudaStream_t s, const StashArgs &g) {
  ProfScope ps(s, "stash_offsets");
  k_stash_offsets<<<1, 1024, 0, s>>>(g);
  return cudaGetLastError();
}

// Points g.roff at a cached table (computing it on a miss), or computes
// the table into the caller's scratch while the stream is being captured.
static cudaError_t stash_offsets(cudaStream_t s, StashArgs &g) {
  cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
  cudaStreamIsCapturing(s, &cs);
  if (cs != cudaStreamCaptureStatusNone) return launch_offsets(s, g);
  int dev = 0;
  cudaGetDevice(&dev);
  const RoffKey key{dev, g.A, g.B, g.b, g.e, g.g, g.margin,
                    (uint32_t)((uintptr_t)g.base & 15)};
  std::lock_guard<std::mutex> lock(g_roff_mu);
  auto it = g_roff.find(key);
  if (it != g_roff.end()) {
    g.roff = reinterpret_cast<const uint64_t *>(it->second.mem);
    return cudaStreamWaitEvent(s, it->second.ready, 0);
  }
  const size_t bytes = (size_t)(g.A + 1) * 8;
  // a full cache admits nothing more (no eviction: freeing device memory
  // would synchronise the device); other shapes use per-call scratch
  size_t total = bytes;
  for (auto &kv : g_roff) total += kv.second.bytes;
  if ((int)g_roff.size() >= kRoffEntries || total > kRoffBytes)
    return launch_offsets(s, g);
  RoffEntry en;
  en.bytes = bytes;
  // stream-ordered: a plain cudaMalloc may synchronise the device
  pool_keep_memory();
  cudaError_t err = cudaMallocAsync(&en.mem, bytes, s);
  if (err != cudaSuccess) {
    cudaGetLastError();  // clear the failed allocation's error
    return launch_offsets(s, g);  // into scratch
  }
  if ((err = cudaEventCreateWithFlags(&en.ready, cudaEventDisableTiming)) !=
      cudaSuccess) {
    cudaFreeAsync(en.mem, s);
    return err;
  }
  StashArgs gc = g;
  gc.roff = reinterpret_cast<const uint64_t *>(en.mem);
  if ((err = launch_offsets(s, gc)) != cudaSuccess ||
      (err = cudaEventRecord(en.ready, s)) != cudaSuccess) {
    cudaFreeAsync(en.mem, s);
    cudaEventDestroy(en.ready);
    return err;
  }
  g_roff[key] = en;
  g.roff = gc.roff;
  return cudaSuccess;
}

void stash_cache_clear() {
  int dev = 0;
  cudaGetDevice(&dev);
  std::lock_guard<std::mutex> lock(g_roff_mu);
  for (auto it = g_roff.begin(); it != g_roff.end();) {
    if (std::get<0>(it->first) != dev) {
      ++it;
      continue;
    }
    cudaEventSynchronize(it->second.ready);
    cudaFree(it->second.mem);
    cudaEventDestroy(it->second.ready);
    it = g_roff.erase(it);
  }
}

template <int E>
static cudaError_t run_stash(cudaStream_t s, StashArgs g, const StashPlan &p) {
  cudaError_t err;
  if ((err = stash_offsets(s, g)) != cudaSuccess) return err;
  {
    // rows stashed: those with J_i < G (a prefix of the rows)
    const DeviceInfo &di = device_info();
    const uint64_t warps = (g.A + 1) / 2;
    const unsigned grid = (unsigned)std::min<uint64_t>(
        (warps * 32 + kSaveThreads - 1) / kSaveThreads, (uint64_t)di.sms * 8);
    ProfScope ps(s, "stash_save");
    k_stash_save<<<grid, kSaveThreads, 0, s>>>(g);
    if ((err = cudaGetLastError()) != cudaSuccess) return err;
  }
  auto kern = k_stash_wave<E>;
  err = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize,
                             (int)p.smem_bytes);
  if (err != cudaSuccess) return err;
  int occ = 0;
  err = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, kern, kWaveThreads,
                                                      p.smem_bytes);
  if (err != cudaSuccess) return err;
  const DeviceInfo &di = device_info();
  if ((uint64_t)occ * di.sms < p.nchunks) return cudaErrorCooperativeLaunchTooLarge;
  if (getenv("LM_VERBOSE"))
    fprintf(stderr, "stash: g=%u G=%u W=%u chunks=%u smem=%zu occ=%d stash=%zu\n",
            p.g, p.G, p.W, p.nchunks, p.smem_bytes, occ, p.stash_bytes);
  void *args[] = {&g};
  ProfScope ps(s, "stash_wave");
  // cooperative launch: every CTA is co-resident, so the waits can end.
  // It is also a programmatic dependent of K1, so its CTAs are set up on
  // the SMs that K1's draining blocks free instead of after K1 exits.
  {
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3(p.nchunks);
    cfg.blockDim = dim3(kWaveThreads);
    cfg.dynamicSmemBytes = p.smem_bytes;
    cfg.stream = s;
    cudaLaunchAttribute at[2];
    at[0].id = cudaLaunchAttributeCooperative;
    at[0].val.cooperative = 1;
    at[1].id = cudaLaunchAttributeProgrammaticStreamSerialization;
    at[1].val.programmaticStreamSerializationAllowed = 1;
    cfg.attrs = at;
    cfg.numAttrs = 2;
    err = cudaLaunchKernelExC(&cfg, (const void *)kern, args);
    if (err == cudaSuccess) return cudaGetLastError();
    cudaGetLastError();  // not accepted: plain cooperative launch below
  }
  err = cudaLaunchCooperativeKernel((const void *)kern, dim3(p.nchunks),
                                    dim3(kWaveThreads), args, p.smem_bytes, s);
  if (err != cudaSuccess) return err;
  return cudaGetLastError();
}

cudaError_t launch_stash100(cudaStream_t s, void *buf, int e, uint64_t A,
                            uint64_t B, uint32_t b, const StashPlan &p,
                            void *scratch, uint32_t *status,
                            uint64_t timeout_ns) {
  if (!p.feasible) return cudaErrorInvalidValue;
  char *sc = reinterpret_cast<char *>(scratch);
  auto align = [](size_t v) { return (v + 255) / 256 * 256; };
  StashArgs g;
  g.base = reinterpret_cast<char *>(buf);
  g.stash = sc;
  size_t off = align(p.stash_bytes);
  g.roff = reinterpret_cast<const uint64_t *>(sc + off);
  off += align((size_t)(A + 1) * 8);
  g.progress = reinterpret_cast<uint32_t *>(sc + off);
  g.progress_words = (uint32_t)(stash_zero_bytes(p) / 4);
  g.status = status;
  g.A = A;
  g.B = B;
  g.b = b;
  g.e = (uint32_t)e;
  g.g = p.g;
  g.G = p.G;
  g.W = p.W;
  g.nchunks = p.nchunks;
  g.pitch = p.pitch;
  g.gb = p.g * b;
  g.div_gb = make_fastdiv(g.gb);
  g.div_b = make_fastdiv(b);
  g.timeout_ns = timeout_ns;
  g.margin = p.margin;
  g.gAk = (uint64_t)p.g * A * p.margin;
  g.div_D = make_fastdiv((uint32_t)((uint64_t)p.g * (A - 1)));
  g.div_Bc = make_fastdiv((uint32_t)B);
  g.div_Wc = make_fastdiv(p.W);
  {
    const char *gm = getenv("LM_STASH_GATHER");
    g.tma = (gm && gm[0] == 'c') ? 0u : 1u;  // "cpasync" selects cp.async
    const char *jc = getenv("LM_STASH_EARLY");
    g.jcut = jc ? (uint32_t)atoi(jc) : kStashEarlySteps;
  }
  switch (e) {
    case 1: return run_stash<1>(s, g, p);
    case 2: return run_stash<2>(s, g, p);
    case 4: return run_stash<4>(s, g, p);
    case 8: return run_stash<8>(s, g, p);
    default: return cudaErrorInvalidValue;
  }
}

}  // namespace lm
