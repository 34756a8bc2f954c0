// lm_batch.cu -- many independent conversions in few launches.
//
// No reference counterpart: the reference converts one buffer per call and
// tunes work-group sizes by hand per shape (src/cl_marshal.cc:165-241,
// 388-465).  Here a batch of jobs (each one in-place 0100 on its own buffer,
// any element width) is split in two:
//  * jobs whose tiles fit one CTA's shared memory become work items of ONE
//    persistent kernel: every CTA claims items from an atomic counter (work
//    stealing) and runs the barrier-synchronised tile transposition on them,
//    whatever their element width; two such kernels run, one for items of at
//    most kSmallItem bytes (several CTAs per SM) and one for large tiles (one
//    CTA per SM);
//  * the remaining (large) jobs go through the per-op planner, each on the
//    batch's stream.
// The job table and the item list are uploaded once per batch from pinned
// host memory; lm_batch_run can record the whole batch into a CUDA graph and
// replay it for an identical job list.
#include <algorithm>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <mutex>
#include <vector>
#include <cooperative_groups.h>

#include "lm_core.cuh"
#include "lm_internal.h"
#include "../../include/lm_marshal.h"

namespace lm {

constexpr int kBatchThreads = 512;
constexpr uint32_t kSmallItem = 40 * 1024;
constexpr int kBandGroups = 4;       // clusters of 2, 4, 8 and 16 CTAs
constexpr int kMaxWaves = 32;        // staged waves per batch
constexpr int kCounterStride = 32;   // counters 128 bytes apart
// small, big, one per cluster size, two per staged wave
constexpr size_t kCounterBytes =
    (size_t)(5 + kBandGroups + 2 * kMaxWaves) * kCounterStride * 4;
constexpr int kT010Counter = 2 + kBandGroups + 2 * kMaxWaves;
constexpr uint64_t kDefaultArenaBytes = 1ull << 30;
// jobs at least this large that the stash plan applies to skip the staged
// form (the stash moves 3 x payload, the staged form 4 x)
constexpr uint64_t kStashPreferBytes = 64ull << 20;
constexpr int kSideStreams = 6;      // streams of the large jobs
constexpr int kGroupStreams = 8;     // streams of the item groups
// jobs at least this large that go through scratch run as the planner's
// staged form on a side stream (measured on the serving trace and the
// 4096-matrix batch: 4 and 64 MB were both slower)
constexpr uint64_t kPlannerStagedBytes = 16ull << 20;
// small jobs of one-element units whose output rows are whole 16-byte
// vectors (a*e a multiple of 16, aligned buffer) with tiles of at most
// this size go to the batched 16-byte tile kernel, in items of about
// this size
constexpr uint32_t kT010BatchBytes = 16 * 1024;
// jobs at least this large that the 16-byte tile kernel applies to run as
// launches of their own; smaller ones are items of the batched tile kernel
// (4096-matrix list: 185 launches per step at 8 MB, 311 at 2 MB and 168
// with every such job an item, at equal time within 2 %)
constexpr uint64_t kTile010PreferBytes = 8ull << 20;

struct BJob {
  char *base;
  uint32_t e;
  uint32_t a, B, b;
  uint32_t row_elems, aB, tile_elems, pitch;
  FastDiv div_row, div_b, div_aB, div_a;
  uint32_t band;  // cluster form: units per CTA band (pitch = band pitch)
  // staged form: blocks of S rows x Sj units, nI x nJ of them per tile,
  // written transposed to `scratch` and copied back; nv16 = units of whole
  // 16-byte vectors (every row and output run 16-byte aligned), else 0
  char *scratch;
  uint32_t S, Sj, nJ, nIJ, nv16;
  FastDiv div_Sb, div_nJ, div_nIJ, div_S, div_nv16;
  uint64_t bytes;
  // b == 1 stores: groups of 8 staged rows (ceil(a/8) for bands, S/8 for
  // staged blocks)
  uint32_t ng8;
  FastDiv div_ng8;
  FastDiv div_na;  // a*e/16: 16-byte vectors per output row (tile kernel)
  // tile kernel, form B (input rows of whole 16-byte vectors): staged row
  // pitch, 16-byte pieces per row, rows of a full item and its tiles
  uint32_t tpitch, kt;
  FastDiv div_nc, div_rows;
  // staged form, b == 1 and 1- or 2-byte elements: staged rows start on
  // 32-bit words and output vectors on 16 bytes (store_b1_vec applies);
  // else vbc = the widest output vector (16, 8 or 4 bytes; 16 for 4- and
  // 8-byte elements) the output rows allow (store_b1_vecc), 0 for none; vrw = staged rows per output vector
  // of either store (their groups are shifted in the stage), 0 for none
  uint32_t vb1, vbc, vrw;
};

struct BItem {
  uint32_t job;
  uint32_t ntiles;
  uint64_t tile0;
};

struct BatchArgs {
  const BJob *jobs;
  const BItem *items;
  uint32_t nitems;
  uint32_t *counter;
  uint32_t *status;  // set to kStatusWaitTimeout if a staged load never lands
  uint32_t stage_bytes;  // staged gather: bytes of one shared-memory stage
  // staged gather of one job without tables (items == nullptr): blocks
  // 0 .. nitems-1 of `single`, taken by the CTAs in a fixed stride
  BJob single;
};

// Warp 0: copies a job descriptor into shared memory (read there by every
// thread instead of being held in registers).
__device__ __forceinline__ void copy_job(BJob *dst, const BJob *src) {
  static_assert(sizeof(BJob) % 4 == 0, "BJob is copied in 32-bit words");
  const uint32_t lane = threadIdx.x & 31;
  for (uint32_t k = lane; k < sizeof(BJob) / 4; k += 32)
    reinterpret_cast<uint32_t *>(dst)[k] =
        reinterpret_cast<const uint32_t *>(src)[k];
}

// One item: `ntiles` whole tiles, a contiguous range of the job's buffer.
// Global memory is read and written in 16-byte vectors (the aligned
// superset of the range; elements outside it are skipped on load and
// written one by one on store), so a thread keeps 32 bytes in flight
// whatever the element width; shared memory holds the rows at a padded
// pitch for the transposed reads.
template <int E>
__device__ void batch_item(const BJob &j, const BItem &it, unsigned char *smem) {
  using T = typename Elem<E>::T;
  constexpr uint32_t VE = 16 / E;  // elements per vector
  const uint32_t n = it.ntiles * j.a * j.row_elems;
  T *buf = reinterpret_cast<T *>(j.base) + it.tile0 * (uint64_t)j.tile_elems;
  const uintptr_t s0 = (uintptr_t)buf;
  const uintptr_t v0 = s0 & ~(uintptr_t)15;
  const uint32_t lead = (uint32_t)(s0 - v0) / E;  // elements before the range
  const uint32_t nv = (lead + n + VE - 1) / VE;
  const uint4 *vsrc = reinterpret_cast<const uint4 *>(v0);
  // load: vector v holds elements idx = v*VE - lead + k
  for (uint32_t base = threadIdx.x; base < nv; base += kBatchThreads * 2) {
    uint4 x[2];
#pragma unroll
    for (int u = 0; u < 2; ++u) {
      const uint32_t v = base + u * kBatchThreads;
      if (v < nv) x[u] = __ldcg(vsrc + v);
    }
#pragma unroll
    for (int u = 0; u < 2; ++u) {
      const uint32_t v = base + u * kBatchThreads;
      if (v >= nv) continue;
      int64_t idx = (int64_t)v * VE - lead;
      const uint32_t k0 = idx < 0 ? (uint32_t)(-idx) : 0u;
      if (idx < 0) idx = 0;
      if ((uint64_t)idx >= n) continue;
      uint32_t row = fdiv((uint32_t)idx, j.div_row);
      uint32_t col = (uint32_t)idx - row * j.row_elems;
#pragma unroll
      for (uint32_t k = 0; k < VE; ++k) {
        if (k < k0 || (uint64_t)idx >= n) continue;
        *reinterpret_cast<T *>(smem + row * j.pitch + col * E) =
            vec_elem<E>(x[u], k);
        ++idx;
        if (++col == j.row_elems) {
          col = 0;
          ++row;
        }
      }
    }
  }
  __syncthreads();
  // store: vector v of the output range, output element o <- (tile t,
  // unit jj of the row, row i, sub-element)
  uint4 *vdst = reinterpret_cast<uint4 *>(v0);
  for (uint32_t v = threadIdx.x; v < nv; v += kBatchThreads) {
    int64_t o = (int64_t)v * VE - lead;
    uint32_t k0 = 0;
    if (o < 0) {
      k0 = (uint32_t)(-o);
      o = 0;
    }
    uint32_t unit = (uint32_t)o, sub = 0;
    if (j.b != 1) {
      unit = fdiv((uint32_t)o, j.div_b);
      sub = (uint32_t)o - unit * j.b;
    }
    uint32_t t = fdiv(unit, j.div_aB);
    const uint32_t u2 = unit - t * j.aB;
    uint32_t jj = fdiv(u2, j.div_a);
    uint32_t i = u2 - jj * j.a;
    uint4 x = make_uint4(0, 0, 0, 0);
    uint32_t kend = VE;
#pragma unroll
    for (uint32_t k = 0; k < VE; ++k) {
      if (k < k0) continue;
      if ((uint64_t)o >= n) {
        if (kend == VE) kend = k;
        continue;
      }
      vec_set<E>(x, k, *reinterpret_cast<const T *>(
                           smem + (t * j.a + i) * j.pitch + (jj * j.b + sub) * E));
      ++o;
      if (++sub == j.b) {
        sub = 0;
        if (++i == j.a) {
          i = 0;
          if (++jj == j.B) {
            jj = 0;
            ++t;
          }
        }
      }
    }
    if (k0 == 0 && kend == VE) {
      __stcg(vdst + v, x);
    } else {
      T *d = reinterpret_cast<T *>(v0 + (uintptr_t)v * 16);
#pragma unroll
      for (uint32_t k = 0; k < VE; ++k)
        if (k >= k0 && k < kend) d[k] = vec_elem<E>(x, k);
    }
  }
  __syncthreads();
}

__global__ void __launch_bounds__(kBatchThreads, 2) k_batch_bs(BatchArgs g) {
  extern __shared__ __align__(128) unsigned char smem[];
  __shared__ uint32_t s_item;
  while (true) {
    if (threadIdx.x == 0) s_item = atomicAdd(g.counter, 1u);
    __syncthreads();
    const uint32_t k = s_item;
    __syncthreads();
    if (k >= g.nitems) break;
    const BItem it = g.items[k];
    const BJob j = g.jobs[it.job];
    switch (j.e) {
      case 1: batch_item<1>(j, it, smem); break;
      case 2: batch_item<2>(j, it, smem); break;
      case 4: batch_item<4>(j, it, smem); break;
      default: batch_item<8>(j, it, smem); break;
    }
  }
}

// Small items (at most kSmallItem bytes), pipelined: the bytes of the next
// item land in a flat staging buffer by 16-byte cp.async copies (nothing
// held in registers) while the current item, already scattered into padded
// rows, is written out.  Shared memory: the flat buffer (g.stage_bytes),
// then the padded rows.
template <int E>
__device__ void small_scatter(const BJob &j, const BItem &it,
                              const unsigned char *flat, unsigned char *rows) {
  constexpr uint32_t VE = 16 / E;
  const uint32_t n = it.ntiles * j.a * j.row_elems;
  const uintptr_t s0 = (uintptr_t)(j.base + it.tile0 * (uint64_t)j.tile_elems * E);
  const uint32_t lead = (uint32_t)(s0 & 15) / E;
  const uint32_t nv = (lead + n + VE - 1) / VE;
  for (uint32_t v = threadIdx.x; v < nv; v += kBatchThreads) {
    const uint4 x = *reinterpret_cast<const uint4 *>(flat + (size_t)v * 16);
    int64_t idx = (int64_t)v * VE - lead;
    const uint32_t k0 = idx < 0 ? (uint32_t)(-idx) : 0u;
    if (idx < 0) idx = 0;
    if ((uint64_t)idx >= n) continue;
    uint32_t row = fdiv((uint32_t)idx, j.div_row);
    uint32_t col = (uint32_t)idx - row * j.row_elems;
#pragma unroll
    for (uint32_t k = 0; k < VE; ++k) {
      if (k < k0 || (uint64_t)idx >= n) continue;
      *reinterpret_cast<typename Elem<E>::T *>(rows + row * j.pitch + col * E) =
          vec_elem<E>(x, k);
      ++idx;
      if (++col == j.row_elems) {
        col = 0;
        ++row;
      }
    }
  }
}

template <int E>
__device__ void small_store(const BJob &j, const BItem &it,
                            const unsigned char *rows) {
  using T = typename Elem<E>::T;
  constexpr uint32_t VE = 16 / E;
  const uint32_t n = it.ntiles * j.a * j.row_elems;
  const uintptr_t s0 = (uintptr_t)(j.base + it.tile0 * (uint64_t)j.tile_elems * E);
  const uintptr_t v0 = s0 & ~(uintptr_t)15;
  const uint32_t lead = (uint32_t)(s0 - v0) / E;
  const uint32_t nv = (lead + n + VE - 1) / VE;
  uint4 *vdst = reinterpret_cast<uint4 *>(v0);
  for (uint32_t v = threadIdx.x; v < nv; v += kBatchThreads) {
    int64_t o = (int64_t)v * VE - lead;
    const uint32_t k0 = o < 0 ? (uint32_t)(-o) : 0u;
    if (o < 0) o = 0;
    uint32_t unit = (uint32_t)o, sub = 0;
    if (j.b != 1) {
      unit = fdiv((uint32_t)o, j.div_b);
      sub = (uint32_t)o - unit * j.b;
    }
    uint32_t t = fdiv(unit, j.div_aB);
    const uint32_t u2 = unit - t * j.aB;
    uint32_t jj = fdiv(u2, j.div_a);
    uint32_t i = u2 - jj * j.a;
    uint4 x = make_uint4(0, 0, 0, 0);
    uint32_t kend = VE;
#pragma unroll
    for (uint32_t k = 0; k < VE; ++k) {
      if (k < k0) continue;
      if ((uint64_t)o >= n) {
        if (kend == VE) kend = k;
        continue;
      }
      vec_set<E>(x, k, *reinterpret_cast<const T *>(
                           rows + (t * j.a + i) * j.pitch + (jj * j.b + sub) * E));
      ++o;
      if (++sub == j.b) {
        sub = 0;
        if (++i == j.a) {
          i = 0;
          if (++jj == j.B) {
            jj = 0;
            ++t;
          }
        }
      }
    }
    if (k0 == 0 && kend == VE) {
      __stcg(vdst + v, x);
    } else {
      T *d = reinterpret_cast<T *>(v0 + (uintptr_t)v * 16);
#pragma unroll
      for (uint32_t k = 0; k < VE; ++k)
        if (k >= k0 && k < kend) d[k] = vec_elem<E>(x, k);
    }
  }
}

// All threads: 16-byte cp.async copies of the item's aligned superset into
// the flat buffer, one commit group.
__device__ __forceinline__ void small_issue(const BJob &j, const BItem &it,
                                            unsigned char *flat) {
  const uint64_t nbytes = (uint64_t)it.ntiles * j.tile_elems * j.e;
  const uintptr_t s0 = (uintptr_t)(j.base + it.tile0 * (uint64_t)j.tile_elems * j.e);
  const uintptr_t v0 = s0 & ~(uintptr_t)15;
  const uint32_t nv = (uint32_t)((s0 - v0 + nbytes + 15) / 16);
  for (uint32_t v = threadIdx.x; v < nv; v += kBatchThreads)
    cp_async16(flat + (size_t)v * 16, (const void *)(v0 + (uintptr_t)v * 16));
  cp_async_commit();
}

__global__ void __launch_bounds__(kBatchThreads, 2) k_batch_small(BatchArgs g) {
  extern __shared__ __align__(128) unsigned char smem[];
  unsigned char *flat = smem;
  unsigned char *rows = smem + g.stage_bytes;
  __shared__ uint32_t s_item;
  __shared__ __align__(16) BJob s_jobs[2];
  __shared__ __align__(16) BItem s_items[2];
  const uint32_t warp = threadIdx.x >> 5;
  // claim an item into slot `sl` (job and item copied to shared memory);
  // returns false when the work is done
  auto claim = [&](int sl) -> bool {
    if (threadIdx.x == 0) s_item = atomicAdd(g.counter, 1u);
    __syncthreads();
    const uint32_t k = s_item;
    if (k < g.nitems && warp == 0) {
      const BItem it = g.items[k];
      copy_job(&s_jobs[sl], &g.jobs[it.job]);
      if ((threadIdx.x & 31) == 0) s_items[sl] = it;
    }
    __syncthreads();
    return k < g.nitems;
  };
  if (!claim(0)) return;
  small_issue(s_jobs[0], s_items[0], flat);
  for (uint32_t n = 0;; ++n) {
    const int st = n & 1, nx = st ^ 1;
    cp_async_wait_all();
    __syncthreads();  // the flat buffer holds item n
    const BJob &j = s_jobs[st];
    switch (j.e) {
      case 1: small_scatter<1>(j, s_items[st], flat, rows); break;
      case 2: small_scatter<2>(j, s_items[st], flat, rows); break;
      case 4: small_scatter<4>(j, s_items[st], flat, rows); break;
      default: small_scatter<8>(j, s_items[st], flat, rows); break;
    }
    // (claim's first barrier also orders the scatter before the next
    // item's copies overwrite the flat buffer)
    const bool more = claim(nx);
    if (more) small_issue(s_jobs[nx], s_items[nx], flat);
    switch (j.e) {
      case 1: small_store<1>(j, s_items[st], rows); break;
      case 2: small_store<2>(j, s_items[st], rows); break;
      case 4: small_store<4>(j, s_items[st], rows); break;
      default: small_store<8>(j, s_items[st], rows); break;
    }
    __syncthreads();  // the padded rows are free
    if (!more) break;
  }
}


// Batched form of the 16-byte tile kernel (lm_tile010.cu, form A): items
// of whole tiles of jobs with one-element units whose output rows are whole
// 16-byte vectors, claimed from a counter; the 16-byte cp.async copies of
// the next item land while the current one is written.  Each output vector
// is built from 16/e rows of one staged column.
template <int E>
__device__ __forceinline__ void t010_item_store(const BJob &j, const BItem &it,
                                                const unsigned char *cur) {
  constexpr uint32_t VE = 16 / E;
  const uint32_t B = j.row_elems, R = B * E, NA = j.a / VE;
  const uint32_t tb_bytes = j.tile_elems * E;
  char *dst = j.base + it.tile0 * (uint64_t)tb_bytes;
  const uint32_t nvec = it.ntiles * B * NA;
  const uint32_t orow = j.a * E;
  for (uint32_t x = threadIdx.x; x < nvec; x += kBatchThreads) {
    const uint32_t q = fdiv(x, j.div_row);
    const uint32_t jj = x - q * B;
    const uint32_t t = fdiv(q, j.div_na);
    const uint32_t ib = q - t * NA;
    const uint32_t tb = t * tb_bytes;
    const uint4 v = gather_column<E, 16>(cur + tb + ib * VE * R + jj * E, R);
    __stcg(reinterpret_cast<uint4 *>(dst + tb + jj * orow + ib * 16), v);
  }
}

// Form B of the same (input rows of whole 16-byte vectors, the ASTA -> AoS
// conversions): rows were staged at an odd number of 16-byte words; lanes
// on consecutive rows read 16-byte pieces and scatter their elements into
// the item's output image (`img`), which is then stored in 16-byte vectors.
template <int E>
__device__ __forceinline__ void t010b_item_store(const BJob &j, const BItem &it,
                                                 const unsigned char *cur,
                                                 unsigned char *img) {
  using T = typename Elem<E>::T;
  constexpr uint32_t VE = 16 / E;
  const uint32_t B = j.row_elems, R = B * E, NC = R / 16;
  const uint32_t tb_bytes = j.tile_elems * E;
  const uint32_t rows = it.ntiles * j.a;
  const FastDiv dr = it.ntiles == j.kt ? j.div_rows : make_fastdiv(rows);
  const uint32_t ostep = j.a * E;  // output row bytes
  for (uint32_t x = threadIdx.x; x < rows * NC; x += kBatchThreads) {
    const uint32_t pc = fdiv(x, dr);
    const uint32_t gi = x - pc * rows;
    const uint32_t t = fdiv(gi, j.div_a);
    const uint32_t i = gi - t * j.a;
    const uint4 v = *reinterpret_cast<const uint4 *>(cur + gi * j.tpitch + pc * 16);
    unsigned char *o = img + t * tb_bytes + (pc * VE * j.a + i) * E;
#pragma unroll
    for (uint32_t k = 0; k < VE; ++k)
      *reinterpret_cast<T *>(o + k * ostep) = vec_elem<E>(v, k);
  }
  __syncthreads();  // the output image is complete
  char *dst = j.base + it.tile0 * (uint64_t)tb_bytes;
  const uint32_t nv = it.ntiles * (tb_bytes / 16);
  for (uint32_t v = threadIdx.x; v < nv; v += kBatchThreads)
    __stcg(reinterpret_cast<uint4 *>(dst) + v,
           *reinterpret_cast<const uint4 *>(img + (size_t)v * 16));
}

template <bool FB>
__global__ void __launch_bounds__(kBatchThreads) k_batch_t010(BatchArgs g) {
  extern __shared__ __align__(128) unsigned char smem[];
  __shared__ uint32_t s_item[2];
  __shared__ __align__(16) BJob s_jobs[2];
  __shared__ __align__(16) BItem s_it[2];
  const uint32_t warp = threadIdx.x >> 5;
  auto claim = [&](int sl) -> bool {
    if (threadIdx.x == 0) s_item[sl] = atomicAdd(g.counter, 1u);
    __syncthreads();
    const uint32_t k = s_item[sl];
    if (k < g.nitems && warp == 0) {
      const BItem it = g.items[k];
      copy_job(&s_jobs[sl], &g.jobs[it.job]);
      if ((threadIdx.x & 31) == 0) s_it[sl] = it;
    }
    __syncthreads();
    return k < g.nitems;
  };
  auto issue = [&](int sl) {
    const BJob &j = s_jobs[sl];
    const BItem &it = s_it[sl];
    const uint64_t tbytes = (uint64_t)j.tile_elems * j.e;
    const char *src = j.base + it.tile0 * tbytes;
    const uint32_t nv = (uint32_t)(it.ntiles * tbytes / 16);
    unsigned char *buf = smem + (size_t)sl * g.stage_bytes;
    for (uint32_t v = threadIdx.x; v < nv; v += kBatchThreads) {
      uint32_t off = v * 16;
      if (FB) {  // rows at their padded pitch
        const uint32_t row = fdiv(v, j.div_nc);
        off = row * j.tpitch + (v - row * j.div_nc.d) * 16;
      }
      cp_async16(buf + off, src + (uint64_t)v * 16);
    }
    cp_async_commit();
  };
  if (!claim(0)) return;
  issue(0);
  for (uint32_t n = 0;; ++n) {
    const int st = n & 1, nx = st ^ 1;
    // slot and stage nx were last read before the previous pass's barrier
    const bool more = claim(nx);
    if (more) {
      issue(nx);
      cp_async_wait_group<1>();
    } else {
      cp_async_wait_all();
    }
    __syncthreads();  // item n staged by every thread's copies
    const BJob &j = s_jobs[st];
    const unsigned char *cur = smem + (size_t)st * g.stage_bytes;
    if (FB) {
      unsigned char *img = smem + 2 * (size_t)g.stage_bytes;
      switch (j.e) {
        case 1: t010b_item_store<1>(j, s_it[st], cur, img); break;
        case 2: t010b_item_store<2>(j, s_it[st], cur, img); break;
        case 4: t010b_item_store<4>(j, s_it[st], cur, img); break;
        default: t010b_item_store<8>(j, s_it[st], cur, img); break;
      }
    } else {
      switch (j.e) {
        case 1: t010_item_store<1>(j, s_it[st], cur); break;
        case 2: t010_item_store<2>(j, s_it[st], cur); break;
        case 4: t010_item_store<4>(j, s_it[st], cur); break;
        default: t010_item_store<8>(j, s_it[st], cur); break;
      }
    }
    __syncthreads();  // stage st and slot st free
    if (!more) break;
  }
}

// Writes nrows x ncols staged elements (b == 1) transposed: output row jj
// (stride `ostride` elements from `dst`) gets staged column jj.  A warp
// reads an 8-row x 4-column patch per step, so its 32 lanes hit rows that
// start in distinct 16-byte bank groups, and writes 4 output segments of 8
// elements; work units are 8 rows x 16 columns, spread over all warps.
template <int E>
__device__ __forceinline__ void store_b1(const unsigned char *buf,
                                         const uint32_t *rowoff, uint32_t nrows,
                                         uint32_t ncols, uint32_t ng8,
                                         const FastDiv &div_ng8,
                                         typename Elem<E>::T *dst,
                                         uint32_t ostride, uint32_t warp,
                                         uint32_t nwarps) {
  using T = typename Elem<E>::T;
  const uint32_t lane = threadIdx.x & 31;
  const uint32_t r = lane & 7, c = lane >> 3;
  const uint32_t nch = (ncols + 15) / 16;
  const uint32_t nunits = ng8 * nch;
  for (uint32_t u0 = warp; u0 < nunits; u0 += nwarps) {
    const uint32_t ch = fdiv(u0, div_ng8);
    const uint32_t i = (u0 - ch * ng8) * 8 + r;
    if (i >= nrows) continue;
    const unsigned char *row = buf + rowoff[i];
    T v[4];
#pragma unroll
    for (int u = 0; u < 4; ++u) {
      const uint32_t jj = ch * 16 + u * 4 + c;
      if (jj < ncols) v[u] = *reinterpret_cast<const T *>(row + jj * E);
    }
#pragma unroll
    for (int u = 0; u < 4; ++u) {
      const uint32_t jj = ch * 16 + u * 4 + c;
      if (jj < ncols) __stcg(dst + (uint64_t)jj * ostride + i, v[u]);
    }
  }
}

// store_b1 for 1- and 2-byte elements with whole 16-byte output vectors.
// A group is 16/E staged rows (one output vector per staged column); lane
// l of a warp takes group 8c + l % 8 and 32-bit word column 4d + l / 8 (4/E
// staged columns), reads the group's 16/E words of that column, transposes
// the bytes in registers and writes one 16-byte vector to each of its 4/E
// output rows: the eight lanes of a word column write eight consecutive
// vectors (128 bytes) of the same output row.  The stage shifts the rows of
// group g by 16 g bytes so the eight groups read at once sit in distinct
// bank groups.  Staged rows must start on 32-bit words,
// nrows be a multiple of 16/E, ncols of 4/E, and the vectors dst +
// jj*ostride + i land on 16 bytes (ostride*E and the block's first row a
// multiple of 16 bytes).
// Row r0 + k of a group starts at rowoff[r0] rounded down to 16 bytes,
// plus k pitches, plus the row's own offset within 16 bytes (which advances
// by rb = the global row length mod 16 from row to row): one table read per
// group instead of one per row (the eight groups' table entries share
// banks).
template <int E>
__device__ __forceinline__ void store_b1_vec(const unsigned char *buf,
                                             const uint32_t *rowoff,
                                             uint32_t nrows, uint32_t ncols,
                                             typename Elem<E>::T *dst,
                                             uint32_t ostride, uint32_t warp,
                                             uint32_t nwarps, uint32_t pitch,
                                             uint32_t rb) {
  static_assert(E == 1 || E == 2, "narrow elements only");
  constexpr uint32_t RW = 16 / E;  // staged rows per output vector
  constexpr uint32_t CW = 4 / E;   // staged columns per 32-bit word
  const uint32_t lane = threadIdx.x & 31;
  const uint32_t ngr = nrows / RW, nwc = ncols / CW;
  const uint32_t ngc = (ngr + 7) / 8, nwd = (nwc + 3) / 4;
  for (uint32_t u = warp; u < ngc * nwd; u += nwarps) {
    const uint32_t d = u / ngc, gc = u - d * ngc;
    const uint32_t g = gc * 8 + (lane & 7), wc = d * 4 + (lane >> 3);
    if (g >= ngr || wc >= nwc) continue;
    const uint32_t r0 = g * RW;
    const uint32_t o0 = rowoff[r0], m0 = o0 & 15;
    const unsigned char *col = buf + wc * 4 + (o0 - m0);
    auto word = [&](uint32_t k) {
      return *reinterpret_cast<const uint32_t *>(col + k * pitch +
                                                 ((m0 + k * rb) & 15));
    };
    uint4 out[CW];
#pragma unroll
    for (uint32_t q = 0; q < 4; ++q) {
      uint32_t c[CW];
      if constexpr (E == 1) {
        // a 4 x 4 byte transpose: rows 4q..4q+3 into word q of each column
        const uint32_t a0 = word(4 * q), a1 = word(4 * q + 1),
                       a2 = word(4 * q + 2), a3 = word(4 * q + 3);
        const uint32_t lo01 = __byte_perm(a0, a1, 0x5140);
        const uint32_t hi01 = __byte_perm(a0, a1, 0x7362);
        const uint32_t lo23 = __byte_perm(a2, a3, 0x5140);
        const uint32_t hi23 = __byte_perm(a2, a3, 0x7362);
        c[0] = __byte_perm(lo01, lo23, 0x5410);
        c[1] = __byte_perm(lo01, lo23, 0x7632);
        c[2] = __byte_perm(hi01, hi23, 0x5410);
        c[3] = __byte_perm(hi01, hi23, 0x7632);
      } else {
        // 2-byte elements: rows 2q, 2q+1 into word q of each column
        const uint32_t a0 = word(2 * q), a1 = word(2 * q + 1);
        c[0] = __byte_perm(a0, a1, 0x5410);
        c[1] = __byte_perm(a0, a1, 0x7632);
      }
#pragma unroll
      for (uint32_t k = 0; k < CW; ++k) {
        if (q == 0) out[k].x = c[k];
        else if (q == 1) out[k].y = c[k];
        else if (q == 2) out[k].z = c[k];
        else out[k].w = c[k];
      }
    }
#pragma unroll
    for (uint32_t c = 0; c < CW; ++c)
      __stcg(reinterpret_cast<uint4 *>(dst + (uint64_t)(wc * CW + c) * ostride +
                                       g * RW),
             out[c]);
  }
}

// store_b1 with whole VB-byte output vectors for staged rows that need not
// start on 32-bit words (and for 4- and 8-byte elements, with 16-byte
// vectors of 4 or 2 rows): lane l of a warp takes group 8c + l % 8 of VB/E
// staged rows and staged column 4d + l / 8, gathers the group's VB/E
// elements of that column one by one and writes them as one vector, so the
// eight lanes of a column write eight consecutive vectors of one output
// row.  Groups are shifted in the stage as for store_b1_vec.  nrows must be
// a multiple of VB/E and the vectors dst + jj*ostride + i land on VB bytes.
template <int E, int VB>
__device__ __forceinline__ void store_b1_vecc(const unsigned char *buf,
                                              const uint32_t *rowoff,
                                              uint32_t nrows, uint32_t ncols,
                                              typename Elem<E>::T *dst,
                                              uint32_t ostride, uint32_t warp,
                                              uint32_t nwarps, uint32_t pitch,
                                              uint32_t rb) {
  static_assert(VB == 4 || VB == 8 || VB == 16, "4-, 8- or 16-byte vectors");
  static_assert(VB >= E, "a vector holds whole elements");
  constexpr uint32_t RW = VB / E;  // staged rows per output vector
  constexpr uint32_t NW = VB / 4;  // 32-bit words per vector
  const uint32_t lane = threadIdx.x & 31;
  const uint32_t ngr = nrows / RW;
  const uint32_t ngc = (ngr + 7) / 8, nd = (ncols + 3) / 4;
  for (uint32_t u = warp; u < ngc * nd; u += nwarps) {
    const uint32_t d = u / ngc, gc = u - d * ngc;
    const uint32_t g = gc * 8 + (lane & 7), jj = d * 4 + (lane >> 3);
    if (g >= ngr || jj >= ncols) continue;
    const uint32_t r0 = g * RW;
    const uint32_t o0 = rowoff[r0], m0 = o0 & 15;
    const unsigned char *col = buf + jj * E;
    // groups of 8 rows and more: offsets from the group's first row (the
    // eight groups' table entries would share banks); shorter groups read
    // the table (their entries fall in distinct banks)
    auto at = [&](uint32_t k) {
      if constexpr (RW >= 8)
        return col + (o0 - m0) + k * pitch + ((m0 + k * rb) & 15);
      else
        return col + rowoff[r0 + k];
    };
    uint32_t w[NW];
#pragma unroll
    for (uint32_t q = 0; q < NW; ++q) {
      if constexpr (E == 1) {
        const uint32_t b0 = *at(4 * q), b1 = *at(4 * q + 1);
        const uint32_t b2 = *at(4 * q + 2), b3 = *at(4 * q + 3);
        w[q] = b0 | (b1 << 8) | (b2 << 16) | (b3 << 24);
      } else if constexpr (E == 2) {
        const uint32_t h0 = *reinterpret_cast<const unsigned short *>(at(2 * q));
        const uint32_t h1 =
            *reinterpret_cast<const unsigned short *>(at(2 * q + 1));
        w[q] = h0 | (h1 << 16);
      } else if constexpr (E == 4) {
        w[q] = *reinterpret_cast<const uint32_t *>(at(q));
      } else {
        // 8-byte elements: word q is half q % 2 of row q / 2
        w[q] = reinterpret_cast<const uint32_t *>(at(q / 2))[q % 2];
      }
    }
    typename Elem<E>::T *p = dst + (uint64_t)jj * ostride + r0;
    if constexpr (VB == 16)
      __stcg(reinterpret_cast<uint4 *>(p), make_uint4(w[0], w[1], w[2], w[3]));
    else if constexpr (VB == 8)
      __stcg(reinterpret_cast<uint2 *>(p), make_uint2(w[0], w[1]));
    else
      __stcg(reinterpret_cast<unsigned int *>(p), w[0]);
  }
}

// Tiles larger than one CTA's shared memory, processed by persistent
// clusters: rank 0 claims items and shares them through distributed shared
// memory; each CTA stages a column band of the tile with bulk copies
// (16-byte aligned supersets of the row segments) and writes the output rows
// of its band from its own shared memory.  Two stages: the band of the next
// item loads while the current one is written.
constexpr uint32_t kBandMaxRows = 1024;
namespace cgb = cooperative_groups;

struct BandPos {
  uint32_t bc0, len;  // first unit of my band, bytes of my row segments
};

__device__ __forceinline__ BandPos band_pos(const BJob &j, uint32_t rank) {
  BandPos p;
  p.bc0 = min(j.B, rank * j.band);
  const uint32_t bc1 = min(j.B, p.bc0 + j.band);
  p.len = (bc1 - p.bc0) * j.b * j.e;
  return p;
}

// A warp's arrival on a stage barrier that expects one arrival per warp,
// with the bytes of the warp's bulk copies.
__device__ __forceinline__ void gather_arrive(uint64_t *bar, uint32_t bytes) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) bytes += __shfl_xor_sync(kFull, bytes, o);
  if ((threadIdx.x & 31) == 0) mbar_arrive_expect_tx(bar, bytes);
}

// All threads: bulk copies of my band of every row of `tile`, spread over
// the warps (a warp issues its lanes' copies one after another): row r by
// lane (r / nw) % 32 of warp r % nw.  band_plan records rowoff[] and returns
// this thread's bytes (for the warp's arrival on the stage barrier, which
// expects one arrival per warp); after a CTA barrier band_issue starts the
// copies.
__device__ __forceinline__ uint32_t band_plan(const BJob &j, uint64_t tile,
                                              uint32_t rank, uint32_t *rowoff) {
  const uint32_t nw = blockDim.x >> 5, lane = threadIdx.x & 31;
  const BandPos p = band_pos(j, rank);
  const uint64_t row_bytes = (uint64_t)j.row_elems * j.e;
  const char *row0 =
      j.base + (tile * j.tile_elems + (uint64_t)p.bc0 * j.b) * j.e;
  uint32_t bytes = 0;
  for (uint32_t r = (threadIdx.x >> 5) + nw * lane; r < j.a; r += nw * 32) {
    const uintptr_t src = (uintptr_t)(row0 + r * row_bytes);
    const uintptr_t a0 = src & ~(uintptr_t)15;
    const uintptr_t a1 = (src + p.len + 15) & ~(uintptr_t)15;
    bytes += (uint32_t)(a1 - a0);
    rowoff[r] = r * j.pitch + (uint32_t)(src - a0);
  }
  return bytes;
}

__device__ __forceinline__ void band_issue(const BJob &j, uint64_t tile,
                                           uint32_t rank, unsigned char *buf,
                                           uint64_t *bar) {
  const uint32_t nw = blockDim.x >> 5, lane = threadIdx.x & 31;
  const BandPos p = band_pos(j, rank);
  const uint64_t row_bytes = (uint64_t)j.row_elems * j.e;
  const char *row0 =
      j.base + (tile * j.tile_elems + (uint64_t)p.bc0 * j.b) * j.e;
  fence_proxy_async_smem();
  for (uint32_t r = (threadIdx.x >> 5) + nw * lane; r < j.a; r += nw * 32) {
    const uintptr_t src = (uintptr_t)(row0 + r * row_bytes);
    const uintptr_t a0 = src & ~(uintptr_t)15;
    const uintptr_t a1 = (src + p.len + 15) & ~(uintptr_t)15;
    bulk_g2s(buf + (size_t)r * j.pitch, (const void *)a0, (uint32_t)(a1 - a0),
             bar);
  }
}

// All threads: output rows of my band (one contiguous range of the tile).
template <int E>
__device__ void band_store(const BJob &j, uint64_t tile, uint32_t rank,
                           const unsigned char *buf, const uint32_t *rowoff,
                           uint32_t t, uint32_t nt) {
  using T = typename Elem<E>::T;
  const BandPos p = band_pos(j, rank);
  const uint32_t n = j.a * (p.len / E);
  T *dst = reinterpret_cast<T *>(j.base) + tile * (uint64_t)j.tile_elems +
           (uint64_t)p.bc0 * j.a * j.b;
  if (E <= 4 && j.b == 1 && (j.a * E) % 16 == 0 && ((uintptr_t)dst & 15) == 0) {
    store_columns16<E>(buf, rowoff, j.a, p.len / E,
                       reinterpret_cast<unsigned char *>(dst), t, nt);
    return;
  }
  if (j.b == 1) {
    store_b1<E>(buf, rowoff, j.a, p.len / E, j.ng8, j.div_ng8, dst, j.a,
                t >> 5, nt >> 5);
    return;
  }
  for (uint32_t base = t; base < n; base += nt * 4) {
    T v[4];
#pragma unroll
    for (int u = 0; u < 4; ++u) {
      const uint32_t o = base + u * nt;
      if (o < n) {
        const uint32_t unit = fdiv(o, j.div_b);
        const uint32_t sub = o - unit * j.b;
        const uint32_t jj = fdiv(unit, j.div_a);
        const uint32_t i = unit - jj * j.a;
        v[u] = *reinterpret_cast<const T *>(buf + rowoff[i] +
                                            (jj * j.b + sub) * E);
      }
    }
#pragma unroll
    for (int u = 0; u < 4; ++u) {
      const uint32_t o = base + u * nt;
      if (o < n) __stcg(dst + o, v[u]);
    }
  }
}

// Warp 0 waits for the bulk copies of item n and arrives on the cluster
// barrier with release semantics (its shared-memory writes: job, tile,
// rank 0's claims); the other warps arrive relaxed: the barrier only has to
// order every CTA's completed loads of a tile before any CTA's stores to
// it, and a relaxed arrive does not wait for the earlier global stores to
// drain.  After it every warp issues its share of item n+1's row copies,
// then the other warps write item n.
__global__ void __launch_bounds__(kBatchThreads, 2) k_batch_band(BatchArgs g) {
  extern __shared__ __align__(128) unsigned char smem[];
  __shared__ __align__(8) uint64_t bar[2];
  __shared__ uint32_t rowoff[2][kBandMaxRows];
  __shared__ uint32_t s_item[2];  // rank 0's claims, by sequence parity
  __shared__ int s_ok;
  __shared__ __align__(16) BJob s_jobs[2];   // job of the item in each stage
  __shared__ uint64_t s_tile[2];
  cgb::cluster_group cl = cgb::this_cluster();
  const uint32_t rank = cl.block_rank();
  const uint32_t warp = threadIdx.x >> 5;
  const bool leader = rank == 0 && threadIdx.x == 0;
  if (threadIdx.x == 0) {
    mbar_init(&bar[0], kBatchThreads / 32);
    mbar_init(&bar[1], kBatchThreads / 32);
    fence_mbar_init();
    s_ok = 1;
  }
  if (leader) s_item[0] = atomicAdd(g.counter, 1u);
  cl.sync();  // claim 0 visible; barriers initialised
  const uint32_t *item0 = cl.map_shared_rank(&s_item[0], 0);
  uint32_t cur = item0[0];
  if (leader) s_item[1] = atomicAdd(g.counter, 1u);  // read after the next sync
  uint32_t parity = 0, pending = 0;
  // stages the band of item k's tile into stage st (every thread)
  auto stage_item = [&](uint32_t k, int st) {
    const BItem it = g.items[k];
    const BJob &j = g.jobs[it.job];
    const bool has = band_pos(j, rank).len > 0;
    if (has) gather_arrive(&bar[st], band_plan(j, it.tile0, rank, rowoff[st]));
    __syncthreads();  // every warp's expected bytes before any copy
    if (has)
      band_issue(j, it.tile0, rank, smem + (size_t)st * g.stage_bytes,
                 &bar[st]);
    if (warp == 0) {
      copy_job(&s_jobs[st], &j);
      if ((threadIdx.x & 31) == 0) s_tile[st] = it.tile0;
    }
  };
  if (cur < g.nitems) stage_item(cur, 0);
  for (uint32_t n = 0; cur < g.nitems; ++n) {
    const int st = n & 1, nx = st ^ 1;
    if (warp == 0) {
      const BandPos p = band_pos(s_jobs[st], rank);
      if (p.len > 0 && s_ok) {
        bool landed = true;
        const uint64_t t0 = global_timer_ns();
        while (!mbar_try_wait(&bar[st], (parity >> st) & 1))
          if (global_timer_ns() - t0 > 2000000000ull) {
            landed = false;
            break;
          }
        if (__all_sync(kFull, landed)) {
          parity ^= 1u << st;
        } else {
          pending |= 1u << st;
          if ((threadIdx.x & 31) == 0) {
            s_ok = 0;  // stage nothing more, write nothing more
            atomicExch(g.status, kStatusWaitTimeout);
          }
        }
      }
      cluster_arrive_release();
    } else {
      cluster_arrive_relaxed();
    }
    cluster_wait_acquire();  // every band of item n staged; claim n+1 visible
    const uint32_t nxt = item0[nx];
    if (nxt < g.nitems && s_ok) stage_item(nxt, nx);
    if (warp == 0) {
      if (leader) s_item[st] = atomicAdd(g.counter, 1u);  // claim n+2
    } else if (s_ok) {
      const BJob &j = s_jobs[st];
      const unsigned char *buf = smem + (size_t)st * g.stage_bytes;
      const uint64_t tile = s_tile[st];
      const uint32_t t = threadIdx.x - 32, nt = kBatchThreads - 32;
      switch (j.e) {
        case 1: band_store<1>(j, tile, rank, buf, rowoff[st], t, nt); break;
        case 2: band_store<2>(j, tile, rank, buf, rowoff[st], t, nt); break;
        case 4: band_store<4>(j, tile, rank, buf, rowoff[st], t, nt); break;
        default: band_store<8>(j, tile, rank, buf, rowoff[st], t, nt); break;
      }
    }
    cur = nxt;
  }
  // a stage whose loads never landed: give them one more bounded wait
  if (warp == 0) {
    for (int st = 0; st < 2; ++st) {
      if (!((pending >> st) & 1)) continue;
      const uint64_t t0 = global_timer_ns();
      while (!mbar_try_wait(&bar[st], (parity >> st) & 1) &&
             global_timer_ns() - t0 < 2000000000ull) {
      }
    }
  }
  cl.sync();  // rank 0's claims stay readable until every CTA is done
}

// Staged form, for tiles too large for any on-chip plan: each S x S block of
// units of a tile is transposed through shared memory into the batch's
// scratch arena (out of place, so blocks need no ordering), then a second
// kernel copies the arena back over the job's buffer.  Items are runs of
// blocks (gather) or of 16-byte vectors (copy back).
constexpr int kStageThreads = 256;
constexpr uint32_t kStageTileBytes = 32 * 1024;  // staged bytes per block
constexpr uint32_t kStageMaxS = 256;             // rows per block
constexpr uint32_t kStageBlocksPerItem = 4;   // fine-grained: balanced tails
constexpr uint64_t kCopyVecsPerItem = 16384;     // 256 KB
// staged jobs in this range copy back with a kernel that drops each scratch
// line from L2 once read, so dirty scratch lines are not written back to
// DRAM (staged 100s of 64-200 MB: 2-7 % faster than cudaMemcpyAsync;
// smaller jobs, whose scratch and buffer both fit L2, copy back 3-8 %
// faster with cudaMemcpyAsync, and from 256 MB the scratch has left L2)
constexpr uint64_t kL2StageMinBytes = 48ull << 20;   // exclusive
constexpr uint64_t kL2StageMaxBytes = 208ull << 20;

// Block q of a staged job: tile t, block row bi, block column bj.
struct GBlock {
  uint32_t t, i0, j0, si, sj;
};

__device__ __forceinline__ GBlock gather_decode(const BJob &j, uint32_t q) {
  GBlock k;
  k.t = fdiv(q, j.div_nIJ);
  const uint32_t r = q - k.t * j.nIJ;
  const uint32_t bi = fdiv(r, j.div_nJ);
  const uint32_t bj = r - bi * j.nJ;
  k.i0 = bi * j.S;
  k.j0 = bj * j.Sj;
  k.si = min(j.S, j.a - k.i0);
  k.sj = min(j.Sj, j.B - k.j0);
  return k;
}

// One bulk copy per row of the block (the 16-byte aligned superset of its
// row segment), spread over all kStageThreads threads: a warp issues its lanes' bulk copies one after another (about
// 30 ns each on GB300), so row r of the block goes to lane r / 8 of warp
// r % 8 and no warp issues more than 32 of a block's 256 rows at most.
// gather_row_plan: this thread's row (rowoff[] recorded); gather_arrive: a
// warp's arrival on `bar` (initialised with one arrival per warp) with the
// bytes of its rows; after a CTA barrier, gather_row_issue starts the copy.
struct RowCopy {
  uintptr_t src;   // 16-byte aligned start
  uint32_t bytes;  // 0: no row for this thread
  uint32_t dst;    // offset in the stage
};

__device__ __forceinline__ RowCopy gather_row_plan(const BJob &j, uint32_t q,
                                                   uint32_t *rowoff) {
  RowCopy c{0, 0, 0};
  const GBlock k = gather_decode(j, q);
  const uint32_t r = (threadIdx.x & 31) * (kStageThreads / 32) + (threadIdx.x >> 5);
  if (r >= k.si) return c;
  const uint32_t len = k.sj * j.b * j.e;
  const uintptr_t src = (uintptr_t)(j.base + ((uint64_t)k.t * j.tile_elems +
                                              (uint64_t)(k.i0 + r) * j.row_elems +
                                              (uint64_t)k.j0 * j.b) * j.e);
  c.src = src & ~(uintptr_t)15;
  c.bytes = (uint32_t)(((src + len + 15) & ~(uintptr_t)15) - c.src);
  // vectorized narrow stores: the rows of group r / vrw shifted by 16 bytes
  // per group (the shifts only grow, so rows never overlap), so the eight
  // consecutive groups a warp reads at once fall in distinct bank groups
  c.dst = r * j.pitch + (j.vrw ? 16 * (r / j.vrw) : 0);
  rowoff[r] = c.dst + (uint32_t)(src - c.src);
  return c;
}

__device__ __forceinline__ void gather_row_issue(const RowCopy &c,
                                                 unsigned char *buf,
                                                 uint64_t *bar) {
  if (!c.bytes) return;
  fence_proxy_async_smem();
  bulk_g2s(buf + c.dst, (const void *)c.src, c.bytes, bar);
}

// All threads: output rows j0..j0+sj-1 of the block, each si*b elements
// long, from the staged rows.
template <int E>
__device__ void gather_store(const BJob &j, uint32_t q, const unsigned char *buf,
                             const uint32_t *rowoff) {
  using T = typename Elem<E>::T;
  const GBlock k = gather_decode(j, q);
  T *dst = reinterpret_cast<T *>(j.scratch) + (uint64_t)k.t * j.tile_elems +
           ((uint64_t)k.j0 * j.a + k.i0) * j.b;
  if (j.nv16) {
    // whole 16-byte vectors: lanes on consecutive vectors of a column's
    // output run (consecutive staged rows: distinct bank groups)
    const uint32_t NS = j.nv16, U = NS * 16;
    const uint32_t n = k.sj * k.si * NS;
    const FastDiv dsi = k.si == j.S ? j.div_S : make_fastdiv(k.si);
    unsigned char *d = reinterpret_cast<unsigned char *>(dst);
    const uint64_t ostride = (uint64_t)j.a * U;  // bytes between output rows
    for (uint32_t x = threadIdx.x; x < n; x += kStageThreads) {
      uint32_t u = x, sv = 0;
      if (NS != 1) {
        u = fdiv(x, j.div_nv16);
        sv = x - u * NS;
      }
      const uint32_t jj = fdiv(u, dsi);
      const uint32_t ii = u - jj * k.si;
      const uint4 v = *reinterpret_cast<const uint4 *>(buf + rowoff[ii] +
                                                       jj * U + sv * 16);
      __stcg(reinterpret_cast<uint4 *>(d + (uint64_t)jj * ostride +
                                       (ii * NS + sv) * 16),
             v);
    }
    return;
  }
  if (j.b == 1) {
    const uint32_t w = threadIdx.x >> 5, nw = kStageThreads / 32;
    const uint32_t rb = (j.row_elems * E) & 15;  // row length mod 16
    if constexpr (E <= 2) {
      if (j.vb1 && k.si % (16 / E) == 0 && k.sj % (4 / E) == 0) {
        store_b1_vec<E>(buf, rowoff, k.si, k.sj, dst, j.a, w, nw, j.pitch, rb);
        return;
      }
    }
    if (j.vbc && k.si % (j.vbc / E) == 0) {
      if (j.vbc == 16)
        store_b1_vecc<E, 16>(buf, rowoff, k.si, k.sj, dst, j.a, w, nw, j.pitch,
                             rb);
      else if constexpr (E <= 2) {
        if (j.vbc == 8)
          store_b1_vecc<E, 8>(buf, rowoff, k.si, k.sj, dst, j.a, w, nw,
                              j.pitch, rb);
        else
          store_b1_vecc<E, 4>(buf, rowoff, k.si, k.sj, dst, j.a, w, nw,
                              j.pitch, rb);
      }
      return;
    }
    store_b1<E>(buf, rowoff, k.si, k.sj, j.ng8, j.div_ng8, dst, j.a,
                threadIdx.x >> 5, kStageThreads / 32);
    return;
  }
  const uint32_t ob = k.si * j.b;  // elements per output row segment
  const uint32_t n = k.sj * ob;
  const FastDiv div_ob = k.si == j.S ? j.div_Sb : make_fastdiv(ob);
  const uint64_t ostride = (uint64_t)j.a * j.b;
  for (uint32_t base = threadIdx.x; base < n; base += kStageThreads * 4) {
    T v[4];
#pragma unroll
    for (int u = 0; u < 4; ++u) {
      const uint32_t o = base + u * kStageThreads;
      if (o < n) {
        const uint32_t jj = fdiv(o, div_ob);
        const uint32_t rem = o - jj * ob;
        uint32_t ii = rem, sub = 0;
        if (j.b != 1) {
          ii = fdiv(rem, j.div_b);
          sub = rem - ii * j.b;
        }
        v[u] = *reinterpret_cast<const T *>(buf + rowoff[ii] +
                                            (jj * j.b + sub) * E);
      }
    }
#pragma unroll
    for (int u = 0; u < 4; ++u) {
      const uint32_t o = base + u * kStageThreads;
      if (o < n) {
        const uint32_t jj = fdiv(o, div_ob);
        __stcg(dst + jj * ostride + (o - jj * ob), v[u]);
      }
    }
  }
}

// Persistent: every CTA walks blocks (claimed item by item from the work
// counter) with two shared-memory stages, loading block n+1 by bulk copies
// (issued by all warps) while it writes block n.
// MB: CTAs per SM the registers are sized for.  Three suit the mixed
// batches and 1-, 4- and 8-byte blocks; 2-byte blocks run 0-3 % faster with
// the registers of two (staged 100s of 2-byte elements, 4096 x 32768:
// gather 0.0933 vs 0.0963 ms; 500 x 268435: 0.161 vs 0.167 ms; 1-byte
// 16384 x 16384 the other way: 0.126 vs 0.121 ms).
template <int MB>
__global__ void __launch_bounds__(kStageThreads, MB) k_batch_gather(BatchArgs g) {
  extern __shared__ __align__(128) unsigned char smem[];
  __shared__ __align__(8) uint64_t bar[2];
  __shared__ uint32_t rowoff[2][kStageMaxS];
  __shared__ uint32_t s_job[2], s_q[2], s_valid[2];
  __shared__ int s_dead;
  __shared__ __align__(16) BJob s_jobs[2];  // job of the block in each stage
  const uint32_t warp = threadIdx.x >> 5;
  const BJob *jobs = g.items ? g.jobs : &g.single;
  uint32_t c_job = 0, c_q = 0, c_end = 0;  // thread 0's cursor
  bool c_first = true;
  auto fetch = [&](int slot) {
    if (!g.items) {
      c_q = c_first ? blockIdx.x : c_q + gridDim.x;
      c_first = false;
      s_valid[slot] = c_q < g.nitems;
      s_job[slot] = 0;
      s_q[slot] = c_q;
      return;
    }
    if (c_q >= c_end) {
      const uint32_t k = atomicAdd(g.counter, 1u);
      if (k >= g.nitems) {
        s_valid[slot] = 0;
        return;
      }
      const BItem it = g.items[k];
      c_job = it.job;
      c_q = (uint32_t)it.tile0;
      c_end = c_q + it.ntiles;
    }
    s_job[slot] = c_job;
    s_q[slot] = c_q++;
    s_valid[slot] = 1;
  };
  if (threadIdx.x == 0) {
    mbar_init(&bar[0], kStageThreads / 32);
    mbar_init(&bar[1], kStageThreads / 32);
    fence_mbar_init();
    s_dead = 0;
    fetch(0);
  }
  __syncthreads();
  if (!s_valid[0]) return;
  uint32_t cq = s_q[0];
  {
    if (warp == 0) copy_job(&s_jobs[0], &jobs[s_job[0]]);
    const RowCopy rc = gather_row_plan(jobs[s_job[0]], cq, rowoff[0]);
    gather_arrive(&bar[0], rc.bytes);
    __syncthreads();  // every warp's expected bytes before any copy
    gather_row_issue(rc, smem, &bar[0]);
  }
  uint32_t parity = 0;   // bit st: phase to wait for on bar[st]
  uint32_t pending = 1;  // bit st: loads issued to stage st, not yet seen

  for (uint32_t n = 0;; ++n) {
    const int st = n & 1, nx = st ^ 1;
    if (threadIdx.x == 0) fetch(nx);
    __syncthreads();  // slot nx visible; stage nx free since the last pass
    const bool more = s_valid[nx] != 0 && !s_dead;
    const uint32_t nj = s_job[nx], nq = s_q[nx];
    if (more) {
      if (warp == 0) copy_job(&s_jobs[nx], &jobs[nj]);
      const RowCopy rc = gather_row_plan(jobs[nj], nq, rowoff[nx]);
      gather_arrive(&bar[nx], rc.bytes);
      __syncthreads();  // every warp's expected bytes before any copy
      gather_row_issue(rc, smem + (size_t)nx * g.stage_bytes, &bar[nx]);
      pending |= 1u << nx;
    }
    // wait for block n (bounded; a load that never lands stops this CTA)
    const uint64_t t0 = global_timer_ns();
    bool landed = true;
    while (!mbar_try_wait(&bar[st], (parity >> st) & 1))
      if (global_timer_ns() - t0 > 2000000000ull) {
        landed = false;
        break;
      }
    if (landed) {
      parity ^= 1u << st;
      pending &= ~(1u << st);
      const BJob &j = s_jobs[st];
      const unsigned char *buf = smem + (size_t)st * g.stage_bytes;
      switch (j.e) {
        case 1: gather_store<1>(j, cq, buf, rowoff[st]); break;
        case 2: gather_store<2>(j, cq, buf, rowoff[st]); break;
        case 4: gather_store<4>(j, cq, buf, rowoff[st]); break;
        default: gather_store<8>(j, cq, buf, rowoff[st]); break;
      }
    } else {
      s_dead = 1;
      if (g.status) atomicExch(g.status, kStatusWaitTimeout);
    }
    __syncthreads();  // stage st read by everyone; slot nx read by everyone
    if (!more || s_dead) break;
    cq = nq;
  }
  // nothing may still be landing in shared memory when the CTA exits
  for (int st = 0; st < 2; ++st) {
    if (!((pending >> st) & 1)) continue;
    const uint64_t t0 = global_timer_ns();
    while (!mbar_try_wait(&bar[st], (parity >> st) & 1) &&
           global_timer_ns() - t0 < 2000000000ull) {
    }
  }
}

// Copy back: the arena copy of a job starts at the same address modulo 16 as
// the job's buffer, so one run of 16-byte vectors serves both; item 0 of a
// job also copies the ragged head and tail bytes.
__global__ void __launch_bounds__(kStageThreads) k_batch_copyback(BatchArgs g) {
  __shared__ uint32_t s_item;
  while (true) {
    if (threadIdx.x == 0) s_item = atomicAdd(g.counter, 1u);
    __syncthreads();
    const uint32_t k = s_item;
    __syncthreads();
    if (k >= g.nitems) break;
    const BItem it = g.items[k];
    const BJob j = g.jobs[it.job];
    const uintptr_t d = (uintptr_t)j.base;
    const uint64_t head = min64((16 - (d & 15)) & 15, j.bytes);
    const uint64_t nvec = (j.bytes - head) / 16;
    const uint4 *vs = reinterpret_cast<const uint4 *>(j.scratch + head);
    uint4 *vd = reinterpret_cast<uint4 *>(j.base + head);
    const uint64_t v1 = min64(it.tile0 + kCopyVecsPerItem, nvec);
    // four independent loads in flight per thread
    for (uint64_t v = it.tile0 + threadIdx.x; v < v1; v += 4 * kStageThreads) {
      uint4 x[4];
#pragma unroll
      for (int u = 0; u < 4; ++u)
        if (v + u * kStageThreads < v1) x[u] = __ldcs(vs + v + u * kStageThreads);
#pragma unroll
      for (int u = 0; u < 4; ++u)
        if (v + u * kStageThreads < v1) __stcs(vd + v + u * kStageThreads, x[u]);
    }
    if (it.tile0 == 0) {
      const uint64_t tail0 = head + nvec * 16;
      for (uint64_t x = threadIdx.x; x < head + (j.bytes - tail0);
           x += kStageThreads) {
        const uint64_t off = x < head ? x : tail0 + (x - head);
        j.base[off] = j.scratch[off];
      }
    }
  }
}

// Copy back of one staged job whose scratch is still in L2 (written by the
// gather just before): 16-byte vectors, a warp on 512 consecutive bytes per
// step, then the scratch lines it has read are dropped from L2 without a
// write-back (discard), so the staging costs DRAM no traffic of its own.
// `dst` and `src` have the same address modulo 16; the ragged head and tail
// bytes are copied by block 0.
__global__ void __launch_bounds__(kStageThreads) k_stage_copyback(
    char *dst, const char *src, uint64_t bytes) {
  const uintptr_t d = (uintptr_t)dst;
  const uint64_t head = min64((16 - (d & 15)) & 15, bytes);
  const uint64_t nvec = (bytes - head) / 16;
  const uint4 *vs = reinterpret_cast<const uint4 *>(src + head);
  uint4 *vd = reinterpret_cast<uint4 *>(dst + head);
  // scratch lines wholly inside [src, src + bytes) may be dropped (the
  // ragged head and tail bytes never lie in one)
  const uintptr_t l0 = ((uintptr_t)src + 127) & ~(uintptr_t)127;
  const uintptr_t l1 = ((uintptr_t)src + bytes) & ~(uintptr_t)127;
  // warps walk 512-byte aligned windows of the scratch: whole lines each
  const uintptr_t s0 = (uintptr_t)src + head, s1 = s0 + nvec * 16;
  const uintptr_t w0 = s0 & ~(uintptr_t)511;
  const uint64_t nwin = nvec ? (s1 - w0 + 511) / 512 : 0;
  const uint32_t lane = threadIdx.x & 31;
  const uint64_t warps = (uint64_t)gridDim.x * (kStageThreads / 32);
  for (uint64_t w = blockIdx.x * (uint64_t)(kStageThreads / 32) +
                    (threadIdx.x >> 5);
       w < nwin; w += warps) {
    const uintptr_t a = w0 + w * 512 + (uintptr_t)lane * 16;
    if (a >= s0 && a < s1) {
      const uint64_t v = (a - s0) / 16;
      __stcs(vd + v, __ldcg(vs + v));
    }
    __syncwarp();  // every lane's load from this window has completed
    const uintptr_t line = w0 + w * 512 + (uintptr_t)lane * 128;
    if (lane < 4 && line >= l0 && line + 128 <= l1)
      discard_l2_line((const void *)line);
  }
  if (blockIdx.x == 0) {
    const uint64_t tail0 = head + nvec * 16;
    for (uint64_t x = threadIdx.x; x < head + (bytes - tail0);
         x += kStageThreads) {
      const uint64_t off = x < head ? x : tail0 + (x - head);
      dst[off] = src[off];
    }
  }
}

// ---- host -------------------------------------------------------------------

// Cluster form of one tile of a x (B*b) elements of e bytes: the smallest
// cluster (2..16 CTAs) whose column bands fit `half` bytes (a stage size
// that leaves room for two CTAs per SM), else the smallest whose bands fit
// `budget` bytes (one of the two shared-memory stages of a CTA).  Returns the
// group index (log2(C) - 1) or -1.
static int band_group(uint64_t a, uint64_t B, uint64_t b, int e, size_t budget,
                      size_t half, uint32_t *band, uint32_t *pitch,
                      bool *two_per_sm) {
  if (a > kBandMaxRows || a * B * b >= 0xffffffffull) return -1;
  for (int pass = 0; pass < 2; ++pass) {
    for (int gi = 0; gi < kBandGroups; ++gi) {
      const uint64_t C = 2ull << gi;
      const uint64_t bd = (B + C - 1) / C;
      // a 16-byte aligned superset of a row segment of len bytes spans at
      // most round16(len) + 16 bytes
      uint64_t bp = (bd * b * e + 15) / 16 * 16 + 16;
      if (((bp / 16) & 1) == 0) bp += 16;  // rows in distinct bank groups
      if (bp * a <= (pass == 0 ? half : budget)) {
        *band = (uint32_t)bd;
        *pitch = (uint32_t)bp;
        *two_per_sm = pass == 0;
        return gi;
      }
    }
  }
  return -1;
}

static uint32_t batch_pitch(uint64_t row_bytes, int e) {
  const uint64_t g = e == 8 ? 8 : 4;
  uint64_t p = (row_bytes + g - 1) / g * g;
  if (((p / g) & 1) == 0) p += g;
  return (uint32_t)p;
}

struct Normalized {
  bool ok = false;
  uint64_t T = 0, a = 0, B = 0, b = 0;
  int e = 0;  // element bytes (widened by plan_batch where units allow)
};

// Every op of the library as a 0100(T, a, B, b).
static Normalized normalize(const lm_job &jb) {
  Normalized n;
  const int64_t d0 = jb.d0, d1 = jb.d1, d2 = jb.d2, d3 = jb.d3;
  switch (jb.op) {
    case LM_OP_0100:  // A a B b
      if (d0 < 0 || d1 < 0 || d2 < 0 || d3 < 0) return n;
      n.T = d0; n.a = d1; n.B = d2; n.b = d3;
      break;
    case LM_OP_010:  // A a B
      if (d0 < 0 || d1 < 0 || d2 < 0) return n;
      n.T = d0; n.a = d1; n.B = d2; n.b = 1;
      break;
    case LM_OP_100:  // A B b
      if (d0 < 0 || d1 < 0 || d2 < 0) return n;
      n.T = 1; n.a = d0; n.B = d1; n.b = d2;
      break;
    case LM_OP_AOS_ASTA:  // height width tile
      if (d2 <= 0 || d0 < 0 || d1 < 0 || d0 % d2) return n;
      n.T = d0 / d2; n.a = d2; n.B = d1; n.b = 1;
      break;
    case LM_OP_ASTA_AOS:  // height width tile: [h/t][w][t] -> [h][w]
      if (d2 <= 0 || d0 < 0 || d1 < 0 || d0 % d2) return n;
      n.T = d0 / d2; n.a = d1; n.B = d2; n.b = 1;
      break;
    case LM_OP_SOA_ASTA:  // height width tile: [w][h] -> [h/t][w][t]
      if (d2 <= 0 || d0 < 0 || d1 < 0 || d0 % d2) return n;
      n.T = 1; n.a = d1; n.B = d0 / d2; n.b = d2;
      break;
    case LM_OP_ASTA_SOA:  // height width tile: [h/t][w][t] -> [w][h]
      if (d2 <= 0 || d0 < 0 || d1 < 0 || d0 % d2) return n;
      n.T = 1; n.a = d0 / d2; n.B = d1; n.b = d2;
      break;
    case LM_OP_TRANSPOSE:  // M N
      if (d0 < 0 || d1 < 0) return n;
      n.T = 1; n.a = d0; n.B = d1; n.b = 1;
      break;
    default:
      return n;
  }
  n.e = jb.elem_bytes;
  n.ok = true;
  return n;
}

bool op_as_0100(int op, long long d0, long long d1, long long d2, long long d3,
                uint64_t *T, uint64_t *a, uint64_t *B, uint64_t *b) {
  lm_job jb{};
  jb.op = op;
  jb.d0 = d0;
  jb.d1 = d1;
  jb.d2 = d2;
  jb.d3 = d3;
  const Normalized n = normalize(jb);
  *T = n.T;
  *a = n.a;
  *B = n.B;
  *b = n.b;
  return n.ok;
}

}  // namespace lm

struct lm_batch_st {
  std::vector<lm::BJob> jobs;
  std::vector<lm::BItem> small, big;
  std::vector<lm::BItem> t010;  // items of the batched 16-byte tile kernel
  std::vector<lm::BItem> t010b;  // the same, one larger tile per item
  std::vector<lm::BItem> t010f;  // its form B (whole-vector input rows)
  size_t t010b_stage = 0;       // bytes of the largest such tile
  std::vector<lm::BItem> band[lm::kBandGroups];  // cluster of 2 << g CTAs
  size_t band_smem[lm::kBandGroups] = {};
  // staged waves: gather items, copy-back items, shared memory of the gather
  std::vector<lm::BItem> wgather[lm::kMaxWaves], wcopy[lm::kMaxWaves];
  size_t wsmem[lm::kMaxWaves] = {};
  int nwaves = 0;
  char *d_arena = nullptr;  // scratch of the staged jobs of one wave
  uint64_t cap_arena = 0, need_arena = 0;
  uint64_t arena_limit = 0;  // lm_batch_set_arena; 0: LM_BATCH_SCRATCH_MB
  cudaStream_t last_stream = nullptr;  // stream of the previous run
  bool used = false;
  std::vector<void *> retired_pinned;  // grown-out staging buffers
  std::vector<uint32_t> large;  // indices of jobs run by the planner
  std::vector<lm::Normalized> norm;
  // device side
  lm::BJob *d_jobs = nullptr;
  lm::BItem *d_items = nullptr;
  uint32_t *d_counters = nullptr;
  size_t cap_jobs = 0, cap_items = 0;
  // pinned staging
  void *h_stage = nullptr;
  size_t cap_stage = 0;
  // graph cache
  cudaGraphExec_t gexec = nullptr;
  uint64_t gkey = 0;
  void *h_gstage = nullptr;  // pinned copy of the job table owned by gexec
  cudaEvent_t uploaded = nullptr;  // last upload from h_stage
  cudaStream_t side[lm::kSideStreams] = {};  // large jobs run here
  cudaEvent_t join[lm::kSideStreams] = {};
  // the item groups (persistent kernels) run on streams of their own, one
  // priority level above the large jobs: they must not wait in stream order
  // behind large jobs, and their CTAs take SMs as the large jobs' blocks
  // free them
  cudaStream_t gside[lm::kGroupStreams] = {};
  cudaEvent_t gjoin[lm::kGroupStreams] = {};
  cudaEvent_t fork = nullptr, fork2 = nullptr;
  uint64_t seen_key = 0;  // job list of the previous graph-mode run
  std::vector<lm_job> gjobs, seen_jobs;  // the lists behind gkey / seen_key
  unsigned gflags = 0, seen_flags = 0;
  // last run statistics
  lm_batch_stats stats;
  int device = -1;
};

using namespace lm;

// Key of a job list and its flags (field by field); a key match is
// confirmed by same_jobs against the kept copy before a graph is replayed.
static uint64_t hash_jobs(const lm_job *jobs, int n, unsigned flags) {
  uint64_t h = 1469598103934665603ull;
  auto mix = [&](uint64_t v) {
    for (int k = 0; k < 8; ++k) {
      h ^= (v >> (8 * k)) & 0xff;
      h *= 1099511628211ull;
    }
  };
  mix(flags);
  mix((uint64_t)n);
  for (int i = 0; i < n; ++i) {
    mix((uint64_t)(uintptr_t)jobs[i].buf);
    mix((uint64_t)(uint32_t)jobs[i].elem_bytes | ((uint64_t)(uint32_t)jobs[i].op << 32));
    mix((uint64_t)jobs[i].d0);
    mix((uint64_t)jobs[i].d1);
    mix((uint64_t)jobs[i].d2);
    mix((uint64_t)jobs[i].d3);
  }
  return h;
}

static bool same_jobs(const std::vector<lm_job> &kept, const lm_job *jobs,
                      int n) {
  if (kept.size() != (size_t)n) return false;
  for (int i = 0; i < n; ++i) {
    const lm_job &a = kept[i], &b = jobs[i];
    if (a.buf != b.buf || a.elem_bytes != b.elem_bytes || a.op != b.op ||
        a.d0 != b.d0 || a.d1 != b.d1 || a.d2 != b.d2 || a.d3 != b.d3)
      return false;
  }
  return true;
}

// A captured graph holds the device addresses of the tables and the arena:
// any reallocation retires it.
static void drop_graph(lm_batch_t bt) {
  if (bt->gexec) cudaGraphExecDestroy(bt->gexec);
  bt->gexec = nullptr;
  bt->gkey = 0;
  bt->gjobs.clear();
}

// Grows the device tables, the arena and the pinned staging buffer.  Device
// memory comes from the stream-ordered pool and is released on the stream of
// the run that last used it: no device-wide synchronisation (a plain
// cudaFree would wait for all work, stalling a server).  Retired pinned
// buffers are kept until the handle is destroyed for the same reason.
static bool grow(lm_batch_t bt, cudaStream_t s, size_t njobs, size_t nitems) {
  const cudaStream_t fs = bt->used ? bt->last_stream : s;
  pool_keep_memory();
  auto regrow = [&](void **p, size_t bytes) -> bool {
    // inside a capture the pool calls would become graph-owned memory
    cudaStreamCaptureStatus cap = cudaStreamCaptureStatusNone;
    if (cudaStreamIsCapturing(s, &cap) != cudaSuccess ||
        cap != cudaStreamCaptureStatusNone)
      return false;
    if (*p) cudaFreeAsync(*p, fs);
    *p = nullptr;
    if (cudaMallocAsync(p, bytes, s) != cudaSuccess) {
      cudaGetLastError();
      *p = nullptr;
      return false;
    }
    return true;
  };
  if (bt->need_arena > bt->cap_arena) {
    drop_graph(bt);
    bt->cap_arena = 0;
    if (!regrow(reinterpret_cast<void **>(&bt->d_arena), bt->need_arena))
      return set_error("batch: cannot allocate the staging arena");
    bt->cap_arena = bt->need_arena;
  }
  if (njobs > bt->cap_jobs) {
    drop_graph(bt);
    const size_t cap = std::max<size_t>(njobs, 2 * bt->cap_jobs);
    bt->cap_jobs = 0;
    if (!regrow(reinterpret_cast<void **>(&bt->d_jobs), cap * sizeof(BJob)))
      return set_error("batch: cannot allocate the job table");
    bt->cap_jobs = cap;
  }
  if (nitems > bt->cap_items) {
    drop_graph(bt);
    const size_t cap = std::max<size_t>(nitems, 2 * bt->cap_items);
    bt->cap_items = 0;
    if (!regrow(reinterpret_cast<void **>(&bt->d_items), cap * sizeof(BItem)))
      return set_error("batch: cannot allocate the item list");
    bt->cap_items = cap;
  }
  if (!bt->d_counters &&
      !regrow(reinterpret_cast<void **>(&bt->d_counters), kCounterBytes))
    return set_error("batch: cannot allocate counters");
  const size_t stage = njobs * sizeof(BJob) + nitems * sizeof(BItem) + 256;
  if (stage > bt->cap_stage) {
    if (bt->h_stage) bt->retired_pinned.push_back(bt->h_stage);
    bt->h_stage = nullptr;
    bt->cap_stage = std::max(stage, 2 * bt->cap_stage);
    if (cudaMallocHost(&bt->h_stage, bt->cap_stage) != cudaSuccess) {
      bt->h_stage = nullptr;
      bt->cap_stage = 0;
      return set_error("batch: cannot allocate the pinned staging buffer");
    }
  }
  return false;
}

// Bytes of scratch the staged jobs of one wave may use (LM_BATCH_SCRATCH_MB
// overrides the default of 1 GiB; 0 turns the staged form off).
static uint64_t arena_bytes() {
  const char *v = getenv("LM_BATCH_SCRATCH_MB");
  if (v && *v) return (uint64_t)strtoull(v, nullptr, 10) << 20;
  return kDefaultArenaBytes;
}

static void fill_job(BJob &j, const lm_job &jb, const Normalized &nz,
                     uint32_t pitch) {
  j.base = (char *)jb.buf;
  j.e = nz.e;
  j.a = (uint32_t)nz.a;
  j.B = (uint32_t)nz.B;
  j.b = (uint32_t)nz.b;
  j.row_elems = (uint32_t)(nz.B * nz.b);
  j.aB = (uint32_t)(nz.a * nz.B);
  j.tile_elems = (uint32_t)(nz.a * nz.B * nz.b);
  j.pitch = pitch;
  j.div_row = make_fastdiv(j.row_elems);
  j.div_b = make_fastdiv(j.b);
  j.div_aB = make_fastdiv(j.aB);
  j.div_a = make_fastdiv(j.a);
  j.band = 0;
  j.ng8 = (uint32_t)((nz.a + 7) / 8);
  j.div_ng8 = make_fastdiv(j.ng8);
  j.div_na = make_fastdiv((uint32_t)std::max<uint64_t>(1, nz.a * nz.e / 16));
  {
    const uint32_t R = (uint32_t)(nz.B * nz.b * nz.e);
    j.tpitch = (R / 16) & 1 ? R : R + 16;  // an odd number of 16-byte words
    j.div_nc = make_fastdiv(std::max<uint32_t>(1, R / 16));
    j.kt = 1;
    j.div_rows = make_fastdiv((uint32_t)std::max<uint64_t>(1, nz.a));
  }
  j.scratch = nullptr;
  j.S = j.Sj = j.nJ = j.nIJ = j.nv16 = 0;
  j.bytes = 0;
}

// Staged form of a job: blocks of S rows x Sj units, rows staged as 16-byte
// aligned supersets at an odd number of 16-byte words, at most
// kStageTileBytes per block: whole rows when a row is short (tall, narrow
// matrices), whole columns when the rows are few (short, wide ones), else
// S x S with S the largest power of two up to 128 that fits.  False when a
// unit exceeds kStageTileBytes or the job has 2^32 blocks or more.
// `scratch` is left for the caller.
static bool staged_job(BJob &j, const lm_job &jb, const Normalized &nz,
                       uint64_t *nblk, size_t *stage_bytes) {
  const uint64_t unit = nz.b * (uint64_t)nz.e;
  // bytes staged per block: the tuned variant of this shape class, if any
  const uint64_t kStageTileBytes = tune_params().staged_block_bytes
                                       ? tune_params().staged_block_bytes
                                       : lm::kStageTileBytes;
  if (unit > kStageTileBytes || nz.a * nz.B * nz.b >= 0xffffffffull)
    return false;
  auto pitch_of = [&](uint64_t sj) {
    uint64_t p = (sj * unit + 15) / 16 * 16 + 16;
    if (((p / 16) & 1) == 0) p += 16;  // rows in distinct bank groups
    return p;
  };
  // whole rows while a block keeps 64 of them (output runs of 64 units);
  // whole columns while a row segment keeps 128 bytes (input runs)
  const uint64_t min_sj = std::max<uint64_t>(8, (128 + unit - 1) / unit);
  uint64_t Si, Sj;
  if (64 * pitch_of(nz.B) <= kStageTileBytes) {
    Sj = nz.B;  // whole rows
    Si = std::min<uint64_t>(kStageMaxS, kStageTileBytes / pitch_of(nz.B));
  } else if (nz.a <= kStageMaxS &&
             nz.a * pitch_of(min_sj) <= kStageTileBytes) {
    Si = nz.a;  // whole columns
    Sj = (kStageTileBytes / nz.a - 32) / unit;
    while (Sj > min_sj && nz.a * pitch_of(Sj) > kStageTileBytes) --Sj;
  } else {
    uint64_t S = 128;
    while (S > 1 && S * S * unit > kStageTileBytes) S >>= 1;
    Si = Sj = S;
    if (tune_params().staged_wide > 1) Sj = S * tune_params().staged_wide;
  }
  Si = std::min<uint64_t>(Si, nz.a);
  Sj = std::min<uint64_t>(Sj, nz.B);
  const uint64_t nI = (nz.a + Si - 1) / Si, nJ = (nz.B + Sj - 1) / Sj;
  if (nz.T * nI * nJ >= 0xffffffffull) return false;
  const uint32_t sp = (uint32_t)pitch_of(Sj);
  const uint32_t S = (uint32_t)Si;
  fill_job(j, jb, nz, sp);
  j.S = S;
  j.Sj = (uint32_t)Sj;
  j.div_S = make_fastdiv(S);
  j.nv16 = (unit % 16 == 0 && ((uintptr_t)jb.buf & 15) == 0)
               ? (uint32_t)(unit / 16) : 0u;
  // staged rows on 32-bit words (row length, buffer and block columns) and
  // output vectors on 16 bytes (output row length and block rows; the
  // scratch sits at the buffer's address modulo 16)
  j.vb1 = (nz.b == 1 && nz.e <= 2 && ((uintptr_t)jb.buf & 15) == 0 &&
           (nz.B * nz.e) % 4 == 0 && (Sj * nz.e) % 4 == 0 &&
           (nz.a * nz.e) % 16 == 0 && (S * nz.e) % 16 == 0)
              ? 1u : 0u;
  j.vbc = 0;
  if (!j.vb1 && nz.b == 1)
    for (uint32_t w : {16u, 8u, 4u})
      if (w >= (uint32_t)nz.e && (w == 16 || nz.e <= 2) &&
          (uintptr_t)jb.buf % w == 0 && (nz.a * nz.e) % w == 0 &&
          (S * nz.e) % w == 0) {
        j.vbc = w;
        break;
      }
  j.vrw = j.vb1 ? 16 / nz.e : j.vbc / nz.e;
  j.div_nv16 = make_fastdiv(j.nv16 ? j.nv16 : 1);
  j.ng8 = (S + 7) / 8;
  j.div_ng8 = make_fastdiv(j.ng8);
  j.nJ = (uint32_t)nJ;
  j.nIJ = (uint32_t)(nI * nJ);
  j.div_Sb = make_fastdiv(S * (uint32_t)nz.b);
  j.div_nJ = make_fastdiv(j.nJ);
  j.div_nIJ = make_fastdiv(j.nIJ);
  j.bytes = nz.T * nz.a * nz.B * nz.b * (uint64_t)nz.e;
  *nblk = nz.T * nI * nJ;
  // (rows shifted by 16 bytes per group of vrw rows for the vectorized
  // narrow stores)
  *stage_bytes =
      ((size_t)S * sp + (j.vrw ? 16 * ((S + j.vrw - 1) / j.vrw) : 0) + 127) /
      128 * 128;
  return true;
}


// Host planning of a job list into small items, big items, cluster items and
// large jobs.
static bool plan_batch(lm_batch_t bt, const lm_job *jobs, int n,
                       unsigned flags) {
  const DeviceInfo &di = device_info();
  const uint64_t max_tile = (uint64_t)di.max_smem_optin - 1024;
  // one of the cluster kernel's two stages, beside its row tables
  const size_t band_static = 2 * kBandMaxRows * 4 + 512;
  const size_t band_budget =
      ((size_t)di.max_smem_optin - band_static) / 2 / 128 * 128;
  // ... and the stage size that lets two CTAs share an SM (each also holds
  // 1 KB of shared memory reserved by the system)
  const size_t band_half =
      ((size_t)di.max_smem_per_sm / 2 - 1024 - band_static) / 2 / 128 * 128;
  bt->jobs.clear();
  bt->small.clear();
  bt->t010.clear();
  bt->t010b.clear();
  bt->t010b_stage = 0;
  bt->t010f.clear();
  bt->big.clear();
  for (int gi = 0; gi < kBandGroups; ++gi) {
    bt->band[gi].clear();
    bt->band_smem[gi] = 0;
  }
  bt->large.clear();
  for (int w = 0; w < kMaxWaves; ++w) {
    bt->wgather[w].clear();
    bt->wcopy[w].clear();
    bt->wsmem[w] = 0;
  }
  bt->nwaves = 0;
  bt->need_arena = 0;
  uint64_t wave_used = 0;
  const uint64_t arena_cap = (flags & LM_BATCH_NO_SCRATCH) ? 0
                             : bt->arena_limit    ? bt->arena_limit
                                                  : arena_bytes();
  bt->norm.assign(n, Normalized());
  memset(&bt->stats, 0, sizeof(bt->stats));
  for (int k = 0; k < n; ++k) {
    const lm_job &jb = jobs[k];
    if (jb.elem_bytes != 1 && jb.elem_bytes != 2 && jb.elem_bytes != 4 &&
        jb.elem_bytes != 8) {
      char m[128];
      snprintf(m, sizeof(m), "batch: job %d: element size must be 1/2/4/8", k);
      return set_error(m);
    }
    Normalized nz = normalize(jb);
    if (!nz.ok) {
      char m[128];
      snprintf(m, sizeof(m), "batch: job %d: bad op or dimensions", k);
      return set_error(m);
    }
    bt->norm[k] = nz;
    const uint64_t bytes = nz.T * nz.a * nz.B * nz.b * (uint64_t)jb.elem_bytes;
    bt->stats.bytes += bytes;
    if (nz.T == 0 || nz.a <= 1 || nz.B <= 1 || nz.b == 0) {
      bt->stats.identity += 1;  // nothing to move
      continue;
    }
    if (jb.buf == nullptr) {
      char m[128];
      snprintf(m, sizeof(m), "batch: job %d: null buffer", k);
      return set_error(m);
    }
    if ((uintptr_t)jb.buf % (uintptr_t)jb.elem_bytes) {
      char m[128];
      snprintf(m, sizeof(m),
               "batch: job %d: buffer must be aligned to the element size", k);
      return set_error(m);
    }
    // units move whole: widen the element where the units and the buffer
    // allow (fewer, wider accesses; the same permutation of bytes)
    widen_units(jb.buf, &nz.e, &nz.b);
    bt->norm[k] = nz;
    const int e = nz.e;
    const uint64_t row_elems = nz.B * nz.b;
    const uint64_t tile_elems = row_elems * nz.a;
    const uint32_t pitch = batch_pitch(row_elems * e, e);
    const uint64_t tile_smem = (uint64_t)pitch * nz.a;
    // a large job of one-element units in small tiles runs as its own
    // launch of the 16-byte tile kernel (on a side stream, beside the rest)
    if (nz.b == 1 && bytes >= kTile010PreferBytes &&
        tile010_applies(jb.buf, e, nz.T, nz.a, nz.B) &&
        !getenv("LM_NO_TILE010")) {
      bt->large.push_back((uint32_t)k);
      bt->stats.large_jobs += 1;
      bt->stats.large_bytes += bytes;
      continue;
    }
    // tiles above kT010BatchBytes up to 112 KB with whole-vector output rows
    // on an aligned buffer: the batched 16-byte tile kernel, one tile per
    // item (two stages of the largest tile)
    if (nz.b == 1 && ((uintptr_t)jb.buf & 15) == 0 &&
        (nz.a * (uint64_t)e) % 16 == 0 && tile_elems * e > kT010BatchBytes &&
        tile_elems * e <= 112 * 1024 &&
        2 * ((tile_elems * e + 127) / 128 * 128) <= max_tile &&
        !getenv("LM_NO_TILE010")) {
      BJob j;
      fill_job(j, jb, nz, pitch);
      const uint32_t jid = (uint32_t)bt->jobs.size();
      bt->jobs.push_back(j);
      for (uint64_t t0 = 0; t0 < nz.T; ++t0) {
        BItem it;
        it.job = jid;
        it.tile0 = t0;
        it.ntiles = 1;
        bt->t010b.push_back(it);
      }
      bt->t010b_stage = std::max<size_t>(
          bt->t010b_stage, (size_t)((tile_elems * e + 127) / 128 * 128));
      bt->stats.small_jobs += 1;
      bt->stats.small_bytes += bytes;
      continue;
    }
    if (tile_elems >= 0xffffffffull || tile_smem > kSmallItem) {
      uint32_t band = 0, bpitch = 0;
      bool two_per_sm = false;
      int gi = (flags & LM_BATCH_NO_CLUSTER)
                   ? -1
                   : band_group(nz.a, nz.B, nz.b, e, band_budget,
                                band_half, &band, &bpitch, &two_per_sm);
      const uint64_t unit = nz.b * (uint64_t)e;
      const uint64_t foot = (bytes + 255) / 256 * 256 + 256;
      const bool stageable = foot <= arena_cap && unit <= kStageTileBytes &&
                             tile_elems < 0xffffffffull;
      // clusters of 8 or 16 CTAs, one per SM, leave a fifth of the SMs idle
      // (whole clusters per GPC) and hold little in flight per CTA: the
      // staged form moves such tiles faster
      if (gi >= 2 && !two_per_sm && stageable) gi = -1;
      if (gi >= 0) {
        BJob j;
        fill_job(j, jb, nz, bpitch);
        j.band = band;
        const uint32_t jid = (uint32_t)bt->jobs.size();
        bt->jobs.push_back(j);
        for (uint64_t t0 = 0; t0 < nz.T; ++t0) {
          BItem it;
          it.job = jid;
          it.tile0 = t0;
          it.ntiles = 1;
          bt->band[gi].push_back(it);
        }
        bt->band_smem[gi] = std::max<size_t>(
            bt->band_smem[gi], ((size_t)bpitch * nz.a + 127) / 128 * 128);
        bt->stats.band_jobs += 1;
        bt->stats.band_bytes += bytes;
        continue;
      }
      if (tile_elems < 0xffffffffull && tile_smem <= max_tile) {
        // one CTA per tile (more than kBandMaxRows rows, or no clusters)
        BJob j;
        fill_job(j, jb, nz, pitch);
        const uint32_t jid = (uint32_t)bt->jobs.size();
        bt->jobs.push_back(j);
        for (uint64_t t0 = 0; t0 < nz.T; ++t0) {
          BItem it;
          it.job = jid;
          it.tile0 = t0;
          it.ntiles = 1;
          bt->big.push_back(it);
        }
        bt->stats.big_jobs += 1;
        bt->stats.big_bytes += bytes;
        continue;
      }
      // a large 100 that the stash plan serves (3 x payload instead of the
      // staged form's 4) goes to the planner
      if (nz.T == 1 && unit < 128 && bytes >= kStashPreferBytes &&
          nz.a >= kStashRowsPerSm * (uint64_t)di.sms &&
          nz.a * nz.B >= (1ull << 20) &&
          plan_stash(nz.a, nz.B, (uint32_t)nz.b, e).feasible)
        goto planner;
      // large jobs of units of kStagedMaxUnit bytes and more: cycle
      // following in the planner (2 x payload) is at least as fast
      if (unit >= kStagedMaxUnit && bytes >= kStashPreferBytes) goto planner;
      // a large job through scratch runs as the planner's own staged form
      // (its gather and copy back overlap the other jobs on a side stream)
      if (bytes >= kPlannerStagedBytes) goto planner;
      // staged: the job fits the arena (in the current wave or a new one)
      if (stageable) {
        if (bt->nwaves == 0 || wave_used + foot > arena_cap) {
          if (bt->nwaves == kMaxWaves) goto planner;
          bt->nwaves += 1;
          wave_used = 0;
        }
        {
          const int w = bt->nwaves - 1;
          BJob j;
          uint64_t nblk = 0;
          size_t stage = 0;
          if (!staged_job(j, jb, nz, &nblk, &stage)) goto planner;
          // same address modulo 16 as the buffer (see k_batch_copyback);
          // the arena base is set when the wave is enqueued
          j.scratch = (char *)(uintptr_t)(wave_used + ((uintptr_t)jb.buf & 15));
          const uint32_t jid = (uint32_t)bt->jobs.size();
          bt->jobs.push_back(j);
          for (uint64_t q = 0; q < nblk; q += kStageBlocksPerItem) {
            BItem it;
            it.job = jid;
            it.tile0 = q;
            it.ntiles = (uint32_t)std::min<uint64_t>(kStageBlocksPerItem, nblk - q);
            bt->wgather[w].push_back(it);
          }
          const uint64_t nvec = bytes / 16 + 1;
          for (uint64_t v = 0; v < nvec; v += kCopyVecsPerItem) {
            BItem it;
            it.job = jid;
            it.tile0 = v;
            it.ntiles = 0;
            bt->wcopy[w].push_back(it);
          }
          bt->wsmem[w] = std::max<size_t>(bt->wsmem[w], stage);
          wave_used += foot;
          bt->need_arena = std::max(bt->need_arena, wave_used);
          bt->stats.staged_jobs += 1;
          bt->stats.staged_bytes += bytes;
          continue;
        }
      }
    planner:
      bt->large.push_back((uint32_t)k);
      bt->stats.large_jobs += 1;
      bt->stats.large_bytes += bytes;
      continue;
    }
    BJob j;
    fill_job(j, jb, nz, pitch);
    const uint32_t jid = (uint32_t)bt->jobs.size();
    bt->jobs.push_back(j);
    const uint64_t tile_bytes = tile_elems * (uint64_t)e;
    // whole-vector output rows on an aligned buffer: the batched 16-byte
    // tile kernel (items of about kT010BatchBytes), else the general one
    const bool vec_ok = nz.b == 1 && ((uintptr_t)jb.buf & 15) == 0 &&
                        tile_bytes <= kT010BatchBytes && !getenv("LM_NO_TILE010");
    const bool vec = vec_ok && (nz.a * (uint64_t)e) % 16 == 0;
    const bool vecb = vec_ok && !vec && (nz.B * (uint64_t)e) % 16 == 0;
    uint64_t k_t = (vec || vecb)
                       ? std::max<uint64_t>(1, kT010BatchBytes / tile_bytes)
                       : std::max<uint64_t>(1, kSmallItem / tile_smem);
    while (k_t > 1 && k_t * tile_elems >= 0xffffffffull) --k_t;
    if (vecb) {  // rows of a full item for the form-B store
      bt->jobs[jid].kt = (uint32_t)k_t;
      bt->jobs[jid].div_rows = make_fastdiv((uint32_t)(k_t * nz.a));
    }
    for (uint64_t t0 = 0; t0 < nz.T; t0 += k_t) {
      BItem it;
      it.job = jid;
      it.tile0 = t0;
      it.ntiles = (uint32_t)std::min<uint64_t>(k_t, nz.T - t0);
      (vec ? bt->t010 : vecb ? bt->t010f : bt->small).push_back(it);
    }
    bt->stats.small_jobs += 1;
    bt->stats.small_bytes += bytes;
  }
  bt->stats.small_items = bt->small.size() + bt->t010.size() +
                          bt->t010b.size() + bt->t010f.size();
  bt->stats.big_items = bt->big.size();
  for (int gi = 0; gi < kBandGroups; ++gi)
    bt->stats.band_items += bt->band[gi].size();
  bt->stats.staged_waves = bt->nwaves;
  return false;
}

static bool launch_band(cudaStream_t s, const BJob *d_jobs,
                        const BItem *d_items, uint32_t nitems,
                        uint32_t *counter, size_t smem, int C) {
  if (nitems == 0) return false;
  const size_t dyn = 2 * smem;  // two stages
  cudaError_t err = cudaFuncSetAttribute(
      k_batch_band, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)dyn);
  if (err == cudaSuccess && C > 8)
    err = cudaFuncSetAttribute(k_batch_band,
                               cudaFuncAttributeNonPortableClusterSizeAllowed, 1);
  if (err != cudaSuccess) return set_error("batch: cluster kernel attributes");
  const DeviceInfo &di = device_info();
  cudaLaunchConfig_t cfg = {};
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributeClusterDimension;
  attr[0].val.clusterDim.x = C;
  attr[0].val.clusterDim.y = 1;
  attr[0].val.clusterDim.z = 1;
  cfg.blockDim = dim3(kBatchThreads);
  cfg.dynamicSmemBytes = dyn;
  cfg.stream = s;
  cfg.attrs = attr;
  cfg.numAttrs = 1;
  cfg.gridDim = dim3((unsigned)(C * std::max(1, di.sms / C)));
  int max_clusters = 0;
  err = cudaOccupancyMaxActiveClusters(&max_clusters, k_batch_band, &cfg);
  if (err != cudaSuccess || max_clusters < 1)
    return set_error("batch: no cluster fits the device");
  const uint64_t ncl = std::min<uint64_t>((uint64_t)max_clusters, nitems);
  cfg.gridDim = dim3((unsigned)(ncl * C));
  BatchArgs g;
  g.jobs = d_jobs;
  g.items = d_items;
  g.nitems = nitems;
  g.counter = counter;
  g.status = device_status_word();
  g.stage_bytes = (uint32_t)smem;
  if (getenv("LM_VERBOSE"))
    fprintf(stderr, "batch_band: C=%d smem=%zu items=%u clusters=%llu\n", C,
            smem, nitems, (unsigned long long)ncl);
  ProfScope ps(s, "batch_band");
  if (cudaLaunchKernelEx(&cfg, k_batch_band, g) != cudaSuccess ||
      cudaGetLastError() != cudaSuccess)
    return set_error("batch: cluster launch");
  return false;
}

static bool launch_staged(cudaStream_t s, const BJob *d_jobs,
                          const BItem *d_items, uint32_t nitems,
                          uint32_t *counter, size_t smem, bool copyback) {
  if (nitems == 0) return false;
  const DeviceInfo &di = device_info();
  auto kern = copyback ? k_batch_copyback : k_batch_gather<3>;
  // the gather keeps two stages of `smem` bytes
  const size_t dyn = copyback ? 0 : 2 * smem;
  if (dyn > 48 * 1024 &&
      cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize,
                           (int)dyn) != cudaSuccess)
    return set_error("batch: smem attribute");
  int occ = 0;
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, kern, kStageThreads,
                                                    dyn) != cudaSuccess ||
      occ < 1)
    return set_error("batch: occupancy");
  const uint32_t grid =
      (uint32_t)std::min<uint64_t>((uint64_t)di.sms * occ, nitems);
  BatchArgs g;
  g.jobs = d_jobs;
  g.items = d_items;
  g.nitems = nitems;
  g.counter = counter;
  g.status = device_status_word();
  g.stage_bytes = (uint32_t)smem;
  ProfScope ps(s, copyback ? "batch_copyback" : "batch_gather");
  kern<<<grid, kStageThreads, dyn, s>>>(g);
  if (cudaGetLastError() != cudaSuccess) return set_error("batch: launch");
  return false;
}

namespace lm {

bool staged0100_applies(uint64_t T, uint64_t a, uint64_t B, uint64_t b,
                        int e) {
  lm_job jb{};
  jb.elem_bytes = e;
  Normalized nz;
  nz.ok = true;
  nz.e = e;
  nz.T = T;
  nz.a = a;
  nz.B = B;
  nz.b = b;
  BJob j;
  uint64_t nblk;
  size_t stage;
  return T > 0 && a > 1 && B > 1 && b > 0 &&
         staged_job(j, jb, nz, &nblk, &stage);
}

// One 0100 through scratch: the staged gather writes the transposed blocks
// to `scratch` (T*a*B*b*e bytes), then a device-to-device copy brings them
// back over the buffer.
cudaError_t launch_staged0100(cudaStream_t s, void *buf, int e, uint64_t T,
                              uint64_t a, uint64_t B, uint64_t b,
                              void *scratch) {
  lm_job jb{};
  jb.buf = buf;
  jb.elem_bytes = e;
  Normalized nz;
  nz.ok = true;
  nz.e = e;
  nz.T = T;
  nz.a = a;
  nz.B = B;
  nz.b = b;
  BatchArgs g{};
  uint64_t nblk = 0;
  size_t stage = 0;
  if (!staged_job(g.single, jb, nz, &nblk, &stage)) return cudaErrorInvalidValue;
  g.single.scratch = reinterpret_cast<char *>(scratch);
  auto gather = e == 2 ? k_batch_gather<2> : k_batch_gather<3>;
  const size_t dyn = 2 * stage;
  cudaError_t err = cudaSuccess;
  if (dyn > 48 * 1024 &&
      (err = cudaFuncSetAttribute(gather,
                                  cudaFuncAttributeMaxDynamicSharedMemorySize,
                                  (int)dyn)) != cudaSuccess)
    return err;
  int occ = 0;
  if ((err = cudaOccupancyMaxActiveBlocksPerMultiprocessor(
           &occ, gather, kStageThreads, dyn)) != cudaSuccess)
    return err;
  const DeviceInfo &di = device_info();
  const uint32_t grid = (uint32_t)std::min<uint64_t>(
      (uint64_t)di.sms * std::max(occ, 1), nblk);
  g.jobs = nullptr;
  g.items = nullptr;
  g.nitems = (uint32_t)nblk;
  g.counter = nullptr;
  g.status = device_status_word();
  g.stage_bytes = (uint32_t)stage;
  {
    ProfScope ps(s, "staged_gather");
    gather<<<grid, kStageThreads, dyn, s>>>(g);
    if ((err = cudaGetLastError()) != cudaSuccess) return err;
  }
  if (g.single.bytes <= kL2StageMinBytes || g.single.bytes > kL2StageMaxBytes ||
      (((uintptr_t)buf ^ (uintptr_t)scratch) & 15) || getenv("LM_NO_L2STAGE"))
    return cudaMemcpyAsync(buf, scratch, g.single.bytes,
                           cudaMemcpyDeviceToDevice, s);
  // much of the scratch is still in L2: copy it back and drop it there
  const uint64_t wins = g.single.bytes / 512 + 2;
  const uint32_t cgrid = (uint32_t)std::max<uint64_t>(
      1, std::min<uint64_t>((uint64_t)di.sms * 8,
                            (wins + kStageThreads / 32 - 1) / (kStageThreads / 32)));
  ProfScope ps(s, "stage_copyback");
  k_stage_copyback<<<cgrid, kStageThreads, 0, s>>>(
      reinterpret_cast<char *>(buf), reinterpret_cast<const char *>(scratch),
      g.single.bytes);
  return cudaGetLastError();
}

// ---- 0100 held whole in shared memory ---------------------------------------
// A payload that fits the shared memory of all SMs together moves in place
// in one cooperative launch at 2 x payload: every CTA copies its blocks of
// the staged form's block grid (blocks blockIdx.x + k * gridDim.x) into
// shared memory, the CTAs meet at a grid barrier (every read of the buffer
// is done before any write), then each writes its blocks transposed straight
// over the buffer.  The barrier counts arrivals in one word of a ring that
// only grows: the host hands every launch a slot and the count that slot
// reaches when all of the launch's CTAs have arrived, so no word is ever
// reset (and a captured launch, whose count would be stale on replay, takes
// the staged form instead).
constexpr uint32_t kResMaxBlocks = 16;  // blocks one CTA holds
constexpr uint32_t kResSlots = 1024;
__device__ uint32_t g_res_arrivals[kResSlots];

struct ResArgs {
  BJob job;              // the staged form's job, written over itself
  uint32_t nblk;         // blocks of the job
  uint32_t nper;         // most blocks of one CTA
  uint32_t stage_bytes;  // shared-memory bytes of one block
  uint32_t slot, target;
  uint32_t *status;
  uint64_t timeout_ns;
};

__global__ void __launch_bounds__(kStageThreads, 1) k_resident(ResArgs g) {
  extern __shared__ __align__(128) unsigned char smem[];
  __shared__ __align__(8) uint64_t bar;
  __shared__ __align__(16) BJob s_job;
  __shared__ int s_ok;
  const uint32_t warp = threadIdx.x >> 5, nw = kStageThreads / 32;
  const uint32_t nmine =
      g.nblk > blockIdx.x ? (g.nblk - blockIdx.x + gridDim.x - 1) / gridDim.x
                          : 0;
  uint32_t *rowoff =
      reinterpret_cast<uint32_t *>(smem + (size_t)g.nper * g.stage_bytes);
  if (threadIdx.x == 0) {
    mbar_init(&bar, nw);
    fence_mbar_init();
    s_ok = 1;
  }
  if (warp == 0) copy_job(&s_job, &g.job);
  __syncthreads();
  // every row of every block by its own bulk copy, spread over all warps;
  // one barrier for all of them
  RowCopy rc[kResMaxBlocks];
  uint32_t bytes = 0;
#pragma unroll
  for (uint32_t k = 0; k < kResMaxBlocks; ++k)
    if (k < nmine) {
      rc[k] = gather_row_plan(s_job, blockIdx.x + k * gridDim.x,
                              rowoff + k * s_job.S);
      bytes += rc[k].bytes;
    }
  gather_arrive(&bar, bytes);
  __syncthreads();  // every warp's expected bytes before any copy
#pragma unroll
  for (uint32_t k = 0; k < kResMaxBlocks; ++k)
    if (k < nmine)
      gather_row_issue(rc[k], smem + (size_t)k * g.stage_bytes, &bar);
  bool landed = true;
  const uint64_t t0 = global_timer_ns();
  while (!mbar_try_wait(&bar, 0))
    if (global_timer_ns() - t0 > g.timeout_ns) {
      landed = false;
      break;
    }
  if (!landed) s_ok = 0;
  __syncthreads();
  // grid barrier: every CTA arrives exactly once, then waits (bounded) for
  // the slot to reach the launch's target
  if (threadIdx.x == 0) {
    uint32_t *ctr = &g_res_arrivals[g.slot];
    __threadfence();
    atomicAdd(ctr, 1u);
    const uint64_t t1 = global_timer_ns();
    while ((int32_t)(ld_acquire_gpu(ctr) - g.target) < 0) {
      if (global_timer_ns() - t1 > g.timeout_ns) {
        s_ok = 0;
        break;
      }
      __nanosleep(32);
    }
    if (!s_ok && g.status) atomicExch(g.status, kStatusWaitTimeout);
  }
  __syncthreads();
  if (s_ok) {
    for (uint32_t k = 0; k < nmine; ++k) {
      const uint32_t q = blockIdx.x + k * gridDim.x;
      const unsigned char *buf = smem + (size_t)k * g.stage_bytes;
      const uint32_t *ro = rowoff + k * s_job.S;
      switch (s_job.e) {
        case 1: gather_store<1>(s_job, q, buf, ro); break;
        case 2: gather_store<2>(s_job, q, buf, ro); break;
        case 4: gather_store<4>(s_job, q, buf, ro); break;
        default: gather_store<8>(s_job, q, buf, ro); break;
      }
    }
    return;
  }
  // nothing may still be landing in shared memory when the CTA exits
  const uint64_t t2 = global_timer_ns();
  while (!mbar_try_wait(&bar, 0) && global_timer_ns() - t2 < g.timeout_ns) {
  }
}

namespace {

// Per device: the dynamic shared memory k_resident may take, and the
// arrivals each barrier slot has been given so far.
struct ResDevice {
  size_t max_dyn = 0;
  uint32_t next = 0;
  uint32_t arrivals[kResSlots] = {};
};
std::mutex g_res_mu;
ResDevice *g_res_dev[64];

// The block grid of a resident 0100.  Candidates: the staged form's blocks
// (the largest of 32, 16 or 8 KB that fits) with 1, 2 or 4 times the
// columns of its square blocks; each CTA holds at most kResMaxBlocks of
// them.  The pick minimises a CTA's load and store time, modelled from the
// 7200 x 1800 and 4000 x 4000 transpositions on GB300 as about 7.6 ns per
// staged row (a bulk copy each, issued by the CTA's warps in turn) plus
// 12.5 ns per KB staged; a tie goes to narrower blocks.  (7200 x 1800
// bytes: 0.0161 ms with 128 x 128 blocks, 0.0126 with 128 x 512.)
bool plan_resident(ResArgs &g, uint32_t *grid, size_t *dyn, void *buf,
                   uint64_t T, uint64_t a, uint64_t B, uint64_t b, int e,
                   size_t max_dyn) {
  const DeviceInfo &di = device_info();
  lm_job jb{};
  jb.buf = buf;
  jb.elem_bytes = e;
  Normalized nz;
  nz.ok = true;
  nz.e = e;
  nz.T = T;
  nz.a = a;
  nz.B = B;
  nz.b = b;
  if (T * a * B * b * (uint64_t)e > (uint64_t)di.sms * max_dyn) return false;
  const TuneParams saved = tune_params();
  double best_cost = 0;
  bool ok = false;
  for (uint32_t wide : {1u, 2u, 4u}) {
    for (uint32_t tb : {32u << 10, 16u << 10, 8u << 10}) {
      tune_params().staged_block_bytes = tb;
      tune_params().staged_wide = wide;
      BJob j;
      uint64_t nblk = 0;
      size_t stage = 0;
      if (!staged_job(j, jb, nz, &nblk, &stage)) continue;
      const uint64_t G = std::min<uint64_t>((uint64_t)di.sms, nblk);
      const uint64_t nper = (nblk + G - 1) / G;
      const size_t need = nper * stage + (nper * j.S * 4 + 15) / 16 * 16;
      if (nper > kResMaxBlocks || need > max_dyn) continue;
      const double cost = 7.6 * (double)(nper * j.S) +
                          12.5 * (double)(nper * stage) / 1024.0;
      if (!ok || cost < best_cost) {
        best_cost = cost;
        g.job = j;
        g.nblk = (uint32_t)nblk;
        g.nper = (uint32_t)nper;
        g.stage_bytes = (uint32_t)stage;
        *grid = (uint32_t)G;
        *dyn = need;
        ok = true;
      }
      break;  // the largest block of this width that fits
    }
  }
  tune_params() = saved;
  return ok;
}

// plan_resident with the last 16 plans of this thread kept (keyed by shape,
// element size, device and the buffer's address modulo 16, which decides
// the vector stores): the planner asks whether the resident form applies
// and then launches it, and small conversions are called again and again.
bool plan_resident_cached(ResArgs &g, uint32_t *grid, size_t *dyn, void *buf,
                          uint64_t T, uint64_t a, uint64_t B, uint64_t b,
                          int e, size_t max_dyn) {
  struct Entry {
    uint64_t T = 0, a = 0, B = 0, b = 0;
    size_t max_dyn = 0;
    int e = 0, dev = -1;
    uint32_t mis = 0;
    bool used = false, ok = false;
    ResArgs g{};
    uint32_t grid = 0;
    size_t dyn = 0;
  };
  static thread_local Entry cache[16];
  static thread_local uint32_t next = 0;
  const int dev = device_info().device;
  const uint32_t mis = (uint32_t)((uintptr_t)buf & 15);
  for (const Entry &c : cache) {
    if (!c.used || c.T != T || c.a != a || c.B != B || c.b != b || c.e != e ||
        c.dev != dev || c.mis != mis || c.max_dyn != max_dyn)
      continue;
    if (c.ok) {
      g = c.g;
      g.job.base = reinterpret_cast<char *>(buf);
      *grid = c.grid;
      *dyn = c.dyn;
    }
    return c.ok;
  }
  Entry &c = cache[next++ % 16];
  c = Entry();
  c.T = T, c.a = a, c.B = B, c.b = b, c.e = e, c.dev = dev, c.mis = mis;
  c.max_dyn = max_dyn;
  c.used = true;
  c.ok = plan_resident(c.g, &c.grid, &c.dyn, buf, T, a, B, b, e, max_dyn);
  if (c.ok) {
    g = c.g;
    *grid = c.grid;
    *dyn = c.dyn;
  }
  return c.ok;
}

// The device's ResDevice, set up on first use (nullptr on failure).
ResDevice *res_device() {
  const DeviceInfo &di = device_info();
  if (di.device < 0 || di.device >= 64) return nullptr;
  std::lock_guard<std::mutex> lock(g_res_mu);
  ResDevice *d = g_res_dev[di.device];
  if (d) return d;
  cudaFuncAttributes fa{};
  if (cudaFuncGetAttributes(&fa, k_resident) != cudaSuccess) return nullptr;
  const size_t max_dyn =
      (size_t)di.max_smem_optin > fa.sharedSizeBytes
          ? ((size_t)di.max_smem_optin - fa.sharedSizeBytes) / 128 * 128
          : 0;
  if (cudaFuncSetAttribute(k_resident,
                           cudaFuncAttributeMaxDynamicSharedMemorySize,
                           (int)max_dyn) != cudaSuccess)
    return nullptr;
  d = new ResDevice;
  d->max_dyn = max_dyn;
  g_res_dev[di.device] = d;
  return d;
}

}  // namespace

bool resident0100_applies(uint64_t T, uint64_t a, uint64_t B, uint64_t b,
                          int e) {
  if (T == 0 || a <= 1 || B <= 1 || b == 0) return false;
  ResDevice *d = res_device();
  if (!d) return false;
  ResArgs g{};
  uint32_t grid = 0;
  size_t dyn = 0;
  return plan_resident_cached(g, &grid, &dyn, nullptr, T, a, B, b, e,
                              d->max_dyn);
}

cudaError_t launch_resident0100(cudaStream_t s, void *buf, int e, uint64_t T,
                                uint64_t a, uint64_t B, uint64_t b,
                                uint32_t *status, uint64_t timeout_ns,
                                uint32_t missing) {
  cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
  cudaError_t err = cudaStreamIsCapturing(s, &cs);
  if (err != cudaSuccess) return err;
  if (cs != cudaStreamCaptureStatusNone) return cudaErrorNotSupported;
  ResDevice *d = res_device();
  if (!d) return cudaErrorNotSupported;
  ResArgs g{};
  uint32_t grid = 0;
  size_t dyn = 0;
  if (!plan_resident_cached(g, &grid, &dyn, buf, T, a, B, b, e, d->max_dyn))
    return cudaErrorNotSupported;
  g.job.scratch = g.job.base;
  g.status = status;
  g.timeout_ns = timeout_ns;
  {
    std::lock_guard<std::mutex> lock(g_res_mu);
    g.slot = d->next++ % kResSlots;
    d->arrivals[g.slot] += grid;
    g.target = d->arrivals[g.slot] + missing;
  }
  void *args[] = {&g};
  ProfScope ps(s, "resident");
  err = cudaLaunchCooperativeKernel((const void *)k_resident, dim3(grid),
                                    dim3(kStageThreads), args, dyn, s);
  if (err != cudaSuccess) {
    // no CTA arrives: the slot keeps the count it had
    std::lock_guard<std::mutex> lock(g_res_mu);
    d->arrivals[g.slot] -= grid;
  }
  return err;
}

}  // namespace lm

static bool launch_small(cudaStream_t s, const BJob *d_jobs,
                         const BItem *d_items, uint32_t nitems,
                         uint32_t *counter) {
  if (nitems == 0) return false;
  // flat buffer: an item's bytes with its 16-byte superset; padded rows
  constexpr size_t kFlat = (kSmallItem + 32 + 127) / 128 * 128;
  const size_t smem = kFlat + kSmallItem + 256;
  const DeviceInfo &di = device_info();
  cudaError_t err = cudaFuncSetAttribute(
      k_batch_small, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  if (err != cudaSuccess) return set_error("batch: smem attribute");
  int occ = 0;
  err = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, k_batch_small,
                                                      kBatchThreads, smem);
  if (err != cudaSuccess || occ < 1) return set_error("batch: occupancy");
  const uint32_t grid =
      (uint32_t)std::min<uint64_t>((uint64_t)di.sms * occ, nitems);
  BatchArgs g{};
  g.jobs = d_jobs;
  g.items = d_items;
  g.nitems = nitems;
  g.counter = counter;
  g.status = nullptr;
  g.stage_bytes = (uint32_t)kFlat;
  ProfScope ps(s, "batch_tiles");
  k_batch_small<<<grid, kBatchThreads, smem, s>>>(g);
  if (cudaGetLastError() != cudaSuccess) return set_error("batch: launch");
  return false;
}

static bool launch_t010(cudaStream_t s, const BJob *d_jobs,
                        const BItem *d_items, uint32_t nitems,
                        uint32_t *counter, uint32_t stage, bool form_b) {
  if (nitems == 0) return false;
  const size_t smem = 2 * (size_t)stage + (form_b ? kT010BatchBytes : 0);
  static LaunchCache cache_a, cache_b;
  auto kern = form_b ? k_batch_t010<true> : k_batch_t010<false>;
  cudaError_t err = cudaSuccess;
  const int occ = prepare_launch((const void *)kern, form_b ? cache_b : cache_a,
                                 smem, kBatchThreads, &err);
  if (err != cudaSuccess || occ < 1) return set_error("batch: tile kernel setup");
  const DeviceInfo &di = device_info();
  const uint32_t grid =
      (uint32_t)std::min<uint64_t>((uint64_t)di.sms * occ, nitems);
  BatchArgs g{};
  g.jobs = d_jobs;
  g.items = d_items;
  g.nitems = nitems;
  g.counter = counter;
  g.status = nullptr;
  g.stage_bytes = stage;
  ProfScope ps(s, form_b ? "batch_tile010b" : "batch_tile010");
  kern<<<grid, kBatchThreads, smem, s>>>(g);
  if (cudaGetLastError() != cudaSuccess) return set_error("batch: launch");
  return false;
}

static bool launch_items(cudaStream_t s, const BJob *d_jobs,
                         const BItem *d_items, uint32_t nitems,
                         uint32_t *counter, size_t smem) {
  if (nitems == 0) return false;
  const DeviceInfo &di = device_info();
  cudaError_t err = cudaFuncSetAttribute(
      k_batch_bs, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  if (err != cudaSuccess) return set_error("batch: smem attribute");
  int occ = 0;
  err = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, k_batch_bs,
                                                      kBatchThreads, smem);
  if (err != cudaSuccess || occ < 1) return set_error("batch: occupancy");
  const uint32_t grid =
      (uint32_t)std::min<uint64_t>((uint64_t)di.sms * occ, nitems);
  BatchArgs g;
  g.jobs = d_jobs;
  g.items = d_items;
  g.nitems = nitems;
  g.counter = counter;
  g.status = nullptr;
  ProfScope ps(s, "batch_tiles");
  k_batch_bs<<<grid, kBatchThreads, smem, s>>>(g);
  if (cudaGetLastError() != cudaSuccess) return set_error("batch: launch");
  return false;
}

// Records the work of the planned batch on stream s.
static size_t item_count(lm_batch_t bt) {
  size_t n = bt->small.size() + bt->big.size() + bt->t010.size() +
             bt->t010b.size() + bt->t010f.size();
  for (int gi = 0; gi < kBandGroups; ++gi) n += bt->band[gi].size();
  for (int w = 0; w < bt->nwaves; ++w)
    n += bt->wgather[w].size() + bt->wcopy[w].size();
  return n;
}

static size_t stage_bytes(lm_batch_t bt) {
  return bt->jobs.size() * sizeof(BJob) + item_count(bt) * sizeof(BItem);
}

// Side streams and the events that fork them from, and join them back to,
// the batch's stream (both work under stream capture).
static bool ensure_side(lm_batch_t bt) {
  if (bt->fork) return false;
  if (cudaEventCreateWithFlags(&bt->fork, cudaEventDisableTiming) !=
          cudaSuccess ||
      cudaEventCreateWithFlags(&bt->fork2, cudaEventDisableTiming) !=
          cudaSuccess)
    return set_error("batch: fork event");
  for (int k = 0; k < kSideStreams; ++k) {
    if (cudaStreamCreateWithFlags(&bt->side[k], cudaStreamNonBlocking) !=
            cudaSuccess ||
        cudaEventCreateWithFlags(&bt->join[k], cudaEventDisableTiming) !=
            cudaSuccess)
      return set_error("batch: side stream");
  }
  // one step above the large jobs' default priority (a server's lanes keep
  // the levels above that for their own streams)
  int least = 0, greatest = 0;
  cudaDeviceGetStreamPriorityRange(&least, &greatest);
  const int prio = least > greatest ? least - 1 : least;
  for (int k = 0; k < kGroupStreams; ++k) {
    if (cudaStreamCreateWithPriority(&bt->gside[k], cudaStreamNonBlocking,
                                     prio) != cudaSuccess ||
        cudaEventCreateWithFlags(&bt->gjoin[k], cudaEventDisableTiming) !=
            cudaSuccess)
      return set_error("batch: group stream");
  }
  return false;
}

// Large jobs, longest first, each on the side stream with the least work so
// far (greedy longest-processing-time order).  Sets a bit in *used for every
// side stream it forks; the caller joins them.
static bool enqueue_large(lm_batch_t bt, cudaStream_t s, const lm_job *jobs,
                          unsigned flags, unsigned *used) {
  if (bt->large.empty()) return false;
  std::vector<uint32_t> order(bt->large);
  auto bytes_of = [&](uint32_t k) {
    const Normalized &nz = bt->norm[k];
    return nz.T * nz.a * nz.B * nz.b * (uint64_t)nz.e;
  };
  std::stable_sort(order.begin(), order.end(), [&](uint32_t x, uint32_t y) {
    return bytes_of(x) > bytes_of(y);
  });
  const int nside = std::min<int>(kSideStreams, (int)order.size());
  if (nside > 1 && ensure_side(bt)) return true;
  if (nside > 1) {
    cudaEventRecord(bt->fork, s);
    for (int k = 0; k < nside; ++k) {
      cudaStreamWaitEvent(bt->side[k], bt->fork, 0);
      *used |= 1u << k;
    }
  }
  uint64_t load[kSideStreams] = {};
  // these jobs run beside the batch's kernels
  struct Beside {
    bool saved = planner_beside_other_work();
    Beside() { planner_beside_other_work() = true; }
    ~Beside() { planner_beside_other_work() = saved; }
  } beside;
  for (uint32_t k : order) {
    int best = 0;
    for (int q = 1; q < nside; ++q)
      if (load[q] < load[best]) best = q;
    load[best] += bytes_of(k);
    const cudaStream_t qs = nside > 1 ? bt->side[best] : s;
    const Normalized &nz = bt->norm[k];
    if (run_0100_planned(qs, jobs[k].buf, nz.e, nz.T, nz.a,
                         nz.B, nz.b, (flags & LM_BATCH_NO_TUNE) ? 0 : 1))
      return true;
  }
  return false;
}

// Records the work of the planned batch on stream s; `stage` (pinned, at
// least stage_bytes) holds the uploaded tables and must stay unchanged until
// the upload has executed (for a captured graph: as long as the graph lives).
static bool enqueue_batch(lm_batch_t bt, cudaStream_t s, const lm_job *jobs,
                          unsigned flags, char *stage) {
  const size_t nj = bt->jobs.size();
  const size_t ni = item_count(bt);
  if (grow(bt, s, std::max<size_t>(nj, 1), std::max<size_t>(ni, 1)))
    return true;
  unsigned used = 0;
  // stage: jobs, then small items, big items and the cluster groups.  The
  // shared staging buffer is reused only after the previous upload from it
  // has executed.
  if (!stage && bt->uploaded) cudaEventSynchronize(bt->uploaded);
  char *h = stage ? stage : (char *)bt->h_stage;
  memcpy(h, bt->jobs.data(), nj * sizeof(BJob));
  {
    // staged jobs hold arena offsets until here
    BJob *hj = reinterpret_cast<BJob *>(h);
    for (size_t k = 0; k < nj; ++k)
      if (hj[k].S) hj[k].scratch = bt->d_arena + (uintptr_t)hj[k].scratch;
  }
  {
    BItem *dst = reinterpret_cast<BItem *>(h + nj * sizeof(BJob));
    auto put = [&](const std::vector<BItem> &v) {
      if (!v.empty()) memcpy(dst, v.data(), v.size() * sizeof(BItem));
      dst += v.size();
    };
    put(bt->small);
    put(bt->big);
    for (int gi = 0; gi < kBandGroups; ++gi) put(bt->band[gi]);
    for (int w = 0; w < bt->nwaves; ++w) {
      put(bt->wgather[w]);
      put(bt->wcopy[w]);
    }
    put(bt->t010);
    put(bt->t010b);
    put(bt->t010f);
  }
  if (nj && cudaMemcpyAsync(bt->d_jobs, h, nj * sizeof(BJob),
                            cudaMemcpyHostToDevice, s) != cudaSuccess)
    return set_error("batch: job upload");
  if (ni && cudaMemcpyAsync(bt->d_items, h + nj * sizeof(BJob),
                            ni * sizeof(BItem), cudaMemcpyHostToDevice,
                            s) != cudaSuccess)
    return set_error("batch: item upload");
  if (!stage) {
    if (!bt->uploaded &&
        cudaEventCreateWithFlags(&bt->uploaded, cudaEventDisableTiming) !=
            cudaSuccess)
      return set_error("batch: upload event");
    cudaEventRecord(bt->uploaded, s);
    bt->last_stream = s;
    bt->used = true;
  }
  if (cudaMemsetAsync(bt->d_counters, 0, kCounterBytes, s) != cudaSuccess)
    return set_error("batch: counter clear");
  // The groups are independent: the staged waves (in order, they share the
  // arena), each cluster size and the one-CTA items run on their own
  // streams, forked here from `s` and joined back at the end, so that one
  // persistent kernel's tail overlaps the others.  Launch order matters: the
  // cluster groups go first, while the SMs are free (a cluster needs all of
  // its CTA slots free in one GPC at once, which rarely happens once other
  // kernels' blocks refill SMs as they drain: the 8-CTA group of the
  // 4096-matrix list then started 5.3 ms late and ran alone at the end),
  // then the large jobs (no tables needed), then the other groups.
  const size_t off_big = bt->small.size();
  size_t off_band[kBandGroups];
  size_t off = off_big + bt->big.size();
  for (int gi = 0; gi < kBandGroups; ++gi) {
    off_band[gi] = off;
    off += bt->band[gi].size();
  }
  const size_t off_waves = off;
  for (int w = 0; w < bt->nwaves; ++w)
    off += bt->wgather[w].size() + bt->wcopy[w].size();
  const size_t off_t010 = off;
  int nq = 0;
  cudaStream_t q[kGroupStreams];
  int ngroups = (bt->nwaves > 0) + (!bt->small.empty() || !bt->big.empty()) +
                (!bt->t010.empty() || !bt->t010b.empty() || !bt->t010f.empty());
  for (int gi = 0; gi < kBandGroups; ++gi) ngroups += !bt->band[gi].empty();
  if (ngroups > 0) {
    if (ensure_side(bt)) return true;
    cudaEventRecord(bt->fork2, s);  // tables uploaded, counters cleared
  }
  unsigned gused = 0;
  auto next_stream = [&]() -> cudaStream_t {
    cudaStream_t side = bt->gside[nq];
    cudaStreamWaitEvent(side, bt->fork2, 0);
    gused |= 1u << nq;
    return q[nq++] = side;
  };
  for (int gi = kBandGroups - 1; gi >= 0; --gi) {
    if (bt->band[gi].empty()) continue;
    const cudaStream_t bs = next_stream();
    if (launch_band(bs, bt->d_jobs, bt->d_items + off_band[gi],
                    (uint32_t)bt->band[gi].size(),
                    bt->d_counters + (2 + gi) * kCounterStride,
                    bt->band_smem[gi], 2 << gi))
      return true;
  }
  if (enqueue_large(bt, s, jobs, flags, &used)) return true;
  if (bt->nwaves > 0) {
    const cudaStream_t ws0 = next_stream();
    off = off_waves;
    for (int w = 0; w < bt->nwaves; ++w) {
      uint32_t *c = bt->d_counters + (2 + kBandGroups + 2 * w) * kCounterStride;
      if (launch_staged(ws0, bt->d_jobs, bt->d_items + off,
                        (uint32_t)bt->wgather[w].size(), c, bt->wsmem[w],
                        false))
        return true;
      off += bt->wgather[w].size();
      if (launch_staged(ws0, bt->d_jobs, bt->d_items + off,
                        (uint32_t)bt->wcopy[w].size(), c + kCounterStride, 0,
                        true))
        return true;
      off += bt->wcopy[w].size();
    }
  }
  if (!bt->small.empty() || !bt->big.empty()) {
    const cudaStream_t ts = next_stream();
    if (launch_small(ts, bt->d_jobs, bt->d_items, (uint32_t)bt->small.size(),
                     bt->d_counters))
      return true;
    if (!bt->big.empty()) {
      const DeviceInfo &di = device_info();
      if (launch_items(ts, bt->d_jobs, bt->d_items + off_big,
                       (uint32_t)bt->big.size(),
                       bt->d_counters + kCounterStride,
                       (size_t)di.max_smem_optin - 1024))
        return true;
    }
  }
  if (!bt->t010.empty() || !bt->t010b.empty() || !bt->t010f.empty()) {
    const cudaStream_t vs = next_stream();
    size_t o = off_t010;
    if (launch_t010(vs, bt->d_jobs, bt->d_items + o, (uint32_t)bt->t010.size(),
                    bt->d_counters + kT010Counter * kCounterStride,
                    kT010BatchBytes, false))
      return true;
    o += bt->t010.size();
    if (launch_t010(vs, bt->d_jobs, bt->d_items + o, (uint32_t)bt->t010b.size(),
                    bt->d_counters + (kT010Counter + 1) * kCounterStride,
                    (uint32_t)bt->t010b_stage, false))
      return true;
    o += bt->t010b.size();
    // form B: rows padded by at most 16 bytes each (at most twice the
    // item's bytes per stage) and an output image of the item's size
    if (launch_t010(vs, bt->d_jobs, bt->d_items + o, (uint32_t)bt->t010f.size(),
                    bt->d_counters + (kT010Counter + 2) * kCounterStride,
                    2 * kT010BatchBytes, true))
      return true;
  }
  for (int k = 0; k < kSideStreams; ++k) {
    if (!((used >> k) & 1)) continue;
    cudaEventRecord(bt->join[k], bt->side[k]);
    cudaStreamWaitEvent(s, bt->join[k], 0);
  }
  for (int k = 0; k < kGroupStreams; ++k) {
    if (!((gused >> k) & 1)) continue;
    cudaEventRecord(bt->gjoin[k], bt->gside[k]);
    cudaStreamWaitEvent(s, bt->gjoin[k], 0);
  }
  return false;
}

extern "C" {

bool lm_batch_create(lm_batch_t *out) {
  if (!out) return set_error("batch: null handle pointer");
  *out = new lm_batch_st();
  cudaGetDevice(&(*out)->device);
  device_status_word();  // allocate outside any capture
  return false;
}

void lm_batch_destroy(lm_batch_t bt) {
  if (!bt) return;
  if (bt->gexec) cudaGraphExecDestroy(bt->gexec);
  if (bt->d_jobs) cudaFree(bt->d_jobs);
  if (bt->d_items) cudaFree(bt->d_items);
  if (bt->d_counters) cudaFree(bt->d_counters);
  if (bt->d_arena) cudaFree(bt->d_arena);  // waits for its users
  if (bt->h_stage) cudaFreeHost(bt->h_stage);
  if (bt->h_gstage) cudaFreeHost(bt->h_gstage);
  for (void *p : bt->retired_pinned) cudaFreeHost(p);
  if (bt->uploaded) cudaEventDestroy(bt->uploaded);
  for (int k = 0; k < lm::kSideStreams; ++k) {
    if (bt->side[k]) cudaStreamDestroy(bt->side[k]);
    if (bt->join[k]) cudaEventDestroy(bt->join[k]);
  }
  for (int k = 0; k < lm::kGroupStreams; ++k) {
    if (bt->gside[k]) cudaStreamDestroy(bt->gside[k]);
    if (bt->gjoin[k]) cudaEventDestroy(bt->gjoin[k]);
  }
  if (bt->fork) cudaEventDestroy(bt->fork);
  if (bt->fork2) cudaEventDestroy(bt->fork2);
  delete bt;
}

bool lm_batch_run(lm_batch_t bt, lm_stream_t stream, const lm_job *jobs,
                  int njobs, unsigned flags) {
  if (!bt) return set_error("batch: null handle");
  if (njobs < 0 || (njobs > 0 && !jobs)) return set_error("batch: bad job list");
  cudaStream_t s = (cudaStream_t)stream;
  if (flags & LM_BATCH_GRAPH) {
    const uint64_t key = hash_jobs(jobs, njobs, flags);
    if (bt->gexec && key == bt->gkey && flags == bt->gflags &&
        same_jobs(bt->gjobs, jobs, njobs)) {
      if (cudaGraphLaunch(bt->gexec, s) != cudaSuccess)
        return set_error("batch: graph launch");
      bt->last_stream = s;
      bt->used = true;
      return false;
    }
    if (key == bt->seen_key && flags == bt->seen_flags &&
        same_jobs(bt->seen_jobs, jobs, njobs)) {
      // second run of this job list: record it (everything it touches was
      // initialised by the first run, outside any capture, and the tuned
      // plans are cached), then replay
      if (plan_batch(bt, jobs, njobs, flags)) return true;
      if (grow(bt, s, std::max<size_t>(bt->jobs.size(), 1),
               std::max<size_t>(item_count(bt), 1)))
        return true;
      if (bt->gexec) {
        cudaGraphExecDestroy(bt->gexec);
        bt->gexec = nullptr;
      }
      if (bt->h_gstage) cudaFreeHost(bt->h_gstage);
      bt->h_gstage = nullptr;
      if (cudaMallocHost(&bt->h_gstage, stage_bytes(bt) + 256) != cudaSuccess) {
        bt->h_gstage = nullptr;
        return set_error("batch: cannot allocate the graph's staging buffer");
      }
      cudaStream_t cs;
      if (cudaStreamCreateWithFlags(&cs, cudaStreamNonBlocking) != cudaSuccess)
        return set_error("batch: capture stream");
      if (cudaStreamBeginCapture(cs, cudaStreamCaptureModeThreadLocal) !=
          cudaSuccess) {
        cudaStreamDestroy(cs);
        return set_error("batch: begin capture");
      }
      const bool failed = enqueue_batch(bt, cs, jobs, flags, (char *)bt->h_gstage);
      cudaGraph_t graph = nullptr;
      const cudaError_t ce = cudaStreamEndCapture(cs, &graph);
      cudaStreamDestroy(cs);
      if (failed || ce != cudaSuccess || !graph) {
        if (graph) cudaGraphDestroy(graph);
        return failed ? true : set_error("batch: end capture");
      }
      if (bt->gexec) cudaGraphExecDestroy(bt->gexec);
      bt->gexec = nullptr;
      const cudaError_t ie = cudaGraphInstantiate(&bt->gexec, graph, 0);
      cudaGraphDestroy(graph);
      if (ie != cudaSuccess) {
        bt->gexec = nullptr;
        return set_error("batch: graph instantiate");
      }
      bt->gkey = key;
      bt->gjobs.assign(jobs, jobs + njobs);
      bt->gflags = flags;
      if (cudaGraphLaunch(bt->gexec, s) != cudaSuccess)
        return set_error("batch: graph launch");
      bt->last_stream = s;
      bt->used = true;
      return false;
    }
    bt->seen_key = key;
    bt->seen_jobs.assign(jobs, jobs + njobs);
    bt->seen_flags = flags;
  }
  if (plan_batch(bt, jobs, njobs, flags)) return true;
  return enqueue_batch(bt, s, jobs, flags, nullptr);
}

bool lm_batch_set_arena(lm_batch_t bt, unsigned long long bytes) {
  if (!bt) return set_error("batch: null handle");
  bt->arena_limit = bytes;
  return false;
}

bool lm_batch_stats_get(lm_batch_t bt, lm_batch_stats *out) {
  if (!bt || !out) return set_error("batch: null argument");
  *out = bt->stats;
  return false;
}

}  // extern "C"
