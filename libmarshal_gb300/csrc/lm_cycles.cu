// lm_cycles.cu -- 100/0100 by whole-cycle moves, for shapes whose cycles are
// all short.
//
// An in-place 100(A, B) on units moves the unit at position p to A*p mod M,
// M = A*B - 1 (positions 0 and M stay): the same rule the reference's
// cycle-following kernels walk one step at a time with a done flag per unit
// (Transposition::Next, include/plan.hpp:54-56; _transpose_100,
// src/cl/cl_aos_asta.cl:352-717).  When the multiplicative order L of A
// modulo M is small (e.g. L = 12 for the SoA->ASTA shape 100(4, 2^22, 32),
// where M = 2^24 - 1), every cycle has at most L units, so:
//  * k_cycle_leaders finds each cycle's smallest position (walk at most L-1
//    steps from every position; a warp appends its leaders with one atomic);
//  * k_cycle_move gives each (cycle, granule of a unit, tile) to one thread,
//    which loads the granule of all L units into registers, then stores each
//    one a step further along the cycle.
// No flags, no waits; every unit is read once and written once, in granules
// of up to 16 bytes (8 for cycles longer than 16 units, to stay in
// registers), so a unit of >= 32 bytes moves as whole sectors.
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <algorithm>
#include <map>
#include <mutex>
#include <tuple>

#include "lm_core.cuh"
#include "lm_internal.h"

namespace lm {

namespace {

constexpr int kCycThreads = 256;

// x * y mod M by Barrett reduction, the quotient estimate off by at most
// one: 64-bit products with minv = floor((2^64 - 1) / M), or, when
// A * (M - 1) < 2^32 (W32), 32-bit products with minv32 =
// floor((2^32 - 1) / M).
struct ModM {
  uint64_t M;
  uint64_t minv;
  uint32_t minv32;
};

template <bool W32>
__device__ __forceinline__ uint32_t mulmod(uint32_t x, uint32_t y,
                                           const ModM &m) {
  if (W32) {
    const uint32_t p = x * y;
    const uint32_t q = __umulhi(p, m.minv32);
    uint32_t r = p - q * (uint32_t)m.M;
    if (r >= (uint32_t)m.M) r -= (uint32_t)m.M;
    return r;
  }
  const uint64_t p = (uint64_t)x * y;
  const uint64_t q = __umul64hi(p, m.minv);
  uint64_t r = p - q * m.M;
  if (r >= m.M) r -= m.M;
  return (uint32_t)r;
}

template <bool W32>
__global__ void __launch_bounds__(kCycThreads)
    k_cycle_leaders(uint32_t A, ModM m, uint32_t L, uint32_t *list,
                    uint32_t *count) {
  const uint32_t lane = threadIdx.x & 31;
  const uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
  // every warp runs the same number of iterations (ballot below)
  const uint64_t n = m.M - 1;  // positions 1 .. M-1
  const uint64_t iters = (n + stride - 1) / stride;
  uint64_t p = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x + 1;
  for (uint64_t it = 0; it < iters; ++it, p += stride) {
    bool lead = false;
    if (p < m.M) {
      uint32_t q = mulmod<W32>(A, (uint32_t)p, m);
      lead = q != p;  // fixed points move nothing
      for (uint32_t k = 1; lead && q != p && k < L; ++k) {
        if (q < p) lead = false;
        q = mulmod<W32>(A, q, m);
      }
    }
    const unsigned mask = __ballot_sync(kFull, lead);
    if (mask) {
      uint32_t base = 0;
      if (lane == 0) base = atomicAdd(count, (uint32_t)__popc(mask));
      base = __shfl_sync(kFull, base, 0);
      if (lead) list[base + __popc(mask & ((1u << lane) - 1))] = (uint32_t)p;
    }
  }
}

// W32: 32-bit products (see ModM) and fewer than 2^32 (cycle, granule,
// tile) triples, decomposed with FastDiv.
template <int G, int LMAX, bool W32>
__global__ void __launch_bounds__(kCycThreads, 2)
    k_cycle_move(char *base, uint64_t T, uint64_t tile_bytes, uint32_t U,
                 uint32_t A, ModM m, const uint32_t *list,
                 const uint32_t *count) {
  using V = typename Vec<G>::T;
  const uint32_t gpu = U / G;  // granules per unit
  const uint64_t ncyc = *count;
  const uint64_t total = ncyc * gpu * T;
  FastDiv div_g, div_c;
  if (W32) {
    div_g = make_fastdiv(gpu);
    div_c = make_fastdiv((uint32_t)ncyc);
  }
  for (uint64_t idx = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
       idx < total; idx += (uint64_t)gridDim.x * blockDim.x) {
    // granule fastest, then cycle, then tile
    uint64_t t;
    uint32_t g, c;
    if (W32) {
      const uint32_t rest = fdiv((uint32_t)idx, div_g);
      g = (uint32_t)idx - rest * gpu;
      const uint32_t tt = fdiv(rest, div_c);
      c = rest - tt * (uint32_t)ncyc;
      t = tt;
    } else {
      const uint64_t rest = idx / gpu;
      g = (uint32_t)(idx - rest * gpu);
      t = rest / ncyc;
      c = (uint32_t)(rest - t * ncyc);
    }
    char *tb = base + t * tile_bytes + (uint64_t)g * G;
    uint32_t pos[LMAX];
    pos[0] = list[c];
    int len = 1;
#pragma unroll
    for (int k = 1; k < LMAX; ++k) {
      const uint32_t q = mulmod<W32>(A, pos[k - 1], m);
      pos[k] = q;
      if (len == k && q != pos[0]) len = k + 1;
    }
    V v[LMAX];
#pragma unroll
    for (int k = 0; k < LMAX; ++k)
      if (k < len)
        v[k] = __ldcs(reinterpret_cast<const V *>(tb + (uint64_t)pos[k] * U));
#pragma unroll
    for (int k = 0; k < LMAX; ++k)
      if (k < len) {
        const uint32_t d = k + 1 < len ? pos[(k + 1) % LMAX] : pos[0];
        __stcs(reinterpret_cast<V *>(tb + (uint64_t)d * U), v[k]);
      }
  }
}

template <int G, bool W32>
void launch_move_w(cudaStream_t s, unsigned grid, char *base, uint64_t T,
                   uint64_t tile_bytes, uint32_t U, uint32_t A, const ModM &m,
                   uint32_t L, const uint32_t *list, const uint32_t *count) {
  if (L <= 8)
    k_cycle_move<G, 8, W32><<<grid, kCycThreads, 0, s>>>(base, T, tile_bytes,
                                                          U, A, m, list, count);
  else if (L <= 16)
    k_cycle_move<G, 16, W32><<<grid, kCycThreads, 0, s>>>(
        base, T, tile_bytes, U, A, m, list, count);
  else
    k_cycle_move<(G > 8 ? 8 : G), 32, W32><<<grid, kCycThreads, 0, s>>>(
        base, T, tile_bytes, U, A, m, list, count);
}

template <int G>
cudaError_t launch_move(cudaStream_t s, char *base, uint64_t T,
                        uint64_t tile_bytes, uint32_t U, uint32_t A,
                        const ModM &m, uint32_t L, const uint32_t *list,
                        const uint32_t *count, bool w32) {
  const DeviceInfo &di = device_info();
  const unsigned grid = (unsigned)di.sms * 8;
  ProfScope ps(s, "cycle_move");
  if (w32)
    launch_move_w<G, true>(s, grid, base, T, tile_bytes, U, A, m, L, list,
                           count);
  else
    launch_move_w<G, false>(s, grid, base, T, tile_bytes, U, A, m, L, list,
                            count);
  return cudaGetLastError();
}

// Cycle leaders depend only on (a, B): lists computed outside stream capture
// are kept per device (the first kCacheEntries shapes, kCacheBytes in all,
// until lm_marshal_finalize) and reused; a later call on another stream
// waits for the producing kernel.
constexpr int kCacheEntries = 16;
constexpr size_t kCacheBytes = 512ull << 20;
struct CycEntry {
  void *mem = nullptr;  // count word + list
  size_t bytes = 0;
  cudaEvent_t ready = nullptr;
};
std::mutex g_cyc_mu;
std::map<std::tuple<int, uint64_t, uint64_t>, CycEntry> g_cyc;

}  // namespace

uint32_t cycle_order(uint64_t A, uint64_t B, uint32_t limit) {
  if (A < 2 || B < 2) return 0;
  const unsigned __int128 M = (unsigned __int128)A * B - 1;
  if (M >= ((unsigned __int128)1 << 32)) return 0;
  const uint64_t m = (uint64_t)M;
  uint64_t x = A % m;
  for (uint32_t k = 1; k <= limit; ++k) {
    if (x == 1) return k;
    x = (uint64_t)(((unsigned __int128)x * A) % m);
  }
  return 0;
}

size_t cycle_scratch_bytes(uint64_t A, uint64_t B) {
  const uint64_t M = A * B - 1;
  // count word (padded) + a list with room for every nontrivial cycle
  return 256 + ((M - 1) / 2 + 1) * sizeof(uint32_t);
}

static cudaError_t run_leaders(cudaStream_t s, uint32_t a, const ModM &m,
                               uint32_t L, bool w32, void *mem) {
  uint32_t *count = reinterpret_cast<uint32_t *>(mem);
  uint32_t *list = reinterpret_cast<uint32_t *>((char *)mem + 256);
  cudaError_t err = cudaMemsetAsync(count, 0, sizeof(uint32_t), s);
  if (err != cudaSuccess) return err;
  const DeviceInfo &di = device_info();
  const uint64_t want = (m.M + kCycThreads - 1) / kCycThreads;
  const unsigned grid =
      (unsigned)std::min<uint64_t>(want, (uint64_t)di.sms * 16);
  ProfScope ps(s, "cycle_leaders");
  if (w32)
    k_cycle_leaders<true><<<grid, kCycThreads, 0, s>>>(a, m, L, list, count);
  else
    k_cycle_leaders<false><<<grid, kCycThreads, 0, s>>>(a, m, L, list, count);
  return cudaGetLastError();
}

// The leader list of 100(a, B): from the cache, or computed into a new
// cache entry, or (during stream capture, or with the cache full) computed
// into `scratch`.
static cudaError_t leaders_for(cudaStream_t s, uint32_t a, uint32_t B,
                               const ModM &m, uint32_t L, bool w32,
                               void *scratch, bool may_cache, void **mem) {
  auto into_scratch = [&]() {
    *mem = scratch;
    return run_leaders(s, a, m, L, w32, scratch);
  };
  if (!may_cache) return into_scratch();
  int dev = 0;
  cudaGetDevice(&dev);
  const auto key = std::make_tuple(dev, (uint64_t)a, (uint64_t)B);
  std::lock_guard<std::mutex> lock(g_cyc_mu);
  auto it = g_cyc.find(key);
  if (it != g_cyc.end()) {
    *mem = it->second.mem;
    return cudaStreamWaitEvent(s, it->second.ready, 0);
  }
  const size_t bytes = cycle_scratch_bytes(a, B);
  // a full cache admits nothing more (no eviction: freeing device memory
  // would synchronise the device); other shapes use per-call memory
  size_t total = bytes;
  for (auto &kv : g_cyc) total += kv.second.bytes;
  if ((int)g_cyc.size() >= kCacheEntries || total > kCacheBytes)
    return into_scratch();
  CycEntry en;
  en.bytes = bytes;
  // stream-ordered: a plain cudaMalloc may synchronise the device
  pool_keep_memory();
  cudaError_t err = cudaMallocAsync(&en.mem, bytes, s);
  if (err != cudaSuccess) {
    cudaGetLastError();  // clear the failed allocation's error
    return into_scratch();
  }
  if ((err = cudaEventCreateWithFlags(&en.ready, cudaEventDisableTiming)) !=
      cudaSuccess) {
    cudaFreeAsync(en.mem, s);
    return err;
  }
  if ((err = run_leaders(s, a, m, L, w32, en.mem)) != cudaSuccess ||
      (err = cudaEventRecord(en.ready, s)) != cudaSuccess) {
    cudaFreeAsync(en.mem, s);
    cudaEventDestroy(en.ready);
    return err;
  }
  g_cyc[key] = en;
  *mem = en.mem;
  return cudaSuccess;
}

void cycle_cache_clear() {
  int dev = 0;
  cudaGetDevice(&dev);
  std::lock_guard<std::mutex> lock(g_cyc_mu);
  for (auto it = g_cyc.begin(); it != g_cyc.end();) {
    if (std::get<0>(it->first) != dev) {
      ++it;
      continue;
    }
    cudaEventSynchronize(it->second.ready);
    cudaFree(it->second.mem);
    cudaEventDestroy(it->second.ready);
    it = g_cyc.erase(it);
  }
}

cudaError_t launch_cycles100(cudaStream_t s, void *buf, int e, uint64_t T,
                             uint32_t a, uint32_t B, uint32_t b, uint32_t L,
                             void *scratch, bool may_cache) {
  const uint64_t M = (uint64_t)a * B - 1;
  if (L == 0 || L > kCycleMaxLen || M >= (1ull << 32))
    return cudaErrorInvalidValue;
  ModM m;
  m.M = M;
  m.minv = ~0ull / M;
  m.minv32 = (uint32_t)(0xffffffffull / M);
  const uint32_t U = b * (uint32_t)e;
  const bool w32 = (uint64_t)a * (M - 1) < (1ull << 32);
  void *mem = nullptr;
  cudaError_t err = leaders_for(s, a, B, m, L, w32, scratch, may_cache, &mem);
  if (err != cudaSuccess) return err;
  const uint32_t *count = reinterpret_cast<const uint32_t *>(mem);
  const uint32_t *list =
      reinterpret_cast<const uint32_t *>((const char *)mem + 256);
  const uint64_t tile_bytes = (uint64_t)a * B * U;
  const uintptr_t addr = (uintptr_t)buf;
  auto fits = [&](uint32_t G) {
    return U % G == 0 && addr % G == 0 && (T == 1 || tile_bytes % G == 0);
  };
  // 32-bit work indices: (M/2 cycles at most) x granules x tiles < 2^32
  auto idx32 = [&](uint32_t G) {
    return w32 && ((M - 1) / 2 + 1) * (U / G) * T < (1ull << 32);
  };
  char *base = reinterpret_cast<char *>(buf);
  if (fits(16))
    return launch_move<16>(s, base, T, tile_bytes, U, a, m, L, list, count,
                           idx32(L > 16 ? 8 : 16));
  if (fits(8))
    return launch_move<8>(s, base, T, tile_bytes, U, a, m, L, list, count,
                          idx32(8));
  if (fits(4))
    return launch_move<4>(s, base, T, tile_bytes, U, a, m, L, list, count,
                          idx32(4));
  if (fits(2))
    return launch_move<2>(s, base, T, tile_bytes, U, a, m, L, list, count,
                          idx32(2));
  return launch_move<1>(s, base, T, tile_bytes, U, a, m, L, list, count,
                        idx32(1));
}

}  // namespace lm
