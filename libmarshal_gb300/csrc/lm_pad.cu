// lm_pad.cu -- in-place row padding and unpadding.
//
// Reference: kernels `padding` / `unpadding` (src/cl/cl_aos_asta.cl:813-938)
// and hosts cl_padding / cl_unpadding (src/cl_marshal.cc:821-956).
//   padding   [y][x]   -> [y][pad], columns x..pad-1 become zero;
//   unpadding [y][pad] -> [y][x],   elements y*x..y*pad-1 become zero.
// The reference orders its work-groups in a chain: every group waits, with an
// unbounded spin, until its predecessor has stored (cl_aos_asta.cl:855-858,
// 914-917), so the stores of the whole buffer are serialised.
//
// GB300 design: each CTA takes a task id from a ticket counter (tasks are
// handed out in start order), loads its outputs' sources into registers,
// publishes "loaded" with a release store, then waits -- with an acquire
// load, a backoff and a time limit -- only for the tasks whose SOURCES lie in
// its own destination range.  Those tasks always have smaller ids, and a task
// never waits before publishing its own flag, so the waits cannot form a
// cycle and the stores of independent tasks overlap.  A wait that runs out
// sets a status word (the host reports an error) and the CTA skips its
// stores; nothing spins forever.
#include "lm_core.cuh"
#include "lm_internal.h"

namespace lm {

constexpr int kPadThreads = 512;
constexpr int kPadPer = 8;
constexpr uint64_t kPadTask = (uint64_t)kPadThreads * kPadPer;

struct PadArgs {
  char *buf;
  uint64_t x, y, pad;
  uint64_t O;        // outputs = y * pad
  uint64_t ntasks;
  uint32_t *ticket;  // scratch[0]
  uint32_t *loaded;  // scratch[1 .. ntasks]
  uint32_t *never;   // scratch[ntasks + 1], never set
  uint32_t *status;
  uint64_t timeout_ns;
  int64_t stall_block;
};

__device__ __forceinline__ bool wait_flag(const uint32_t *f, uint64_t t0,
                                          uint64_t timeout_ns) {
  unsigned ns = 32;
  while (ld_acquire_gpu(f) == 0) {
    if (global_timer_ns() - t0 > timeout_ns) return false;
    __nanosleep(ns);
    if (ns < 4096) ns <<= 1;
  }
  return true;
}

// Waits (thread 0) for tasks [k_lo, k_hi] except `self`; returns false on
// timeout.  Result is broadcast through shared memory.
__device__ bool wait_range(const PadArgs &g, int64_t k_lo, int64_t k_hi,
                           uint64_t self, bool stall) {
  __shared__ int ok;
  if (threadIdx.x == 0) {
    const uint64_t t0 = global_timer_ns();
    bool good = true;
    if (stall) good = wait_flag(g.never, t0, g.timeout_ns);
    for (int64_t k = k_lo; good && k <= k_hi; ++k) {
      if ((uint64_t)k == self) continue;
      good = wait_flag(g.loaded + k, t0, g.timeout_ns);
    }
    if (!good) atomicOr(g.status, kStatusWaitTimeout);
    ok = good;
  }
  __syncthreads();
  return ok != 0;
}

template <int E>
__global__ void __launch_bounds__(kPadThreads) k_padding(PadArgs g) {
  using T = typename Elem<E>::T;
  __shared__ uint64_t task_s;
  if (threadIdx.x == 0) task_s = atomicAdd(g.ticket, 1u);
  __syncthreads();
  const uint64_t k = task_s;
  if (k >= g.ntasks) return;
  T *b = reinterpret_cast<T *>(g.buf);
  // outputs of task k: [lo, hi), counted from the back
  const uint64_t hi = g.O - k * kPadTask;
  const uint64_t lo = hi > kPadTask ? hi - kPadTask : 0;
  T v[kPadPer];
#pragma unroll
  for (int u = 0; u < kPadPer; ++u) {
    const uint64_t o = lo + (uint64_t)u * kPadThreads + threadIdx.x;
    v[u] = T(0);
    if (o < hi) {
      const uint64_t r = o / g.pad, c = o - r * g.pad;
      if (c < g.x) v[u] = __ldcg(b + r * g.x + c);
    }
  }
  __syncthreads();
  if (threadIdx.x == 0) st_release_gpu(g.loaded + k, 1u);
  // sources located in [lo, hi) are read by outputs g(s) = (s/x)*pad + s%x
  int64_t k_lo = 0, k_hi = -1;
  const uint64_t yx = g.y * g.x;
  if (lo < yx && g.x > 0) {
    const uint64_t s0 = lo, s1 = (hi < yx ? hi : yx) - 1;
    const uint64_t o_min = (s0 / g.x) * g.pad + s0 % g.x;
    const uint64_t o_max = (s1 / g.x) * g.pad + s1 % g.x;
    k_lo = (int64_t)((g.O - 1 - o_max) / kPadTask);
    k_hi = (int64_t)((g.O - 1 - o_min) / kPadTask);
  }
  if (!wait_range(g, k_lo, k_hi, k, (int64_t)k == g.stall_block)) return;
#pragma unroll
  for (int u = 0; u < kPadPer; ++u) {
    const uint64_t o = lo + (uint64_t)u * kPadThreads + threadIdx.x;
    if (o < hi) __stcg(b + o, v[u]);
  }
}

template <int E>
__global__ void __launch_bounds__(kPadThreads) k_unpadding(PadArgs g) {
  using T = typename Elem<E>::T;
  __shared__ uint64_t task_s;
  if (threadIdx.x == 0) task_s = atomicAdd(g.ticket, 1u);
  __syncthreads();
  const uint64_t k = task_s;
  if (k >= g.ntasks) return;
  T *b = reinterpret_cast<T *>(g.buf);
  const uint64_t lo = k * kPadTask;
  const uint64_t hi = (lo + kPadTask < g.O) ? lo + kPadTask : g.O;
  const uint64_t yx = g.y * g.x;
  T v[kPadPer];
#pragma unroll
  for (int u = 0; u < kPadPer; ++u) {
    const uint64_t o = lo + (uint64_t)u * kPadThreads + threadIdx.x;
    v[u] = T(0);
    if (o < hi && o < yx) {
      const uint64_t r = o / g.x, c = o - r * g.x;
      v[u] = __ldcg(b + r * g.pad + c);
    }
  }
  __syncthreads();
  if (threadIdx.x == 0) st_release_gpu(g.loaded + k, 1u);
  // sources in [lo, hi) belong to outputs [hinv(lo), hinv(hi)) where
  // hinv(s) = (s/pad)*x + min(s%pad, x)
  auto hinv = [&](uint64_t s) {
    const uint64_t r = s / g.pad, c = s - r * g.pad;
    return r * g.x + (c < g.x ? c : g.x);
  };
  int64_t k_lo = 0, k_hi = -1;
  uint64_t a0 = hinv(lo), a1 = hinv(hi);
  if (a1 > yx) a1 = yx;
  if (a0 < a1) {
    k_lo = (int64_t)(a0 / kPadTask);
    k_hi = (int64_t)((a1 - 1) / kPadTask);
  }
  if (!wait_range(g, k_lo, k_hi, k, (int64_t)k == g.stall_block)) return;
#pragma unroll
  for (int u = 0; u < kPadPer; ++u) {
    const uint64_t o = lo + (uint64_t)u * kPadThreads + threadIdx.x;
    if (o < hi) __stcg(b + o, v[u]);
  }
}

size_t pad_scratch_bytes(uint64_t x, uint64_t y, uint64_t pad) {
  const uint64_t O = y * pad;
  const uint64_t ntasks = (O + kPadTask - 1) / kPadTask;
  return (size_t)(ntasks + 2) * 4;
}

template <bool PAD>
static cudaError_t run_pad(cudaStream_t s, void *buf, int e, uint64_t x,
                           uint64_t y, uint64_t pad, uint32_t *scratch,
                           uint32_t *status, uint64_t timeout_ns,
                           int64_t stall_block) {
  if (pad < x) return cudaErrorInvalidValue;
  const uint64_t O = y * pad;
  if (O == 0 || (pad == x && stall_block < 0)) return cudaSuccess;
  PadArgs g;
  g.buf = reinterpret_cast<char *>(buf);
  g.x = x;
  g.y = y;
  g.pad = pad;
  g.O = O;
  g.ntasks = (O + kPadTask - 1) / kPadTask;
  if (g.ntasks >= 0xffffffffull) return cudaErrorInvalidValue;
  g.ticket = scratch;
  g.loaded = scratch + 1;
  g.never = scratch + 1 + g.ntasks;
  g.status = status;
  g.timeout_ns = timeout_ns;
  g.stall_block = stall_block;
  const unsigned grid = (unsigned)g.ntasks;
  ProfScope ps(s, PAD ? "padding" : "unpadding");
  switch (e) {
    case 1: PAD ? k_padding<1><<<grid, kPadThreads, 0, s>>>(g)
                : k_unpadding<1><<<grid, kPadThreads, 0, s>>>(g); break;
    case 2: PAD ? k_padding<2><<<grid, kPadThreads, 0, s>>>(g)
                : k_unpadding<2><<<grid, kPadThreads, 0, s>>>(g); break;
    case 4: PAD ? k_padding<4><<<grid, kPadThreads, 0, s>>>(g)
                : k_unpadding<4><<<grid, kPadThreads, 0, s>>>(g); break;
    case 8: PAD ? k_padding<8><<<grid, kPadThreads, 0, s>>>(g)
                : k_unpadding<8><<<grid, kPadThreads, 0, s>>>(g); break;
    default: return cudaErrorInvalidValue;
  }
  return cudaGetLastError();
}

cudaError_t launch_padding(cudaStream_t s, void *buf, int e, uint64_t x,
                           uint64_t y, uint64_t pad, uint32_t *scratch,
                           uint32_t *status, uint64_t timeout_ns,
                           int64_t stall_block) {
  return run_pad<true>(s, buf, e, x, y, pad, scratch, status, timeout_ns,
                       stall_block);
}

cudaError_t launch_unpadding(cudaStream_t s, void *buf, int e, uint64_t x,
                             uint64_t y, uint64_t pad, uint32_t *scratch,
                             uint32_t *status, uint64_t timeout_ns,
                             int64_t stall_block) {
  return run_pad<false>(s, buf, e, x, y, pad, scratch, status, timeout_ns,
                        stall_block);
}

}  // namespace lm
