// lm_noalloc.cu -- lm_transpose_100_noalloc: the 100 transposition by cycle
// following, with its done bits in a fixed device array instead of memory
// allocated per call.
//
// Who needs it: callers that must not allocate device memory while they run.
// Two common cases are a memory manager or allocator that converts layouts
// from inside its own allocation path (calling cudaMalloc or cudaMallocAsync
// there would re-enter the allocator it is implementing), and real-time
// pipelines that reserve all device memory at start-up and forbid any
// allocation afterwards.  lm_transpose_100 takes its done bits from the
// stream-ordered pool; this entry point takes them from the array below.
//
// Limits and sharing:
//  * the array holds kNoAllocFlagBytes = 4 MiB, one bit per unit (a unit is
//    b elements; a unit larger than one slice -- at most 4 KiB -- counts once
//    per slice), so at most 33,554,432 units per call; larger shapes are
//    rejected with an error;
//  * every GPU that loads the library holds the array until the process exits;
//  * all calls on a device share the array and it keeps the last call's
//    contents: each call clears the bits it uses (cudaMemsetAsync on its
//    stream) before its kernel, so calls that overlap on the GPU (different
//    streams, or the same buffer from several host threads without ordering)
//    race on the bits and give wrong results -- order them on one stream;
//  * the first call on each device sets the device up: it looks up the
//    array's device address (cudaGetSymbolAddress, with that device
//    current), loads every variant of the transposition kernel (where the
//    CUDA runtime loads modules lazily, a first launch could otherwise take
//    device memory), and clears one word of the array on the call's stream.
//    A call with zero sizes does exactly this and nothing else, so make one
//    at start-up, before the phase in which nothing may be allocated, and
//    before any stream capture.
// Nothing here calls cudaMalloc, cudaFree or any allocating routine.
#include <cstdio>
#include <mutex>

#include "lm_core.cuh"
#include "lm_internal.h"
#include "../../include/lm_marshal.h"

namespace lm {

constexpr size_t kNoAllocFlagBytes = 4u << 20;

static __device__ __align__(256) uint32_t
    g_noalloc_done_bits[kNoAllocFlagBytes / sizeof(uint32_t)];

// Device address of g_noalloc_done_bits, looked up once per device with that
// device current, together with the rest of the device's set-up.  In host
// code the array's name is only a host-side handle, so it is never passed to
// a kernel directly.
static bool noalloc_bits(cudaStream_t s, uint32_t **out) {
  static std::mutex mu;
  static uint32_t *addr[64] = {nullptr};
  int dev = 0;
  cudaError_t err = cudaGetDevice(&dev);
  if (err != cudaSuccess)
    return set_error("lm_transpose_100_noalloc: no current device");
  if (dev < 0 || dev >= 64)
    return set_error("lm_transpose_100_noalloc: device index out of range");
  std::lock_guard<std::mutex> lock(mu);
  if (addr[dev] == nullptr) {
    void *p = nullptr;
    err = cudaGetSymbolAddress(&p, g_noalloc_done_bits);
    if (err != cudaSuccess || p == nullptr)
      return set_error("lm_transpose_100_noalloc: cannot resolve the "
                       "device address of the done-bit array");
    if (pttwac_prepare() != cudaSuccess ||
        cudaMemsetAsync(p, 0, sizeof(uint32_t), s) != cudaSuccess) {
      cudaGetLastError();
      return set_error("lm_transpose_100_noalloc: device set-up failed");
    }
    addr[dev] = static_cast<uint32_t *>(p);
  }
  *out = addr[dev];
  return false;
}

}  // namespace lm

extern "C" bool lm_transpose_100_noalloc(lm_stream_t stream, void *buf,
                                         int elem_bytes, int A, int B, int b) {
  using namespace lm;
  if (elem_bytes != 1 && elem_bytes != 2 && elem_bytes != 4 && elem_bytes != 8)
    return set_error("lm_transpose_100_noalloc: element size must be 1, 2, 4 "
                     "or 8");
  if (A < 0 || B < 0 || b < 0)
    return set_error("lm_transpose_100_noalloc: dimensions must be >= 0");
  // argument checks first (no CUDA call), then the device's set-up, which
  // every call runs (a zero-size call does nothing else)
  const bool trivial = A <= 1 || B <= 1 || b == 0;  // empty or identity
  size_t need = 0;
  if (!trivial) {
    if (buf == nullptr)
      return set_error("lm_transpose_100_noalloc: null buffer");
    if (((uintptr_t)buf & (uintptr_t)(elem_bytes - 1)) != 0)
      return set_error("lm_transpose_100_noalloc: buffer must be aligned to "
                       "the element size");
    need = pttwac_flag_bytes(buf, 1, (uint32_t)A, (uint32_t)B, (uint32_t)b,
                             elem_bytes);
    if (need == 0)
      return set_error("lm_transpose_100_noalloc: A*B must be < 2^32");
    if (need > kNoAllocFlagBytes) {
      char msg[256];
      snprintf(msg, sizeof(msg),
               "lm_transpose_100_noalloc: shape needs %zu bytes of done bits; "
               "this entry point holds at most %zu (use lm_transpose_100)",
               need, kNoAllocFlagBytes);
      return set_error(msg);
    }
  }
  cudaStream_t s = (cudaStream_t)stream;
  uint32_t *bits = nullptr;
  if (noalloc_bits(s, &bits)) return true;
  if (trivial) return false;
  cudaError_t err = cudaMemsetAsync(bits, 0, need, s);
  if (err != cudaSuccess)
    return set_error("lm_transpose_100_noalloc: clearing the done bits failed");
  err = launch_pttwac0100(s, buf, elem_bytes, 1, (uint32_t)A, (uint32_t)B,
                          (uint32_t)b, bits);
  if (err != cudaSuccess)
    return set_error("lm_transpose_100_noalloc: kernel launch failed");
  return false;
}
