// lm_core.cuh -- device utilities shared by the layout-conversion kernels.
//
// All kernels move raw bytes; nothing is interpreted as a number, so every
// result is a pure permutation of the input and must be bit-exact.
#pragma once

#include <cstdint>
#include <cuda_runtime.h>

namespace lm {

constexpr unsigned kFull = 0xffffffffu;

// Unsigned 32-bit division by a runtime-invariant divisor: one multiply-high,
// one add and one shift (Granlund & Montgomery, "Division by invariant
// integers using multiplication", PLDI 1994, round-up variant).  Valid for
// every n < 2^32 and 1 <= d < 2^32.
struct FastDiv {
  uint32_t d;
  uint32_t mul;
  uint32_t shift;
};

inline FastDiv make_fastdiv(uint32_t d) {
  FastDiv f;
  f.d = d ? d : 1;
  uint32_t l = 0;
  while (l < 32 && (1ull << l) < f.d) l++;
  f.mul = (uint32_t)((((1ull << 32) * ((1ull << l) - f.d)) / f.d) + 1);
  f.shift = l;
  return f;
}

__device__ __forceinline__ uint32_t fdiv(uint32_t n, const FastDiv &f) {
  const uint32_t hi = __umulhi(n, f.mul);
  return (uint32_t)(((uint64_t)hi + n) >> f.shift);
}

// Vector type of V bytes.
template <int V> struct Vec;
template <> struct Vec<1> { using T = unsigned char; };
template <> struct Vec<2> { using T = unsigned short; };
template <> struct Vec<4> { using T = unsigned int; };
template <> struct Vec<8> { using T = uint2; };
template <> struct Vec<16> { using T = uint4; };

__device__ __forceinline__ uint32_t low_word(unsigned char v) { return v; }
__device__ __forceinline__ uint32_t low_word(unsigned short v) { return v; }
__device__ __forceinline__ uint32_t low_word(unsigned int v) { return v; }
__device__ __forceinline__ uint32_t low_word(uint2 v) { return v.x; }
__device__ __forceinline__ uint32_t low_word(uint4 v) { return v.x; }
__device__ __forceinline__ uint32_t low_word(unsigned long long v) {
  return (uint32_t)v;
}

// Element type of E bytes for the tile kernels.
template <int E> struct Elem;
template <> struct Elem<1> { using T = unsigned char; };
template <> struct Elem<2> { using T = unsigned short; };
template <> struct Elem<4> { using T = unsigned int; };
template <> struct Elem<8> { using T = unsigned long long; };

// Coherent (L2) 32-bit load with relaxed gpu-scope semantics.
__device__ __forceinline__ uint32_t ld_relaxed_gpu(const uint32_t *p) {
  uint32_t v;
  asm volatile("ld.relaxed.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
  return v;
}

__device__ __forceinline__ uint32_t ld_acquire_gpu(const uint32_t *p) {
  uint32_t v;
  asm volatile("ld.acquire.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
  return v;
}

__device__ __forceinline__ void st_release_gpu(uint32_t *p, uint32_t v) {
  asm volatile("st.release.gpu.global.u32 [%0], %1;" :: "l"(p), "r"(v) : "memory");
}

__device__ __forceinline__ uint64_t global_timer_ns() {
  uint64_t t;
  asm volatile("mov.u64 %0, %globaltimer;" : "=l"(t));
  return t;
}

// Status word written by kernels that wait on other CTAs; the host turns a
// non-zero value into an error return.
enum : uint32_t {
  kStatusOk = 0,
  kStatusWaitTimeout = 1,
};

}  // namespace lm
