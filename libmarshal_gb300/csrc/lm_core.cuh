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

__host__ __device__ inline FastDiv make_fastdiv(uint32_t d) {
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

__host__ __device__ __forceinline__ uint64_t min64(uint64_t a, uint64_t b) {
  return a < b ? a : b;
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

// Element k (a compile-time index after unrolling) of a 16-byte vector, and
// its replacement, for E-byte elements.
template <int E>
__device__ __forceinline__ typename Elem<E>::T vec_elem(const uint4 &x,
                                                        uint32_t k) {
  const uint32_t w = k * E / 4;  // 32-bit word holding the element
  const uint32_t word = w == 0 ? x.x : w == 1 ? x.y : w == 2 ? x.z : x.w;
  if (E == 8) {
    const uint32_t hi = w == 0 ? x.y : w == 2 ? x.w : 0u;
    return (typename Elem<E>::T)(((uint64_t)hi << 32) | word);
  }
  if (E == 4) return (typename Elem<E>::T)word;
  const uint32_t sh = (k * E % 4) * 8;
  return (typename Elem<E>::T)(word >> sh);
}

template <int E>
__device__ __forceinline__ void vec_set(uint4 &x, uint32_t k,
                                        typename Elem<E>::T v) {
  const uint32_t w = k * E / 4;
  uint32_t *p = w == 0 ? &x.x : w == 1 ? &x.y : w == 2 ? &x.z : &x.w;
  if (E == 8) {
    const uint64_t v64 = (uint64_t)v;
    *p = (uint32_t)v64;
    if (w == 0) x.y = (uint32_t)(v64 >> 32);
    else x.w = (uint32_t)(v64 >> 32);
    return;
  }
  if (E == 4) {
    *p = (uint32_t)v;
    return;
  }
  const uint32_t sh = (k * E % 4) * 8;
  const uint32_t mask = (E == 1 ? 0xffu : 0xffffu) << sh;
  *p = (*p & ~mask) | (((uint32_t)v << sh) & mask);
}

// 16/E elements packed into one 16-byte vector, element 0 in the lowest
// bytes.
template <int E>
__device__ __forceinline__ uint4 pack16(const typename Elem<E>::T (&x)[16 / E]) {
  if constexpr (E == 1) {
    uint32_t w[4];
#pragma unroll
    for (int q = 0; q < 4; ++q)
      w[q] = __byte_perm(__byte_perm(x[4 * q], x[4 * q + 1], 0x0040),
                         __byte_perm(x[4 * q + 2], x[4 * q + 3], 0x0040),
                         0x5410);
    return make_uint4(w[0], w[1], w[2], w[3]);
  } else if constexpr (E == 2) {
    return make_uint4(__byte_perm(x[0], x[1], 0x5410),
                      __byte_perm(x[2], x[3], 0x5410),
                      __byte_perm(x[4], x[5], 0x5410),
                      __byte_perm(x[6], x[7], 0x5410));
  } else if constexpr (E == 4) {
    return make_uint4(x[0], x[1], x[2], x[3]);
  } else {
    return make_uint4((uint32_t)x[0], (uint32_t)(x[0] >> 32), (uint32_t)x[1],
                      (uint32_t)(x[1] >> 32));
  }
}

// Output rows of `ncol` staged columns, `a` elements each, written as 16-byte
// vectors (a*E a multiple of 16 and dst 16-byte aligned): vector (ib, c)
// holds rows ib*16/E .. ib*16/E + 16/E - 1 of column c.  Lane pairs take
// the two vectors of one 32-byte sector of a column (whole-sector stores),
// pairs on consecutive columns (neighbouring shared addresses; the row
// offsets are broadcast).  Staged row r starts at buf + rowoff[r], column c
// of it at + c*E; column c is output row c at dst + c*a*E.  Threads t of nt
// take part.
template <int E>
__device__ __forceinline__ void store_columns16(const unsigned char *buf,
                                                const uint32_t *rowoff,
                                                uint32_t a, uint32_t ncol,
                                                unsigned char *dst, uint32_t t,
                                                uint32_t nt) {
  using T = typename Elem<E>::T;
  constexpr uint32_t VE = 16 / E;
  if (ncol == 0) return;
  const uint32_t NA = a / VE;             // vectors per output row
  const uint32_t G = NA >= 2 ? 2u : 1u;   // vectors of a column per lane group
  const uint32_t nvec = ((NA + G - 1) / G) * G * ncol;
  const FastDiv dc = make_fastdiv(ncol);
  const uint64_t orow = (uint64_t)a * E;
#pragma unroll 1
  for (uint32_t x = t; x < nvec; x += nt) {
    const uint32_t lo = G == 2 ? (x & 1u) : 0u;
    const uint32_t y = G == 2 ? (x >> 1) : x;
    const uint32_t hi = fdiv(y, dc);
    const uint32_t c = y - hi * ncol;
    const uint32_t ib = hi * G + lo;
    if (ib >= NA) continue;
    T v[VE];
#pragma unroll
    for (uint32_t k = 0; k < VE; ++k)
      v[k] = *reinterpret_cast<const T *>(buf + rowoff[ib * VE + k] + c * E);
    __stcg(reinterpret_cast<uint4 *>(dst + c * orow + ib * 16), pack16<E>(v));
  }
}

// V/E elements at p, p + R, p + 2R, ... packed into one V-byte vector
// (element 0 in the lowest bytes).
template <int E, int V> struct Vout;
template <int E> struct Vout<E, 16> { using T = uint4; };
template <int E> struct Vout<E, 8> { using T = uint2; };
template <int E> struct Vout<E, 4> { using T = uint32_t; };

template <int E>
__device__ __forceinline__ uint32_t gather_word(const unsigned char *p,
                                                uint32_t R) {
  // one 32-bit word: 4/E elements of a column
  if (E == 1) {
    const uint32_t x0 = p[0], x1 = p[R], x2 = p[2 * R], x3 = p[3 * R];
    return __byte_perm(__byte_perm(x0, x1, 0x0040), __byte_perm(x2, x3, 0x0040),
                       0x5410);
  } else if (E == 2) {
    const unsigned short *s = reinterpret_cast<const unsigned short *>(p);
    return __byte_perm((uint32_t)s[0], (uint32_t)s[R / 2], 0x5410);
  } else {
    return *reinterpret_cast<const uint32_t *>(p);
  }
}

template <int E, int V>
__device__ __forceinline__ typename Vout<E, V>::T gather_column(
    const unsigned char *p, uint32_t R) {
  constexpr uint32_t RW = E >= 4 ? 1 : 4 / E;  // rows per 32-bit word
  if constexpr (E == 8) {
    const uint2 lo = *reinterpret_cast<const uint2 *>(p);
    if constexpr (V == 16) {
      const uint2 hi = *reinterpret_cast<const uint2 *>(p + R);
      return make_uint4(lo.x, lo.y, hi.x, hi.y);
    } else {
      return lo;
    }
  } else if constexpr (V == 16) {
    return make_uint4(gather_word<E>(p, R), gather_word<E>(p + RW * R, R),
                      gather_word<E>(p + 2 * RW * R, R),
                      gather_word<E>(p + 3 * RW * R, R));
  } else if constexpr (V == 8) {
    return make_uint2(gather_word<E>(p, R), gather_word<E>(p + RW * R, R));
  } else {
    return gather_word<E>(p, R);
  }
}

// Drops the 128-byte L2 line at p (128-byte aligned) without writing it
// back: its contents become undefined.  For scratch that has been read for
// the last time, so that dirty staging lines never reach DRAM.
__device__ __forceinline__ void discard_l2_line(const void *p) {
  asm volatile("discard.global.L2 [%0], 128;" ::"l"(p) : "memory");
}

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

// ---- shared-memory barriers and bulk (TMA) copies ---------------------------

__device__ __forceinline__ uint32_t smem_u32(const void *p) {
  return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}

__device__ __forceinline__ void mbar_init(uint64_t *bar, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)),
               "r"(count)
               : "memory");
}

__device__ __forceinline__ void fence_mbar_init() {
  asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
}

// Orders this thread's earlier generic-proxy shared accesses before later
// async-proxy (bulk copy) accesses.
__device__ __forceinline__ void fence_proxy_async_smem() {
  asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
}

__device__ __forceinline__ void mbar_arrive_expect_tx(uint64_t *bar,
                                                      uint32_t bytes) {
  asm volatile(
      "mbarrier.arrive.expect_tx.release.cta.shared::cta.b64 _, [%0], %1;" ::
          "r"(smem_u32(bar)),
      "r"(bytes)
      : "memory");
}

__device__ __forceinline__ bool mbar_try_wait(uint64_t *bar, uint32_t parity) {
  uint32_t ok;
  asm volatile(
      "{\n\t.reg .pred p;\n\t"
      "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
      "selp.u32 %0, 1, 0, p;\n\t}"
      : "=r"(ok)
      : "r"(smem_u32(bar)), "r"(parity)
      : "memory");
  return ok != 0;
}

__device__ __forceinline__ void mbar_arrive(uint64_t *bar) {
  asm volatile("mbarrier.arrive.release.cta.shared::cta.b64 _, [%0];" ::"r"(
                   smem_u32(bar))
               : "memory");
}

// 16-byte asynchronous copy global -> shared (both addresses 16-byte aligned).
__device__ __forceinline__ void cp_async16(void *dst, const void *src) {
  asm volatile("cp.async.cg.shared.global [%0], [%1], 16;" ::"r"(smem_u32(dst)),
               "l"(src)
               : "memory");
}

__device__ __forceinline__ void cp_async_commit() {
  asm volatile("cp.async.commit_group;" ::: "memory");
}

// Waits until at most N of this thread's committed cp.async groups are
// still pending.
template <int N>
__device__ __forceinline__ void cp_async_wait_group() {
  asm volatile("cp.async.wait_group %0;" ::"n"(N) : "memory");
}

// Waits for all of this thread's committed cp.async groups.
__device__ __forceinline__ void cp_async_wait_all() {
  asm volatile("cp.async.wait_all;" ::: "memory");
}

// Arrives on `bar` once all of this thread's earlier cp.async copies have
// completed (the barrier's expected count must include this arrival).
__device__ __forceinline__ void cp_async_mbar_arrive_noinc(uint64_t *bar) {
  asm volatile("cp.async.mbarrier.arrive.noinc.shared::cta.b64 [%0];" ::"r"(
                   smem_u32(bar))
               : "memory");
}

// 1-D bulk copy global -> shared (the TMA engine); addresses and size must be
// multiples of 16 bytes; completion is signalled on `bar` as transaction bytes.
__device__ __forceinline__ void bulk_g2s(void *dst, const void *src,
                                         uint32_t bytes, uint64_t *bar) {
  asm volatile(
      "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes "
      "[%0], [%1], %2, [%3];" ::"r"(smem_u32(dst)),
      "l"(src), "r"(bytes), "r"(smem_u32(bar))
      : "memory");
}

// L2 eviction-priority policy for st_hint16: lines written under
// evict_last are chosen last when the L2 needs room.
__device__ __forceinline__ uint64_t l2_policy_evict_last() {
  uint64_t p;
  asm volatile("createpolicy.fractional.L2::evict_last.b64 %0, 1.0;" : "=l"(p));
  return p;
}

// 16-byte store with an L2 eviction-priority policy.
__device__ __forceinline__ void st_hint16(void *p, const uint4 &v,
                                          uint64_t policy) {
  asm volatile("st.global.L2::cache_hint.v4.u32 [%0], {%1, %2, %3, %4}, %5;" ::
                   "l"(p), "r"(v.x), "r"(v.y), "r"(v.z), "r"(v.w), "l"(policy)
               : "memory");
}

// Cluster barrier halves.  A relaxed arrive orders no memory accesses (use it
// where the barrier only has to order execution); the default arrive has
// release semantics and the wait acquire semantics, at cluster scope.
__device__ __forceinline__ void cluster_arrive_relaxed() {
  asm volatile("barrier.cluster.arrive.relaxed.aligned;" ::: "memory");
}
__device__ __forceinline__ void cluster_arrive_release() {
  asm volatile("barrier.cluster.arrive.release.aligned;" ::: "memory");
}
__device__ __forceinline__ void cluster_wait_acquire() {
  asm volatile("barrier.cluster.wait.acquire.aligned;" ::: "memory");
}

// Status word written by kernels that wait on other CTAs; the host turns a
// non-zero value into an error return.
enum : uint32_t {
  kStatusOk = 0,
  kStatusWaitTimeout = 1,
  kStatusBadLayout = 2,  // a kernel refused an unaligned bulk copy
};

}  // namespace lm
