// lm_pttwac.cu -- in-place transposition by parallel cycle following with
// atomic done-bits (PTTWAC).
//
// Reference algorithm: the 100/0100 kernels _transpose_100 / _transpose_100_b
// (src/cl/cl_aos_asta.cl:352-717), PTTWAC_marshal_soa
// (src/marshal_kernel.cu:96-128) and the 010 in-tile variant
// transpose_010_PTTWAC (src/cl/cl_aos_asta.cl:202-278).  The permutation is
// the reference's successor  next = (p mod B) * A + p / B  of [A][B] -> [B][A]
// (include/plan.hpp:54-56, cl_aos_asta.cl:409): positions 0 and A*B-1 are
// fixed points.
//
// GB300 design (not a translation):
//  * a "walker" is a group of L lanes (L = 1..32, power of two) that moves one
//    super-element ("unit", b*e bytes) per step with V-byte vector loads, so
//    a 128-byte unit is 8 lanes x 16 B and a warp runs 4 walkers in lockstep;
//    the reference used one (virtual) warp per unit with 4-byte accesses;
//  * one done BIT per unit in global memory (the reference used one int per
//    element on the CUDA path, 16 bits per int on OpenCL);
//  * units larger than 4 KiB are split into independent slices, each with
//    its own done bits (every slice follows the same cycles);
//  * data moves through L2 only (ld/st .cg); the claim is an atomicOr whose
//    returned old value decides the store;
//  * claim and start are the two sides of a message-passing pattern on each
//    unit: a claimer sets the unit's bit and then overwrites the unit, a
//    starter reads the unit and then checks the bit.  The claimer's lanes
//    store only after a warp barrier and a gpu-scope fence that follow the
//    atomicOr (a release); the starter's lanes fence after their data loads
//    (an acquire) before the warp barrier after which the leader reads the
//    bit.  So a starter that finds the bit clear read the unit before any
//    claimer wrote it -- otherwise a concurrent claimer could overwrite the
//    unit between our load and our check.
//  There are no waits: every step either claims a fresh bit or stops, so each
//  walk ends after at most A*B steps.
#include <algorithm>
#include <cstdio>
#include <cstdlib>

#include "lm_core.cuh"
#include "lm_internal.h"

namespace lm {

struct PttArgs {
  char *base;
  uint64_t inst_stride;  // bytes between instances
  uint64_t total;        // planes * AB start positions
  uint32_t nslices;      // slices per unit
  uint32_t A, B, AB;     // [A][B] -> [B][A] on units
  FastDiv divB;
  FastDiv divAB;         // used when total < 2^32
  FastDiv divSlices;
  uint32_t unit_bytes;
  uint32_t slice_bytes;
  uint32_t last_slice_bytes;
  uint32_t *flags;
};

template <typename VT, int K>
__global__ void __launch_bounds__(256) k_pttwac(PttArgs g, int logL) {
  constexpr int VB = (int)sizeof(VT);
  const int L = 1 << logL;
  const int lane = threadIdx.x & 31;
  const int glane = lane & (L - 1);
  const int leader = lane & ~(L - 1);
  const uint64_t walker =
      ((uint64_t)blockIdx.x * blockDim.x + threadIdx.x) >> logL;
  const uint64_t nwalkers = ((uint64_t)gridDim.x * blockDim.x) >> logL;
  const uint32_t m = g.AB - 1;
  const bool narrow = g.total <= 0xffffffffull;

  uint64_t s = walker;   // next start position (flattened plane*AB + p)
  bool walking = false;
  uint32_t pos = 0;      // unit to claim next (walking) or to start at
  uint64_t fbase = 0;    // plane * AB
  char *pbase = nullptr; // plane base address
  uint32_t slen = 0;     // bytes in this plane's slice
  VT data[K], tmp[K];

  while (true) {
    bool active = walking;
    if (!walking) {
#pragma unroll 1
      for (int tries = 0; tries < 4 && !active && s < g.total; ++tries) {
        const uint64_t cur = s;
        s += nwalkers;
        uint64_t pl;
        uint32_t p;
        if (narrow) {
          pl = fdiv((uint32_t)cur, g.divAB);
          p = (uint32_t)cur - (uint32_t)pl * g.AB;
        } else {
          pl = cur / g.AB;
          p = (uint32_t)(cur - pl * g.AB);
        }
        if (p == 0 || p >= m) continue;
        const uint32_t qq = fdiv(p, g.divB);
        const uint32_t nx = (p - qq * g.B) * g.A + qq;
        if (nx == p) continue;
        const uint64_t f = pl * g.AB + p;
        if ((__ldcg(g.flags + (f >> 5)) >> (f & 31)) & 1u) continue;
        active = true;
        pos = p;
        fbase = pl * g.AB;
        uint64_t z = pl, k = 0;
        if (g.nslices > 1) {
          z = (pl <= 0xffffffffull) ? fdiv((uint32_t)pl, g.divSlices)
                                    : pl / g.nslices;
          k = pl - z * g.nslices;
        }
        pbase = g.base + z * g.inst_stride + k * (uint64_t)g.slice_bytes;
        slen = (k + 1 == g.nslices) ? g.last_slice_bytes : g.slice_bytes;
      }
    }
    const bool more = walking || active || (s < g.total);
    if (!__any_sync(kFull, more)) break;

    const bool starting = active && !walking;
    char *uptr = pbase + (uint64_t)pos * g.unit_bytes;
#pragma unroll
    for (int c = 0; c < K; ++c) {
      const uint32_t off = (uint32_t)(glane + c * L) * VB;
      if (active && off < slen) tmp[c] = __ldcg(reinterpret_cast<const VT *>(uptr + off));
    }
    if (__any_sync(kFull, starting)) {
      // acquire: every lane's data loads before the leader's start check
      if (starting) __threadfence();
      __syncwarp();
    }
    const uint64_t f = fbase + pos;
    const uint32_t bit = 1u << (uint32_t)(f & 31);
    uint32_t old = 0;
    if (glane == 0 && active) {
      uint32_t *wp = g.flags + (f >> 5);
      old = walking ? atomicOr(wp, bit) : ld_relaxed_gpu(wp);
    }
    old = __shfl_sync(kFull, old, leader);
    const bool hit = (old & bit) != 0;
    const bool claimed = active && walking && !hit;
    if (__any_sync(kFull, claimed)) {
      // release: the leader's claim before every lane's data stores
      __syncwarp();
      if (claimed) __threadfence();
    }
    if (claimed) {
#pragma unroll
      for (int c = 0; c < K; ++c) {
        const uint32_t off = (uint32_t)(glane + c * L) * VB;
        if (off < slen) __stcg(reinterpret_cast<VT *>(uptr + off), data[c]);
      }
    }
    if (active) {
      if (!hit) {
#pragma unroll
        for (int c = 0; c < K; ++c) data[c] = tmp[c];
        const uint32_t qq = fdiv(pos, g.divB);
        pos = (pos - qq * g.B) * g.A + qq;
        walking = true;
      } else {
        walking = false;
      }
    }
  }
}

// --- host side ---------------------------------------------------------------

static int pow2_align(uint64_t v) {
  int a = 16;
  while (a > 1 && (v % (uint64_t)a) != 0) a >>= 1;
  return a;
}

struct PttShape {
  uint32_t AB = 0;
  uint32_t unit = 0, slice = 0, last = 0, nslices = 1;
  int VB = 1, K = 1, logL = 0;
  uint64_t total = 0;
};

static bool ptt_shape(const void *buf, uint64_t T, uint32_t a, uint32_t B,
                      uint32_t b, int e, PttShape &sh) {
  const uint64_t AB = (uint64_t)a * B;
  const uint64_t unit = (uint64_t)b * e;
  if (AB >= 0xffffffffull || unit >= 0xffffffffull) return false;
  sh.AB = (uint32_t)AB;
  sh.unit = (uint32_t)unit;
  const uint64_t inst = AB * unit;
  int VB = pow2_align((uint64_t)(uintptr_t)buf);
  VB = std::min(VB, pow2_align(unit));
  if (T > 1) VB = std::min(VB, pow2_align(inst));
  const uint32_t max_slice = 32u * 8u * (uint32_t)VB;
  if (sh.unit <= max_slice) {
    sh.slice = sh.unit;
    sh.nslices = 1;
  } else {
    sh.slice = max_slice;
    sh.nslices = (sh.unit + max_slice - 1) / max_slice;
  }
  sh.last = sh.unit - (sh.nslices - 1) * sh.slice;
  const uint32_t chunks = (sh.slice + VB - 1) / VB;
  int logL = 0;
  while (logL < 5 && (1u << logL) < chunks) logL++;
  const uint32_t L = 1u << logL;
  uint32_t K = (chunks + L - 1) / L;
  K = K <= 1 ? 1 : K <= 2 ? 2 : K <= 4 ? 4 : 8;
  sh.VB = VB;
  sh.K = (int)K;
  sh.logL = logL;
  sh.total = T * sh.nslices * AB;
  return true;
}

size_t pttwac_flag_bytes(const void *buf, uint64_t T, uint32_t a, uint32_t B,
                         uint32_t b, int e) {
  // The slice count (hence the bit count) depends on the buffer's alignment.
  PttShape sh;
  if (!ptt_shape(buf, T, a, B, b, e, sh)) return 0;
  return (size_t)((sh.total + 31) / 32) * 4;
}

// CTAs per SM of k_pttwac<VT, K> on the current device, queried once (the
// query also loads the kernel where modules load lazily).
template <typename VT, int K>
static cudaError_t ptt_occupancy(int *out) {
  const DeviceInfo &di = device_info();
  static int occ_cache[64] = {0};
  int &occ = occ_cache[di.device & 63];
  if (occ == 0) {
    int o = 0;
    cudaError_t err = cudaOccupancyMaxActiveBlocksPerMultiprocessor(
        &o, k_pttwac<VT, K>, 256, 0);
    if (err != cudaSuccess) return err;
    occ = o < 1 ? 1 : o;
  }
  *out = occ;
  return cudaSuccess;
}

template <typename VT, int K>
static cudaError_t run_ptt(cudaStream_t s, const PttArgs &g, int logL) {
  const DeviceInfo &di = device_info();
  int occ = 0;
  cudaError_t oerr = ptt_occupancy<VT, K>(&occ);
  if (oerr != cudaSuccess) return oerr;
  const uint64_t L = 1ull << logL;
  const uint64_t need = (g.total * L + 255) / 256;
  uint64_t blocks = (uint64_t)di.sms * occ;
  if (need < blocks) blocks = need < 1 ? 1 : need;
  if (getenv("LM_VERBOSE"))
    fprintf(stderr, "pttwac_units: VB=%d K=%d L=%d unit=%u slices=%u occ=%d "
            "blocks=%llu total=%llu\n", (int)sizeof(VT), K, 1 << logL,
            g.unit_bytes, g.nslices, occ, (unsigned long long)blocks,
            (unsigned long long)g.total);
  ProfScope ps(s, "pttwac_units");
  k_pttwac<VT, K><<<(unsigned)blocks, 256, 0, s>>>(g, logL);
  return cudaGetLastError();
}

template <typename VT>
static cudaError_t run_ptt_k(cudaStream_t s, const PttArgs &g, int logL,
                             int K) {
  switch (K) {
    case 1: return run_ptt<VT, 1>(s, g, logL);
    case 2: return run_ptt<VT, 2>(s, g, logL);
    case 4: return run_ptt<VT, 4>(s, g, logL);
    default: return run_ptt<VT, 8>(s, g, logL);
  }
}

template <typename VT>
static cudaError_t ptt_prepare_vt() {
  int occ = 0;
  cudaError_t err;
  if ((err = ptt_occupancy<VT, 1>(&occ)) != cudaSuccess) return err;
  if ((err = ptt_occupancy<VT, 2>(&occ)) != cudaSuccess) return err;
  if ((err = ptt_occupancy<VT, 4>(&occ)) != cudaSuccess) return err;
  return ptt_occupancy<VT, 8>(&occ);
}

cudaError_t pttwac_prepare() {
  cudaError_t err;
  if ((err = ptt_prepare_vt<uint4>()) != cudaSuccess) return err;
  if ((err = ptt_prepare_vt<uint2>()) != cudaSuccess) return err;
  if ((err = ptt_prepare_vt<unsigned int>()) != cudaSuccess) return err;
  if ((err = ptt_prepare_vt<unsigned short>()) != cudaSuccess) return err;
  return ptt_prepare_vt<unsigned char>();
}

cudaError_t launch_pttwac0100(cudaStream_t s, void *buf, int e, uint64_t T,
                              uint32_t a, uint32_t B, uint32_t b,
                              uint32_t *flags) {
  PttShape sh;
  if (!ptt_shape(buf, T, a, B, b, e, sh)) return cudaErrorInvalidValue;
  if (T == 0 || sh.AB <= 2 || a == 1 || B == 1 || b == 0) return cudaSuccess;
  PttArgs g;
  g.base = reinterpret_cast<char *>(buf);
  g.inst_stride = (uint64_t)sh.AB * sh.unit;
  g.total = sh.total;
  g.nslices = sh.nslices;
  g.A = a;
  g.B = B;
  g.AB = sh.AB;
  g.divB = make_fastdiv(B);
  g.divAB = make_fastdiv(sh.AB);
  g.divSlices = make_fastdiv(sh.nslices);
  g.unit_bytes = sh.unit;
  g.slice_bytes = sh.slice;
  g.last_slice_bytes = sh.last;
  g.flags = flags;
  switch (sh.VB) {
    case 16: return run_ptt_k<uint4>(s, g, sh.logL, sh.K);
    case 8: return run_ptt_k<uint2>(s, g, sh.logL, sh.K);
    case 4: return run_ptt_k<unsigned int>(s, g, sh.logL, sh.K);
    case 2: return run_ptt_k<unsigned short>(s, g, sh.logL, sh.K);
    default: return run_ptt_k<unsigned char>(s, g, sh.logL, sh.K);
  }
}

// ---- 010 in-tile cycle following, done bits in shared memory --------------

struct Ptt010Args {
  char *base;
  uint64_t A;            // tiles
  uint32_t a, B, aB;     // tile [a][B] -> [B][a]
  FastDiv divB;
  FastDiv divWords;      // by nwords
  uint32_t nwords;       // R * ceil(aB/32)
  uint32_t P;            // padding words per 32
  uint32_t padded_words;
};

template <int E>
__global__ void __launch_bounds__(1024) k_pttwac010(Ptt010Args g) {
  using T = typename Elem<E>::T;
  extern __shared__ uint32_t done[];
  const uint32_t m = g.aB - 1;
  for (uint64_t tile = blockIdx.x; tile < g.A; tile += gridDim.x) {
    for (uint32_t w = threadIdx.x; w < g.padded_words; w += blockDim.x)
      done[w] = 0;
    __syncthreads();
    T *t = reinterpret_cast<T *>(g.base) + tile * g.aB;
    for (uint32_t i = threadIdx.x; i < m; i += blockDim.x) {
      if (i == 0) continue;
      uint32_t q = fdiv(i, g.divB);
      uint32_t pos = (i - q * g.B) * g.a + q;
      if (pos == i) continue;
      // done-bit map with spreading factor: word i % nwords, bit i / nwords
      uint32_t bq = fdiv(i, g.divWords);
      uint32_t w = i - bq * g.nwords;
      w += (w >> 5) * g.P;
      if ((done[w] >> bq) & 1u) continue;
      T data = __ldcg(t + i);
      // the start check after the data load (acquire at CTA scope: every
      // claimer of this tile is a thread of this CTA)
      __threadfence_block();
      if ((reinterpret_cast<volatile uint32_t *>(done)[w] >> bq) & 1u)
        continue;
      while (true) {
        const T backup = __ldcg(t + pos);
        uint32_t pb = fdiv(pos, g.divWords);
        uint32_t pw = pos - pb * g.nwords;
        pw += (pw >> 5) * g.P;
        const uint32_t old = atomicOr(&done[pw], 1u << pb);
        if ((old >> pb) & 1u) break;
        __threadfence_block();  // release: the claim before the store
        __stcg(t + pos, data);
        data = backup;
        q = fdiv(pos, g.divB);
        pos = (pos - q * g.B) * g.a + q;
      }
    }
    __syncthreads();
  }
}

static uint32_t ptt010_words(uint32_t a, uint32_t B, int R, int P,
                             uint32_t *nwords_out) {
  const uint64_t aB = (uint64_t)a * B;
  uint64_t nwords = (uint64_t)R * ((aB + 31) / 32);
  if (nwords_out) *nwords_out = (uint32_t)nwords;
  return (uint32_t)(nwords + (nwords >> 5) * (uint64_t)P);
}

bool pttwac010_smem_fits(uint32_t a, uint32_t B, int R, int P) {
  if (R < 1 || R > 32 || (R & (R - 1)) || P < 0 || P > 32) return false;
  const uint64_t aB = (uint64_t)a * B;
  if (aB >= 0xffffffffull) return false;
  const uint64_t words = ptt010_words(a, B, R, P, nullptr);
  return words * 4 <= (uint64_t)device_info().max_smem_optin;
}

cudaError_t launch_pttwac010_smem(cudaStream_t s, void *buf, int e,
                                  uint64_t A, uint32_t a, uint32_t B, int R,
                                  int P) {
  if (!pttwac010_smem_fits(a, B, R, P)) return cudaErrorInvalidValue;
  if (A == 0 || a <= 1 || B <= 1) return cudaSuccess;
  Ptt010Args g;
  g.base = reinterpret_cast<char *>(buf);
  g.A = A;
  g.a = a;
  g.B = B;
  g.aB = a * B;
  g.divB = make_fastdiv(B);
  g.padded_words = ptt010_words(a, B, R, P, &g.nwords);
  g.divWords = make_fastdiv(g.nwords);
  g.P = (uint32_t)P;
  const size_t smem = (size_t)g.padded_words * 4;
  const DeviceInfo &di = device_info();
  cudaError_t err = cudaSuccess;
  auto go = [&](auto kern) {
    if (smem > 48 * 1024) {
      err = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                 (int)smem);
      if (err != cudaSuccess) return;
    }
    int occ = 0;
    err = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, kern, 1024, smem);
    if (err != cudaSuccess) return;
    uint64_t blocks = (uint64_t)di.sms * std::max(occ, 1);
    if (A < blocks) blocks = A;
    ProfScope ps(s, "pttwac010_smem");
    kern<<<(unsigned)blocks, 1024, smem, s>>>(g);
    err = cudaGetLastError();
  };
  switch (e) {
    case 1: go(k_pttwac010<1>); break;
    case 2: go(k_pttwac010<2>); break;
    case 4: go(k_pttwac010<4>); break;
    case 8: go(k_pttwac010<8>); break;
    default: return cudaErrorInvalidValue;
  }
  return err;
}

}  // namespace lm
