// lm_tile010.cu -- 010 tiles [a][B] -> [B][a] of 1..8-byte elements with
// 16-byte global accesses on both sides.
//
// Reference algorithm: the BS form of the in-tile transposition (stage a
// tile on chip, write it back transposed; src/cl/cl_aos_asta.cl:53-161).
// With narrow elements the element-wise form (k_bs0100: one load, one
// shared store, one shared load and one store per element) is bound by
// instruction issue, not by HBM.  Here every global access is a 16-byte
// vector and each element costs one shared-memory access plus a byte-lane
// insert or extract:
//  * form A, a*e a multiple of 16 (every output row is whole vectors; the
//    AoS -> ASTA conversions): the chunk lands unchanged in shared memory;
//    a thread builds one output vector from 16/e consecutive rows of one
//    column -- lanes on consecutive columns, so the shared reads are free
//    of bank conflicts -- and stores it.  When a*e is only a multiple of 8
//    or 4, the output vectors are 8 or 4 bytes and the chunk (no longer
//    16-byte aligned) is loaded as its 16-byte aligned superset;
//  * form B, B*e a multiple of 16 (every input row is whole vectors; the
//    ASTA -> AoS conversions): rows land at a pitch of an odd number of
//    16-byte words; a thread reads one 16-byte piece of a row -- lanes on
//    consecutive rows -- and writes its elements into the chunk's output
//    image in shared memory, which is then stored with 16-byte vectors.
// A CTA walks chunks of whole tiles (about 16 KB) with two input stages:
// the 16-byte cp.async copies of the next chunk are in flight while the
// current one is written.  A chunk's output range is its own input range,
// so CTAs need no ordering.
#include <algorithm>
#include <cstdio>
#include <cstdlib>

#include "lm_core.cuh"
#include "lm_internal.h"

namespace lm {

constexpr int kT010Threads = 256;
constexpr uint32_t kT010Chunk = 16 * 1024;     // target input bytes per chunk
constexpr uint32_t kT010MaxTile = 112 * 1024;  // larger: the cluster form

struct T010Args {
  char *base;        // 16-byte aligned
  uint64_t T;        // tiles
  uint64_t nchunks;  // ceil(T / k)
  uint32_t a, B, k;  // rows and row elements of a tile, tiles per chunk
  uint32_t R, P;     // row bytes (B*e); staged row pitch (form B)
  uint32_t tile_bytes;
  uint32_t stage;    // shared bytes of one input stage
  uint32_t V;        // form A: output vector bytes (16, 8 or 4)
  uint32_t form_b;   // 1: form B
  FastDiv div_B;     // form A: output vectors -> (column, row block)
  FastDiv div_NA;    // form A: a*e/V vectors per output row
  FastDiv div_a;     // form B: staged row -> (tile, row)
  FastDiv div_NC;    // form B: R/16 pieces per input row
  FastDiv div_rows;  // form B: k*a rows of a full chunk
};

// All threads: 16-byte cp.async copies of chunk c into `buf` (rows at pitch
// P when PAD, else unchanged), one commit group.
template <bool PAD>
__device__ __forceinline__ void t010_issue(const T010Args &g, uint64_t c,
                                           unsigned char *buf) {
  const uint32_t nt = (uint32_t)min64(g.k, g.T - c * g.k);
  const char *src = g.base + c * g.k * (uint64_t)g.tile_bytes;
  uint32_t nv = nt * (g.tile_bytes / 16);
  if (!PAD) {
    // the 16-byte aligned superset of the chunk (whole vectors when the
    // tiles are; else up to 15 bytes more at each end)
    const uintptr_t s0 = (uintptr_t)src & ~(uintptr_t)15;
    const uintptr_t s1 = ((uintptr_t)src + (uint64_t)nt * g.tile_bytes + 15) &
                         ~(uintptr_t)15;
    nv = (uint32_t)((s1 - s0) / 16);
    src = reinterpret_cast<const char *>(s0);
  }
  for (uint32_t v = threadIdx.x; v < nv; v += kT010Threads) {
    uint32_t off = v * 16;
    if (PAD) {
      const uint32_t row = fdiv(v, g.div_NC);
      off = row * g.P + (v - row * (g.R / 16)) * 16;
    }
    cp_async16(buf + off, src + (uint64_t)v * 16);
  }
  cp_async_commit();
}

template <int E, int VA, bool FORM_B>
__global__ void __launch_bounds__(kT010Threads) k_tile010(T010Args g) {
  using T = typename Elem<E>::T;
  constexpr uint32_t VE = 16 / E;
  constexpr uint32_t VEA = VA / E;  // form A: elements per output vector
  extern __shared__ __align__(128) unsigned char smem[];
  unsigned char *img = smem + 2 * (size_t)g.stage;  // form B output image
  if (blockIdx.x >= g.nchunks) return;
  t010_issue<FORM_B>(g, blockIdx.x, smem);
  for (uint64_t c = blockIdx.x, n = 0;; c += gridDim.x, ++n) {
    const unsigned char *cur = smem + (n & 1) * (size_t)g.stage;
    const uint64_t cn = c + gridDim.x;
    const bool more = cn < g.nchunks;
    if (more) {
      // the other stage was last read before the previous pass's barrier
      t010_issue<FORM_B>(g, cn, smem + ((n & 1) ^ 1) * (size_t)g.stage);
      cp_async_wait_group<1>();
    } else {
      cp_async_wait_all();
    }
    __syncthreads();  // chunk c staged by every thread's copies
    const uint32_t nt = (uint32_t)min64(g.k, g.T - c * g.k);
    char *dst = g.base + c * g.k * (uint64_t)g.tile_bytes;
    if (!FORM_B) {
      using VT = typename Vout<E, VA>::T;
      const unsigned char *c0 = cur + ((uintptr_t)dst & 15);  // chunk start
      const uint32_t NA = g.a / VEA;
      const uint32_t nvec = nt * g.B * NA;
      const uint32_t orow = g.a * E;  // output row bytes
      for (uint32_t x = threadIdx.x; x < nvec; x += kT010Threads) {
        const uint32_t q = fdiv(x, g.div_B);
        const uint32_t jj = x - q * g.B;
        const uint32_t t = fdiv(q, g.div_NA);
        const uint32_t ib = q - t * NA;
        const uint32_t tb = t * g.tile_bytes;
        const VT v = gather_column<E, VA>(c0 + tb + ib * VEA * g.R + jj * E, g.R);
        *reinterpret_cast<VT *>(dst + tb + jj * orow + ib * VA) = v;
      }
    } else {
      const uint32_t rows = nt * g.a;
      const FastDiv dr = nt == g.k ? g.div_rows : make_fastdiv(rows);
      const uint32_t NC = g.R / 16;
      const uint32_t units = rows * NC;
      const uint32_t ostep = g.a * E;  // output row bytes
      for (uint32_t x = threadIdx.x; x < units; x += kT010Threads) {
        const uint32_t pc = fdiv(x, dr);
        const uint32_t gi = x - pc * rows;
        const uint32_t t = fdiv(gi, g.div_a);
        const uint32_t i = gi - t * g.a;
        const uint4 v = *reinterpret_cast<const uint4 *>(cur + gi * g.P + pc * 16);
        unsigned char *o = img + t * g.tile_bytes + (pc * VE * g.a + i) * E;
#pragma unroll
        for (uint32_t k = 0; k < VE; ++k)
          *reinterpret_cast<T *>(o + k * ostep) = vec_elem<E>(v, k);
      }
      __syncthreads();  // the output image is complete
      const uint32_t nv = nt * (g.tile_bytes / 16);
      for (uint32_t v = threadIdx.x; v < nv; v += kT010Threads)
        __stcg(reinterpret_cast<uint4 *>(dst) + v,
               *reinterpret_cast<const uint4 *>(img + (size_t)v * 16));
    }
    __syncthreads();  // stage and image free for the next pass
    if (!more) break;
  }
}

// --- host side ---------------------------------------------------------------

// Chunk geometry of a 010(T, a, B) on e-byte elements; false when the
// 16-byte form does not apply (unaligned buffer, no whole-vector side, or
// a tile too large for two stages in shared memory).
static bool t010_plan(const void *buf, int e, uint64_t T, uint64_t a,
                      uint64_t B, T010Args *g, size_t *smem) {
  if (e != 1 && e != 2 && e != 4 && e != 8) return false;
  if (T == 0 || a < 2 || B < 2 || ((uintptr_t)buf & 15)) return false;
  const uint64_t tile = a * B * (uint64_t)e;
  if (tile > kT010MaxTile) return false;
  // form A when both apply; form A also with 8- or 4-byte output vectors
  // when the output rows are whole such vectors (and a vector holds two
  // elements or more)
  uint32_t V = 0;
  for (uint32_t v : {16u, 8u, 4u})
    if (!V && (a * e) % v == 0 && (uint64_t)e < v) V = v;
  const bool form_b = !(V == 16) && (B * e) % 16 == 0;
  if (!form_b && !V) return false;
  const bool form_a = !form_b;
  g->base = reinterpret_cast<char *>(const_cast<void *>(buf));
  g->T = T;
  g->a = (uint32_t)a;
  g->B = (uint32_t)B;
  g->R = (uint32_t)(B * e);
  g->tile_bytes = (uint32_t)tile;
  // about 16 KB per chunk, but at least two chunks per SM when the tiles
  // are few (a small op spread over the whole GPU)
  const uint64_t spread = (T + 2 * (uint64_t)device_info().sms - 1) /
                          (2 * (uint64_t)device_info().sms);
  g->k = (uint32_t)std::max<uint64_t>(
      1, std::min<uint64_t>({T, kT010Chunk / tile, spread}));
  g->nchunks = (T + g->k - 1) / g->k;
  g->P = g->R;
  if (!form_a && ((g->P / 16) & 1) == 0) g->P += 16;  // odd 16-byte words
  g->V = form_a ? V : 16u;
  g->form_b = form_b ? 1u : 0u;
  g->stage = (uint32_t)(((form_a ? (uint64_t)g->k * tile + 32
                                 : (uint64_t)g->k * a * g->P) + 127) / 128 * 128);
  *smem = 2 * (size_t)g->stage + (form_a ? 0 : (size_t)g->k * tile);
  if (*smem > (size_t)device_info().max_smem_optin) return false;
  g->div_B = make_fastdiv(g->B);
  g->div_NA = make_fastdiv(std::max<uint32_t>(1, g->a * (uint32_t)e / g->V));
  g->div_a = make_fastdiv(g->a);
  g->div_NC = make_fastdiv(std::max<uint32_t>(1, g->R / 16));
  g->div_rows = make_fastdiv(g->k * g->a);
  return true;
}

bool tile010_applies(const void *buf, int e, uint64_t T, uint64_t a,
                     uint64_t B) {
  T010Args g;
  size_t smem;
  return t010_plan(buf, e, T, a, B, &g, &smem);
}

template <int E, int VA, bool FORM_B>
static cudaError_t run_tile010(cudaStream_t s, const T010Args &g,
                               size_t smem) {
  auto kern = k_tile010<E, VA, FORM_B>;
  static LaunchCache cache;
  cudaError_t err = cudaSuccess;
  const int occ = prepare_launch((const void *)kern, cache, smem, kT010Threads,
                                 &err);
  if (err != cudaSuccess) return err;
  uint64_t blocks = (uint64_t)device_info().sms * std::max(occ, 1);
  if (g.nchunks < blocks) blocks = g.nchunks;
  if (getenv("LM_VERBOSE"))
    fprintf(stderr, "tile010: form %c e=%d V=%d k=%u stage=%u smem=%zu occ=%d "
            "blocks=%llu chunks=%llu\n", FORM_B ? 'B' : 'A', E, VA, g.k,
            g.stage, smem, occ, (unsigned long long)blocks,
            (unsigned long long)g.nchunks);
  ProfScope ps(s, "tile010");
  kern<<<(unsigned)blocks, kT010Threads, smem, s>>>(g);
  return cudaGetLastError();
}

cudaError_t launch_tile010(cudaStream_t s, void *buf, int e, uint64_t T,
                           uint32_t a, uint32_t B) {
  T010Args g;
  size_t smem = 0;
  if (!t010_plan(buf, e, T, a, B, &g, &smem)) return cudaErrorInvalidValue;
  if (g.form_b) {
    switch (e) {
      case 1: return run_tile010<1, 16, true>(s, g, smem);
      case 2: return run_tile010<2, 16, true>(s, g, smem);
      case 4: return run_tile010<4, 16, true>(s, g, smem);
      default: return run_tile010<8, 16, true>(s, g, smem);
    }
  }
  switch (e * 100 + g.V) {
    case 116: return run_tile010<1, 16, false>(s, g, smem);
    case 108: return run_tile010<1, 8, false>(s, g, smem);
    case 104: return run_tile010<1, 4, false>(s, g, smem);
    case 216: return run_tile010<2, 16, false>(s, g, smem);
    case 208: return run_tile010<2, 8, false>(s, g, smem);
    case 204: return run_tile010<2, 4, false>(s, g, smem);
    case 416: return run_tile010<4, 16, false>(s, g, smem);
    case 408: return run_tile010<4, 8, false>(s, g, smem);
    case 816: return run_tile010<8, 16, false>(s, g, smem);
    default: return cudaErrorInvalidValue;
  }
}

}  // namespace lm
