// lm_bs.cu -- 0100 / 010 by barrier-synchronised tiling ("BS").
//
// Reference algorithm: BS_marshal / BS_marshal_vw (src/cl/cl_aos_asta.cl:53-161)
// stage one contiguous tile [a][B] in local memory and write it back as
// [B][a] after a barrier.  The reference caps a tile at 48 KB (MAX_MEM,
// src/cl_marshal.cc:45-59) and hands anything larger to PTTWAC.
//
// GB300 design:
//  * the op is generalised to 0100: tile [a][B][b] -> [B][a][b] with b-element
//    super-elements, so 010 is b == 1 and "010 with b-element units" (the first
//    pass of the two-pass 100 plan) is the same kernel;
//  * small tiles are batched: one CTA stages k consecutive tiles (one
//    contiguous range) so a launch-bound shape like 2048 tiles of 896 B uses
//    a few hundred CTAs, each streaming tens of KB;
//  * tiles up to 227 KB fit one CTA (opt-in shared memory);
//  * larger tiles are spread over a thread-block cluster of 2..16 CTAs: each
//    CTA stages a COLUMN band of every row and writes the output rows of that
//    band (one contiguous range) from its own shared memory; the cluster
//    barrier only orders all loads before all stores.  A 32 x 12289 fp32
//    tile (1.57 MB) fits an 8-CTA cluster; the reference would fall back to
//    PTTWAC;
//  * rows are padded in shared memory so the transposed read (stride = one
//    row) touches distinct banks; global loads and stores are coalesced;
//  * the grid is persistent (at most the co-resident CTAs / clusters).
#include <algorithm>
#include <cstdio>
#include <cstdlib>
#include <cooperative_groups.h>

#include "lm_core.cuh"
#include "lm_internal.h"

namespace cg = cooperative_groups;

namespace lm {

struct BsArgs {
  char *base;
  uint64_t T;
  uint64_t nchunks;
  uint32_t a, B, b;
  uint32_t row_elems;   // B*b
  uint32_t aB;          // units per tile
  uint32_t tile_elems;  // a*B*b
  uint32_t k;           // tiles per chunk
  uint32_t rpc;         // rows per CTA
  uint32_t pitch;       // shared-memory bytes per row
  FastDiv div_row, div_b, div_aB, div_a, div_rpc;
};

constexpr int kBsThreads = 512;
constexpr int kBsUnroll = 8;
constexpr uint32_t kBandMaxRows = 1024;  // rows of a tile in cluster form

// One CTA per chunk of k consecutive tiles (k >= 1), staged whole.
template <int E>
__global__ void __launch_bounds__(kBsThreads) k_bs0100(BsArgs g) {
  using T = typename Elem<E>::T;
  extern __shared__ __align__(128) unsigned char smem[];
  const uint32_t C = 1, rank = 0;
  const uint64_t cid = blockIdx.x, ncl = gridDim.x;

  for (uint64_t chunk = cid; chunk < g.nchunks; chunk += ncl) {
    const uint64_t t0 = chunk * g.k;
    const uint32_t nt = (uint32_t)min((uint64_t)g.k, g.T - t0);
    const uint32_t rows = nt * g.a;
    const uint64_t e0 = t0 * (uint64_t)g.tile_elems;
    const uint32_t r0 = rank * g.rpc;
    const uint32_t my_rows = r0 < rows ? min(g.rpc, rows - r0) : 0u;

    // ---- load: my band of rows (contiguous in global) -> padded smem rows
    {
      const T *src = reinterpret_cast<const T *>(g.base) + e0 +
                     (uint64_t)r0 * g.row_elems;
      const uint32_t n = my_rows * g.row_elems;
      for (uint32_t base = threadIdx.x; base < n;
           base += kBsThreads * kBsUnroll) {
        T v[kBsUnroll];
#pragma unroll
        for (int u = 0; u < kBsUnroll; ++u) {
          const uint32_t idx = base + u * kBsThreads;
          if (idx < n) v[u] = __ldcg(src + idx);
        }
#pragma unroll
        for (int u = 0; u < kBsUnroll; ++u) {
          const uint32_t idx = base + u * kBsThreads;
          if (idx < n) {
            const uint32_t row = fdiv(idx, g.div_row);
            const uint32_t col = idx - row * g.row_elems;
            *reinterpret_cast<T *>(smem + row * g.pitch + col * E) = v[u];
          }
        }
      }
    }
    __syncthreads();

    // ---- store: the chunk's outputs from the staged rows
    {
      const uint32_t nout = rows * g.row_elems;
      const uint32_t per = (nout + C - 1) / C;
      const uint32_t o0 = min(nout, rank * per);
      const uint32_t o1 = min(nout, o0 + per);
      T *dst = reinterpret_cast<T *>(g.base) + e0;
      for (uint32_t base = o0 + threadIdx.x; base < o1;
           base += kBsThreads * kBsUnroll) {
        T v[kBsUnroll];
#pragma unroll
        for (int u = 0; u < kBsUnroll; ++u) {
          const uint32_t o = base + u * kBsThreads;
          if (o < o1) {
            uint32_t unit = o, sub = 0;
            if (g.b != 1) {
              unit = fdiv(o, g.div_b);
              sub = o - unit * g.b;
            }
            const uint32_t t = fdiv(unit, g.div_aB);
            const uint32_t u2 = unit - t * g.aB;
            const uint32_t j = fdiv(u2, g.div_a);
            const uint32_t i = u2 - j * g.a;
            const uint32_t row = t * g.a + i;
            const uint32_t col = j * g.b + sub;
            v[u] = *reinterpret_cast<const T *>(smem + row * g.pitch + col * E);
          }
        }
#pragma unroll
        for (int u = 0; u < kBsUnroll; ++u) {
          const uint32_t o = base + u * kBsThreads;
          if (o < o1) __stcg(dst + o, v[u]);
        }
      }
    }
    __syncthreads();
  }
}

// Cluster form for tiles larger than one CTA's shared memory: CTA r of the
// cluster stages COLUMN band r (units [r*band, (r+1)*band) of every row of the
// tile), so the output rows of its band -- one contiguous output range -- are
// produced from its own shared memory.  The cluster barrier only separates
// every CTA's loads from every CTA's stores (the output range of one band
// overlaps input rows staged by the others); no shared memory is read across
// CTAs.
template <int E>
__global__ void __launch_bounds__(kBsThreads) k_bs0100_band(BsArgs g) {
  using T = typename Elem<E>::T;
  extern __shared__ __align__(128) unsigned char smem[];
  __shared__ __align__(8) uint64_t bar;
  __shared__ uint32_t rowoff[kBandMaxRows];
  __shared__ int s_ok;
  cg::cluster_group cl = cg::this_cluster();
  const uint32_t C = cl.num_blocks();
  const uint32_t rank = cl.block_rank();
  const uint64_t cid = blockIdx.x / C, ncl = gridDim.x / C;
  const uint32_t bc0 = min(g.B, rank * g.rpc);  // rpc = units per band
  const uint32_t bc1 = min(g.B, bc0 + g.rpc);
  const uint32_t nbu = bc1 - bc0;               // units in my band
  const uint32_t band_elems = nbu * g.b;
  const uint32_t len = band_elems * E;          // bytes per row segment
  const uint32_t warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  constexpr uint32_t nw = kBsThreads / 32;
  if (threadIdx.x == 0) {
    mbar_init(&bar, nw);  // one arrival per warp
    fence_mbar_init();
    s_ok = 1;
  }
  __syncthreads();
  uint32_t parity = 0;
  for (uint64_t tile = cid; tile < g.T; tile += ncl) {
    const uint64_t e0 = tile * (uint64_t)g.tile_elems;
    T *t = reinterpret_cast<T *>(g.base) + e0;
    // ---- load: one bulk copy per row (16-byte aligned superset of the band
    // segment; rowoff[] records where the segment starts in shared memory),
    // spread over the warps (a warp issues its lanes' copies one after
    // another): row r by lane (r / nw) % 32 of warp r % nw.  Each warp
    // arrives with its bytes; a CTA barrier; then the copies.
    if (len > 0) {
      uint32_t bytes = 0;
      for (uint32_t r = warp + nw * lane; r < g.a; r += nw * 32) {
        const char *src = reinterpret_cast<const char *>(
            t + (uint64_t)r * g.row_elems + (uint64_t)bc0 * g.b);
        const uintptr_t a0 = (uintptr_t)src & ~(uintptr_t)15;
        const uintptr_t a1 = ((uintptr_t)src + len + 15) & ~(uintptr_t)15;
        bytes += (uint32_t)(a1 - a0);
        rowoff[r] = r * g.pitch + (uint32_t)((uintptr_t)src - a0);
      }
#pragma unroll
      for (int o = 16; o > 0; o >>= 1) bytes += __shfl_xor_sync(kFull, bytes, o);
      if (lane == 0) mbar_arrive_expect_tx(&bar, bytes);
      __syncthreads();  // every warp's expected bytes before any copy
      fence_proxy_async_smem();
      for (uint32_t r = warp + nw * lane; r < g.a; r += nw * 32) {
        const char *src = reinterpret_cast<const char *>(
            t + (uint64_t)r * g.row_elems + (uint64_t)bc0 * g.b);
        const uintptr_t a0 = (uintptr_t)src & ~(uintptr_t)15;
        const uintptr_t a1 = ((uintptr_t)src + len + 15) & ~(uintptr_t)15;
        bulk_g2s(smem + (size_t)r * g.pitch, (const void *)a0,
                 (uint32_t)(a1 - a0), &bar);
      }
    }
    if (len > 0) {
      const uint64_t t0 = global_timer_ns();
      while (!mbar_try_wait(&bar, parity)) {
        if (global_timer_ns() - t0 > 2000000000ull) {  // cannot happen: bounded anyway
          s_ok = 0;
          break;
        }
      }
      parity ^= 1;
    }
    cl.sync();  // every band staged before any output is written
    // ---- store: output rows bc0..bc1-1 = elements [bc0*a*b, bc1*a*b)
    const uint32_t n = g.a * band_elems;
    T *dst = t + (uint64_t)bc0 * g.a * g.b;
    if (s_ok && E <= 4 && g.b == 1 && (g.a * E) % 16 == 0 &&
        ((uintptr_t)dst & 15) == 0) {
      // whole-vector output rows: 16-byte stores
      store_columns16<E>(smem, rowoff, g.a, nbu,
                         reinterpret_cast<unsigned char *>(dst), threadIdx.x,
                         kBsThreads);
    } else if (s_ok) {
      for (uint32_t base = threadIdx.x; base < n;
           base += kBsThreads * kBsUnroll) {
        T v[kBsUnroll];
#pragma unroll
        for (int u = 0; u < kBsUnroll; ++u) {
          const uint32_t o = base + u * kBsThreads;
          if (o < n) {
            uint32_t unit = o, sub = 0;
            if (g.b != 1) {
              unit = fdiv(o, g.div_b);
              sub = o - unit * g.b;
            }
            const uint32_t j = fdiv(unit, g.div_a);  // output row in band
            const uint32_t i = unit - j * g.a;
            v[u] = *reinterpret_cast<const T *>(smem + rowoff[i] +
                                                (j * g.b + sub) * E);
          }
        }
#pragma unroll
        for (int u = 0; u < kBsUnroll; ++u) {
          const uint32_t o = base + u * kBsThreads;
          if (o < n) __stcg(dst + o, v[u]);
        }
      }
    }
    __syncthreads();  // my shared band is free for the next tile
  }
}

// --- host side ---------------------------------------------------------------

static uint32_t bs_pitch(uint64_t row_bytes, int e) {
  const uint64_t g = e == 8 ? 8 : 4;
  uint64_t p = (row_bytes + g - 1) / g * g;
  if (((p / g) & 1) == 0) p += g;  // odd word stride: conflict-free columns
  return (uint32_t)p;
}

BsPlan plan_bs0100(uint64_t T, uint32_t a, uint32_t B, uint32_t b, int e,
                   size_t smem_budget) {
  BsPlan p;
  if (e != 1 && e != 2 && e != 4 && e != 8) return p;
  if (T == 0 || a == 0 || B == 0 || b == 0) return p;
  const uint64_t row_elems = (uint64_t)B * b;
  const uint64_t tile_elems = row_elems * a;
  if (tile_elems >= 0xffffffffull) return p;
  const DeviceInfo &di = device_info();
  // leave room for the kernels' static shared memory (the cluster form keeps
  // a row-offset table of kBandMaxRows words)
  const size_t max_smem = (smem_budget ? smem_budget
                                       : (size_t)di.max_smem_optin) -
                          (kBandMaxRows * 4 + 512);
  const uint64_t pitch = bs_pitch(row_elems * e, e);
  const uint64_t tile_smem = pitch * a;
  const uint64_t target = 40 * 1024;  // a few CTAs per SM overlap load/store
  if (tile_smem <= target) {
    uint64_t k = std::max<uint64_t>(1, target / tile_smem);
    k = std::min<uint64_t>(k, T);
    while (k > 1 && k * tile_elems >= 0xffffffffull) k--;
    p.tiles_per_chunk = (uint32_t)k;
    p.cluster = 1;
    p.rows_per_cta = (uint32_t)(k * a);
  } else if (tile_smem <= max_smem &&
             !(b == 1 && e <= 4 && tile_smem > 112 * 1024 &&
               a <= kBandMaxRows)) {
    // (one-element units of narrow types in tiles above 112 KB go to the
    // cluster form, whose bands write 16-byte vectors)
    p.tiles_per_chunk = 1;
    p.cluster = 1;
    p.rows_per_cta = a;
  } else {
    // cluster of C CTAs, each staging a column band of ceil(B/C) units
    p.tiles_per_chunk = 1;
    for (int C = 2; C <= 16; C *= 2) {
      if ((uint64_t)C > B) break;
      const uint64_t band = (B + C - 1) / C;
      // bulk-copy destination rows: 16-byte aligned, room for the aligned
      // superset (up to 30 extra bytes), an odd number of 16-byte words
      uint64_t bp = (band * b * e + 15) / 16 * 16 + 32;
      if (((bp / 16) & 1) == 0) bp += 16;
      if (a > kBandMaxRows) break;
      if (bp * a <= max_smem) {
        p.cluster = C;
        p.rows_per_cta = (uint32_t)band;  // units per band in cluster form
        p.pitch = (uint32_t)bp;
        p.smem_bytes = (size_t)(bp * a);
        p.threads = kBsThreads;
        p.feasible = true;
        return p;
      }
    }
    return p;
  }
  p.pitch = (uint32_t)pitch;
  p.smem_bytes = (size_t)p.rows_per_cta * pitch;
  p.threads = kBsThreads;
  p.feasible = true;
  return p;
}

template <int E, bool CLUSTER>
static cudaError_t run_bs(cudaStream_t s, const BsArgs &g, const BsPlan &p) {
  auto kern = CLUSTER ? k_bs0100_band<E> : k_bs0100<E>;
  const DeviceInfo &di = device_info();
  cudaError_t err = cudaSuccess;
  if (!CLUSTER) {
    static LaunchCache cache;
    const int occ = prepare_launch((const void *)kern, cache, p.smem_bytes,
                                   kBsThreads, &err);
    if (err != cudaSuccess) return err;
    uint64_t blocks = (uint64_t)di.sms * std::max(occ, 1);
    if (g.nchunks < blocks) blocks = g.nchunks;
    if (getenv("LM_VERBOSE"))
      fprintf(stderr, "bs_tile: k=%u smem=%zu occ=%d blocks=%llu chunks=%llu\n",
              p.tiles_per_chunk, p.smem_bytes, occ,
              (unsigned long long)blocks, (unsigned long long)g.nchunks);
    ProfScope ps(s, "bs_tile");
    kern<<<(unsigned)blocks, kBsThreads, p.smem_bytes, s>>>(g);
    return cudaGetLastError();
  }
  err = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize,
                             (int)p.smem_bytes);
  if (err != cudaSuccess) return err;
  if (p.cluster > 8) {
    err = cudaFuncSetAttribute(kern,
                               cudaFuncAttributeNonPortableClusterSizeAllowed, 1);
    if (err != cudaSuccess) return err;
  }
  cudaLaunchConfig_t cfg = {};
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributeClusterDimension;
  attr[0].val.clusterDim.x = p.cluster;
  attr[0].val.clusterDim.y = 1;
  attr[0].val.clusterDim.z = 1;
  cfg.blockDim = dim3(kBsThreads);
  cfg.dynamicSmemBytes = p.smem_bytes;
  cfg.stream = s;
  cfg.attrs = attr;
  cfg.numAttrs = 1;
  int max_clusters = 0;
  cfg.gridDim = dim3((unsigned)(p.cluster * std::max(1, di.sms / p.cluster)));
  err = cudaOccupancyMaxActiveClusters(&max_clusters, kern, &cfg);
  if (err != cudaSuccess) return err;
  if (max_clusters < 1) return cudaErrorInvalidConfiguration;
  uint64_t ncl = (uint64_t)max_clusters;
  if (g.nchunks < ncl) ncl = g.nchunks;
  cfg.gridDim = dim3((unsigned)(ncl * p.cluster));
  if (getenv("LM_VERBOSE"))
    fprintf(stderr, "bs_cluster: C=%d smem=%zu band=%u pitch=%u tiles=%llu "
            "max_clusters=%d grid=%u\n", p.cluster, p.smem_bytes,
            p.rows_per_cta, p.pitch, (unsigned long long)g.nchunks,
            max_clusters, cfg.gridDim.x);
  ProfScope ps(s, "bs_cluster");
  err = cudaLaunchKernelEx(&cfg, kern, g);
  if (err != cudaSuccess) return err;
  return cudaGetLastError();
}

cudaError_t launch_bs0100(cudaStream_t s, void *buf, int e, uint64_t T,
                          uint32_t a, uint32_t B, uint32_t b,
                          const BsPlan &p) {
  if (!p.feasible) return cudaErrorInvalidValue;
  if (T == 0 || a <= 1 || B <= 1) return cudaSuccess;  // empty or identity
  // single-element units in small tiles: the 16-byte form (lm_tile010.cu)
  if (b == 1 && p.cluster == 1 && tile010_applies(buf, e, T, a, B) &&
      !getenv("LM_NO_TILE010"))
    return launch_tile010(s, buf, e, T, a, B);
  BsArgs g;
  g.base = reinterpret_cast<char *>(buf);
  g.T = T;
  g.k = p.tiles_per_chunk;
  g.nchunks = (T + g.k - 1) / g.k;
  g.a = a;
  g.B = B;
  g.b = b;
  g.row_elems = B * b;
  g.aB = a * B;
  g.tile_elems = a * B * b;
  g.rpc = p.rows_per_cta;
  g.pitch = p.pitch;
  g.div_row = make_fastdiv(g.row_elems);
  g.div_b = make_fastdiv(b);
  g.div_aB = make_fastdiv(g.aB);
  g.div_a = make_fastdiv(a);
  g.div_rpc = make_fastdiv(g.rpc);
  const bool cl = p.cluster > 1;
  switch (e) {
    case 1: return cl ? run_bs<1, true>(s, g, p) : run_bs<1, false>(s, g, p);
    case 2: return cl ? run_bs<2, true>(s, g, p) : run_bs<2, false>(s, g, p);
    case 4: return cl ? run_bs<4, true>(s, g, p) : run_bs<4, false>(s, g, p);
    case 8: return cl ? run_bs<8, true>(s, g, p) : run_bs<8, false>(s, g, p);
    default: return cudaErrorInvalidValue;
  }
}

}  // namespace lm
