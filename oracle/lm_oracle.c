/*
 * lm_oracle.c -- CPU oracle (test infrastructure; see lm_oracle.h).
 *
 * Each function restates one reference algorithm in plain C and names the
 * reference file:line it follows.  Nothing here is used by the product.
 */
#include "lm_oracle.h"

#include <math.h>
#include <pthread.h>
#include <stdlib.h>
#include <string.h>

/* ---- element-width dispatch ------------------------------------------- */

#define LMO_DISPATCH(e, FN, ...)                                              \
  do {                                                                        \
    switch (e) {                                                              \
      case 1: FN##_t(uint8_t, __VA_ARGS__); break;                            \
      case 2: FN##_t(uint16_t, __VA_ARGS__); break;                           \
      case 4: FN##_t(uint32_t, __VA_ARGS__); break;                           \
      case 8: FN##_t(uint64_t, __VA_ARGS__); break;                           \
      default: return -1;                                                     \
    }                                                                         \
  } while (0)

/* cpu_aos_asta (test/cl_unittest.cc:138-151): for every tile i, for j < t,
 * for k < w: dst_tile[j + k*t] = src_tile[j*w + k].  Rows [k0, k1) of the
 * tile loop are done (k0/k1 index tiles) so threads can split it. */
#define AOS_ASTA_t(T, src, dst, height, width, tile, i0, i1)                  \
  {                                                                           \
    const T *s_ = (const T *)(src);                                           \
    T *d_ = (T *)(dst);                                                       \
    for (int64_t i = (i0); i < (i1); i++) {                                   \
      const T *ss = s_ + i * (tile) * (width);                                \
      T *dd = d_ + i * (tile) * (width);                                      \
      for (int64_t j = 0; j < (tile); j++)                                    \
        for (int64_t k = 0; k < (width); k++)                                 \
          dd[j + k * (tile)] = ss[j * (width) + k];                           \
    }                                                                         \
  }

/* cpu_soa_asta (test/cl_unittest.cc:153-166): for k < w, for i < h/t,
 * for j < t: dst[i*w*t + k*t + j] = src[k*h + i*t + j].  Outer k in [k0,k1). */
#define SOA_ASTA_t(T, src, dst, height, width, tile, k0, k1)                  \
  {                                                                           \
    const T *s_ = (const T *)(src);                                           \
    T *d_ = (T *)(dst);                                                       \
    const int64_t nt_ = (height) / (tile);                                    \
    for (int64_t k = (k0); k < (k1); k++)                                     \
      for (int64_t i = 0; i < nt_; i++)                                       \
        for (int64_t j = 0; j < (tile); j++)                                  \
          d_[i * (width) * (tile) + k * (tile) + j] =                         \
              s_[k * (height) + i * (tile) + j];                              \
  }

int lmo_aos_asta(const void *src, void *dst, int64_t height, int64_t width,
                 int64_t tile, int e) {
  if (tile <= 0 || width < 0 || height < 0 || (height / tile) * tile != height)
    return -1;
  LMO_DISPATCH(e, AOS_ASTA, src, dst, height, width, tile, 0, height / tile);
  return 0;
}

int lmo_soa_asta(const void *src, void *dst, int64_t height, int64_t width,
                 int64_t tile, int e) {
  if (tile <= 0 || width < 0 || height < 0 || (height / tile) * tile != height)
    return -1;
  LMO_DISPATCH(e, SOA_ASTA, src, dst, height, width, tile, 0, width);
  return 0;
}

/* ---- threaded variants (CPU baseline only) ----------------------------- */

typedef struct {
  const void *src;
  void *dst;
  int64_t height, width, tile, lo, hi;
  int e, soa;
} lmo_job;

static int lmo_run_job(lmo_job *jb) {
  if (jb->soa) {
    LMO_DISPATCH(jb->e, SOA_ASTA, jb->src, jb->dst, jb->height, jb->width,
                 jb->tile, jb->lo, jb->hi);
  } else {
    LMO_DISPATCH(jb->e, AOS_ASTA, jb->src, jb->dst, jb->height, jb->width,
                 jb->tile, jb->lo, jb->hi);
  }
  return 0;
}

static void *lmo_thread_main(void *p) {
  lmo_run_job((lmo_job *)p);
  return NULL;
}

static int lmo_split(const void *src, void *dst, int64_t height, int64_t width,
                     int64_t tile, int e, int nthreads, int soa) {
  if (tile <= 0 || (height / tile) * tile != height) return -1;
  if (e != 1 && e != 2 && e != 4 && e != 8) return -1;
  if (nthreads < 1) nthreads = 1;
  if (nthreads > 256) nthreads = 256;
  int64_t total = soa ? width : height / tile;
  pthread_t th[256];
  lmo_job jobs[256];
  int started = 0;
  for (int t = 0; t < nthreads; t++) {
    jobs[t].src = src;
    jobs[t].dst = dst;
    jobs[t].height = height;
    jobs[t].width = width;
    jobs[t].tile = tile;
    jobs[t].e = e;
    jobs[t].soa = soa;
    jobs[t].lo = total * t / nthreads;
    jobs[t].hi = total * (t + 1) / nthreads;
  }
  for (int t = 1; t < nthreads; t++) {
    if (pthread_create(&th[t], NULL, lmo_thread_main, &jobs[t]) != 0) break;
    started = t;
  }
  lmo_run_job(&jobs[0]);
  for (int t = 1; t <= started; t++) pthread_join(th[t], NULL);
  for (int t = started + 1; t < nthreads; t++) lmo_run_job(&jobs[t]);
  return 0;
}

int lmo_soa_asta_mt(const void *src, void *dst, int64_t height, int64_t width,
                    int64_t tile, int e, int nthreads) {
  return lmo_split(src, dst, height, width, tile, e, nthreads, 1);
}

int lmo_aos_asta_mt(const void *src, void *dst, int64_t height, int64_t width,
                    int64_t tile, int e, int nthreads) {
  return lmo_split(src, dst, height, width, tile, e, nthreads, 0);
}

/* ---- elementary transpositions via the CPU layouts --------------------- */

int lmo_010(const void *src, void *dst, int64_t A, int64_t a, int64_t B,
            int e) {
  return lmo_aos_asta(src, dst, A * a, B, a, e);
}

int lmo_100(const void *src, void *dst, int64_t A, int64_t B, int64_t b,
            int e) {
  return lmo_soa_asta(src, dst, B * b, A, b, e);
}

int lmo_0100(const void *src, void *dst, int64_t A, int64_t a, int64_t B,
             int64_t b, int e) {
  const int64_t slice = a * B * b * (int64_t)e;
  for (int64_t i = 0; i < A; i++) {
    int r = lmo_soa_asta((const char *)src + i * slice, (char *)dst + i * slice,
                         B * b, a, b, e);
    if (r) return r;
  }
  return 0;
}

int lmo_transpose(const void *src, void *dst, int64_t M, int64_t N, int e) {
  /* cpu_aos_asta(src, tmp, M, N, 1) is the identity copy; then
   * cpu_soa_asta(tmp, dst, height=N, width=M, tile=1). */
  size_t bytes = (size_t)(M * N * e);
  void *tmp = malloc(bytes ? bytes : 1);
  if (!tmp) return -1;
  int r = lmo_aos_asta(src, tmp, M, N, 1, e);
  if (!r) r = lmo_soa_asta(tmp, dst, N, M, 1, e);
  free(tmp);
  return r;
}

/* ---- in-place cycle follower (plan.hpp:54-56 successor) ---------------- */

int64_t lmo_inplace_100(void *buf, int64_t A, int64_t B, int64_t b, int e) {
  if (A <= 0 || B <= 0 || b <= 0) return -1;
  if (e != 1 && e != 2 && e != 4 && e != 8) return -1;
  const int64_t n = A * B;
  const int64_t m = n - 1;
  const size_t unit = (size_t)(b * e);
  if (n <= 1) return 0;
  uint8_t *seen = (uint8_t *)calloc((size_t)((n + 7) / 8), 1);
  uint8_t *carry = (uint8_t *)malloc(unit);
  uint8_t *save = (uint8_t *)malloc(unit);
  if (!seen || !carry || !save) {
    free(seen); free(carry); free(save);
    return -1;
  }
  uint8_t *base = (uint8_t *)buf;
  int64_t cycles = 0;
  /* Position p of [A][B] goes to (p % B) * A + p / B, i.e. Next(p) with
   * m = A, n = B; 0 and A*B-1 are fixed. */
  for (int64_t p = 1; p < m; p++) {
    if (seen[p >> 3] & (1u << (p & 7))) continue;
    int64_t q = (p % B) * A + p / B;
    if (q == p) {
      seen[p >> 3] |= (uint8_t)(1u << (p & 7));
      continue;
    }
    cycles++;
    memcpy(carry, base + p * unit, unit);
    int64_t cur = p;
    do {
      int64_t nx = (cur % B) * A + cur / B;
      memcpy(save, base + nx * unit, unit);
      memcpy(base + nx * unit, carry, unit);
      memcpy(carry, save, unit);
      seen[nx >> 3] |= (uint8_t)(1u << (nx & 7));
      cur = nx;
    } while (cur != p);
  }
  free(seen); free(carry); free(save);
  return cycles;
}

/* ---- padding / unpadding semantics (cl_aos_asta.cl:813-938) ------------ */

#define PAD_t(T, buf, x, y, pad)                                              \
  {                                                                           \
    T *b_ = (T *)(buf);                                                       \
    for (int64_t r = (y)-1; r >= 0; r--)                                      \
      for (int64_t c = (pad)-1; c >= 0; c--)                                  \
        b_[r * (pad) + c] = c < (x) ? b_[r * (x) + c] : (T)0;                 \
  }

#define UNPAD_t(T, buf, x, y, pad)                                            \
  {                                                                           \
    T *b_ = (T *)(buf);                                                       \
    for (int64_t r = 0; r < (y); r++)                                         \
      for (int64_t c = 0; c < (x); c++) b_[r * (x) + c] = b_[r * (pad) + c];  \
    for (int64_t i = (y) * (x); i < (y) * (pad); i++) b_[i] = (T)0;           \
  }

int lmo_padding(void *buf, int64_t x, int64_t y, int64_t pad, int e) {
  if (x < 0 || y < 0 || pad < x) return -1;
  /* Walking rows and columns from the back never reads an element that
   * was already overwritten, because r*x + c <= r*pad + c. */
  LMO_DISPATCH(e, PAD, buf, x, y, pad);
  return 0;
}

int lmo_unpadding(void *buf, int64_t x, int64_t y, int64_t pad, int e) {
  if (x < 0 || y < 0 || pad < x) return -1;
  LMO_DISPATCH(e, UNPAD, buf, x, y, pad);
  return 0;
}

/* ---- planner model (include/plan.hpp) ---------------------------------- */

uint32_t lmo_next(uint32_t i, int m, int n) {
  /* plan.hpp:54-56: (i*m) - mn_*(i/n) with unsigned wrap-around. */
  uint32_t mn = (uint32_t)m * (uint32_t)n - 1u;
  return i * (uint32_t)m - mn * (i / (uint32_t)n);
}

int64_t lmo_num_cycles(int m, int n) {
  /* plan.hpp:57-73: i from 1 to mn_ inclusive; a cycle is counted at its
   * smallest member. */
  int mn = m * n - 1;
  int64_t nontrivial = 0;
  for (int i = 1; i <= mn; i++) {
    int j = (int)lmo_next((uint32_t)i, m, n);
    if (j == i) continue;
    for (; j > i; j = (int)lmo_next((uint32_t)j, m, n)) {
    }
    if (j != i) continue;
    nontrivial++;
  }
  return nontrivial;
}

int64_t lmo_num_cycles_fast(int64_t m, int64_t n) {
  const int64_t total = m * n;
  if (total <= 2) return 0;
  uint8_t *seen = (uint8_t *)calloc((size_t)((total + 7) / 8), 1);
  if (!seen) return -1;
  int64_t cycles = 0;
  for (int64_t i = 1; i < total - 1; i++) {
    if (seen[i >> 3] & (1u << (i & 7))) continue;
    int64_t j = (i % n) * m + i / n;
    if (j == i) continue;
    cycles++;
    int64_t cur = i;
    do {
      seen[cur >> 3] |= (uint8_t)(1u << (cur & 7));
      cur = (cur % n) * m + cur / n;
    } while (cur != i);
  }
  free(seen);
  return cycles;
}

int lmo_factorize(int n, int *primes, int *exps, int cap) {
  /* plan.hpp:166-185: trial division by 2 then odd d while d < n; the
   * final quotient is recorded as the last prime factor. */
  int count = 0;
  if (n < 2) return 0;
  int d = 2;
  int P[64], E[64];
  int np = 0;
#define LMO_ADD(p)                                                            \
  do {                                                                        \
    int k_;                                                                   \
    for (k_ = 0; k_ < np && P[k_] != (p); k_++) {                             \
    }                                                                         \
    if (k_ == np) { P[np] = (p); E[np] = 0; np++; }                           \
    E[k_]++;                                                                  \
  } while (0)
  while (d < n) {
    if (n % d == 0) {
      LMO_ADD(d);
      n /= d;
    } else {
      d = (d == 2) ? 3 : d + 2;
    }
  }
  LMO_ADD(d);
#undef LMO_ADD
  /* std::map keeps primes ascending. */
  for (int a = 0; a < np; a++)
    for (int b = a + 1; b < np; b++)
      if (P[b] < P[a]) {
        int t = P[a]; P[a] = P[b]; P[b] = t;
        t = E[a]; E[a] = E[b]; E[b] = t;
      }
  for (int a = 0; a < np && count < cap; a++) {
    primes[count] = P[a];
    exps[count] = E[a];
    count++;
  }
  return np;
}

static void lmo_tile_rec(const int *P, const int *E, int np, int idx, int t,
                         int *out, int cap, int *count) {
  if (idx == np) {
    if (t > 1) {
      if (*count < cap) out[*count] = t;
      (*count)++;
    }
    return;
  }
  for (int i = 0; i <= E[idx]; i++) {
    if (i) t *= P[idx];
    lmo_tile_rec(P, E, np, idx + 1, t, out, cap, count);
  }
}

int lmo_tile_options(int n, int *out, int cap) {
  int P[64], E[64];
  int np = lmo_factorize(n, P, E, 64);
  int count = 0;
  lmo_tile_rec(P, E, np, 0, 1, out, cap, &count);
  return count;
}

static int lmo_pick(int n, int lo, int hi, int *found) {
  /* Largest tiling option in [lo, hi]; the reference sorts the options
   * ascending (gsl_sort_int_index) and scans from the top. */
  int opts[4096];
  int cnt = lmo_tile_options(n, opts, 4096);
  if (cnt > 4096) cnt = 4096;
  int best = -1;
  for (int i = 0; i < cnt; i++)
    if (opts[i] >= lo && opts[i] <= hi && opts[i] > best) best = opts[i];
  *found = best > 0;
  return best;
}

int lmo_alg5(int h, int w, int max_mem, int *out6) {
  const int min_limit = 24;
  const int max_limit = (int)sqrt((double)max_mem);
  int pad_h = 0, pad_w = 0;
  int done_h = 0, done_w = 0;
  int aa = max_mem, bb = max_mem;
  int guard = 0;
  do {
    int f;
    if (!done_h) {
      int v = lmo_pick(h, min_limit, max_limit, &f);
      if (f) { aa = v; done_h = 1; }
    }
    if (!done_w) {
      int v = lmo_pick(w, min_limit, max_limit, &f);
      if (f) { bb = v; done_w = 1; }
    }
    if (!done_h) { pad_h++; h++; }
    if (!done_w) { pad_w++; w++; }
    if (++guard > 1000000) return -1;
  } while (!done_h || !done_w);
  out6[0] = h / aa;
  out6[1] = aa;
  out6[2] = w / bb;
  out6[3] = bb;
  out6[4] = pad_h;
  out6[5] = pad_w;
  return 0;
}

int lmo_alg3(int A, int a, int B, int b, int max_mem) {
  if (a >= 6 && (int64_t)a * B * b <= max_mem) return 2;
  if (b >= 6 && (int64_t)b * A * a <= max_mem) return 22;
  return a <= b ? 3 : 32;
}

/* ---- seeded inputs ----------------------------------------------------- */

void lmo_fill_splitmix64(void *buf, int64_t nbytes, uint64_t seed) {
  uint8_t *p = (uint8_t *)buf;
  uint64_t x = seed;
  int64_t i = 0;
  for (; i + 8 <= nbytes; i += 8) {
    x += 0x9E3779B97F4A7C15ull;
    uint64_t z = x;
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    z ^= z >> 31;
    memcpy(p + i, &z, 8); /* little-endian on both build hosts */
  }
  if (i < nbytes) {
    x += 0x9E3779B97F4A7C15ull;
    uint64_t z = x;
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    z ^= z >> 31;
    memcpy(p + i, &z, (size_t)(nbytes - i));
  }
}

void lmo_fill_index(void *buf, int64_t n, int e) {
  for (int64_t i = 0; i < n; i++) {
    switch (e) {
      case 1: ((uint8_t *)buf)[i] = (uint8_t)i; break;
      case 2: ((uint16_t *)buf)[i] = (uint16_t)i; break;
      case 4: ((uint32_t *)buf)[i] = (uint32_t)i; break;
      case 8: ((uint64_t *)buf)[i] = (uint64_t)i; break;
      default: return;
    }
  }
}
