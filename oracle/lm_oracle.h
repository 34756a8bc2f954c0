/*
 * lm_oracle.h -- CPU oracle for the in-place layout conversions.
 *
 * TEST INFRASTRUCTURE ONLY.  This library is the checker: tests, the smoke
 * check and bench.py's CPU-baseline leg may load it; the product library
 * (libmarshal_gb300) never does.  Every function restates an algorithm of the
 * reference (libmarshal) and cites the file:line it follows.  Elements are
 * moved as raw bytes of width e in {1,2,4,8}; data is never interpreted.
 *
 * Parity is pinned two ways (see tests/test_oracle.py):
 *   - against golden vectors produced by the reference's own CPU code
 *     (test/cl_unittest.cc:138-166, include/plan.hpp:48-219) compiled from
 *     the reference sources by oracle/build_ref.sh, committed under
 *     tests/golden/;
 *   - against the known answers in the reference's tests
 *     (test/cl_unittest.cc:705-709).
 */
#ifndef LM_ORACLE_H_
#define LM_ORACLE_H_
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* cpu_aos_asta, test/cl_unittest.cc:138-151:
 * src[h/t][t][w] -> dst[h/t][w][t]; out-of-place. Returns 0, or -1 if t does
 * not divide h (the reference asserts). */
int lmo_aos_asta(const void *src, void *dst, int64_t height, int64_t width,
                 int64_t tile, int e);
/* cpu_soa_asta, test/cl_unittest.cc:152-166:
 * src[w][h/t][t] -> dst[h/t][w][t]; out-of-place, same loop order. */
int lmo_soa_asta(const void *src, void *dst, int64_t height, int64_t width,
                 int64_t tile, int e);
/* Same as lmo_soa_asta but the outer `width` loop is split over nthreads
 * POSIX threads (used only for the timed CPU baseline). */
int lmo_soa_asta_mt(const void *src, void *dst, int64_t height, int64_t width,
                    int64_t tile, int e, int nthreads);
int lmo_aos_asta_mt(const void *src, void *dst, int64_t height, int64_t width,
                    int64_t tile, int e, int nthreads);

/* Elementary transpositions expressed through the CPU layouts exactly as the
 * reference's tests check them:
 *   010  [A][a][B] -> [A][B][a]   == cpu_aos_asta(h=A*a, w=B, t=a)
 *        (cl_unittest.cc:265,272; cl_marshal.cc:793-799)
 *   100  [A][B][b] -> [B][A][b]   == cpu_soa_asta(h=B*b, w=A, t=b)
 *        (cl_unittest.cc:200,207)
 *   0100 [A][a][B][b] -> [A][B][a][b] == A slices of cpu_soa_asta(h=B*b,w=a,t=b)
 *        (cl_unittest.cc:689-696) */
int lmo_010(const void *src, void *dst, int64_t A, int64_t a, int64_t B, int e);
int lmo_100(const void *src, void *dst, int64_t A, int64_t B, int64_t b, int e);
int lmo_0100(const void *src, void *dst, int64_t A, int64_t a, int64_t B,
             int64_t b, int e);
/* Full M x N transpose golden: cpu_aos_asta(t=1) then cpu_soa_asta(w<->h,t=1)
 * (cl_unittest.cc:549-552). */
int lmo_transpose(const void *src, void *dst, int64_t M, int64_t N, int e);

/* In-place sequential cycle follower for 100 on super-elements of b*e bytes,
 * using the successor Transposition::Next (include/plan.hpp:54-56).  A second,
 * independent in-place restatement; returns the number of non-trivial cycles
 * it moved, or -1 on bad arguments / allocation failure. */
int64_t lmo_inplace_100(void *buf, int64_t A, int64_t B, int64_t b, int e);

/* Row padding / unpadding semantics of the reference's `padding` and
 * `unpadding` kernels (src/cl/cl_aos_asta.cl:813-938) on a buffer that holds
 * y*pad elements:
 *   padding:   [y][x] -> [y][pad], new columns x..pad-1 are zero;
 *   unpadding: [y][pad] -> [y][x], elements y*x .. y*pad-1 become zero. */
int lmo_padding(void *buf, int64_t x, int64_t y, int64_t pad, int e);
int lmo_unpadding(void *buf, int64_t x, int64_t y, int64_t pad, int e);

/* Transposition::Next (plan.hpp:54-56) with its 32-bit unsigned wrap-around. */
uint32_t lmo_next(uint32_t i, int m, int n);
/* Transposition::GetNumCycles (plan.hpp:57-73), literal algorithm. */
int64_t lmo_num_cycles(int m, int n);
/* Same count with a visited bitmap (linear time); used for large shapes. */
int64_t lmo_num_cycles_fast(int64_t m, int64_t n);

/* Factorize(n).get_factors() (plan.hpp:166-185): writes (prime, exponent)
 * pairs in ascending prime order; returns the number of pairs. */
int lmo_factorize(int n, int *primes, int *exps, int cap);
/* Factorize::tiling_options order (plan.hpp:189-214): all divisors > 1 in the
 * reference's enumeration order; returns the count. */
int lmo_tile_options(int n, int *out, int cap);

/* "Algorithm 5" super-element choice of the reference's full test
 * (test/cl_unittest.cc:396-467) for the single-precision NVIDIA build:
 * out = {A, a, B, b, pad_h, pad_w}.  max_mem is MAX_MEM in elements
 * (12288 there), min_limit 24, max_limit (int)sqrt(max_mem). */
int lmo_alg5(int h, int w, int max_mem, int *out6);
/* "Algorithm 3" stage choice (test/cl_unittest.cc:515-640): 2, 22, 3 or 32. */
int lmo_alg3(int A, int a, int B, int b, int max_mem);

/* splitmix64 byte generator used for seeded inputs in tests. */
void lmo_fill_splitmix64(void *buf, int64_t nbytes, uint64_t seed);
/* Linear-index fill mod 2^(8e) (the reference's "detectable misplacement"
 * pattern for 7200x1800). */
void lmo_fill_index(void *buf, int64_t n, int e);

#ifdef __cplusplus
}
#endif
#endif
