/*
 * lm_marshal.h -- C ABI of libmarshal_gb300 (liblmarshal.so).
 *
 * One entry per function of the reference's OpenCL interface
 * (include/cl_marshal.h:25-50 of libmarshal, implemented in
 * src/cl_marshal.cc) with (cl_command_queue queue, cl_mem src) replaced by
 * (lm_stream_t stream, void *buf, int elem_bytes):
 *   - stream: a cudaStream_t (lm_stream_t is the same type); NULL is the
 *     legacy default stream;
 *   - buf: device pointer to the array, converted IN PLACE;
 *   - elem_bytes: 1, 2, 4 or 8 (the reference fixes float or double at build
 *     time, src/cl_marshal.cc:34-43); elements are moved as raw bits.
 * The remaining arguments keep the reference's order and meaning.
 *
 * Conventions (as the reference, API.wiki:12,20):
 *   - return false on success, true on error; lm_last_error() returns the
 *     message of the calling thread's last error;
 *   - calls are stream ordered and asynchronous, EXCEPT: when the
 *     elapsed-time pointer `et` is non-NULL the call waits for its own work
 *     and adds its GPU time in nanoseconds to *et (the reference's
 *     Profiling::Report, include/cl_profile.h:23-25), and padding/unpadding
 *     always wait in order to read their status word;
 *   - "in place" means the array's pointer does not change; the planner may
 *     take device scratch from the device's stream-ordered memory pool on
 *     the caller's stream (calls on different streams never share it):
 *       cycle following (PTTWAC): one done bit per unit (a 16384 x 12289
 *         fp32 transpose: 786 KB);
 *       the stash plan (100 on units under 128 bytes, e.g. the plain
 *         transpose of a large matrix): the stash, about half the payload
 *         (421 MB for 16384 x 12289 fp32), plus 8 bytes per row;
 *       the staged form (blocks transposed out of place, then copied back):
 *         the payload's size plus 16 bytes;
 *       padding: 8 bytes per 4096-element task;
 *     payloads that fit the shared memory of all SMs (about 30 MB on GB300)
 *     move through shared memory instead and take no scratch.
 *     When the pool cannot supply the stash or the staged form's scratch
 *     the planner falls through to a method that needs less (ultimately
 *     cycle following); lm_transpose_100_noalloc allocates nothing.
 *
 * Notation: 010  [A][a][B]     -> [A][B][a]
 *           100  [A][B][b]     -> [B][A][b]
 *           0100 [A][a][B][b]  -> [A][B][a][b]
 */
#ifndef LIBMARSHAL_GB300_LM_MARSHAL_H_
#define LIBMARSHAL_GB300_LM_MARSHAL_H_

#ifndef __cplusplus
#include <stdbool.h>
#endif

#ifdef __cplusplus
extern "C" {
#endif

struct CUstream_st;
typedef struct CUstream_st *lm_stream_t; /* == cudaStream_t */

/* Message of the calling thread's last failed call ("" if none). */
const char *lm_last_error(void);
const char *lm_version(void);

/* Releases pooled scratch memory.  Reference: cl_marshal_finalize
 * (src/cl_marshal.cc:116-119; declared by the reference's tests,
 * test/cl_unittest.cc:99).  Both names are exported. */
void lm_marshal_finalize(void);
void cl_marshal_finalize(void);

/* AoS [height][width] -> ASTA [height/tile][width][tile] (010).
 * Reference: cl_aos_asta_bs, cl_marshal.h:26-27 / cl_marshal.cc:793-800. */
bool lm_aos_asta_bs(lm_stream_t stream, void *buf, int elem_bytes, int height,
                    int width, int tile_size);
/* Reference: cl_aos_asta_pttwac, cl_marshal.h:28-29 / cl_marshal.cc:803-812.
 * R: spreading factor of the done-bit map (power of two, 1..32); P: padding
 * words per 32 flag words. */
bool lm_aos_asta_pttwac(lm_stream_t stream, void *buf, int elem_bytes,
                        int height, int width, int tile_size, int R, int P);
/* BS first, PTTWAC only if BS failed; true only if both failed.
 * Reference: cl_aos_asta, cl_marshal.h:30-31 / cl_marshal.cc:814-818. */
bool lm_aos_asta(lm_stream_t stream, void *buf, int elem_bytes, int height,
                 int width, int tile_size, int R);

/* Full in-place transposition [A*a][B*b] -> [B*b][A*a].  Every stage code
 * of the reference (2, 22, 3, 32, 4, anything else the element-wise
 * fallback) yields this same layout; this call runs it as one planned 100
 * (A*a, B*b, 1), which is faster than the staged sequence, and checks the
 * arguments as the reference does.  lm_transpose_ex with a forced 010
 * variant runs the staged elementary transpositions themselves.  et may be
 * NULL.  Reference: cl_transpose, cl_marshal.h:32-33 / cl_marshal.cc:561-776. */
bool lm_transpose(lm_stream_t stream, void *buf, int elem_bytes, int A, int a,
                  int B, int b, int R, int stages, unsigned long long *et);
/* Full in-place transposition of an arbitrary M x N matrix ([M][N] ->
 * [N][M]) by the reference's flow for general matrices
 * (test/cl_unittest.cc:396-640): "Algorithm 5" chooses the super-element
 * sizes a and b as the largest divisors in [24, floor(sqrt(MAX_MEM))] of M
 * and N, each padded by the fewest elements that give it one, "Algorithm 3"
 * the stage code; then padding (cl_padding) -> the staged transposition
 * (cl_transpose) -> unpadding (cl_unpadding).  MAX_MEM is the reference's
 * 48 KB of local memory in elements: 12288 (elements of 1-4 bytes) or 6144
 * (8 bytes).
 * lm_full_transpose_plan writes {A, a, B, b, pad_h, pad_w, stages} to plan7
 * (may be NULL) and the elements the padded flow needs, (M + pad_h) *
 * (N + pad_w), to padded_elems (may be NULL).
 * lm_full_transpose: buf holds capacity_elems elements, the M x N matrix
 * first.  variant010 1 or 2 runs the reference's flow with BS or PTTWAC 010
 * steps and needs capacity_elems >= the padded count; 0 runs the same
 * permutation as one planned 100(M, N, 1), with no padding (capacity M*N).
 * The result is [N][M] in the first M*N elements either way.  et may be
 * NULL.  The reference has this flow in its test, not as a library call. */
bool lm_full_transpose_plan(int M, int N, int elem_bytes, int *plan7,
                            long long *padded_elems);
bool lm_full_transpose(lm_stream_t stream, void *buf, int elem_bytes, int M,
                       int N, long long capacity_elems, int variant010,
                       unsigned long long *et);
/* Same with the variant of every 010 step: 0 = as lm_transpose (one planned
 * 100), 1 = the stages with BS 010 steps, 2 = the stages with PTTWAC 010
 * steps.  No reference counterpart (the reference picks by MAX_MEM,
 * cl_marshal.cc:578-585). */
bool lm_transpose_ex(lm_stream_t stream, void *buf, int elem_bytes, int A,
                     int a, int B, int b, int R, int stages, int variant010,
                     unsigned long long *et);

/* 010 by barrier-synchronised tiles.  Reference: cl_transpose_010_bs,
 * cl_marshal.h:35-36 / cl_marshal.cc:136-277.  Returns true when the tile
 * exceeds on-chip capacity (the reference fails the same way past MAX_MEM). */
bool lm_transpose_010_bs(lm_stream_t stream, void *buf, int elem_bytes, int A,
                         int a, int B, unsigned long long *et);
/* 010 by in-tile cycle following.  Reference: cl_transpose_010_pttwac,
 * cl_marshal.h:37-38 / cl_marshal.cc:280-336. */
bool lm_transpose_010_pttwac(lm_stream_t stream, void *buf, int elem_bytes,
                             int A, int a, int B, unsigned long long *et,
                             int R, int P);
/* 100 [A][B][b] -> [B][A][b].  Reference: cl_transpose_100,
 * cl_marshal.h:40-41 / cl_marshal.cc:779-782. */
bool lm_transpose_100(lm_stream_t stream, void *buf, int elem_bytes, int A,
                      int B, int b, unsigned long long *et);
/* 0100 [A][a][B][b] -> [A][B][a][b].  Reference: cl_transpose_0100,
 * cl_marshal.h:43-44 / cl_marshal.cc:785-788. */
bool lm_transpose_0100(lm_stream_t stream, void *buf, int elem_bytes, int A,
                       int a, int B, int b, unsigned long long *et);
/* 0100 with the algorithm forced: 0 = planner, 1 = BS (on-chip tiles),
 * 2 = PTTWAC on b-element units, 3 = stash (A == 1 only: save the half that
 * is overwritten first, then a streaming wavefront), 4 = two passes (BS on
 * tiles that make >= 128-byte units, then PTTWAC on those units), 5 = whole
 * cycles (when every cycle of 100(a, B) has at most 32 units: find each
 * cycle's smallest position, then move whole cycles through registers),
 * 6 = through scratch (each tile's blocks transposed out of place into a
 * stream-ordered scratch buffer of the payload's size, then copied back),
 * 7 = held in shared memory (payloads up to about 30 MB: every CTA loads its
 * blocks, all CTAs meet at a grid barrier, then write their blocks
 * transposed over the buffer; one cooperative launch, no scratch; not
 * under stream capture).  Returns
 * true when the forced algorithm does not apply to the shape.  No reference
 * counterpart (the reference picks by super-element size,
 * cl_marshal.cc:365-370). */
bool lm_transpose_0100_method(lm_stream_t stream, void *buf, int elem_bytes,
                              int A, int a, int B, int b, int method,
                              unsigned long long *et);

/* Row padding [y_size][x_size] -> [y_size][pad_size] (new columns zero) and
 * unpadding [y_size][pad_size] -> [y_size][x_size] (tail zero).  buf holds
 * y_size*pad_size elements.  Reference: cl_padding / cl_unpadding,
 * cl_marshal.h:46-49 / cl_marshal.cc:821-956. */
bool lm_padding(lm_stream_t stream, void *buf, int elem_bytes, int x_size,
                int y_size, int pad_size, unsigned long long *et);
bool lm_unpadding(lm_stream_t stream, void *buf, int elem_bytes, int x_size,
                  int y_size, int pad_size, unsigned long long *et);

/* 100 [A][B][b] -> [B][A][b] like lm_transpose_100, for callers that cannot
 * allocate device memory while they run -- for example an allocator or
 * memory manager converting layouts from inside its own allocation path
 * (calling cudaMalloc there would re-enter it), or a real-time pipeline that
 * reserves all device memory at start-up.  No counterpart in the reference.
 * It allocates nothing: its scratch (one done bit per unit) is a fixed 4 MiB
 * device array that every GPU loading this library keeps until exit, so a
 * call handles at most 33,554,432 units (a unit larger than one slice, at
 * most 4 KiB, counts once per slice); larger shapes return true with an
 * error.  All calls on a
 * device share that array (each clears what it uses first): calls that
 * overlap on the GPU race -- order them on one stream.  The first call on a
 * device sets it up (looks the array up with that device current, loads the
 * kernel's variants, clears one word of the array on `stream`); a call with
 * zero sizes (e.g. A = B = b = 0, buf NULL) does only that: make one at
 * start-up, before allocation is forbidden and before any stream capture.
 * Asynchronous, stream ordered; false on success. */
bool lm_transpose_100_noalloc(lm_stream_t stream, void *buf, int elem_bytes,
                              int A, int B, int b);

/* Waits for `stream`, then returns and clears the accumulated failure status
 * of this device's waiting kernels (0 = ok, 1 = an inter-CTA wait timed out).
 * Asynchronous calls (et == NULL) report such failures only here; timed calls
 * (et != NULL) check it themselves.  No reference counterpart. */
unsigned lm_device_status(lm_stream_t stream);

/* 1 when a 0100 tile [a][B][b] (T tiles) of elem_bytes elements can be staged
 * on chip (shared memory of one CTA or of a thread-block cluster), else 0.
 * Counterpart of T010_BS::IsFeasible (include/plan.hpp:108-111). */
int lm_bs_feasible(long long T, int a, int B, int b, int elem_bytes);

/* Failure-detection hook (no reference counterpart): padding (unpad == 0) or
 * unpadding whose task `stall_block` waits on a flag nothing sets.  The wait
 * gives up after timeout_ns; the call must return true and leave the CUDA
 * context usable. */
bool lm_debug_pad_stall(lm_stream_t stream, void *buf, int elem_bytes,
                        int x_size, int y_size, int pad_size, int unpad,
                        long long stall_block, unsigned long long timeout_ns);

/* Failure-detection hook (no reference counterpart): the shared-memory
 * resident form of 0100(A, a, B, b) (lm_transpose_0100_method, method 7)
 * with its grid barrier waiting for one arrival more than there are CTAs.
 * Every CTA gives up after timeout_ns without writing; the call must return
 * true, leave the buffer unchanged and the CUDA context usable. */
bool lm_debug_resident_stall(lm_stream_t stream, void *buf, int elem_bytes,
                             int A, int a, int B, int b,
                             unsigned long long timeout_ns);

/* ---- batched conversion (no reference counterpart) -------------------------
 * A batch is a list of independent in-place jobs, each on its own device
 * buffer (buffers must not overlap), of any op and element width.
 * lm_batch_run plans the list: jobs whose tiles fit one CTA's shared memory
 * become work items of one persistent work-stealing kernel (mixed widths);
 * jobs whose tiles fit the shared memory of a thread-block cluster become
 * items of a persistent clustered kernel (one launch per cluster size; not
 * with LM_BATCH_NO_CLUSTER); jobs that fit the batch's scratch arena
 * (LM_BATCH_SCRATCH_MB, default 1024; not with LM_BATCH_NO_SCRATCH) are
 * staged: transposed block by block into the arena, then copied back, in
 * waves of at most one arena each (two launches per wave, at most 32 waves);
 * the rest go through the per-op planner, spread over the batch's side
 * streams, whose algorithm choice per shape class is autotuned (timed once
 * on a scratch buffer, then remembered; LM_TUNE_FILE persists the table).  With LM_BATCH_GRAPH, the second run of an identical
 * job list is captured into a CUDA graph and later runs replay it.  Ordered
 * on `stream` as a whole. */
enum {
  LM_OP_0100 = 0,      /* d0..d3 = A, a, B, b:  [A][a][B][b] -> [A][B][a][b] */
  LM_OP_010 = 1,       /* A, a, B:              [A][a][B] -> [A][B][a] */
  LM_OP_100 = 2,       /* A, B, b:              [A][B][b] -> [B][A][b] */
  LM_OP_AOS_ASTA = 3,  /* height, width, tile:  [h][w] -> [h/t][w][t] */
  LM_OP_ASTA_AOS = 4,  /* height, width, tile:  [h/t][w][t] -> [h][w] */
  LM_OP_SOA_ASTA = 5,  /* height, width, tile:  [w][h] -> [h/t][w][t] */
  LM_OP_ASTA_SOA = 6,  /* height, width, tile:  [h/t][w][t] -> [w][h] */
  LM_OP_TRANSPOSE = 7  /* M, N:                 [M][N] -> [N][M] */
};
enum {
  LM_BATCH_GRAPH = 1,
  LM_BATCH_NO_TUNE = 2,
  LM_BATCH_NO_CLUSTER = 4,
  LM_BATCH_NO_SCRATCH = 8 /* strictly in place: no staged form */
};
typedef struct {
  void *buf;      /* device buffer, converted in place */
  int elem_bytes; /* 1, 2, 4 or 8 */
  int op;         /* LM_OP_* */
  long long d0, d1, d2, d3;
} lm_job;
typedef struct {
  unsigned long long bytes, small_bytes, big_bytes, large_bytes;
  unsigned long long small_jobs, big_jobs, large_jobs, identity;
  unsigned long long small_items, big_items;
  unsigned long long band_bytes, band_jobs, band_items;
  unsigned long long staged_bytes, staged_jobs, staged_waves;
} lm_batch_stats;
typedef struct lm_batch_st *lm_batch_t;
bool lm_batch_create(lm_batch_t *out);
void lm_batch_destroy(lm_batch_t batch);
bool lm_batch_run(lm_batch_t batch, lm_stream_t stream, const lm_job *jobs,
                  int njobs, unsigned flags);
bool lm_batch_stats_get(lm_batch_t batch, lm_batch_stats *out);
/* Bytes of the staging arena of this handle (0: LM_BATCH_SCRATCH_MB, whose
 * default is 1024 MiB); applies from the next lm_batch_run. */
bool lm_batch_set_arena(lm_batch_t batch, unsigned long long bytes);
/* Autotuner table: entries tuned so far (and loaded from LM_TUNE_FILE).  The
 * batch executor's large jobs (and the server's) run the variant tuned for
 * their shape class -- key (element width, log2 a, log2 B, log2 b, T > 1)
 * after widening the units -- found by timing every applicable variant
 * once: the planner's own choice; the staged form with 16, 32 or 64 KB
 * blocks; whole-cycle moves; the stash plan with the planner's, one or two
 * CTAs per SM; the two-pass split; cycle following (variants 0..9 in that
 * order).  lm_tune_variant pins a class's variant (variant >= 0) or reads it
 * (variant < 0); it returns the class's variant, or -1 if it has none.  No
 * reference counterpart (the reference's hand tables, cl_marshal.cc:165-241,
 * 388-465). */
int lm_tune_entries(void);
int lm_tune_variant(int elem_bytes, long long T, long long a, long long B,
                    long long b, int variant);

/* ---- conversion server (no reference counterpart) -------------------------
 * lm_serve_create starts a worker thread on the current device.  Each
 * lm_serve_submit queues one request; requests are admitted in submission
 * order while the payload of admitted, unfinished requests stays within
 * `budget_bytes`, sorted by payload into three lanes (<= 2 MiB, <= 64 MiB,
 * larger) with their own prioritised streams, and run as batches
 * (lm_batch_run) whenever a lane has a free slot.  A request on a device
 * buffer (`buf`) is converted in place; with buf == NULL the host array
 * `src` is copied to a device pool of budget_bytes, converted, and copied
 * back to `dst` (which may equal src).  The caller keeps every buffer alive
 * and untouched until the request's completion is polled.  lm_serve_poll
 * returns up to cap completions (ticket, status 0 = ok, latency from
 * submission to completion and time spent waiting for admission), or -1 on
 * bad arguments. */
typedef struct {
  int elem_bytes; /* 1, 2, 4 or 8 */
  int op;         /* LM_OP_* */
  long long d0, d1, d2, d3;
  void *buf;       /* device buffer converted in place, or NULL */
  const void *src; /* host input when buf == NULL */
  void *dst;       /* host output when buf == NULL */
} lm_request;
typedef struct {
  unsigned long long ticket;
  int status;
  long long latency_ns, queue_ns;
  long long done_ns; /* completion time, CLOCK_MONOTONIC nanoseconds */
} lm_serve_done;
typedef struct {
  unsigned long long submitted, completed, batches, bytes, peak_inflight_bytes;
} lm_serve_stats;
typedef struct lm_serve_st *lm_serve_t;
bool lm_serve_create(lm_serve_t *out, unsigned long long budget_bytes);
bool lm_serve_submit(lm_serve_t server, const lm_request *req,
                     unsigned long long *ticket);
int lm_serve_poll(lm_serve_t server, lm_serve_done *out, int cap);
/* Waits until every submitted request has completed (timeout_ms < 0: no
 * limit); true on timeout or if a batch failed (lm_last_error says why). */
bool lm_serve_drain(lm_serve_t server, long long timeout_ms);
bool lm_serve_stats_get(lm_serve_t server, lm_serve_stats *out);
void lm_serve_destroy(lm_serve_t server);
/* Trace replay (load generator): request k is submitted arrival_ns[k] after
 * the call starts, and not before requests 0..after[k] (-1: none; after[k]
 * must be < k) have all completed, so a trace can reuse buffers ring-wise.  out[k] receives request k's
 * completion, latency and queueing measured from its scheduled arrival.
 * With LM_SERVE_PLAIN (server may be NULL) each request instead runs alone
 * through the per-op planner on one stream at its arrival. */
enum { LM_SERVE_PLAIN = 1 };
bool lm_serve_replay(lm_serve_t server, const lm_request *reqs,
                     const long long *arrival_ns, const int *after, int n,
                     unsigned flags, lm_serve_done *out);

/* ---- profiling (counterpart of include/cl_profile.h:6-63) ----------------
 * lm_launch_count: kernels launched by this library since it was loaded.
 * lm_prof_enable(1): from now on every launch is bracketed by a CUDA event
 * pair on its stream.  lm_prof_collect: waits for the recorded events, writes
 * up to cap per-kernel entries (launches, summed device ms), clears the
 * record, and returns the number of distinct kernels. */
typedef struct {
  char name[48];
  long long launches;
  double total_ms;
} lm_prof_entry;
unsigned long long lm_launch_count(void);
void lm_prof_enable(int on);
int lm_prof_collect(lm_prof_entry *out, int cap);
/* Instead of lm_prof_collect: the recorded launches one by one, in launch
 * order, with start and end in ms from the earliest recorded start (launches
 * on several streams show their overlap); clears the record and returns the
 * number of launches recorded (up to cap are written). */
typedef struct {
  char name[48];
  double start_ms, end_ms;
} lm_prof_span;
int lm_prof_timeline(lm_prof_span *out, int cap);

#ifdef __cplusplus
}
#endif

#endif /* LIBMARSHAL_GB300_LM_MARSHAL_H_ */
