/* cl_marshal_compat.h -- the reference's OpenCL entry-point names
 * (include/cl_marshal.h:26-49 of libmarshal) on top of lm_marshal.h, for
 * code that was written against cl_marshal and is moved to CUDA without
 * touching its call sites.
 *
 * Include it INSTEAD of CL/cl.h and cl_marshal.h: the queue becomes a CUDA
 * stream, a cl_mem a device pointer, and cl_ulong the 64-bit elapsed-time
 * counter.  The reference builds its kernels for one element type (float by
 * default); LM_CL_ELEM_BYTES (default 4) is that type's size.  Every
 * function keeps the reference's argument order, its false-on-success
 * convention and its elapsed-time accumulation; cl_marshal_finalize comes
 * from the library itself.
 */
#ifndef LM_CL_MARSHAL_COMPAT_H
#define LM_CL_MARSHAL_COMPAT_H

#include "lm_marshal.h"

#ifndef LM_CL_ELEM_BYTES
#define LM_CL_ELEM_BYTES 4
#endif

typedef lm_stream_t cl_command_queue;
typedef void *cl_mem;
typedef unsigned long long cl_ulong;

#ifdef __cplusplus
extern "C" {
#endif

static inline bool cl_transpose(cl_command_queue q, cl_mem src, int A, int a,
                                int B, int b, int R, int stages, cl_ulong *et) {
  return lm_transpose(q, src, LM_CL_ELEM_BYTES, A, a, B, b, R, stages, et);
}

static inline bool cl_transpose_010_bs(cl_command_queue q, cl_mem src, int A,
                                       int a, int B, cl_ulong *et) {
  return lm_transpose_010_bs(q, src, LM_CL_ELEM_BYTES, A, a, B, et);
}

static inline bool cl_transpose_010_pttwac(cl_command_queue q, cl_mem src,
                                           int A, int a, int B, cl_ulong *et,
                                           int R, int P) {
  return lm_transpose_010_pttwac(q, src, LM_CL_ELEM_BYTES, A, a, B, et, R, P);
}

static inline bool cl_transpose_100(cl_command_queue q, cl_mem src, int A,
                                    int B, int b, cl_ulong *et) {
  return lm_transpose_100(q, src, LM_CL_ELEM_BYTES, A, B, b, et);
}

static inline bool cl_transpose_0100(cl_command_queue q, cl_mem src, int A,
                                     int a, int B, int b, cl_ulong *et) {
  return lm_transpose_0100(q, src, LM_CL_ELEM_BYTES, A, a, B, b, et);
}

static inline bool cl_aos_asta_bs(cl_command_queue q, cl_mem src, int height,
                                  int width, int tile_size) {
  return lm_aos_asta_bs(q, src, LM_CL_ELEM_BYTES, height, width, tile_size);
}

static inline bool cl_aos_asta_pttwac(cl_command_queue q, cl_mem src,
                                      int height, int width, int tile_size,
                                      int R, int P) {
  return lm_aos_asta_pttwac(q, src, LM_CL_ELEM_BYTES, height, width,
                            tile_size, R, P);
}

static inline bool cl_aos_asta(cl_command_queue q, cl_mem src, int height,
                               int width, int tile_size, int R) {
  return lm_aos_asta(q, src, LM_CL_ELEM_BYTES, height, width, tile_size, R);
}

static inline bool cl_padding(cl_command_queue q, cl_mem src, int x_size,
                              int y_size, int pad_size, cl_ulong *et) {
  return lm_padding(q, src, LM_CL_ELEM_BYTES, x_size, y_size, pad_size, et);
}

static inline bool cl_unpadding(cl_command_queue q, cl_mem src, int x_size,
                                int y_size, int pad_size, cl_ulong *et) {
  return lm_unpadding(q, src, LM_CL_ELEM_BYTES, x_size, y_size, pad_size, et);
}

#ifdef __cplusplus
}
#endif

#endif /* LM_CL_MARSHAL_COMPAT_H */
