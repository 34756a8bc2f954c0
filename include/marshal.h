/*
 * marshal.h -- drop-in for the reference's CUDA interface.
 *
 * Replaces include/marshal.h:24-33 of libmarshal (declarations) whose
 * implementation is src/marshal.cu:27-80.  Same names, same signatures, same
 * convention: the functions convert a DEVICE buffer in place, launch on the
 * legacy default stream without synchronising, and return false on success,
 * true on error (lm_last_error() in lm_marshal.h gives the message).
 *
 * Differences a caller can observe, all in the direction of "works":
 *   - every function is bit-exact for every shape whose height is a multiple
 *     of tile_size (the reference's BS_marshal writes the tile back unchanged
 *     and PTTWAC_marshal converts only the first 1024 tiles);
 *   - a height that is not a multiple of tile_size returns true instead of
 *     tripping an assert;
 *   - `timer` is accepted and never written (the reference's kernels never
 *     write it either).
 */
#ifndef LIBMARSHAL_GB300_MARSHAL_H_
#define LIBMARSHAL_GB300_MARSHAL_H_

#include <time.h>
#ifndef __cplusplus
#include <stdbool.h>
#endif

#ifdef __cplusplus
extern "C" {
#endif

/* AoS [height][width] -> ASTA [height/tile][width][tile]: 010(h/t, t, w).
 * Reference: include/marshal.h:26-27, src/marshal.cu:27-49. */
bool gpu_aos_asta_bs_float(float *src, int height, int width, int tile_size,
                           clock_t *timer);
bool gpu_aos_asta_bs_double(double *src, int height, int width, int tile_size,
                            clock_t *timer);

/* Same conversion by in-tile cycle following (done bits in shared memory).
 * Reference: include/marshal.h:29, src/marshal.cu:51-62. */
bool gpu_aos_asta_pttwac(float *src, int height, int width, int tile_size,
                         clock_t *timer);

/* SoA [width][height] -> ASTA [height/tile][width][tile]: 100(w, h/t, t).
 * Reference: include/marshal.h:31, src/marshal.cu:64-80. */
bool gpu_soa_asta_pttwac(float *src, int height, int width, int tile_size,
                         clock_t *timer);

#ifdef __cplusplus
}
#endif

#endif /* LIBMARSHAL_GB300_MARSHAL_H_ */
