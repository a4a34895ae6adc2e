/*
 * iwpp_oracle.h -- CPU oracle for reconstruction by dilation.
 * TEST INFRASTRUCTURE ONLY: linked by the tests, the smoke check and the
 * bench's CPU-baseline leg as the checker; never by the product library.
 *
 * All functions work in place on `marker` (row-major, byte pitches), accept
 * uint8 / uint16 / int32 pixels and 4- or 8-connectivity, and treat pixels
 * outside the image as non-existent.  They return ORACLE_OK or an error.
 */
#ifndef IWPP_ORACLE_H
#define IWPP_ORACLE_H

#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

enum { ORACLE_U8 = 0, ORACLE_U16 = 1, ORACLE_I32 = 2 };
enum { ORACLE_OK = 0, ORACLE_ERR_INVALID = 1, ORACLE_ERR_OOM = 2 };

/* Vincent 1993 hybrid algorithm (raster, anti-raster, FIFO). */
int oracle_reconstruct(void *marker, const void *mask, int width, int height, size_t pitch_marker,
                       size_t pitch_mask, int dtype, int conn);
/* Raster / anti-raster scans repeated to a fixed point. */
int oracle_reconstruct_sr(void *marker, const void *mask, int width, int height, size_t pitch_marker,
                          size_t pitch_mask, int dtype, int conn);
/* All pixels updated at once until stable (small images only). */
int oracle_reconstruct_jacobi(void *marker, const void *mask, int width, int height, size_t pitch_marker,
                              size_t pitch_mask, int dtype, int conn);
/* marker = min(marker, mask). */
int oracle_clip(void *marker, const void *mask, int width, int height, size_t pitch_marker, size_t pitch_mask,
                int dtype);
int oracle_version(void);

#ifdef __cplusplus
}
#endif
#endif
