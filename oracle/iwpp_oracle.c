/*
 * iwpp_oracle.c -- CPU oracle for grayscale morphological reconstruction by
 * dilation.  TEST INFRASTRUCTURE ONLY: the tests, the smoke check and the
 * bench's CPU-baseline leg link this file as the checker.  The product path
 * (libiwpp.so) never calls it.
 *
 * What the reference computes (IWPP MP/src/MorphologicalReconstruction.cu):
 *   - propagation rule, MR.cu:43-44 (and the three other sweeps, :75-76,
 *     :107-108, :140-141):
 *         if (m[p] > m[c] && m[c] < mask[c]) m[c] = min(m[p], mask[c]);
 *     which is m[c] = max(m[c], min(m[p], mask[c])) for every neighbour p;
 *   - neighbourhood: 4-connectivity (the +-X / +-Y sweeps, MR.cu:34-161);
 *     8-connectivity is the standard extension (the 4 diagonals added);
 *   - border: pixels outside the image do not exist (the reference pads
 *     the out-of-image halo with marker = mask = 0, MR.cu:252-256, :267-270,
 *     :280-283, :293-296, which is inert for unsigned pixels; here the
 *     neighbour is simply skipped, which is what that padding means);
 *   - precondition clip, MR.cu:827-836: marker = min(marker, mask), run by
 *     the caller (IWPP MP/src/main.cu:55).  The rule above never lowers a
 *     pixel, so without the clip the result is the least image m >= marker
 *     with m[c] >= min(m[p], mask[c]) for all neighbour pairs; every
 *     function here computes exactly that fixed point.
 *
 * The reference has no CPU implementation, so this is a restatement of the
 * published sequential algorithms:
 *   - oracle_reconstruct: L. Vincent, "Morphological grayscale reconstruction
 *     in image analysis: applications and efficient algorithms", IEEE TIP
 *     2(2), 1993 -- the hybrid algorithm (one raster scan, one anti-raster
 *     scan, then a FIFO propagation);
 *   - oracle_reconstruct_sr: the same paper's "sequential reconstruction"
 *     (raster / anti-raster scans repeated until nothing changes);
 *   - oracle_reconstruct_jacobi: the definition itself, applied to all pixels
 *     at once until stable (small images only).
 * Three different schedules of the same monotone operator; the fixed point is
 * unique, so they must agree bit for bit.
 */
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

#include "iwpp_oracle.h"

/* ---------------------------------------------------------------- FIFO */
typedef struct {
    int64_t *buf;
    int64_t cap, head, count;
} fifo_t;

static int fifo_init(fifo_t *q, int64_t cap) {
    if (cap < 1024) cap = 1024;
    q->buf = (int64_t *)malloc((size_t)cap * sizeof(int64_t));
    q->cap = cap;
    q->head = 0;
    q->count = 0;
    return q->buf ? 0 : -1;
}

static int fifo_push(fifo_t *q, int64_t v) {
    if (q->count == q->cap) {
        int64_t ncap = q->cap * 2;
        int64_t *nb = (int64_t *)malloc((size_t)ncap * sizeof(int64_t));
        if (!nb) return -1;
        for (int64_t i = 0; i < q->count; ++i) nb[i] = q->buf[(q->head + i) % q->cap];
        free(q->buf);
        q->buf = nb;
        q->cap = ncap;
        q->head = 0;
    }
    q->buf[(q->head + q->count) % q->cap] = v;
    q->count++;
    return 0;
}

static int64_t fifo_pop(fifo_t *q) {
    int64_t v = q->buf[q->head];
    q->head = (q->head + 1) % q->cap;
    q->count--;
    return v;
}

/* Neighbour offsets.  The first half of each list is N+ (already visited by
 * a raster scan), the second half N- (visited first by an anti-raster scan). */
static const int NB8_DX[8] = {-1, -1, 0, 1, 1, 1, 0, -1};
static const int NB8_DY[8] = {0, -1, -1, -1, 0, 1, 1, 1};
static const int NB4_DX[4] = {-1, 0, 1, 0};
static const int NB4_DY[4] = {0, -1, 0, 1};

/* ------------------------------------------------ type-generic bodies */
#define ORACLE_T uint8_t
#define ORACLE_SUFFIX u8
#include "iwpp_oracle_impl.inc"
#undef ORACLE_T
#undef ORACLE_SUFFIX

#define ORACLE_T uint16_t
#define ORACLE_SUFFIX u16
#include "iwpp_oracle_impl.inc"
#undef ORACLE_T
#undef ORACLE_SUFFIX

#define ORACLE_T int32_t
#define ORACLE_SUFFIX i32
#include "iwpp_oracle_impl.inc"
#undef ORACLE_T
#undef ORACLE_SUFFIX

/* ---------------------------------------------------------- dispatch */
static int check_args(const void *marker, const void *mask, int width, int height,
                      size_t pitch_marker, size_t pitch_mask, int dtype, int conn) {
    size_t bpp;
    if (width < 0 || height < 0) return ORACLE_ERR_INVALID;
    if ((width == 0 || height == 0) && conn >= 0) {
        if (conn != 4 && conn != 8) return ORACLE_ERR_INVALID;
        return dtype >= ORACLE_U8 && dtype <= ORACLE_I32 ? ORACLE_OK : ORACLE_ERR_INVALID;
    }
    if (!marker || !mask) return ORACLE_ERR_INVALID;
    if (conn != 4 && conn != 8) return ORACLE_ERR_INVALID;
    switch (dtype) {
        case ORACLE_U8: bpp = 1; break;
        case ORACLE_U16: bpp = 2; break;
        case ORACLE_I32: bpp = 4; break;
        default: return ORACLE_ERR_INVALID;
    }
    if (pitch_marker < (size_t)width * bpp || pitch_mask < (size_t)width * bpp) return ORACLE_ERR_INVALID;
    return ORACLE_OK;
}

#define ORACLE_DISPATCH(fn)                                                                       \
    int rc = check_args(marker, mask, width, height, pitch_marker, pitch_mask, dtype, conn);     \
    if (rc != ORACLE_OK) return rc;                                                              \
    if (width == 0 || height == 0) return ORACLE_OK;                                             \
    switch (dtype) {                                                                             \
        case ORACLE_U8: return fn##_u8(marker, mask, width, height, pitch_marker, pitch_mask, conn);   \
        case ORACLE_U16: return fn##_u16(marker, mask, width, height, pitch_marker, pitch_mask, conn); \
        default: return fn##_i32(marker, mask, width, height, pitch_marker, pitch_mask, conn);         \
    }

int oracle_reconstruct(void *marker, const void *mask, int width, int height, size_t pitch_marker,
                       size_t pitch_mask, int dtype, int conn) {
    ORACLE_DISPATCH(hybrid)
}

int oracle_reconstruct_sr(void *marker, const void *mask, int width, int height, size_t pitch_marker,
                          size_t pitch_mask, int dtype, int conn) {
    ORACLE_DISPATCH(sr)
}

int oracle_reconstruct_jacobi(void *marker, const void *mask, int width, int height, size_t pitch_marker,
                              size_t pitch_mask, int dtype, int conn) {
    ORACLE_DISPATCH(jacobi)
}

int oracle_clip(void *marker, const void *mask, int width, int height, size_t pitch_marker,
                size_t pitch_mask, int dtype) {
    int conn = 4;
    ORACLE_DISPATCH(clip)
}

int oracle_version(void) { return 1; }
