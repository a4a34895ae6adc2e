/*
 * iwpp_synth.h -- deterministic synthetic inputs for reconstruction by
 * dilation (host C, no CUDA).  Identical output on x86-64 and AArch64 and for
 * any thread count.  Functions return 0 on success.
 */
#ifndef IWPP_SYNTH_H
#define IWPP_SYNTH_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

enum { IWPP_SYNTH_U8 = 0, IWPP_SYNTH_U16 = 1, IWPP_SYNTH_I32 = 2 };

/* Mask = uniform 8-bit noise (SplitMix64 of seed and pixel index), Gaussian
 * smoothed (separable, truncated at 4 sigma, mirrored borders), rescaled to
 * the dtype's full range, then `ndiscs` filled discs (radius in [rmin, rmax],
 * 8-bit level in [vmin8, vmax8] scaled to the dtype) painted as max(). */
int iwpp_synth_noise_mask(void *mask, int W, int H, size_t pitch, int dtype, uint64_t seed, double sigma,
                          int ndiscs, int rmin, int rmax, int vmin8, int vmax8, int nthreads);
/* marker = max(mask - h, dtype min), h given in 8-bit levels. */
int iwpp_synth_hdome_marker(void *marker, const void *mask, int W, int H, size_t pitch_marker, size_t pitch_mask,
                            int dtype, int h8);
/* marker = dtype min except round(fraction * W * H) random pixels = mask. */
int iwpp_synth_sparse_marker(void *marker, const void *mask, int W, int H, size_t pitch_marker, size_t pitch_mask,
                             int dtype, uint64_t seed, double fraction);
/* Paints a one-pixel square spiral corridor of the dtype maximum into mask. */
int64_t iwpp_synth_spiral_corridor(void *mask, int W, int H, size_t pitch, int dtype, int arm_pitch, int *start_x,
                                   int *start_y);
/* marker = dtype min except nseeds pixels = mask; the first seed is
 * (first_x, first_y) when both are >= 0, the rest are random. */
int iwpp_synth_seed_marker(void *marker, const void *mask, int W, int H, size_t pitch_marker, size_t pitch_mask,
                           int dtype, uint64_t seed, int nseeds, int first_x, int first_y);
/* uint8 only: marker uniform, mask = marker + r % (256 - marker). */
int iwpp_synth_uniform_pair(void *marker, void *mask, int W, int H, size_t pitch_marker, size_t pitch_mask,
                            uint64_t seed);
/* An 8-bit level mapped to the dtype's full range. */
int64_t iwpp_synth_scale8(int dtype, int v8);
/* The n-th (1-based) MT19937-64 output for a seed (self-test of the RNG). */
uint64_t iwpp_synth_mt64_nth(uint64_t seed, uint64_t n);
int iwpp_synth_version(void);

#ifdef __cplusplus
}
#endif
#endif
