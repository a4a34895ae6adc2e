/*
 * iwpp_synth.c -- deterministic synthetic marker/mask generators.
 *
 * The reference ships no usable inputs (its JPEG test images are partly
 * missing and its golden TIFFs are outside the repository), so every
 * workload here is synthesised from a seed.  The results must be identical
 * on x86-64 and AArch64 hosts and for any thread count:
 *   - structural draws (disc centres, radii, values, seed positions) use
 *     MT19937-64 (Matsumoto & Nishimura, ACM TOMACS 2000) with explicit
 *     integer mappings;
 *   - per-pixel noise is a SplitMix64 hash of (seed, pixel index), so rows can
 *     be generated in parallel;
 *   - Gaussian weights use a series exp() written here (IEEE basic operations
 *     only), the convolution is done in double precision with a fixed
 *     summation order, and the file is compiled with -ffp-contract=off so no
 *     fused multiply-add changes a rounding on either architecture;
 *   - the smoothed image is quantised to 16.16 fixed point and rescaled with
 *     64-bit integer arithmetic (round half up).
 *
 * The uniform-marker generator restates the value law of the reference's
 * cuRAND test-case generator (IWPP MP/src/testCaseGenerator.cu:28-35:
 * marker = r1 % 256, mask = marker + (r2 % 256) % (256 - marker)) with the
 * SplitMix64 stream instead of cuRAND XORWOW.
 */
#include <math.h>
#include <pthread.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>
#include <unistd.h>

#include "iwpp_synth.h"

/* ------------------------------------------------------------- MT19937-64 */
#define MT_NN 312
#define MT_MM 156
typedef struct {
    uint64_t mt[MT_NN];
    int mti;
} mt64_t;

static void mt64_seed(mt64_t *s, uint64_t seed) {
    s->mt[0] = seed;
    for (int i = 1; i < MT_NN; ++i)
        s->mt[i] = 6364136223846793005ULL * (s->mt[i - 1] ^ (s->mt[i - 1] >> 62)) + (uint64_t)i;
    s->mti = MT_NN;
}

static uint64_t mt64_next(mt64_t *s) {
    static const uint64_t mag01[2] = {0ULL, 0xB5026F5AA96619E9ULL};
    const uint64_t UM = 0xFFFFFFFF80000000ULL, LM = 0x7FFFFFFFULL;
    uint64_t x;
    if (s->mti >= MT_NN) {
        int i;
        for (i = 0; i < MT_NN - MT_MM; ++i) {
            x = (s->mt[i] & UM) | (s->mt[i + 1] & LM);
            s->mt[i] = s->mt[i + MT_MM] ^ (x >> 1) ^ mag01[(int)(x & 1ULL)];
        }
        for (; i < MT_NN - 1; ++i) {
            x = (s->mt[i] & UM) | (s->mt[i + 1] & LM);
            s->mt[i] = s->mt[i + (MT_MM - MT_NN)] ^ (x >> 1) ^ mag01[(int)(x & 1ULL)];
        }
        x = (s->mt[MT_NN - 1] & UM) | (s->mt[0] & LM);
        s->mt[MT_NN - 1] = s->mt[MT_MM - 1] ^ (x >> 1) ^ mag01[(int)(x & 1ULL)];
        s->mti = 0;
    }
    x = s->mt[s->mti++];
    x ^= (x >> 29) & 0x5555555555555555ULL;
    x ^= (x << 17) & 0x71D67FFFEDA60000ULL;
    x ^= (x << 37) & 0xFFF7EEE000000000ULL;
    x ^= (x >> 43);
    return x;
}

/* uniform integer in [lo, hi] (modulo mapping; the tiny bias is part of the
 * definition of the workload, not an error) */
static int64_t mt64_range(mt64_t *s, int64_t lo, int64_t hi) {
    uint64_t span = (uint64_t)(hi - lo) + 1ULL;
    return lo + (int64_t)(mt64_next(s) % span);
}

uint64_t iwpp_synth_mt64_nth(uint64_t seed, uint64_t n) {
    mt64_t s;
    uint64_t v = 0;
    mt64_seed(&s, seed);
    for (uint64_t i = 0; i < n; ++i) v = mt64_next(&s);
    return v;
}

/* ---------------------------------------------------------- SplitMix64 hash */
static inline uint64_t mix64(uint64_t z) {
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ULL;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBULL;
    return z ^ (z >> 31);
}

static inline uint64_t hash2(uint64_t seed, uint64_t idx) {
    return mix64(seed * 0x9E3779B97F4A7C15ULL + idx * 0xD1B54A32D192ED03ULL + 0x632BE59BD9B4E019ULL);
}

/* --------------------------------------------------------- deterministic exp */
/* exp(x) for x <= 0 from basic IEEE operations: x = k ln2 + r, |r| <= ln2/2,
 * Taylor series for e^r (terms until they vanish), then an exact ldexp. */
static double det_exp(double x) {
    const double LN2 = 0.6931471805599453094172321;
    if (x < -700.0) return 0.0;
    double kf = floor(x / LN2 + 0.5);
    double r = x - kf * LN2;
    double term = 1.0, sum = 1.0;
    for (int i = 1; i < 40; ++i) {
        term = term * r / (double)i;
        sum = sum + term;
    }
    return ldexp(sum, (int)kf);
}

/* ------------------------------------------------------------ pixel helpers */
static size_t bpp_of(int dtype) { return dtype == IWPP_SYNTH_U8 ? 1 : dtype == IWPP_SYNTH_U16 ? 2 : 4; }

static void type_range(int dtype, int64_t *lo, int64_t *hi) {
    if (dtype == IWPP_SYNTH_U8) {
        *lo = 0;
        *hi = 255;
    } else if (dtype == IWPP_SYNTH_U16) {
        *lo = 0;
        *hi = 65535;
    } else {
        *lo = INT32_MIN;
        *hi = INT32_MAX;
    }
}

/* An 8-bit level scaled to the dtype's full range (u16: x257,
 * i32: INT32_MIN + x * 16843009, so 0 -> min and 255 -> max exactly). */
int64_t iwpp_synth_scale8(int dtype, int v8) {
    if (dtype == IWPP_SYNTH_U8) return v8;
    if (dtype == IWPP_SYNTH_U16) return (int64_t)v8 * 257;
    return (int64_t)INT32_MIN + (int64_t)v8 * 16843009LL;
}

static inline int64_t get_px(const void *base, size_t pitch, int dtype, int x, int y) {
    const char *row = (const char *)base + (size_t)y * pitch;
    if (dtype == IWPP_SYNTH_U8) return ((const uint8_t *)row)[x];
    if (dtype == IWPP_SYNTH_U16) return ((const uint16_t *)row)[x];
    return ((const int32_t *)row)[x];
}

static inline void set_px(void *base, size_t pitch, int dtype, int x, int y, int64_t v) {
    char *row = (char *)base + (size_t)y * pitch;
    if (dtype == IWPP_SYNTH_U8)
        ((uint8_t *)row)[x] = (uint8_t)v;
    else if (dtype == IWPP_SYNTH_U16)
        ((uint16_t *)row)[x] = (uint16_t)v;
    else
        ((int32_t *)row)[x] = (int32_t)v;
}

static int resolve_threads(int nthreads) {
    if (nthreads > 0) return nthreads > 256 ? 256 : nthreads;
    long n = sysconf(_SC_NPROCESSORS_ONLN);
    if (n < 1) n = 1;
    if (n > 64) n = 64;
    return (int)n;
}

static inline int reflect_idx(int i, int n) {
    /* (d c b a | a b c d | d c b a) */
    while (i < 0 || i >= n) {
        if (i < 0) i = -i - 1;
        if (i >= n) i = 2 * n - i - 1;
    }
    return i;
}

/* ------------------------------------------------------- smoothed noise */
typedef struct {
    int W, H, R, tid, nthreads;
    uint64_t seed;
    const double *w; /* 2R+1 weights, w[R] at the centre */
    float *hbuf;     /* W*H, horizontally smoothed noise */
    int32_t *fixed;  /* W*H, 16.16 fixed-point smoothed noise */
    int32_t vmin, vmax;
} smooth_job_t;

static void *smooth_h_worker(void *arg) {
    smooth_job_t *j = (smooth_job_t *)arg;
    int W = j->W, R = j->R;
    uint8_t *noise = (uint8_t *)malloc((size_t)W);
    for (int y = j->tid; y < j->H; y += j->nthreads) {
        uint64_t base = (uint64_t)y * (uint64_t)W;
        for (int x = 0; x < W; ++x) noise[x] = (uint8_t)(hash2(j->seed, base + (uint64_t)x) & 0xFF);
        float *out = j->hbuf + (size_t)y * W;
        for (int x = 0; x < W; ++x) {
            double acc = 0.0;
            for (int i = -R; i <= R; ++i) acc = acc + j->w[i + R] * (double)noise[reflect_idx(x + i, W)];
            out[x] = (float)acc;
        }
    }
    free(noise);
    return NULL;
}

static void *smooth_v_worker(void *arg) {
    smooth_job_t *j = (smooth_job_t *)arg;
    int W = j->W, H = j->H, R = j->R;
    double *acc = (double *)malloc((size_t)W * sizeof(double));
    int32_t vmin = INT32_MAX, vmax = INT32_MIN;
    for (int y = j->tid; y < H; y += j->nthreads) {
        for (int x = 0; x < W; ++x) acc[x] = 0.0;
        for (int i = -R; i <= R; ++i) {
            const float *src = j->hbuf + (size_t)reflect_idx(y + i, H) * W;
            double wi = j->w[i + R];
            for (int x = 0; x < W; ++x) acc[x] = acc[x] + wi * (double)src[x];
        }
        int32_t *out = j->fixed + (size_t)y * W;
        for (int x = 0; x < W; ++x) {
            int32_t v = (int32_t)nearbyint(acc[x] * 65536.0);
            out[x] = v;
            if (v < vmin) vmin = v;
            if (v > vmax) vmax = v;
        }
    }
    j->vmin = vmin;
    j->vmax = vmax;
    free(acc);
    return NULL;
}

int iwpp_synth_noise_mask(void *mask, int W, int H, size_t pitch, int dtype, uint64_t seed, double sigma,
                          int ndiscs, int rmin, int rmax, int vmin8, int vmax8, int nthreads) {
    if (!mask || W <= 0 || H <= 0 || pitch < (size_t)W * bpp_of(dtype) || sigma <= 0.0) return 1;
    if (dtype != IWPP_SYNTH_U8 && dtype != IWPP_SYNTH_U16 && dtype != IWPP_SYNTH_I32) return 1;
    int nt = resolve_threads(nthreads);
    int R = (int)ceil(4.0 * sigma);
    double *w = (double *)malloc((size_t)(2 * R + 1) * sizeof(double));
    float *hbuf = (float *)malloc((size_t)W * H * sizeof(float));
    int32_t *fixed = (int32_t *)malloc((size_t)W * H * sizeof(int32_t));
    smooth_job_t *jobs = (smooth_job_t *)calloc((size_t)nt, sizeof(smooth_job_t));
    pthread_t *th = (pthread_t *)calloc((size_t)nt, sizeof(pthread_t));
    if (!w || !hbuf || !fixed || !jobs || !th) {
        free(w);
        free(hbuf);
        free(fixed);
        free(jobs);
        free(th);
        return 2;
    }
    double wsum = 0.0;
    for (int i = -R; i <= R; ++i) {
        w[i + R] = det_exp(-((double)i * (double)i) / (2.0 * sigma * sigma));
    }
    for (int i = -R; i <= R; ++i) wsum = wsum + w[i + R];
    for (int i = -R; i <= R; ++i) w[i + R] = w[i + R] / wsum;

    for (int t = 0; t < nt; ++t) {
        jobs[t].W = W;
        jobs[t].H = H;
        jobs[t].R = R;
        jobs[t].tid = t;
        jobs[t].nthreads = nt;
        jobs[t].seed = seed;
        jobs[t].w = w;
        jobs[t].hbuf = hbuf;
        jobs[t].fixed = fixed;
    }
    for (int t = 0; t < nt; ++t) pthread_create(&th[t], NULL, smooth_h_worker, &jobs[t]);
    for (int t = 0; t < nt; ++t) pthread_join(th[t], NULL);
    for (int t = 0; t < nt; ++t) pthread_create(&th[t], NULL, smooth_v_worker, &jobs[t]);
    for (int t = 0; t < nt; ++t) pthread_join(th[t], NULL);
    int32_t smin = INT32_MAX, smax = INT32_MIN;
    for (int t = 0; t < nt; ++t) {
        if (jobs[t].vmin < smin) smin = jobs[t].vmin;
        if (jobs[t].vmax > smax) smax = jobs[t].vmax;
    }
    int64_t lo, hi;
    type_range(dtype, &lo, &hi);
    uint64_t span = (uint64_t)(hi - lo);
    uint64_t range = (uint64_t)((int64_t)smax - (int64_t)smin);
    for (int y = 0; y < H; ++y) {
        const int32_t *src = fixed + (size_t)y * W;
        for (int x = 0; x < W; ++x) {
            int64_t v = lo;
            if (range > 0) v = lo + (int64_t)(((uint64_t)((int64_t)src[x] - smin) * span + range / 2) / range);
            set_px(mask, pitch, dtype, x, y, v);
        }
    }
    free(w);
    free(hbuf);
    free(fixed);
    free(jobs);
    free(th);

    /* discs: mask = max(mask, v) inside each disc */
    mt64_t rng;
    mt64_seed(&rng, seed);
    for (int d = 0; d < ndiscs; ++d) {
        int cx = (int)mt64_range(&rng, 0, W - 1);
        int cy = (int)mt64_range(&rng, 0, H - 1);
        int r = (int)mt64_range(&rng, rmin, rmax);
        int64_t v = iwpp_synth_scale8(dtype, (int)mt64_range(&rng, vmin8, vmax8));
        int y0 = cy - r < 0 ? 0 : cy - r, y1 = cy + r >= H ? H - 1 : cy + r;
        int x0 = cx - r < 0 ? 0 : cx - r, x1 = cx + r >= W ? W - 1 : cx + r;
        for (int y = y0; y <= y1; ++y)
            for (int x = x0; x <= x1; ++x) {
                int64_t dx = x - cx, dy = y - cy;
                if (dx * dx + dy * dy <= (int64_t)r * r && get_px(mask, pitch, dtype, x, y) < v)
                    set_px(mask, pitch, dtype, x, y, v);
            }
    }
    return 0;
}

int iwpp_synth_hdome_marker(void *marker, const void *mask, int W, int H, size_t pitch_marker, size_t pitch_mask,
                            int dtype, int h8) {
    if (!marker || !mask || W <= 0 || H <= 0) return 1;
    int64_t lo, hi;
    type_range(dtype, &lo, &hi);
    int64_t h = iwpp_synth_scale8(dtype, h8) - iwpp_synth_scale8(dtype, 0);
    for (int y = 0; y < H; ++y)
        for (int x = 0; x < W; ++x) {
            int64_t v = get_px(mask, pitch_mask, dtype, x, y) - h;
            set_px(marker, pitch_marker, dtype, x, y, v < lo ? lo : v);
        }
    return 0;
}

int iwpp_synth_sparse_marker(void *marker, const void *mask, int W, int H, size_t pitch_marker, size_t pitch_mask,
                             int dtype, uint64_t seed, double fraction) {
    if (!marker || !mask || W <= 0 || H <= 0) return 1;
    int64_t lo, hi;
    type_range(dtype, &lo, &hi);
    for (int y = 0; y < H; ++y) {
        char *row = (char *)marker + (size_t)y * pitch_marker;
        if (dtype == IWPP_SYNTH_I32)
            for (int x = 0; x < W; ++x) ((int32_t *)row)[x] = INT32_MIN;
        else
            memset(row, 0, (size_t)W * bpp_of(dtype));
    }
    int64_t n = (int64_t)llround(fraction * (double)W * (double)H);
    if (n < 1) n = 1;
    mt64_t rng;
    mt64_seed(&rng, seed ^ 0x5EED5EED5EED5EEDULL);
    for (int64_t i = 0; i < n; ++i) {
        int x = (int)mt64_range(&rng, 0, W - 1), y = (int)mt64_range(&rng, 0, H - 1);
        set_px(marker, pitch_marker, dtype, x, y, get_px(mask, pitch_mask, dtype, x, y));
    }
    return 0;
}

/* Square spiral corridor, one pixel wide, drawn inward and clockwise: right
 * along the top row, down the right column, left along the bottom row, up the
 * left column, then the next turn inside, adjacent parallel arms `arm_pitch`
 * pixels apart.  Starts at (arm_pitch/2, arm_pitch/2).  Returns the number of
 * corridor pixels (all set to the dtype's maximum). */
int64_t iwpp_synth_spiral_corridor(void *mask, int W, int H, size_t pitch, int dtype, int arm_pitch, int *start_x,
                                   int *start_y) {
    int64_t lo, hi, count = 0;
    type_range(dtype, &lo, &hi);
    int p = arm_pitch < 2 ? 2 : arm_pitch;
    int l = p / 2, r = W - 1 - p / 2, t = p / 2, b = H - 1 - p / 2;
    if (start_x) *start_x = l;
    if (start_y) *start_y = t;
    if (l > r || t > b) return 0;
    int x = l, y = t;
    set_px(mask, pitch, dtype, x, y, hi);
    ++count;
    for (;;) {
        if (r <= x) break; /* right along row y to column r */
        for (int i = x + 1; i <= r; ++i) set_px(mask, pitch, dtype, i, y, hi), ++count;
        x = r;
        t += p;
        if (b <= y) break; /* down column x to row b */
        for (int i = y + 1; i <= b; ++i) set_px(mask, pitch, dtype, x, i, hi), ++count;
        y = b;
        r -= p;
        if (x <= l) break; /* left along row y to column l */
        for (int i = x - 1; i >= l; --i) set_px(mask, pitch, dtype, i, y, hi), ++count;
        x = l;
        b -= p;
        if (y <= t) break; /* up column x to row t */
        for (int i = y - 1; i >= t; --i) set_px(mask, pitch, dtype, x, i, hi), ++count;
        y = t;
        l += p;
    }
    return count;
}

int iwpp_synth_seed_marker(void *marker, const void *mask, int W, int H, size_t pitch_marker, size_t pitch_mask,
                           int dtype, uint64_t seed, int nseeds, int first_x, int first_y) {
    if (!marker || !mask || W <= 0 || H <= 0) return 1;
    for (int y = 0; y < H; ++y) {
        char *row = (char *)marker + (size_t)y * pitch_marker;
        if (dtype == IWPP_SYNTH_I32)
            for (int x = 0; x < W; ++x) ((int32_t *)row)[x] = INT32_MIN;
        else
            memset(row, 0, (size_t)W * bpp_of(dtype));
    }
    mt64_t rng;
    mt64_seed(&rng, seed ^ 0xA5A5A5A5DEADBEEFULL);
    for (int i = 0; i < nseeds; ++i) {
        int x, y;
        if (i == 0 && first_x >= 0 && first_y >= 0) {
            x = first_x;
            y = first_y;
        } else {
            x = (int)mt64_range(&rng, 0, W - 1);
            y = (int)mt64_range(&rng, 0, H - 1);
        }
        set_px(marker, pitch_marker, dtype, x, y, get_px(mask, pitch_mask, dtype, x, y));
    }
    return 0;
}

int iwpp_synth_uniform_pair(void *marker, void *mask, int W, int H, size_t pitch_marker, size_t pitch_mask,
                            uint64_t seed) {
    if (!marker || !mask || W <= 0 || H <= 0) return 1;
    for (int y = 0; y < H; ++y) {
        uint8_t *mrow = (uint8_t *)marker + (size_t)y * pitch_marker;
        uint8_t *krow = (uint8_t *)mask + (size_t)y * pitch_mask;
        for (int x = 0; x < W; ++x) {
            uint64_t idx = ((uint64_t)y * (uint64_t)W + (uint64_t)x) * 2ULL;
            unsigned mv = (unsigned)(hash2(seed, idx) % 256ULL);
            unsigned kv = (unsigned)(hash2(seed, idx + 1) % 256ULL);
            kv = kv % (255U - mv + 1U);
            mrow[x] = (uint8_t)mv;
            krow[x] = (uint8_t)(mv + kv);
        }
    }
    return 0;
}

int iwpp_synth_version(void) { return 1; }
