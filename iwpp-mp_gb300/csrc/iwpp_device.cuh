// iwpp_device.cuh -- device building blocks of the GB300 reconstruction
// engine: one-warp tile visits (TMA fetch with halo, raster / anti-raster
// sweeps to local convergence, write-back, neighbour detection).
//
// Layout: a tile is TH rows x TW pixels with TW * sizeof(pixel) = 128 bytes
// (TW = 128 uint8, 64 uint16, 32 int32).  One warp owns one tile at a time.
// Shared memory holds the tile plus the halo rows above and below as dense
// 128-byte rows (SMEM row r = image row y0 - 1 + r), so one TMA box load per
// image plane fetches it.  Lane L owns the 32-bit word with pixels
// [L*PPW, L*PPW + PPW) of every row (PPW = 4 / 2 / 1); during a row step it
// unpacks them to one pixel per register so every min / max is a native
// 32-bit instruction.  Vertical propagation runs row by row; horizontal
// propagation is a warp scan over the max-min semiring.
//
// Reference counterparts (IWPP MP/src/MorphologicalReconstruction.cu):
//   tile fetch with a one-pixel halo        MR.cu:232-312
//   in-tile directional sweeps to stability MR.cu:34-161, loop MR.cu:320-325
//   write-back + neighbour detection        MR.cu:335-512
// The rule everywhere is MR.cu:43-44: m[c] = max(m[c], min(m[p], mask[c])).
#pragma once

#include <cstdint>
#include <cuda_runtime.h>

namespace iwpp {

constexpr unsigned FULL = 0xffffffffu;

enum : int { DT_U8 = 0, DT_U16 = 1, DT_I32 = 2 };

// ------------------------------------------------------------------ pixels
// Pixels are carried as uint32 (zero-extended for the unsigned types, the
// bit pattern for int32); Px<DT> supplies the order and the packing.
template <int DT>
struct Px;

template <>
struct Px<DT_U8> {
    static constexpr int PPW = 4;
    static constexpr int BPP = 1;
    static constexpr uint32_t MINPX = 0u;
    static constexpr uint32_t MINW = 0u;
    static constexpr uint32_t FIRST_MASK = 0x000000ffu, LAST_MASK = 0xff000000u;
    __device__ static __forceinline__ uint32_t mx(uint32_t a, uint32_t b) { return max(a, b); }
    __device__ static __forceinline__ uint32_t mn(uint32_t a, uint32_t b) { return min(a, b); }
    __device__ static __forceinline__ uint32_t mx3(uint32_t a, uint32_t b, uint32_t c) { return __vimax3_u32(a, b, c); }
    __device__ static __forceinline__ bool gt(uint32_t a, uint32_t b) { return a > b; }
    __device__ static __forceinline__ void unpack(uint32_t w, uint32_t (&p)[4]) {
        p[0] = __byte_perm(w, 0u, 0x4440);
        p[1] = __byte_perm(w, 0u, 0x4441);
        p[2] = __byte_perm(w, 0u, 0x4442);
        p[3] = __byte_perm(w, 0u, 0x4443);
    }
    __device__ static __forceinline__ uint32_t pack(const uint32_t (&p)[4]) {
        const uint32_t lo = __byte_perm(p[0], p[1], 0x0040);
        const uint32_t hi = __byte_perm(p[2], p[3], 0x0040);
        return __byte_perm(lo, hi, 0x5410);
    }
    __device__ static __forceinline__ uint32_t ld_px(const unsigned char* p) { return *p; }
    __device__ static __forceinline__ uint32_t ld_px_cg(const unsigned char* p) { return __ldcg(p); }
    __device__ static __forceinline__ void st_px(unsigned char* p, uint32_t v) { *p = (unsigned char)v; }
};

template <>
struct Px<DT_U16> {
    static constexpr int PPW = 2;
    static constexpr int BPP = 2;
    static constexpr uint32_t MINPX = 0u;
    static constexpr uint32_t MINW = 0u;
    static constexpr uint32_t FIRST_MASK = 0x0000ffffu, LAST_MASK = 0xffff0000u;
    __device__ static __forceinline__ uint32_t mx(uint32_t a, uint32_t b) { return max(a, b); }
    __device__ static __forceinline__ uint32_t mn(uint32_t a, uint32_t b) { return min(a, b); }
    __device__ static __forceinline__ uint32_t mx3(uint32_t a, uint32_t b, uint32_t c) { return __vimax3_u32(a, b, c); }
    __device__ static __forceinline__ bool gt(uint32_t a, uint32_t b) { return a > b; }
    __device__ static __forceinline__ void unpack(uint32_t w, uint32_t (&p)[2]) {
        p[0] = w & 0xffffu;
        p[1] = w >> 16;
    }
    __device__ static __forceinline__ uint32_t pack(const uint32_t (&p)[2]) { return __byte_perm(p[0], p[1], 0x5410); }
    __device__ static __forceinline__ uint32_t ld_px(const unsigned char* p) {
        return *reinterpret_cast<const unsigned short*>(p);
    }
    __device__ static __forceinline__ uint32_t ld_px_cg(const unsigned char* p) {
        return __ldcg(reinterpret_cast<const unsigned short*>(p));
    }
    __device__ static __forceinline__ void st_px(unsigned char* p, uint32_t v) {
        *reinterpret_cast<unsigned short*>(p) = (unsigned short)v;
    }
};

template <>
struct Px<DT_I32> {
    static constexpr int PPW = 1;
    static constexpr int BPP = 4;
    static constexpr uint32_t MINPX = 0x80000000u;
    static constexpr uint32_t MINW = 0x80000000u;
    static constexpr uint32_t FIRST_MASK = 0xffffffffu, LAST_MASK = 0xffffffffu;
    __device__ static __forceinline__ uint32_t mx(uint32_t a, uint32_t b) { return (uint32_t)max((int)a, (int)b); }
    __device__ static __forceinline__ uint32_t mn(uint32_t a, uint32_t b) { return (uint32_t)min((int)a, (int)b); }
    __device__ static __forceinline__ uint32_t mx3(uint32_t a, uint32_t b, uint32_t c) {
        return (uint32_t)__vimax3_s32((int)a, (int)b, (int)c);
    }
    __device__ static __forceinline__ bool gt(uint32_t a, uint32_t b) { return (int)a > (int)b; }
    __device__ static __forceinline__ void unpack(uint32_t w, uint32_t (&p)[1]) { p[0] = w; }
    __device__ static __forceinline__ uint32_t pack(const uint32_t (&p)[1]) { return p[0]; }
    __device__ static __forceinline__ uint32_t ld_px(const unsigned char* p) {
        return (uint32_t)*reinterpret_cast<const int*>(p);
    }
    __device__ static __forceinline__ uint32_t ld_px_cg(const unsigned char* p) {
        return (uint32_t)__ldcg(reinterpret_cast<const int*>(p));
    }
    __device__ static __forceinline__ void st_px(unsigned char* p, uint32_t v) { *reinterpret_cast<int*>(p) = (int)v; }
};

// ------------------------------------------------------------ image / tiles
// One image of a (possibly single-image) job.  Pitches are in bytes.
struct ImgDesc {
    unsigned char* marker;
    const unsigned char* mask;
    long long pitch_m;
    long long pitch_k;
    const void* tmaps;  // two CUtensorMap (marker, mask) or nullptr (plain loads)
    int W, H;
    int dtype, conn;
    int tiles_x, tiles_y;
    int tile_base;  // first global tile index of this image
    int tile_rows;  // TH used for this image
    // Nullable.  The front-stage kernels (top-level labelling, whole-image
    // passes, seed check) over this image return at once while *gate is 0:
    // the job decided on the device to leave the image to the tile engine.
    const unsigned* gate;
};

__device__ __forceinline__ bool gated_off(const ImgDesc& d) {
    return d.gate != nullptr && *(const volatile unsigned*)d.gate == 0u;
}

// neighbour direction bits returned by a tile visit
enum : unsigned {
    NB_N = 1u << 0, NB_S = 1u << 1, NB_W = 1u << 2, NB_E = 1u << 3,
    NB_NW = 1u << 4, NB_NE = 1u << 5, NB_SW = 1u << 6, NB_SE = 1u << 7
};
__device__ __constant__ static const int kNbDx[8] = {0, 0, -1, 1, -1, 1, -1, 1};
__device__ __constant__ static const int kNbDy[8] = {-1, 1, 0, 0, -1, -1, 1, 1};

// Per-warp shared memory (128-byte aligned; TMA writes tm / tk densely).
// SMEM row r holds image row y0 - 1 + r: row 0 is the halo above the tile,
// rows 1..TH the tile, row TH+1 the halo below.  hL* / hR* hold the left /
// right halo column pixels of the same rows.
constexpr int kPqCap = 448;  // pixel-queue solver: FIFO entries per warp
template <int TH>
struct __align__(128) WarpSmem {
    uint32_t tm[(TH + 2) * 32];
    uint32_t tk[(TH + 2) * 32];
    uint32_t hLm[TH + 2];
    uint32_t hLk[TH + 2];
    uint32_t hRm[TH + 2];
    uint32_t hRk[TH + 2];
    unsigned long long mbar;
    unsigned short pq[kPqCap];  // pixel-queue solver: tile pixel indices r * TW + c
};

// ------------------------------------------------------- async-copy helpers
__device__ __forceinline__ uint32_t smem_u32(const void* p) {
    return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}

__device__ __forceinline__ void mbar_init(unsigned long long* bar, unsigned count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count) : "memory");
}

__device__ __forceinline__ void mbar_arrive_expect_tx(unsigned long long* bar, unsigned bytes) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)), "r"(bytes)
                 : "memory");
}

__device__ __forceinline__ bool mbar_try_wait(unsigned long long* bar, unsigned parity) {
    uint32_t ok;
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
        "selp.u32 %0, 1, 0, p;\n\t}"
        : "=r"(ok)
        : "r"(smem_u32(bar)), "r"(parity)
        : "memory");
    return ok != 0u;
}

// 2-D TMA box load: box origin (x bytes, y rows) of the tensor map into smem.
__device__ __forceinline__ void tma_load_2d(void* smem_dst, const void* tmap, int x, int y,
                                            unsigned long long* bar) {
    asm volatile(
        "cp.async.bulk.tensor.2d.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3}], [%4];" ::
            "r"(smem_u32(smem_dst)),
        "l"(tmap), "r"(x), "r"(y), "r"(smem_u32(bar))
        : "memory");
}

__device__ __forceinline__ void fence_proxy_async_smem() { asm volatile("fence.proxy.async.shared::cta;" ::: "memory"); }
__device__ __forceinline__ void fence_proxy_async_global() { asm volatile("fence.proxy.async.global;" ::: "memory"); }

// Global-memory flag accesses with acquire / release ordering at GPU scope.
__device__ __forceinline__ unsigned ld_acquire(const unsigned* p) {
    unsigned v;
    asm volatile("ld.acquire.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
    return v;
}
__device__ __forceinline__ void st_release(unsigned* p, unsigned v) {
    asm volatile("st.release.gpu.global.u32 [%0], %1;" ::"l"(p), "r"(v) : "memory");
}

__device__ __forceinline__ long long globaltimer_ns() {
    long long t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    return t;
}

// ------------------------------------------------ packed-word min / max
// Per-pixel max / min of two packed words (uint8: four bytes, uint16: two
// halves, int32: one signed value), and whether some pixel of a is above
// the same pixel of b.
template <int DT>
__device__ __forceinline__ uint32_t word_max(uint32_t a, uint32_t b) {
    if (DT == DT_U8) return __vmaxu4(a, b);
    if (DT == DT_U16) return __vmaxu2(a, b);
    return (uint32_t)max((int)a, (int)b);
}
template <int DT>
__device__ __forceinline__ uint32_t word_min(uint32_t a, uint32_t b) {
    if (DT == DT_U8) return __vminu4(a, b);
    if (DT == DT_U16) return __vminu2(a, b);
    return (uint32_t)min((int)a, (int)b);
}
template <int DT>
__device__ __forceinline__ bool word_any_gt(uint32_t a, uint32_t b) {
    if (DT == DT_U8) return __vcmpgtu4(a, b) != 0u;
    if (DT == DT_U16) return __vcmpgtu2(a, b) != 0u;
    return (int)a > (int)b;
}

// ------------------------------------------------ clamp-map scan steps
// Carrying a value x through a run of pixels along the scan direction maps
// it to max(min(x, B), A) (B: the run's least mask, A: the run's last pixel
// without a carry).  One step of the warp's inclusive scan composes a lane's
// map after the map of the lanes d before it:
//   A = max(min(A_prev, B), A),  B = min(B_prev, B).
// A lane with no source at distance d reads its own map back, and a clamp
// map composed with itself is itself, so no lane predicate is needed.
// uint8 / uint16: (A, B) share one word, A in the low half, and a step is
// one shuffle, one 16x2 min and one 16x2 max on the critical path.
template <bool FWD>
__device__ __forceinline__ uint32_t map_step_packed(uint32_t cur, int d) {
    const uint32_t prev = FWD ? __shfl_up_sync(FULL, cur, d) : __shfl_down_sync(FULL, cur, d);
    return __vmaxu2(__vminu2(prev, __byte_perm(cur, 0u, 0x3232)), cur & 0xffffu);
}
// int32: A and B in two words, signed order.
template <bool FWD>
__device__ __forceinline__ void map_step_i32(uint32_t& A, uint32_t& B, int d) {
    const int Ap = FWD ? __shfl_up_sync(FULL, (int)A, d) : __shfl_down_sync(FULL, (int)A, d);
    const int Bp = FWD ? __shfl_up_sync(FULL, (int)B, d) : __shfl_down_sync(FULL, (int)B, d);
    A = (uint32_t)max(min(Ap, (int)B), (int)A);
    B = (uint32_t)min(Bp, (int)B);
}

// ---------------------------------------------------- horizontal warp scan
// Propagates along one row in scan order (FWD: left to right) with `cin` the
// marker value of the halo pixel entering the row at the first lane.  The
// transfer function of a word for the value x entering it is
// f(x) = max(min(x, B), A) with B = min of its mask pixels and A = its exit
// pixel after the in-word pass; these compose associatively:
// (A2,B2) o (A1,B1) = (max(min(A1, B2), A2), min(B1, B2)).
// N: pixels per lane (one 32-bit word by default; the 16-byte-lane sweeps
// hold four words).
template <int DT, bool FWD, int N = Px<DT>::PPW>
__device__ __forceinline__ void hscan(uint32_t (&m)[N], const uint32_t (&k)[N], uint32_t cin, int lane) {
    using P = Px<DT>;
#pragma unroll
    for (int s = 1; s < N; ++s) {
        const int j = FWD ? s : N - 1 - s;
        const int jp = FWD ? j - 1 : j + 1;
        m[j] = P::mx(m[j], P::mn(m[jp], k[j]));
    }
    const int first = FWD ? 0 : N - 1, last = FWD ? N - 1 : 0;
    const int edge_lane = FWD ? 0 : 31;
    uint32_t in_px = FWD ? __shfl_up_sync(FULL, m[last], 1) : __shfl_down_sync(FULL, m[last], 1);
    if (lane == edge_lane) in_px = cin;
    // A carry that does not raise a word's entry pixel raises nothing after it.
    const bool need = P::gt(P::mn(in_px, k[first]), m[first]);
    if (!__any_sync(FULL, need)) return;

    uint32_t A = m[last], B = k[0];
#pragma unroll
    for (int j = 1; j < N; ++j) B = P::mn(B, k[j]);
    if (lane == edge_lane) {
        A = P::mx(A, P::mn(cin, B));
        B = P::MINPX;  // the entry lane becomes a constant: nothing before it
    }
    if (DT == DT_I32) {
#pragma unroll
        for (int d = 1; d < 32; d <<= 1) map_step_i32<FWD>(A, B, d);
    } else {
        uint32_t cur = A | (B << 16);
#pragma unroll
        for (int d = 1; d < 32; d <<= 1) cur = map_step_packed<FWD>(cur, d);
        A = cur & 0xffffu;
    }
    uint32_t c = FWD ? __shfl_up_sync(FULL, A, 1) : __shfl_down_sync(FULL, A, 1);
    if (lane == edge_lane) c = cin;
#pragma unroll
    for (int s = 0; s < N; ++s) {
        const int j = FWD ? s : N - 1 - s;
        c = P::mn(c, k[j]);
        m[j] = P::mx(m[j], c);
    }
}

// ------------------------------------------------------------- one sweep
// DOWN = raster order (rows top to bottom, each row left to right),
// otherwise anti-raster.  After a complete raster sweep every pixel satisfies
// its constraints towards N+ = {left, up-left, up, up-right}; after an
// anti-raster sweep towards N-.
//
// Rows are skipped when nothing they depend on can have changed since they
// last satisfied this sweep's constraints: a row is processed when the row
// before it (in sweep order) rose in this sweep, or when it or a vertical
// neighbour rose in the previous sweep (`dil`, already dilated by one row),
// or when its halo inputs are new (`force`, folded into `dil` by the caller).
// `chg` receives the rows that rose (bit r-1 for SMEM row r).
template <int DT, int CONN, int TH, bool DOWN>
__device__ __forceinline__ void sweep(WarpSmem<TH>& sm, int lane, unsigned long long dil, unsigned long long& chg,
                                      bool& col_changed, uint32_t edge_mask, unsigned& row_steps) {
    using P = Px<DT>;
    constexpr int N = P::PPW;
    uint32_t prev[N];
    bool prev_valid = false, prev_changed = false;
    // the row words of step i are read during step i - 1 (only step i
    // writes its row), so their shared-memory latency overlaps a scan
    uint32_t next_m = sm.tm[(DOWN ? 1 : TH) * 32 + lane], next_k = sm.tk[(DOWN ? 1 : TH) * 32 + lane];
#pragma unroll 1
    for (int i = 0; i < TH; ++i) {
        const int r = DOWN ? 1 + i : TH - i;  // SMEM row
        const int rp = DOWN ? r - 1 : r + 1;  // SMEM row before it in sweep order
        const uint32_t old = next_m, kw = next_k;
        if (i + 1 < TH) {
            const int rn = DOWN ? r + 1 : r - 1;
            next_m = sm.tm[rn * 32 + lane];
            next_k = sm.tk[rn * 32 + lane];
        }
        if (!prev_changed && !((dil >> (r - 1)) & 1ull)) {
            prev_valid = false;
            continue;
        }
        if (!prev_valid) P::unpack(sm.tm[rp * 32 + lane], prev);
        ++row_steps;
        uint32_t m[N], k[N];
        P::unpack(old, m);
        P::unpack(kw, k);
        if (CONN == 8) {
            uint32_t left = __shfl_up_sync(FULL, prev[N - 1], 1);
            uint32_t right = __shfl_down_sync(FULL, prev[0], 1);
            if (lane == 0) left = sm.hLm[rp];
            if (lane == 31) right = sm.hRm[rp];
            if (N == 1) {
                m[0] = P::mx(m[0], P::mn(P::mx3(left, prev[0], right), k[0]));
            } else {
                // shared pairwise maxima of the previous row
                uint32_t pair[N > 1 ? N - 1 : 1];
#pragma unroll
                for (int j = 0; j + 1 < N; ++j) pair[j] = P::mx(prev[j], prev[j + 1]);
#pragma unroll
                for (int j = 0; j < N; ++j) {
                    const uint32_t v = j == 0 ? P::mx(left, pair[0]) : j == N - 1 ? P::mx(pair[N - 2], right)
                                                                                   : P::mx(prev[j - 1], pair[j]);
                    m[j] = P::mx(m[j], P::mn(v, k[j]));
                }
            }
        } else {
#pragma unroll
            for (int j = 0; j < N; ++j) m[j] = P::mx(m[j], P::mn(prev[j], k[j]));
        }
        hscan<DT, DOWN>(m, k, DOWN ? sm.hLm[r] : sm.hRm[r], lane);
        const uint32_t nw = P::pack(m);
        prev_changed = __any_sync(FULL, nw != old);
        if (prev_changed) {
            sm.tm[r * 32 + lane] = nw;
            chg |= 1ull << (r - 1);
            col_changed |= ((nw ^ old) & edge_mask) != 0u;
        }
#pragma unroll
        for (int j = 0; j < N; ++j) prev[j] = m[j];
        prev_valid = true;
    }
    __syncwarp();
}

// ------------------------------------------------------- in-tile passes
// The tile converges through three kinds of pass, the separable form of the
// reference's XForward / XBackward / YDownward / YUpward propagation
// (MR.cu:34-161):
//   vertical down / up: each lane walks its own columns over the rows, one
//     row per step, taking the row before it (8-connectivity: its three
//     upper / lower neighbours, the outer two through one shuffle each);
//     no vote or scan per row, so a row costs a few dependent operations;
//   horizontal: rows are independent, each gets a forward and a backward
//     max-min scan across the warp (hscan); four rows are scanned together
//     so their shuffle latencies overlap.
// Rows are numbered as in shared memory (1..TH); masks use bit r-1.

// OR of a per-lane 64-bit mask over the warp.
__device__ __forceinline__ unsigned long long warp_or64(unsigned long long v) {
    const unsigned lo = __reduce_or_sync(FULL, (unsigned)v);
    const unsigned hi = __reduce_or_sync(FULL, (unsigned)(v >> 32));
    return ((unsigned long long)hi << 32) | lo;
}

// Vertical pass, downward (rows in increasing order) or upward, from the
// first row of `dirty` (rows whose constraint towards the row before them,
// in pass order, may be violated) to the tile's far edge.  It does not stop
// where the rows stop rising: a vote there costs more latency on long
// fronts than the rows it would save.  Returns the rows that rose
// (warp-uniform); `col_now` (per lane) records a rise in the tile's first /
// last pixel column; `steps` counts the rows processed.
template <int DT, int CONN, int TH, bool DOWN>
__device__ __forceinline__ unsigned long long vpass(WarpSmem<TH>& sm, int lane, unsigned long long dirty,
                                                    uint32_t edge_mask, bool& col_now, unsigned& steps) {
    using P = Px<DT>;
    constexpr int N = P::PPW;
    const int first = DOWN ? __ffsll((long long)dirty) : 64 - __clzll((long long)dirty);
    const int count = DOWN ? TH - first + 1 : first;
    steps += (unsigned)count;
    unsigned long long chg = 0ull;
    uint32_t diff = 0u;
    if (CONN == 4) {
        // columns are independent: packed min / max per word and row; uint8
        // words run as two u16x2 chains (even and odd bytes), whose min / max
        // are single instructions, so the chain is two of them per row
        const uint32_t first_prev = sm.tm[(DOWN ? first - 1 : first + 1) * 32 + lane];
        uint32_t plo = first_prev & 0x00ff00ffu, phi = (first_prev >> 8) & 0x00ff00ffu, prevw = first_prev;
#pragma unroll 4
        for (int i = 0; i < count; ++i) {
            const int r = DOWN ? first + i : first - i;
            const uint32_t old = sm.tm[r * 32 + lane];
            const uint32_t kw = sm.tk[r * 32 + lane];
            uint32_t nw;
            if (DT == DT_U8) {
                plo = __vmaxu2(old & 0x00ff00ffu, __vminu2(plo, kw & 0x00ff00ffu));
                phi = __vmaxu2((old >> 8) & 0x00ff00ffu, __vminu2(phi, (kw >> 8) & 0x00ff00ffu));
                nw = plo | (phi << 8);
            } else {
                nw = word_max<DT>(old, word_min<DT>(prevw, kw));
                prevw = nw;
            }
            sm.tm[r * 32 + lane] = nw;
            const uint32_t x = nw ^ old;
            diff |= x;
            if (x != 0u) chg |= 1ull << (r - 1);
        }
        col_now |= (diff & edge_mask) != 0u;
        __syncwarp();
        return warp_or64(chg);
    }
    if (CONN == 8 && DT != DT_I32) {
        // packed 8-connected rows: the previous row's three-pixel maximum
        // from the word itself and the words 16 bits to either side, built
        // by funnel shifts from the neighbour lanes' words (the tile's halo
        // columns at lanes 0 / 31).  uint16 words are u16x2 as they are;
        // uint8 words run as their even (lo) and odd (hi) bytes, where the
        // even bytes' neighbours are the odd half and the odd half shifted
        // in from the left, the odd bytes' the even half and the even half
        // shifted in from the right.
        constexpr uint32_t E = 0x00ff00ffu;
        const uint32_t first_prev = sm.tm[(DOWN ? first - 1 : first + 1) * 32 + lane];
        uint32_t plo = DT == DT_U8 ? first_prev & E : first_prev;
        uint32_t phi = (first_prev >> 8) & E;
#pragma unroll 4
        for (int i = 0; i < count; ++i) {
            const int r = DOWN ? first + i : first - i;
            const int rp = DOWN ? r - 1 : r + 1;
            const uint32_t old = sm.tm[r * 32 + lane];
            const uint32_t kw = sm.tk[r * 32 + lane];
            uint32_t nw;
            if (DT == DT_U8) {
                uint32_t left = __shfl_up_sync(FULL, phi, 1), right = __shfl_down_sync(FULL, plo, 1);
                if (lane == 0) left = sm.hLm[rp] << 16;
                if (lane == 31) right = sm.hRm[rp];
                const uint32_t dlo = __vimax3_u16x2(plo, phi, __funnelshift_l(left, phi, 16));
                const uint32_t dhi = __vimax3_u16x2(phi, plo, __funnelshift_r(plo, right, 16));
                plo = __vmaxu2(old & E, __vminu2(dlo, kw & E));
                phi = __vmaxu2((old >> 8) & E, __vminu2(dhi, (kw >> 8) & E));
                nw = plo | (phi << 8);
            } else {
                uint32_t left = __shfl_up_sync(FULL, plo, 1), right = __shfl_down_sync(FULL, plo, 1);
                if (lane == 0) left = sm.hLm[rp] << 16;
                if (lane == 31) right = sm.hRm[rp];
                const uint32_t dil =
                    __vimax3_u16x2(plo, __funnelshift_l(left, plo, 16), __funnelshift_r(plo, right, 16));
                nw = __vmaxu2(old, __vminu2(dil, kw));
                plo = nw;
            }
            sm.tm[r * 32 + lane] = nw;
            const uint32_t x = nw ^ old;
            diff |= x;
            if (x != 0u) chg |= 1ull << (r - 1);
        }
        col_now |= (diff & edge_mask) != 0u;
        __syncwarp();
        return warp_or64(chg);
    }
    uint32_t prev[N];
    P::unpack(sm.tm[(DOWN ? first - 1 : first + 1) * 32 + lane], prev);
#pragma unroll 4
    for (int i = 0; i < count; ++i) {
        const int r = DOWN ? first + i : first - i;
        const int rp = DOWN ? r - 1 : r + 1;
        const uint32_t old = sm.tm[r * 32 + lane];
        uint32_t m[N], k[N];
        P::unpack(old, m);
        P::unpack(sm.tk[r * 32 + lane], k);
        if (CONN == 8) {
            uint32_t left = __shfl_up_sync(FULL, prev[N - 1], 1);
            uint32_t right = __shfl_down_sync(FULL, prev[0], 1);
            if (lane == 0) left = sm.hLm[rp];
            if (lane == 31) right = sm.hRm[rp];
            if (N == 1) {
                m[0] = P::mx(m[0], P::mn(P::mx3(left, prev[0], right), k[0]));
            } else {
#pragma unroll
                for (int j = 0; j < N; ++j) {
                    const uint32_t a = j == 0 ? left : prev[j - 1];
                    const uint32_t c = j == N - 1 ? right : prev[j + 1];
                    m[j] = P::mx(m[j], P::mn(P::mx3(a, prev[j], c), k[j]));
                }
            }
        } else {
#pragma unroll
            for (int j = 0; j < N; ++j) m[j] = P::mx(m[j], P::mn(prev[j], k[j]));
        }
        const uint32_t nw = P::pack(m);
        sm.tm[r * 32 + lane] = nw;
        const uint32_t x = nw ^ old;
        diff |= x;
        if (x != 0u) chg |= 1ull << (r - 1);
#pragma unroll
        for (int j = 0; j < N; ++j) prev[j] = m[j];
    }
    col_now |= (diff & edge_mask) != 0u;
    __syncwarp();
    return warp_or64(chg);
}

// R independent rows scanned together in one direction (see hscan).
template <int DT, bool FWD, int R>
__device__ __forceinline__ void hscan_rows(uint32_t (&m)[R][Px<DT>::PPW], const uint32_t (&k)[R][Px<DT>::PPW],
                                           const uint32_t (&cin)[R], int lane) {
    using P = Px<DT>;
    constexpr int N = P::PPW;
    const int first = FWD ? 0 : N - 1, last = FWD ? N - 1 : 0;
    const int edge_lane = FWD ? 0 : 31;
    bool need = false;
#pragma unroll
    for (int q = 0; q < R; ++q) {
#pragma unroll
        for (int s = 1; s < N; ++s) {
            const int j = FWD ? s : N - 1 - s;
            const int jp = FWD ? j - 1 : j + 1;
            m[q][j] = P::mx(m[q][j], P::mn(m[q][jp], k[q][j]));
        }
        uint32_t in_px = FWD ? __shfl_up_sync(FULL, m[q][last], 1) : __shfl_down_sync(FULL, m[q][last], 1);
        if (lane == edge_lane) in_px = cin[q];
        need |= P::gt(P::mn(in_px, k[q][first]), m[q][first]);
    }
    // A carry that does not raise a word's entry pixel raises nothing after
    // it; rows that need no scan come out of it unchanged.
    if (!__any_sync(FULL, need)) return;
    uint32_t A[R], B[R];
#pragma unroll
    for (int q = 0; q < R; ++q) {
        A[q] = m[q][last];
        B[q] = k[q][0];
#pragma unroll
        for (int j = 1; j < N; ++j) B[q] = P::mn(B[q], k[q][j]);
        if (lane == edge_lane) {
            A[q] = P::mx(A[q], P::mn(cin[q], B[q]));
            B[q] = P::MINPX;  // the entry lane becomes a constant: nothing before it
        }
    }
    if (DT == DT_I32) {
#pragma unroll
        for (int d = 1; d < 32; d <<= 1)
#pragma unroll
            for (int q = 0; q < R; ++q) map_step_i32<FWD>(A[q], B[q], d);
    } else {
        uint32_t cur[R];
#pragma unroll
        for (int q = 0; q < R; ++q) cur[q] = A[q] | (B[q] << 16);
#pragma unroll
        for (int d = 1; d < 32; d <<= 1)
#pragma unroll
            for (int q = 0; q < R; ++q) cur[q] = map_step_packed<FWD>(cur[q], d);
#pragma unroll
        for (int q = 0; q < R; ++q) A[q] = cur[q] & 0xffffu;
    }
#pragma unroll
    for (int q = 0; q < R; ++q) {
        uint32_t c = FWD ? __shfl_up_sync(FULL, A[q], 1) : __shfl_down_sync(FULL, A[q], 1);
        if (lane == edge_lane) c = cin[q];
#pragma unroll
        for (int s = 0; s < N; ++s) {
            const int j = FWD ? s : N - 1 - s;
            c = P::mn(c, k[q][j]);
            m[q][j] = P::mx(m[q][j], c);
        }
    }
}

// Q pairs of rows scanned together in one direction, uint8 / uint16: pixel
// j of a pair's two rows shares one word as u16x2 (first row low), so every
// min / max, and each step of the clamp-map scan (A and B in a word each),
// serves two rows at once.  The algebra is hscan's, element-wise.
template <bool FWD, int Q, int N>
__device__ __forceinline__ void hscan_pairs(uint32_t (&m)[Q][N], const uint32_t (&k)[Q][N], const uint32_t (&cin)[Q],
                                            int lane) {
    const int first = FWD ? 0 : N - 1, last = FWD ? N - 1 : 0;
    const int edge_lane = FWD ? 0 : 31;
    bool need = false;
#pragma unroll
    for (int q = 0; q < Q; ++q) {
#pragma unroll
        for (int s = 1; s < N; ++s) {
            const int j = FWD ? s : N - 1 - s;
            const int jp = FWD ? j - 1 : j + 1;
            m[q][j] = __vmaxu2(m[q][j], __vminu2(m[q][jp], k[q][j]));
        }
        uint32_t in_px = FWD ? __shfl_up_sync(FULL, m[q][last], 1) : __shfl_down_sync(FULL, m[q][last], 1);
        if (lane == edge_lane) in_px = cin[q];
        need |= __vcmpgtu2(__vminu2(in_px, k[q][first]), m[q][first]) != 0u;
    }
    if (!__any_sync(FULL, need)) return;
    uint32_t A[Q], B[Q];
#pragma unroll
    for (int q = 0; q < Q; ++q) {
        A[q] = m[q][last];
        B[q] = k[q][0];
#pragma unroll
        for (int j = 1; j < N; ++j) B[q] = __vminu2(B[q], k[q][j]);
        if (lane == edge_lane) {
            A[q] = __vmaxu2(A[q], __vminu2(cin[q], B[q]));
            B[q] = 0u;  // the entry lane becomes a constant: nothing before it
        }
    }
#pragma unroll
    for (int d = 1; d < 32; d <<= 1)
#pragma unroll
        for (int q = 0; q < Q; ++q) {
            const uint32_t Ap = FWD ? __shfl_up_sync(FULL, A[q], d) : __shfl_down_sync(FULL, A[q], d);
            const uint32_t Bp = FWD ? __shfl_up_sync(FULL, B[q], d) : __shfl_down_sync(FULL, B[q], d);
            A[q] = __vmaxu2(__vminu2(Ap, B[q]), A[q]);
            B[q] = __vminu2(Bp, B[q]);
        }
#pragma unroll
    for (int q = 0; q < Q; ++q) {
        uint32_t c = FWD ? __shfl_up_sync(FULL, A[q], 1) : __shfl_down_sync(FULL, A[q], 1);
        if (lane == edge_lane) c = cin[q];
#pragma unroll
        for (int s = 0; s < N; ++s) {
            const int j = FWD ? s : N - 1 - s;
            c = __vminu2(c, k[q][j]);
            m[q][j] = __vmaxu2(m[q][j], c);
        }
    }
}

// Two row words (a: first row, b: second) as the pair words of hscan_pairs
// and back.  uint8: pixel j of both rows from the words' even / odd bytes;
// uint16: the words' low / high halves.
template <int DT>
__device__ __forceinline__ void pair_pack(uint32_t a, uint32_t b, uint32_t (&p)[Px<DT>::PPW]) {
    if constexpr (DT == DT_U8) {
        constexpr uint32_t E = 0x00ff00ffu;
        const uint32_t la = a & E, ha = (a >> 8) & E, lb = b & E, hb = (b >> 8) & E;
        p[0] = __byte_perm(la, lb, 0x5410);
        p[1] = __byte_perm(ha, hb, 0x5410);
        p[2] = __byte_perm(la, lb, 0x7632);
        p[3] = __byte_perm(ha, hb, 0x7632);
    } else {
        p[0] = __byte_perm(a, b, 0x5410);
        p[1] = __byte_perm(a, b, 0x7632);
    }
}
template <int DT>
__device__ __forceinline__ void pair_unpack(const uint32_t (&p)[Px<DT>::PPW], uint32_t& a, uint32_t& b) {
    if constexpr (DT == DT_U8) {
        const uint32_t t = __byte_perm(p[0], p[1], 0x6240), u = __byte_perm(p[2], p[3], 0x6240);
        a = __byte_perm(t, u, 0x5410);
        b = __byte_perm(t, u, 0x7632);
    } else {
        a = __byte_perm(p[0], p[1], 0x5410);
        b = __byte_perm(p[0], p[1], 0x7632);
    }
}

// Horizontal pass over the rows in `rows` (in blocks of eight as four row
// pairs for uint8 / uint16, of four for int32): forward then backward scan,
// which leaves each row at its one-dimensional fixed point.  `nrows` counts
// the rows of the blocks processed.
template <int DT, int TH>
__device__ __forceinline__ unsigned long long hpass(WarpSmem<TH>& sm, int lane, unsigned long long rows,
                                                    uint32_t edge_mask, bool& col_now, unsigned& nrows) {
    using P = Px<DT>;
    constexpr int N = P::PPW;
    unsigned long long chg = 0ull;
    uint32_t diff = 0u;
    if constexpr (DT != DT_I32) {
        constexpr int Q = 4, R = 2 * Q;
        static_assert(TH % R == 0, "tile rows: a multiple of 8");
#pragma unroll 1
        for (int b = 0; b < TH; b += R) {
            if (((rows >> b) & ((1ull << R) - 1ull)) == 0ull) continue;
            nrows += R;
            uint32_t m[Q][N], k[Q][N], olda[Q], oldb[Q], cin[Q];
#pragma unroll
            for (int q = 0; q < Q; ++q) {
                const int r = b + 2 * q + 1;
                olda[q] = sm.tm[r * 32 + lane];
                oldb[q] = sm.tm[(r + 1) * 32 + lane];
                pair_pack<DT>(olda[q], oldb[q], m[q]);
                pair_pack<DT>(sm.tk[r * 32 + lane], sm.tk[(r + 1) * 32 + lane], k[q]);
                cin[q] = sm.hLm[r] | (sm.hLm[r + 1] << 16);
            }
            hscan_pairs<true, Q, N>(m, k, cin, lane);
#pragma unroll
            for (int q = 0; q < Q; ++q) cin[q] = sm.hRm[b + 2 * q + 1] | (sm.hRm[b + 2 * q + 2] << 16);
            hscan_pairs<false, Q, N>(m, k, cin, lane);
#pragma unroll
            for (int q = 0; q < Q; ++q) {
                const int r = b + 2 * q + 1;
                uint32_t na, nb;
                pair_unpack<DT>(m[q], na, nb);
                sm.tm[r * 32 + lane] = na;
                sm.tm[(r + 1) * 32 + lane] = nb;
                const uint32_t xa = na ^ olda[q], xb = nb ^ oldb[q];
                diff |= xa | xb;
                if (xa != 0u) chg |= 1ull << (b + 2 * q);
                if (xb != 0u) chg |= 1ull << (b + 2 * q + 1);
            }
        }
        col_now |= (diff & edge_mask) != 0u;
        __syncwarp();
        return warp_or64(chg);
    }
    constexpr int R = 4;
#pragma unroll 1
    for (int b = 0; b < TH; b += R) {
        if (((rows >> b) & ((1ull << R) - 1ull)) == 0ull) continue;
        nrows += R;
        uint32_t m[R][N], k[R][N], old[R], cin[R];
#pragma unroll
        for (int q = 0; q < R; ++q) {
            const int r = b + q + 1;
            old[q] = sm.tm[r * 32 + lane];
            P::unpack(old[q], m[q]);
            P::unpack(sm.tk[r * 32 + lane], k[q]);
            cin[q] = sm.hLm[r];
        }
        hscan_rows<DT, true, R>(m, k, cin, lane);
#pragma unroll
        for (int q = 0; q < R; ++q) cin[q] = sm.hRm[b + q + 1];
        hscan_rows<DT, false, R>(m, k, cin, lane);
#pragma unroll
        for (int q = 0; q < R; ++q) {
            const uint32_t nw = P::pack(m[q]);
            sm.tm[(b + q + 1) * 32 + lane] = nw;
            const uint32_t x = nw ^ old[q];
            diff |= x;
            if (x != 0u) chg |= 1ull << (b + q);
        }
    }
    col_now |= (diff & edge_mask) != 0u;
    __syncwarp();
    return warp_or64(chg);
}

// --------------------------------------------------------------- tile visit
struct VisitResult {
    unsigned nb;         // NB_* bits: neighbours to notify
    unsigned sweeps;     // sweeps run
    unsigned row_steps;  // rows processed by the sweeps
    bool ok;             // false: a bounded wait ran out (job error)
    bool stored;         // rows of the tile were stored at the end of the visit
    long long t_fetch, t_proc, t_dump;  // clock64 cycles per phase
};

template <int DT>
__device__ __forceinline__ uint32_t load_word_plain(const unsigned char* row, int npx, bool coherent) {
    using P = Px<DT>;
    if (npx >= P::PPW)
        return coherent ? __ldcg(reinterpret_cast<const unsigned int*>(row))
                        : __ldg(reinterpret_cast<const unsigned int*>(row));
    uint32_t p[P::PPW];
#pragma unroll
    for (int i = 0; i < P::PPW; ++i)
        p[i] = i < npx ? (coherent ? P::ld_px_cg(row + i * P::BPP) : P::ld_px(row + i * P::BPP)) : P::MINPX;
    return P::pack(p);
}

// Stores the rows of `rows` (bit r for tile row r) from shared memory to the
// tile's own pixels (MR.cu:335-364; here plain stores: the visiting warp owns
// the tile).
template <int DT, int TH>
__device__ __forceinline__ void write_back_rows(const ImgDesc& d, const WarpSmem<TH>& sm, int lane, int y0, int rows,
                                                int npx, size_t col_off, unsigned long long mask) {
    using P = Px<DT>;
    if (npx <= 0) return;
    for (int r = 0; r < rows; ++r) {
        if ((mask >> r) & 1ull) {
            unsigned char* mrow = d.marker + (size_t)(y0 + r) * d.pitch_m + col_off;
            const uint32_t w = sm.tm[(r + 1) * 32 + lane];
            if (npx >= P::PPW) {
                __stcg(reinterpret_cast<unsigned int*>(mrow), w);
            } else {
                uint32_t p[P::PPW];
                P::unpack(w, p);
#pragma unroll
                for (int i = 0; i < P::PPW; ++i)
                    if (i < npx) P::st_px(mrow + i * P::BPP, p[i]);
            }
        }
    }
}

// Neighbour detection (MR.cu:366-512, pull form): the NB_* bits of the
// neighbour tiles holding a pixel q next to a pixel p of this tile with
// marker[q] < min(marker[p], mask[q]), looking only at the sides that rose.
// The halo values in shared memory are the neighbours' pixels as fetched;
// they can only have risen since, so a stale halo gives at most an extra
// notification, never a missed one.
template <int DT, int CONN, int TH>
__device__ __forceinline__ unsigned detect_neighbours(const WarpSmem<TH>& sm, int lane, bool top_rose, bool bot_rose,
                                                      bool side_rose) {
    using P = Px<DT>;
    unsigned nb = 0u;
    uint32_t r0[P::PPW], r1[P::PPW], t_m[P::PPW], t_k[P::PPW], b_m[P::PPW], b_k[P::PPW];
    P::unpack(sm.tm[32 + lane], r0);
    P::unpack(sm.tm[TH * 32 + lane], r1);
    P::unpack(sm.tm[lane], t_m);
    P::unpack(sm.tk[lane], t_k);
    P::unpack(sm.tm[(TH + 1) * 32 + lane], b_m);
    P::unpack(sm.tk[(TH + 1) * 32 + lane], b_k);
    uint32_t l0 = __shfl_up_sync(FULL, r0[P::PPW - 1], 1), n0 = __shfl_down_sync(FULL, r0[0], 1);
    uint32_t l1 = __shfl_up_sync(FULL, r1[P::PPW - 1], 1), n1 = __shfl_down_sync(FULL, r1[0], 1);
    if (lane == 0) l0 = l1 = P::MINPX;  // pixels of other tiles are not sources here
    if (lane == 31) n0 = n1 = P::MINPX;
    bool need_n = false, need_s = false;
#pragma unroll
    for (int j = 0; j < P::PPW; ++j) {
        uint32_t v0 = r0[j], v1 = r1[j];
        if (CONN == 8) {
            v0 = P::mx3(j == 0 ? l0 : r0[j - 1], v0, j == P::PPW - 1 ? n0 : r0[j + 1]);
            v1 = P::mx3(j == 0 ? l1 : r1[j - 1], v1, j == P::PPW - 1 ? n1 : r1[j + 1]);
        }
        need_n |= P::gt(P::mn(v0, t_k[j]), t_m[j]);
        need_s |= P::gt(P::mn(v1, b_k[j]), b_m[j]);
    }
    if (top_rose && __any_sync(FULL, need_n)) nb |= NB_N;
    if (bot_rose && __any_sync(FULL, need_s)) nb |= NB_S;

    if (side_rose) {
        // W / E: lanes walk the tile's first / last pixel column
        bool need_w = false, need_e = false;
        for (int r = 1 + lane; r <= TH; r += 32) {
            uint32_t f[P::PPW], l[P::PPW];
            P::unpack(sm.tm[r * 32], f);
            P::unpack(sm.tm[r * 32 + 31], l);
            uint32_t fv = f[0], lv = l[P::PPW - 1];
            if (CONN == 8) {
                uint32_t fa[P::PPW], la[P::PPW];
                if (r > 1) {
                    P::unpack(sm.tm[(r - 1) * 32], fa);
                    P::unpack(sm.tm[(r - 1) * 32 + 31], la);
                    fv = P::mx(fv, fa[0]);
                    lv = P::mx(lv, la[P::PPW - 1]);
                }
                if (r < TH) {
                    P::unpack(sm.tm[(r + 1) * 32], fa);
                    P::unpack(sm.tm[(r + 1) * 32 + 31], la);
                    fv = P::mx(fv, fa[0]);
                    lv = P::mx(lv, la[P::PPW - 1]);
                }
            }
            need_w |= P::gt(P::mn(fv, sm.hLk[r]), sm.hLm[r]);
            need_e |= P::gt(P::mn(lv, sm.hRk[r]), sm.hRm[r]);
        }
        if (__any_sync(FULL, need_w)) nb |= NB_W;
        if (__any_sync(FULL, need_e)) nb |= NB_E;
    }
    if (CONN == 8) {
        uint32_t a[P::PPW], b[P::PPW], c[P::PPW], e[P::PPW];
        P::unpack(sm.tm[32], a);
        P::unpack(sm.tm[32 + 31], b);
        P::unpack(sm.tm[TH * 32], c);
        P::unpack(sm.tm[TH * 32 + 31], e);
        if (top_rose && P::gt(P::mn(a[0], sm.hLk[0]), sm.hLm[0])) nb |= NB_NW;
        if (top_rose && P::gt(P::mn(b[P::PPW - 1], sm.hRk[0]), sm.hRm[0])) nb |= NB_NE;
        if (bot_rose && P::gt(P::mn(c[0], sm.hLk[TH + 1]), sm.hLm[TH + 1])) nb |= NB_SW;
        if (bot_rose && P::gt(P::mn(e[P::PPW - 1], sm.hRk[TH + 1]), sm.hRm[TH + 1])) nb |= NB_SE;
    }
    return nb;
}

// Early flush that does nothing: the tile's neighbours are notified once,
// after the visit.
struct NoEarlyFlush {
    static constexpr bool kEnabled = false;
    bool use_passes;
    bool use_pq;  // revisits by the pixel queue (pq_solve)
    __device__ bool passes(int) { return use_passes; }
    __device__ bool pq() { return use_pq; }
    __device__ bool want(int) { return false; }
    __device__ void flush(unsigned, int) {}
};

// ------------------------------------------------------- pixel queue
// Third in-tile solver, for revisits: a FIFO of tile pixels in shared memory
// instead of whole-tile passes.  Seeds: the pixels of the tile's boundary
// ring whose constraint towards any neighbour (halo included) is violated;
// each is raised to what its neighbours allow and queued.  A round pops up to
// 32 pixels, one per lane; each raises its in-tile neighbours q to
// min(value, mask[q]) when that is higher (a compare-and-swap on the packed
// word, lanes may share a word) and newly raised pixels are queued, placed
// by ballot and population count.  Every update is a valid monotone step of
// the propagation rule (MR.cu:43-44) and the queue empties only when no
// queued pixel can raise a neighbour, so the tile ends at its fixed point.
// Returns false (the caller finishes the tile with passes over every row)
// when the FIFO would overflow or a bound is reached; what was raised stands.
// `rows_chg` (per lane) collects the rows that rose (bit r - 1), `col_now`
// whether the tile's first / last pixel column rose.
template <int DT>
__device__ __forceinline__ uint32_t pq_get(const uint32_t* words, int r, int c) {
    using P = Px<DT>;
    const uint32_t w = *(const volatile uint32_t*)&words[r * 32 + c / P::PPW];
    constexpr int B = 8 * P::BPP;
    return B == 32 ? w : (w >> (B * (c % P::PPW))) & ((1u << B) - 1u);
}

// Raises pixel (r, c) of `words` to v when v is higher; true when this lane
// raised it.  *fail is set when the compare-and-swap loop gives up.
template <int DT>
__device__ __forceinline__ bool pq_raise(uint32_t* words, int r, int c, uint32_t v, bool* fail) {
    using P = Px<DT>;
    uint32_t* w = &words[r * 32 + c / P::PPW];
    if constexpr (DT == DT_I32) {
        return atomicMax(reinterpret_cast<int*>(w), (int)v) < (int)v;
    } else {
        constexpr int B = 8 * P::BPP;
        const int sh = B * (c % P::PPW);
        const uint32_t msk = ((1u << B) - 1u) << sh;
        uint32_t old = *(volatile uint32_t*)w;
        for (int it = 0; it < 64; ++it) {
            if (((old & msk) >> sh) >= v) return false;
            const uint32_t got = atomicCAS(w, old, (old & ~msk) | (v << sh));
            if (got == old) return true;
            old = got;
        }
        *fail = true;
        return false;
    }
}

template <int DT, int CONN, int TH>
__device__ bool pq_solve(WarpSmem<TH>& sm, int lane, unsigned long long& rows_chg, bool& col_now, unsigned& rounds) {
    using P = Px<DT>;
    constexpr int TW = 32 * P::PPW;
    int head = 0, tail = 0;  // warp-uniform
    bool fail = false;
    // value of any pixel of rows 0..TH+1, columns -1..TW (halo columns)
    auto val = [&](int r, int c) -> uint32_t {
        if (c < 0) return sm.hLm[r];
        if (c >= TW) return sm.hRm[r];
        return pq_get<DT>(sm.tm, r, c);
    };
    // queue the pixels of the lanes with `want` (warp-uniform call)
    auto enqueue = [&](bool want, int r, int c) {
        const unsigned b = __ballot_sync(FULL, want);
        const int n = __popc(b);
        if (n == 0) return;
        if (tail - head + n > kPqCap) {
            fail = true;
            return;
        }
        if (want) {
            const int rank = __popc(b & ((1u << lane) - 1u));
            sm.pq[(tail + rank) % kPqCap] = (unsigned short)(r * TW + c);
        }
        tail += n;
    };
    auto raised = [&](int r, int c) {
        rows_chg |= 1ull << (r - 1);
        if (c == 0 || c == TW - 1) col_now = true;
    };
    // seeds: the boundary ring (top and bottom rows, first and last columns)
    constexpr int RING = 2 * TW + 2 * TH;
    for (int i0 = 0; i0 < RING; i0 += 32) {
        const int i = i0 + lane;
        int r = 0, c = 0;
        bool on = i < RING;
        if (i < TW) { r = 1; c = i; }
        else if (i < 2 * TW) { r = TH; c = i - TW; }
        else if (i < 2 * TW + TH) { r = i - 2 * TW + 1; c = 0; }
        else { r = i - 2 * TW - TH + 1; c = TW - 1; }
        bool up = false;
        if (on) {
            const uint32_t k = pq_get<DT>(sm.tk, r, c);
            uint32_t best = P::mx(val(r - 1, c), val(r + 1, c));
            best = P::mx(best, P::mx(val(r, c - 1), val(r, c + 1)));
            if (CONN == 8) {
                best = P::mx(best, P::mx(val(r - 1, c - 1), val(r - 1, c + 1)));
                best = P::mx(best, P::mx(val(r + 1, c - 1), val(r + 1, c + 1)));
            }
            const uint32_t cand = P::mn(best, k);
            if (P::gt(cand, pq_get<DT>(sm.tm, r, c)) && pq_raise<DT>(sm.tm, r, c, cand, &fail)) {
                up = true;
                raised(r, c);
            }
        }
        enqueue(up, r, c);
        if (__any_sync(FULL, fail)) return false;
    }
    // rounds
    constexpr int DR[8] = {-1, 1, 0, 0, -1, -1, 1, 1};
    constexpr int DC[8] = {0, 0, -1, 1, -1, 1, -1, 1};
    while (head != tail) {
        if (++rounds > 4096u) return false;
        const int k = min(tail - head, 32);
        int r = 0, c = 0;
        uint32_t v = 0u;
        const bool mine = lane < k;
        if (mine) {
            const int p = sm.pq[(head + lane) % kPqCap];
            r = p / TW;
            c = p - r * TW;
            v = pq_get<DT>(sm.tm, r, c);
        }
        __syncwarp();
        head += k;
#pragma unroll
        for (int dir = 0; dir < CONN; ++dir) {
            const int rq = r + DR[dir], cq = c + DC[dir];
            bool up = false;
            if (mine && rq >= 1 && rq <= TH && cq >= 0 && cq < TW) {
                const uint32_t cand = P::mn(v, pq_get<DT>(sm.tk, rq, cq));
                if (P::gt(cand, pq_get<DT>(sm.tm, rq, cq)) && pq_raise<DT>(sm.tm, rq, cq, cand, &fail)) {
                    up = true;
                    raised(rq, cq);
                }
            }
            enqueue(up, rq, cq);
            if (__any_sync(FULL, fail)) return false;
        }
    }
    return true;
}

// One warp: fetch tile (tx, ty) of image d with its one-pixel halo, run
// raster / anti-raster sweeps until a sweep after the first changes nothing,
// store the rows that rose, and report the neighbour tiles to notify: those
// holding a pixel q next to a pixel p of this tile with
// marker[q] < min(marker[p], mask[q]) where p's side of the tile rose.
// `sides` (NB_* bits) names the halo sides whose pixels are new since the
// tile last converged (all sides on a first visit).
//
// `early` can publish intermediate results: after a sweep that raised a
// boundary row or column, if early.want() says so (the engine asks for it
// when the work queue runs dry, i.e. when the job is bound by its
// propagation front), the rows risen so far are stored and the neighbours
// they raise are handed to early.flush() while the sweeps go on.  The
// returned `nb` then covers only what rose after the last flush.
//
// Inlined into the worker: as a called function its result, its
// descriptor and its shared-memory tile reached it through generic
// pointers, and its row loops re-read counters from the stack (two to four
// local loads per row step); inlined, the kernel has no stack frame and
// the tile is addressed as shared memory (15 % faster on 4096^2 h-domes).
template <int DT, int CONN, int TH, class Early>
__device__ __forceinline__ VisitResult visit_tile(const ImgDesc& d, int tx, int ty, WarpSmem<TH>& sm, int lane,
                                               unsigned& phase, long long timeout_ns, unsigned sides, Early& early) {
    using P = Px<DT>;
    constexpr int TW = 32 * P::PPW;
    VisitResult res{0u, 0u, 0u, true, false, 0, 0, 0};
    const long long c0 = clock64();
    const int x0 = tx * TW, y0 = ty * TH;
    const int W = d.W, H = d.H;
    const int px0 = x0 + lane * P::PPW;  // first pixel of this lane's word
    const int npx = W - px0;             // >= PPW: full word, (0, PPW): partial, <= 0: outside
    const size_t col_off = (size_t)(npx > 0 ? px0 : 0) * P::BPP;
    const int rows = min(TH, H - y0);

    // ---- fetch (MR.cu:232-312)
    const bool tma = d.tmaps != nullptr;
    if (tma) {
        // one box of TH+2 rows x 128 bytes per plane, halo rows included;
        // rows / columns outside the image arrive as zeros
        fence_proxy_async_smem();  // earlier generic reads of tm / tk before the async writes
        __syncwarp();
        if (lane == 0) {
            fence_proxy_async_global();
            mbar_arrive_expect_tx(&sm.mbar, 2u * 128u * (TH + 2));
            const unsigned char* maps = static_cast<const unsigned char*>(d.tmaps);
            tma_load_2d(sm.tm, maps, x0 * P::BPP, y0 - 1, &sm.mbar);
            tma_load_2d(sm.tk, maps + 128, x0 * P::BPP, y0 - 1, &sm.mbar);
        }
    } else {
#pragma unroll 8
        for (int r = 0; r < TH + 2; ++r) {
            const int y = y0 - 1 + r;
            uint32_t mw = P::MINW, kw = P::MINW;
            if (y >= 0 && y < H && npx > 0) {
                mw = load_word_plain<DT>(d.marker + (size_t)y * d.pitch_m + col_off, npx, true);
                kw = load_word_plain<DT>(d.mask + (size_t)y * d.pitch_k + col_off, npx, false);
            }
            sm.tm[r * 32 + lane] = mw;
            sm.tk[r * 32 + lane] = kw;
        }
    }
    // halo columns (single pixels), in flight together with the box loads
    for (int i = lane; i < TH + 2; i += 32) {
        const int y = y0 - 1 + i;
        uint32_t lm = P::MINPX, lk = P::MINPX, rm = P::MINPX, rk = P::MINPX;
        if (y >= 0 && y < H) {
            const unsigned char* mrow = d.marker + (size_t)y * d.pitch_m;
            const unsigned char* krow = d.mask + (size_t)y * d.pitch_k;
            if (x0 > 0) {
                lm = P::ld_px_cg(mrow + (size_t)(x0 - 1) * P::BPP);
                lk = P::ld_px(krow + (size_t)(x0 - 1) * P::BPP);
            }
            if (x0 + TW < W) {
                rm = P::ld_px_cg(mrow + (size_t)(x0 + TW) * P::BPP);
                rk = P::ld_px(krow + (size_t)(x0 + TW) * P::BPP);
            }
        }
        sm.hLm[i] = lm;
        sm.hLk[i] = lk;
        sm.hRm[i] = rm;
        sm.hRk[i] = rk;
    }
    if (tma) {
        // bounded wait for the box loads
        const long long t0 = globaltimer_ns();
        unsigned spins = 0;
        while (!mbar_try_wait(&sm.mbar, phase)) {
            if ((++spins & 1023u) == 0u && globaltimer_ns() - t0 > timeout_ns) {
                res.ok = false;
                break;
            }
        }
        phase ^= 1u;
        if (!res.ok) return res;
        if (DT == DT_I32) {
            // zero fill is not the int32 minimum: rewrite what lies outside
            if (y0 == 0) sm.tm[lane] = sm.tk[lane] = P::MINW;
            for (int r = rows + 1; r < TH + 2; ++r) {
                if (y0 - 1 + r >= H) sm.tm[r * 32 + lane] = sm.tk[r * 32 + lane] = P::MINW;
            }
            if (npx <= 0)
                for (int r = 0; r < TH + 2; ++r) sm.tm[r * 32 + lane] = sm.tk[r * 32 + lane] = P::MINW;
        }
    }
    __syncwarp();
    const long long c1 = clock64();
    res.t_fetch = c1 - c0;

    // ---- local convergence (MR.cu:320-325), by one of two solvers:
    //   row sweeps (early.passes() false): raster / anti-raster sweeps, each
    //     row a vertical update and a warp scan, until a sweep after the
    //     first two changes nothing; fewest instructions per converged tile,
    //     for when the GPU is full of work;
    //   passes (early.passes() true): vertical and horizontal passes (see
    //     vpass / hpass) until no rows are left whose constraints may be
    //     violated; the shortest latency from a raised halo to a raised far
    //     edge, for when the job is bound by its propagation front.
    // Both are sequences of valid monotone updates that stop at the tile's
    // fixed point, so they give the same bytes.
    constexpr unsigned long long ALL = TH == 64 ? ~0ull : ((1ull << TH) - 1ull);
    constexpr unsigned long long TOP = 1ull, BOT = 1ull << (TH - 1);
    const uint32_t edge_mask = lane == 0 ? P::FIRST_MASK : lane == 31 ? P::LAST_MASK : 0u;
    unsigned long long pend_rows = 0ull;  // rows risen since the last flush
    bool col_changed = false;             // a side column rose since the last flush (per lane)
    unsigned sweeps = 0;
    long long t_flush = 0;
    // After a pass that raised a boundary, with more passes to come: publish
    // early if the engine asks for it.
    auto maybe_flush = [&](unsigned long long chg, bool col_now) {
        if (!Early::kEnabled) return;
        const bool boundary = (chg & (TOP | BOT)) != 0ull || __any_sync(FULL, col_now);
        if (!boundary || !early.want(lane)) return;
        const long long f0 = clock64();
        write_back_rows<DT, TH>(d, sm, lane, y0, rows, npx, col_off, pend_rows);
        const unsigned nb = detect_neighbours<DT, CONN, TH>(sm, lane, (pend_rows & TOP) != 0ull,
                                                            (pend_rows & BOT) != 0ull, __any_sync(FULL, col_changed));
        __syncwarp();
        if (nb != 0u) early.flush(nb, lane);
        pend_rows = 0ull;
        col_changed = false;
        t_flush += clock64() - f0;
    };
    // A revisit by the pixel queue when asked for; if it cannot finish, the
    // passes take the tile with every row dirty.
    bool solved = false;
    bool run_passes = early.passes(lane);
    if (early.pq() && sides != 0xffu) {
        unsigned long long rows_chg = 0ull;
        bool col_now = false;
        unsigned rounds = 0u;
        solved = pq_solve<DT, CONN, TH>(sm, lane, rows_chg, col_now, rounds);
        __syncwarp();
        const unsigned long long chg = warp_or64(rows_chg);
        pend_rows |= chg;
        col_changed |= col_now;
        res.row_steps += rounds;
        ++sweeps;
        if (!solved) {
            run_passes = true;
            sides = 0xffu;
        }
    }
    if (solved) {
    } else if (!run_passes) {
        // Rows whose halo inputs are new are processed by the first two
        // sweeps: the top row by the raster sweep (N, NW, NE), the bottom row
        // by the anti-raster sweep (S, SW, SE), every row when a side column
        // that feeds the sweep changed (W, and E through the up-right /
        // down-right diagonals for 8-connectivity; the reverse for the
        // anti-raster sweep).  Other rows are skipped while nothing they
        // depend on has changed.
        const unsigned side_down = CONN == 8 ? (NB_W | NB_E) : NB_W;
        const unsigned side_up = CONN == 8 ? (NB_W | NB_E) : NB_E;
        const unsigned long long force_down =
            (sides & side_down) ? ALL : (sides & (NB_N | NB_NW | NB_NE)) ? TOP : 0ull;
        const unsigned long long force_up = (sides & side_up) ? ALL : (sides & (NB_S | NB_SW | NB_SE)) ? BOT : 0ull;
        unsigned long long chg_prev = 0ull;
        for (;;) {
            unsigned long long dil = chg_prev | (chg_prev << 1) | (chg_prev >> 1);
            if (sweeps == 0) dil |= force_down;
            if (sweeps == 1) dil |= force_up;
            dil &= ALL;
            unsigned long long chg = 0ull;
            bool col_now = false;
            if (dil != 0ull) {
                if ((sweeps & 1u) == 0u)
                    sweep<DT, CONN, TH, true>(sm, lane, dil, chg, col_now, edge_mask, res.row_steps);
                else
                    sweep<DT, CONN, TH, false>(sm, lane, dil, chg, col_now, edge_mask, res.row_steps);
            }
            ++sweeps;
            pend_rows |= chg;
            col_changed |= col_now;
            chg_prev = chg;
            if (chg == 0ull && sweeps >= 2) break;
            if (chg != 0ull) maybe_flush(chg, col_now);
        }
    } else {
        // dVd / dVu: rows whose constraint towards the row above / below may
        // be violated; dH: rows whose horizontal constraints may be violated.
        // A first visit has every row dirty; a revisit only the rows fed by
        // the halo sides that rose: N (and the N corners) the top row for the
        // downward pass, S the bottom row for the upward pass, W / E every
        // row for the horizontal pass and, with 8-connectivity, for both
        // vertical passes (their diagonals read the side columns).
        const bool fresh = sides == 0xffu;
        const bool side_we = (sides & (NB_W | NB_E)) != 0u;
        unsigned long long dVd = (sides & (NB_N | NB_NW | NB_NE)) ? TOP : 0ull;
        unsigned long long dVu = (sides & (NB_S | NB_SW | NB_SE)) ? BOT : 0ull;
        unsigned long long dH = side_we ? ALL : 0ull;
        if (fresh || (CONN == 8 && side_we)) dVd = dVu = ALL;
        for (int it = 0; (dVd | dVu | dH) != 0ull; it = (it + 1) & 3) {
            unsigned long long chg;
            bool col_now = false;
            if (it == 0) {
                if (dVd == 0ull) continue;
                chg = vpass<DT, CONN, TH, true>(sm, lane, dVd, edge_mask, col_now, res.row_steps);
                dVd = 0ull;
                dVu |= chg >> 1;
                dH |= chg;
            } else if (it == 2) {
                if (dVu == 0ull) continue;
                chg = vpass<DT, CONN, TH, false>(sm, lane, dVu, edge_mask, col_now, res.row_steps);
                dVu = 0ull;
                dVd |= (chg << 1) & ALL;
                dH |= chg;
            } else {
                if (dH == 0ull) continue;
                chg = hpass<DT, TH>(sm, lane, dH, edge_mask, col_now, res.row_steps);
                dH = 0ull;
                dVd |= (chg << 1) & ALL;
                dVu |= chg >> 1;
            }
            ++sweeps;
            pend_rows |= chg;
            col_changed |= col_now;
            if (chg != 0ull && (dVd | dVu | dH) != 0ull) maybe_flush(chg, col_now);
        }
    }
    res.sweeps = sweeps;
    const long long c2 = clock64();
    res.t_proc = c2 - c1 - t_flush;
    res.t_dump = t_flush;
    if (pend_rows == 0ull) return res;  // nothing rose since the last flush: nothing to store or notify

    // ---- write back the rows that rose, then neighbour detection
    write_back_rows<DT, TH>(d, sm, lane, y0, rows, npx, col_off, pend_rows);
    res.stored = true;
    const unsigned nb = detect_neighbours<DT, CONN, TH>(sm, lane, (pend_rows & TOP) != 0ull,
                                                        (pend_rows & BOT) != 0ull, __any_sync(FULL, col_changed));
    __syncwarp();
    res.nb = nb;
    res.t_dump += clock64() - c2;
    return res;
}

}  // namespace iwpp
