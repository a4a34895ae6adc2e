// iwpp_device.cuh -- device building blocks of the GB300 reconstruction
// engine: packed-pixel arithmetic, one-warp tile visits (load, raster /
// anti-raster sweeps to local convergence, write-back, neighbour detection).
//
// Layout: a tile is TH rows x TW pixels with TW * sizeof(pixel) = 128 bytes
// (TW = 128 uint8, 64 uint16, 32 int32).  One warp owns one tile at a time;
// lane L keeps the 32-bit word holding pixels [L*PPW, L*PPW + PPW) of every
// row in registers (PPW = pixels per word = 4 / 2 / 1), for both marker and
// mask.  Vertical propagation is therefore register-serial inside a lane and
// horizontal propagation is a warp scan over the max-min semiring.
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

// --------------------------------------------------------------- pixel words
template <int DT>
struct Px;

template <>
struct Px<DT_U8> {
    static constexpr int PPW = 4;
    static constexpr int BPP = 1;
    static constexpr uint32_t MINPX = 0u;
    static constexpr uint32_t MINW = 0u;
    __device__ static __forceinline__ uint32_t vmax(uint32_t a, uint32_t b) { return __vmaxu4(a, b); }
    __device__ static __forceinline__ uint32_t vmin(uint32_t a, uint32_t b) { return __vminu4(a, b); }
    __device__ static __forceinline__ bool any_gt(uint32_t a, uint32_t b) { return __vcmpgtu4(a, b) != 0u; }
    __device__ static __forceinline__ uint32_t smax(uint32_t a, uint32_t b) { return a > b ? a : b; }
    __device__ static __forceinline__ uint32_t smin(uint32_t a, uint32_t b) { return a < b ? a : b; }
    __device__ static __forceinline__ bool gt(uint32_t a, uint32_t b) { return a > b; }
    __device__ static __forceinline__ uint32_t first(uint32_t w) { return w & 0xffu; }
    __device__ static __forceinline__ uint32_t last(uint32_t w) { return w >> 24; }
    __device__ static __forceinline__ uint32_t as_last(uint32_t px) { return px << 24; }
    __device__ static __forceinline__ uint32_t bcast(uint32_t px) { return px * 0x01010101u; }
    // pixel i <- pixel i-1 (pixel 0 <- last pixel of `prev`)
    __device__ static __forceinline__ uint32_t shl1(uint32_t w, uint32_t prev) { return __funnelshift_l(prev, w, 8); }
    // pixel i <- pixel i+1 (last pixel <- first pixel of `next`)
    __device__ static __forceinline__ uint32_t shr1(uint32_t w, uint32_t next) { return __funnelshift_r(w, next, 8); }
    __device__ static __forceinline__ uint32_t hmin(uint32_t w) {
        uint32_t t = vmin(w, __funnelshift_r(w, w, 8));
        t = vmin(t, __funnelshift_r(t, t, 16));
        return t & 0xffu;
    }
    // prefix (forward) or suffix (backward) minimum of the pixels of a word
    template <bool FWD>
    __device__ static __forceinline__ uint32_t scanmin(uint32_t w) {
        if (FWD) {
            w = vmin(w, (w << 8) | 0x000000ffu);
            return vmin(w, (w << 16) | 0x0000ffffu);
        } else {
            w = vmin(w, (w >> 8) | 0xff000000u);
            return vmin(w, (w >> 16) | 0xffff0000u);
        }
    }
    __device__ static __forceinline__ uint32_t pack2(uint32_t a, uint32_t b) { return a | (b << 16); }
    __device__ static __forceinline__ uint32_t unpack_a(uint32_t p) { return p & 0xffffu; }
    __device__ static __forceinline__ uint32_t unpack_b(uint32_t p) { return p >> 16; }
    __device__ static __forceinline__ uint32_t get(uint32_t w, int i) { return (w >> (8 * i)) & 0xffu; }
    __device__ static __forceinline__ uint32_t ld_px(const unsigned char* p) { return *p; }
    __device__ static __forceinline__ uint32_t ld_px_cg(const unsigned char* p) {
        return __ldcg(reinterpret_cast<const unsigned char*>(p));
    }
    __device__ static __forceinline__ void st_px(unsigned char* p, uint32_t v) { *p = (unsigned char)v; }
};

template <>
struct Px<DT_U16> {
    static constexpr int PPW = 2;
    static constexpr int BPP = 2;
    static constexpr uint32_t MINPX = 0u;
    static constexpr uint32_t MINW = 0u;
    __device__ static __forceinline__ uint32_t vmax(uint32_t a, uint32_t b) { return __vmaxu2(a, b); }
    __device__ static __forceinline__ uint32_t vmin(uint32_t a, uint32_t b) { return __vminu2(a, b); }
    __device__ static __forceinline__ bool any_gt(uint32_t a, uint32_t b) { return __vcmpgtu2(a, b) != 0u; }
    __device__ static __forceinline__ uint32_t smax(uint32_t a, uint32_t b) { return a > b ? a : b; }
    __device__ static __forceinline__ uint32_t smin(uint32_t a, uint32_t b) { return a < b ? a : b; }
    __device__ static __forceinline__ bool gt(uint32_t a, uint32_t b) { return a > b; }
    __device__ static __forceinline__ uint32_t first(uint32_t w) { return w & 0xffffu; }
    __device__ static __forceinline__ uint32_t last(uint32_t w) { return w >> 16; }
    __device__ static __forceinline__ uint32_t as_last(uint32_t px) { return px << 16; }
    __device__ static __forceinline__ uint32_t bcast(uint32_t px) { return px | (px << 16); }
    __device__ static __forceinline__ uint32_t shl1(uint32_t w, uint32_t prev) { return __funnelshift_l(prev, w, 16); }
    __device__ static __forceinline__ uint32_t shr1(uint32_t w, uint32_t next) { return __funnelshift_r(w, next, 16); }
    __device__ static __forceinline__ uint32_t hmin(uint32_t w) { return vmin(w, __funnelshift_r(w, w, 16)) & 0xffffu; }
    template <bool FWD>
    __device__ static __forceinline__ uint32_t scanmin(uint32_t w) {
        return FWD ? vmin(w, (w << 16) | 0x0000ffffu) : vmin(w, (w >> 16) | 0xffff0000u);
    }
    __device__ static __forceinline__ uint32_t pack2(uint32_t a, uint32_t b) { return a | (b << 16); }
    __device__ static __forceinline__ uint32_t unpack_a(uint32_t p) { return p & 0xffffu; }
    __device__ static __forceinline__ uint32_t unpack_b(uint32_t p) { return p >> 16; }
    __device__ static __forceinline__ uint32_t get(uint32_t w, int i) { return (w >> (16 * i)) & 0xffffu; }
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
    __device__ static __forceinline__ uint32_t vmax(uint32_t a, uint32_t b) { return (uint32_t)max((int)a, (int)b); }
    __device__ static __forceinline__ uint32_t vmin(uint32_t a, uint32_t b) { return (uint32_t)min((int)a, (int)b); }
    __device__ static __forceinline__ bool any_gt(uint32_t a, uint32_t b) { return (int)a > (int)b; }
    __device__ static __forceinline__ uint32_t smax(uint32_t a, uint32_t b) { return vmax(a, b); }
    __device__ static __forceinline__ uint32_t smin(uint32_t a, uint32_t b) { return vmin(a, b); }
    __device__ static __forceinline__ bool gt(uint32_t a, uint32_t b) { return (int)a > (int)b; }
    __device__ static __forceinline__ uint32_t first(uint32_t w) { return w; }
    __device__ static __forceinline__ uint32_t last(uint32_t w) { return w; }
    __device__ static __forceinline__ uint32_t as_last(uint32_t px) { return px; }
    __device__ static __forceinline__ uint32_t bcast(uint32_t px) { return px; }
    __device__ static __forceinline__ uint32_t shl1(uint32_t, uint32_t prev) { return prev; }
    __device__ static __forceinline__ uint32_t shr1(uint32_t, uint32_t next) { return next; }
    __device__ static __forceinline__ uint32_t hmin(uint32_t w) { return w; }
    template <bool FWD>
    __device__ static __forceinline__ uint32_t scanmin(uint32_t w) { return w; }
    __device__ static __forceinline__ uint32_t get(uint32_t w, int) { return w; }
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
    int W, H;
    int dtype, conn;
    int tiles_x, tiles_y;
    int tile_base;  // first global tile index of this image
    int tile_rows;  // TH used for this image
};

// neighbour direction bits returned by a tile visit
enum : unsigned {
    NB_N = 1u << 0, NB_S = 1u << 1, NB_W = 1u << 2, NB_E = 1u << 3,
    NB_NW = 1u << 4, NB_NE = 1u << 5, NB_SW = 1u << 6, NB_SE = 1u << 7
};
__device__ __constant__ static const int kNbDx[8] = {0, 0, -1, 1, -1, 1, -1, 1};
__device__ __constant__ static const int kNbDy[8] = {-1, 1, 0, 0, -1, -1, 1, 1};

// Per-warp shared memory: the tile's marker and mask words (row stride 33
// words so that a row is conflict-free for the 32 lanes and so is a column),
// and the left / right halo columns, where index i holds row i-1 (index 0 is
// the row above the tile, index TH+1 the row below).
constexpr int kRowStride = 33;

template <int TH>
struct WarpSmem {
    uint32_t tm[TH * kRowStride];
    uint32_t tk[TH * kRowStride];
    uint32_t hLm[TH + 2];
    uint32_t hLk[TH + 2];
    uint32_t hRm[TH + 2];
    uint32_t hRk[TH + 2];
};

// ---------------------------------------------------- horizontal warp scan
// Propagates along one row in scan order (FWD: left to right), with `cin` the
// marker value of the halo pixel entering the row at the first lane.  The
// per-word transfer function of x (the value entering a word) is
// f(x) = max(min(x, B), A) with B = min of the word's mask pixels and A = the
// word's exit pixel after the intra-word pass; these compose associatively:
// (A2,B2) o (A1,B1) = (max(min(A1, B2), A2), min(B1, B2)).
template <int DT, bool FWD>
__device__ __forceinline__ uint32_t hscan(uint32_t m, uint32_t k, uint32_t cin, int lane) {
    using P = Px<DT>;
#pragma unroll
    for (int s = 1; s < P::PPW; ++s) m = P::vmax(m, P::vmin(FWD ? P::shl1(m, P::MINW) : P::shr1(m, P::MINW), k));
    const int edge_lane = FWD ? 0 : 31;
    const uint32_t out_px = FWD ? P::last(m) : P::first(m);
    uint32_t in_px = FWD ? __shfl_up_sync(FULL, out_px, 1) : __shfl_down_sync(FULL, out_px, 1);
    if (lane == edge_lane) in_px = cin;
    const uint32_t k_in = FWD ? P::first(k) : P::last(k);
    const uint32_t m_in = FWD ? P::first(m) : P::last(m);
    // A carry that does not raise a word's entry pixel raises nothing after it.
    const bool need = P::gt(P::smin(in_px, k_in), m_in);
    if (!__any_sync(FULL, need)) return m;

    uint32_t A = out_px, B = P::hmin(k);
    if (lane == edge_lane) {
        A = P::smax(A, P::smin(cin, B));
        B = P::MINPX;  // the entry lane becomes a constant: nothing before it
    }
#pragma unroll
    for (int d = 1; d < 32; d <<= 1) {
        uint32_t Ap, Bp;
        if (DT == DT_I32) {
            Ap = FWD ? __shfl_up_sync(FULL, A, d) : __shfl_down_sync(FULL, A, d);
            Bp = FWD ? __shfl_up_sync(FULL, B, d) : __shfl_down_sync(FULL, B, d);
        } else {
            uint32_t pk = (A & 0xffffu) | (B << 16);
            pk = FWD ? __shfl_up_sync(FULL, pk, d) : __shfl_down_sync(FULL, pk, d);
            Ap = pk & 0xffffu;
            Bp = pk >> 16;
        }
        const bool valid = FWD ? (lane >= d) : (lane + d < 32);
        if (valid) {
            A = P::smax(P::smin(Ap, B), A);
            B = P::smin(Bp, B);
        }
    }
    uint32_t c = FWD ? __shfl_up_sync(FULL, A, 1) : __shfl_down_sync(FULL, A, 1);
    if (lane == edge_lane) c = cin;
    return P::vmax(m, P::vmin(P::bcast(c), P::template scanmin<FWD>(k)));
}

// ------------------------------------------------------------- one sweep
// DOWN = raster order (rows top to bottom, each row left to right),
// otherwise anti-raster.  After a complete raster sweep every pixel satisfies
// its constraints towards N+ = {left, up-left, up, up-right}; after an
// anti-raster sweep towards N-.  Returns whether any pixel rose.
template <int DT, int CONN, int TH, bool DOWN>
__device__ __forceinline__ bool sweep(WarpSmem<TH>& sm, uint32_t halo_row, int lane,
                                      unsigned long long& rows_changed) {
    using P = Px<DT>;
    bool any = false;
    uint32_t prev = halo_row;  // final values of the row processed before
#pragma unroll 2
    for (int i = 0; i < TH; ++i) {
        const int r = DOWN ? i : TH - 1 - i;
        const int rp = DOWN ? r - 1 : r + 1;  // row of `prev` (-1 / TH = halo)
        const uint32_t old = sm.tm[r * kRowStride + lane];
        const uint32_t kr = sm.tk[r * kRowStride + lane];
        uint32_t v = prev;
        if (CONN == 8) {
            uint32_t pw = __shfl_up_sync(FULL, prev, 1);
            uint32_t nw = __shfl_down_sync(FULL, prev, 1);
            if (lane == 0) pw = P::as_last(sm.hLm[rp + 1]);
            if (lane == 31) nw = sm.hRm[rp + 1];
            v = P::vmax(v, P::vmax(P::shl1(prev, pw), P::shr1(prev, nw)));
        }
        uint32_t x = P::vmax(old, P::vmin(v, kr));
        x = hscan<DT, DOWN>(x, kr, DOWN ? sm.hLm[r + 1] : sm.hRm[r + 1], lane);
        if (__any_sync(FULL, x != old)) {
            sm.tm[r * kRowStride + lane] = x;
            rows_changed |= 1ull << r;
            any = true;
        }
        prev = x;
    }
    __syncwarp();
    return any;
}

// --------------------------------------------------------------- tile visit
struct VisitResult {
    unsigned nb;      // NB_* bits: neighbours whose pixels this tile can raise
    unsigned sweeps;  // sweeps run
    bool wrote;       // any pixel of this tile rose
};

template <int DT>
__device__ __forceinline__ void load_word(const unsigned char* mrow, const unsigned char* krow, int npx,
                                          uint32_t& mw, uint32_t& kw) {
    using P = Px<DT>;
    if (npx >= P::PPW) {
        mw = __ldcg(reinterpret_cast<const unsigned int*>(mrow));
        kw = __ldg(reinterpret_cast<const unsigned int*>(krow));
    } else if (P::PPW == 1) {
        mw = P::MINW;
        kw = P::MINW;
    } else {
        // partial word at the right image edge: per-pixel loads, the rest
        // filled with the type's minimum (inert: it never rises or raises)
        mw = 0u;
        kw = 0u;
#pragma unroll
        for (int i = 0; i < P::PPW; ++i) {
            if (i < npx) {
                mw |= P::ld_px_cg(mrow + i * P::BPP) << (8 * P::BPP * i);
                kw |= P::ld_px(krow + i * P::BPP) << (8 * P::BPP * i);
            }
        }
    }
}

// One warp: fetch tile (tx, ty) of image d with its one-pixel halo, run
// raster / anti-raster sweeps until a sweep after the first changes nothing,
// store the rows that rose, and report every neighbour tile holding a pixel q
// next to a pixel p of this tile with marker[q] < min(marker[p], mask[q]).
template <int DT, int CONN, int TH>
__device__ __noinline__ VisitResult visit_tile(const ImgDesc& d, int tx, int ty, WarpSmem<TH>& sm, int lane) {
    using P = Px<DT>;
    constexpr int TW = 32 * P::PPW;
    const int x0 = tx * TW, y0 = ty * TH;
    const int W = d.W, H = d.H;
    const int px0 = x0 + lane * P::PPW;  // first pixel of this lane's word
    const int npx = W - px0;             // >= PPW: full word, (0, PPW): partial, <= 0: outside
    const size_t col_off = (size_t)(npx > 0 ? px0 : 0) * P::BPP;
    const int rows = min(TH, H - y0);

    // ---- fetch (MR.cu:232-312): interior words, coalesced 128-byte rows
#pragma unroll 4
    for (int r = 0; r < TH; ++r) {
        uint32_t mw = P::MINW, kw = P::MINW;
        if (r < rows && npx > 0) {
            const int y = y0 + r;
            load_word<DT>(d.marker + (size_t)y * d.pitch_m + col_off, d.mask + (size_t)y * d.pitch_k + col_off, npx,
                          mw, kw);
        }
        sm.tm[r * kRowStride + lane] = mw;
        sm.tk[r * kRowStride + lane] = kw;
    }
    uint32_t top_m = P::MINW, top_k = P::MINW, bot_m = P::MINW, bot_k = P::MINW;
    if (npx > 0) {
        if (y0 > 0)
            load_word<DT>(d.marker + (size_t)(y0 - 1) * d.pitch_m + col_off,
                          d.mask + (size_t)(y0 - 1) * d.pitch_k + col_off, npx, top_m, top_k);
        if (y0 + TH < H)
            load_word<DT>(d.marker + (size_t)(y0 + TH) * d.pitch_m + col_off,
                          d.mask + (size_t)(y0 + TH) * d.pitch_k + col_off, npx, bot_m, bot_k);
    }
    for (int i = lane; i < TH + 2; i += 32) {
        const int y = y0 + i - 1;
        uint32_t lm = P::MINPX, lk = P::MINPX, rm = P::MINPX, rk = P::MINPX;
        if (y >= 0 && y < H && i - 1 < rows + 1) {
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
    __syncwarp();

    // ---- local convergence (MR.cu:320-325, here with full-length scans)
    unsigned long long rows_changed = 0ull;
    unsigned sweeps = 0;
    for (;;) {
        const bool ch = (sweeps & 1u) == 0u ? sweep<DT, CONN, TH, true>(sm, top_m, lane, rows_changed)
                                            : sweep<DT, CONN, TH, false>(sm, bot_m, lane, rows_changed);
        ++sweeps;
        if (!ch && sweeps >= 2) break;
    }

    // ---- write back the rows that rose (own tile only; MR.cu:335-364)
    if (rows_changed != 0ull && npx > 0) {
        for (int r = 0; r < rows; ++r) {
            if ((rows_changed >> r) & 1ull) {
                unsigned char* mrow = d.marker + (size_t)(y0 + r) * d.pitch_m + col_off;
                const uint32_t w = sm.tm[r * kRowStride + lane];
                if (npx >= P::PPW) {
                    __stcg(reinterpret_cast<unsigned int*>(mrow), w);
                } else {
#pragma unroll
                    for (int i = 0; i < P::PPW; ++i)
                        if (i < npx) P::st_px(mrow + i * P::BPP, P::get(w, i));
                }
            }
        }
    }

    // ---- neighbour detection (MR.cu:366-512, pull form): which neighbour
    // tiles hold a pixel q that some pixel p of this tile can raise.
    unsigned nb = 0u;
    {
        const uint32_t r0 = sm.tm[lane], r1 = sm.tm[(TH - 1) * kRowStride + lane];
        uint32_t v0 = r0, v1 = r1;
        if (CONN == 8) {
            uint32_t pw0 = __shfl_up_sync(FULL, r0, 1), nw0 = __shfl_down_sync(FULL, r0, 1);
            uint32_t pw1 = __shfl_up_sync(FULL, r1, 1), nw1 = __shfl_down_sync(FULL, r1, 1);
            if (lane == 0) pw0 = pw1 = P::MINW;
            if (lane == 31) nw0 = nw1 = P::MINW;
            v0 = P::vmax(v0, P::vmax(P::shl1(r0, pw0), P::shr1(r0, nw0)));
            v1 = P::vmax(v1, P::vmax(P::shl1(r1, pw1), P::shr1(r1, nw1)));
        }
        if (__any_sync(FULL, P::any_gt(P::vmin(v0, top_k), top_m))) nb |= NB_N;
        if (__any_sync(FULL, P::any_gt(P::vmin(v1, bot_k), bot_m))) nb |= NB_S;

        // W / E: lanes walk the tile's first / last pixel column (rows lane,
        // lane+32, ...); stride-33 rows keep these reads conflict-free.
        bool need_w = false, need_e = false;
        for (int r = lane; r < TH; r += 32) {
            uint32_t fv = P::first(sm.tm[r * kRowStride]);
            uint32_t lv = P::last(sm.tm[r * kRowStride + 31]);
            if (CONN == 8) {
                if (r > 0) {
                    fv = P::smax(fv, P::first(sm.tm[(r - 1) * kRowStride]));
                    lv = P::smax(lv, P::last(sm.tm[(r - 1) * kRowStride + 31]));
                }
                if (r + 1 < TH) {
                    fv = P::smax(fv, P::first(sm.tm[(r + 1) * kRowStride]));
                    lv = P::smax(lv, P::last(sm.tm[(r + 1) * kRowStride + 31]));
                }
            }
            need_w |= P::gt(P::smin(fv, sm.hLk[r + 1]), sm.hLm[r + 1]);
            need_e |= P::gt(P::smin(lv, sm.hRk[r + 1]), sm.hRm[r + 1]);
        }
        if (__any_sync(FULL, need_w)) nb |= NB_W;
        if (__any_sync(FULL, need_e)) nb |= NB_E;

        if (CONN == 8) {
            const uint32_t p_nw = P::first(sm.tm[0]);
            const uint32_t p_ne = P::last(sm.tm[31]);
            const uint32_t p_sw = P::first(sm.tm[(TH - 1) * kRowStride]);
            const uint32_t p_se = P::last(sm.tm[(TH - 1) * kRowStride + 31]);
            if (P::gt(P::smin(p_nw, sm.hLk[0]), sm.hLm[0])) nb |= NB_NW;
            if (P::gt(P::smin(p_ne, sm.hRk[0]), sm.hRm[0])) nb |= NB_NE;
            if (P::gt(P::smin(p_sw, sm.hLk[TH + 1]), sm.hLm[TH + 1])) nb |= NB_SW;
            if (P::gt(P::smin(p_se, sm.hRk[TH + 1]), sm.hRm[TH + 1])) nb |= NB_SE;
        }
    }
    __syncwarp();
    VisitResult res;
    res.nb = nb;
    res.sweeps = sweeps;
    res.wrote = rows_changed != 0ull;
    return res;
}

}  // namespace iwpp
