// iwpp_front.cu -- front passes: whole-image directional sweeps restricted to
// the tiles that changed, repeated until nothing changes, in one persistent
// cooperative kernel; then the check that seeds the tile engine with the
// tiles still violating a constraint.
//
// Reference counterparts: the whole-image raster / anti-raster propagation
// kernels (*PropagationEntireImage, IWPP MP/src/MorphologicalReconstruction.cu:
// 547-753; iRec1D*, IWPP MP DQ/src/MorphologicalReconstruction.cu:817-1074),
// which the reference runs (commented out, MR.cu:792-795) a fixed number of
// times over the whole image.  The rule is MR.cu:43-44,
// m[c] = max(m[c], min(m[p], mask[c])), applied along rows (+X, -X) and
// along columns from the pixel above / below (+Y, -Y; a valid update for
// either connectivity, the tile engine completes the diagonals).
//
// Why: a long propagation path (a corridor spiralling through the image)
// advances one tile per dependent tile visit in the tile engine, but one
// whole arm per sweep here.  Whole-image sweeps re-read both planes every
// time; these read only what can change:
//
// * Each 128-byte x 64-row tile keeps the index of the last sweep that raised
//   one of its pixels (chg).  Sweep s (direction s % 4) needs a tile only if
//   it changed in one of the three sweeps since the last sweep in the same
//   direction (chg >= s - 3); every tile is needed in the first pass.  Row
//   bands keep the last sweep that raised a pixel in them, so a warp skips a
//   clean row at the cost of one load (gathered 32 rows at a time).
// * +X / -X: one warp per row walks the row's 128-byte chunks, scanning a
//   chunk (warp max-min scan) when its tile is dirty or the carry from the
//   previous chunk raised that chunk's last pixel; other chunks are not read.
// * +Y / -Y: per pixel column, the update through one tile's 64 rows is a
//   clamp map x -> max(min(x, B), A) of the value entering it (B: the
//   tile's least mask, a constant kept per tile; A: its exit pixel when
//   nothing enters), and such maps compose.  Phase A: one warp per dirty
//   tile finds A by walking its rows, staged into shared memory by one burst
//   of cp.async copies.  Phase B: per tile column and lane word, a warp
//   scans the column's maps into the value entering every tile (a clean
//   tile's A is its exit row as it is).  Phase C: each tile of those columns
//   is swept from that value, walking only dirty tiles and clean tiles whose
//   first row the entering value raises.  A vertical arm of any length is
//   crossed in one sweep.
// * The passes end after four sweeps in a row changed nothing (every 4-
//   connected constraint then holds), or at a sweep cap.
//
// Every pixel is written by one warp per sweep, so the result of each sweep
// is deterministic; every update is monotone and never exceeds the
// reconstruction, so any prefix of the passes is a valid start for the tile
// engine.
#include "iwpp_engine.cuh"
#include "iwpp_front.cuh"

namespace iwpp {

// Launch shape and pipelining depths (compile-time; -D overrides for sweeps).
#ifndef IWPP_FP_WARPS
#define IWPP_FP_WARPS 32  // warps per CTA (one CTA per SM, 64 registers a thread)
#endif
#ifndef IWPP_FP_YWARPS
#define IWPP_FP_YWARPS 12  // of them, warps with a 16 KB tile stage for the vertical phases
#endif
#ifndef IWPP_FP_XAHEAD
#define IWPP_FP_XAHEAD 4  // chunks of a row whose loads are in flight together
#endif
constexpr int kFpWarps = IWPP_FP_WARPS;
constexpr int kFpYWarps = IWPP_FP_YWARPS;
constexpr int kFpTileRows = 64;  // rows of a tracking tile
constexpr int kFpBatch = 4;      // rows loaded at once where a tile cannot be staged by cp.async

// ------------------------------------------------------- vertical lane words
// A lane's 4-byte word of a row, as the vertical chain sees it: uint8 as two
// u16x2 pairs (pixels 0, 1 and 2, 3), uint16 as one u16x2 pair, int32 as one
// signed value.  The clamp map of a run of rows is (A, B) in the same form.
template <int DT>
struct VW;

template <>
struct VW<DT_U8> {
    uint32_t a, b;
    __device__ static VW from(uint32_t w) { return VW{__byte_perm(w, 0u, 0x4140), __byte_perm(w, 0u, 0x4342)}; }
    __device__ uint32_t pack() const { return __byte_perm(a, b, 0x6420); }
    __device__ static VW lo() { return VW{0u, 0u}; }
    __device__ static VW hi() { return VW{0x00ff00ffu, 0x00ff00ffu}; }
    // max(m, min(x, k))
    __device__ static VW step(VW m, VW x, VW k) {
        return VW{__vmaxu2(m.a, __vminu2(x.a, k.a)), __vmaxu2(m.b, __vminu2(x.b, k.b))};
    }
    __device__ static VW mn(VW x, VW y) { return VW{__vminu2(x.a, y.a), __vminu2(x.b, y.b)}; }
    // some pixel of x is above the one of y
    __device__ static bool any_gt(VW x, VW y) { return (__vcmpgtu2(x.a, y.a) | __vcmpgtu2(x.b, y.b)) != 0u; }
};

template <>
struct VW<DT_U16> {
    uint32_t a;
    __device__ static VW from(uint32_t w) { return VW{w}; }
    __device__ uint32_t pack() const { return a; }
    __device__ static VW lo() { return VW{0u}; }
    __device__ static VW hi() { return VW{0xffffffffu}; }
    __device__ static VW step(VW m, VW x, VW k) { return VW{__vmaxu2(m.a, __vminu2(x.a, k.a))}; }
    __device__ static VW mn(VW x, VW y) { return VW{__vminu2(x.a, y.a)}; }
    __device__ static bool any_gt(VW x, VW y) { return __vcmpgtu2(x.a, y.a) != 0u; }
};

template <>
struct VW<DT_I32> {
    int a;
    __device__ static VW from(uint32_t w) { return VW{(int)w}; }
    __device__ uint32_t pack() const { return (uint32_t)a; }
    __device__ static VW lo() { return VW{INT_MIN}; }
    __device__ static VW hi() { return VW{INT_MAX}; }
    __device__ static VW step(VW m, VW x, VW k) { return VW{max(m.a, min(x.a, k.a))}; }
    __device__ static VW mn(VW x, VW y) { return VW{min(x.a, y.a)}; }
    __device__ static bool any_gt(VW x, VW y) { return x.a > y.a; }
};

// ------------------------------------------------------------ diagnostics
// Built with -DIWPP_FP_TRACE: the end of every phase records the time and
// the work done (rows walked, chunks scanned, tiles walked, clean-tile
// checks), read back through iwpp_front_trace (not part of include/iwpp.h).
#ifdef IWPP_FP_TRACE
constexpr int kTraceMax = 4096;
__device__ unsigned long long g_fp_trace[kTraceMax][6];
__device__ unsigned g_fp_trace_n;
__device__ unsigned long long g_fp_work[4];  // rows, chunks, tiles walked, clean checks
#define FP_COUNT(i, n) atomicAdd(&g_fp_work[i], (unsigned long long)(n))
#else
#define FP_COUNT(i, n) ((void)0)
#endif

// ------------------------------------------------------------ grid barrier
// All CTAs of the cooperative launch.  The last CTA to arrive runs `last`
// (bookkeeping between phases) before it releases the others.  Waits are
// bounded by the job's timeout; returns false when the passes failed.
template <class Last>
__device__ bool front_barrier(const FrontArgs& f, Last last, int tag = 0) {
    __shared__ int s_ok;
    __syncthreads();
    if (threadIdx.x == 0) {
        FrontCtrl* c = f.fc;
        int ok = 1;
        const unsigned gen = *(volatile unsigned*)&c->bar_gen;
        __threadfence();
        const unsigned arrived = atomicAdd(&c->bar_count, 1u);
        if (arrived == gridDim.x - 1u) {
            __threadfence();
            last(c);
#ifdef IWPP_FP_TRACE
            const unsigned n = g_fp_trace_n;
            if (n < kTraceMax) {
                g_fp_trace[n][0] = (unsigned long long)globaltimer_ns();
                g_fp_trace[n][1] = (unsigned long long)tag;
                for (int q = 0; q < 4; ++q) g_fp_trace[n][2 + q] = *(volatile unsigned long long*)&g_fp_work[q];
                g_fp_trace_n = n + 1;
            }
#endif
            c->bar_count = 0u;
            __threadfence();
            atomicAdd(&c->bar_gen, 1u);
        } else {
            const long long t0 = globaltimer_ns();
            unsigned ns = 32;
            while (*(volatile unsigned*)&c->bar_gen == gen) {
                __nanosleep(ns);
                if (ns < 256) ns <<= 1;
                if (*(volatile unsigned*)&c->error != 0u) {
                    ok = 0;
                    break;
                }
                if (globaltimer_ns() - t0 > f.timeout_ns) {
                    atomicCAS(&c->error, 0u, 3u);
                    atomicCAS(f.job_error, 0u, 3u);
                    ok = 0;
                    break;
                }
            }
            __threadfence();
        }
        if (*(volatile unsigned*)&c->error != 0u) ok = 0;
        s_ok = ok;
    }
    __syncthreads();
    return s_ok != 0;
}

// Sweep s raised a pixel of tile t (lane 0 of the warp).  Plain stores,
// never a read first: a warp must not wait on a round trip per change.
// Every writer in sweep s writes the same value, and readers look only at
// values of earlier sweeps (after a grid barrier).
__device__ __forceinline__ void mark_tile(const FrontArgs& f, int t, int s) { f.chg[t] = s; }

__device__ __forceinline__ bool is_dirty(int chg, int s) { return s < 4 || chg >= s - 3; }

// ------------------------------------------------------------ X sweep: a row
// Walks row y in the sweep direction over 128-byte chunks (tile columns):
// a chunk is read and scanned when its tile is dirty or the carry into it is
// live (the previous chunk's exit pixel rose).  A run of such chunks keeps
// the loads of the chunk kXAheadF steps further on in flight (a register
// ring, the walk unrolled by its length), so its chain is the scans, not a
// memory latency per chunk; between runs the walk jumps to the next dirty
// chunk.  Dirty bits come from a 64-chunk window of tile flags read with two
// warp ballots.  Returns whether the row rose (warp-uniform).
constexpr int kXAheadF = IWPP_FP_XAHEAD;

template <int DT, bool FWD>
__device__ bool front_row(const FrontArgs& f, int y, int s, int lane) {
    using P = Px<DT>;
    constexpr int TW = 32 * P::PPW;  // pixels per chunk
    constexpr int K = kXAheadF;
    const ImgDesc& d = f.d;
    const int ty = y / kFpTileRows;
    const int nch = f.tx_n;
    unsigned char* mrow = d.marker + (size_t)y * d.pitch_m;
    const unsigned char* krow = d.mask + (size_t)y * d.pitch_k;
    const int* chg_row = f.chg + (size_t)ty * nch;
    auto chunk_of = [&](int i) { return FWD ? i : nch - 1 - i; };  // chunk of walk step i
    // dirty bits of walk steps [wbase, wbase + 64) (warp-uniform)
    unsigned long long win = 0ull;
    int wbase = -1000;
    auto refill = [&](int i) {
        // the window holds the 32 steps before i's group of 32 and that
        // group: the walk reads steps j and j + kXAheadF, both inside
        wbase = (i & ~31) - 32;
        const int j0 = wbase + lane, j1 = wbase + 32 + lane;
        const bool d0 = j0 >= 0 && j0 < nch && is_dirty(__ldcg(&chg_row[chunk_of(j0)]), s);
        const bool d1 = j1 >= 0 && j1 < nch && is_dirty(__ldcg(&chg_row[chunk_of(j1)]), s);
        win = (unsigned long long)__ballot_sync(FULL, d0) | ((unsigned long long)__ballot_sync(FULL, d1) << 32);
    };
    auto dirty = [&](int i) -> bool {
        if (i >= nch) return false;
        if (i < wbase || i >= wbase + 64) refill(i);
        return (win >> (i - wbase)) & 1ull;
    };
    // the first dirty step at or after i (nch if none)
    auto next_dirty = [&](int i) -> int {
        while (i < nch) {
            if (i < wbase || i >= wbase + 64) refill(i);
            const unsigned long long rest = win >> (i - wbase);
            if (rest) return i + __ffsll((long long)rest) - 1;
            i = wbase + 64;
        }
        return nch;
    };
    auto fetch = [&](int i, uint32_t& mw, uint32_t& kw) {
        mw = P::MINW;
        kw = P::MINW;
        const int px0 = chunk_of(i) * TW + lane * P::PPW, npx = d.W - px0;
        if (i < nch && npx > 0) {
            mw = load_word_plain<DT>(mrow + (size_t)px0 * P::BPP, npx, true);
            kw = load_word_plain<DT>(krow + (size_t)px0 * P::BPP, npx, false);
        }
    };
    uint32_t qm[K], qk[K];
    bool row_rose = false;
    int i = next_dirty(0);
    if (i < nch && lane == 0) FP_COUNT(0, 1);
    while (i < nch) {
        // a run starts at the dirty step i with a dead carry: the lap holding
        // it, its dirty steps' loads issued at once
        int base = i - i % K;
        unsigned issued = 0u;
#pragma unroll
        for (int q = 0; q < K; ++q) {
            qm[q] = qk[q] = 0u;
            if (base + q >= i && dirty(base + q)) {
                fetch(base + q, qm[q], qk[q]);
                issued |= 1u << q;
            }
        }
        bool live = false;
        uint32_t carry = P::MINPX;
        for (;;) {
#pragma unroll
            for (int q = 0; q < K; ++q) {
                const int j = base + q;
                if (j >= i && j < nch) {
                    if (live || dirty(j)) {
                        if (!live) {
                            // the carry entering: the pixel before the chunk
                            const int c = chunk_of(j);
                            const int xin = FWD ? c * TW - 1 : (c + 1) * TW;
                            carry = xin >= 0 && xin < d.W ? P::ld_px_cg(mrow + (size_t)xin * P::BPP) : P::MINPX;
                        }
                        if (!((issued >> q) & 1u)) fetch(j, qm[q], qk[q]);
                        if (lane == 0) FP_COUNT(1, 1);
                        const uint32_t mw = qm[q], kw = qk[q];
                        uint32_t m[P::PPW], k[P::PPW];
                        P::unpack(mw, m);
                        P::unpack(kw, k);
                        const uint32_t exit_old =
                            FWD ? __shfl_sync(FULL, m[P::PPW - 1], 31) : __shfl_sync(FULL, m[0], 0);
                        hscan<DT, FWD>(m, k, carry, lane);
                        const uint32_t nw = P::pack(m);
                        const bool chg = nw != mw;
                        if (chg) {
                            const int px0 = chunk_of(j) * TW + lane * P::PPW, npx = d.W - px0;
                            if (npx >= P::PPW) {
                                *reinterpret_cast<unsigned int*>(mrow + (size_t)px0 * P::BPP) = nw;
                            } else if (npx > 0) {
                                uint32_t p[P::PPW];
                                P::unpack(nw, p);
#pragma unroll
                                for (int jj = 0; jj < P::PPW; ++jj)
                                    if (jj < npx) P::st_px(mrow + (size_t)(px0 + jj) * P::BPP, p[jj]);
                            }
                        }
                        if (__any_sync(FULL, chg)) {
                            row_rose = true;
                            if (lane == 0) mark_tile(f, ty * nch + chunk_of(j), s);
                        }
                        carry = FWD ? __shfl_sync(FULL, m[P::PPW - 1], 31) : __shfl_sync(FULL, m[0], 0);
                        live = P::gt(carry, exit_old);
                    }
                    // slot q now serves step j + K
                    issued &= ~(1u << q);
                    if (j + K < nch && (live || dirty(j + K))) {
                        fetch(j + K, qm[q], qk[q]);
                        issued |= 1u << q;
                    }
                }
            }
            base += K;
            i = base;
            if (base >= nch) break;
            if (!live) {
                // dead carry: go on into the next lap if it holds a dirty
                // chunk, else jump to the next run
                const int nd = next_dirty(base);
                if (nd >= base + K) {
                    i = nd;
                    break;
                }
            }
        }
    }
    if (row_rose && lane == 0) f.bchg[ty] = s;
    return row_rose;
}

// ------------------------------------------------------- Y sweep: one tile
// The lane word of one row of tile column tx (a ragged right edge pixel by
// pixel; lanes past the row's end get the type's minimum).
template <int DT>
__device__ __forceinline__ void load_row_word(const FrontArgs& f, int tx, int y, int lane, uint32_t& mw, uint32_t& kw) {
    using P = Px<DT>;
    const ImgDesc& d = f.d;
    const long long byte0 = (long long)tx * 128 + lane * 4;
    const long long row_bytes = (long long)d.W * P::BPP;
    mw = kw = P::MINW;
    if (byte0 + 4 <= row_bytes) {
        mw = __ldcg(reinterpret_cast<const unsigned int*>(d.marker + (size_t)y * d.pitch_m + byte0));
        kw = __ldg(reinterpret_cast<const unsigned int*>(d.mask + (size_t)y * d.pitch_k + byte0));
    } else if (byte0 < row_bytes) {
        const int npx = (int)((row_bytes - byte0) / P::BPP);
        const int px0 = (int)(byte0 / P::BPP);
        mw = load_word_plain<DT>(d.marker + (size_t)y * d.pitch_m + (size_t)px0 * P::BPP, npx, true);
        kw = load_word_plain<DT>(d.mask + (size_t)y * d.pitch_k + (size_t)px0 * P::BPP, npx, false);
    }
}

// Stores one lane word of row y of tile column tx (a ragged right edge pixel
// by pixel).
template <int DT>
__device__ __forceinline__ void store_row_word(const FrontArgs& f, int tx, int y, int lane, uint32_t w) {
    using P = Px<DT>;
    const ImgDesc& d = f.d;
    const long long byte0 = (long long)tx * 128 + lane * 4;
    const long long row_bytes = (long long)d.W * P::BPP;
    unsigned char* row = d.marker + (size_t)y * d.pitch_m;
    if (byte0 + 4 <= row_bytes) {
        *reinterpret_cast<unsigned int*>(row + byte0) = w;
    } else if (byte0 < row_bytes) {
        const int npx = (int)((row_bytes - byte0) / P::BPP), px0 = (int)(byte0 / P::BPP);
        uint32_t p[P::PPW];
        P::unpack(w, p);
#pragma unroll
        for (int j = 0; j < P::PPW; ++j)
            if (j < npx) P::st_px(row + (size_t)(px0 + j) * P::BPP, p[j]);
    }
}

// A Y-phase warp's stage: the 64 rows x 128 bytes of one tile, both planes.
struct __align__(16) TileStage {
    uint32_t m[kFpTileRows][32];
    uint32_t k[kFpTileRows][32];
};

__device__ __forceinline__ void fp_cp_async16(void* smem_dst, const void* gmem_src) {
    asm volatile("cp.async.cg.shared.global [%0], [%1], 16;" ::"r"(smem_u32(smem_dst)), "l"(gmem_src) : "memory");
}
__device__ __forceinline__ void fp_cp_async_wait_all() {
    asm volatile("cp.async.commit_group;\n\tcp.async.wait_group 0;" ::: "memory");
}

// Copies rows [y0, y0 + rows) of tile column tx into the warp's stage (one
// lane word per row): one burst of 16-byte cp.async pieces when the image
// allows them (rows on 16-byte boundaries, the tile column inside the row),
// else lane-word loads that handle a ragged right edge.
template <int DT>
__device__ void stage_tile(const FrontArgs& f, int tx, int y0, int rows, TileStage& st, int lane) {
    using P = Px<DT>;
    const ImgDesc& d = f.d;
    const long long row_bytes = (long long)d.W * P::BPP;
    if (f.aligned16 && (long long)(tx + 1) * 128 <= row_bytes) {
        const int piece = lane & 7, r0 = lane >> 3;
        const size_t off = (size_t)tx * 128 + (size_t)piece * 16;
        for (int r = r0; r < rows; r += 4) {
            fp_cp_async16(&st.m[r][piece * 4], d.marker + (size_t)(y0 + r) * d.pitch_m + off);
            fp_cp_async16(&st.k[r][piece * 4], d.mask + (size_t)(y0 + r) * d.pitch_k + off);
        }
        fp_cp_async_wait_all();
    } else {
        for (int b = 0; b < rows; b += kFpBatch) {
            uint32_t mw[kFpBatch], kw[kFpBatch];
#pragma unroll
            for (int q = 0; q < kFpBatch; ++q)
                if (b + q < rows) load_row_word<DT>(f, tx, y0 + b + q, lane, mw[q], kw[q]);
#pragma unroll
            for (int q = 0; q < kFpBatch; ++q)
                if (b + q < rows) {
                    st.m[b + q][lane] = mw[q];
                    st.k[b + q][lane] = kw[q];
                }
        }
    }
    __syncwarp();
}

// Phase A (dirty tiles): the clamp map of tile (tx, ty) for the value
// entering it in sweep order, x -> max(min(x, B), A): B is the tile's least
// mask per pixel column (a constant, in the bmin table, filled by the first
// vertical sweep, which walks every tile), A its exit pixel when nothing
// enters, found by walking its staged rows.  (A clean tile's A is its exit
// row as it is: its rows already satisfy this direction; phase B reads it.)
template <int DT, bool DOWN>
__device__ void tile_map(const FrontArgs& f, int tx, int ty, int s, TileStage& st, int lane) {
    using V = VW<DT>;
    const int t = ty * f.tx_n + tx;
    const int y0 = ty * kFpTileRows, rows = min(kFpTileRows, f.d.H - y0);
    if (lane == 0) FP_COUNT(2, 1);
    stage_tile<DT>(f, tx, y0, rows, st, lane);
    V x = V::lo(), kmin = V::hi();
    for (int i = 0; i < rows; ++i) {
        const int r = DOWN ? i : rows - 1 - i;
        const V k = V::from(st.k[r][lane]);
        x = V::step(V::from(st.m[r][lane]), x, k);
        kmin = V::mn(kmin, k);
    }
    if (s < 4) f.bmin[(size_t)t * 32 + lane] = kmin.pack();
    f.segA[(size_t)t * 32 + lane] = x.pack();
}

// Lane word w of marker row y of tile column tx (a ragged right edge pixel
// by pixel, past the row's end the type's minimum).
template <int DT>
__device__ __forceinline__ uint32_t marker_word(const FrontArgs& f, int tx, int w, int y) {
    using P = Px<DT>;
    const ImgDesc& d = f.d;
    const long long byte0 = (long long)tx * 128 + w * 4;
    const long long row_bytes = (long long)d.W * P::BPP;
    const unsigned char* row = d.marker + (size_t)y * d.pitch_m;
    if (byte0 + 4 <= row_bytes) return __ldcg(reinterpret_cast<const unsigned int*>(row + byte0));
    if (byte0 < row_bytes) return load_word_plain<DT>(row + byte0, (int)((row_bytes - byte0) / P::BPP), true);
    return P::MINW;
}

// Phase B: for lane word w of tile column tx, the value entering every tile
// of the column in sweep order -- an exclusive scan of the tiles' clamp maps
// over the warp (each lane composes a run of consecutive tiles, the warp
// scans the runs, each lane applies its prefix through its run).  Nothing
// enters the column at the image edge.  A dirty tile's A comes from phase A,
// a clean tile's is its exit row as it is.  A column with no dirty tile is
// left alone; the first lane word's warp flags the others for phase C.
template <int DT, bool DOWN>
__device__ void column_chain(const FrontArgs& f, int tx, int w, int s, int lane) {
    using V = VW<DT>;
    const int n = f.ty_n;
    const int per = (n + 31) / 32;
    const int j0 = lane * per, j1 = min(j0 + per, n);
    auto tile_at = [&](int j) { return (DOWN ? j : n - 1 - j) * f.tx_n + tx; };
    bool any = false;
    for (int j = j0; j < j1; ++j) any |= is_dirty(__ldcg(&f.chg[tile_at(j)]), s);
    if (!__any_sync(FULL, any)) return;
    if (w == 0 && lane == 0) f.cchg[tx] = s;
    auto tile_A = [&](int j) -> V {
        const int t = tile_at(j);
        if (is_dirty(__ldcg(&f.chg[t]), s)) return V::from(__ldcg(&f.segA[(size_t)t * 32 + w]));
        const int ty = t / f.tx_n, y0 = ty * kFpTileRows, rows = min(kFpTileRows, f.d.H - y0);
        return V::from(marker_word<DT>(f, tx, w, DOWN ? y0 + rows - 1 : y0));
    };
    // this lane's run: composed map (A, B)
    V A = V::lo(), B = V::hi();
    for (int j = j0; j < j1; ++j) {
        const V At = tile_A(j), Bt = V::from(__ldcg(&f.bmin[(size_t)tile_at(j) * 32 + w]));
        A = V::step(At, A, Bt);
        B = V::mn(B, Bt);
    }
    // inclusive scan of the runs over the lanes: (A, B) after the runs before it
    for (int dd = 1; dd < 32; dd <<= 1) {
        V Ap, Bp;
        if constexpr (DT == DT_U8) {
            Ap = V{__shfl_up_sync(FULL, A.a, dd), __shfl_up_sync(FULL, A.b, dd)};
            Bp = V{__shfl_up_sync(FULL, B.a, dd), __shfl_up_sync(FULL, B.b, dd)};
        } else {
            Ap = V{__shfl_up_sync(FULL, A.a, dd)};
            Bp = V{__shfl_up_sync(FULL, B.a, dd)};
        }
        if (lane >= dd) {
            A = V::step(A, Ap, B);  // (A, B) after (Ap, Bp)
            B = V::mn(Bp, B);
        }
    }
    // the value entering this lane's run: the A of the runs before it
    V x;
    if constexpr (DT == DT_U8) {
        x = V{__shfl_up_sync(FULL, A.a, 1), __shfl_up_sync(FULL, A.b, 1)};
    } else {
        x = V{__shfl_up_sync(FULL, A.a, 1)};
    }
    if (lane == 0) x = V::lo();
    for (int j = j0; j < j1; ++j) {
        const size_t slot = (size_t)tile_at(j) * 32 + w;
        f.segIn[slot] = x.pack();
        x = V::step(tile_A(j), x, V::from(__ldcg(&f.bmin[slot])));
    }
}

// Phase C: sweep tile (tx, ty) from the value entering it, walking it when
// it is dirty or the entering value raises its first row (a clean tile's
// rows already satisfy this direction among themselves).  Returns whether
// it rose (warp-uniform).
template <int DT, bool DOWN>
__device__ bool tile_apply(const FrontArgs& f, int tx, int ty, int s, bool dirty, TileStage& st, int lane) {
    using V = VW<DT>;
    const int t = ty * f.tx_n + tx;
    const int y0 = ty * kFpTileRows, rows = min(kFpTileRows, f.d.H - y0);
    V x = V::from(__ldcg(&f.segIn[(size_t)t * 32 + lane]));
    if (!dirty) {
        if (lane == 0) FP_COUNT(3, 1);
        uint32_t mw, kw;
        load_row_word<DT>(f, tx, DOWN ? y0 : y0 + rows - 1, lane, mw, kw);
        const V m = V::from(mw);
        if (!__any_sync(FULL, V::any_gt(V::step(m, x, V::from(kw)), m))) return false;
    }
    if (lane == 0) FP_COUNT(2, 1);
    stage_tile<DT>(f, tx, y0, rows, st, lane);
    bool rose = false;
    for (int i = 0; i < rows; ++i) {
        const int r = DOWN ? i : rows - 1 - i;
        const uint32_t mw = st.m[r][lane];
        x = V::step(V::from(mw), x, V::from(st.k[r][lane]));
        const uint32_t nw = x.pack();
        if (nw != mw) {
            rose = true;
            store_row_word<DT>(f, tx, y0 + r, lane, nw);
        }
    }
    rose = __any_sync(FULL, rose);
    if (rose && lane == 0) {
        mark_tile(f, t, s);
        f.bchg[ty] = s;
    }
    return rose;
}

// A warp's share of n work items (item = first + k * stride), 32 at a
// time: the lanes evaluate pred for 32 items at once (their flag loads in
// one memory round trip), then fn(item) runs for those it holds for.
template <class Pred, class Fn>
__device__ __forceinline__ void for_items(int first, int stride, int n, int lane, Pred pred, Fn fn) {
    for (int base = first; base < n; base += 32 * stride) {
        const int it = base + lane * stride;
        const bool dd = it < n && pred(it);
        unsigned bits = __ballot_sync(FULL, dd);
        while (bits) {
            const int q = __ffs(bits) - 1;
            bits &= bits - 1u;
            fn(base + q * stride);
        }
    }
}

// ---------------------------------------------------------------- kernel
// One CTA per SM.  Rows (X sweeps) are shared by all warps; tiles (the
// vertical phases) by the first kFpYWarps warps of each CTA, which own a
// 16 KB tile stage each.
template <int DT>
__global__ void __launch_bounds__(kFpWarps * 32, 1) front_kernel(FrontArgs f) {
    extern __shared__ __align__(16) unsigned char fp_smem[];
    const int lane = threadIdx.x & 31;
    const int warp = threadIdx.x >> 5;
    const int wg = (int)(blockIdx.x * kFpWarps + warp);
    const int nw = (int)(gridDim.x * kFpWarps);
    const bool ywarp = warp < kFpYWarps;
    TileStage& st = reinterpret_cast<TileStage*>(fp_smem)[ywarp ? warp : 0];
    const int wy = (int)(blockIdx.x * kFpYWarps + warp);
    const int ny = (int)(gridDim.x * kFpYWarps);
    const int G = f.tx_n * f.ty_n;
    for (int s = 0;; ++s) {
        const int dir = s & 3;
        bool rose = false;  // this warp raised a pixel in sweep s
        if (dir == 0 || dir == 2) {
            for_items(
                wg, nw, f.d.H, lane, [&](int y) { return is_dirty(__ldcg(&f.bchg[y / kFpTileRows]), s); },
                [&](int y) {
                    if (dir == 0)
                        rose |= front_row<DT, true>(f, y, s, lane);
                    else
                        rose |= front_row<DT, false>(f, y, s, lane);
                });
        } else {
            const bool down = dir == 1;
            // phase A: the dirty tiles (a column's tiles are tx_n apart in t,
            // so they spread over the warps)
            if (ywarp)
                for_items(
                    wy, ny, G, lane, [&](int t) { return is_dirty(__ldcg(&f.chg[t]), s); },
                    [&](int t) {
                        const int ty = t / f.tx_n, tx = t - ty * f.tx_n;
                        if (down)
                            tile_map<DT, true>(f, tx, ty, s, st, lane);
                        else
                            tile_map<DT, false>(f, tx, ty, s, st, lane);
                    });
            if (!front_barrier(f, [](FrontCtrl*) {}, 1)) return;
            // phase B: one warp per (column, lane word); columns without a
            // dirty tile return at once
            for (int it = wg; it < f.tx_n * 32; it += nw) {
                if (down)
                    column_chain<DT, true>(f, it >> 5, it & 31, s, lane);
                else
                    column_chain<DT, false>(f, it >> 5, it & 31, s, lane);
            }
            if (!front_barrier(f, [](FrontCtrl*) {}, 2)) return;
            // phase C: every tile of the columns phase B flagged
            if (ywarp)
                for_items(
                    wy, ny, G, lane, [&](int t) { return __ldcg(&f.cchg[t % f.tx_n]) == s; },
                    [&](int t) {
                        const int ty = t / f.tx_n, tx = t - ty * f.tx_n;
                        const bool dt_ = is_dirty(__ldcg(&f.chg[t]), s);
                        if (down)
                            rose |= tile_apply<DT, true>(f, tx, ty, s, dt_, st, lane);
                        else
                            rose |= tile_apply<DT, false>(f, tx, ty, s, dt_, st, lane);
                    });
        }
        if (rose && lane == 0) f.fc->changed[s & 3] = 1u;
        // end of sweep s: stop after four sweeps in a row changed nothing, or
        // at the cap; clear the flag the next sweep sets
        const int cap = f.max_sweeps;
        unsigned long long* acc = f.job_sweeps;
        const bool ok = front_barrier(
            f,
            [s, cap, acc](FrontCtrl* c) {
                volatile unsigned* ch = c->changed;
                c->sweeps = (unsigned)(s + 1);
                const bool quiet = s >= 3 && ch[0] == 0u && ch[1] == 0u && ch[2] == 0u && ch[3] == 0u;
                if (quiet || s + 1 >= cap) {
                    c->done = 1u;
                    atomicAdd(acc, (unsigned long long)(s + 1));
                }
                ch[(s + 1) & 3] = 0u;
            },
            3 + 4 * s);
        if (!ok) return;
        if (*(volatile unsigned*)&f.fc->done != 0u) return;
    }
}

// --------------------------------------------------------- engine seeding
// After the passes every 4-connected constraint holds (when they converged);
// the tile engine must still visit every tile holding a pixel that a
// neighbour could raise (with 8-connectivity: across the diagonals).  One
// warp per engine tile (TH rows, 128 bytes wide) streams the tile's rows
// with the rows above and below, one word per lane, neighbours across lanes
// by shuffles and across tiles by the halo columns (lanes 0 / 31), and marks
// a tile with such a pixel DIRTY on all sides and appends it to the seed
// list; other tiles get state 0.
template <int DT>
__device__ __forceinline__ uint32_t seed_word(const ImgDesc& d, const unsigned char* base, long long pitch, int y,
                                              int px0) {
    using P = Px<DT>;
    if (y < 0 || y >= d.H || px0 >= d.W) return P::MINW;
    return load_word_plain<DT>(base + (size_t)y * pitch + (size_t)px0 * P::BPP, d.W - px0, false);
}

template <int DT>
__device__ __forceinline__ uint32_t seed_px(const ImgDesc& d, int y, int x) {
    using P = Px<DT>;
    if (y < 0 || y >= d.H || x < 0 || x >= d.W) return P::MINPX;
    return P::ld_px(d.marker + (size_t)y * d.pitch_m + (size_t)x * P::BPP);
}

template <int DT>
__global__ void seed_kernel(const ImgDesc d, unsigned* state, unsigned* list, unsigned* nlist) {
    using P = Px<DT>;
    constexpr int N = P::PPW;
    constexpr int TW = 32 * N;
    const int lane = threadIdx.x & 31;
    const long long tiles = (long long)d.tiles_x * d.tiles_y;
    const long long wg = ((long long)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const long long nw = ((long long)gridDim.x * blockDim.x) >> 5;
    const int TH = d.tile_rows;
    for (long long t = wg; t < tiles; t += nw) {
        const int ty = (int)(t / d.tiles_x), tx = (int)(t - (long long)ty * d.tiles_x);
        const int x0 = tx * TW, y0 = ty * TH, rows = min(TH, d.H - y0);
        const int px0 = x0 + lane * N;
        // marker words of rows y - 1, y, y + 1 (rolling), and for lanes 0 / 31
        // the halo column pixel beside the tile in the same three rows
        uint32_t wu = seed_word<DT>(d, d.marker, d.pitch_m, y0 - 1, px0);
        uint32_t wc = seed_word<DT>(d, d.marker, d.pitch_m, y0, px0);
        const int hx = lane == 0 ? x0 - 1 : x0 + TW;
        uint32_t hu = seed_px<DT>(d, y0 - 1, hx), hc = seed_px<DT>(d, y0, hx);
        bool bad = false;
        for (int r = 0; r < rows; ++r) {
            const int y = y0 + r;
            const uint32_t wd = seed_word<DT>(d, d.marker, d.pitch_m, y + 1, px0);
            const uint32_t wk = seed_word<DT>(d, d.mask, d.pitch_k, y, px0);
            const uint32_t hd = seed_px<DT>(d, y + 1, hx);
            uint32_t u[N], c[N], dn[N], k[N];
            P::unpack(wu, u);
            P::unpack(wc, c);
            P::unpack(wd, dn);
            P::unpack(wk, k);
            // per column: the largest of the pixels above and below (the
            // vertical neighbours) and of all three (what a column offers
            // its side neighbours with 8-connectivity)
            uint32_t v2[N], v3[N];
#pragma unroll
            for (int j = 0; j < N; ++j) {
                v2[j] = P::mx(u[j], dn[j]);
                v3[j] = P::mx(v2[j], c[j]);
            }
            // the columns left of the lane's first pixel and right of its last
            const uint32_t side_l = d.conn == 8 ? v3[N - 1] : c[N - 1];
            const uint32_t side_r = d.conn == 8 ? v3[0] : c[0];
            uint32_t left = __shfl_up_sync(FULL, side_l, 1), right = __shfl_down_sync(FULL, side_r, 1);
            const uint32_t halo = d.conn == 8 ? P::mx(P::mx(hu, hc), hd) : hc;
            if (lane == 0) left = halo;
            if (lane == 31) right = halo;
            bool mine = false;
#pragma unroll
            for (int j = 0; j < N; ++j) {
                const uint32_t l = j == 0 ? left : (d.conn == 8 ? v3[j - 1] : c[j - 1]);
                const uint32_t rr = j == N - 1 ? right : (d.conn == 8 ? v3[j + 1] : c[j + 1]);
                const uint32_t best = P::mx(v2[j], P::mx(l, rr));
                mine |= P::gt(P::mn(best, k[j]), c[j]) && px0 + j < d.W;
            }
            if (__any_sync(FULL, mine)) {
                bad = true;
                break;
            }
            wu = wc;
            wc = wd;
            hu = hc;
            hc = hd;
        }
        const unsigned g = (unsigned)d.tile_base + (unsigned)t;
        if (lane == 0) {
            state[g] = bad ? (ST_DIRTY | ST_SIDES) : 0u;
            if (bad) list[atomicAdd(nlist, 1u)] = g;
        }
    }
}

// ------------------------------------------------------------------ host
static void front_dims(const ImgDesc& d, int* tx_n, int* ty_n) {
    *tx_n = (int)(((long long)d.W * (d.dtype == DT_U8 ? 1 : d.dtype == DT_U16 ? 2 : 4) + 127) / 128);
    *ty_n = (d.H + kFpTileRows - 1) / kFpTileRows;
}

static size_t al(size_t v) { return (v + 255) / 256 * 256; }

size_t front_scratch_bytes(const ImgDesc& d) {
    int tx_n, ty_n;
    front_dims(d, &tx_n, &ty_n);
    const size_t G = (size_t)tx_n * ty_n;
    return al(sizeof(FrontCtrl)) + al((G + ty_n + tx_n) * 4) + 3 * al(G * 128);
}

template <int DT>
static void* front_kernel_ptr() {
    return reinterpret_cast<void*>(&front_kernel<DT>);
}

cudaError_t launch_front(const ImgDesc& d, void* scratch, unsigned* job_error, unsigned long long* job_sweeps,
                         int max_sweeps, long long timeout_ns, int device, cudaStream_t s, int* launches) {
    if (d.W == 0 || d.H == 0) return cudaSuccess;
    FrontArgs f{};
    f.d = d;
    front_dims(d, &f.tx_n, &f.ty_n);
    const size_t G = (size_t)f.tx_n * f.ty_n;
    char* p = static_cast<char*>(scratch);
    f.fc = reinterpret_cast<FrontCtrl*>(p);
    p += al(sizeof(FrontCtrl));
    f.chg = reinterpret_cast<int*>(p);
    f.bchg = f.chg + G;
    f.cchg = f.bchg + f.ty_n;
    p += al((G + f.ty_n + f.tx_n) * 4);
    f.bmin = reinterpret_cast<uint32_t*>(p);
    p += al(G * 128);
    f.segA = reinterpret_cast<uint32_t*>(p);
    p += al(G * 128);
    f.segIn = reinterpret_cast<uint32_t*>(p);
    f.aligned16 = ((reinterpret_cast<uintptr_t>(d.marker) | reinterpret_cast<uintptr_t>(d.mask)) & 15u) == 0u &&
                  ((d.pitch_m | d.pitch_k) & 15) == 0;
    f.job_error = job_error;
    f.job_sweeps = job_sweeps;
    f.max_sweeps = max_sweeps;
    f.timeout_ns = timeout_ns;
    // counters zero, every tile "changed before the first pass" (-1)
    cudaError_t e = cudaMemsetAsync(f.fc, 0, sizeof(FrontCtrl), s);
    if (e == cudaSuccess) e = cudaMemsetAsync(f.chg, 0xff, (G + f.ty_n + f.tx_n) * 4, s);
    if (e != cudaSuccess) return e;
    void* k = d.dtype == DT_U8 ? front_kernel_ptr<DT_U8>() : d.dtype == DT_U16 ? front_kernel_ptr<DT_U16>()
                                                                                : front_kernel_ptr<DT_I32>();
    const size_t smem = kFpYWarps * sizeof(TileStage);
    e = cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    int per_sm = 0, sms = 0;
    if (e == cudaSuccess) e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k, kFpWarps * 32, smem);
    if (e == cudaSuccess) e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device);
    if (e != cudaSuccess) return e;
    if (per_sm < 1) return cudaErrorInvalidConfiguration;
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3((unsigned)(per_sm * sms));
    cfg.blockDim = dim3(kFpWarps * 32);
    cfg.dynamicSmemBytes = smem;
    cfg.stream = s;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeCooperative;
    attr[0].val.cooperative = 1;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    void* params[] = {&f};
    e = cudaLaunchKernelExC(&cfg, k, params);
    if (e == cudaSuccess && launches) ++*launches;
    return e;
}

cudaError_t launch_seed(const ImgDesc& d, unsigned* state, unsigned* list, unsigned* nlist, cudaStream_t s,
                        int* launches) {
    if (d.W == 0 || d.H == 0) return cudaSuccess;
    const long long tiles = (long long)d.tiles_x * d.tiles_y;
    long long blocks = (tiles * 32 + 255) / 256;
    if (blocks > 152ll * 16) blocks = 152ll * 16;
    if (blocks < 1) blocks = 1;
    if (d.dtype == DT_U8)
        seed_kernel<DT_U8><<<(unsigned)blocks, 256, 0, s>>>(d, state, list, nlist);
    else if (d.dtype == DT_U16)
        seed_kernel<DT_U16><<<(unsigned)blocks, 256, 0, s>>>(d, state, list, nlist);
    else
        seed_kernel<DT_I32><<<(unsigned)blocks, 256, 0, s>>>(d, state, list, nlist);
    if (launches) ++*launches;
    return cudaGetLastError();
}

}  // namespace iwpp

#ifdef IWPP_FP_TRACE
// Diagnostics of a -DIWPP_FP_TRACE build: copies up to `max` trace records
// (6 values each) to `out` and returns their number; clears the trace.
extern "C" __attribute__((visibility("default"))) int iwpp_front_trace(unsigned long long* out, int max) {
    unsigned n = 0;
    cudaMemcpyFromSymbol(&n, iwpp::g_fp_trace_n, sizeof(n));
    if ((int)n > max) n = (unsigned)max;
    if (n) cudaMemcpyFromSymbol(out, iwpp::g_fp_trace, n * 6 * sizeof(unsigned long long));
    const unsigned zero = 0u;
    const unsigned long long z4[4] = {0ull, 0ull, 0ull, 0ull};
    cudaMemcpyToSymbol(iwpp::g_fp_trace_n, &zero, sizeof(zero));
    cudaMemcpyToSymbol(iwpp::g_fp_work, z4, sizeof(z4));
    return (int)n;
}
#endif
