// iwpp_sweeps.cu -- elementwise precondition clip and whole-image directional
// sweeps.
//
// clip:   the reference's clipImage (IWPP MP/src/MorphologicalReconstruction.cu:827-836),
//         marker = min(marker, mask), one 32-bit word per thread.
// sweeps: the reference's *PropagationEntireImage kernels (MR.cu:547-753)
//         and the iRec1D* alternatives (IWPP MP DQ/src/MorphologicalReconstruction.cu:817-1074),
//         rule m = max(m, min(prev, mask)) along one axis.
//   +X / -X: one warp per row, the whole row as one max-min scan (128-byte
//            chunks, carry from chunk to chunk), exact and coalesced.
//   +Y / -Y: one warp per 128-byte column strip walking the full height,
//            rows streamed through shared memory with cp.async far ahead;
//            8-connectivity also takes the two diagonal pixels of the
//            previous row inside the strip.  Every pixel is written by one
//            thread, so the result is deterministic.
#include "iwpp_engine.cuh"

namespace iwpp {

template <int DT>
__device__ __forceinline__ void load_pair(const unsigned char* mrow, const unsigned char* krow, int npx,
                                          uint32_t& mw, uint32_t& kw) {
    mw = load_word_plain<DT>(mrow, npx, true);
    kw = load_word_plain<DT>(krow, npx, false);
}

template <int DT>
__device__ __forceinline__ void store_word_plain(unsigned char* mrow, int npx, uint32_t w) {
    using P = Px<DT>;
    if (npx >= P::PPW) {
        *reinterpret_cast<unsigned int*>(mrow) = w;
    } else {
        uint32_t p[P::PPW];
        P::unpack(w, p);
#pragma unroll
        for (int i = 0; i < P::PPW; ++i)
            if (i < npx) P::st_px(mrow + i * P::BPP, p[i]);
    }
}

// ------------------------------------------------------------------- clip
template <int DT>
__global__ void clip_kernel(ImgDesc d) {
    using P = Px<DT>;
    const int words = (d.W + P::PPW - 1) / P::PPW;
    const long long total = (long long)words * d.H;
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < total;
         i += (long long)gridDim.x * blockDim.x) {
        const int y = (int)(i / words), wi = (int)(i - (long long)y * words);
        const int px0 = wi * P::PPW, npx = d.W - px0;
        unsigned char* mrow = d.marker + (size_t)y * d.pitch_m + (size_t)px0 * P::BPP;
        const unsigned char* krow = d.mask + (size_t)y * d.pitch_k + (size_t)px0 * P::BPP;
        uint32_t mw, kw;
        load_pair<DT>(mrow, krow, npx, mw, kw);
        uint32_t m[P::PPW], k[P::PPW];
        P::unpack(mw, m);
        P::unpack(kw, k);
#pragma unroll
        for (int j = 0; j < P::PPW; ++j) m[j] = P::mn(m[j], k[j]);
        const uint32_t c = P::pack(m);
        if (c != mw) store_word_plain<DT>(mrow, npx, c);
    }
}

// ------------------------------------------------------ fixed-point check
// Counts the pixels c that a neighbour p could still raise:
// min(m[p], mask[c]) > m[c].  Zero on every reconstruction (it is a fixed
// point of the propagation rule, MR.cu:43-44); a size-independent check for
// images too large for a CPU comparison.
template <int DT>
__global__ void fixed_point_kernel(ImgDesc d, unsigned long long* count) {
    using P = Px<DT>;
    const long long total = (long long)d.W * d.H;
    unsigned long long mine = 0ull;
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < total;
         i += (long long)gridDim.x * blockDim.x) {
        const int y = (int)(i / d.W), x = (int)(i - (long long)y * d.W);
        const unsigned char* mrow = d.marker + (size_t)y * d.pitch_m;
        const uint32_t m = P::ld_px(mrow + (size_t)x * P::BPP);
        const uint32_t k = P::ld_px(d.mask + (size_t)y * d.pitch_k + (size_t)x * P::BPP);
        if (!P::gt(k, m)) continue;  // m == mask[c] (or above it): nothing can raise it
        uint32_t best = P::MINPX;
        for (int dy = -1; dy <= 1; ++dy) {
            const int yy = y + dy;
            if (yy < 0 || yy >= d.H) continue;
            const unsigned char* row = d.marker + (size_t)yy * d.pitch_m;
            for (int dx = -1; dx <= 1; ++dx) {
                const int xx = x + dx;
                if ((dx == 0 && dy == 0) || xx < 0 || xx >= d.W) continue;
                if (d.conn == 4 && dx != 0 && dy != 0) continue;
                best = P::mx(best, P::ld_px(row + (size_t)xx * P::BPP));
            }
        }
        if (P::gt(P::mn(best, k), m)) ++mine;
    }
    const unsigned long long warp_sum = __reduce_add_sync(0xffffffffu, (unsigned)mine);
    if ((threadIdx.x & 31) == 0 && warp_sum) atomicAdd(count, warp_sum);
}

// --------------------------------------------------------------- X sweeps
// Chunks a warp keeps in flight ahead of the one it scans: the row's loads
// do not depend on the carry, so they are issued kXAhead chunks early into a
// register ring (the walk is otherwise one global-memory latency per chunk).
// A chunk is loaded before any store of this warp to it, and no other warp
// touches the row, so no load reads a value this sweep has replaced.
// Measured on 16384^2 rows: 2 ahead takes 14-24 % off a uint8 / uint16
// sweep and 5 % off int32; 4 or 8 ahead gain less (int32: lose).
constexpr int kXAhead = 2;

template <int DT, bool FWD>
__global__ void sweep_x_kernel(ImgDesc d) {
    if (gated_off(d)) return;
    using P = Px<DT>;
    constexpr int TW = 32 * P::PPW;
    const int lane = threadIdx.x & 31;
    const int row = (int)((blockIdx.x * blockDim.x + threadIdx.x) >> 5);
    if (row >= d.H) return;
    const int chunks = (d.W + TW - 1) / TW;
    unsigned char* mbase = d.marker + (size_t)row * d.pitch_m;
    const unsigned char* kbase = d.mask + (size_t)row * d.pitch_k;
    // chunk cc in walk order: its first pixel for this lane and how many of
    // the lane's pixels lie inside the row
    auto px0_of = [&](int cc) { return (FWD ? cc : chunks - 1 - cc) * TW + lane * P::PPW; };
    auto fetch = [&](int cc, uint32_t& mw, uint32_t& kw) {
        mw = P::MINW;
        kw = P::MINW;
        if (cc >= chunks) return;
        const int px0 = px0_of(cc), npx = d.W - px0;
        if (npx > 0) load_pair<DT>(mbase + (size_t)px0 * P::BPP, kbase + (size_t)px0 * P::BPP, npx, mw, kw);
    };
    uint32_t mq[kXAhead], kq[kXAhead];
#pragma unroll
    for (int q = 0; q < kXAhead; ++q) fetch(q, mq[q], kq[q]);
    uint32_t carry = P::MINPX;
    for (int c0 = 0; c0 < chunks; c0 += kXAhead) {
#pragma unroll
        for (int q = 0; q < kXAhead; ++q) {
            const int cc = c0 + q;
            if (cc >= chunks) break;  // warp-uniform
            const uint32_t mw = mq[q], kw = kq[q];
            fetch(cc + kXAhead, mq[q], kq[q]);
            uint32_t m[P::PPW], k[P::PPW];
            P::unpack(mw, m);
            P::unpack(kw, k);
            hscan<DT, FWD>(m, k, carry, lane);
            const uint32_t nw = P::pack(m);
            const int px0 = px0_of(cc), npx = d.W - px0;
            if (npx > 0 && nw != mw) store_word_plain<DT>(mbase + (size_t)px0 * P::BPP, npx, nw);
            carry = FWD ? __shfl_sync(FULL, m[P::PPW - 1], 31) : __shfl_sync(FULL, m[0], 0);
        }
    }
}

// The same sweep with 16-byte lanes (a warp chunk is 512 bytes): the lane's
// four words are scanned in registers and the warp's clamp-map composition
// runs once per 16 bytes instead of once per 4, which is what the 4-byte form
// spends its issue slots on.  Rows must start on 16-byte boundaries (base
// and pitch of both planes); the row's last partial lane is loaded and
// stored word by word.
template <int DT, bool FWD>
__global__ void sweep_x16_kernel(ImgDesc d) {
    if (gated_off(d)) return;
    using P = Px<DT>;
    constexpr int WPL = 4;             // words per lane
    constexpr int N = WPL * P::PPW;    // pixels per lane
    constexpr int CW = 32 * N;         // pixels per chunk
    const int lane = threadIdx.x & 31;
    const int row = (int)((blockIdx.x * blockDim.x + threadIdx.x) >> 5);
    if (row >= d.H) return;
    const int chunks = (d.W + CW - 1) / CW;
    unsigned char* mbase = d.marker + (size_t)row * d.pitch_m;
    const unsigned char* kbase = d.mask + (size_t)row * d.pitch_k;
    auto px0_of = [&](int cc) { return (FWD ? cc : chunks - 1 - cc) * CW + lane * N; };
    auto fetch = [&](int cc, uint4& mv, uint4& kv) {
        mv = make_uint4(P::MINW, P::MINW, P::MINW, P::MINW);
        kv = mv;
        if (cc >= chunks) return;
        const int px0 = px0_of(cc), npx = d.W - px0;
        if (npx >= N) {
            mv = __ldcg(reinterpret_cast<const uint4*>(mbase + (size_t)px0 * P::BPP));
            kv = __ldg(reinterpret_cast<const uint4*>(kbase + (size_t)px0 * P::BPP));
        } else if (npx > 0) {
            uint32_t mw[WPL], kw[WPL];
#pragma unroll
            for (int w = 0; w < WPL; ++w) {
                const int n = npx - w * P::PPW;
                mw[w] = P::MINW;
                kw[w] = P::MINW;
                if (n > 0)
                    load_pair<DT>(mbase + (size_t)(px0 + w * P::PPW) * P::BPP,
                                  kbase + (size_t)(px0 + w * P::PPW) * P::BPP, n, mw[w], kw[w]);
            }
            mv = make_uint4(mw[0], mw[1], mw[2], mw[3]);
            kv = make_uint4(kw[0], kw[1], kw[2], kw[3]);
        }
    };
    uint4 mq[kXAhead], kq[kXAhead];
#pragma unroll
    for (int q = 0; q < kXAhead; ++q) fetch(q, mq[q], kq[q]);
    uint32_t carry = P::MINPX;
    for (int c0 = 0; c0 < chunks; c0 += kXAhead) {
#pragma unroll
        for (int q = 0; q < kXAhead; ++q) {
            const int cc = c0 + q;
            if (cc >= chunks) break;  // warp-uniform
            const uint4 mv = mq[q], kv = kq[q];
            fetch(cc + kXAhead, mq[q], kq[q]);
            const uint32_t mw[WPL] = {mv.x, mv.y, mv.z, mv.w}, kw[WPL] = {kv.x, kv.y, kv.z, kv.w};
            uint32_t m[N], k[N];
#pragma unroll
            for (int w = 0; w < WPL; ++w) {
                uint32_t a[P::PPW], b[P::PPW];
                P::unpack(mw[w], a);
                P::unpack(kw[w], b);
#pragma unroll
                for (int j = 0; j < P::PPW; ++j) {
                    m[w * P::PPW + j] = a[j];
                    k[w * P::PPW + j] = b[j];
                }
            }
            hscan<DT, FWD, N>(m, k, carry, lane);
            uint32_t nw[WPL];
            bool chg = false;
#pragma unroll
            for (int w = 0; w < WPL; ++w) {
                uint32_t a[P::PPW];
#pragma unroll
                for (int j = 0; j < P::PPW; ++j) a[j] = m[w * P::PPW + j];
                nw[w] = P::pack(a);
                chg |= nw[w] != mw[w];
            }
            const int px0 = px0_of(cc), npx = d.W - px0;
            if (chg && npx > 0) {
                unsigned char* dst = mbase + (size_t)px0 * P::BPP;
                if (npx >= N) {
                    *reinterpret_cast<uint4*>(dst) = make_uint4(nw[0], nw[1], nw[2], nw[3]);
                } else {
#pragma unroll
                    for (int w = 0; w < WPL; ++w)
                        if (npx - w * P::PPW > 0) store_word_plain<DT>(dst + w * 4, npx - w * P::PPW, nw[w]);
                }
            }
            carry = FWD ? __shfl_sync(FULL, m[N - 1], 31) : __shfl_sync(FULL, m[0], 0);
        }
    }
}

// The same sweep over two rows per warp (uint8; the pairing also holds for
// uint16).  Pixel j of a lane's 16 bytes in both rows shares one word as
// u16x2 (first row low), so the in-lane scan, the carry vote and the
// clamp-map scan (hscan_pairs) run once for the two rows: about half the
// issue slots of two sweep_x16_kernel rows.  An odd image's last warp has no
// second row: it reads as the minimum and is not stored.
template <int DT, bool FWD>
__global__ void sweep_x16p_kernel(ImgDesc d) {
    if (gated_off(d)) return;
    using P = Px<DT>;
    static_assert(DT != DT_I32, "int32 rows are not paired");
    constexpr int WPL = 4;             // words per lane
    constexpr int N = WPL * P::PPW;    // pixels per lane (and pair words)
    constexpr int CW = 32 * N;         // pixels per chunk
    const int lane = threadIdx.x & 31;
    const int ra = (int)((blockIdx.x * blockDim.x + threadIdx.x) >> 5) * 2, rb = ra + 1;
    if (ra >= d.H) return;
    const bool has_b = rb < d.H;
    const int chunks = (d.W + CW - 1) / CW;
    unsigned char* ma = d.marker + (size_t)ra * d.pitch_m;
    const unsigned char* ka = d.mask + (size_t)ra * d.pitch_k;
    unsigned char* mb = has_b ? ma + d.pitch_m : ma;
    const unsigned char* kb = has_b ? ka + d.pitch_k : ka;
    auto px0_of = [&](int cc) { return (FWD ? cc : chunks - 1 - cc) * CW + lane * N; };
    auto fetch_row = [&](const unsigned char* mrow, const unsigned char* krow, bool live, int cc, uint4& mv,
                         uint4& kv) {
        mv = make_uint4(P::MINW, P::MINW, P::MINW, P::MINW);
        kv = mv;
        if (cc >= chunks || !live) return;
        const int px0 = px0_of(cc), npx = d.W - px0;
        if (npx >= N) {
            mv = __ldcg(reinterpret_cast<const uint4*>(mrow + (size_t)px0 * P::BPP));
            kv = __ldg(reinterpret_cast<const uint4*>(krow + (size_t)px0 * P::BPP));
        } else if (npx > 0) {
            uint32_t mw[WPL], kw[WPL];
#pragma unroll
            for (int w = 0; w < WPL; ++w) {
                const int n = npx - w * P::PPW;
                mw[w] = P::MINW;
                kw[w] = P::MINW;
                if (n > 0)
                    load_pair<DT>(mrow + (size_t)(px0 + w * P::PPW) * P::BPP,
                                  krow + (size_t)(px0 + w * P::PPW) * P::BPP, n, mw[w], kw[w]);
            }
            mv = make_uint4(mw[0], mw[1], mw[2], mw[3]);
            kv = make_uint4(kw[0], kw[1], kw[2], kw[3]);
        }
    };
    auto store_row = [&](unsigned char* mrow, int cc, const uint32_t (&nw)[WPL]) {
        const int px0 = px0_of(cc), npx = d.W - px0;
        if (npx <= 0) return;
        unsigned char* dst = mrow + (size_t)px0 * P::BPP;
        if (npx >= N) {
            *reinterpret_cast<uint4*>(dst) = make_uint4(nw[0], nw[1], nw[2], nw[3]);
        } else {
#pragma unroll
            for (int w = 0; w < WPL; ++w)
                if (npx - w * P::PPW > 0) store_word_plain<DT>(dst + w * 4, npx - w * P::PPW, nw[w]);
        }
    };
    uint4 maq[kXAhead], kaq[kXAhead], mbq[kXAhead], kbq[kXAhead];
#pragma unroll
    for (int q = 0; q < kXAhead; ++q) {
        fetch_row(ma, ka, true, q, maq[q], kaq[q]);
        fetch_row(mb, kb, has_b, q, mbq[q], kbq[q]);
    }
    uint32_t carry[1] = {0u};  // both rows' entry pixel: the minimum
    for (int c0 = 0; c0 < chunks; c0 += kXAhead) {
#pragma unroll
        for (int q = 0; q < kXAhead; ++q) {
            const int cc = c0 + q;
            if (cc >= chunks) break;  // warp-uniform
            const uint4 mav = maq[q], kav = kaq[q], mbv = mbq[q], kbv = kbq[q];
            fetch_row(ma, ka, true, cc + kXAhead, maq[q], kaq[q]);
            fetch_row(mb, kb, has_b, cc + kXAhead, mbq[q], kbq[q]);
            const uint32_t wa[WPL] = {mav.x, mav.y, mav.z, mav.w}, wb[WPL] = {mbv.x, mbv.y, mbv.z, mbv.w};
            const uint32_t va[WPL] = {kav.x, kav.y, kav.z, kav.w}, vb[WPL] = {kbv.x, kbv.y, kbv.z, kbv.w};
            uint32_t m[1][N], k[1][N];
#pragma unroll
            for (int w = 0; w < WPL; ++w) {
                uint32_t pm[P::PPW], pk[P::PPW];
                pair_pack<DT>(wa[w], wb[w], pm);
                pair_pack<DT>(va[w], vb[w], pk);
#pragma unroll
                for (int j = 0; j < P::PPW; ++j) {
                    m[0][w * P::PPW + j] = pm[j];
                    k[0][w * P::PPW + j] = pk[j];
                }
            }
            hscan_pairs<FWD, 1, N>(m, k, carry, lane);
            uint32_t na[WPL], nb[WPL];
            bool chg_a = false, chg_b = false;
#pragma unroll
            for (int w = 0; w < WPL; ++w) {
                uint32_t pm[P::PPW];
#pragma unroll
                for (int j = 0; j < P::PPW; ++j) pm[j] = m[0][w * P::PPW + j];
                pair_unpack<DT>(pm, na[w], nb[w]);
                chg_a |= na[w] != wa[w];
                chg_b |= nb[w] != wb[w];
            }
            if (chg_a) store_row(ma, cc, na);
            if (chg_b && has_b) store_row(mb, cc, nb);
            carry[0] = FWD ? __shfl_sync(FULL, m[0][N - 1], 31) : __shfl_sync(FULL, m[0][0], 0);
        }
    }
}

// --------------------------------------------------------------- Y sweeps
// 4-byte asynchronous global -> shared copy (cp.async, LDGSTS) and its
// group bookkeeping.
__device__ __forceinline__ void cp_async4(void* smem_dst, const void* gmem_src) {
    asm volatile("cp.async.ca.shared.global [%0], [%1], 4;" ::"r"(smem_u32(smem_dst)), "l"(gmem_src) : "memory");
}
__device__ __forceinline__ void cp_async16(void* smem_dst, const void* gmem_src) {
    asm volatile("cp.async.cg.shared.global [%0], [%1], 16;" ::"r"(smem_u32(smem_dst)), "l"(gmem_src) : "memory");
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;" ::: "memory"); }
template <int N>
__device__ __forceinline__ void cp_async_wait() {
    asm volatile("cp.async.wait_group %0;" ::"n"(N) : "memory");
}

// One warp per 128-byte column strip, walking the full height.  The chain
// through the rows is a few operations per row; memory latency is hidden by
// a ring of kRing rows per plane in shared memory, filled with cp.async
// kRing rows ahead (groups of kGroup rows).  Each lane reads and writes its
// own word of every row only, so no row is read after this thread wrote it.
constexpr int kRing = 64, kGroup = 8;

template <int DT, int CONN, bool DOWN>
__global__ void __launch_bounds__(32) sweep_y_kernel(ImgDesc d) {
    if (gated_off(d)) return;
    using P = Px<DT>;
    constexpr int TW = 32 * P::PPW;
    constexpr int N = P::PPW;
    constexpr int NG = kRing / kGroup;
    __shared__ uint32_t ring_m[kRing][32];
    __shared__ uint32_t ring_k[kRing][32];
    const int lane = threadIdx.x & 31;
    const int strip = (int)blockIdx.x;
    const int strips = (d.W + TW - 1) / TW;
    if (strip >= strips) return;
    const int px0 = strip * TW + lane * P::PPW, npx = d.W - px0;
    const size_t off = (size_t)(npx > 0 ? px0 : 0) * P::BPP;
    const int H = d.H;
    auto row_of = [&](int i) { return DOWN ? i : H - 1 - i; };
    // row i (in sweep order) into slot i % kRing: a full word asynchronously,
    // a partial word (right edge) or a word past the image by plain loads
    auto issue = [&](int i) {
        const int slot = i % kRing;
        if (i >= H) return;
        const int y = row_of(i);
        const unsigned char* mrow = d.marker + (size_t)y * d.pitch_m + off;
        const unsigned char* krow = d.mask + (size_t)y * d.pitch_k + off;
        if (npx >= P::PPW) {
            cp_async4(&ring_m[slot][lane], mrow);
            cp_async4(&ring_k[slot][lane], krow);
        } else {
            uint32_t mw = P::MINW, kw = P::MINW;
            if (npx > 0) load_pair<DT>(mrow, krow, npx, mw, kw);
            ring_m[slot][lane] = mw;
            ring_k[slot][lane] = kw;
        }
    };
    for (int g = 0; g < NG; ++g) {
        for (int q = 0; q < kGroup; ++q) issue(g * kGroup + q);
        cp_async_commit();
    }
    uint32_t prev[N];
#pragma unroll
    for (int j = 0; j < N; ++j) prev[j] = P::MINPX;
    for (int base = 0; base < H; base += kGroup) {
        cp_async_wait<NG - 1>();  // the group holding rows base .. base + kGroup - 1
        __syncwarp();
        // Straight-line code for the group: all ring reads first, then the
        // chain through the rows (two operations per pixel), then the
        // stores; rows past the image are computed on stale slots and not
        // stored.
        const int sb = base % kRing;
        uint32_t mw[kGroup], kw[kGroup], out[kGroup];
#pragma unroll
        for (int q = 0; q < kGroup; ++q) {
            mw[q] = ring_m[sb + q][lane];
            kw[q] = ring_k[sb + q][lane];
        }
#pragma unroll
        for (int q = 0; q < kGroup; ++q) {
            uint32_t m[N], k[N];
            P::unpack(mw[q], m);
            P::unpack(kw[q], k);
            if (CONN == 8) {
                uint32_t left = __shfl_up_sync(FULL, prev[N - 1], 1), right = __shfl_down_sync(FULL, prev[0], 1);
                if (lane == 0) left = P::MINPX;
                if (lane == 31) right = P::MINPX;
#pragma unroll
                for (int j = 0; j < N; ++j) {
                    const uint32_t a = j == 0 ? left : prev[j - 1];
                    const uint32_t b = j == N - 1 ? right : prev[j + 1];
                    m[j] = P::mx(m[j], P::mn(P::mx3(a, prev[j], b), k[j]));
                }
            } else {
#pragma unroll
                for (int j = 0; j < N; ++j) m[j] = P::mx(m[j], P::mn(prev[j], k[j]));
            }
            out[q] = P::pack(m);
#pragma unroll
            for (int j = 0; j < N; ++j) prev[j] = m[j];
        }
#pragma unroll
        for (int q = 0; q < kGroup; ++q)
            if (base + q < H && npx > 0 && out[q] != mw[q])
                store_word_plain<DT>(d.marker + (size_t)row_of(base + q) * d.pitch_m + off, npx, out[q]);
        __syncwarp();  // the slots just read are refilled next
        for (int q = 0; q < kGroup; ++q) issue(base + kRing + q);
        cp_async_commit();
    }
    cp_async_wait<0>();
}

// Vertical sweep for 4-connectivity, int32 (the whole-image init passes use
// the 4-connected vertical sweeps for either connectivity: the pixel above /
// below alone is a valid update).  One pixel per lane, 128-byte strips,
// segments and modes as in sweep_y4n_kernel below.
template <bool DOWN, int MODE>
__global__ void __launch_bounds__(32) sweep_y4i_kernel(ImgDesc d, uint32_t* seg_a, uint32_t* seg_b,
                                                       const uint32_t* seg_in);

constexpr int kRingN = 64;  // rows in flight per plane in the narrow variant

// Narrow variant for uint8 / uint16: a warp covers a 64-byte strip, two
// bytes per lane (uint8: two pixels as one u16x2 register; uint16: one
// pixel), so the chain per row is one min and one max, and twice as many
// warps share the image.
//
// Tall images are cut into segments of kSegRows rows so that more warps
// share each column: the update of one column over a run of rows is
// x -> max(min(x, B), A) for the value x entering the run (A = the run's
// last value when nothing enters, B = the minimum of the mask over the run),
// and such maps compose.  MODE 1 computes (A, B) per segment and column
// without storing; sweep_y_carry_kernel chains them into the value entering
// each segment; MODE 2 sweeps every segment from that value and stores.
// MODE 0 is one warp over the whole column.
constexpr int kSegRows = 1024;

template <int DT, bool DOWN, int MODE>
__global__ void __launch_bounds__(32) sweep_y4n_kernel(ImgDesc d, uint32_t* seg_a, uint32_t* seg_b,
                                                       const uint32_t* seg_in) {
    if (gated_off(d)) return;
    static_assert(DT == DT_U8 || DT == DT_U16, "two-byte lanes");
    using P = Px<DT>;
    constexpr int NR = kRingN, NG = kRingN / kGroup;
    __shared__ __align__(16) uint16_t ring_m[kRingN][32];
    __shared__ __align__(16) uint16_t ring_k[kRingN][32];
    const int lane = threadIdx.x & 31;
    const int strip = (int)blockIdx.x;
    const long long row_bytes = (long long)d.W * P::BPP;
    const long long b0 = (long long)strip * 64 + lane * 2;  // this lane's first byte in a row
    const long long nbytes = row_bytes - b0;                 // >= 2: whole element, 1: half, <= 0: none
    // rows (in sweep order) of this block's segment
    const int i0 = MODE == 0 ? 0 : (int)blockIdx.y * kSegRows;
    const int H = MODE == 0 ? d.H : min(kSegRows, d.H - i0);
    const size_t seg_idx = ((size_t)blockIdx.y * gridDim.x + strip) * 32 + lane;
    const long long step_m = DOWN ? d.pitch_m : -d.pitch_m, step_k = DOWN ? d.pitch_k : -d.pitch_k;
    const unsigned char* m0 = d.marker + (size_t)(DOWN ? 0 : d.H - 1) * d.pitch_m + (long long)i0 * step_m;
    const unsigned char* k0 = d.mask + (size_t)(DOWN ? 0 : d.H - 1) * d.pitch_k + (long long)i0 * step_k;
    const bool wide = (long long)(strip + 1) * 64 <= row_bytes &&
                      ((reinterpret_cast<uintptr_t>(d.marker) | reinterpret_cast<uintptr_t>(d.mask)) & 15u) == 0u &&
                      ((d.pitch_m | d.pitch_k) & 15) == 0;
    auto issue_group = [&](int g0) {
        if (wide) {  // 4 pieces of 16 bytes per row and plane, 8 rows per instruction
            const int piece = lane & 3;
            const int rr = lane >> 2;
            const int i = g0 + rr;
            if (i < H) {
                const int slot = i % NR;
                const long long o = (long long)strip * 64 + piece * 16;
                cp_async16(&ring_m[slot][piece * 8], m0 + (long long)i * step_m + o);
                cp_async16(&ring_k[slot][piece * 8], k0 + (long long)i * step_k + o);
            }
        } else {
            for (int q = 0; q < kGroup; ++q) {
                const int i = g0 + q;
                if (i >= H) break;
                const int slot = i % NR;
                const unsigned char* mrow = m0 + (long long)i * step_m + (nbytes > 0 ? b0 : 0);
                const unsigned char* krow = k0 + (long long)i * step_k + (nbytes > 0 ? b0 : 0);
                uint16_t mv = 0, kv = 0;
                if (nbytes >= 2) {
                    mv = *reinterpret_cast<const uint16_t*>(mrow);
                    kv = *reinterpret_cast<const uint16_t*>(krow);
                } else if (nbytes == 1) {  // uint8 only: the last pixel of the row
                    mv = *mrow;
                    kv = *krow;
                }
                ring_m[slot][lane] = mv;
                ring_k[slot][lane] = kv;
            }
        }
    };
    for (int g = 0; g < NG; ++g) {
        issue_group(g * kGroup);
        cp_async_commit();
    }
    uint32_t prev = MODE == 2 ? seg_in[seg_idx] : 0u;
    uint32_t kmin = DT == DT_U8 ? 0x00ff00ffu : 0xffffu;
    unsigned char* mo = const_cast<unsigned char*>(m0) + (nbytes > 0 ? b0 : 0);
    for (int base = 0; base < H; base += kGroup) {
        cp_async_wait<NG - 1>();
        __syncwarp();
        const int sb = base % NR;
        uint32_t out[kGroup], orig[kGroup];
#pragma unroll
        for (int q = 0; q < kGroup; ++q) {
            uint32_t m = ring_m[sb + q][lane], k = ring_k[sb + q][lane];
            orig[q] = m;
            const bool live = base + q < H;  // rows past the segment: stale slots
            if (DT == DT_U8) {
                m = __byte_perm(m, 0u, 0x4140);
                k = __byte_perm(k, 0u, 0x4140);
                const uint32_t v = __vmaxu2(m, __vminu2(prev, k));
                if (MODE == 1) {
                    if (live) {
                        prev = v;
                        kmin = __vminu2(kmin, k);
                    }
                } else {
                    prev = v;
                }
                out[q] = __byte_perm(v, 0u, 0x0020);
            } else {
                const uint32_t v = max(m, min(prev, k));
                if (MODE == 1) {
                    if (live) {
                        prev = v;
                        kmin = min(kmin, k);
                    }
                } else {
                    prev = v;
                }
                out[q] = v;
            }
        }
        if (MODE != 1) {
            // only the elements that rose are stored: an unchanged store
            // would still dirty its L2 sector and cost a DRAM write-back
            if (nbytes >= 2) {
#pragma unroll
                for (int q = 0; q < kGroup; ++q)
                    if (base + q < H && out[q] != orig[q])
                        *reinterpret_cast<uint16_t*>(mo + (long long)(base + q) * step_m) = (uint16_t)out[q];
            } else if (nbytes == 1) {
                for (int q = 0; q < kGroup; ++q)
                    if (base + q < H && (out[q] & 0xffu) != (orig[q] & 0xffu))
                        *(mo + (long long)(base + q) * step_m) = (unsigned char)out[q];
            }
        }
        __syncwarp();
        issue_group(base + NR);
        cp_async_commit();
    }
    cp_async_wait<0>();
    if (MODE == 1) {
        seg_a[seg_idx] = prev;
        seg_b[seg_idx] = kmin;
    }
}

template <bool DOWN, int MODE>
__global__ void __launch_bounds__(32) sweep_y4i_kernel(ImgDesc d, uint32_t* seg_a, uint32_t* seg_b,
                                                       const uint32_t* seg_in) {
    if (gated_off(d)) return;
    constexpr int NG = kRing / kGroup;
    __shared__ __align__(16) uint32_t ring_m[kRing][32];
    __shared__ __align__(16) uint32_t ring_k[kRing][32];
    const int lane = threadIdx.x & 31;
    const int strip = (int)blockIdx.x;
    const int x = strip * 32 + lane;
    const bool inside = x < d.W;
    const int i0 = MODE == 0 ? 0 : (int)blockIdx.y * kSegRows;
    const int H = MODE == 0 ? d.H : min(kSegRows, d.H - i0);
    const size_t seg_idx = ((size_t)blockIdx.y * gridDim.x + strip) * 32 + lane;
    const long long step_m = DOWN ? d.pitch_m : -d.pitch_m, step_k = DOWN ? d.pitch_k : -d.pitch_k;
    const unsigned char* m0 = d.marker + (size_t)(DOWN ? 0 : d.H - 1) * d.pitch_m + (long long)i0 * step_m;
    const unsigned char* k0 = d.mask + (size_t)(DOWN ? 0 : d.H - 1) * d.pitch_k + (long long)i0 * step_k;
    const long long sbase = (long long)strip * 128;
    const bool wide = (long long)(strip + 1) * 32 <= (long long)d.W &&
                      ((reinterpret_cast<uintptr_t>(d.marker) | reinterpret_cast<uintptr_t>(d.mask)) & 15u) == 0u &&
                      ((d.pitch_m | d.pitch_k) & 15) == 0;
    auto issue_group = [&](int g0) {
        if (wide) {  // 8 pieces of 16 bytes per row and plane, 4 rows per instruction
            const int piece = lane & 7;
#pragma unroll
            for (int rr = 0; rr < kGroup; rr += 4) {
                const int i = g0 + rr + (lane >> 3);
                if (i < H) {
                    const int slot = i % kRing;
                    cp_async16(&ring_m[slot][piece * 4], m0 + (long long)i * step_m + sbase + piece * 16);
                    cp_async16(&ring_k[slot][piece * 4], k0 + (long long)i * step_k + sbase + piece * 16);
                }
            }
        } else {
            for (int q = 0; q < kGroup; ++q) {
                const int i = g0 + q;
                if (i >= H) break;
                const int slot = i % kRing;
                uint32_t mv = 0x80000000u, kv = 0x80000000u;
                if (inside) {
                    mv = *reinterpret_cast<const uint32_t*>(m0 + (long long)i * step_m + (long long)x * 4);
                    kv = *reinterpret_cast<const uint32_t*>(k0 + (long long)i * step_k + (long long)x * 4);
                }
                ring_m[slot][lane] = mv;
                ring_k[slot][lane] = kv;
            }
        }
    };
    for (int g = 0; g < NG; ++g) {
        issue_group(g * kGroup);
        cp_async_commit();
    }
    int prev = MODE == 2 ? (int)seg_in[seg_idx] : INT_MIN;
    int kmin = INT_MAX;
    unsigned char* mo = const_cast<unsigned char*>(m0) + (long long)(inside ? x : 0) * 4;
    for (int base = 0; base < H; base += kGroup) {
        cp_async_wait<NG - 1>();
        __syncwarp();  // pieces copied by other lanes are visible to this one
        const int sb = base % kRing;
        int out[kGroup];
#pragma unroll
        for (int q = 0; q < kGroup; ++q) {
            const int m = (int)ring_m[sb + q][lane], k = (int)ring_k[sb + q][lane];
            const int v = max(m, min(prev, k));
            if (MODE == 1) {
                if (base + q < H) {  // rows past the segment: stale slots
                    prev = v;
                    kmin = min(kmin, k);
                }
            } else {
                prev = v;
            }
            out[q] = v;
        }
        if (MODE != 1 && inside) {
#pragma unroll
            for (int q = 0; q < kGroup; ++q)
                if (base + q < H) *reinterpret_cast<int*>(mo + (long long)(base + q) * step_m) = out[q];
        }
        __syncwarp();  // the slots just read are refilled next
        issue_group(base + kRing);
        cp_async_commit();
    }
    cp_async_wait<0>();
    if (MODE == 1) {
        seg_a[seg_idx] = (uint32_t)prev;
        seg_b[seg_idx] = (uint32_t)kmin;
    }
}

// The value entering every segment of every column: x_0 = nothing (0),
// x_{j+1} = max(min(x_j, B_j), A_j).  One thread per lane slot of a strip.
template <int DT>
__global__ void sweep_y_carry_kernel(int nseg, int slots, const uint32_t* seg_a, const uint32_t* seg_b,
                                     uint32_t* seg_in) {
    const int t = (int)(blockIdx.x * blockDim.x + threadIdx.x);
    if (t >= slots) return;
    uint32_t x = DT == DT_I32 ? 0x80000000u : 0u;
    for (int j = 0; j < nseg; ++j) {
        const size_t idx = (size_t)j * slots + t;
        seg_in[idx] = x;
        if (DT == DT_U8)
            x = __vmaxu2(__vminu2(x, seg_b[idx]), seg_a[idx]);
        else if (DT == DT_U16)
            x = max(min(x, seg_b[idx]), seg_a[idx]);
        else
            x = (uint32_t)max(min((int)x, (int)seg_b[idx]), (int)seg_a[idx]);
    }
}

// int32 is not segmented: at four bytes a pixel the two extra plane reads
// cost more than the parallelism gains (its strips already give 512 warps
// on a 16384-wide image).
size_t sweep_scratch_bytes(const ImgDesc& d) {
    if (d.conn != 4 || d.dtype == DT_I32 || d.H <= 2 * kSegRows) return 0;
    const long long strips = d.dtype == DT_I32 ? ((long long)d.W + 31) / 32
                                               : ((long long)d.W * (d.dtype == DT_U8 ? 1 : 2) + 63) / 64;
    const long long nseg = (d.H + kSegRows - 1) / kSegRows;
    return (size_t)(3 * nseg * strips * 32 * 4);
}

// ------------------------------------------------------------ host side
static unsigned blocks_for(long long threads, int block) {
    long long b = (threads + block - 1) / block;
    if (b < 1) b = 1;
    if (b > (1ll << 30)) b = 1ll << 30;
    return (unsigned)b;
}

cudaError_t launch_fixed_point_check(const ImgDesc& d, unsigned long long* count, cudaStream_t s) {
    if (d.W == 0 || d.H == 0) return cudaSuccess;
    unsigned blocks = blocks_for((long long)d.W * d.H, 256);
    if (blocks > 152u * 16u) blocks = 152u * 16u;
    if (d.dtype == DT_U8)
        fixed_point_kernel<DT_U8><<<blocks, 256, 0, s>>>(d, count);
    else if (d.dtype == DT_U16)
        fixed_point_kernel<DT_U16><<<blocks, 256, 0, s>>>(d, count);
    else
        fixed_point_kernel<DT_I32><<<blocks, 256, 0, s>>>(d, count);
    return cudaGetLastError();
}

cudaError_t launch_clip(const ImgDesc& d, cudaStream_t s) {
    if (d.W == 0 || d.H == 0) return cudaSuccess;
    const int ppw = d.dtype == DT_U8 ? 4 : d.dtype == DT_U16 ? 2 : 1;
    const long long words = (long long)((d.W + ppw - 1) / ppw) * d.H;
    unsigned blocks = blocks_for(words, 256);
    if (blocks > 152u * 16u) blocks = 152u * 16u;
    if (d.dtype == DT_U8)
        clip_kernel<DT_U8><<<blocks, 256, 0, s>>>(d);
    else if (d.dtype == DT_U16)
        clip_kernel<DT_U16><<<blocks, 256, 0, s>>>(d);
    else
        clip_kernel<DT_I32><<<blocks, 256, 0, s>>>(d);
    return cudaGetLastError();
}

template <int DT>
static int launch_sweep_t(const ImgDesc& d, int direction, cudaStream_t s, void* scratch) {
    using P = Px<DT>;
    constexpr int TW = 32 * P::PPW;
    if (direction == 0 || direction == 2) {
        const unsigned blocks = blocks_for((long long)d.H * 32, 128);
        const bool aligned16 =
            ((reinterpret_cast<uintptr_t>(d.marker) | reinterpret_cast<uintptr_t>(d.mask)) & 15u) == 0u &&
            ((d.pitch_m | d.pitch_k) & 15) == 0;
        if (aligned16 && DT == DT_U8) {
            // two rows per warp (uint16 measured no faster: its lanes hold
            // half as many pixels, so the scan is a smaller share)
            const unsigned pblocks = blocks_for((long long)((d.H + 1) / 2) * 32, 128);
            if (direction == 0)
                sweep_x16p_kernel<DT_U8, true><<<pblocks, 128, 0, s>>>(d);
            else
                sweep_x16p_kernel<DT_U8, false><<<pblocks, 128, 0, s>>>(d);
        } else if (aligned16) {
            if (direction == 0)
                sweep_x16_kernel<DT, true><<<blocks, 128, 0, s>>>(d);
            else
                sweep_x16_kernel<DT, false><<<blocks, 128, 0, s>>>(d);
        } else if (direction == 0) {
            sweep_x_kernel<DT, true><<<blocks, 128, 0, s>>>(d);
        } else {
            sweep_x_kernel<DT, false><<<blocks, 128, 0, s>>>(d);
        }
        return 1;
    } else {
        const int strips = (d.W + TW - 1) / TW;
        const unsigned blocks = (unsigned)strips;
        const bool down = direction == 1;
        if (d.conn == 8) {
            if (down)
                sweep_y_kernel<DT, 8, true><<<blocks, 32, 0, s>>>(d);
            else
                sweep_y_kernel<DT, 8, false><<<blocks, 32, 0, s>>>(d);
        } else if (DT == DT_I32) {
            const unsigned nblocks = (unsigned)((d.W + 31) / 32);
            if (scratch && sweep_scratch_bytes(d) > 0) {
                const int nseg = (d.H + kSegRows - 1) / kSegRows;
                const int slots = (int)nblocks * 32;
                uint32_t* a = static_cast<uint32_t*>(scratch);
                uint32_t* b = a + (size_t)nseg * slots;
                uint32_t* in = b + (size_t)nseg * slots;
                const dim3 grid(nblocks, (unsigned)nseg);
                if (down)
                    sweep_y4i_kernel<true, 1><<<grid, 32, 0, s>>>(d, a, b, nullptr);
                else
                    sweep_y4i_kernel<false, 1><<<grid, 32, 0, s>>>(d, a, b, nullptr);
                sweep_y_carry_kernel<DT_I32><<<(unsigned)((slots + 127) / 128), 128, 0, s>>>(nseg, slots, a, b, in);
                if (down)
                    sweep_y4i_kernel<true, 2><<<grid, 32, 0, s>>>(d, nullptr, nullptr, in);
                else
                    sweep_y4i_kernel<false, 2><<<grid, 32, 0, s>>>(d, nullptr, nullptr, in);
                return 3;
            } else if (down) {
                sweep_y4i_kernel<true, 0><<<nblocks, 32, 0, s>>>(d, nullptr, nullptr, nullptr);
            } else {
                sweep_y4i_kernel<false, 0><<<nblocks, 32, 0, s>>>(d, nullptr, nullptr, nullptr);
            }
        } else {
            constexpr int NDT = DT == DT_I32 ? DT_U8 : DT;  // (never i32 here)
            const unsigned nblocks = (unsigned)(((long long)d.W * P::BPP + 63) / 64);
            if (scratch && sweep_scratch_bytes(d) > 0) {
                // segments: aggregate, chain, sweep
                const int nseg = (d.H + kSegRows - 1) / kSegRows;
                const int slots = (int)nblocks * 32;
                uint32_t* a = static_cast<uint32_t*>(scratch);
                uint32_t* b = a + (size_t)nseg * slots;
                uint32_t* in = b + (size_t)nseg * slots;
                const dim3 grid(nblocks, (unsigned)nseg);
                if (down)
                    sweep_y4n_kernel<NDT, true, 1><<<grid, 32, 0, s>>>(d, a, b, nullptr);
                else
                    sweep_y4n_kernel<NDT, false, 1><<<grid, 32, 0, s>>>(d, a, b, nullptr);
                sweep_y_carry_kernel<NDT><<<(unsigned)((slots + 127) / 128), 128, 0, s>>>(nseg, slots, a, b, in);
                if (down)
                    sweep_y4n_kernel<NDT, true, 2><<<grid, 32, 0, s>>>(d, nullptr, nullptr, in);
                else
                    sweep_y4n_kernel<NDT, false, 2><<<grid, 32, 0, s>>>(d, nullptr, nullptr, in);
                return 3;
            } else if (down) {
                sweep_y4n_kernel<NDT, true, 0><<<nblocks, 32, 0, s>>>(d, nullptr, nullptr, nullptr);
            } else {
                sweep_y4n_kernel<NDT, false, 0><<<nblocks, 32, 0, s>>>(d, nullptr, nullptr, nullptr);
            }
        }
        return 1;
    }
}

cudaError_t launch_sweep(const ImgDesc& d, int direction, cudaStream_t s, void* scratch, int* launches) {
    if (d.W == 0 || d.H == 0) return cudaSuccess;
    int n;
    if (d.dtype == DT_U8)
        n = launch_sweep_t<DT_U8>(d, direction, s, scratch);
    else if (d.dtype == DT_U16)
        n = launch_sweep_t<DT_U16>(d, direction, s, scratch);
    else
        n = launch_sweep_t<DT_I32>(d, direction, s, scratch);
    if (launches) *launches += n;
    return cudaGetLastError();
}

}  // namespace iwpp
