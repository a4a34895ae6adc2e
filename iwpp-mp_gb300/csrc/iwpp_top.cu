// iwpp_top.cu -- the front stage: reconstruction of the image's highest level
// set by connected-component labelling; and the check that seeds the tile
// engine with the tiles still violating a constraint after the whole-image
// passes.
//
// Only pixels whose mask is at the image's largest value T can rise in this
// stage; each rises to the largest marker (capped at T) of the connected set
// of such pixels it belongs to (the image's connectivity).  This is the
// reconstruction restricted to that level set, so it never exceeds the full
// reconstruction (every member of a component reaches every other through
// pixels whose mask is T): a valid start for the whole-image passes and the
// tile engine that follow.  The rule is the reference's
// (IWPP MP/src/MorphologicalReconstruction.cu:43-44) applied to closure.
//
// Why: a long path at the top level (a one-pixel corridor spiralling through
// the image) needs one directional sweep per straight run, or one dependent
// tile visit per tile it crosses; labelling finds its component in a fixed
// number of passes over the tiles that hold top-level pixels:
//   1. top_max_kernel: every tile's largest mask value (as an unsigned key)
//      and the image's (T).
//   2. top_local_kernel (one CTA per tile holding T): the tile's top-level
//      pixels compacted into a list, union-find over them in shared memory;
//      each local component gets one of kTopSlots node slots (rootidx: its
//      least pixel index, the root union-by-least-index leaves), its largest
//      capped marker (gmax) and the slots of the tile's edge pixels (edge).
//      A tile with more components than slots leaves the extra ones out
//      (they only keep their own values: still valid).
//   3. top_union_kernel: union of the nodes of top-level pixels that touch
//      across tile edges (and corners with 8-connectivity), a lock-free
//      global union-find (link the larger root under the smaller).
//   4. top_flatten_kernel: every node to its root; each root's gmax the
//      largest of its component.
//   5. top_apply_list_kernel (a warp per tile): each top-level pixel of a
//      tile with at most kTopListCap of them raised to its component's
//      value, from the (pixel, slot) list the local kernel saved;
//      top_apply_label_kernel (a CTA per tile with more): the local
//      labelling again (the roots are the least pixel indices, so it is the
//      same), then the same raise.
#include <vector>

#include "iwpp_engine.cuh"
#include "iwpp_top.cuh"

namespace iwpp {

constexpr int kTopRows = 64;    // rows of a tile (tiles are 128 bytes wide)
constexpr int kTopSlots = 64;   // component nodes one tile can export
constexpr int kTopThreads = 256;
constexpr int kTopListCap = 256;  // (pixel, slot) entries a tile saves for the apply step

// Order-preserving unsigned key of a pixel value (int32 with its sign bit
// flipped), and back.
template <int DT>
__device__ __forceinline__ uint32_t top_key(uint32_t v) { return DT == DT_I32 ? v ^ 0x80000000u : v; }

struct TopArgs {
    ImgDesc d;
    int tx_n, ty_n, tw;      // tiles across, down; pixels per tile row
    int conn;
    unsigned* tmax;          // per tile: largest mask key
    unsigned* thr_key;       // the image's largest mask key
    int* ns;                 // per tile: node slots used
    int* gparent;            // per node (tile * kTopSlots + slot): parent node
    unsigned* gmax;          // per node: largest capped marker key of its component
    unsigned short* rootidx; // per node: the component's least pixel index in its tile
    signed char* edge;       // per tile: left (64), right (64), top (tw), bottom (tw) slot or -1
    int edge_stride;         // 128 + 2 * tw
    int* tn;                 // per tile: its top-level pixels
    unsigned* tlist;         // per tile: kTopListCap entries, pixel | slot << 16 (slot 0xff: none)
    unsigned* ncount;        // [0]: tiles with a saved list, [1]: tiles to label again
    unsigned* listed;        // the tiles with a saved list
    unsigned* relabel;       // the tiles with more top-level pixels than a list holds
    int aligned16;           // mask rows start on 16-byte boundaries
    unsigned long long* top_pixels;  // the job's count of pixels labelled
};

__device__ __forceinline__ int g_find(int* parent, int x) {
    for (;;) {
        const int p = __ldcg(&parent[x]);
        if (p == x) return x;
        const int gp = __ldcg(&parent[p]);
        if (gp != p) atomicCAS(&parent[x], p, gp);  // path halving
        x = gp;
    }
}

__device__ __forceinline__ void g_union(int* parent, int a, int b) {
    for (;;) {
        a = g_find(parent, a);
        b = g_find(parent, b);
        if (a == b) return;
        if (a < b) {
            const int t = a;
            a = b;
            b = t;
        }
        // link the larger root under the smaller
        const int old = atomicCAS(&parent[a], a, b);
        if (old == a) return;
        a = old;
    }
}

// The same in shared memory, over a tile's pixel indices (16 bits).
__device__ __forceinline__ int s_find(unsigned short* parent, int x) {
    for (;;) {
        const int p = *(volatile unsigned short*)&parent[x];
        if (p == x) return x;
        x = p;
    }
}

__device__ __forceinline__ void s_union(unsigned short* parent, int a, int b) {
    for (;;) {
        a = s_find(parent, a);
        b = s_find(parent, b);
        if (a == b) return;
        if (a < b) {
            const int t = a;
            a = b;
            b = t;
        }
        const int old = atomicCAS(&parent[a], (unsigned short)a, (unsigned short)b);
        if (old == a) return;
        a = old;
    }
}

// ------------------------------------------------------------ 1. maxima
// Largest key of a word's pixels (pixels past the row end hold the type's
// least value, key 0).
template <int DT>
__device__ __forceinline__ uint32_t word_max_key(uint32_t w) {
    if (DT == DT_U8) {
        const uint32_t h = __vmaxu4(w, w >> 16);
        return max(h & 0xffu, (h >> 8) & 0xffu);
    } else if (DT == DT_U16) {
        return max(w & 0xffffu, w >> 16);
    } else {
        return w ^ 0x80000000u;
    }
}


// One warp per tile; with 16-byte rows each lane reads 16 bytes of a row
// (8 lanes a row, 4 rows per step), else one word of each row.
template <int DT>
__global__ void top_max_kernel(TopArgs a) {
    if (gated_off(a.d)) return;
    using P = Px<DT>;
    const int lane = threadIdx.x & 31;
    const long long G = (long long)a.tx_n * a.ty_n;
    const long long wg = ((long long)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const long long nw = ((long long)gridDim.x * blockDim.x) >> 5;
    const ImgDesc& d = a.d;
    const long long row_bytes = (long long)d.W * P::BPP;
    for (long long t = wg; t < G; t += nw) {
        const int ty = (int)(t / a.tx_n), tx = (int)(t - (long long)ty * a.tx_n);
        const int y0 = ty * kTopRows, rows = min(kTopRows, d.H - y0);
        uint32_t acc = P::MINW;
        if (a.aligned16) {
            const long long byte0 = (long long)tx * 128 + (lane & 7) * 16;
            if (byte0 < row_bytes) {
                const bool full = byte0 + 16 <= row_bytes;
#pragma unroll 4
                for (int r = lane >> 3; r < rows; r += 4) {
                    const unsigned char* src = d.mask + (size_t)(y0 + r) * d.pitch_k + byte0;
                    if (full) {
                        const uint4 v = __ldg(reinterpret_cast<const uint4*>(src));
                        acc = word_max<DT>(word_max<DT>(acc, v.x), word_max<DT>(word_max<DT>(v.y, v.z), v.w));
                    } else {
#pragma unroll
                        for (int w = 0; w < 4; ++w) {
                            const long long b = byte0 + w * 4;
                            if (b < row_bytes)
                                acc = word_max<DT>(acc, load_word_plain<DT>(src + w * 4,
                                                                            (int)((row_bytes - b) / P::BPP), false));
                        }
                    }
                }
            }
        } else {
            const long long byte0 = (long long)tx * 128 + lane * 4;
            if (byte0 < row_bytes) {
                const int npx = (int)min((long long)P::PPW, (row_bytes - byte0) / P::BPP);
                for (int r = 0; r < rows; ++r)
                    acc = word_max<DT>(acc, load_word_plain<DT>(d.mask + (size_t)(y0 + r) * d.pitch_k + byte0, npx,
                                                                false));
            }
        }
        const uint32_t best = __reduce_max_sync(FULL, word_max_key<DT>(acc));
        if (lane == 0) {
            a.tmax[t] = best;
            atomicMax(a.thr_key, best);
        }
    }
}

// ------------------------------------------------- 2 / 5. local labelling
// Shared memory of a CTA working on one tile: which pixels are at the top
// level (per row, word j bit l: pixel l * PPW + j), the union-find parents
// of those pixels (the others' entries are not written), the list of them,
// the node slot of each root and per slot its component's value.
template <int DT>
struct TopSmem {
    static constexpr int NPX = kTopRows * 32 * Px<DT>::PPW;
    unsigned topbits[kTopRows][Px<DT>::PPW];
    unsigned short parent[NPX];
    unsigned short list[NPX];
    signed char slot[NPX];
    unsigned sval[kTopSlots];  // local: largest capped marker key; apply: the component's
    int warp_count[kTopThreads / 32];
    int nlist;
    int nslots;
};

// Lane words a thread of the labelling CTA covers: word w = threadIdx.x +
// i * kTopThreads is tile row w / 32, lane word w % 32.
constexpr int kTopWpt = kTopRows * 32 / kTopThreads;

// Pixel p of the tile is at the top level.
template <int DT>
__device__ __forceinline__ bool is_top(const TopSmem<DT>& sm, int p) {
    constexpr int TW = 32 * Px<DT>::PPW;
    const int r = p / TW, c = p - r * TW;
    return (sm.topbits[r][c % Px<DT>::PPW] >> (c / Px<DT>::PPW)) & 1u;
}

// The tile's top-level pixels labelled: sm.list[0, sm.nlist) holds them,
// sm.parent[p] the least pixel index of p's component (top-level p only).
// Returns the thread's top-level flags: bit i * PPW + j for pixel j of its
// word i.  All threads of the CTA.
template <int DT>
__device__ unsigned label_tile(const TopArgs& a, int tx, int ty, unsigned tkey, TopSmem<DT>& sm) {
    using P = Px<DT>;
    constexpr int TW = 32 * P::PPW;
    const ImgDesc& d = a.d;
    const int x0 = tx * TW, y0 = ty * kTopRows;
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    // the tile's mask one lane word at a time, all of a thread's words in
    // flight together
    uint32_t kw[kTopWpt];
#pragma unroll
    for (int i = 0; i < kTopWpt; ++i) {
        const int w = threadIdx.x + i * kTopThreads;
        const int y = y0 + (w >> 5), px0 = x0 + (w & 31) * P::PPW;
        kw[i] = y < d.H && px0 < d.W
                    ? load_word_plain<DT>(d.mask + (size_t)y * d.pitch_k + (size_t)px0 * P::BPP, d.W - px0, false)
                    : P::MINW;
    }
    unsigned bits = 0u;
#pragma unroll
    for (int i = 0; i < kTopWpt; ++i) {
        const int w = threadIdx.x + i * kTopThreads;
        const int r = w >> 5, c0 = (w & 31) * P::PPW;
        uint32_t k[P::PPW];
        P::unpack(kw[i], k);
#pragma unroll
        for (int j = 0; j < P::PPW; ++j) {
            const int p = r * TW + c0 + j;
            const bool top = y0 + r < d.H && x0 + c0 + j < d.W && top_key<DT>(k[j]) >= tkey;
            if (top) {
                sm.parent[p] = (unsigned short)p;
                bits |= 1u << (i * P::PPW + j);
            }
            // the warp holds the whole row r: one ballot per pixel position
            const unsigned row_bits = __ballot_sync(FULL, top);
            if (lane == j) sm.topbits[r][j] = row_bits;
        }
    }
    // the list: each thread's place by a CTA-wide exclusive scan of counts
    const int cnt = __popc(bits);
    int incl = cnt;
#pragma unroll
    for (int dd = 1; dd < 32; dd <<= 1) {
        const int v = __shfl_up_sync(FULL, incl, dd);
        if (lane >= dd) incl += v;
    }
    if (lane == 31) sm.warp_count[warp] = incl;
    __syncthreads();
    int pos = incl - cnt;
    for (int q = 0; q < warp; ++q) pos += sm.warp_count[q];
    if (threadIdx.x == kTopThreads - 1) sm.nlist = pos + cnt;
    for (unsigned b = bits; b; b &= b - 1u) {
        const int bit = __ffs(b) - 1;
        const int i = bit / P::PPW, j = bit - i * P::PPW;
        const int w = threadIdx.x + i * kTopThreads;
        sm.list[pos++] = (unsigned short)((w >> 5) * TW + (w & 31) * P::PPW + j);
    }
    __syncthreads();
    const int n = sm.nlist;
    for (int e = threadIdx.x; e < n; e += blockDim.x) {
        const int p = sm.list[e];
        const int r = p / TW, c = p - r * TW;
        if (c > 0 && is_top<DT>(sm, p - 1)) s_union(sm.parent, p, p - 1);
        if (r > 0) {
            if (is_top<DT>(sm, p - TW)) s_union(sm.parent, p, p - TW);
            if (a.conn == 8) {
                if (c > 0 && is_top<DT>(sm, p - TW - 1)) s_union(sm.parent, p, p - TW - 1);
                if (c + 1 < TW && is_top<DT>(sm, p - TW + 1)) s_union(sm.parent, p, p - TW + 1);
            }
        }
    }
    __syncthreads();
    for (int e = threadIdx.x; e < n; e += blockDim.x) {
        const int p = sm.list[e];
        sm.parent[p] = s_find(sm.parent, p);
    }
    __syncthreads();
    return bits;
}

// The thread's marker words that hold a top-level pixel (per `bits`), all in
// flight together; the others are left 0.
template <int DT>
__device__ __forceinline__ void load_top_words(const ImgDesc& d, int tx, int ty, unsigned bits,
                                               uint32_t (&mw)[kTopWpt]) {
    using P = Px<DT>;
    constexpr int TW = 32 * P::PPW;
    constexpr unsigned WMASK = (1u << P::PPW) - 1u;
#pragma unroll
    for (int i = 0; i < kTopWpt; ++i) {
        const int w = threadIdx.x + i * kTopThreads;
        const int y = ty * kTopRows + (w >> 5), px0 = tx * TW + (w & 31) * P::PPW;
        mw[i] = (bits >> (i * P::PPW)) & WMASK
                    ? load_word_plain<DT>(d.marker + (size_t)y * d.pitch_m + (size_t)px0 * P::BPP, d.W - px0, true)
                    : 0u;
    }
}

template <int DT>
__global__ void __launch_bounds__(kTopThreads, 4) top_local_kernel(TopArgs a) {
    if (gated_off(a.d)) return;
    using P = Px<DT>;
    constexpr int TW = 32 * P::PPW;
    extern __shared__ __align__(16) unsigned char top_smem[];
    TopSmem<DT>& sm = *reinterpret_cast<TopSmem<DT>*>(top_smem);
    const ImgDesc& d = a.d;
    const unsigned tkey = *(const volatile unsigned*)a.thr_key;
    const uint32_t tval = top_key<DT>(tkey);
    const long long G = (long long)a.tx_n * a.ty_n;
    for (long long t = blockIdx.x; t < G; t += gridDim.x) {
        if (a.tmax[t] < tkey) continue;  // no top-level pixel (CTA-uniform)
        const int ty = (int)(t / a.tx_n), tx = (int)(t - (long long)ty * a.tx_n);
        if (threadIdx.x == 0) sm.nslots = 0;
        const unsigned bits = label_tile<DT>(a, tx, ty, tkey, sm);
        const int n = sm.nlist;
        // the marker words with top-level pixels in flight while the roots
        // take their node slots
        uint32_t mw[kTopWpt];
        load_top_words<DT>(d, tx, ty, bits, mw);
        for (int e = threadIdx.x; e < n; e += blockDim.x) {
            const int p = sm.list[e];
            if (sm.parent[p] != p) continue;
            const int s = atomicAdd(&sm.nslots, 1);
            sm.slot[p] = s < kTopSlots ? (signed char)s : (signed char)-1;
            if (s < kTopSlots) {
                const long long node = t * kTopSlots + s;
                a.rootidx[node] = (unsigned short)p;
                a.gparent[node] = (int)node;
                sm.sval[s] = 0u;
            }
        }
        __syncthreads();
        // each component's largest marker capped at the level (its mask): a
        // thread's pixels run by component, one shared atomic per run
        constexpr unsigned WMASK = (1u << P::PPW) - 1u;
        int cur = -1;
        unsigned best = 0u;
#pragma unroll
        for (int i = 0; i < kTopWpt; ++i) {
            const unsigned wb = (bits >> (i * P::PPW)) & WMASK;
            if (!wb) continue;
            const int w = threadIdx.x + i * kTopThreads;
            const int pbase = (w >> 5) * TW + (w & 31) * P::PPW;
            uint32_t m[P::PPW];
            P::unpack(mw[i], m);
#pragma unroll
            for (int j = 0; j < P::PPW; ++j) {
                if (!((wb >> j) & 1u)) continue;
                const int s = sm.slot[sm.parent[pbase + j]];
                if (s < 0) continue;
                const unsigned v = top_key<DT>(P::mn(m[j], tval));
                if (s != cur) {
                    if (cur >= 0) atomicMax(&sm.sval[cur], best);
                    cur = s;
                    best = v;
                } else {
                    best = max(best, v);
                }
            }
        }
        if (cur >= 0) atomicMax(&sm.sval[cur], best);
        // the slots of the edge pixels: left and right columns, top and
        // bottom rows (-1: not at the top level, or a component left out)
        signed char* e = a.edge + t * a.edge_stride;
        for (int i = threadIdx.x; i < 128 + 2 * TW; i += blockDim.x) {
            int p;
            if (i < 64) p = i * TW;                          // left column, row i
            else if (i < 128) p = (i - 64) * TW + TW - 1;    // right column
            else if (i < 128 + TW) p = i - 128;              // top row
            else p = (kTopRows - 1) * TW + (i - 128 - TW);   // bottom row
            e[i] = is_top<DT>(sm, p) ? sm.slot[sm.parent[p]] : (signed char)-1;
        }
        // the (pixel, slot) list for the apply step, when it fits
        if (n <= kTopListCap)
            for (int q = threadIdx.x; q < n; q += blockDim.x) {
                const int p = sm.list[q];
                a.tlist[t * kTopListCap + q] = (unsigned)p | ((unsigned)(unsigned char)sm.slot[sm.parent[p]] << 16);
            }
        __syncthreads();
        const int ns = min(sm.nslots, kTopSlots);
        for (int q = threadIdx.x; q < ns; q += blockDim.x) a.gmax[t * kTopSlots + q] = sm.sval[q];
        if (threadIdx.x == 0) {
            a.ns[t] = ns;
            a.tn[t] = n;
            atomicAdd(a.top_pixels, (unsigned long long)n);
            if (n <= kTopListCap)
                a.listed[atomicAdd(&a.ncount[0], 1u)] = (unsigned)t;
            else
                a.relabel[atomicAdd(&a.ncount[1], 1u)] = (unsigned)t;
        }
        __syncthreads();
    }
}

// ------------------------------------------------------ 3. edge unions
// One thread per edge pixel pair of a tile and its right / lower neighbour
// (and the corners for 8-connectivity); both tiles must hold top-level
// pixels (their edge slots are written).
__global__ void top_union_kernel(TopArgs a) {
    if (gated_off(a.d)) return;
    const int TW = a.tw;
    const long long G = (long long)a.tx_n * a.ty_n;
    const int per = 2 * kTopRows + 2 * TW + 2;  // work items per tile
    const unsigned tkey = *(const volatile unsigned*)a.thr_key;
    const long long total = G * per;
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < total;
         i += (long long)gridDim.x * blockDim.x) {
        const long long t = i / per;
        const int k = (int)(i - t * per);
        if (a.tmax[t] < tkey) continue;
        const int ty = (int)(t / a.tx_n), tx = (int)(t - (long long)ty * a.tx_n);
        const signed char* e = a.edge + t * a.edge_stride;
        auto node = [&](long long tile, int s) { return (int)(tile * kTopSlots + s); };
        auto link = [&](int sa, long long tb, int sb) {
            if (sa >= 0 && sb >= 0) g_union(a.gparent, node(t, sa), node(tb, sb));
        };
        if (k < 2 * kTopRows) {
            // right neighbour: this tile's right column against its left column
            if (tx + 1 >= a.tx_n) continue;
            const long long tb = t + 1;
            if (a.tmax[tb] < tkey) continue;
            const signed char* eb = a.edge + tb * a.edge_stride;
            const int r = k >> 1;
            const int sa = e[64 + r];
            if (sa < 0) continue;
            if ((k & 1) == 0) {
                link(sa, tb, eb[r]);
            } else if (a.conn == 8) {
                if (r > 0) link(sa, tb, eb[r - 1]);
                if (r + 1 < kTopRows) link(sa, tb, eb[r + 1]);
            }
        } else if (k < 2 * kTopRows + 2 * TW) {
            // lower neighbour: this tile's bottom row against its top row
            if (ty + 1 >= a.ty_n) continue;
            const long long tb = t + a.tx_n;
            if (a.tmax[tb] < tkey) continue;
            const signed char* eb = a.edge + tb * a.edge_stride;
            const int j = k - 2 * kTopRows;
            const int c = j >> 1;
            const int sa = e[128 + TW + c];
            if (sa < 0) continue;
            if ((j & 1) == 0) {
                link(sa, tb, eb[128 + c]);
            } else if (a.conn == 8) {
                if (c > 0) link(sa, tb, eb[128 + c - 1]);
                if (c + 1 < TW) link(sa, tb, eb[128 + c + 1]);
            }
        } else if (a.conn == 8 && ty + 1 < a.ty_n) {
            // corners: bottom-right pixel to the lower-right tile's top-left,
            // bottom-left pixel to the lower-left tile's top-right
            if (k == 2 * kTopRows + 2 * TW) {
                if (tx + 1 >= a.tx_n) continue;
                const long long tb = t + a.tx_n + 1;
                if (a.tmax[tb] < tkey) continue;
                link(e[128 + TW + TW - 1], tb, a.edge[tb * a.edge_stride + 128]);
            } else {
                if (tx == 0) continue;
                const long long tb = t + a.tx_n - 1;
                if (a.tmax[tb] < tkey) continue;
                link(e[128 + TW], tb, a.edge[tb * a.edge_stride + 128 + TW - 1]);
            }
        }
    }
}

// ---------------------------------------------------------- 4. flatten
__global__ void top_flatten_kernel(TopArgs a) {
    if (gated_off(a.d)) return;
    const long long total = (long long)a.tx_n * a.ty_n * kTopSlots;
    const unsigned tkey = *(const volatile unsigned*)a.thr_key;
    for (long long node = blockIdx.x * (long long)blockDim.x + threadIdx.x; node < total;
         node += (long long)gridDim.x * blockDim.x) {
        const long long t = node / kTopSlots;
        const int s = (int)(node - t * kTopSlots);
        if (a.tmax[t] < tkey || s >= a.ns[t]) continue;
        const int root = g_find(a.gparent, (int)node);
        a.gparent[node] = root;
        if (root != (int)node) atomicMax(&a.gmax[root], __ldcg(&a.gmax[node]));
    }
}

// ------------------------------------------------------------ 5. apply
// Tiles whose list was saved: a warp per tile, a lane per entry; the nodes
// point at their roots after the flatten step.
template <int DT>
__global__ void top_apply_list_kernel(TopArgs a) {
    if (gated_off(a.d)) return;
    using P = Px<DT>;
    constexpr int TW = 32 * P::PPW;
    const int lane = threadIdx.x & 31;
    const ImgDesc& d = a.d;
    const long long count = *(const volatile unsigned*)&a.ncount[0];
    const long long wg = ((long long)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const long long nw = ((long long)gridDim.x * blockDim.x) >> 5;
    for (long long i = wg; i < count; i += nw) {
        const long long t = a.listed[i];
        const int n = a.tn[t];
        const int ty = (int)(t / a.tx_n), tx = (int)(t - (long long)ty * a.tx_n);
        for (int e = lane; e < n; e += 32) {
            const unsigned u = a.tlist[t * kTopListCap + e];
            const unsigned s = u >> 16;
            if (s >= (unsigned)kTopSlots) continue;
            const int p = (int)(u & 0xffffu), r = p / TW, c = p - r * TW;
            const uint32_t v = top_key<DT>(__ldcg(&a.gmax[__ldcg(&a.gparent[t * kTopSlots + s])]));
            unsigned char* px = d.marker + (size_t)(ty * kTopRows + r) * d.pitch_m + (size_t)(tx * TW + c) * P::BPP;
            if (P::gt(v, P::ld_px(px))) P::st_px(px, v);
        }
    }
}

// Tiles with more top-level pixels than the list holds: a CTA per tile
// labels the tile again.
template <int DT>
__global__ void __launch_bounds__(kTopThreads, 4) top_apply_label_kernel(TopArgs a) {
    if (gated_off(a.d)) return;
    using P = Px<DT>;
    constexpr int TW = 32 * P::PPW;
    extern __shared__ __align__(16) unsigned char top_smem[];
    TopSmem<DT>& sm = *reinterpret_cast<TopSmem<DT>*>(top_smem);
    const ImgDesc& d = a.d;
    const unsigned tkey = *(const volatile unsigned*)a.thr_key;
    const long long count = *(const volatile unsigned*)&a.ncount[1];
    for (long long i = blockIdx.x; i < count; i += gridDim.x) {
        const long long t = a.relabel[i];
        const int ty = (int)(t / a.tx_n), tx = (int)(t - (long long)ty * a.tx_n);
        const unsigned bits = label_tile<DT>(a, tx, ty, tkey, sm);
        const int n = sm.nlist;
        uint32_t mw[kTopWpt];
        load_top_words<DT>(d, tx, ty, bits, mw);
        // the slot of each root, from the node table's least pixel indices,
        // and each slot's component value, read once
        const int ns = a.ns[t];
        for (int e = threadIdx.x; e < n; e += blockDim.x) {
            const int p = sm.list[e];
            if (sm.parent[p] != p) continue;
            signed char s = -1;
            for (int q = 0; q < ns; ++q)
                if (a.rootidx[t * kTopSlots + q] == (unsigned short)p) s = (signed char)q;
            sm.slot[p] = s;
        }
        for (int q = threadIdx.x; q < ns; q += blockDim.x)
            sm.sval[q] = __ldcg(&a.gmax[g_find(a.gparent, (int)(t * kTopSlots + q))]);
        __syncthreads();
        // the words with a top-level pixel raised and written back
        constexpr unsigned WMASK = (1u << P::PPW) - 1u;
#pragma unroll
        for (int i = 0; i < kTopWpt; ++i) {
            const unsigned wb = (bits >> (i * P::PPW)) & WMASK;
            if (!wb) continue;
            const int w = threadIdx.x + i * kTopThreads;
            const int pbase = (w >> 5) * TW + (w & 31) * P::PPW;
            uint32_t m[P::PPW];
            P::unpack(mw[i], m);
            bool chg = false;
#pragma unroll
            for (int j = 0; j < P::PPW; ++j) {
                if (!((wb >> j) & 1u)) continue;
                const int s = sm.slot[sm.parent[pbase + j]];
                if (s < 0) continue;
                const uint32_t v = top_key<DT>(sm.sval[s]);
                if (P::gt(v, m[j])) {
                    m[j] = v;
                    chg = true;
                }
            }
            if (!chg) continue;
            const int y = ty * kTopRows + (w >> 5), px0 = tx * TW + (w & 31) * P::PPW;
            unsigned char* row = d.marker + (size_t)y * d.pitch_m + (size_t)px0 * P::BPP;
            const int npx = d.W - px0;
            if (npx >= P::PPW) {
                *reinterpret_cast<unsigned int*>(row) = P::pack(m);
            } else {
#pragma unroll
                for (int j = 0; j < P::PPW; ++j)
                    if (j < npx) P::st_px(row + j * P::BPP, m[j]);
            }
        }
        __syncthreads();
    }
}

// --------------------------------------------------------- engine seeding
// After the front stage and the whole-image passes (or instead of them) the
// tile engine must visit every tile holding a pixel that a neighbour could
// raise (with 8-connectivity: across the diagonals too).  The check streams
// each tile's rows with the rows above and below, marks a tile with such a
// pixel DIRTY on all sides and appends it to the seed list; other tiles get
// state 0.

// A marker pixel, the least value outside the image.
template <int DT>
__device__ __forceinline__ uint32_t seed_px(const ImgDesc& d, int y, int x) {
    using P = Px<DT>;
    if (y < 0 || y >= d.H || x < 0 || x >= d.W) return P::MINPX;
    return P::ld_px(d.marker + (size_t)y * d.pitch_m + (size_t)x * P::BPP);
}

// The check with wide lanes: a lane holds WPL words (8 or 16 bytes) of
// a row, so a warp covers WPL engine tiles side by side (32 / WPL lanes
// each); the words are updated with byte / half-word SIMD, the side
// neighbours of a word's pixels come from funnel shifts of the adjacent
// words, and rows are loaded kSeedAhead ahead into a register ring (one
// vector load per lane where the address allows it, else word by word;
// rows start on 4-byte boundaries).  Eight-byte lanes keep the registers
// per thread low enough for eight CTAs per SM.
constexpr int kSeedAhead = 2;
constexpr int kSeedThreads = 128;
constexpr int kSeedWords = 2;  // words per lane

// WPL words of row y from byte b0 (pixels past the row or outside the image:
// the least value).
template <int DT, int WPL>
__device__ __forceinline__ void seed_load(const ImgDesc& d, const unsigned char* base, long long pitch, int y,
                                          long long b0, long long row_bytes, uint32_t (&w)[WPL]) {
    using P = Px<DT>;
#pragma unroll
    for (int i = 0; i < WPL; ++i) w[i] = P::MINW;
    if (y < 0 || y >= d.H || b0 >= row_bytes) return;
    const unsigned char* p = base + (size_t)y * pitch + b0;
    if (b0 + 4 * WPL <= row_bytes && (reinterpret_cast<uintptr_t>(p) & (4 * WPL - 1)) == 0) {
        if constexpr (WPL == 4) {
            const uint4 v = __ldg(reinterpret_cast<const uint4*>(p));
            w[0] = v.x;
            w[1] = v.y;
            w[2] = v.z;
            w[3] = v.w;
        } else {
            const uint2 v = __ldg(reinterpret_cast<const uint2*>(p));
            w[0] = v.x;
            w[1] = v.y;
        }
        return;
    }
    // rows only 4-byte aligned, or the row's last lane: word by word
#pragma unroll
    for (int i = 0; i < WPL; ++i) {
        const long long b = b0 + 4 * i;
        if (b < row_bytes) w[i] = load_word_plain<DT>(p + 4 * i, (int)((row_bytes - b) / P::BPP), false);
    }
}

// One unit of the check: the WPL engine tiles of tile row ty, group gx of
// image d.  All lanes of the warp.
template <int DT, int WPL>
__device__ __forceinline__ void seed_unit(const ImgDesc& d, int ty, int gx, unsigned* state, unsigned* list,
                                          unsigned* nlist) {
    using P = Px<DT>;
    constexpr int BITS = 8 * P::BPP;  // bits per pixel
    constexpr int TW = 32 * P::PPW;   // pixels per engine tile row
    constexpr int LPT = 32 / WPL;     // lanes per tile
    const int lane = threadIdx.x & 31;
    const int q = lane / LPT;         // this lane's tile of the WPL
    const int TH = d.tile_rows;
    const long long row_bytes = (long long)d.W * P::BPP;
    const int y0 = ty * TH, rows = min(TH, d.H - y0);
    const long long b0 = (long long)gx * (128 * WPL) + lane * (4 * WPL);
    const int xl = gx * WPL * TW - 1, xr = (gx + 1) * WPL * TW;  // halo columns
    auto halo = [&](int y) -> uint32_t {
        if (lane == 0) return seed_px<DT>(d, y, xl);
        if (lane == 31) return seed_px<DT>(d, y, xr);
        return P::MINPX;
    };
    // window: marker rows r - 1, r, mask row r, halo pixels
    uint32_t mu[WPL], mc[WPL], kc[WPL];
    seed_load<DT, WPL>(d, d.marker, d.pitch_m, y0 - 1, b0, row_bytes, mu);
    seed_load<DT, WPL>(d, d.marker, d.pitch_m, y0, b0, row_bytes, mc);
    seed_load<DT, WPL>(d, d.mask, d.pitch_k, y0, b0, row_bytes, kc);
    uint32_t hu = halo(y0 - 1), hc = halo(y0);
    // ring slot i holds marker / mask / halo of row r + 1 + i
    uint32_t rm[kSeedAhead][WPL], rk[kSeedAhead][WPL];
    uint32_t rh[kSeedAhead];
#pragma unroll
    for (int i = 0; i < kSeedAhead; ++i) {
        const int y = y0 + 1 + i;
        seed_load<DT, WPL>(d, d.marker, d.pitch_m, y, b0, row_bytes, rm[i]);
        if (i + 1 < rows) {
            seed_load<DT, WPL>(d, d.mask, d.pitch_k, y, b0, row_bytes, rk[i]);
        } else {
#pragma unroll
            for (int w = 0; w < WPL; ++w) rk[i][w] = P::MINW;
        }
        rh[i] = halo(y);
    }
    bool mine = false;
    for (int r0 = 0; r0 < rows; r0 += kSeedAhead) {
#pragma unroll
        for (int i = 0; i < kSeedAhead; ++i) {
            const int r = r0 + i;
            if (r >= rows) break;  // warp-uniform
            uint32_t md[WPL], kn[WPL];
#pragma unroll
            for (int w = 0; w < WPL; ++w) {
                md[w] = rm[i][w];
                kn[w] = rk[i][w];
            }
            const uint32_t hd = rh[i];
            {
                const int y = y0 + r + 1 + kSeedAhead;
                seed_load<DT, WPL>(d, d.marker, d.pitch_m, y, b0, row_bytes, rm[i]);
                if (r + 1 + kSeedAhead < rows) {
                    seed_load<DT, WPL>(d, d.mask, d.pitch_k, y, b0, row_bytes, rk[i]);
                } else {
#pragma unroll
                    for (int w = 0; w < WPL; ++w) rk[i][w] = P::MINW;
                }
                rh[i] = halo(y);
            }
            // what a column offers its side neighbours: itself, or with
            // 8-connectivity the largest of its three rows
            uint32_t V[WPL], S[WPL];
#pragma unroll
            for (int w = 0; w < WPL; ++w) {
                V[w] = word_max<DT>(mu[w], md[w]);
                S[w] = d.conn == 8 ? word_max<DT>(V[w], mc[w]) : mc[w];
            }
            const uint32_t hs = d.conn == 8 ? P::mx(P::mx(hu, hc), hd) : hc;
            uint32_t left = __shfl_up_sync(FULL, S[WPL - 1], 1), right = __shfl_down_sync(FULL, S[0], 1);
            if (lane == 0) left = BITS == 32 ? hs : hs << (32 - BITS);
            if (lane == 31) right = hs;
#pragma unroll
            for (int w = 0; w < WPL; ++w) {
                // clamped funnel shifts: a shift of 32 (int32) yields the
                // adjacent word itself
                const uint32_t lw = __funnelshift_lc(w == 0 ? left : S[w - 1], S[w], BITS);
                const uint32_t rw = __funnelshift_rc(S[w], w == WPL - 1 ? right : S[w + 1], BITS);
                const uint32_t best = word_max<DT>(V[w], word_max<DT>(lw, rw));
                mine |= word_any_gt<DT>(word_min<DT>(best, kc[w]), mc[w]);
            }
#pragma unroll
            for (int w = 0; w < WPL; ++w) {
                mu[w] = mc[w];
                mc[w] = md[w];
                kc[w] = kn[w];
            }
            hu = hc;
            hc = hd;
        }
    }
    // a tile is bad when one of its lanes saw a pixel to raise
    const unsigned bad = __ballot_sync(FULL, mine);
    const int tx = gx * WPL + q;
    if (lane % LPT == 0 && tx < d.tiles_x) {
        const bool b = ((bad >> (q * LPT)) & (LPT == 32 ? FULL : ((1u << LPT) - 1u))) != 0u;
        const unsigned g = (unsigned)d.tile_base + (unsigned)(ty * d.tiles_x + tx);
        state[g] = b ? (ST_DIRTY | ST_SIDES) : 0u;
        if (b) list[atomicAdd(nlist, 1u)] = g;
    }
}

template <int DT, int WPL>
__global__ void __launch_bounds__(kSeedThreads, 8)
    seed_wide_kernel(const ImgDesc d, unsigned* state, unsigned* list, unsigned* nlist) {
    static_assert(WPL == 2 || WPL == 4, "8- or 16-byte lanes");
    if (gated_off(d)) return;
    const int gx_n = (d.tiles_x + WPL - 1) / WPL;
    const long long units = (long long)gx_n * d.tiles_y;
    const long long wg = ((long long)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const long long nw = ((long long)gridDim.x * blockDim.x) >> 5;
    for (long long unit = wg; unit < units; unit += nw) {
        const int ty = (int)(unit / gx_n), gx = (int)(unit - (long long)ty * gx_n);
        seed_unit<DT, WPL>(d, ty, gx, state, list, nlist);
    }
}

// All images of a job in one launch (their rows on 16-byte boundaries): each
// CTA forms the prefix of the images' unit counts in shared memory, and a
// warp finds its unit's image by binary search.  `gate` (nullable) as
// ImgDesc::gate.
constexpr int kSeedMaxImages = 1024;

template <int WPL>
__global__ void __launch_bounds__(kSeedThreads, 6)
    seed_batch_kernel(const ImgDesc* descs, int nimg, const unsigned* gate, unsigned* state, unsigned* list,
                      unsigned* nlist) {
    if (gate != nullptr && *(const volatile unsigned*)gate == 0u) return;
    __shared__ long long ubase[kSeedMaxImages + 1];
    __shared__ long long chunk_sum;
    // the prefix of unit counts, kSeedThreads images at a time
    if (threadIdx.x == 0) {
        ubase[0] = 0;
        chunk_sum = 0;
    }
    __syncthreads();
    for (int i0 = 0; i0 < nimg; i0 += kSeedThreads) {
        const int i = i0 + (int)threadIdx.x;
        long long u = 0;
        if (i < nimg) {
            const ImgDesc& d = descs[i];
            u = (long long)((d.tiles_x + WPL - 1) / WPL) * d.tiles_y;
        }
        // inclusive scan over the CTA (warp scans, then the warp totals)
        const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
        long long v = u;
#pragma unroll
        for (int dd = 1; dd < 32; dd <<= 1) {
            const long long t = __shfl_up_sync(FULL, v, dd);
            if (lane >= dd) v += t;
        }
        __shared__ long long wsum[kSeedThreads / 32];
        if (lane == 31) wsum[warp] = v;
        __syncthreads();
        long long before = chunk_sum;
        for (int w = 0; w < warp; ++w) before += wsum[w];
        if (i < nimg) ubase[i + 1] = before + v;
        __syncthreads();
        if (threadIdx.x == kSeedThreads - 1) chunk_sum = before + v;
        __syncthreads();
    }
    const long long total = ubase[nimg];
    const long long wg = ((long long)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const long long nw = ((long long)gridDim.x * blockDim.x) >> 5;
    for (long long unit = wg; unit < total; unit += nw) {
        int lo = 0, hi = nimg - 1;  // the last image whose first unit is <= unit
        while (lo < hi) {
            const int mid = (lo + hi + 1) >> 1;
            if (ubase[mid] <= unit)
                lo = mid;
            else
                hi = mid - 1;
        }
        const ImgDesc d = descs[lo];
        const long long u = unit - ubase[lo];
        const int gx_n = (d.tiles_x + WPL - 1) / WPL;
        const int ty = (int)(u / gx_n), gx = (int)(u - (long long)ty * gx_n);
        if (d.dtype == DT_U8)
            seed_unit<DT_U8, WPL>(d, ty, gx, state, list, nlist);
        else if (d.dtype == DT_U16)
            seed_unit<DT_U16, WPL>(d, ty, gx, state, list, nlist);
        else
            seed_unit<DT_I32, WPL>(d, ty, gx, state, list, nlist);
    }
}

// --------------------------------------------------- the device decision
// Decides, from the seed check over the untouched images, whether the job
// takes the front stage: a small initial front (some tiles, but fewer than
// one in kFrontDecideRatio, holding a pixel a neighbour can raise: a few
// sparse seeds) propagates over long paths, one dependent tile visit per tile for
// the engine alone, which the labelling and the whole-image passes cover
// in a fixed number of sweeps; a large front (h-dome markers, dense seeds)
// is short-range work the engine does faster alone.  With the stage the
// seed list is emptied for the check after the passes; without it the list
// of this check seeds the engine.
constexpr unsigned kFrontDecideRatio = 64;

__global__ void front_decide_kernel(unsigned* gate, unsigned* count, unsigned G) {
    const unsigned n = *(volatile unsigned*)count;
    const unsigned front = n > 0u && (unsigned long long)n * kFrontDecideRatio < (unsigned long long)G ? 1u : 0u;
    *gate = front;
    if (front) *count = 0u;
}

// ------------------------------------------------------------------ host
static size_t tal(size_t v) { return (v + 255) / 256 * 256; }

static void top_dims(const ImgDesc& d, int* tx_n, int* ty_n, int* tw) {
    const int bpp = d.dtype == DT_U8 ? 1 : d.dtype == DT_U16 ? 2 : 4;
    *tw = 128 / bpp;
    *tx_n = (int)(((long long)d.W * bpp + 127) / 128);
    *ty_n = (d.H + kTopRows - 1) / kTopRows;
}

size_t top_scratch_bytes(const ImgDesc& d) {
    int tx_n, ty_n, tw;
    top_dims(d, &tx_n, &ty_n, &tw);
    const size_t G = (size_t)tx_n * ty_n, nodes = G * kTopSlots;
    return tal(256) + tal(G * 4) + tal(G * 4) + tal(nodes * 4) + tal(nodes * 4) + tal(nodes * 2) +
           tal(G * (128 + 2 * (size_t)tw)) + tal(G * 4) + tal(G * kTopListCap * 4) + tal(8) + 2 * tal(G * 4);
}

template <int DT>
static cudaError_t launch_top_t(const TopArgs& a, int sms, cudaStream_t s) {
    const size_t smem = sizeof(TopSmem<DT>);
    cudaError_t e = cudaFuncSetAttribute(top_local_kernel<DT>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e == cudaSuccess)
        e = cudaFuncSetAttribute(top_apply_label_kernel<DT>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
    const long long G = (long long)a.tx_n * a.ty_n;
    long long wblocks = (G * 32 + 255) / 256;
    if (wblocks > (long long)sms * 16) wblocks = (long long)sms * 16;
    top_max_kernel<DT><<<(unsigned)wblocks, 256, 0, s>>>(a);
    long long cblocks = G < (long long)sms * 4 ? G : (long long)sms * 4;
    top_local_kernel<DT><<<(unsigned)cblocks, kTopThreads, smem, s>>>(a);
    const long long upairs = G * (2 * kTopRows + 2 * a.tw + 2);
    long long ublocks = (upairs + 255) / 256;
    if (ublocks > (long long)sms * 32) ublocks = (long long)sms * 32;
    top_union_kernel<<<(unsigned)ublocks, 256, 0, s>>>(a);
    long long fblocks = (G * kTopSlots + 255) / 256;
    if (fblocks > (long long)sms * 32) fblocks = (long long)sms * 32;
    top_flatten_kernel<<<(unsigned)fblocks, 256, 0, s>>>(a);
    top_apply_list_kernel<DT><<<(unsigned)wblocks, 256, 0, s>>>(a);
    top_apply_label_kernel<DT><<<(unsigned)cblocks, kTopThreads, smem, s>>>(a);
    return cudaGetLastError();
}

cudaError_t launch_top(const ImgDesc& d, void* scratch, unsigned long long* top_pixels, int device, cudaStream_t s,
                       int* launches) {
    if (d.W == 0 || d.H == 0) return cudaSuccess;
    TopArgs a{};
    a.d = d;
    top_dims(d, &a.tx_n, &a.ty_n, &a.tw);
    a.conn = d.conn;
    const size_t G = (size_t)a.tx_n * a.ty_n, nodes = G * kTopSlots;
    char* p = static_cast<char*>(scratch);
    a.thr_key = reinterpret_cast<unsigned*>(p);
    p += tal(256);
    a.tmax = reinterpret_cast<unsigned*>(p);
    p += tal(G * 4);
    a.ns = reinterpret_cast<int*>(p);
    p += tal(G * 4);
    a.gparent = reinterpret_cast<int*>(p);
    p += tal(nodes * 4);
    a.gmax = reinterpret_cast<unsigned*>(p);
    p += tal(nodes * 4);
    a.rootidx = reinterpret_cast<unsigned short*>(p);
    p += tal(nodes * 2);
    a.edge = reinterpret_cast<signed char*>(p);
    a.edge_stride = 128 + 2 * a.tw;
    p += tal(G * (size_t)a.edge_stride);
    a.tn = reinterpret_cast<int*>(p);
    p += tal(G * 4);
    a.tlist = reinterpret_cast<unsigned*>(p);
    p += tal(G * kTopListCap * 4);
    a.ncount = reinterpret_cast<unsigned*>(p);
    p += tal(8);
    a.listed = reinterpret_cast<unsigned*>(p);
    p += tal(G * 4);
    a.relabel = reinterpret_cast<unsigned*>(p);
    a.aligned16 = (reinterpret_cast<uintptr_t>(d.mask) & 15u) == 0u && (d.pitch_k & 15) == 0;
    a.top_pixels = top_pixels;
    int sms = 0;
    cudaError_t e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device);
    if (e == cudaSuccess) e = cudaMemsetAsync(a.thr_key, 0, sizeof(unsigned), s);
    if (e == cudaSuccess) e = cudaMemsetAsync(a.ncount, 0, 2 * sizeof(unsigned), s);
    if (e != cudaSuccess) return e;
    if (d.dtype == DT_U8)
        e = launch_top_t<DT_U8>(a, sms, s);
    else if (d.dtype == DT_U16)
        e = launch_top_t<DT_U16>(a, sms, s);
    else
        e = launch_top_t<DT_I32>(a, sms, s);
    if (e == cudaSuccess && launches) *launches += 6;
    return e;
}

cudaError_t launch_seed_batch(const ImgDesc* dev_descs, const std::vector<ImgDesc>& host_descs, const unsigned* gate,
                              unsigned* state, unsigned* list, unsigned* nlist, cudaStream_t s, int* launches) {
    const int nimg = (int)host_descs.size();
    long long units = 0;
    for (const auto& d : host_descs) units += (long long)((d.tiles_x + kSeedWords - 1) / kSeedWords) * d.tiles_y;
    if (nimg == 0 || nimg > kSeedMaxImages) {
        // one launch per image
        for (auto d : host_descs) {
            d.gate = gate;
            const cudaError_t e = launch_seed(d, state, list, nlist, s, launches);
            if (e != cudaSuccess) return e;
        }
        return cudaSuccess;
    }
    if (units == 0) return cudaSuccess;
    long long blocks = (units * 32 + kSeedThreads - 1) / kSeedThreads;
    if (blocks > 152ll * 64) blocks = 152ll * 64;
    seed_batch_kernel<kSeedWords><<<(unsigned)blocks, kSeedThreads, 0, s>>>(dev_descs, nimg, gate, state, list, nlist);
    if (launches) ++*launches;
    return cudaGetLastError();
}

cudaError_t launch_front_decide(unsigned* gate, unsigned* count, unsigned G, cudaStream_t s, int* launches) {
    front_decide_kernel<<<1, 1, 0, s>>>(gate, count, G);
    if (launches) ++*launches;
    return cudaGetLastError();
}

cudaError_t launch_seed(const ImgDesc& d, unsigned* state, unsigned* list, unsigned* nlist, cudaStream_t s,
                        int* launches) {
    if (d.W == 0 || d.H == 0) return cudaSuccess;
    constexpr int WPL = kSeedWords;
    const long long units = (long long)((d.tiles_x + WPL - 1) / WPL) * d.tiles_y;
    long long blocks = (units * 32 + kSeedThreads - 1) / kSeedThreads;
    if (blocks > 152ll * 64) blocks = 152ll * 64;
    if (blocks < 1) blocks = 1;
    if (d.dtype == DT_U8)
        seed_wide_kernel<DT_U8, WPL><<<(unsigned)blocks, kSeedThreads, 0, s>>>(d, state, list, nlist);
    else if (d.dtype == DT_U16)
        seed_wide_kernel<DT_U16, WPL><<<(unsigned)blocks, kSeedThreads, 0, s>>>(d, state, list, nlist);
    else
        seed_wide_kernel<DT_I32, WPL><<<(unsigned)blocks, kSeedThreads, 0, s>>>(d, state, list, nlist);
    if (launches) ++*launches;
    return cudaGetLastError();
}

}  // namespace iwpp
