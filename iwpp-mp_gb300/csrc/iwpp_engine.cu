// iwpp_engine.cu -- device side of the persistent tile engine (see
// iwpp_engine.cuh for the design and the reference citations).
#include <cstdio>

#include "iwpp_engine.cuh"

namespace iwpp {

__device__ __forceinline__ unsigned ld_volatile(const unsigned* p) { return *(const volatile unsigned*)p; }
__device__ __forceinline__ int ld_volatile(const int* p) { return *(const volatile int*)p; }

__device__ __forceinline__ void set_error(Ctrl* c, unsigned code) { atomicCAS(&c->error, 0u, code); }

// Async ring: positions below this are the job's initial entries (every
// tile, or the seed list after the front stage), the rest map to ring slots.
__device__ __forceinline__ unsigned ring_base(const EngineArgs& a) {
    return a.init_list ? ld_volatile(&a.ctrl->ninit) : a.G;
}

// Image of global tile g: the last image whose tile_base <= g.
__device__ __forceinline__ int find_image(const EngineArgs& a, unsigned g) {
    int lo = 0, hi = a.nimg - 1;
    while (lo < hi) {
        const int mid = (lo + hi + 1) >> 1;
        if ((unsigned)__ldg(&a.imgs[mid].tile_base) <= g)
            lo = mid;
        else
            hi = mid - 1;
    }
    return lo;
}

template <int TH, class Early>
__device__ __forceinline__ VisitResult dispatch_visit(const ImgDesc& d, int tx, int ty, WarpSmem<TH>& sm, int lane,
                                                     unsigned& phase, long long timeout_ns, unsigned sides,
                                                     Early& early) {
    const int mode = d.dtype * 2 + (d.conn == 8 ? 1 : 0);
    switch (mode) {
        case 0: return visit_tile<DT_U8, 4, TH>(d, tx, ty, sm, lane, phase, timeout_ns, sides, early);
        case 1: return visit_tile<DT_U8, 8, TH>(d, tx, ty, sm, lane, phase, timeout_ns, sides, early);
        case 2: return visit_tile<DT_U16, 4, TH>(d, tx, ty, sm, lane, phase, timeout_ns, sides, early);
        case 3: return visit_tile<DT_U16, 8, TH>(d, tx, ty, sm, lane, phase, timeout_ns, sides, early);
        case 4: return visit_tile<DT_I32, 4, TH>(d, tx, ty, sm, lane, phase, timeout_ns, sides, early);
        default: return visit_tile<DT_I32, 8, TH>(d, tx, ty, sm, lane, phase, timeout_ns, sides, early);
    }
}

// The side of a neighbour tile that faces direction `dir` of this tile.
__device__ __constant__ static const int kNbOpposite[8] = {1, 0, 3, 2, 7, 6, 5, 4};

struct WarpCounters {
    unsigned long long visits = 0, sweeps = 0, pushes = 0, row_steps = 0;
    long long phase[5] = {0, 0, 0, 0, 0};  // queue read, fetch, processing, dump, queue write
};

// ---------------------------------------------------------------- mutex

// The global mutex (IWPP MP/src/globalQueue.cu:35, :114, a CAS spin without
// a bound) as a ticket lock: one atomic per acquisition instead of a CAS
// storm from every waiting warp, hand-over in arrival order, acquire /
// release ordering instead of full fences; waiters poll the ticket being
// served with a back-off proportional to their place in line, and a
// wall-clock bound ends in DEV_ERR_TIMEOUT.  A waiter that gives up leaves
// the error flag set, which ends every other waiter too.
__device__ __forceinline__ unsigned long long ld_acquire64(const unsigned long long* p) {
    unsigned long long v;
    asm volatile("ld.acquire.gpu.global.u64 %0, [%1];" : "=l"(v) : "l"(p) : "memory");
    return v;
}
__device__ __forceinline__ void st_release64(unsigned long long* p, unsigned long long v) {
    asm volatile("st.release.gpu.global.u64 [%0], %1;" ::"l"(p), "l"(v) : "memory");
}
// The mutex stack's entry count and the ticket being served, read without
// the lock (hints: look-ahead, quiescence).
__device__ __forceinline__ int stack_top(const Ctrl* c) {
    return (int)(unsigned)(*(const volatile unsigned long long*)&c->lock_word >> 32);
}
__device__ __forceinline__ unsigned lock_serving(const Ctrl* c) {
    return (unsigned)*(const volatile unsigned long long*)&c->lock_word;
}

// Acquires the lock; *top is the stack's entry count at the hand-over.
__device__ bool mutex_lock(const EngineArgs& a, unsigned* ticket, int* top) {
    const unsigned t = atomicAdd(&a.ctrl->lock_next, 1u);
    *ticket = t;
    const long long t0 = globaltimer_ns();
    unsigned spins = 0;
    for (;;) {
        const unsigned long long w = ld_acquire64(&a.ctrl->lock_word);
        const unsigned s = (unsigned)w;
        if (s == t) {
            *top = (int)(unsigned)(w >> 32);
            return true;
        }
        const unsigned place = t - s;
        __nanosleep(32u * (place < 32u ? place : 32u));
        if ((++spins & 15u) == 0u) {
            if (ld_volatile(&a.ctrl->error) != 0u) return false;
            if (globaltimer_ns() - t0 > a.timeout_ns) {
                set_error(a.ctrl, DEV_ERR_TIMEOUT);
                return false;
            }
        }
    }
}

// Releases the lock, publishing the stack's new entry count with it.
__device__ __forceinline__ void mutex_unlock(const EngineArgs& a, unsigned ticket, int top) {
    st_release64(&a.ctrl->lock_word, ((unsigned long long)(unsigned)top << 32) | (unsigned long long)(ticket + 1u));
}

// ------------------------------------------------------------------ push
// Inserts the entries of the lanes with `want` set into the queue: the mutex
// stack under one lock acquisition (IWPP MP/src/globalQueue.cu:25-81), or the
// write queue with one atomicAdd reservation per warp
// (IWPP MP DQ/src/globalQueue.cu:14-47).  A short insertion sets the
// overflow flag (the reference's memLeak, MR.cu:524-526); the tiles stay
// DIRTY and are recovered by the restart.
// The mutex stack's insertion: one lock acquisition for the warp's entries.
// `counted`: `pending` already holds them (entries moving from a CTA
// buffer); else they are added to it before the release can publish them.
__device__ void mutex_push_global(const EngineArgs& a, bool want, unsigned gn, int lane, bool counted) {
    const unsigned ballot = __ballot_sync(FULL, want);
    if (ballot == 0u) return;
    const int n = __popc(ballot);
    const int rank = __popc(ballot & ((1u << lane) - 1u));
    int base = -1;
    unsigned ticket = 0u;
    if (lane == 0) {
        int top = 0;
        if (mutex_lock(a, &ticket, &top)) {
            if ((unsigned)top + (unsigned)n <= a.cap) {
                base = top;
                if (!counted) atomicAdd(&a.ctrl->pending, n);  // before the entries can be taken
            } else {
                atomicExch(&a.ctrl->overflow, 1u);
                if (counted) atomicSub(&a.ctrl->pending, n);  // lost: the restart recovers the tiles
                mutex_unlock(a, ticket, top);
            }
        }
    }
    base = __shfl_sync(FULL, base, 0);
    if (base < 0) return;
    if (want) {
        a.q0[base + rank] = gn;
        __threadfence();  // the entry before the release that publishes it
    }
    __syncwarp();
    if (lane == 0) mutex_unlock(a, ticket, base + n);
}

template <int VAR>
__device__ void push_entries(const EngineArgs& a, bool want, unsigned gn, int lane, unsigned* wq,
                             WarpCounters& cnt) {
    const unsigned ballot = __ballot_sync(FULL, want);
    if (ballot == 0u) return;
    const int n = __popc(ballot);
    const int rank = __popc(ballot & ((1u << lane) - 1u));
    if (VAR == VAR_MUTEX) {
        mutex_push_global(a, want, gn, lane, false);
    } else if (VAR == VAR_ASYNC) {
        // positions [base, base + n) of the ring; `pending` first, so the job
        // cannot look finished while these entries exist
        unsigned base = 0u;
        if (lane == 0) {
            atomicAdd(&a.ctrl->pending, n);
            base = atomicAdd(&a.ctrl->atail, (unsigned)n);
        }
        base = __shfl_sync(FULL, base, 0);
        if (want) {
            const unsigned slot = (base + (unsigned)rank - ring_base(a)) % a.cap;
            const long long t0 = globaltimer_ns();
            unsigned spins = 0;
            // the slot's previous occupant has normally been taken long ago
            while (atomicCAS(&a.q0[slot], 0u, gn + 1u) != 0u) {
                __nanosleep(64);
                if ((++spins & 255u) == 0u && globaltimer_ns() - t0 > a.timeout_ns) {
                    set_error(a.ctrl, DEV_ERR_TIMEOUT);
                    break;
                }
            }
        }
    } else {
        unsigned base = 0u;
        if (lane == 0) base = atomicAdd(&a.ctrl->wn, (unsigned)n);
        base = __shfl_sync(FULL, base, 0);
        if (want) {
            const unsigned pos = base + (unsigned)rank;
            if (pos < a.cap)
                wq[pos] = gn;
            else
                atomicExch(&a.ctrl->overflow, 1u);
        }
    }
    cnt.pushes += (unsigned)n;
}

// ------------------------------------------------- mutex: CTA buffers
// The MP discipline keeps one LIFO stack under one lock, and what
// serialises it is one acquisition per insertion and per take.  Each CTA
// therefore keeps the entries its warps insert in a shared-memory buffer and
// takes from it first; the global stack sees a batch take when the buffer
// runs dry, a spill when it fills, and a share when the global stack is empty
// while warps elsewhere wait.  Buffered entries count in `pending`, so the
// termination rule (nothing pending, nothing stacked) is unchanged.
constexpr int kCtaBuf = 64;    // entries a CTA buffers
constexpr int kCtaSpill = 48;  // above this a push spills the buffer down to kCtaKeep
constexpr int kCtaKeep = 16;

struct MutexCtaBuf {
    int lock;
    int n;
    int taker;    // 1 while one of this CTA's warps works the global stack
    int waiting;  // this CTA's warps waiting for work
    unsigned e[kCtaBuf];
};
__shared__ MutexCtaBuf s_cq;

// The buffer's lock, held by one of this CTA's warps for a few shared-memory
// accesses at a time; the bound is never reached in a working job.
__device__ __forceinline__ bool cq_lock(const EngineArgs& a) {
    unsigned spins = 0;
    while (atomicCAS(&s_cq.lock, 0, 1) != 0) {
        __nanosleep(32);
        if (++spins > (1u << 22)) {
            set_error(a.ctrl, DEV_ERR_TIMEOUT);
            return false;
        }
    }
    __threadfence_block();
    return true;
}
__device__ __forceinline__ void cq_unlock() {
    __threadfence_block();
    atomicExch(&s_cq.lock, 0);
}

__device__ __forceinline__ int cq_count() { return *(volatile int*)&s_cq.n; }

// Moves up to 32 of the buffer's newest entries beyond `keep` to the global
// stack (one acquisition).
__device__ void cta_spill(const EngineArgs& a, int lane, int keep) {
    int m = 0, base = 0;
    if (lane == 0 && cq_lock(a)) {
        m = min(max(s_cq.n - keep, 0), 32);
        s_cq.n -= m;
        base = s_cq.n;
        if (m == 0) cq_unlock();
    }
    m = __shfl_sync(FULL, m, 0);
    base = __shfl_sync(FULL, base, 0);
    if (m == 0) return;
    const unsigned mine = lane < m ? *(volatile unsigned*)&s_cq.e[base + lane] : 0u;
    __syncwarp();
    if (lane == 0) cq_unlock();
    mutex_push_global(a, lane < m, mine, lane, true);
}

// Inserts the entries of the lanes with `want` set into this CTA's buffer
// (what does not fit goes to the global stack), spilling a full buffer.
// `counted`: `pending` already holds them.
__device__ void cta_push(const EngineArgs& a, bool want, unsigned gn, int lane, WarpCounters& cnt,
                         bool counted = false) {
    const unsigned ballot = __ballot_sync(FULL, want);
    if (ballot == 0u) return;
    const int n = __popc(ballot);
    const int rank = __popc(ballot & ((1u << lane) - 1u));
    int base = 0, k = 0;
    bool locked = false;
    if (lane == 0) {
        if (!counted) atomicAdd(&a.ctrl->pending, n);  // before any of them can be taken
        locked = cq_lock(a);
        if (locked) {
            k = min(n, kCtaBuf - s_cq.n);
            base = s_cq.n;
            s_cq.n += k;
        }
    }
    k = __shfl_sync(FULL, k, 0);
    base = __shfl_sync(FULL, base, 0);
    if (want && rank < k) *(volatile unsigned*)&s_cq.e[base + rank] = gn;
    __syncwarp();
    if (locked) cq_unlock();
    if (!counted) cnt.pushes += (unsigned)n;
    if (n > k) mutex_push_global(a, want && rank >= k, gn, lane, true);
    if (__shfl_sync(FULL, cq_count(), 0) > kCtaSpill) cta_spill(a, lane, kCtaKeep);
}

// The buffer's newest entry, or ~0u.
__device__ unsigned cta_take(const EngineArgs& a, int lane) {
    unsigned g = ~0u;
    if (lane == 0 && cq_count() > 0 && cq_lock(a)) {
        if (s_cq.n > 0) g = *(volatile unsigned*)&s_cq.e[--s_cq.n];
        cq_unlock();
    }
    return __shfl_sync(FULL, g, 0);
}

// Marks the neighbour tiles in `nb` DIRTY and inserts them (VAR_UNIQUE /
// VAR_ASYNC: only those that were neither pending nor being visited).  With
// the async queue one of the newly dirty tiles is not inserted but returned:
// the warp visits it next itself, following the propagation front without a
// trip through the queue.  Returns ~0u when there is none.
template <int VAR>
__device__ unsigned notify(const EngineArgs& a, const ImgDesc& d, int tx, int ty, unsigned nb, int lane, unsigned* wq,
                           WarpCounters& cnt, bool keep_one = true) {
    bool want = false, fresh = false;
    unsigned gn = 0u;
    if (lane < 8 && ((nb >> lane) & 1u)) {
        const int nx = tx + kNbDx[lane], ny = ty + kNbDy[lane];
        if (nx >= 0 && nx < d.tiles_x && ny >= 0 && ny < d.tiles_y) {
            gn = (unsigned)d.tile_base + (unsigned)(ny * d.tiles_x + nx);
            const unsigned old =
                atomicOr(&a.state[gn], ST_DIRTY | (1u << (ST_SIDE_SHIFT + (unsigned)kNbOpposite[lane])));
            fresh = (old & (ST_DIRTY | ST_ACTIVE)) == 0u;
            want = (VAR == VAR_UNIQUE || VAR == VAR_ASYNC) ? fresh : true;
        }
    }
    unsigned cont = ~0u;
    if ((VAR == VAR_ASYNC || VAR == VAR_MUTEX) && keep_one) {
        // one newly dirty neighbour is kept by this warp (its next visit)
        // instead of going through the queue
        const unsigned ballot = __ballot_sync(FULL, want && fresh);
        if (ballot != 0u) {
            const int leader = __ffs(ballot) - 1;
            cont = __shfl_sync(FULL, gn, leader);
            if (lane == leader) want = false;
        }
    }
    if (VAR == VAR_MUTEX)
        cta_push(a, want, gn, lane, cnt);
    else
        push_entries<VAR>(a, want, gn, lane, wq, cnt);
    return cont;
}

// Early publication for the async queue: while many warps wait for work
// (the job is bound by its propagation front), a visit that raised a
// boundary of its tile stores what it has and notifies those neighbours at
// once instead of after its last sweep, so they can start while this tile is
// still converging.  While the warps are busy it would only add revisits.
template <int VAR>
struct EarlyFlush {
    static constexpr bool kEnabled = VAR == VAR_ASYNC;
    const EngineArgs* a;
    const ImgDesc* d;
    int tx, ty;
    WarpCounters* cnt;
    bool use_passes;  // in-tile solver of this visit
    bool use_pq;      // revisits by the pixel queue
    // Front-bound: more than half of the grid's warps have claimed a ring
    // position that no producer has filled yet (they wait for work).  A
    // quarter or an eighth switches too early on h-dome images, three
    // quarters too late on long corridors.
    __device__ static bool sample(const EngineArgs& a, int lane) {
        unsigned v = 0u;
        if (lane == 0) {
            const unsigned head = ld_volatile(&a.ctrl->ahead), tail = ld_volatile(&a.ctrl->atail);
            v = (int)(head - tail) > (int)(gridDim.x * (unsigned)kWarps / 2u) ? 1u : 0u;
        }
        return __shfl_sync(FULL, v, 0) != 0u;
    }
    __device__ bool passes(int) { return use_passes; }
    __device__ bool pq() { return use_pq; }
    __device__ bool want(int lane) { return sample(*a, lane); }
    __device__ void flush(unsigned nb, int lane) {
        __threadfence();  // release: the rows just stored before the neighbours' DIRTY
        __syncwarp();
        notify<VAR>(*a, *d, tx, ty, nb, lane, nullptr, *cnt, false);
    }
};

// ------------------------------------------------------------ one entry
// Takes tile g unless another warp owns it (that owner sees DIRTY when it
// releases), visits it once if it is DIRTY, notifies the neighbours it
// raised, and releases it; if it was marked DIRTY meanwhile it is queued
// again (next round for the double / unique queues) instead of being
// revisited at once with half-updated neighbours.
template <int VAR, int TH>
__device__ bool process_entry(const EngineArgs& a, unsigned g, WarpSmem<TH>& sm, int lane, unsigned* wq,
                              WarpCounters& cnt, unsigned& phase, unsigned* next = nullptr) {
    if (next) *next = ~0u;
    unsigned old = 0u;
    if (lane == 0) old = atomicOr(&a.state[g], ST_ACTIVE);
    old = __shfl_sync(FULL, old, 0);
    if (old & ST_ACTIVE) return true;
    if (lane == 0) old = atomicAnd(&a.state[g], ~(ST_DIRTY | ST_SIDES));
    old = __shfl_sync(FULL, old, 0);
    if (old & ST_DIRTY) {
        unsigned sides = (old & ST_SIDES) >> ST_SIDE_SHIFT;
        if (sides == 0u) sides = 0xffu;
        __threadfence();  // acquire: neighbours' stores before their DIRTY
        __syncwarp();
        const int ii = find_image(a, g);
        const ImgDesc d = a.imgs[ii];
        const int t = (int)(g - (unsigned)d.tile_base);
        const int ty = t / d.tiles_x, tx = t - ty * d.tiles_x;
        // In-tile solver: row sweeps (fewest instructions) while the warps
        // are busy, passes (shortest latency) while many wait for work (async
        // queue; the round-based queues use the sweeps unless told otherwise).
        // Solver 3: revisits by the pixel queue, first visits by passes.
        bool use_passes = a.solver == 2 || a.solver == 3;
        if (a.solver == 0 && VAR == VAR_ASYNC) use_passes = EarlyFlush<VAR_ASYNC>::sample(a, lane);
        const bool use_pq = a.solver == 3;
        VisitResult r;
        if (VAR == VAR_ASYNC) {
            EarlyFlush<VAR> early{&a, &d, tx, ty, &cnt, use_passes, use_pq};
            r = dispatch_visit<TH>(d, tx, ty, sm, lane, phase, a.timeout_ns, sides, early);
        } else {
            NoEarlyFlush early{use_passes, use_pq};
            r = dispatch_visit<TH>(d, tx, ty, sm, lane, phase, a.timeout_ns, sides, early);
        }
        if (!r.ok) {
            if (lane == 0) set_error(a.ctrl, DEV_ERR_TIMEOUT);
            return false;
        }
        cnt.visits += 1;
        cnt.sweeps += r.sweeps;
        cnt.row_steps += r.row_steps;
        cnt.phase[1] += r.t_fetch;
        cnt.phase[2] += r.t_proc;
        cnt.phase[3] += r.t_dump;
        const long long q0 = clock64();
        if (r.nb != 0u || r.stored) {
            // release: this tile's stores before the neighbours' DIRTY and
            // before the tile's ACTIVE bit clears (its next owner reads them)
            __threadfence();
            __syncwarp();
        }
        if (r.nb != 0u) {
            const unsigned cont = notify<VAR>(a, d, tx, ty, r.nb, lane, wq, cnt);
            if (next) *next = cont;
        }
        cnt.phase[4] += clock64() - q0;
    }
    const long long q1 = clock64();
    if (lane == 0) old = atomicAnd(&a.state[g], ~ST_ACTIVE);
    old = __shfl_sync(FULL, old, 0);
    if (old & ST_DIRTY) {
        if (VAR == VAR_MUTEX)
            cta_push(a, lane == 0, g, lane, cnt);
        else
            push_entries<VAR>(a, lane == 0, g, lane, wq, cnt);
    }
    cnt.phase[4] += clock64() - q1;
    return true;
}

// ------------------------------------------------------- mutex worker
// The global stack's side of a take, for the one warp of its CTA that works
// it: up to kMutexBatch entries under the lock (enough for this CTA's
// waiting warps, or the stack divided among the CTAs while it is long; the
// reference takes one, IWPP MP/src/MorphologicalReconstruction.cu:221), the
// first returned in *g, the rest buffered for the CTA.  Returns 0 with an
// entry, 1 when the job is over for this warp (finished or an error), 2 when
// there is nothing to take now.  On overflow the quiescent stack is refilled
// with every tile (MR.cu:785-806).
__device__ int mutex_global_take(const EngineArgs& a, int lane, WarpCounters& cnt, unsigned* g) {
    // Look before queueing for the lock: a ticket only while the stack holds
    // more entries than there are warps in line (a ticket lock serves in
    // arrival order, so warps queued for an empty stack would delay every
    // warp that inserts), or when the job looks finished but an overflow
    // needs the refill.  A finished job (nothing stacked or pending, no
    // overflow) is left without the lock.
    int look = 0;  // 0 back off, 1 take a ticket, 2 finished
    if (lane == 0) {
        const int top = stack_top(a.ctrl);
        const int pend = ld_volatile(&a.ctrl->pending);
        const unsigned line = ld_volatile(&a.ctrl->lock_next) - lock_serving(a.ctrl);
        if (pend == 0 && top == 0 && ld_volatile(&a.ctrl->overflow) == 0u)
            look = 2;
        else if (top > (int)line || pend == 0)
            look = 1;
    }
    look = __shfl_sync(FULL, look, 0);
    if (look == 2) return 1;
    if (look == 0) return 2;
    int n = 0, base = 0, outcome = 0;  // outcome: 0 entries / nothing, 1 exit, 2 refill
    unsigned ticket = 0u;
    int top = 0;
    if (lane == 0) {
        if (!mutex_lock(a, &ticket, &top)) {
            outcome = 1;
        } else {
            if (top > 0) {
                const int want = *(volatile int*)&s_cq.waiting + 1;
                n = top / (int)gridDim.x;
                n = n < want ? want : n;
                n = n > kMutexBatch ? kMutexBatch : n;
                n = n > top ? top : n;
                base = top - n;
            } else if (ld_volatile(&a.ctrl->pending) == 0) {
                if (ld_volatile(&a.ctrl->overflow) != 0u) {
                    if ((int)ld_volatile(&a.ctrl->restarts) >= a.max_restarts) {
                        set_error(a.ctrl, DEV_ERR_OVERFLOW);
                        outcome = 1;
                    } else {
                        outcome = 2;
                    }
                } else {
                    outcome = 1;
                }
            }
            if (n == 0 && outcome != 2) mutex_unlock(a, ticket, top);
        }
    }
    n = __shfl_sync(FULL, n, 0);
    base = __shfl_sync(FULL, base, 0);
    outcome = __shfl_sync(FULL, outcome, 0);
    if (outcome == 1) return 1;
    if (outcome == 2) {
        // quiescent with lost insertions: refill with every tile (lock held)
        for (unsigned i = (unsigned)lane; i < a.G && i < a.cap; i += 32u) a.q0[i] = a.G - 1u - i;
        __threadfence();
        __syncwarp();
        if (lane == 0) {
            const int cnt_all = (int)(a.G < a.cap ? a.G : a.cap);
            atomicAdd(&a.ctrl->pending, cnt_all);
            atomicExch(&a.ctrl->overflow, 0u);
            atomicAdd(&a.ctrl->restarts, 1u);
            mutex_unlock(a, ticket, cnt_all);
        }
        __syncwarp();
        return 2;
    }
    if (n == 0) return 2;
    // copy the taken entries out before the lock is released
    unsigned mine = 0u;
    if (lane < n) mine = __ldcg(&a.q0[base + lane]);  // from L2: the slot may have been cached before
    // (the vote needs every lane's value: the loads are done before the release)
    __ballot_sync(FULL, mine == ~0u);
    if (lane == 0) mutex_unlock(a, ticket, base);
    *g = __shfl_sync(FULL, mine, 0);
    cta_push(a, lane >= 1 && lane < n, mine, lane, cnt, true);
    return 0;
}

// One persistent launch.  A warp takes its next entry from its CTA's buffer;
// when that is empty, one warp of the CTA at a time takes a batch from the
// global LIFO stack for the CTA (mutex_global_take) while the others wait
// for it.  Termination: nothing is stacked and no inserted entry is
// unfinished (`pending` == 0, buffered entries included), which replaces
// activeBlocksCount (IWPP MP/src/globalQueue.cu:134-145).
template <int TH>
__device__ void mutex_worker(const EngineArgs& a, WarpSmem<TH>& sm, int lane, WarpCounters& cnt, unsigned& phase) {
    if (threadIdx.x == 0) {
        s_cq.lock = 0;
        s_cq.n = 0;
        s_cq.taker = 0;
        s_cq.waiting = 0;
    }
    __syncthreads();
    // this CTA's slice of the initial stack, without the lock (it lies above
    // the stack's top, and `pending` counts it already); the lowest position
    // ends on the buffer's top, so it is taken first, as from the stack
    {
        const unsigned pf = ld_volatile(&a.ctrl->prefill);
        const unsigned base = ld_volatile(&a.ctrl->prefill_base) + blockIdx.x * pf;
        for (unsigned j = threadIdx.x; j < pf; j += blockDim.x)
            s_cq.e[j] = __ldcg(&a.q0[base + pf - 1u - j]);
        if (threadIdx.x == 0) s_cq.n = (int)pf;
        __syncthreads();
    }
    long long idle_since = 0;
    unsigned idle_progress = 0u;
    unsigned ns = 64;
    bool idle = false;  // counted in ctrl->idle and s_cq.waiting
    auto leave_idle = [&]() {
        if (idle && lane == 0) {
            atomicSub(&a.ctrl->idle, 1u);
            atomicSub(&s_cq.waiting, 1);
        }
        idle = false;
    };
    for (;;) {
        if (ld_volatile(&a.ctrl->error) != 0u) break;
        const long long qr0 = clock64();
        unsigned g = cta_take(a, lane);
        int outcome = 0;  // 0 an entry, 1 exit, 2 nothing now
        if (g == ~0u) {
            int taker = 0;
            if (lane == 0) taker = atomicCAS(&s_cq.taker, 0, 1) == 0 ? 1 : 0;
            taker = __shfl_sync(FULL, taker, 0);
            if (taker) {
                outcome = mutex_global_take(a, lane, cnt, &g);
                __syncwarp();
                if (lane == 0) atomicExch(&s_cq.taker, 0);
            } else {
                // another warp of this CTA is at the global stack: wait for
                // its batch, leaving when the job is over
                int over = 0;
                if (lane == 0)
                    over = ld_volatile(&a.ctrl->pending) == 0 && stack_top(a.ctrl) == 0 &&
                           ld_volatile(&a.ctrl->overflow) == 0u;
                outcome = __shfl_sync(FULL, over, 0) ? 1 : 2;
            }
        }
        if (outcome == 1) break;
        if (outcome == 2) {
            // nothing to take but work in flight: back off, bounded by progress
            if (!idle) {
                if (lane == 0) {
                    atomicAdd(&a.ctrl->idle, 1u);
                    atomicAdd(&s_cq.waiting, 1);
                }
                idle = true;
            }
            const unsigned prog = ld_volatile(&a.ctrl->progress);
            const long long now = globaltimer_ns();
            if (idle_since == 0 || prog != idle_progress) {
                idle_since = now;
                idle_progress = prog;
            } else if (now - idle_since > a.timeout_ns) {
                if (lane == 0) set_error(a.ctrl, DEV_ERR_TIMEOUT);
                break;
            }
            __nanosleep(ns);
            if (ns < 2048) ns <<= 1;
            cnt.phase[0] += clock64() - qr0;
            continue;
        }
        leave_idle();
        idle_since = 0;
        ns = 64;
        cnt.phase[0] += clock64() - qr0;
        if (g >= a.G) {  // a consistency check: an entry names no tile
            if (lane == 0) set_error(a.ctrl, DEV_ERR_INTERNAL);
            break;
        }
        bool ok = true;
        for (;;) {  // the entry, then the newly dirty neighbours it leaves behind
            unsigned nxt = ~0u;
            ok = process_entry<VAR_MUTEX, TH>(a, g, sm, lane, nullptr, cnt, phase, &nxt);
            if (!ok || nxt == ~0u) break;
            g = nxt;
        }
        if (!ok) break;
        if (lane == 0) {
            __threadfence();
            atomicAdd(&a.ctrl->progress, 1u);
            atomicSub(&a.ctrl->pending, 1);  // after this entry's insertions
        }
        // share: the global stack is empty while warps elsewhere wait
        int share = 0;
        if (lane == 0 && cq_count() >= 2 && stack_top(a.ctrl) == 0 &&
            ld_volatile(&a.ctrl->idle) > (unsigned)*(volatile int*)&s_cq.waiting)
            share = 1;
        if (__shfl_sync(FULL, share, 0)) cta_spill(a, lane, __shfl_sync(FULL, cq_count(), 0) / 2);
    }
    leave_idle();
}

// ------------------------------------------------------- async worker
// Ring positions 0..n0-1 are the initial tiles (no storage: every tile in
// id order, or the seed list after the front stage); position p >= n0 lives in
// slot (p - n0) % cap.  A warp claims the next position with one
// atomicAdd and waits for a producer to fill it.  Every filled position is
// claimed by exactly one warp, and when `pending` (filled, unfinished
// entries) reaches zero no producer is left, so waiting warps leave.
template <int TH>
__device__ void async_worker(const EngineArgs& a, WarpSmem<TH>& sm, int lane, WarpCounters& cnt, unsigned& phase) {
    const unsigned n0 = ring_base(a);
    for (;;) {
        const long long qr0 = clock64();
        unsigned p = 0u;
        if (lane == 0) p = atomicAdd(&a.ctrl->ahead, 1u);
        p = __shfl_sync(FULL, p, 0);
        unsigned g = a.init_list && p < n0 ? __ldcg(&a.init_list[p]) : p;
        if (p >= n0) {
            int outcome = 0;  // 0 got an entry, 1 exit
            unsigned v = 0u;
            if (lane == 0) {
                const unsigned slot = (p - n0) % a.cap;
                long long idle_since = globaltimer_ns();
                unsigned idle_progress = ld_volatile(&a.ctrl->progress);
                unsigned ns = 32, spins = 0;
                for (;;) {
                    // The slot is this warp's alone: watch it with plain loads
                    // (a waiting warp issues no atomics) and take it once set.
                    if (ld_volatile(&a.q0[slot]) != 0u) {
                        v = atomicExch(&a.q0[slot], 0u);
                        break;
                    }
                    // the job's counters every eighth look
                    if ((++spins & 7u) == 0u) {
                        if (ld_volatile(&a.ctrl->pending) == 0 || ld_volatile(&a.ctrl->error) != 0u) {
                            outcome = 1;
                            break;
                        }
                        const unsigned prog = ld_volatile(&a.ctrl->progress);
                        const long long now = globaltimer_ns();
                        if (prog != idle_progress) {
                            idle_progress = prog;
                            idle_since = now;
                        } else if (now - idle_since > a.timeout_ns) {
                            set_error(a.ctrl, DEV_ERR_TIMEOUT);
                            outcome = 1;
                            break;
                        }
                    }
                    __nanosleep(ns);
                    if (ns < 256) ns <<= 1;
                }
            }
            outcome = __shfl_sync(FULL, outcome, 0);
            cnt.phase[0] += clock64() - qr0;
            if (outcome) return;
            g = __shfl_sync(FULL, v, 0) - 1u;
        } else {
            cnt.phase[0] += clock64() - qr0;
        }
        // visit the entry, then keep following the front while the visits
        // leave a newly dirty neighbour behind
        bool ok = true;
        for (;;) {
            unsigned nxt = ~0u;
            ok = process_entry<VAR_ASYNC, TH>(a, g, sm, lane, nullptr, cnt, phase, &nxt);
            if (!ok || nxt == ~0u) break;
            g = nxt;
        }
        if (lane == 0) {
            __threadfence();
            atomicAdd(&a.ctrl->progress, 1u);
            atomicSub(&a.ctrl->pending, 1);  // after this entry's insertions
        }
        if (!ok) return;
    }
}

// --------------------------------------------------------- grid barrier
// All CTAs of the (cooperative) launch.  The last CTA to arrive performs the
// round transition.  Waits are bounded; returns false when the job failed.
__device__ bool grid_barrier_round(const EngineArgs& a) {
    __shared__ int s_ok;
    __syncthreads();
    if (threadIdx.x == 0) {
        Ctrl* c = a.ctrl;
        int ok = 1;
        const unsigned gen = ld_volatile(&c->bar_gen);
        __threadfence();
        const unsigned arrived = atomicAdd(&c->bar_count, 1u);
        // (with the phantom-work test hook the barrier waits for one CTA
        // more than the grid has, so every waiter runs out of time)
        if (arrived == gridDim.x - 1u + (a.phantom ? 1u : 0u)) {
            // Round transition (IWPP MP DQ/src/globalQueue.cu:139-157 swapQueues,
            // UQ/src/globalQueue.cu:159-168 resetReadQueue, and the overflow
            // restart of DQ/MR.cu:1242-1323, all on the device).
            __threadfence();
            const unsigned wn = ld_volatile(&c->wn);
            unsigned rn;
            if (ld_volatile(&c->overflow) != 0u) {
                if ((int)c->restarts >= a.max_restarts) {
                    set_error(c, DEV_ERR_OVERFLOW);
                    rn = 0u;
                } else {
                    c->restarts += 1u;
                    c->vfull = 1u;
                    rn = a.G;
                }
                c->overflow = 0u;
            } else {
                c->vfull = 0u;
                rn = wn < a.cap ? wn : a.cap;
            }
            c->qsel ^= 1u;
            c->rn = rn;
            c->wn = 0u;
            c->rcur = 0u;
            c->rounds += 1u;
            if (rn == 0u || ld_volatile(&c->error) != 0u) c->done = 1u;
            c->bar_count = 0u;
            __threadfence();
            atomicAdd(&c->bar_gen, 1u);
        } else {
            const long long t0 = globaltimer_ns();
            unsigned ns = 64;
            while (ld_volatile(&c->bar_gen) == gen) {
                __nanosleep(ns);
                if (ns < 2048) ns <<= 1;
                if (ld_volatile(&c->error) != 0u) {
                    ok = 0;
                    break;
                }
                if (globaltimer_ns() - t0 > a.timeout_ns) {
                    set_error(c, DEV_ERR_TIMEOUT);
                    ok = 0;
                    break;
                }
            }
            __threadfence();
        }
        s_ok = ok;
    }
    __syncthreads();
    return s_ok != 0;
}

// ------------------------------------------------------- round worker
template <int VAR, int TH>
__device__ void round_worker(const EngineArgs& a, WarpSmem<TH>& sm, int lane, WarpCounters& cnt, unsigned& phase) {
    for (;;) {
        const unsigned rn = ld_volatile(&a.ctrl->rn);
        const unsigned vfull = ld_volatile(&a.ctrl->vfull);
        const unsigned qsel = ld_volatile(&a.ctrl->qsel);
        const unsigned* rq = qsel ? a.q1 : a.q0;
        unsigned* wq = qsel ? a.q0 : a.q1;
        for (;;) {
            const long long qr0 = clock64();
            unsigned idx = 0u;
            if (lane == 0) idx = atomicAdd(&a.ctrl->rcur, 1u);
            idx = __shfl_sync(FULL, idx, 0);
            cnt.phase[0] += clock64() - qr0;
            if (idx >= rn) break;
            if (ld_volatile(&a.ctrl->error) != 0u) break;
            const unsigned g = vfull ? idx : __ldcg(&rq[idx]);
            if (!process_entry<VAR, TH>(a, g, sm, lane, wq, cnt, phase)) break;
        }
        const long long qb0 = clock64();
        const bool ok_barrier = grid_barrier_round(a);
        cnt.phase[0] += clock64() - qb0;
        if (!ok_barrier) return;
        if (ld_volatile(&a.ctrl->done) != 0u) return;
    }
}

// --------------------------------------------------------------- kernels
template <int VAR, int TH>
__global__ void __launch_bounds__(kWarps * 32) engine_kernel(EngineArgs a) {
    extern __shared__ __align__(128) unsigned char smem_raw[];
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    // 128-byte align the per-warp areas (the launch adds 128 bytes of slack)
    const uint32_t base = smem_u32(smem_raw);
    unsigned char* aligned = smem_raw + ((128u - (base & 127u)) & 127u);
    WarpSmem<TH>& sm = reinterpret_cast<WarpSmem<TH>*>(aligned)[warp];
    if (lane == 0) {
        mbar_init(&sm.mbar, 1u);
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    __syncthreads();
    unsigned phase = 0u;
    WarpCounters cnt;
    if (VAR == VAR_MUTEX)
        mutex_worker<TH>(a, sm, lane, cnt, phase);
    else if (VAR == VAR_ASYNC)
        async_worker<TH>(a, sm, lane, cnt, phase);
    else
        round_worker<VAR, TH>(a, sm, lane, cnt, phase);
    if (lane == 0) {
        if (cnt.visits) atomicAdd(&a.ctrl->visits, cnt.visits);
        if (cnt.sweeps) atomicAdd(&a.ctrl->sweeps, cnt.sweeps);
        if (cnt.pushes) atomicAdd(&a.ctrl->pushes, cnt.pushes);
        if (cnt.row_steps) atomicAdd(&a.ctrl->row_steps, cnt.row_steps);
        for (int i = 0; i < 5; ++i)
            if (cnt.phase[i] > 0) atomicAdd(&a.ctrl->phase[i], (unsigned long long)cnt.phase[i]);
    }
}

// Job initialisation: every tile DIRTY; round 0 (double / unique) is the
// virtual list of all tiles; the mutex stack holds every tile so that the
// first pops come out in raster order (IWPP MP/src/globalQueue.cu:83-97,
// initFillGlobalQueue).  After the front stage (or a seed check alone) the
// check has set the tile states and listed the tiles to start from: the
// mutex stack and the first round's read queue are that list, the async
// ring starts from it; the stage's error word and top-pixel count stand.
__global__ void engine_init_kernel(EngineArgs a, int variant) {
    const unsigned stride = gridDim.x * blockDim.x;
    const bool seeded = a.init_list != nullptr;
    unsigned n0 = a.G;
    if (seeded) n0 = min(*(const volatile unsigned*)a.init_count, a.G);
    for (unsigned g = blockIdx.x * blockDim.x + threadIdx.x; g < a.G; g += stride) {
        if (!seeded && !a.states_set) a.state[g] = ST_DIRTY | ST_SIDES;
        if (variant == VAR_MUTEX && g < a.cap) a.q0[g] = seeded ? (g < n0 ? a.init_list[g] : 0u) : a.G - 1u - g;
        if ((variant == VAR_DOUBLE || variant == VAR_UNIQUE) && seeded && g < n0 && g < a.cap) a.q0[g] = a.init_list[g];
    }
    if (variant == VAR_ASYNC)
        for (unsigned i = blockIdx.x * blockDim.x + threadIdx.x; i < a.cap; i += stride) a.q0[i] = 0u;
    if (blockIdx.x == 0 && threadIdx.x == 0) {
        Ctrl* c = a.ctrl;
        c->rn = n0;
        c->wn = 0u;
        c->rcur = 0u;
        c->qsel = 0u;
        c->vfull = seeded ? 0u : 1u;
        c->done = n0 == 0u ? 1u : 0u;
        c->overflow = n0 > a.cap && variant == VAR_MUTEX ? 1u : 0u;
        c->restarts = 0u;
        c->rounds = 0u;
        c->bar_count = 0u;
        c->bar_gen = 0u;
        if (!a.front) c->error = 0u;  // else the seed check's job keeps its error word
        c->lock_next = 0u;
        // the mutex stack's first entries: a slice per CTA taken without the
        // lock when the kernel starts (at most half a CTA buffer each), the
        // rest stacked
        const unsigned stacked = n0 < a.cap ? n0 : a.cap;
        const unsigned ctas = a.grid > 0 ? (unsigned)a.grid : 1u;
        unsigned pf = variant == VAR_MUTEX ? stacked / ctas : 0u;
        if (pf > (unsigned)kMutexPrefill) pf = (unsigned)kMutexPrefill;
        c->prefill = pf;
        c->prefill_base = stacked - pf * ctas;
        c->lock_word = (unsigned long long)(stacked - pf * ctas) << 32;  // ticket 0 served
        c->pending = (int)(n0 < a.cap ? n0 : a.cap);
        c->progress = 0u;
        c->idle = 0u;
        c->ahead = 0u;
        c->atail = n0;
        c->ninit = n0;
        if (variant == VAR_ASYNC) c->pending = (int)n0;
        // test hook: one pending entry that nobody inserts or finishes, so
        // the waiting warps never see the job end and their bounded waits
        // run out (the round-based queues stall at their barrier instead)
        if (a.phantom) c->pending += 1;
        c->visits = 0ull;
        c->sweeps = 0ull;
        c->pushes = 0ull;
        c->row_steps = 0ull;
        for (int i = 0; i < 5; ++i) c->phase[i] = 0ull;
        if (!a.front) c->top_pixels = 0ull;  // else the top-level stage's count stands
        if (!a.front_gated) c->front_gate = a.front_ran ? 1u : 0u;  // else the device's decision stands
    }
}

// ------------------------------------------------------- queue self-test
// The counterpart of the reference's queue test (IWPP MP DQ/src/
// globalQueue.cu:161-253: fill a 128 x 128 tile-id queue several times, read
// it back, check every id's count): all warps insert every tile id `copies`
// times at once through the variant's own insertion path (push_entries:
// mutex stack, warp-aggregated write-queue reservations, async ring; the
// unique queue deduplicates through the tile state word as notify does),
// then the queue's contents are counted per id.
struct QueueTest {
    unsigned* hist;          // G counters
    unsigned long long* out;  // [0] entries found, [1] ids with a wrong count, [2] smallest such id
};

__global__ void queue_test_init_kernel(EngineArgs a, QueueTest t) {
    const unsigned stride = gridDim.x * blockDim.x;
    for (unsigned g = blockIdx.x * blockDim.x + threadIdx.x; g < a.G; g += stride) {
        a.state[g] = 0u;
        t.hist[g] = 0u;
    }
    for (unsigned i = blockIdx.x * blockDim.x + threadIdx.x; i < a.cap; i += stride) {
        a.q0[i] = 0u;
        a.q1[i] = 0u;
    }
    if (blockIdx.x == 0 && threadIdx.x == 0) {
        Ctrl* c = a.ctrl;
        c->wn = 0u;
        c->overflow = 0u;
        c->error = 0u;
        c->lock_next = 0u;
        c->lock_word = 0ull;
        c->pending = 0;
        c->atail = a.G;  // ring positions below G are the (absent) initial tiles
        t.out[0] = 0ull;
        t.out[1] = 0ull;
        t.out[2] = ~0ull;
    }
}

template <int VAR>
__global__ void queue_test_insert_kernel(EngineArgs a, int copies) {
    const int lane = threadIdx.x & 31;
    const unsigned warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const unsigned nwarps = (gridDim.x * blockDim.x) >> 5;
    const unsigned total = a.G * (unsigned)copies;
    WarpCounters cnt;
    for (unsigned base = warp * 32u; base < total; base += nwarps * 32u) {
        const unsigned idx = base + (unsigned)lane;
        bool want = idx < total;
        const unsigned g = want ? idx % a.G : 0u;
        if (VAR == VAR_UNIQUE && want) want = (atomicOr(&a.state[g], ST_DIRTY) & ST_DIRTY) == 0u;
        push_entries<VAR>(a, want, g, lane, a.q1, cnt);
        if (ld_volatile(&a.ctrl->error) != 0u) return;
    }
}

__global__ void queue_test_count_kernel(EngineArgs a, int variant, QueueTest t) {
    const Ctrl* c = a.ctrl;
    unsigned n;
    if (variant == VAR_MUTEX) n = (unsigned)stack_top(c);
    else if (variant == VAR_ASYNC) n = c->atail - a.G;
    else n = c->wn;
    if (n > a.cap) n = a.cap;
    if (blockIdx.x == 0 && threadIdx.x == 0) t.out[0] = n;
    const unsigned stride = gridDim.x * blockDim.x;
    for (unsigned i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += stride) {
        unsigned e = variant == VAR_MUTEX ? a.q0[i] : variant == VAR_ASYNC ? a.q0[i] - 1u : a.q1[i];
        if (e < a.G) atomicAdd(&t.hist[e], 1u);
    }
}

__global__ void queue_test_check_kernel(EngineArgs a, QueueTest t, unsigned expect) {
    const unsigned stride = gridDim.x * blockDim.x;
    for (unsigned g = blockIdx.x * blockDim.x + threadIdx.x; g < a.G; g += stride) {
        if (t.hist[g] != expect) {
            atomicAdd(&t.out[1], 1ull);
            atomicMin(&t.out[2], (unsigned long long)g);
        }
    }
}

cudaError_t queue_selftest(const EngineArgs& a, int variant, int copies, unsigned* hist, unsigned long long* out,
                           int device, cudaStream_t s) {
    int sms = 0;
    cudaError_t e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device);
    if (e != cudaSuccess) return e;
    QueueTest t{hist, out};
    const unsigned blocks = (unsigned)sms * 4u;
    queue_test_init_kernel<<<blocks, 256, 0, s>>>(a, t);
    switch (variant) {
        case VAR_MUTEX: queue_test_insert_kernel<VAR_MUTEX><<<blocks, 128, 0, s>>>(a, copies); break;
        case VAR_DOUBLE: queue_test_insert_kernel<VAR_DOUBLE><<<blocks, 128, 0, s>>>(a, copies); break;
        case VAR_UNIQUE: queue_test_insert_kernel<VAR_UNIQUE><<<blocks, 128, 0, s>>>(a, copies); break;
        default: queue_test_insert_kernel<VAR_ASYNC><<<blocks, 128, 0, s>>>(a, copies); break;
    }
    queue_test_count_kernel<<<blocks, 256, 0, s>>>(a, variant, t);
    queue_test_check_kernel<<<blocks, 256, 0, s>>>(a, t, variant == VAR_UNIQUE ? 1u : (unsigned)copies);
    return cudaGetLastError();
}

// ------------------------------------------------------------ host side
template <int VAR, int TH>
static void* kernel_ptr() {
    return reinterpret_cast<void*>(&engine_kernel<VAR, TH>);
}

static void* select_kernel(int variant, int tile_rows) {
    if (tile_rows == 32) {
        if (variant == VAR_MUTEX) return kernel_ptr<VAR_MUTEX, 32>();
        if (variant == VAR_DOUBLE) return kernel_ptr<VAR_DOUBLE, 32>();
        if (variant == VAR_ASYNC) return kernel_ptr<VAR_ASYNC, 32>();
        return kernel_ptr<VAR_UNIQUE, 32>();
    }
    if (variant == VAR_MUTEX) return kernel_ptr<VAR_MUTEX, 64>();
    if (variant == VAR_DOUBLE) return kernel_ptr<VAR_DOUBLE, 64>();
    if (variant == VAR_ASYNC) return kernel_ptr<VAR_ASYNC, 64>();
    return kernel_ptr<VAR_UNIQUE, 64>();
}

static size_t smem_bytes(int tile_rows) {
    return 128 + (tile_rows == 32 ? kWarps * sizeof(WarpSmem<32>) : kWarps * sizeof(WarpSmem<64>));
}

cudaError_t engine_prepare(int variant, int tile_rows, int device, LaunchInfo* li) {
    void* k = select_kernel(variant, tile_rows);
    const size_t smem = smem_bytes(tile_rows);
    cudaError_t e = cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
    int per_sm = 0, sms = 0;
    e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k, kWarps * 32, smem);
    if (e != cudaSuccess) return e;
    e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device);
    if (e != cudaSuccess) return e;
    li->grid = per_sm * sms;
    li->block = kWarps * 32;
    li->smem = smem;
    return li->grid > 0 ? cudaSuccess : cudaErrorInvalidConfiguration;
}

cudaError_t engine_launch_init(const EngineArgs& a, int variant, cudaStream_t s) {
    unsigned blocks = (a.G + 255u) / 256u;
    if (blocks == 0u) blocks = 1u;
    if (blocks > 4096u) blocks = 4096u;
    engine_init_kernel<<<blocks, 256, 0, s>>>(a, variant);
    return cudaGetLastError();
}

cudaError_t engine_launch(const EngineArgs& a, int variant, int tile_rows, int grid, cudaStream_t s) {
    void* k = select_kernel(variant, tile_rows);
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3((unsigned)grid);
    cfg.blockDim = dim3(kWarps * 32);
    cfg.dynamicSmemBytes = smem_bytes(tile_rows);
    cfg.stream = s;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeCooperative;
    attr[0].val.cooperative = 1;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    EngineArgs args = a;
    void* params[] = {&args};
    return cudaLaunchKernelExC(&cfg, k, params);
}

}  // namespace iwpp
