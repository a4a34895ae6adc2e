// iwpp_engine.cuh -- the persistent tile engine and its three work queues.
//
// Reference counterparts:
//   MUTEX  IWPP MP/src/globalQueue.cu:25-81 (insert under a spin mutex),
//          :100-155 (read one entry under the mutex, activeBlocksCount
//          termination), MR.cu:163-542 (one persistent launch), overflow
//          restart MR.cu:785-806.
//   DOUBLE IWPP MP DQ/src/globalQueue.cu:14-47 (atomicAdd reservation),
//          :139-157 (swapQueues), MR.cu:1242-1323 (one launch per round,
//          host reads the queue size back every round).
//   UNIQUE IWPP MP UQ/src/MorphologicalReconstruction.cu:1152-1293
//          (per-tile flag de-duplication between rounds).
//   ASYNC  no reference counterpart: the unique queue without rounds, as a
//          lock-free ring of tile ids claimed and filled with fetch-and-add.
//
// GB300 form: one persistent launch for all of them.  The double / unique
// rounds are separated by a device-wide barrier (cooperative launch) instead
// of a host round trip, the unique queue de-duplicates when a tile is
// inserted, and all insertions are warp-aggregated (one atomic per warp).
//
// Tile ownership.  Each tile has a state word: DIRTY (needs a visit) and
// ACTIVE (a warp is visiting it).  A warp that takes a tile sets ACTIVE; if
// it was already set the entry is dropped (the owner will see DIRTY and
// revisit).  The owner clears DIRTY before it reads the tile and releases
// with CAS(ACTIVE -> 0), revisiting while DIRTY reappears.  So at most one
// warp writes a tile's pixels, with plain stores, and every write that can
// raise a neighbour is followed by DIRTY on that neighbour after a fence.
#pragma once

#include "iwpp_device.cuh"

namespace iwpp {

// Tile state word: DIRTY, ACTIVE, and (bits 8-15, NB_* << 8) the sides whose
// halo pixels rose since the tile last converged.
enum : unsigned { ST_DIRTY = 1u, ST_ACTIVE = 2u, ST_SIDE_SHIFT = 8u, ST_SIDES = 0xffu << 8 };
enum : int { VAR_MUTEX = 0, VAR_DOUBLE = 1, VAR_UNIQUE = 2, VAR_ASYNC = 3 };
enum : unsigned { DEV_OK = 0u, DEV_ERR_TIMEOUT = 3u, DEV_ERR_OVERFLOW = 5u, DEV_ERR_INTERNAL = 9u };

constexpr int kWarps = 4;       // warps (independent tile workers) per CTA
constexpr int kMutexBatch = 8;  // entries taken per mutex acquisition
constexpr int kMutexPrefill = 32;  // initial stack entries a CTA takes without the lock

struct Ctrl {
    unsigned rn;        // entries in the read queue (this round)
    unsigned wn;        // insertions into the write queue (may exceed cap)
    unsigned rcur;      // read cursor
    unsigned qsel;      // read queue = qsel ? q1 : q0
    unsigned vfull;     // the read queue is every tile 0..G-1
    unsigned done;
    unsigned overflow;  // an insertion did not fit since the last restart
    unsigned restarts;
    unsigned rounds;
    unsigned bar_count;
    unsigned bar_gen;
    unsigned error;
    unsigned lock_next;  // mutex stack: the ticket lock's next ticket
    // mutex stack: the ticket being served (low half) and the number of
    // stacked entries (high half) in one word, so a hand-over publishes the
    // stack's top with the lock and the next holder reads both in one load
    unsigned long long lock_word;
    int pending;        // mutex: entries in the stack or taken and unfinished
    unsigned progress;  // finished entries (for the no-progress timeout)
    unsigned ahead;     // async ring: next position to claim
    unsigned atail;     // async ring: next position to fill
    unsigned long long visits;
    unsigned long long sweeps;
    unsigned long long pushes;
    unsigned long long row_steps;
    unsigned long long phase[5];  // cycles: queue read, fetch, processing, dump, queue write
    unsigned long long top_pixels;    // pixels the top-level stage labelled
    unsigned ninit;     // initial entries (every tile, or the seed list after the front stage)
    unsigned front_gate;  // front stage decided on the device: 1 run it, 0 leave the job to the engine
    unsigned idle;        // mutex: warps waiting for work
    unsigned prefill;     // mutex: initial entries each CTA takes without the lock
    unsigned prefill_base;  // mutex: stack position of CTA 0's slice (the stack's top below it)
};

struct EngineArgs {
    const ImgDesc* imgs;
    int nimg;
    unsigned G;         // tiles in the job
    unsigned* state;    // G tile state words
    unsigned* q0;       // queue buffers, cap entries each
    unsigned* q1;
    unsigned cap;
    Ctrl* ctrl;
    long long timeout_ns;
    int max_restarts;
    int solver;  // 0 automatic, 1 row sweeps, 2 passes
    int phantom;  // test hook: one unit of work that never arrives (every wait runs out)
    int grid;     // CTAs of the engine launch (the mutex stack's first entries are split among them)
    int front;    // a seed check ran: the job's error word and top-pixel count stand
    int states_set;   // the seed check set every tile's state: the queue holds every tile in order,
                      // clean tiles are released at once
    int front_ran;    // the front stage ran (not gated)
    int front_gated;  // the device decided whether the stage ran (Ctrl::front_gate)
    // After the front stage: the tiles to start from (ids) and their count (a
    // device counter); nullptr: every tile, in id order.  The tile states
    // were set by the seed check.
    const unsigned* init_list;
    const unsigned* init_count;
};

}  // namespace iwpp

// Host-side entry points implemented in iwpp_engine.cu.
namespace iwpp {
struct LaunchInfo {
    int grid;
    int block;
    size_t smem;
};
cudaError_t engine_prepare(int variant, int tile_rows, int device, LaunchInfo* li);
cudaError_t engine_launch_init(const EngineArgs& a, int variant, cudaStream_t s);
cudaError_t engine_launch(const EngineArgs& a, int variant, int tile_rows, int grid, cudaStream_t s);
cudaError_t launch_clip(const ImgDesc& d, cudaStream_t s);
// Adds to *count the pixels of d.marker that a neighbour could still raise.
cudaError_t launch_fixed_point_check(const ImgDesc& d, unsigned long long* count, cudaStream_t s);
// Queue self-test on workspace `a` (state G words, q0 / q1 cap entries each):
// insert every tile id `copies` times through the variant's insertion path,
// count the queue's contents into hist (G words); out[0] entries found,
// out[1] ids with a wrong count, out[2] the smallest such id.
cudaError_t queue_selftest(const EngineArgs& a, int variant, int copies, unsigned* hist, unsigned long long* out,
                           int device, cudaStream_t s);
// Whole-image sweep; 4-connected vertical sweeps of tall uint8 / uint16
// images use `scratch` (sweep_scratch_bytes(d) bytes, nullable) to split the
// columns into segments.
// `launches` (nullable) is incremented by the number of kernels launched.
cudaError_t launch_sweep(const ImgDesc& d, int direction, cudaStream_t s, void* scratch = nullptr,
                         int* launches = nullptr);
size_t sweep_scratch_bytes(const ImgDesc& d);
}  // namespace iwpp
