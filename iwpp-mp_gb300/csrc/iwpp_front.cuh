// iwpp_front.cuh -- front passes (iwpp_front.cu): whole-image directional
// sweeps restricted to the tiles that changed, and the check that seeds the
// tile engine afterwards.
#pragma once

#include "iwpp_device.cuh"

namespace iwpp {

// Bookkeeping of one front-pass run (device memory, zeroed before the run).
struct FrontCtrl {
    unsigned bar_count;   // grid barrier: CTAs arrived
    unsigned bar_gen;     // grid barrier: generation
    unsigned error;       // 3: a bounded wait ran out
    unsigned done;        // the passes are over
    unsigned changed[4];  // sweep s raised a pixel (slot s % 4)
    unsigned sweeps;      // sweeps run
    unsigned pad[7];
};

struct FrontArgs {
    ImgDesc d;          // the image (marker, mask, pitches, size, pixel type)
    int tx_n, ty_n;     // tracking tiles: 128 bytes x 64 rows
    int aligned16;      // rows start on 16-byte boundaries (tiles staged by cp.async)
    int* chg;           // per tile: last sweep that raised one of its pixels (-1: before the first)
    int* bchg;          // per row band of tiles: last sweep that raised a pixel in it
    int* cchg;          // per tile column: the last vertical sweep in which it held a dirty tile
    uint32_t* bmin;     // per tile and lane word: the least mask of the tile's pixel columns
    uint32_t* segA;     // per tile and lane word: exit pixels of the tile when nothing enters
    uint32_t* segIn;    // per tile and lane word: the value entering the tile
    FrontCtrl* fc;
    unsigned* job_error;             // the job's error word: set on a timeout
    unsigned long long* job_sweeps;  // the job's sweep count: the passes add theirs
    int max_sweeps;
    long long timeout_ns;
};

// Device scratch one front-pass run over image d needs.
size_t front_scratch_bytes(const ImgDesc& d);
// Enqueues the front passes over image d (scratch: front_scratch_bytes(d)
// bytes).  A timeout sets *job_error; the sweeps run are added to
// *job_sweeps.  `launches` (nullable) counts the kernels launched.
cudaError_t launch_front(const ImgDesc& d, void* scratch, unsigned* job_error, unsigned long long* job_sweeps,
                         int max_sweeps, long long timeout_ns, int device, cudaStream_t s, int* launches);
// Marks every engine tile of image d (tile height d.tile_rows) that holds a
// pixel a neighbour could raise DIRTY in `state` (others 0) and appends its
// global id to `list`, counting in *nlist.
cudaError_t launch_seed(const ImgDesc& d, unsigned* state, unsigned* list, unsigned* nlist, cudaStream_t s,
                        int* launches);

}  // namespace iwpp
