// iwpp_top.cuh -- the front stage (iwpp_top.cu): reconstruction of the
// image's top level set by connected-component labelling, and the check that
// seeds the tile engine after the whole-image passes.
#pragma once

#include <vector>

#include "iwpp_device.cuh"

namespace iwpp {

// Device scratch the top-level stage over image d needs.
size_t top_scratch_bytes(const ImgDesc& d);
// Enqueues the top-level stage over image d: the pixels whose mask is at the
// image's largest value rise to the largest marker (capped at that value) of
// their connected set of such pixels.  *top_pixels (device) counts the
// pixels labelled.  `launches` (nullable) counts the kernels launched.
cudaError_t launch_top(const ImgDesc& d, void* scratch, unsigned long long* top_pixels, int device, cudaStream_t s,
                       int* launches);
// Marks every engine tile of image d (tile height d.tile_rows) that holds a
// pixel a neighbour could raise DIRTY in `state` (others 0) and appends its
// global id to `list`, counting in *nlist.  With d.gate set it does nothing
// while *d.gate is 0 (so do the top-level stage and the sweeps).
cudaError_t launch_seed(const ImgDesc& d, unsigned* state, unsigned* list, unsigned* nlist, cudaStream_t s,
                        int* launches);
// The same check over every image of a job in one launch (one launch per
// image when the job has more than 1024).  `dev_descs`: the job's descriptors in device
// memory (`host_descs` the same on the host); `gate` (nullable) as
// ImgDesc::gate.
cudaError_t launch_seed_batch(const ImgDesc* dev_descs, const std::vector<ImgDesc>& host_descs, const unsigned* gate,
                              unsigned* state, unsigned* list, unsigned* nlist, cudaStream_t s, int* launches);
// After a seed check over a job's G tiles (its count in *count): *gate = 1
// and *count = 0 when the initial front is small enough for the front stage
// to pay, else *gate = 0 (the list stands and seeds the engine).
cudaError_t launch_front_decide(unsigned* gate, unsigned* count, unsigned G, cudaStream_t s, int* launches);

}  // namespace iwpp
