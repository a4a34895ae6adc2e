// iwpp_tune.h -- the process-wide tuning table (internal to libiwpp).
//
// Entries map a workload class to the configuration the autotuner found
// fastest for it.  The class is (queue variant, pixel type, connectivity,
// pixel-count class = floor(log2(total pixels)), single image or batch);
// a batch of mixed types or connectivities uses -1 for that field.
#pragma once

#include <string>

namespace iwpp {

struct TuneKey {
    int variant;
    int dtype;    // IWPP_U8 / U16 / I32, or -1 for a mixed batch
    int conn;     // 4 / 8, or -1 for a mixed batch
    int pxclass;  // floor(log2(total pixels))
    int batch;    // 0 single image, 1 several
    bool operator<(const TuneKey& o) const;
};

struct TuneEntry {
    int tile_rows;   // 32 / 64
    int solver;      // 0 / 1 / 2
    int init_passes;
    int queue_mult;  // queue capacity in tiles per tile of the job; 0 = the variant's default
    int front_passes;  // 0 = no front stage, 1 = always, 2 = decided on the device, 3 = the seed check alone
};

// iwpp_config.front_passes (1 always, 2 never, 3 decided on the device, 4 the
// seed check alone) of a table entry's front_passes, and back.
inline int tune_front_code(int stored) { return stored == 1 ? 1 : stored == 2 ? 3 : stored == 3 ? 4 : 2; }
inline int tune_front_store(int code) { return code == 1 ? 1 : code == 3 ? 2 : code == 4 ? 3 : 0; }

int resolve_queue_variant(int variant);  // iwpp_api.cu: IWPP_QUEUE_DEFAULT -> the variant used
TuneKey tune_key(int variant, const int* dtypes, const int* conns, const long long* pixels, int n);
bool tune_lookup(const TuneKey& k, TuneEntry* e);
void tune_store(const TuneKey& k, const TuneEntry& e);

}  // namespace iwpp
