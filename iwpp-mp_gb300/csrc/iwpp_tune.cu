// iwpp_tune.cu -- the tuning table behind iwpp_autotune: lookup / store for
// the library and save / load / clear / lookup for callers.  Host code only.
// Declarations: include/iwpp.h (iwpp_tune_*), iwpp_tune.h.
#include <cstdio>
#include <map>
#include <mutex>
#include <tuple>

#include "iwpp.h"
#include "iwpp_tune.h"

namespace iwpp {

bool TuneKey::operator<(const TuneKey& o) const {
    return std::tie(variant, dtype, conn, pxclass, batch) < std::tie(o.variant, o.dtype, o.conn, o.pxclass, o.batch);
}

namespace {
std::mutex g_mu;
std::map<TuneKey, TuneEntry>& table() {
    static std::map<TuneKey, TuneEntry> t;
    return t;
}
}  // namespace

TuneKey tune_key(int variant, const int* dtypes, const int* conns, const long long* pixels, int n) {
    TuneKey k{variant, n > 0 ? dtypes[0] : 0, n > 0 ? conns[0] : 8, 0, n > 1 ? 1 : 0};
    long long total = 0;
    for (int i = 0; i < n; ++i) {
        if (dtypes[i] != k.dtype) k.dtype = -1;
        if (conns[i] != k.conn) k.conn = -1;
        total += pixels[i];
    }
    int c = 0;
    while (c < 62 && (2ll << c) <= total) ++c;
    k.pxclass = total > 0 ? c : 0;
    return k;
}

bool tune_lookup(const TuneKey& k, TuneEntry* e) {
    std::lock_guard<std::mutex> lk(g_mu);
    auto it = table().find(k);
    if (it == table().end()) return false;
    *e = it->second;
    return true;
}

void tune_store(const TuneKey& k, const TuneEntry& e) {
    std::lock_guard<std::mutex> lk(g_mu);
    table()[k] = e;
}

}  // namespace iwpp

using namespace iwpp;

namespace {
bool valid_entry(const TuneEntry& e) {
    return (e.tile_rows == 32 || e.tile_rows == 64) && e.solver >= 0 && e.solver <= 3 && e.init_passes >= 0 &&
           e.init_passes <= 64 && e.queue_mult >= 0 && e.queue_mult <= 1024 && e.front_passes >= 0 &&
           e.front_passes <= 3;
}
}  // namespace

extern "C" {

int iwpp_tune_save(const char* path) {
    if (!path) return IWPP_ERR_INVALID;
    FILE* f = std::fopen(path, "w");
    if (!f) return IWPP_ERR_INVALID;
    std::lock_guard<std::mutex> lk(g_mu);
    std::fprintf(f,
                 "# iwpp tuning table v2: variant dtype conn pxclass batch tile_rows solver init_passes queue_mult "
                 "front_passes\n");
    for (const auto& kv : table()) {
        const TuneKey& k = kv.first;
        const TuneEntry& e = kv.second;
        std::fprintf(f, "%d %d %d %d %d %d %d %d %d %d\n", k.variant, k.dtype, k.conn, k.pxclass, k.batch,
                     e.tile_rows, e.solver, e.init_passes, e.queue_mult, e.front_passes);
    }
    const bool ok = std::fclose(f) == 0;
    return ok ? IWPP_OK : IWPP_ERR_INVALID;
}

int iwpp_tune_load(const char* path) {
    if (!path) return IWPP_ERR_INVALID;
    FILE* f = std::fopen(path, "r");
    if (!f) return IWPP_ERR_INVALID;
    char line[256];
    int rc = IWPP_OK;
    std::map<TuneKey, TuneEntry> loaded;
    while (std::fgets(line, sizeof(line), f)) {
        if (line[0] == '#' || line[0] == '\n') continue;
        TuneKey k;
        TuneEntry e{};
        // v1 lines have nine fields (no front_passes: 0), v2 lines ten
        char extra = 0;
        const int got = std::sscanf(line, "%d %d %d %d %d %d %d %d %d %d %c", &k.variant, &k.dtype, &k.conn,
                                    &k.pxclass, &k.batch, &e.tile_rows, &e.solver, &e.init_passes, &e.queue_mult,
                                    &e.front_passes, &extra);
        if (got == 9) e.front_passes = 0;
        if ((got != 9 && got != 10) || !valid_entry(e)) {
            rc = IWPP_ERR_INVALID;
            break;
        }
        loaded[k] = e;
    }
    std::fclose(f);
    if (rc != IWPP_OK) return rc;  // a malformed file changes nothing
    std::lock_guard<std::mutex> lk(g_mu);
    for (const auto& kv : loaded) table()[kv.first] = kv.second;
    return IWPP_OK;
}

int iwpp_tune_clear(void) {
    std::lock_guard<std::mutex> lk(g_mu);
    table().clear();
    return IWPP_OK;
}

int iwpp_tune_entries(void) {
    std::lock_guard<std::mutex> lk(g_mu);
    return (int)table().size();
}

int iwpp_tune_lookup(int variant, int dtype, int connectivity, long long pixels, int batch, iwpp_config* out) {
    if (!out || pixels < 0) return IWPP_ERR_INVALID;
    const int dt[1] = {dtype};
    const int cn[1] = {connectivity};
    const long long px[1] = {pixels};
    TuneKey k = tune_key(resolve_queue_variant(variant), dt, cn, px, 1);
    k.batch = batch ? 1 : 0;
    TuneEntry e;
    if (!tune_lookup(k, &e)) return IWPP_ERR_INVALID;
    *out = iwpp_config{};
    out->tile_rows = e.tile_rows;
    out->solver = e.solver;
    out->init_passes = e.init_passes;
    out->queue_capacity = -e.queue_mult;  // negative: a multiple of the job's tile count
    out->front_passes = tune_front_code(e.front_passes);
    return IWPP_OK;
}

}  // extern "C"
