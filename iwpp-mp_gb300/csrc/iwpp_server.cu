// iwpp_server.cu -- the serving loop: requests admitted by a device-memory
// budget, continuous batching over several lanes (stream + workspace +
// worker thread each), device memory from a pool that stays resident.
// Declarations: include/iwpp.h (iwpp_server_*).
//
// The reference has no serving form: its only caller reconstructs one image
// per process (IWPP MP/src/main.cu:59).  This file sits above the library's
// own batch entry point (iwpp_reconstruct_batch_async): every batch is one
// persistent launch over all the tiles of its requests.
#include <algorithm>
#include <chrono>
#include <condition_variable>
#include <cstdint>
#include <cstring>
#include <deque>
#include <mutex>
#include <new>
#include <thread>
#include <unordered_map>
#include <vector>

#include <cuda_runtime.h>

#include "iwpp.h"

namespace iwpp {
int handle_reserve(iwpp_handle h, size_t bytes);  // iwpp_api.cu
}

namespace {

using Clock = std::chrono::steady_clock;

int bpp_of(int dtype) { return dtype == IWPP_U8 ? 1 : dtype == IWPP_U16 ? 2 : 4; }
size_t round_up(size_t v, size_t a) { return (v + a - 1) / a * a; }

double us_between(Clock::time_point a, Clock::time_point b) {
    return std::chrono::duration<double, std::micro>(b - a).count();
}

struct Request {
    unsigned long long id = 0;
    const void* marker = nullptr;
    const void* mask = nullptr;
    void* out = nullptr;
    size_t pm = 0, pk = 0, po = 0;
    int w = 0, h = 0, dtype = 0, conn = 8;
    size_t pitch = 0;       // device row pitch of the staging copies
    size_t bytes = 0;       // device bytes charged against the budget
    void* d_marker = nullptr;
    void* d_mask = nullptr;
    Clock::time_point t_submit, t_admit, t_done;
    int status = IWPP_OK;
    int lane = -1;
    int batch_size = 0;
    bool done = false;
};

}  // namespace

struct iwpp_server_s {
    int device = 0;
    int lanes_n = 3;
    int max_batch = 256;
    int max_pending = 65536;
    int variant = IWPP_QUEUE_DEFAULT;
    int tile_rows = 0;
    iwpp_config cfg{};
    long long budget = 0;
    long long headroom = 0;  // < 0: no live check
    cudaMemPool_t pool = nullptr;

    std::mutex mu;
    std::condition_variable cv_work;  // lanes: a request arrived or memory came free
    std::condition_variable cv_done;  // waiters: a request finished
    std::deque<Request*> pending;
    std::unordered_map<unsigned long long, Request*> live;
    unsigned long long next_id = 1;
    long long in_use = 0;
    long long unallocated = 0;  // admitted bytes whose pool allocations are not made yet
    bool stopping = false;
    iwpp_server_stats stats{};

    struct Lane {
        std::thread th;
        cudaStream_t stream = nullptr;
        iwpp_handle handle = nullptr;
    };
    std::vector<Lane> lanes;

    void lane_main(int li);
    int run_batch(Lane& lane, std::vector<Request*>& batch);
    long long live_room();
};

namespace {

// Device bytes one request holds while admitted: aligned copies of both
// planes, its share of the tile-state words and queue ring, its descriptor.
size_t request_bytes(int w, int h, int dtype, int tile_rows, size_t* pitch_out) {
    const size_t pitch = round_up((size_t)w * (size_t)bpp_of(dtype), 128);
    // a batch may pick either tile height when none is set: count the smaller
    const long long tiles = iwpp_tile_count(w, h, dtype, tile_rows ? tile_rows : 32);
    *pitch_out = pitch;
    return 2 * pitch * (size_t)h + (size_t)std::max(0ll, tiles) * 16u + 1024u;
}

}  // namespace

// Device bytes that admission may still hand out right now: the device's
// free memory plus what the pool holds without using it, less the bytes
// already admitted but not yet taken from the pool and the headroom left for
// other users of the device.  Called with `mu` held.
long long iwpp_server_s::live_room() {
    size_t free_b = 0, total_b = 0;
    if (cudaMemGetInfo(&free_b, &total_b) != cudaSuccess) {
        cudaGetLastError();
        return 0;
    }
    unsigned long long reserved = 0, used = 0;
    if (cudaMemPoolGetAttribute(pool, cudaMemPoolAttrReservedMemCurrent, &reserved) != cudaSuccess ||
        cudaMemPoolGetAttribute(pool, cudaMemPoolAttrUsedMemCurrent, &used) != cudaSuccess) {
        cudaGetLastError();
        reserved = used = 0;
    }
    const long long idle = reserved > used ? (long long)(reserved - used) : 0ll;
    return (long long)free_b + idle - unallocated - headroom;
}

int iwpp_server_s::run_batch(Lane& lane, std::vector<Request*>& batch) {
    cudaStream_t s = lane.stream;
    std::vector<iwpp_image> imgs;
    imgs.reserve(batch.size());
    cudaError_t e = cudaSuccess;
    long long taken = 0;
    for (Request* r : batch) {
        if (r->w == 0 || r->h == 0) continue;
        const size_t row = (size_t)r->w * bpp_of(r->dtype);
        const size_t plane = r->pitch * (size_t)r->h;
        if (e == cudaSuccess) e = cudaMallocFromPoolAsync(&r->d_marker, plane, pool, s);
        if (e == cudaSuccess) e = cudaMallocFromPoolAsync(&r->d_mask, plane, pool, s);
        if (e == cudaSuccess)
            e = cudaMemcpy2DAsync(r->d_marker, r->pitch, r->marker, r->pm, row, r->h, cudaMemcpyHostToDevice, s);
        if (e == cudaSuccess)
            e = cudaMemcpy2DAsync(r->d_mask, r->pitch, r->mask, r->pk, row, r->h, cudaMemcpyHostToDevice, s);
        imgs.push_back(iwpp_image{r->d_marker, r->d_mask, r->pitch, r->pitch, r->w, r->h, r->dtype, r->conn});
        taken += (long long)r->bytes;
    }
    if (headroom >= 0) {
        // the batch's planes are now the pool's (used) memory
        std::lock_guard<std::mutex> lk(mu);
        unallocated -= taken;
    }
    int rc = IWPP_OK;
    if (e != cudaSuccess) rc = e == cudaErrorMemoryAllocation ? IWPP_ERR_OOM : IWPP_ERR_CUDA;
    if (rc == IWPP_OK && !imgs.empty())
        rc = iwpp_reconstruct_batch_async(lane.handle, imgs.data(), (int)imgs.size(), variant, &cfg, s);
    for (Request* r : batch) {
        if (r->w == 0 || r->h == 0) continue;
        if (rc == IWPP_OK && r->d_marker) {
            const size_t row = (size_t)r->w * bpp_of(r->dtype);
            cudaError_t e2 =
                cudaMemcpy2DAsync(r->out, r->po, r->d_marker, r->pitch, row, r->h, cudaMemcpyDeviceToHost, s);
            if (e2 != cudaSuccess) rc = IWPP_ERR_CUDA;
        }
        if (r->d_marker) cudaFreeAsync(r->d_marker, s);
        if (r->d_mask) cudaFreeAsync(r->d_mask, s);
        r->d_marker = r->d_mask = nullptr;
    }
    if (!imgs.empty()) {
        // waits for the launch and the copies queued behind it
        const int rc_sync = iwpp_handle_sync(lane.handle, nullptr);
        if (rc == IWPP_OK) rc = rc_sync;
    }
    const cudaError_t e3 = cudaStreamSynchronize(s);
    if (rc == IWPP_OK && e3 != cudaSuccess) rc = IWPP_ERR_CUDA;
    return rc;
}

void iwpp_server_s::lane_main(int li) {
    cudaSetDevice(device);
    Lane& lane = lanes[(size_t)li];
    std::vector<Request*> batch;
    for (;;) {
        batch.clear();
        {
            std::unique_lock<std::mutex> lk(mu);
            // Admission: in arrival order while the budget holds and (live
            // check) the device's free memory right now covers the batch
            // plus the headroom.  Memory that another user of the device
            // takes or gives back is seen here; since nothing signals it,
            // a request held back by it is looked at again every millisecond.
            long long room = 0;
            for (;;) {
                cv_work.wait(lk, [&] {
                    if (pending.empty()) return stopping;
                    return in_use + (long long)pending.front()->bytes <= budget;
                });
                if (pending.empty()) return;  // stopping and drained
                // a server being destroyed finishes what is left regardless
                // (a request the device cannot hold ends in IWPP_ERR_OOM)
                if (headroom < 0 || stopping) break;
                room = live_room();
                if ((long long)pending.front()->bytes <= room) break;
                stats.held_back += 1;
                cv_work.wait_for(lk, std::chrono::milliseconds(1));
            }
            const Clock::time_point now = Clock::now();
            while (!pending.empty() && (int)batch.size() < max_batch &&
                   in_use + (long long)pending.front()->bytes <= budget &&
                   (headroom < 0 || stopping || (long long)pending.front()->bytes <= room)) {
                Request* r = pending.front();
                pending.pop_front();
                in_use += (long long)r->bytes;
                if (headroom >= 0) {
                    room -= (long long)r->bytes;
                    unallocated += (long long)r->bytes;
                }
                r->t_admit = now;
                r->lane = li;
                batch.push_back(r);
            }
            stats.bytes_in_use = in_use;
            stats.bytes_peak = std::max(stats.bytes_peak, in_use);
            stats.batches += 1;
            stats.largest_batch = std::max(stats.largest_batch, (long long)batch.size());
            // another lane may take the requests that did not fit this batch
            if (!pending.empty()) cv_work.notify_one();
        }
        const int rc = run_batch(lane, batch);
        const Clock::time_point now = Clock::now();
        {
            std::lock_guard<std::mutex> lk(mu);
            for (Request* r : batch) {
                r->status = rc;
                r->batch_size = (int)batch.size();
                r->t_done = now;
                r->done = true;
                in_use -= (long long)r->bytes;
                stats.completed += 1;
                if (rc != IWPP_OK) stats.failed += 1;
                else stats.pixels += (long long)r->w * r->h;
            }
            stats.bytes_in_use = in_use;
        }
        cv_done.notify_all();
        cv_work.notify_all();
    }
}

extern "C" {

int iwpp_server_create(iwpp_server* out, int device, const iwpp_server_config* cfg) {
    if (!out) return IWPP_ERR_INVALID;
    *out = nullptr;
    iwpp_server_config c{};
    if (cfg) c = *cfg;
    if (c.lanes < 0 || c.lanes > 64 || c.max_batch < 0 || c.max_pending < 0 || c.memory_budget < 0 ||
        c.lane_ctas < 0 || c.timeout_ms < 0 || (c.tile_rows != 0 && c.tile_rows != 32 && c.tile_rows != 64))
        return IWPP_ERR_INVALID;
    // A handle validates the device (sm_103) before anything is allocated.
    iwpp_handle probe = nullptr;
    int rc = iwpp_handle_create(&probe, device);
    if (rc != IWPP_OK) return rc;
    iwpp_server s = new (std::nothrow) iwpp_server_s();
    if (!s) {
        iwpp_handle_destroy(probe);
        return IWPP_ERR_OOM;
    }
    s->device = device;
    s->lanes_n = c.lanes ? c.lanes : 3;
    s->max_batch = c.max_batch ? c.max_batch : 256;
    s->max_pending = c.max_pending ? c.max_pending : 65536;
    s->variant = c.variant;
    s->tile_rows = c.tile_rows;
    s->cfg.tile_rows = c.tile_rows;
    s->cfg.init_passes = -1;
    s->cfg.grid_ctas = c.lane_ctas;
    s->cfg.timeout_ms = c.timeout_ms ? c.timeout_ms : 60000;
    // Batches of independent requests start the tile engine from a seed
    // check (the tiles holding a pixel a neighbour can raise; for sparse
    // markers most tiles hold none) but take no front stage: its scratch is
    // not in the lane workspaces sized below (a workspace that grows
    // mid-stream synchronises the device), and its decision would be one
    // for the whole mixed batch.
    s->cfg.front_passes = 4;

    int prev = 0;
    cudaGetDevice(&prev);
    cudaSetDevice(device);
    size_t free_b = 0, total_b = 0;
    cudaError_t e = cudaMemGetInfo(&free_b, &total_b);
    s->budget = c.memory_budget ? c.memory_budget : (long long)(free_b / 2);
    s->headroom = c.memory_headroom ? (c.memory_headroom < 0 ? -1ll : c.memory_headroom) : (256ll << 20);
    s->stats.memory_budget = s->budget;
    cudaMemPoolProps props;
    std::memset(&props, 0, sizeof(props));
    props.allocType = cudaMemAllocationTypePinned;
    props.location.type = cudaMemLocationTypeDevice;
    props.location.id = device;
    if (e == cudaSuccess) e = cudaMemPoolCreate(&s->pool, &props);
    if (e == cudaSuccess) {
        // keep what the pool allocated: requests reuse it without new allocations
        unsigned long long keep = ~0ull;
        e = cudaMemPoolSetAttribute(s->pool, cudaMemPoolAttrReleaseThreshold, &keep);
    }
    // Each lane's workspace is sized once for the most tiles the budget can
    // admit: with the tile height left to each batch, its smaller choice.
    const int th = c.tile_rows ? c.tile_rows : 32;
    const long long max_tiles = std::max(1ll, s->budget / (2ll * 128ll * th));
    const long long ws_bytes =
        iwpp_workspace_bytes(max_tiles, s->variant, 0) + 4ll * (max_tiles + 64) + (long long)s->max_batch * 512ll +
        4096ll;  // (the seed list: a word per tile and the count)
    s->lanes.resize((size_t)s->lanes_n);
    rc = e == cudaSuccess ? IWPP_OK : IWPP_ERR_CUDA;
    for (int i = 0; i < s->lanes_n && rc == IWPP_OK; ++i) {
        auto& L = s->lanes[(size_t)i];
        if (i == 0) {
            L.handle = probe;
            probe = nullptr;
        } else {
            rc = iwpp_handle_create(&L.handle, device);
        }
        if (rc == IWPP_OK && cudaStreamCreateWithFlags(&L.stream, cudaStreamNonBlocking) != cudaSuccess)
            rc = IWPP_ERR_CUDA;
        if (rc == IWPP_OK && ws_bytes > 0) rc = iwpp::handle_reserve(L.handle, (size_t)ws_bytes);
    }
    if (rc == IWPP_OK && !s->lanes.empty()) {
        // Map part of the budget into the pool now, so that admitting more
        // requests at once than ever before does not stall a lane on the
        // driver growing the pool in the middle of serving.
        const size_t warm = (size_t)std::min<long long>(s->budget, 4ll << 30);
        cudaStream_t ws = s->lanes[0].stream;
        void* p = nullptr;
        if (warm > 0 && cudaMallocFromPoolAsync(&p, warm, s->pool, ws) == cudaSuccess) {
            cudaFreeAsync(p, ws);
            cudaStreamSynchronize(ws);
        }
        cudaGetLastError();  // a pool that cannot be warmed still serves
    }
    cudaSetDevice(prev);
    if (probe) iwpp_handle_destroy(probe);
    if (rc != IWPP_OK) {
        for (auto& L : s->lanes) {
            if (L.stream) cudaStreamDestroy(L.stream);
            if (L.handle) iwpp_handle_destroy(L.handle);
        }
        if (s->pool) cudaMemPoolDestroy(s->pool);
        delete s;
        return rc;
    }
    for (int i = 0; i < s->lanes_n; ++i) s->lanes[(size_t)i].th = std::thread(&iwpp_server_s::lane_main, s, i);
    *out = s;
    return IWPP_OK;
}

int iwpp_server_submit(iwpp_server s, const void* marker, const void* mask, void* out, size_t pitch_marker,
                       size_t pitch_mask, size_t pitch_out, int width, int height, int dtype, int connectivity,
                       unsigned long long* ticket) {
    if (!s || !ticket) return IWPP_ERR_INVALID;
    *ticket = 0;
    if (dtype != IWPP_U8 && dtype != IWPP_U16 && dtype != IWPP_I32) return IWPP_ERR_INVALID;
    if (connectivity != 4 && connectivity != 8) return IWPP_ERR_INVALID;
    if (width < 0 || height < 0 || width > (1 << 28) || height > (1 << 28)) return IWPP_ERR_INVALID;
    const size_t row = (size_t)width * (size_t)bpp_of(dtype);
    if (width > 0 && height > 0) {
        if (!marker || !mask || !out) return IWPP_ERR_INVALID;
        if (pitch_marker < row || pitch_mask < row || pitch_out < row) return IWPP_ERR_INVALID;
    }
    Request* r = new (std::nothrow) Request();
    if (!r) return IWPP_ERR_OOM;
    r->marker = marker;
    r->mask = mask;
    r->out = out;
    r->pm = pitch_marker;
    r->pk = pitch_mask;
    r->po = pitch_out;
    r->w = width;
    r->h = height;
    r->dtype = dtype;
    r->conn = connectivity;
    r->bytes = width && height ? request_bytes(width, height, dtype, s->tile_rows, &r->pitch) : 0;
    r->t_submit = Clock::now();
    {
        std::lock_guard<std::mutex> lk(s->mu);
        if (s->stopping || (long long)s->pending.size() >= s->max_pending) {
            s->stats.rejected += 1;
            delete r;
            return IWPP_ERR_BUSY;
        }
        if ((long long)r->bytes > s->budget) {
            s->stats.rejected += 1;
            delete r;
            return IWPP_ERR_TOO_LARGE;
        }
        r->id = s->next_id++;
        s->live[r->id] = r;
        s->pending.push_back(r);
        s->stats.submitted += 1;
        *ticket = r->id;
    }
    s->cv_work.notify_one();
    return IWPP_OK;
}

int iwpp_server_wait(iwpp_server s, unsigned long long ticket, int timeout_ms, iwpp_request_result* result) {
    if (!s) return IWPP_ERR_INVALID;
    std::unique_lock<std::mutex> lk(s->mu);
    if (s->live.find(ticket) == s->live.end()) return IWPP_ERR_INVALID;
    // Looked up again on every wake-up: another thread waiting on the same
    // ticket may have taken the result (and freed the request) meanwhile.
    auto ready = [&] {
        auto f = s->live.find(ticket);
        return f == s->live.end() || f->second->done;
    };
    if (timeout_ms < 0) {
        s->cv_done.wait(lk, ready);
    } else if (!s->cv_done.wait_for(lk, std::chrono::milliseconds(timeout_ms), ready)) {
        return IWPP_ERR_BUSY;
    }
    auto it = s->live.find(ticket);
    if (it == s->live.end()) return IWPP_ERR_INVALID;  // taken by another waiter
    Request* r = it->second;
    if (result) {
        result->status = r->status;
        result->lane = r->lane;
        result->batch_size = r->batch_size;
        result->reserved = 0;
        result->latency_us = us_between(r->t_submit, r->t_done);
        result->queue_us = us_between(r->t_submit, r->t_admit);
        result->service_us = us_between(r->t_admit, r->t_done);
    }
    const int st = r->status;
    s->live.erase(it);
    delete r;
    return st;
}

int iwpp_server_stats_get(iwpp_server s, iwpp_server_stats* stats) {
    if (!s || !stats) return IWPP_ERR_INVALID;
    std::lock_guard<std::mutex> lk(s->mu);
    *stats = s->stats;
    return IWPP_OK;
}

int iwpp_server_destroy(iwpp_server s) {
    if (!s) return IWPP_OK;
    {
        std::lock_guard<std::mutex> lk(s->mu);
        s->stopping = true;
    }
    s->cv_work.notify_all();
    for (auto& L : s->lanes)
        if (L.th.joinable()) L.th.join();
    int prev = 0;
    cudaGetDevice(&prev);
    cudaSetDevice(s->device);
    for (auto& L : s->lanes) {
        if (L.stream) {
            cudaStreamSynchronize(L.stream);
            cudaStreamDestroy(L.stream);
        }
        if (L.handle) iwpp_handle_destroy(L.handle);
    }
    if (s->pool) cudaMemPoolDestroy(s->pool);
    cudaSetDevice(prev);
    for (auto& kv : s->live) delete kv.second;
    delete s;
    return IWPP_OK;
}

}  // extern "C"
