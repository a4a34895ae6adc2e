// iwpp_noalloc.cu -- reconstruction without any device allocation.
//
// Who needs this: callers that cannot call cudaMalloc at the point where
// they reconstruct.  Two common cases: a host framework whose caching
// allocator owns the whole device-memory budget and does not allow other
// code to allocate behind its back, and latency-critical loops where the
// implicit device-wide synchronisation of cudaMalloc / cudaFree would stall
// every other stream.  Such callers own their marker and mask buffers; this
// entry point brings nothing else but a fixed scratch array that is part of
// the loaded library (below), so the reconstruction itself allocates
// nothing.
//
// The scratch array is a file-scope __device__ array: every GPU on which the
// library is loaded holds IWPP_NOALLOC_SCRATCH_BYTES of it until the process
// exits.  In host code the array's name is only a host-side stand-in, not a
// device address, so the device address is obtained once per device with
// cudaGetSymbolAddress (with that device current) and passed to the kernels.
// That address is kept for the life of the process: a cudaDeviceReset
// between calls (which reloads the module) is not supported.
#include <cstdio>
#include <cstring>
#include <mutex>

#include "iwpp.h"
#include "iwpp_engine.cuh"

namespace iwpp {
namespace {

static __device__ __align__(256) unsigned char g_noalloc_scratch[IWPP_NOALLOC_SCRATCH_BYTES];

// The counters and the one image descriptor each take one 256-byte slot at
// the start of the scratch (the size bound below counts on it).
static_assert(sizeof(Ctrl) <= 256 && sizeof(ImgDesc) <= 256, "scratch header slots");

constexpr int kMaxDevices = 64;
constexpr int kNoallocTileRows = 64;

std::mutex g_setup_mu;
unsigned char* g_scratch_ptr[kMaxDevices] = {};
LaunchInfo g_launch[kMaxDevices] = {};

// Per-device set-up, done by the first call on a device with that device
// current: the device address of the scratch array and the engine's launch
// shape (kernel attributes, occupancy, SM count), both kept for the life of
// the process so that later calls do no host-side queries.  A
// cudaDeviceReset between calls would leave both stale; it is not supported.
int device_setup(int device, unsigned char** out, LaunchInfo* li) {
    std::lock_guard<std::mutex> lk(g_setup_mu);
    if (!g_scratch_ptr[device]) {
        void* p = nullptr;
        cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
        if (e != cudaSuccess || p == nullptr) {
            cudaGetLastError();
            return IWPP_ERR_CUDA;
        }
        LaunchInfo l{};
        e = engine_prepare(VAR_ASYNC, kNoallocTileRows, device, &l);
        if (e != cudaSuccess) {
            cudaGetLastError();
            return IWPP_ERR_CUDA;
        }
        g_launch[device] = l;
        g_scratch_ptr[device] = static_cast<unsigned char*>(p);
    }
    *out = g_scratch_ptr[device];
    *li = g_launch[device];
    return IWPP_OK;
}

// Writes the single image descriptor into the scratch (a kernel parameter,
// so no host-to-device copy is needed).
__global__ void noalloc_store_desc(ImgDesc* dst, ImgDesc d) { *dst = d; }

size_t align_up(size_t v, size_t a) { return (v + a - 1) / a * a; }

}  // namespace
}  // namespace iwpp

using namespace iwpp;

extern "C" int iwpp_reconstruct_noalloc(void* marker, const void* mask, size_t pitch_marker, size_t pitch_mask,
                                        int width, int height, int dtype, int connectivity, void* stream) {
    if (dtype != IWPP_U8 && dtype != IWPP_U16 && dtype != IWPP_I32) return IWPP_ERR_INVALID;
    if (connectivity != 4 && connectivity != 8) return IWPP_ERR_INVALID;
    if (width < 0 || height < 0 || width > (1 << 28) || height > (1 << 28)) return IWPP_ERR_INVALID;
    if (width == 0 || height == 0) return IWPP_OK;
    if (!marker || !mask) return IWPP_ERR_INVALID;
    const int bpp = dtype == IWPP_U8 ? 1 : dtype == IWPP_U16 ? 2 : 4;
    const size_t row = (size_t)width * (size_t)bpp;
    if (pitch_marker < row || pitch_mask < row) return IWPP_ERR_INVALID;
    // rows must start on 4-byte boundaries: unaligned images would need a
    // staging copy, which needs memory
    if ((reinterpret_cast<uintptr_t>(marker) & 3u) || (reinterpret_cast<uintptr_t>(mask) & 3u) ||
        (pitch_marker & 3u) || (pitch_mask & 3u))
        return IWPP_ERR_INVALID;

    const int ppw = 4 / bpp;
    const long long tiles_x = (width + 32ll * ppw - 1) / (32ll * ppw);
    const long long tiles_y = ((long long)height + kNoallocTileRows - 1) / kNoallocTileRows;
    const long long G = tiles_x * tiles_y;
    const long long cap = G * 2 > 1024 ? G * 2 : 1024;  // async ring
    const size_t off_img = align_up(sizeof(Ctrl), 256);
    const size_t off_state = align_up(off_img + sizeof(ImgDesc), 256);
    const size_t off_ring = align_up(off_state + (size_t)G * 4u, 256);
    const size_t need = off_ring + (size_t)cap * 4u;
    if (G > 0x7fffffffll || need > (size_t)IWPP_NOALLOC_SCRATCH_BYTES) return IWPP_ERR_TOO_LARGE;

    int device = 0;
    if (cudaGetDevice(&device) != cudaSuccess || device < 0 || device >= kMaxDevices) {
        cudaGetLastError();
        return IWPP_ERR_NO_DEVICE;
    }
    unsigned char* base = nullptr;
    LaunchInfo li;
    int rc = device_setup(device, &base, &li);
    if (rc != IWPP_OK) return rc;

    ImgDesc d{};
    d.marker = static_cast<unsigned char*>(marker);
    d.mask = static_cast<const unsigned char*>(mask);
    d.pitch_m = (long long)pitch_marker;
    d.pitch_k = (long long)pitch_mask;
    d.tmaps = nullptr;  // plain loads: tensor maps would have to be copied in
    d.W = width;
    d.H = height;
    d.dtype = dtype;
    d.conn = connectivity;
    d.tiles_x = (int)tiles_x;
    d.tiles_y = (int)tiles_y;
    d.tile_base = 0;
    d.tile_rows = kNoallocTileRows;

    EngineArgs a{};
    a.imgs = reinterpret_cast<const ImgDesc*>(base + off_img);
    a.nimg = 1;
    a.G = (unsigned)G;
    a.state = reinterpret_cast<unsigned*>(base + off_state);
    a.q0 = reinterpret_cast<unsigned*>(base + off_ring);
    a.q1 = a.q0;
    a.cap = (unsigned)cap;
    a.ctrl = reinterpret_cast<Ctrl*>(base);
    a.timeout_ns = 10000ll * 1000000ll;
    a.max_restarts = 64;
    a.solver = 0;

    cudaStream_t s = static_cast<cudaStream_t>(stream);
    noalloc_store_desc<<<1, 1, 0, s>>>(reinterpret_cast<ImgDesc*>(base + off_img), d);
    cudaError_t e = cudaGetLastError();
    // the init kernel clears the state words, the ring and the counters that
    // the previous call left in the scratch
    if (e == cudaSuccess) e = engine_launch_init(a, VAR_ASYNC, s);
    if (e == cudaSuccess) {
        long long grid = li.grid;
        const long long useful = (G + kWarps - 1) / kWarps;
        if (grid > useful) grid = useful;
        if (grid < 1) grid = 1;
        e = engine_launch(a, VAR_ASYNC, kNoallocTileRows, (int)grid, s);
    }
    Ctrl c;
    if (e == cudaSuccess) e = cudaMemcpyAsync(&c, base, sizeof(Ctrl), cudaMemcpyDeviceToHost, s);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    if (e != cudaSuccess) {
        cudaGetLastError();
        return e == cudaErrorMemoryAllocation ? IWPP_ERR_OOM : IWPP_ERR_CUDA;
    }
    if (c.error == DEV_ERR_TIMEOUT) return IWPP_ERR_TIMEOUT;
    if (c.error == DEV_ERR_OVERFLOW) return IWPP_ERR_OVERFLOW;
    return IWPP_OK;
}
