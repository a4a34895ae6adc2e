// refrun_harness.cpp -- runs the reference's own reconstruction kernels.
// TEST INFRASTRUCTURE ONLY (produces the outputs the oracle is pinned to).
//
// The kernels come unmodified from the reference sources
// (IWPP MP DQ/src/*.cu, IWPP MP UQ/src/*.cu), compiled for sm_103a into one
// device-linked cubin per variant by oracle/refrun.py.  This host program
// loads that cubin with the CUDA driver API and issues the reference's own
// host-side call sequence, restated from
//   DQ: IWPP MP DQ/src/MorphologicalReconstruction.cu:1183-1351
//   UQ: IWPP MP UQ/src/MorphologicalReconstruction.cu:1324-1508
// after the precondition clip the reference's main runs
// (IWPP MP DQ/src/main.cu:223, clipImage = elementwise min(marker, mask),
// MR.cu:1355-1364), applied here on the host before the upload because the
// device link of the relocatable objects does not keep that kernel.
// The device heap is raised as configureHeapSize does
// (IWPP MP DQ/src/globalQueue.cu:3-6) because the reference allocates its
// queues with in-kernel cudaMalloc.
//
// usage: refrun_harness <cubin> <dq|uq> <size> <marker.raw> <mask.raw> <out.raw>
// Images are size x size uint8, size a multiple of 512 (the reference's
// queue-fill launch needs it).  Exit status 0 on success.
#include <cuda.h>
#include <signal.h>
#include <unistd.h>

#include <chrono>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <vector>

#define CK(x)                                                                        \
    do {                                                                             \
        CUresult r_ = (x);                                                           \
        if (r_ != CUDA_SUCCESS) {                                                    \
            const char* s_ = nullptr;                                                \
            cuGetErrorString(r_, &s_);                                               \
            std::fprintf(stderr, "%s:%d %s -> %s\n", __FILE__, __LINE__, #x, s_);    \
            std::exit(2);                                                            \
        }                                                                            \
    } while (0)

static CUfunction find_kernel(CUmodule mod, const char* needle) {
    unsigned n = 0;
    CK(cuModuleGetFunctionCount(&n, mod));
    std::vector<CUfunction> fns(n);
    CK(cuModuleEnumerateFunctions(fns.data(), n, mod));
    for (CUfunction f : fns) {
        const char* name = nullptr;
        CK(cuFuncGetName(&name, f));
        // Itanium mangling: _Z<len><name>...
        std::string want = std::to_string(std::strlen(needle)) + needle;
        if (name && std::strncmp(name, "_Z", 2) == 0 && std::strstr(name, want.c_str()) == name + 2) return f;
    }
    std::fprintf(stderr, "kernel %s not found in the cubin\n", needle);
    std::exit(3);
}

static void launch(CUfunction f, unsigned gx, unsigned gy, unsigned bx, unsigned by, void** args) {
    CK(cuLaunchKernel(f, gx, gy, 1, bx, by, 1, 0, nullptr, args, nullptr));
}

static std::vector<unsigned char> read_raw(const char* path, size_t n) {
    std::vector<unsigned char> v(n);
    FILE* f = std::fopen(path, "rb");
    if (!f || std::fread(v.data(), 1, n, f) != n) {
        std::fprintf(stderr, "cannot read %s\n", path);
        std::exit(4);
    }
    std::fclose(f);
    return v;
}

int main(int argc, char** argv) {
    if (argc != 7) {
        std::fprintf(stderr, "usage: %s <cubin> <dq|uq> <size> <marker.raw> <mask.raw> <out.raw>\n", argv[0]);
        return 1;
    }
    alarm(300);  // watchdog: the process ends (and its context with it) if anything stalls
    const std::string variant = argv[2];
    const int size = std::atoi(argv[3]);
    if (size <= 0 || size % 512 != 0 || (variant != "dq" && variant != "uq")) {
        std::fprintf(stderr, "size must be a positive multiple of 512, variant dq or uq\n");
        return 1;
    }
    const int G = size / 32;  // megapixel grid side (MEGAPIXEL_SIZE 32)
    std::vector<unsigned char> marker = read_raw(argv[4], (size_t)size * size);
    std::vector<unsigned char> mask = read_raw(argv[5], (size_t)size * size);
    for (size_t i = 0; i < marker.size(); ++i)
        if (mask[i] < marker[i]) marker[i] = mask[i];  // clipImage

    CK(cuInit(0));
    CUdevice dev;
    CK(cuDeviceGet(&dev, 0));
    CUcontext ctx;
    CK(cuDevicePrimaryCtxRetain(&ctx, dev));
    CK(cuCtxSetCurrent(ctx));
    CK(cuCtxSetLimit(CU_LIMIT_MALLOC_HEAP_SIZE, 1073741824ull));  // DEVICE_MALLOC_LIMIT
    CUmodule mod;
    CK(cuModuleLoad(&mod, argv[1]));
    CUfunction k_alloc = find_kernel(mod, "allocGlobalQueue");
    CUfunction k_free = find_kernel(mod, "freeGlobalQueue");
    CUfunction k_fill = find_kernel(mod, "initFillGlobalQueue");
    CUfunction k_recon = find_kernel(mod, "MorphologicalReconstructionKernel");
    CUfunction k_swap = variant == "dq" ? find_kernel(mod, "swapQueues") : nullptr;
    CUfunction k_reset = variant == "uq" ? find_kernel(mod, "resetReadQueue") : nullptr;
    CUfunction k_extract = variant == "uq" ? find_kernel(mod, "extractUniques") : nullptr;
    CUfunction k_clear = variant == "uq" ? find_kernel(mod, "clearHashAndResetWriteQueue") : nullptr;

    // pitched images, as the reference's main does (cudaMallocPitch + cudaMemcpy2D)
    CUdeviceptr d_marker, d_mask;
    size_t pitchMarker = 0, pitchMask = 0;
    CK(cuMemAllocPitch(&d_marker, &pitchMarker, size, size, 16));
    CK(cuMemAllocPitch(&d_mask, &pitchMask, size, size, 16));
    CUDA_MEMCPY2D cp;
    std::memset(&cp, 0, sizeof(cp));
    cp.srcMemoryType = CU_MEMORYTYPE_HOST;
    cp.dstMemoryType = CU_MEMORYTYPE_DEVICE;
    cp.WidthInBytes = size;
    cp.Height = size;
    cp.srcHost = marker.data();
    cp.srcPitch = size;
    cp.dstDevice = d_marker;
    cp.dstPitch = pitchMarker;
    CK(cuMemcpy2D(&cp));
    cp.srcHost = mask.data();
    cp.dstDevice = d_mask;
    cp.dstPitch = pitchMask;
    CK(cuMemcpy2D(&cp));

    // struct GlobalQueue { ushort2* readQueue; ushort2* writeQueue; int readQueueSize; int writeQueueSize; }
    CUdeviceptr gq, d_memleak;
    CK(cuMemAlloc(&gq, 24));
    CK(cuMemAlloc(&d_memleak, sizeof(int)));
    CUdeviceptr flags = 0;
    size_t flags_pitch = 0;
    if (variant == "uq") {
        CK(cuMemAllocPitch(&flags, &flags_pitch, (size_t)G * sizeof(int), G, 16));
        CK(cuMemsetD2D8(flags, flags_pitch, 0, (size_t)G * sizeof(int), G));
    }
    // timed like the reference's main times its call (main.cu:225-232):
    // from the queue allocation to after the queue is freed
    CK(cuCtxSynchronize());
    const auto t_start = std::chrono::steady_clock::now();
    {
        void* args[] = {&gq};
        launch(k_alloc, 1, 1, 1, 1, args);
        CK(cuCtxSynchronize());
        unsigned long long ptrs[2] = {0, 0};
        CK(cuMemcpyDtoH(ptrs, gq, sizeof(ptrs)));
        if (ptrs[0] == 0 || ptrs[1] == 0) {  // in-kernel cudaMalloc failed: do not launch on it
            std::fprintf(stderr, "device-side queue allocation failed\n");
            return 5;
        }
    }
    int size_arg = size;
    int hMemLeak = 0, restarts = 0;
    long long rounds = 0;
    do {
        CK(cuMemsetD32(d_memleak, 0, 1));
        {
            void* args[] = {&gq};
            launch(k_fill, G / 16, G / 16, 16, 16, args);
        }
        int readQueueSize = G * G;
        while (readQueueSize > 0) {
            const unsigned grid = readQueueSize < 2048 ? (unsigned)readQueueSize : 2048u;
            void* rargs[] = {&gq, &d_marker, &d_mask, &pitchMarker, &pitchMask, &size_arg, &d_memleak};
            launch(k_recon, grid, 1, 32, 1, rargs);
            void* gargs[] = {&gq};
            if (variant == "dq") {
                launch(k_swap, 1, 1, 1, 1, gargs);
            } else {
                void* fargs[] = {&gq, &flags, &flags_pitch};
                launch(k_reset, 1, 1, 1, 1, gargs);
                launch(k_extract, 2048, 1, 32, 1, fargs);
                launch(k_clear, 2048, 1, 32, 1, fargs);
            }
            CK(cuMemcpyDtoH(&readQueueSize, gq + 16, sizeof(int)));
            ++rounds;
        }
        CK(cuMemcpyDtoH(&hMemLeak, d_memleak, sizeof(int)));
        restarts += hMemLeak ? 1 : 0;
    } while (hMemLeak);
    {
        void* args[] = {&gq};
        launch(k_free, 1, 1, 1, 1, args);
        CK(cuCtxSynchronize());
    }
    const double ms = std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t_start).count();

    std::vector<unsigned char> out((size_t)size * size);
    CUDA_MEMCPY2D back;
    std::memset(&back, 0, sizeof(back));
    back.srcMemoryType = CU_MEMORYTYPE_DEVICE;
    back.dstMemoryType = CU_MEMORYTYPE_HOST;
    back.srcDevice = d_marker;
    back.srcPitch = pitchMarker;
    back.dstHost = out.data();
    back.dstPitch = size;
    back.WidthInBytes = size;
    back.Height = size;
    CK(cuMemcpy2D(&back));
    FILE* f = std::fopen(argv[6], "wb");
    if (!f || std::fwrite(out.data(), 1, out.size(), f) != out.size()) {
        std::fprintf(stderr, "cannot write %s\n", argv[6]);
        return 4;
    }
    std::fclose(f);
    std::printf("{\"variant\": \"%s\", \"size\": %d, \"rounds\": %lld, \"restarts\": %d, \"ms\": %.3f}\n",
                variant.c_str(), size, rounds, restarts, ms);
    cuMemFree(d_marker);
    cuMemFree(d_mask);
    cuMemFree(gq);
    cuMemFree(d_memleak);
    if (flags) cuMemFree(flags);
    cuModuleUnload(mod);
    cuDevicePrimaryCtxRelease(dev);
    return 0;
}
