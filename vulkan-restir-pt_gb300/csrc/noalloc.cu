/*
 * noalloc.cu — grisPassRenderNoAlloc: the GRIS pass without any device allocation.
 *
 * No counterpart in the reference. Some callers cannot call cudaMalloc while they render (a host
 * callback or plugin that must not allocate, a process whose device allocator belongs to another
 * framework). For them the pass's scratch — the temporary reservoirs that the temporal kernel
 * writes and the spatial kernel reads, and the ray-counter words every kernel adds to — lives in
 * the static device array below instead of caller- or library-allocated buffers. The kernels and
 * their launches are the ones grisPassRender uses; only where the scratch lives differs.
 */
#include <cuda_runtime.h>

#include <mutex>

#include "../../include/grisrt.h"
#include "gris_kernels.h"
#include "grisrt_internal.h"

namespace {

constexpr size_t kTempBytes = (size_t)GRIS_NOALLOC_MAX_PIXELS * sizeof(GrisReservoir);
constexpr size_t kCounterBytes = 256;   /* 32 counter words */

/* The scratch: temporary reservoirs, then the counter words. Held by every GPU that loads the
 * library until the process exits. */
static __device__ __align__(256) unsigned char g_noallocScratch[kTempBytes + kCounterBytes];

constexpr int kMaxDevices = 64;
std::mutex g_setupLock;
void* g_scratchAddr[kMaxDevices] = {nullptr};

/* Once per device, with that device current: the device address of the array (its name in host
 * code is only a host-side stand-in). */
cudaError_t scratch_address(int device, void** out) {
    std::lock_guard<std::mutex> lock(g_setupLock);
    if (!g_scratchAddr[device]) {
        void* p = nullptr;
        cudaError_t e = cudaGetSymbolAddress(&p, g_noallocScratch);
        if (e != cudaSuccess) return e;
        g_scratchAddr[device] = p;
    }
    *out = g_scratchAddr[device];
    return cudaSuccess;
}

}  // namespace

namespace {

/* Makes `device` current for the lifetime of the guard and gives the caller's current device back
 * on every return path: the callers of these entry points run inside other frameworks' threads. */
struct DeviceGuard {
    int saved = -1;
    bool ok = false;
    explicit DeviceGuard(int device) {
        if (cudaGetDevice(&saved) != cudaSuccess) saved = -1;
        ok = cudaSetDevice(device) == cudaSuccess;
    }
    ~DeviceGuard() {
        if (saved >= 0) cudaSetDevice(saved);
    }
};

constexpr uint64_t kErrorWord = GRIS_COUNTER_ERROR;   /* the counter word the kernels OR errors into */

}  // namespace

extern "C" int grisPassRenderNoAlloc(const GrisScene* scene, const GrisPassBindings* b, const GrisCamera* cam,
                                     const GrisCamera* prevCam, const GrisSettings* settings, void* stream) {
    if (!scene || !b || !cam || !prevCam || !settings) return GRIS_ERR_INVALID_ARGUMENT;
    if (b->width == 0 || b->height == 0 || !b->depthNormal || !b->depthNormalPrev || !b->albedoMatId ||
        !b->albedoMatIdPrev || !b->motion || !b->reservoirThis || !b->reservoirPrev || !b->output ||
        b->reservoirTemp != nullptr)
        return GRIS_ERR_INVALID_ARGUMENT;
    if (cam->filmSize[0] != b->width || cam->filmSize[1] != b->height) return GRIS_ERR_INVALID_ARGUMENT;
    if (settings->maxDepth == 0 || settings->maxDepth > 255 || settings->spatialNeighbors > 64 ||
        settings->envRadiance[0] != 0.0f || settings->envRadiance[1] != 0.0f || settings->envRadiance[2] != 0.0f)
        return GRIS_ERR_INVALID_ARGUMENT;
    uint64_t pixels = (uint64_t)b->width * (uint64_t)b->height;
    if (pixels > (uint64_t)GRIS_NOALLOC_MAX_PIXELS) return GRIS_ERR_TOO_LARGE;
    grisrt::DeviceSceneView view;
    int device = 0;
    if (!grisrt::scene_device(scene, &view, &device) || device < 0 || device >= kMaxDevices)
        return GRIS_ERR_INVALID_ARGUMENT;
    DeviceGuard guard(device);
    if (!guard.ok) return GRIS_ERR_CUDA;
    void* base = nullptr;
    if (scratch_address(device, &base) != cudaSuccess) return GRIS_ERR_CUDA;
    cudaStream_t s = (cudaStream_t)stream;
    unsigned char* temp = (unsigned char*)base;
    unsigned long long* counters = (unsigned long long*)(temp + kTempBytes);
    /* what must start at zero: the reservoirs of this frame's size and the ray-counter words; the
     * error word (counter 3) is left alone, so that errors of earlier calls stay readable until
     * grisNoAllocReadError takes them */
    if (cudaMemsetAsync(temp, 0, pixels * sizeof(GrisReservoir), s) != cudaSuccess) return GRIS_ERR_CUDA;
    if (cudaMemsetAsync(counters, 0, kErrorWord * sizeof(unsigned long long), s) != cudaSuccess) return GRIS_ERR_CUDA;
    if (cudaMemsetAsync(counters + kErrorWord + 1, 0, kCounterBytes - (kErrorWord + 1) * sizeof(unsigned long long), s) !=
        cudaSuccess)
        return GRIS_ERR_CUDA;
    GrisPassBindings pb = *b;
    pb.reservoirTemp = (GrisReservoir*)temp;
    cudaError_t e = grisrt::launch_gris(view, pb, *cam, *prevCam, *settings, 7, counters, 0, nullptr, s);
    return e == cudaSuccess ? GRIS_OK : GRIS_ERR_CUDA;
}

extern "C" int grisNoAllocReadError(int device, void* stream, uint64_t* errorWord) {
    if (!errorWord || device < 0 || device >= kMaxDevices) return GRIS_ERR_INVALID_ARGUMENT;
    *errorWord = 0;
    DeviceGuard guard(device);
    if (!guard.ok) return GRIS_ERR_CUDA;
    void* base = nullptr;
    if (scratch_address(device, &base) != cudaSuccess) return GRIS_ERR_CUDA;
    cudaStream_t s = (cudaStream_t)stream;
    unsigned long long* word = (unsigned long long*)((unsigned char*)base + kTempBytes) + kErrorWord;
    unsigned long long v = 0;
    /* after the caller's work on `stream`: read the word into this host variable, then clear it */
    if (cudaMemcpyAsync(&v, word, sizeof(v), cudaMemcpyDeviceToHost, s) != cudaSuccess) return GRIS_ERR_CUDA;
    if (cudaMemsetAsync(word, 0, sizeof(v), s) != cudaSuccess) return GRIS_ERR_CUDA;
    if (cudaStreamSynchronize(s) != cudaSuccess) return GRIS_ERR_CUDA;
    *errorWord = (uint64_t)v;
    return v ? GRIS_ERR_DEVICE_FAULT : GRIS_OK;
}
