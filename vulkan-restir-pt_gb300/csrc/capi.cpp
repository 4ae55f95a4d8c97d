/*
 * capi.cpp — the grisrt C ABI (include/grisrt.h): contexts, scene upload + BVH build,
 * caller-bound passes, library-owned frames with the renderer's ping-pong.
 *
 * Reference roles: GRISReSTIR::createPipeline / render (src/GRISReSTIR.cpp:9-67),
 * DeviceScene (src/Scene.cpp:324-446), Renderer's per-frame resources and ping-pong
 * (src/Renderer.cpp:193-257, 329-347, 539-569).
 */
#include <cuda_runtime.h>
#include <string.h>

#include <algorithm>
#include <mutex>
#include <string>
#include <vector>

#include "../../include/grisrt.h"
#include "bvh_traverse.h"
#include "gris_kernels.h"
#include "grisrt_internal.h"

static_assert(sizeof(GrisMaterial) == 32, "Material is 32 B (layouts.glsl:6-25)");
static_assert(sizeof(GrisMeshVertex) == 32, "MeshVertex is 32 B");
static_assert(sizeof(GrisObjectInstance) == 224, "ObjectInstance is 224 B");
static_assert(sizeof(GrisTriangleLight) == 64, "TriangleLight is 64 B");
static_assert(sizeof(GrisLightTableEntry) == 8, "LightSampleTableElement is 8 B");
static_assert(sizeof(GrisCamera) == 352, "Camera is 352 B");
static_assert(sizeof(GrisReservoir) == 96, "GRISReservoir is 96 B");
static_assert(sizeof(GrisSettings) == 64, "GrisSettings is 64 B");
static_assert(sizeof(GrisDIReservoir) == 64, "DIReservoir is 64 B");
static_assert(sizeof(GrisDISettings) == 16, "TestReSTIR::Settings is 16 B");
static_assert(sizeof(GrisPostSettings) == 16, "PostProcessFrag::PushConstant is 16 B");

/* Per-kernel CUDA-event timing of every launch while enabled (events recorded on the
 * launch stream around each kernel; read back and summed on request). */
struct Profiler : grisrt::KernelTimer {
    static const int kSlots = GRIS_PROFILE_SLOTS;
    bool enabled = false;
    struct Pair { cudaEvent_t a, b; int kernel; };
    std::vector<Pair> pending, free;
    double ms[kSlots] = {};
    uint64_t launches[kSlots] = {};
    Pair open[kSlots] = {};   /* slots nest (the wavefront stages inside the path-trace span) */
    void mark(int kernel, bool begin, cudaStream_t stream) override {
        if (!enabled || kernel < 0 || kernel >= kSlots) return;
        if (begin) {
            if (free.empty()) {
                Pair p{};
                cudaEventCreate(&p.a);
                cudaEventCreate(&p.b);
                free.push_back(p);
            }
            open[kernel] = free.back();
            free.pop_back();
            open[kernel].kernel = kernel;
            cudaEventRecord(open[kernel].a, stream);
        } else {
            cudaEventRecord(open[kernel].b, stream);
            pending.push_back(open[kernel]);
        }
    }
    void collect() {
        for (Pair& p : pending) {
            float t = 0.0f;
            cudaEventSynchronize(p.b);
            cudaEventElapsedTime(&t, p.a, p.b);
            ms[p.kernel] += t;
            launches[p.kernel]++;
            free.push_back(p);
        }
        pending.clear();
    }
    void reset() {
        for (int k = 0; k < kSlots; k++) { ms[k] = 0.0; launches[k] = 0; }
    }
    ~Profiler() override {
        for (Pair& p : pending) { cudaEventDestroy(p.a); cudaEventDestroy(p.b); }
        for (Pair& p : free) { cudaEventDestroy(p.a); cudaEventDestroy(p.b); }
    }
};

#define GRIS_NUM_COUNTERS 48

/* Scratch of the wavefront path tracer for the single-view entry points, grown on demand. */
struct WaveScratch {
    grisrt::WaveBuffers wb{};
    std::vector<void*> allocations;
    void* dViews = nullptr;
    void* hViews[2] = {nullptr, nullptr};
    cudaEvent_t staged[2] = {nullptr, nullptr};
    int stage = 0;
    void release() {
        for (void* p : allocations) cudaFree(p);
        allocations.clear();
        if (wb.reuse.block) cudaFree(wb.reuse.block);
        grisrt::wave_streams_destroy(wb);
        for (int i = 0; i < 2; i++) {
            if (hViews[i]) cudaFreeHost(hViews[i]);
            if (staged[i]) cudaEventDestroy(staged[i]);
            hViews[i] = nullptr; staged[i] = nullptr;
        }
        dViews = nullptr;
        wb = grisrt::WaveBuffers{};
    }
};

struct GrisContext {
    int device = 0;
    WaveScratch wave;
    cudaStream_t stream = nullptr;
    unsigned long long* dCounters = nullptr;
    unsigned long long* hCounters = nullptr;   /* pinned */
    int countWork = 0;
    int launchMode = GRIS_LAUNCH_GRID;
    int pathForm = GRIS_PATH_WAVEFRONT;
    int useGraphs = 1;
    grisrt::WaveLaunch waveLaunch;
    double* dReduce = nullptr;      /* relMSE partial sums (allocated on first use) */
    void* diSplit = nullptr;        /* the DI spatial pass's three-launch scratch (grown on demand) */
    uint64_t diSplitPixels = 0;
    grisrt::DISide diSide{nullptr, nullptr, nullptr};   /* the DI candidates pass's side stream */
    Profiler prof;
    /* pipelined downloads: a staging area, the copy stream and its two events (created on first use) */
    cudaStream_t copyStream = nullptr;
    cudaEvent_t evStaged = nullptr, evCopied = nullptr;
    char* staging = nullptr;
    size_t stagingBytes = 0, stagingUsed = 0;
    std::string err;
};

struct GrisScene {
    GrisContext* ctx = nullptr;
    std::vector<void*> allocations;
    grisrt::DeviceSceneView view{};
    grisrt::BvhHost bvh;
    GrisSceneStats stats{};
};

struct GrisFrame {
    GrisContext* ctx = nullptr;
    uint32_t w = 0, h = 0;
    float* depthNormal[2] = {nullptr, nullptr};
    uint32_t* albedoMatId[2] = {nullptr, nullptr};
    uint16_t* motion = nullptr;
    GrisReservoir* resv[2] = {nullptr, nullptr};
    GrisReservoir* temp = nullptr;
    float* output = nullptr;
    /* ReSTIR DI buffers (grisFrameRenderDI allocates them on first use) */
    GrisDIReservoir* diResv[2] = {nullptr, nullptr};
    GrisDIReservoir* diTemp = nullptr;
    float* directOutput = nullptr;
    int next = 0;   /* slot the next render writes */
};

namespace {

int fail(GrisContext* ctx, int code, const std::string& msg) {
    if (ctx) ctx->err = msg;
    return code;
}
int cuda_fail(GrisContext* ctx, cudaError_t e, const char* what) {
    return fail(ctx, e == cudaErrorMemoryAllocation ? GRIS_ERR_OUT_OF_MEMORY : GRIS_ERR_CUDA,
                std::string(what) + ": " + cudaGetErrorString(e));
}
#define GRIS_CK(ctx, call)                                   \
    do {                                                     \
        cudaError_t e_ = (call);                             \
        if (e_ != cudaSuccess) return cuda_fail(ctx, e_, #call); \
    } while (0)

template <typename T>
int upload(GrisContext* ctx, GrisScene* s, const T* src, uint64_t n, const T** dst) {
    size_t bytes = (size_t)n * sizeof(T);
    void* p = nullptr;
    GRIS_CK(ctx, cudaMalloc(&p, bytes < 256 ? 256 : bytes));
    s->allocations.push_back(p);
    if (bytes) GRIS_CK(ctx, cudaMemcpyAsync(p, src, bytes, cudaMemcpyHostToDevice, ctx->stream));
    *dst = (const T*)p;
    return GRIS_OK;
}

grisrt::DeviceSceneView scene_view(const GrisScene* s) { return s->view; }

}  // namespace

int grisrt::ctx_device(GrisContext* ctx) { return ctx->device; }

namespace {
constexpr int kCacheDevices = 64;
std::mutex g_deviceCacheLock;
int g_deviceCache[kCacheDevices][grisrt::kDeviceKeys];
bool g_deviceCached[kCacheDevices][grisrt::kDeviceKeys];
}  // namespace

int grisrt::once_per_device(int key, int (*f)()) {
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= kCacheDevices || key < 0 || key >= kDeviceKeys)
        return f();
    std::lock_guard<std::mutex> lock(g_deviceCacheLock);
    if (g_deviceCached[dev][key]) return g_deviceCache[dev][key];
    int v = f();
    if (v >= 0) { g_deviceCache[dev][key] = v; g_deviceCached[dev][key] = true; }
    return v;
}

int grisrt::current_sm_count() {
    int v = once_per_device(kDeviceKeySMs, []() {
        int dev = 0, sm = 0;
        if (cudaGetDevice(&dev) != cudaSuccess || cudaDeviceGetAttribute(&sm, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess)
            return -1;
        return sm;
    });
    return v > 0 ? v : 1;
}
cudaStream_t grisrt::ctx_stream(GrisContext* ctx) { return ctx->stream; }
unsigned long long* grisrt::ctx_counters(GrisContext* ctx) { return ctx->dCounters; }
int grisrt::ctx_count_work(GrisContext* ctx) { return ctx->countWork; }
int grisrt::ctx_path_form(GrisContext* ctx) { return ctx->pathForm; }
grisrt::KernelTimer* grisrt::ctx_timer(GrisContext* ctx) { return &ctx->prof; }
int grisrt::ctx_fail(GrisContext* ctx, int code, const std::string& msg) { return fail(ctx, code, msg); }
bool grisrt::ctx_graphs(GrisContext* ctx) { return ctx->useGraphs && !ctx->prof.enabled; }
bool grisrt::ctx_profiling(GrisContext* ctx) { return ctx->prof.enabled; }

int grisrt::ctx_download_async(GrisContext* ctx, const void* dev, void* host, size_t bytes, const char* what) {
    cudaSetDevice(ctx->device);
    cudaStreamCaptureStatus cap = cudaStreamCaptureStatusNone;
    GRIS_CK(ctx, cudaStreamIsCapturing(ctx->stream, &cap));
    if (cap != cudaStreamCaptureStatusNone) return fail(ctx, GRIS_ERR_INVALID_ARGUMENT, std::string(what) + ": stream is capturing");
    if (!ctx->copyStream) {
        GRIS_CK(ctx, cudaStreamCreateWithFlags(&ctx->copyStream, cudaStreamNonBlocking));
        GRIS_CK(ctx, cudaEventCreateWithFlags(&ctx->evStaged, cudaEventDisableTiming));
        GRIS_CK(ctx, cudaEventCreateWithFlags(&ctx->evCopied, cudaEventDisableTiming));
    }
    const size_t need = (bytes + 255) & ~(size_t)255;
    if (ctx->stagingUsed + need > ctx->stagingBytes) {
        /* every staged region is free once the copies to host are done (each waited for its
         * device-to-device copy); then the area is reused from its start, or replaced */
        GRIS_CK(ctx, cudaEventSynchronize(ctx->evCopied));
        ctx->stagingUsed = 0;
        if (need > ctx->stagingBytes) {
            if (ctx->staging) GRIS_CK(ctx, cudaFree(ctx->staging));
            ctx->staging = nullptr;
            ctx->stagingBytes = 0;
            const size_t sz = std::max(need, (size_t)2 << 20);
            GRIS_CK(ctx, cudaMalloc(&ctx->staging, sz));
            ctx->stagingBytes = sz;
        }
    }
    char* st = ctx->staging + ctx->stagingUsed;
    ctx->stagingUsed += need;
    GRIS_CK(ctx, cudaMemcpyAsync(st, dev, bytes, cudaMemcpyDeviceToDevice, ctx->stream));
    GRIS_CK(ctx, cudaEventRecord(ctx->evStaged, ctx->stream));
    GRIS_CK(ctx, cudaStreamWaitEvent(ctx->copyStream, ctx->evStaged, 0));
    GRIS_CK(ctx, cudaMemcpyAsync(host, st, bytes, cudaMemcpyDeviceToHost, ctx->copyStream));
    GRIS_CK(ctx, cudaEventRecord(ctx->evCopied, ctx->copyStream));
    return GRIS_OK;
}
grisrt::WaveLaunch grisrt::ctx_wave_launch(GrisContext* ctx) { return ctx->waveLaunch; }
void grisrt::ctx_set_tuning(GrisContext* ctx, int pathForm, grisrt::WaveLaunch wl) { ctx->pathForm = pathForm; ctx->waveLaunch = wl; }

bool grisrt::scene_device(const GrisScene* s, grisrt::DeviceSceneView* view, int* device) {
    if (!s || !s->ctx) return false;
    *view = s->view;
    *device = s->ctx->device;
    return true;
}

extern "C" {

int grisGetVersion(void) { return 1; }

size_t grisSizeof(int which) {
    switch (which) {
    case 0: return sizeof(GrisCamera);
    case 1: return sizeof(GrisReservoir);
    case 2: return sizeof(GrisMaterial);
    case 3: return sizeof(GrisMeshVertex);
    case 4: return sizeof(GrisObjectInstance);
    case 5: return sizeof(GrisTriangleLight);
    case 6: return sizeof(GrisLightTableEntry);
    case 7: return sizeof(GrisSettings);
    case 8: return sizeof(GrisDIReservoir);
    case 9: return sizeof(GrisDISettings);
    }
    return 0;
}

int grisCreate(int device, GrisContext** out) {
    if (!out) return GRIS_ERR_INVALID_ARGUMENT;
    *out = nullptr;
    int count = 0;
    cudaError_t e = cudaGetDeviceCount(&count);
    if (e != cudaSuccess || count == 0) return GRIS_ERR_CUDA;
    if (device < 0 || device >= count) return GRIS_ERR_INVALID_ARGUMENT;
    GrisContext* ctx = new GrisContext();
    ctx->device = device;
    if (cudaSetDevice(device) != cudaSuccess || cudaStreamCreateWithFlags(&ctx->stream, cudaStreamNonBlocking) != cudaSuccess ||
        cudaMalloc(&ctx->dCounters, GRIS_NUM_COUNTERS * sizeof(unsigned long long)) != cudaSuccess ||
        cudaMallocHost(&ctx->hCounters, GRIS_NUM_COUNTERS * sizeof(unsigned long long)) != cudaSuccess ||
        cudaMemset(ctx->dCounters, 0, GRIS_NUM_COUNTERS * sizeof(unsigned long long)) != cudaSuccess) {
        delete ctx;
        return GRIS_ERR_CUDA;
    }
    *out = ctx;
    return GRIS_OK;
}

int grisDestroy(GrisContext* ctx) {
    if (!ctx) return GRIS_ERR_INVALID_ARGUMENT;
    cudaSetDevice(ctx->device);
    if (ctx->stream) cudaStreamSynchronize(ctx->stream);
    ctx->wave.release();
    if (ctx->dReduce) cudaFree(ctx->dReduce);
    if (ctx->diSplit) cudaFree(ctx->diSplit);
    if (ctx->diSide.aux) { cudaStreamSynchronize(ctx->diSide.aux); cudaStreamDestroy(ctx->diSide.aux); }
    if (ctx->diSide.evFork) cudaEventDestroy(ctx->diSide.evFork);
    if (ctx->diSide.evJoin) cudaEventDestroy(ctx->diSide.evJoin);
    if (ctx->copyStream) { cudaStreamSynchronize(ctx->copyStream); cudaStreamDestroy(ctx->copyStream); }
    if (ctx->evStaged) cudaEventDestroy(ctx->evStaged);
    if (ctx->evCopied) cudaEventDestroy(ctx->evCopied);
    if (ctx->staging) cudaFree(ctx->staging);
    cudaFree(ctx->dCounters);
    cudaFreeHost(ctx->hCounters);
    if (ctx->stream) cudaStreamDestroy(ctx->stream);
    delete ctx;
    return GRIS_OK;
}

const char* grisGetError(const GrisContext* ctx) { return ctx ? ctx->err.c_str() : "null context"; }

void* grisGetStream(GrisContext* ctx) { return ctx ? (void*)ctx->stream : nullptr; }

int grisReadCounters(GrisContext* ctx, uint64_t out[4], int reset) {
    if (!ctx || !out) return GRIS_ERR_INVALID_ARGUMENT;
    cudaSetDevice(ctx->device);
    GRIS_CK(ctx, cudaMemcpyAsync(ctx->hCounters, ctx->dCounters, 4 * sizeof(unsigned long long), cudaMemcpyDeviceToHost, ctx->stream));
    if (reset) GRIS_CK(ctx, cudaMemsetAsync(ctx->dCounters, 0, 4 * sizeof(unsigned long long), ctx->stream));
    GRIS_CK(ctx, cudaStreamSynchronize(ctx->stream));
    for (int i = 0; i < 4; i++) out[i] = ctx->hCounters[i];
    return GRIS_OK;
}

int grisSetProfiling(GrisContext* ctx, int enable) {
    if (!ctx) return GRIS_ERR_INVALID_ARGUMENT;
    ctx->prof.enabled = enable != 0;
    return GRIS_OK;
}

int grisReadProfile(GrisContext* ctx, double msTotal[4], uint64_t launches[4], int reset) {
    if (!ctx || !msTotal || !launches) return GRIS_ERR_INVALID_ARGUMENT;
    cudaSetDevice(ctx->device);
    ctx->prof.collect();
    for (int k = 0; k < 4; k++) {
        msTotal[k] = ctx->prof.ms[k];
        launches[k] = ctx->prof.launches[k];
    }
    if (reset) ctx->prof.reset();
    return GRIS_OK;
}

int grisReadKernelProfile(GrisContext* ctx, GrisKernelProfile out[GRIS_PROFILE_SLOTS], int reset) {
    if (!ctx || !out) return GRIS_ERR_INVALID_ARGUMENT;
    cudaSetDevice(ctx->device);
    ctx->prof.collect();
    GRIS_CK(ctx, cudaMemcpyAsync(ctx->hCounters + 8, ctx->dCounters + 8, 39 * sizeof(unsigned long long),
                                 cudaMemcpyDeviceToHost, ctx->stream));
    if (reset) {
        GRIS_CK(ctx, cudaMemsetAsync(ctx->dCounters + 8, 0, 16 * sizeof(unsigned long long), ctx->stream));
        GRIS_CK(ctx, cudaMemsetAsync(ctx->dCounters + 26, 0, 21 * sizeof(unsigned long long), ctx->stream));
    }
    GRIS_CK(ctx, cudaStreamSynchronize(ctx->stream));
    const unsigned long long* c = ctx->hCounters;
    for (int k = 0; k < GRIS_PROFILE_SLOTS; k++) {
        GrisKernelProfile& o = out[k];
        o.ms = ctx->prof.ms[k];
        o.launches = ctx->prof.launches[k];
        o.nodes = o.tris = o.rays = 0;
        if (k < 4) { o.nodes = c[8 + 2 * k]; o.tris = c[9 + 2 * k]; o.rays = c[16 + k]; }
        if (k == GRIS_SLOT_WAVE_EXTEND || k == GRIS_SLOT_WAVE_SHADOW) {
            int s = k == GRIS_SLOT_WAVE_EXTEND ? 0 : 1;
            o.nodes = c[26 + 3 * s]; o.tris = c[27 + 3 * s]; o.rays = c[28 + 3 * s];
        }
        if (k == GRIS_SLOT_REUSE_VIS_TEMPORAL || k == GRIS_SLOT_REUSE_VIS_SPATIAL) {
            int r = k - GRIS_SLOT_REUSE_VIS_TEMPORAL;
            o.nodes = c[41 + 3 * r]; o.tris = c[42 + 3 * r]; o.rays = c[43 + 3 * r];
        }
        if (k >= GRIS_SLOT_DI_CANDIDATES && k <= GRIS_SLOT_DI_SPATIAL) {
            int d = k - GRIS_SLOT_DI_CANDIDATES;
            o.nodes = c[32 + 3 * d]; o.tris = c[33 + 3 * d]; o.rays = c[34 + 3 * d];
        }
    }
    if (reset) ctx->prof.reset();
    return GRIS_OK;
}

int grisSetLaunchMode(GrisContext* ctx, int mode) {
    if (!ctx || (mode != GRIS_LAUNCH_GRID && mode != GRIS_LAUNCH_PERSISTENT)) return GRIS_ERR_INVALID_ARGUMENT;
    ctx->launchMode = mode;
    return GRIS_OK;
}

int grisSetGraphs(GrisContext* ctx, int enable) {
    if (!ctx) return GRIS_ERR_INVALID_ARGUMENT;
    ctx->useGraphs = enable != 0;
    return GRIS_OK;
}

int grisSetWaveLaunch(GrisContext* ctx, int traceBlocksPerSM, int shadeBlocksPerSM) {
    if (!ctx || traceBlocksPerSM < 1 || traceBlocksPerSM > 64 || shadeBlocksPerSM < 1 || shadeBlocksPerSM > 64)
        return GRIS_ERR_INVALID_ARGUMENT;
    ctx->waveLaunch.traceBlocksPerSM = traceBlocksPerSM;
    ctx->waveLaunch.shadeBlocksPerSM = shadeBlocksPerSM;
    return GRIS_OK;
}

int grisSetWaveRefill(GrisContext* ctx, int enable) {
    if (!ctx) return GRIS_ERR_INVALID_ARGUMENT;
    ctx->waveLaunch.refill = enable != 0;
    return GRIS_OK;
}

int grisSetPathForm(GrisContext* ctx, int form) {
    if (!ctx || (form != GRIS_PATH_MEGAKERNEL && form != GRIS_PATH_WAVEFRONT)) return GRIS_ERR_INVALID_ARGUMENT;
    ctx->pathForm = form;
    return GRIS_OK;
}

int grisSetWorkCounting(GrisContext* ctx, int enable) {
    if (!ctx) return GRIS_ERR_INVALID_ARGUMENT;
    ctx->countWork = enable != 0;
    return GRIS_OK;
}

int grisReadWorkCounters(GrisContext* ctx, uint64_t nodes[4], uint64_t tris[4], uint64_t rays[4], int reset) {
    if (!ctx || !nodes || !tris || !rays) return GRIS_ERR_INVALID_ARGUMENT;
    cudaSetDevice(ctx->device);
    GRIS_CK(ctx, cudaMemcpyAsync(ctx->hCounters + 8, ctx->dCounters + 8, 16 * sizeof(unsigned long long),
                                 cudaMemcpyDeviceToHost, ctx->stream));
    if (reset) {
        GRIS_CK(ctx, cudaMemsetAsync(ctx->dCounters + 8, 0, 16 * sizeof(unsigned long long), ctx->stream));
        GRIS_CK(ctx, cudaMemsetAsync(ctx->dCounters + 26, 0, 17 * sizeof(unsigned long long), ctx->stream));
    }
    GRIS_CK(ctx, cudaStreamSynchronize(ctx->stream));
    for (int k = 0; k < 4; k++) {
        nodes[k] = ctx->hCounters[8 + 2 * k];
        tris[k] = ctx->hCounters[9 + 2 * k];
        rays[k] = ctx->hCounters[16 + k];
    }
    return GRIS_OK;
}

int grisSync(GrisContext* ctx) {
    if (!ctx) return GRIS_ERR_INVALID_ARGUMENT;
    cudaSetDevice(ctx->device);
    GRIS_CK(ctx, cudaStreamSynchronize(ctx->stream));
    GRIS_CK(ctx, cudaMemcpy(ctx->hCounters + 3, ctx->dCounters + 3, sizeof(unsigned long long), cudaMemcpyDeviceToHost));
    if (ctx->hCounters[3]) {
        const unsigned long long w = ctx->hCounters[3];
        std::string what;
        if (w & 1ull) what += " traversal stack limit";
        if (w & 2ull) what += " tensor-core wait gave up";
        return fail(ctx, GRIS_ERR_DEVICE_FAULT, "a kernel raised the error word (bits " + std::to_string(w) + ":" + what + ")");
    }
    return GRIS_OK;
}

/* ------------------------------------------------------------------ scene */
int grisSceneCreate(GrisContext* ctx, const GrisSceneDesc* d, GrisScene** out) {
    if (!ctx || !d || !out) return fail(ctx, GRIS_ERR_INVALID_ARGUMENT, "null argument");
    *out = nullptr;
    if ((d->vertexCount && !d->vertices) || (d->indexCount && !d->indices) || (d->instanceCount && !d->instances) ||
        (d->materialCount && !d->materials) || (d->materialIndexCount && !d->materialIndices) ||
        (d->lightCount && !d->lights) || (d->lightTableCount && !d->lightTable))
        return fail(ctx, GRIS_ERR_INVALID_ARGUMENT, "array pointer is null but its count is not");
    if (d->lightCount && d->lightTableCount != d->lightCount + 1)
        return fail(ctx, GRIS_ERR_INVALID_ARGUMENT, "light table needs lightCount + 1 entries");
    for (uint64_t i = 0; i < d->materialCount; i++)
        if (d->materials[i].textureIdx != 0xffffffffu)
            return fail(ctx, GRIS_ERR_UNSUPPORTED, "textured materials are not supported");
    cudaSetDevice(ctx->device);
    GrisScene* s = new GrisScene();
    s->ctx = ctx;
    std::string err;
    if (!grisrt::build_bvh(*d, s->bvh, err)) { delete s; return fail(ctx, GRIS_ERR_INVALID_ARGUMENT, err); }
    {
        float mn[3] = {3.0e38f, 3.0e38f, 3.0e38f}, mx[3] = {-3.0e38f, -3.0e38f, -3.0e38f};
        const std::vector<float>& T = s->bvh.tris;
        for (size_t t = 0; t + 12 <= T.size(); t += 12)   /* v0, instance, e1, triangle, e2, 0 */
            for (int c = 0; c < 3; c++) {
                float v0 = T[t + c], p1 = v0 + T[t + 4 + c], p2 = v0 + T[t + 8 + c];
                mn[c] = std::min(mn[c], std::min(v0, std::min(p1, p2)));
                mx[c] = std::max(mx[c], std::max(v0, std::max(p1, p2)));
            }
        for (int c = 0; c < 3; c++) { s->view.boxMin[c] = mn[c]; s->view.boxMax[c] = mx[c]; }
    }
    int rc = GRIS_OK;
#define UP(src, n, dst) if (rc == GRIS_OK) rc = upload(ctx, s, src, n, dst)
    UP(d->vertices, d->vertexCount, &s->view.vertices);
    UP(d->indices, d->indexCount, &s->view.indices);
    UP(d->instances, d->instanceCount, &s->view.instances);
    UP(d->materials, d->materialCount, &s->view.materials);
    UP(d->materialIndices, d->materialIndexCount, &s->view.matIndices);
    UP(d->lights, d->lightCount, &s->view.lights);
    UP(d->lightTable, d->lightTableCount, &s->view.table);
    UP(s->bvh.nodes.data(), (uint64_t)s->bvh.nodes.size(), &s->view.nodes);
    UP(s->bvh.tris.data(), (uint64_t)s->bvh.tris.size(), &s->view.tris);
#undef UP
    if (rc == GRIS_OK) {
        cudaError_t e = cudaStreamSynchronize(ctx->stream);
        if (e != cudaSuccess) rc = cuda_fail(ctx, e, "scene upload");
    }
    if (rc != GRIS_OK) { grisSceneDestroy(s); return rc; }
    s->view.nVertices = d->vertexCount; s->view.nIndices = d->indexCount; s->view.nInstances = d->instanceCount;
    s->view.nMaterials = d->materialCount; s->view.nMatIndices = d->materialIndexCount;
    s->view.nLights = d->lightCount; s->view.nTable = d->lightTableCount;
    s->stats.triangleCount = s->bvh.triangleCount;
    s->stats.nodeCount = s->bvh.nodes.size() / GRIS_NODE_WORDS;
    s->stats.nodeBytes = s->bvh.nodes.size() * 4ull;
    s->stats.triangleBytes = s->bvh.tris.size() * 4ull;
    s->stats.maxDepth = s->bvh.maxDepth;
    s->stats.buildSeconds = s->bvh.buildSeconds;
    *out = s;
    return GRIS_OK;
}

int grisSceneDestroy(GrisScene* s) {
    if (!s) return GRIS_ERR_INVALID_ARGUMENT;
    if (s->ctx) {
        cudaSetDevice(s->ctx->device);
        cudaStreamSynchronize(s->ctx->stream);
    }
    for (void* p : s->allocations) cudaFree(p);
    delete s;
    return GRIS_OK;
}

int grisDebugHostSceneCreate(const GrisSceneDesc* d, GrisScene** out) {
    if (!d || !out) return GRIS_ERR_INVALID_ARGUMENT;
    *out = nullptr;
    GrisScene* s = new GrisScene();
    std::string err;
    if (!grisrt::build_bvh(*d, s->bvh, err)) { delete s; return GRIS_ERR_INVALID_ARGUMENT; }
    s->stats.triangleCount = s->bvh.triangleCount;
    s->stats.nodeCount = s->bvh.nodes.size() / GRIS_NODE_WORDS;
    s->stats.nodeBytes = s->bvh.nodes.size() * 4ull;
    s->stats.triangleBytes = s->bvh.tris.size() * 4ull;
    s->stats.maxDepth = s->bvh.maxDepth;
    s->stats.buildSeconds = s->bvh.buildSeconds;
    *out = s;
    return GRIS_OK;
}

int grisSceneGetStats(const GrisScene* s, GrisSceneStats* out) {
    if (!s || !out) return GRIS_ERR_INVALID_ARGUMENT;
    *out = s->stats;
    return GRIS_OK;
}

int grisDebugTraceHost(const GrisScene* s, const float* rays, uint64_t n, int anyHit, float* hitTUV, uint32_t* hitInst,
                       uint32_t* hitTri) {
    if (!s || (n && (!rays || !hitTUV || !hitInst || !hitTri))) return GRIS_ERR_INVALID_ARGUMENT;
    const uint32_t* nodes = s->bvh.nodes.data();
    const float* tris = s->bvh.tris.data();
    int anyErr = 0;
#pragma omp parallel for schedule(dynamic, 256) reduction(| : anyErr)
    for (int64_t i = 0; i < (int64_t)n; i++) {
        const float* r = rays + i * 8;
        GrisRayHit h;
        int err = 0;
        bool hit = anyHit ? gris_bvh_trace<true>(nodes, tris, r[0], r[1], r[2], r[4], r[5], r[6], r[3], r[7], false, &h, &err, nullptr)
                          : gris_bvh_trace<false>(nodes, tris, r[0], r[1], r[2], r[4], r[5], r[6], r[3], r[7], false, &h, &err, nullptr);
        anyErr |= err;
        if (hit) { hitTUV[i * 4] = h.t; hitTUV[i * 4 + 1] = h.u; hitTUV[i * 4 + 2] = h.v; hitTUV[i * 4 + 3] = 0.0f; hitInst[i] = h.inst; hitTri[i] = h.tri; }
        else { hitTUV[i * 4] = -1.0f; hitTUV[i * 4 + 1] = 0.0f; hitTUV[i * 4 + 2] = 0.0f; hitTUV[i * 4 + 3] = 0.0f; hitInst[i] = GRIS_INVALID_HIT; hitTri[i] = GRIS_INVALID_HIT; }
    }
    return anyErr ? GRIS_ERR_DEVICE_FAULT : GRIS_OK;
}

int grisDebugTraceDevice(GrisContext* ctx, const GrisScene* s, const float* dRays, uint64_t n, int anyHit, float* dHitTUV,
                         uint32_t* dHitInst, uint32_t* dHitTri) {
    if (!ctx || !s) return GRIS_ERR_INVALID_ARGUMENT;
    cudaSetDevice(ctx->device);
    GRIS_CK(ctx, grisrt::launch_debug_trace(s->view.nodes, s->view.tris, dRays, n, anyHit, dHitTUV, dHitInst, dHitTri,
                                            ctx->dCounters, ctx->stream));
    return GRIS_OK;
}

/* ------------------------------------------------------------------ passes on caller buffers */
int grisPassGBuffer(GrisContext* ctx, const GrisScene* s, const GrisGBufferBindings* b, const GrisCamera* cam) {
    if (!ctx || !s || !b || !cam) return fail(ctx, GRIS_ERR_INVALID_ARGUMENT, "null argument");
    if (!b->depthNormal || !b->albedoMatId || !b->motion || b->width == 0 || b->height == 0)
        return fail(ctx, GRIS_ERR_INVALID_ARGUMENT, "G-buffer bindings incomplete");
    if (cam->filmSize[0] != b->width || cam->filmSize[1] != b->height)
        return fail(ctx, GRIS_ERR_INVALID_ARGUMENT, "camera filmSize differs from the bound extent");
    cudaSetDevice(ctx->device);
    GRIS_CK(ctx, grisrt::launch_gbuffer(scene_view(s), *b, *cam, ctx->dCounters, ctx->countWork, &ctx->prof, ctx->stream));
    return GRIS_OK;
}

int grisConvergedAccumulate(GrisContext* ctx, const GrisScene* s, const GrisConvergedBindings* b, const GrisCamera* cam,
                            const GrisSettings* set, uint32_t sppBegin, uint32_t sppCount, int estimator) {
    if (!ctx || !s || !b || !cam || !set) return fail(ctx, GRIS_ERR_INVALID_ARGUMENT, "null argument");
    if (b->width == 0 || b->height == 0 || !b->depthNormal || !b->albedoMatId || !b->sum)
        return fail(ctx, GRIS_ERR_INVALID_ARGUMENT, "converged bindings incomplete");
    if (cam->filmSize[0] != b->width || cam->filmSize[1] != b->height)
        return fail(ctx, GRIS_ERR_INVALID_ARGUMENT, "camera filmSize differs from the bound extent");
    if (set->maxDepth == 0 || set->maxDepth > 255) return fail(ctx, GRIS_ERR_INVALID_ARGUMENT, "maxDepth must be 1..255");
    if (estimator != GRIS_ESTIMATOR_CANDIDATES && estimator != GRIS_ESTIMATOR_INDIRECT)
        return fail(ctx, GRIS_ERR_INVALID_ARGUMENT, "unknown estimator");
    if ((uint64_t)sppBegin + sppCount > 0xffffffffull) return fail(ctx, GRIS_ERR_INVALID_ARGUMENT, "sample range overflows");
    if (sppCount == 0) return GRIS_OK;
    cudaSetDevice(ctx->device);
    GRIS_CK(ctx, grisrt::launch_converged(scene_view(s), *b, *cam, *set, sppBegin, sppCount, estimator, ctx->dCounters,
                                          ctx->stream));
    return GRIS_OK;
}

int grisRelMSE(GrisContext* ctx, const float* image, const double* refSum, double refScale, uint64_t pixels, double eps,
               double out[2]) {
    if (!ctx || !image || !refSum || !out || !(eps >= 0.0)) return fail(ctx, GRIS_ERR_INVALID_ARGUMENT, "bad relMSE arguments");
    cudaSetDevice(ctx->device);
    if (!ctx->dReduce)
        GRIS_CK(ctx, cudaMalloc(&ctx->dReduce, grisrt::relmse_scratch_doubles() * sizeof(double)));
    GRIS_CK(ctx, grisrt::launch_relmse(image, refSum, refScale, pixels, eps, ctx->dReduce, ctx->stream));
    double h[2] = {0.0, 0.0};
    GRIS_CK(ctx, cudaMemcpyAsync(h, ctx->dReduce, sizeof(h), cudaMemcpyDeviceToHost, ctx->stream));
    GRIS_CK(ctx, cudaStreamSynchronize(ctx->stream));
    out[0] = h[0];
    out[1] = h[1];
    return GRIS_OK;
}

int grisPassRender(GrisContext* ctx, const GrisScene* s, const GrisPassBindings* b, const GrisCamera* cam,
                   const GrisCamera* prevCam, const GrisSettings* set, int passes) {
    if (!ctx || !s || !b || !cam || !prevCam || !set) return fail(ctx, GRIS_ERR_INVALID_ARGUMENT, "null argument");
    if (b->width == 0 || b->height == 0 || !b->depthNormal || !b->albedoMatId || !b->reservoirThis || !b->reservoirTemp ||
        ((passes & 2) && (!b->depthNormalPrev || !b->albedoMatIdPrev || !b->motion || !b->reservoirPrev)) ||
        ((passes & 4) && !b->output))
        return fail(ctx, GRIS_ERR_INVALID_ARGUMENT, "pass bindings incomplete");
    if (cam->filmSize[0] != b->width || cam->filmSize[1] != b->height)
        return fail(ctx, GRIS_ERR_INVALID_ARGUMENT, "camera filmSize differs from the bound extent");
    if (set->maxDepth == 0 || set->maxDepth > 255) return fail(ctx, GRIS_ERR_INVALID_ARGUMENT, "maxDepth must be 1..255");
    if (set->spatialNeighbors > 64) return fail(ctx, GRIS_ERR_INVALID_ARGUMENT, "spatialNeighbors must be <= 64");
    if (set->envRadiance[0] != 0.0f || set->envRadiance[1] != 0.0f || set->envRadiance[2] != 0.0f)
        return fail(ctx, GRIS_ERR_INVALID_ARGUMENT, "envRadiance is reserved and must be 0");
    cudaSetDevice(ctx->device);
    if (ctx->pathForm == GRIS_PATH_WAVEFRONT && (passes & 1)) {
        /* the wavefront path tracer through the batch launcher, as a one-view batch */
        uint64_t pixels = (uint64_t)b->width * b->height;
        WaveScratch& w = ctx->wave;
        if (w.wb.capacity < pixels) {
            cudaStreamSynchronize(ctx->stream);
            w.release();
            cudaError_t e = cudaSuccess;
            auto alloc = [&](void** p, size_t bytes) {
                if (e == cudaSuccess) e = cudaMalloc(p, bytes < 256 ? 256 : bytes);
                if (e == cudaSuccess) w.allocations.push_back(*p);
            };
            size_t P = (size_t)pixels;
            alloc(&w.wb.state, P * grisrt::kWaveStateBytes);
            alloc(&w.wb.nee, P * grisrt::kWaveNeeBytes);
            alloc(&w.wb.hit, P * 16);
            alloc((void**)&w.wb.blocked, P);
            alloc((void**)&w.wb.queue[0], P * 4);
            alloc((void**)&w.wb.queue[1], P * 4);
            alloc((void**)&w.wb.shadowQueue, P * 4);
            alloc(&w.wb.ray, P * 32);
            alloc((void**)&w.wb.counts, 1536 * 4);
            if (e == cudaSuccess) e = grisrt::wave_streams_create(w.wb);
            alloc(&w.dViews, grisrt::view_entry_bytes());
            for (int i = 0; i < 2 && e == cudaSuccess; i++) {
                e = cudaMallocHost(&w.hViews[i], grisrt::view_entry_bytes());
                if (e == cudaSuccess) e = cudaEventCreateWithFlags(&w.staged[i], cudaEventDisableTiming);
            }
            if (e != cudaSuccess) { w.release(); return cuda_fail(ctx, e, "wavefront scratch"); }
            w.wb.capacity = pixels;
        }
        /* the reuse passes' three-launch form: per-slot records for every pixel and neighbour */
        const uint32_t slots = set->spatialNeighbors > 1u ? set->spatialNeighbors : 1u;
        if (!set->misWeights && slots <= grisrt::kReuseMaxSlots &&
            (w.wb.reuse.slots < slots || w.wb.reuse.capacity < pixels)) {
            cudaStreamSynchronize(ctx->stream);
            if (w.wb.reuse.block) cudaFree(w.wb.reuse.block);
            w.wb.reuse = grisrt::ReuseBuffers{};
            void* p = nullptr;
            cudaError_t e = cudaMalloc(&p, grisrt::reuse_bytes(pixels, slots));
            if (e != cudaSuccess) return cuda_fail(ctx, e, "reuse pass buffers");
            grisrt::reuse_carve(w.wb.reuse, p, pixels, slots);
        }
        grisrt::BatchView v;
        memset(&v, 0, sizeof(v));
        v.scene = scene_view(s);
        v.b = *b;
        v.cam = *cam; v.prev = *prevCam; v.set = *set;
        int k = w.stage;
        GRIS_CK(ctx, cudaEventSynchronize(w.staged[k]));
        GRIS_CK(ctx, grisrt::launch_batch(&v, 1, w.dViews, w.hViews[k], w.wb, ctx->dCounters, ctx->countWork, &ctx->prof,
                                          ctx->stream, GRIS_PATH_WAVEFRONT, passes & 7, ctx->waveLaunch));
        GRIS_CK(ctx, cudaEventRecord(w.staged[k], ctx->stream));
        w.stage ^= 1;
        return GRIS_OK;
    }
    GRIS_CK(ctx, grisrt::launch_gris(scene_view(s), *b, *cam, *prevCam, *set, passes & 7, ctx->dCounters, ctx->countWork,
                                     &ctx->prof, ctx->stream, ctx->launchMode));
    return GRIS_OK;
}

/* ------------------------------------------------------------------ frames */
int grisFrameCreate(GrisContext* ctx, uint32_t w, uint32_t h, GrisFrame** out) {
    if (!ctx || !out || w == 0 || h == 0) return fail(ctx, GRIS_ERR_INVALID_ARGUMENT, "bad frame size");
    *out = nullptr;
    cudaSetDevice(ctx->device);
    GrisFrame* f = new GrisFrame();
    f->ctx = ctx; f->w = w; f->h = h;
    size_t n = (size_t)w * h;
    cudaError_t e = cudaSuccess;
    auto alloc = [&](void** p, size_t bytes) {
        if (e == cudaSuccess) e = cudaMalloc(p, bytes);
        if (e == cudaSuccess) e = cudaMemsetAsync(*p, 0, bytes, ctx->stream);
    };
    for (int i = 0; i < 2; i++) {
        alloc((void**)&f->depthNormal[i], n * 16);
        alloc((void**)&f->albedoMatId[i], n * 8);
        alloc((void**)&f->resv[i], n * sizeof(GrisReservoir));
    }
    alloc((void**)&f->motion, n * 4);
    alloc((void**)&f->temp, n * sizeof(GrisReservoir));
    alloc((void**)&f->output, n * 16);
    if (e == cudaSuccess) e = cudaStreamSynchronize(ctx->stream);
    if (e != cudaSuccess) { grisFrameDestroy(f); return cuda_fail(ctx, e, "frame allocation"); }
    *out = f;
    return GRIS_OK;
}

int grisFrameDestroy(GrisFrame* f) {
    if (!f) return GRIS_ERR_INVALID_ARGUMENT;
    cudaSetDevice(f->ctx->device);
    cudaStreamSynchronize(f->ctx->stream);
    for (int i = 0; i < 2; i++) {
        cudaFree(f->depthNormal[i]); cudaFree(f->albedoMatId[i]); cudaFree(f->resv[i]); cudaFree(f->diResv[i]);
    }
    cudaFree(f->motion); cudaFree(f->temp); cudaFree(f->output); cudaFree(f->diTemp); cudaFree(f->directOutput);
    delete f;
    return GRIS_OK;
}

int grisFrameRender(GrisContext* ctx, const GrisScene* s, GrisFrame* f, const GrisCamera* cam, const GrisCamera* prevCam,
                    const GrisSettings* set) {
    if (!ctx || !s || !f || !cam || !prevCam || !set) return fail(ctx, GRIS_ERR_INVALID_ARGUMENT, "null argument");
    int j = f->next;
    GrisGBufferBindings gb;
    gb.width = f->w; gb.height = f->h;
    gb.depthNormal = f->depthNormal[j]; gb.albedoMatId = f->albedoMatId[j]; gb.motion = f->motion;
    int rc = grisPassGBuffer(ctx, s, &gb, cam);
    if (rc != GRIS_OK) return rc;
    GrisPassBindings b;
    b.width = f->w; b.height = f->h;
    b.depthNormal = f->depthNormal[j]; b.depthNormalPrev = f->depthNormal[j ^ 1];
    b.albedoMatId = f->albedoMatId[j]; b.albedoMatIdPrev = f->albedoMatId[j ^ 1];
    b.motion = f->motion;
    b.reservoirThis = f->resv[j]; b.reservoirPrev = f->resv[j ^ 1]; b.reservoirTemp = f->temp;
    b.output = f->output;
    rc = grisPassRender(ctx, s, &b, cam, prevCam, set, 7);
    if (rc != GRIS_OK) return rc;
    f->next = j ^ 1;
    return GRIS_OK;
}

/* ------------------------------------------------------------------ ReSTIR DI */
int grisPassDI(GrisContext* ctx, const GrisScene* s, const GrisDIBindings* b, const GrisCamera* cam,
               const GrisCamera* prevCam, const GrisDISettings* set, int passes) {
    if (!ctx || !s || !b || !cam || !prevCam || !set) return fail(ctx, GRIS_ERR_INVALID_ARGUMENT, "null argument");
    if (b->width == 0 || b->height == 0 || !b->depthNormal || !b->albedoMatId || !b->reservoirThis ||
        ((passes & 6) && !b->reservoirTemp) ||
        ((passes & 2) && (!b->depthNormalPrev || !b->albedoMatIdPrev || !b->motion || !b->reservoirPrev)) ||
        ((passes & 4) && !b->directOutput))
        return fail(ctx, GRIS_ERR_INVALID_ARGUMENT, "DI pass bindings incomplete");
    if (cam->filmSize[0] != b->width || cam->filmSize[1] != b->height)
        return fail(ctx, GRIS_ERR_INVALID_ARGUMENT, "camera filmSize differs from the bound extent");
    if (set->shiftType > GRIS_DI_SHIFT_HYBRID || set->sampleType > GRIS_DI_SAMPLE_BOTH)
        return fail(ctx, GRIS_ERR_INVALID_ARGUMENT, "DI shiftType must be 0..2 and sampleType 0..2");
    grisrt::DeviceSceneView view;
    int dev = -1;
    if (!grisrt::scene_device(s, &view, &dev)) return fail(ctx, GRIS_ERR_INVALID_ARGUMENT, "scene has no device copy");
    if (dev != ctx->device) return fail(ctx, GRIS_ERR_INVALID_ARGUMENT, "scene lives on another device");
    cudaSetDevice(ctx->device);
    /* the candidates pass and the spatial pass (reconnection shift) in three launches want their
     * scratch (one block, used by one pass at a time): grown here, outside a stream capture
     * (inside one the single kernels run) */
    const uint64_t px = (uint64_t)b->width * b->height;
    cudaStreamCaptureStatus cap = cudaStreamCaptureStatusNone;
    cudaStreamIsCapturing(ctx->stream, &cap);
    const bool split = (passes & 1) || ((passes & 4) && set->spatialReuse && set->shiftType == GRIS_DI_SHIFT_RECONNECTION);
    if (split && ctx->diSplitPixels < px && cap == cudaStreamCaptureStatusNone) {
        cudaStreamSynchronize(ctx->stream);
        if (ctx->diSplit) cudaFree(ctx->diSplit);
        ctx->diSplit = nullptr;
        ctx->diSplitPixels = 0;
        if (cudaMalloc(&ctx->diSplit, grisrt::di_split_bytes_per_pixel() * px + 256) == cudaSuccess) ctx->diSplitPixels = px;
        else ctx->diSplit = nullptr;
    }
    if (split && !ctx->diSide.aux && cap == cudaStreamCaptureStatusNone) {
        grisrt::DISide d{nullptr, nullptr, nullptr};
        if (cudaStreamCreateWithFlags(&d.aux, cudaStreamNonBlocking) == cudaSuccess &&
            cudaEventCreateWithFlags(&d.evFork, cudaEventDisableTiming) == cudaSuccess &&
            cudaEventCreateWithFlags(&d.evJoin, cudaEventDisableTiming) == cudaSuccess) {
            ctx->diSide = d;
        } else {   /* without them the walks run in order */
            if (d.aux) cudaStreamDestroy(d.aux);
            if (d.evFork) cudaEventDestroy(d.evFork);
            if (d.evJoin) cudaEventDestroy(d.evJoin);
            cudaGetLastError();
        }
    }
    GRIS_CK(ctx, grisrt::launch_di(view, *b, *cam, *prevCam, *set, passes & 7, ctx->dCounters, ctx->countWork,
                                   ctx->prof.enabled ? &ctx->prof : nullptr, ctx->stream, ctx->diSplit,
                                   ctx->diSplitPixels, ctx->diSide.aux ? &ctx->diSide : nullptr));
    return GRIS_OK;
}

int grisFrameRenderDI(GrisContext* ctx, const GrisScene* s, GrisFrame* f, const GrisCamera* cam,
                      const GrisCamera* prevCam, const GrisSettings* set, const GrisDISettings* di) {
    if (!ctx || !s || !f || !cam || !prevCam || !di) return fail(ctx, GRIS_ERR_INVALID_ARGUMENT, "null argument");
    cudaSetDevice(ctx->device);
    size_t n = (size_t)f->w * f->h;
    if (!f->directOutput) {
        cudaError_t e = cudaSuccess;
        auto alloc = [&](void** p, size_t bytes) {
            if (e == cudaSuccess) e = cudaMalloc(p, bytes);
            if (e == cudaSuccess) e = cudaMemsetAsync(*p, 0, bytes, ctx->stream);
        };
        alloc((void**)&f->diResv[0], n * sizeof(GrisDIReservoir));
        alloc((void**)&f->diResv[1], n * sizeof(GrisDIReservoir));
        alloc((void**)&f->diTemp, n * sizeof(GrisDIReservoir));
        alloc((void**)&f->directOutput, n * 16);
        if (e != cudaSuccess) {
            for (int i = 0; i < 2; i++) { cudaFree(f->diResv[i]); f->diResv[i] = nullptr; }
            cudaFree(f->diTemp); cudaFree(f->directOutput);
            f->diTemp = nullptr; f->directOutput = nullptr;
            return cuda_fail(ctx, e, "DI buffers");
        }
    }
    int j = f->next;
    GrisGBufferBindings gb;
    gb.width = f->w; gb.height = f->h;
    gb.depthNormal = f->depthNormal[j]; gb.albedoMatId = f->albedoMatId[j]; gb.motion = f->motion;
    int rc = grisPassGBuffer(ctx, s, &gb, cam);
    if (rc != GRIS_OK) return rc;
    GrisDIBindings d;
    d.width = f->w; d.height = f->h;
    d.depthNormal = f->depthNormal[j]; d.depthNormalPrev = f->depthNormal[j ^ 1];
    d.albedoMatId = f->albedoMatId[j]; d.albedoMatIdPrev = f->albedoMatId[j ^ 1];
    d.motion = f->motion;
    d.reservoirThis = f->diResv[j]; d.reservoirPrev = f->diResv[j ^ 1]; d.reservoirTemp = f->diTemp;
    d.directOutput = f->directOutput;
    rc = grisPassDI(ctx, s, &d, cam, prevCam, di, 7);
    if (rc != GRIS_OK) return rc;
    if (set) {
        GrisPassBindings b;
        b.width = f->w; b.height = f->h;
        b.depthNormal = f->depthNormal[j]; b.depthNormalPrev = f->depthNormal[j ^ 1];
        b.albedoMatId = f->albedoMatId[j]; b.albedoMatIdPrev = f->albedoMatId[j ^ 1];
        b.motion = f->motion;
        b.reservoirThis = f->resv[j]; b.reservoirPrev = f->resv[j ^ 1]; b.reservoirTemp = f->temp;
        b.output = f->output;
        rc = grisPassRender(ctx, s, &b, cam, prevCam, set, 7);
        if (rc != GRIS_OK) return rc;
    }
    f->next = j ^ 1;
    return GRIS_OK;
}

/* ------------------------------------------------------------------ post-processing */
int grisPostProcess(GrisContext* ctx, const GrisPostBindings* b, const GrisPostSettings* set) {
    if (!ctx || !b || !set) return fail(ctx, GRIS_ERR_INVALID_ARGUMENT, "null argument");
    if (b->width == 0 || b->height == 0 || (!b->color && !b->rgba8) || (!set->noDirect && !b->directOutput) ||
        (!set->noIndirect && !b->indirectOutput))
        return fail(ctx, GRIS_ERR_INVALID_ARGUMENT, "post-processing bindings incomplete");
    if (set->toneMapping > GRIS_TONEMAP_ACES) return fail(ctx, GRIS_ERR_INVALID_ARGUMENT, "toneMapping must be 0..2");
    if (b->height > 65535u) return fail(ctx, GRIS_ERR_INVALID_ARGUMENT, "height must be <= 65535");
    cudaSetDevice(ctx->device);
    GRIS_CK(ctx, grisrt::launch_post(*b, *set, ctx->stream));
    return GRIS_OK;
}

int grisFrameGetBuffer(const GrisFrame* f, int which, int slot, void** devPtr, size_t* bytes) {
    if (!f || !devPtr || slot < 0 || slot > 1) return GRIS_ERR_INVALID_ARGUMENT;
    int j = (f->next ^ 1) ^ slot;   /* slot 0: written by the last render */
    size_t n = (size_t)f->w * f->h;
    void* p = nullptr;
    size_t sz = 0;
    switch (which) {
    case 0: p = f->depthNormal[j]; sz = n * 16; break;
    case 1: p = f->albedoMatId[j]; sz = n * 8; break;
    case 2: p = f->motion; sz = n * 4; break;
    case 3: p = f->resv[j]; sz = n * sizeof(GrisReservoir); break;
    case 4: p = f->temp; sz = n * sizeof(GrisReservoir); break;
    case 5: p = f->output; sz = n * 16; break;
    case 6: p = f->diResv[j]; sz = n * sizeof(GrisDIReservoir); break;
    case 7: p = f->diTemp; sz = n * sizeof(GrisDIReservoir); break;
    case 8: p = f->directOutput; sz = n * 16; break;
    default: return GRIS_ERR_INVALID_ARGUMENT;
    }
    if (!p) return GRIS_ERR_INVALID_ARGUMENT;
    *devPtr = p;
    if (bytes) *bytes = sz;
    return GRIS_OK;
}

int grisFrameDownload(GrisContext* ctx, const GrisFrame* f, int which, int slot, void* host, size_t bytes) {
    void* p; size_t sz;
    int rc = grisFrameGetBuffer(f, which, slot, &p, &sz);
    if (rc != GRIS_OK || !ctx || !host || bytes != sz) return fail(ctx, GRIS_ERR_INVALID_ARGUMENT, "bad download request");
    cudaSetDevice(ctx->device);
    GRIS_CK(ctx, cudaMemcpyAsync(host, p, sz, cudaMemcpyDeviceToHost, ctx->stream));
    GRIS_CK(ctx, cudaStreamSynchronize(ctx->stream));
    return GRIS_OK;
}

int grisFrameDownloadAsync(GrisContext* ctx, const GrisFrame* f, int which, int slot, void* host, size_t bytes) {
    void* p; size_t sz;
    int rc = grisFrameGetBuffer(f, which, slot, &p, &sz);
    if (rc != GRIS_OK || !ctx || !host || bytes != sz) return fail(ctx, GRIS_ERR_INVALID_ARGUMENT, "bad download request");
    return grisrt::ctx_download_async(ctx, p, host, sz, "grisFrameDownloadAsync");
}

int grisDownloadWait(GrisContext* ctx) {
    if (!ctx) return GRIS_ERR_INVALID_ARGUMENT;
    if (!ctx->copyStream) return GRIS_OK;
    cudaSetDevice(ctx->device);
    GRIS_CK(ctx, cudaEventSynchronize(ctx->evCopied));
    ctx->stagingUsed = 0;
    return GRIS_OK;
}

int grisFrameUpload(GrisContext* ctx, GrisFrame* f, int which, int slot, const void* host, size_t bytes) {
    void* p; size_t sz;
    int rc = grisFrameGetBuffer(f, which, slot, &p, &sz);
    if (rc != GRIS_OK || !ctx || !host || bytes != sz) return fail(ctx, GRIS_ERR_INVALID_ARGUMENT, "bad upload request");
    cudaSetDevice(ctx->device);
    GRIS_CK(ctx, cudaMemcpyAsync(p, host, sz, cudaMemcpyHostToDevice, ctx->stream));
    GRIS_CK(ctx, cudaStreamSynchronize(ctx->stream));
    return GRIS_OK;
}

}  /* extern "C" */
