/*
 * batch.cpp — batches of views rendered with one launch per pass (C ABI: grisBatch*).
 *
 * The per-view buffers are the renderer's per-frame resources (src/Renderer.cpp:193-257) with
 * its ping-pong (Renderer.cpp:329-347, 567), laid out view after view in one allocation per
 * buffer kind; the wavefront path tracer's state and queues are sized for all views' pixels.
 */
#include <cuda_runtime.h>
#include <string.h>

#include <string>
#include <vector>

#include "../../include/grisrt.h"
#include "gris_kernels.h"
#include "guide.cuh"
#include "guide_kernels.h"
#include "grisrt_internal.h"

struct GrisBatch {
    GrisContext* ctx = nullptr;
    uint32_t n = 0;
    std::vector<const GrisScene*> scenes;
    std::vector<uint32_t> w, h;
    std::vector<uint64_t> base;   /* first pixel of each view */
    uint64_t pixels = 0;
    /* per-view frame buffers, view after view */
    float* depthNormal[2] = {nullptr, nullptr};
    uint32_t* albedoMatId[2] = {nullptr, nullptr};
    uint16_t* motion = nullptr;
    GrisReservoir* resv[2] = {nullptr, nullptr};
    GrisReservoir* temp = nullptr;
    float* output = nullptr;
    /* wavefront path tracer */
    grisrt::WaveBuffers wave{};
    std::vector<void*> allocations;
    /* view table: device copy, double-buffered pinned staging guarded by events */
    void* dViews = nullptr;
    void* hViews[2] = {nullptr, nullptr};
    cudaEvent_t staged[2] = {nullptr, nullptr};
    int stage = 0;
    int next = 0;
    /* captured frames, one per staging slot, valid for one frame shape */
    struct Graph {
        cudaGraphExec_t exec = nullptr;
        int pathForm = -1, maxDepth = -1, trace = 0, shade = 0, refill = -1, countWork = -1;
        bool pairwise = false;
        uint32_t pixels = 0, tiles = 0;
        const GrisGuide* guide = nullptr;
        int train = -1;
    } graph[2];
    GrisGuide* guide = nullptr;
    void* guideBlock = nullptr;   /* the guided-wavefront buffers (allocated with the first guide) */
};

static void drop_graphs(GrisBatch* b) {
    for (auto& g : b->graph) {
        if (g.exec) cudaGraphExecDestroy(g.exec);
        g = GrisBatch::Graph();
    }
}

using namespace grisrt;

/* The reuse passes' three-launch form keeps per-slot records for every pixel and neighbour: sized
 * for the largest neighbour count seen so far (growing drops the captured frames, whose launches
 * hold the old buffers). */
static cudaError_t ensure_reuse(GrisBatch* b, uint32_t slots, cudaStream_t st) {
    if (b->wave.reuse.slots >= slots && b->wave.reuse.capacity >= b->pixels) return cudaSuccess;
    cudaError_t e = cudaStreamSynchronize(st);
    if (e != cudaSuccess) return e;
    drop_graphs(b);
    if (b->wave.reuse.block) cudaFree(b->wave.reuse.block);
    b->wave.reuse = ReuseBuffers{};
    void* p = nullptr;
    e = cudaMalloc(&p, reuse_bytes(b->pixels, slots));
    if (e != cudaSuccess) return e;
    reuse_carve(b->wave.reuse, p, b->pixels, slots);
    return cudaSuccess;
}

extern "C" {

int grisBatchCreate(GrisContext* ctx, uint32_t n, const GrisScene* const* scenes, const uint32_t* widths,
                    const uint32_t* heights, GrisBatch** out) {
    if (!ctx || !out || !scenes || !widths || !heights || n == 0 || n > 4096)
        return ctx_fail(ctx, GRIS_ERR_INVALID_ARGUMENT, "bad batch description");
    *out = nullptr;
    cudaSetDevice(ctx_device(ctx));
    GrisBatch* b = new GrisBatch();
    b->ctx = ctx;
    b->n = n;
    for (uint32_t i = 0; i < n; i++) {
        DeviceSceneView v;
        int dev = -1;
        if (!scenes[i] || !scene_device(scenes[i], &v, &dev) || dev != ctx_device(ctx) || widths[i] == 0 || heights[i] == 0) {
            delete b;
            return ctx_fail(ctx, GRIS_ERR_INVALID_ARGUMENT, "batch view " + std::to_string(i) + ": bad scene or size");
        }
        b->scenes.push_back(scenes[i]);
        b->w.push_back(widths[i]);
        b->h.push_back(heights[i]);
        b->base.push_back(b->pixels);
        b->pixels += (uint64_t)widths[i] * heights[i];
    }
    if (b->pixels >= 0xffffffffull) { delete b; return ctx_fail(ctx, GRIS_ERR_TOO_LARGE, "batch has too many pixels"); }
    cudaError_t e = cudaSuccess;
    cudaStream_t st = ctx_stream(ctx);
    auto alloc = [&](void** p, size_t bytes, bool zero) {
        if (e != cudaSuccess) return;
        e = cudaMalloc(p, bytes < 256 ? 256 : bytes);
        if (e == cudaSuccess) b->allocations.push_back(*p);
        if (e == cudaSuccess && zero) e = cudaMemsetAsync(*p, 0, bytes, st);
    };
    size_t P = (size_t)b->pixels;
    for (int i = 0; i < 2; i++) {
        alloc((void**)&b->depthNormal[i], P * 16, true);
        alloc((void**)&b->albedoMatId[i], P * 8, true);
        alloc((void**)&b->resv[i], P * sizeof(GrisReservoir), true);
    }
    alloc((void**)&b->motion, P * 4, true);
    alloc((void**)&b->temp, P * sizeof(GrisReservoir), true);
    alloc((void**)&b->output, P * 16, true);
    alloc(&b->wave.state, P * kWaveStateBytes, false);
    alloc(&b->wave.nee, P * kWaveNeeBytes, false);
    alloc(&b->wave.hit, P * 16, false);
    alloc((void**)&b->wave.blocked, P, false);
    alloc((void**)&b->wave.queue[0], P * 4, false);
    alloc((void**)&b->wave.queue[1], P * 4, false);
    alloc((void**)&b->wave.shadowQueue, P * 4, false);
    alloc(&b->wave.ray, P * 32, false);
    alloc((void**)&b->wave.counts, 1536 * 4, true);
    b->wave.capacity = P;
    if (e == cudaSuccess) e = wave_streams_create(b->wave);
    alloc(&b->dViews, view_entry_bytes() * n, false);
    for (int i = 0; i < 2 && e == cudaSuccess; i++) {
        e = cudaMallocHost(&b->hViews[i], view_entry_bytes() * n);
        if (e == cudaSuccess) e = cudaEventCreateWithFlags(&b->staged[i], cudaEventDisableTiming);
    }
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    if (e != cudaSuccess) {
        grisBatchDestroy(b);
        return ctx_fail(ctx, e == cudaErrorMemoryAllocation ? GRIS_ERR_OUT_OF_MEMORY : GRIS_ERR_CUDA,
                        std::string("batch allocation: ") + cudaGetErrorString(e));
    }
    *out = b;
    return GRIS_OK;
}

int grisBatchDestroy(GrisBatch* b) {
    if (!b) return GRIS_ERR_INVALID_ARGUMENT;
    cudaSetDevice(ctx_device(b->ctx));
    cudaStreamSynchronize(ctx_stream(b->ctx));
    drop_graphs(b);
    if (b->guideBlock) cudaFree(b->guideBlock);
    if (b->wave.reuse.block) cudaFree(b->wave.reuse.block);
    wave_streams_destroy(b->wave);
    for (void* p : b->allocations) cudaFree(p);
    for (int i = 0; i < 2; i++) {
        if (b->hViews[i]) cudaFreeHost(b->hViews[i]);
        if (b->staged[i]) cudaEventDestroy(b->staged[i]);
    }
    delete b;
    return GRIS_OK;
}

int grisBatchRender(GrisContext* ctx, GrisBatch* b, const GrisCamera* cams, const GrisCamera* prevCams,
                    const GrisSettings* settings) {
    if (!ctx || !b || !cams || !prevCams || !settings || b->ctx != ctx)
        return ctx_fail(ctx, GRIS_ERR_INVALID_ARGUMENT, "null argument");
    cudaSetDevice(ctx_device(ctx));
    std::vector<BatchView> views(b->n);
    int j = b->next;
    for (uint32_t i = 0; i < b->n; i++) {
        if (cams[i].filmSize[0] != b->w[i] || cams[i].filmSize[1] != b->h[i])
            return ctx_fail(ctx, GRIS_ERR_INVALID_ARGUMENT, "view " + std::to_string(i) + ": camera filmSize differs from the view size");
        if (settings[i].maxDepth == 0 || settings[i].maxDepth > 255 || settings[i].spatialNeighbors > 64 ||
            settings[i].envRadiance[0] != 0.0f || settings[i].envRadiance[1] != 0.0f || settings[i].envRadiance[2] != 0.0f)
            return ctx_fail(ctx, GRIS_ERR_INVALID_ARGUMENT, "view " + std::to_string(i) + ": bad settings");
        BatchView& v = views[i];
        int dummy = 0;
        scene_device(b->scenes[i], &v.scene, &dummy);
        uint64_t o = b->base[i];
        v.b.width = b->w[i]; v.b.height = b->h[i];
        v.b.depthNormal = b->depthNormal[j] + o * 4; v.b.depthNormalPrev = b->depthNormal[j ^ 1] + o * 4;
        v.b.albedoMatId = b->albedoMatId[j] + o * 2; v.b.albedoMatIdPrev = b->albedoMatId[j ^ 1] + o * 2;
        v.b.motion = b->motion + o * 2;
        v.b.reservoirThis = b->resv[j] + o; v.b.reservoirPrev = b->resv[j ^ 1] + o; v.b.reservoirTemp = b->temp + o;
        v.b.output = b->output + o * 4;
        v.gb.width = b->w[i]; v.gb.height = b->h[i];
        v.gb.depthNormal = b->depthNormal[j] + o * 4; v.gb.albedoMatId = b->albedoMatId[j] + o * 2; v.gb.motion = b->motion + o * 2;
        v.cam = cams[i]; v.prev = prevCams[i]; v.set = settings[i];
    }
    int k = b->stage;
    cudaStream_t st = ctx_stream(ctx);
    cudaError_t e = cudaEventSynchronize(b->staged[k]);   /* the staging slot's previous copy is done */
    if (e != cudaSuccess) return ctx_fail(ctx, GRIS_ERR_CUDA, std::string("grisBatchRender: ") + cudaGetErrorString(e));
    {
        uint32_t slots = 1;
        bool pairwise = false;
        for (uint32_t i = 0; i < b->n; i++) {
            if (settings[i].spatialNeighbors > slots) slots = settings[i].spatialNeighbors;
            if (settings[i].misWeights) pairwise = true;
        }
        if (!pairwise && slots <= kReuseMaxSlots) {
            e = ensure_reuse(b, slots, st);
            if (e != cudaSuccess)
                return ctx_fail(ctx, e == cudaErrorMemoryAllocation ? GRIS_ERR_OUT_OF_MEMORY : GRIS_ERR_CUDA,
                                std::string("reuse pass buffers: ") + cudaGetErrorString(e));
        }
    }
    int form = ctx_path_form(ctx);
    WaveLaunch wl = ctx_wave_launch(ctx);
    guide::GuideDevice gd{};
    int train = 0;
    if (b->guide) {
        if (form != GRIS_PATH_WAVEFRONT) return ctx_fail(ctx, GRIS_ERR_UNSUPPORTED, "guided batches need the wavefront path form");
        gd = guide_device(b->guide);
        train = guide_config(b->guide).train ? 1 : 0;
    }
    BatchShape sh = fill_view_table(views.data(), (int)b->n, b->hViews[k], ctx_counters(ctx), ctx_count_work(ctx),
                                    b->guide ? b->wave.gPrimOut : nullptr, b->guide ? gd.mix : 0.0f);
    if (ctx_graphs(ctx)) {
        GrisBatch::Graph& g = b->graph[k];
        if (!g.exec || g.pathForm != form || g.maxDepth != sh.maxDepth || g.pixels != sh.pixels || g.tiles != sh.tiles ||
            g.trace != wl.traceBlocksPerSM || g.shade != wl.shadeBlocksPerSM || g.refill != wl.refill ||
            g.countWork != ctx_count_work(ctx) || g.pairwise != sh.pairwise ||
            g.guide != b->guide || g.train != train) {
            if (g.exec) { cudaGraphExecDestroy(g.exec); g.exec = nullptr; }
            cudaGraph_t graph = nullptr;
            e = cudaStreamBeginCapture(st, cudaStreamCaptureModeThreadLocal);
            if (e == cudaSuccess) {
                cudaError_t ee = enqueue_batch(sh, b->dViews, b->hViews[k], b->wave, ctx_counters(ctx), ctx_count_work(ctx),
                                               nullptr, st, form, 15, wl, b->guide ? &gd : nullptr);
                if (ee == cudaSuccess && train) ee = guide_train_frame(b->guide, st);
                e = cudaStreamEndCapture(st, &graph);
                if (e == cudaSuccess) e = ee;
            }
            if (e == cudaSuccess) e = cudaGraphInstantiate(&g.exec, graph, 0);
            if (graph) cudaGraphDestroy(graph);
            if (e != cudaSuccess) return ctx_fail(ctx, GRIS_ERR_CUDA, std::string("graph capture: ") + cudaGetErrorString(e));
            g.pathForm = form; g.maxDepth = sh.maxDepth; g.pixels = sh.pixels; g.tiles = sh.tiles;
            g.trace = wl.traceBlocksPerSM; g.shade = wl.shadeBlocksPerSM; g.refill = wl.refill; g.countWork = ctx_count_work(ctx);
            g.guide = b->guide; g.train = train; g.pairwise = sh.pairwise;
        }
        e = cudaGraphLaunch(g.exec, st);
    } else {
        /* eager launches: the side streams as in the captured graph unless per-kernel profiling
         * wants every kernel in order on one stream */
        e = enqueue_batch(sh, b->dViews, b->hViews[k], b->wave, ctx_counters(ctx), ctx_count_work(ctx),
                          ctx_profiling(ctx) ? ctx_timer(ctx) : nullptr, st, form, 15, wl, b->guide ? &gd : nullptr);
        if (e == cudaSuccess && train) {
            KernelTimer* tm = ctx_timer(ctx);
            if (tm) tm->mark(10, true, st);
            e = guide_train_frame(b->guide, st);
            if (tm) tm->mark(10, false, st);
        }
    }
    if (e == cudaSuccess) e = cudaEventRecord(b->staged[k], st);
    if (e != cudaSuccess) return ctx_fail(ctx, GRIS_ERR_CUDA, std::string("grisBatchRender: ") + cudaGetErrorString(e));
    b->stage ^= 1;
    b->next ^= 1;
    return GRIS_OK;
}

int grisBatchGetBuffer(const GrisBatch* b, uint32_t view, int which, int slot, void** devPtr, size_t* bytes) {
    if (!b || !devPtr || (view >= b->n && view != GRIS_BATCH_ALL_VIEWS) || slot < 0 || slot > 1)
        return GRIS_ERR_INVALID_ARGUMENT;
    int j = (b->next ^ 1) ^ slot;
    const bool all = view == GRIS_BATCH_ALL_VIEWS;
    size_t n = all ? (size_t)b->pixels : (size_t)b->w[view] * b->h[view];
    uint64_t o = all ? 0 : b->base[view];
    void* p = nullptr;
    size_t sz = 0;
    switch (which) {
    case 0: p = b->depthNormal[j] + o * 4; sz = n * 16; break;
    case 1: p = b->albedoMatId[j] + o * 2; sz = n * 8; break;
    case 2: p = b->motion + o * 2; sz = n * 4; break;
    case 3: p = b->resv[j] + o; sz = n * sizeof(GrisReservoir); break;
    case 4: p = b->temp + o; sz = n * sizeof(GrisReservoir); break;
    case 5: p = b->output + o * 4; sz = n * 16; break;
    default: return GRIS_ERR_INVALID_ARGUMENT;
    }
    *devPtr = p;
    if (bytes) *bytes = sz;
    return GRIS_OK;
}

int grisBatchSetGuide(GrisBatch* b, GrisGuide* g) {
    if (!b) return GRIS_ERR_INVALID_ARGUMENT;
    GrisContext* ctx = b->ctx;
    cudaSetDevice(ctx_device(ctx));
    if (g && !b->guideBlock) {
        size_t P = (size_t)b->pixels;
        auto up = [](size_t n) { return (n + 255) & ~(size_t)255; };
        size_t bytes = up(P * 4) + up(P * 9 * 4) + up(P * guide::kRaw * 4) + up(P * 18 * 4) + up(P * 9 * 4) +
                       up(P * guide::kRaw * 4) + 256;
        cudaError_t e = cudaMalloc(&b->guideBlock, bytes);
        if (e != cudaSuccess) { b->guideBlock = nullptr; return ctx_fail(ctx, GRIS_ERR_OUT_OF_MEMORY, "guided batch buffers"); }
        char* p = (char*)b->guideBlock;
        b->wave.postQueue = (uint32_t*)p; p += up(P * 4);
        b->wave.gFeat = (float*)p; p += up(P * 9 * 4);
        b->wave.gOut = (float*)p; p += up(P * guide::kRaw * 4);
        b->wave.gRec = (float*)p; p += up(P * 18 * 4);
        b->wave.gPrimFeat = (float*)p; p += up(P * 9 * 4);
        b->wave.gPrimOut = (float*)p; p += up(P * guide::kRaw * 4);
        b->wave.gFrame = (uint32_t*)p;
        e = cudaMemsetAsync(b->wave.gFrame, 0, 256, ctx_stream(ctx));
        if (e == cudaSuccess) e = cudaStreamSynchronize(ctx_stream(ctx));
        if (e != cudaSuccess) return ctx_fail(ctx, GRIS_ERR_CUDA, std::string("guided batch buffers: ") + cudaGetErrorString(e));
    }
    b->guide = g;
    return GRIS_OK;
}

int grisBatchAutotune(GrisContext* ctx, GrisBatch* b, const GrisCamera* cams, const GrisCamera* prevCams,
                      const GrisSettings* settings, int frames, GrisTuneResult* out) {
    if (!ctx || !b || !out || frames < 1) return ctx_fail(ctx, GRIS_ERR_INVALID_ARGUMENT, "bad autotune request");
    cudaSetDevice(ctx_device(ctx));
    struct Cand { int form, trace, shade, refill; };
    std::vector<Cand> cands = {{GRIS_PATH_MEGAKERNEL, 16, 8, 0}};
    for (int t : {8, 16, 32})
        for (int sh : {4, 8, 16}) cands.push_back({GRIS_PATH_WAVEFRONT, t, sh, 0});
    for (int t : {4, 8, 16}) cands.push_back({GRIS_PATH_WAVEFRONT, t, 16, 1});
    memset(out, 0, sizeof(*out));
    cudaStream_t st = ctx_stream(ctx);
    cudaEvent_t e0, e1;
    cudaEventCreate(&e0);
    cudaEventCreate(&e1);
    int savedForm = ctx_path_form(ctx);
    WaveLaunch savedWl = ctx_wave_launch(ctx);
    double best = 1e30;
    int bestI = 0;
    int rc = GRIS_OK;
    for (size_t i = 0; i < cands.size() && i < 16 && rc == GRIS_OK; i++) {
        WaveLaunch wl;
        wl.traceBlocksPerSM = cands[i].trace;
        wl.shadeBlocksPerSM = cands[i].shade;
        wl.refill = cands[i].refill;
        ctx_set_tuning(ctx, cands[i].form, wl);
        rc = grisBatchRender(ctx, b, cams, prevCams, settings);   /* warm-up (and graph capture) */
        cudaEventRecord(e0, st);
        for (int f = 0; f < frames && rc == GRIS_OK; f++) rc = grisBatchRender(ctx, b, cams, prevCams, settings);
        cudaEventRecord(e1, st);
        cudaEventSynchronize(e1);
        float ms = 0.0f;
        cudaEventElapsedTime(&ms, e0, e1);
        out->candidateMs[i] = ms / frames;
        out->candidates = (int)i + 1;
        if (ms / frames < best) { best = ms / frames; bestI = (int)i; }
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    if (rc != GRIS_OK) { ctx_set_tuning(ctx, savedForm, savedWl); return rc; }
    WaveLaunch wl;
    wl.traceBlocksPerSM = cands[bestI].trace;
    wl.shadeBlocksPerSM = cands[bestI].shade;
    wl.refill = cands[bestI].refill;
    ctx_set_tuning(ctx, cands[bestI].form, wl);
    out->pathForm = cands[bestI].form;
    out->refill = wl.refill;
    out->traceBlocksPerSM = wl.traceBlocksPerSM;
    out->shadeBlocksPerSM = wl.shadeBlocksPerSM;
    out->msPerFrame = best;
    return GRIS_OK;
}

int grisBatchDownload(GrisContext* ctx, const GrisBatch* b, uint32_t view, int which, int slot, void* host, size_t bytes) {
    void* p = nullptr;
    size_t sz = 0;
    if (!ctx || !host || grisBatchGetBuffer(b, view, which, slot, &p, &sz) != GRIS_OK || bytes != sz)
        return ctx_fail(ctx, GRIS_ERR_INVALID_ARGUMENT, "bad download request");
    cudaSetDevice(ctx_device(ctx));
    cudaError_t e = cudaMemcpyAsync(host, p, sz, cudaMemcpyDeviceToHost, ctx_stream(ctx));
    if (e == cudaSuccess) e = cudaStreamSynchronize(ctx_stream(ctx));
    if (e != cudaSuccess) return ctx_fail(ctx, GRIS_ERR_CUDA, std::string("grisBatchDownload: ") + cudaGetErrorString(e));
    return GRIS_OK;
}

int grisBatchDownloadAsync(GrisContext* ctx, const GrisBatch* b, uint32_t view, int which, int slot, void* host,
                           size_t bytes) {
    void* p = nullptr;
    size_t sz = 0;
    if (!ctx || !host || grisBatchGetBuffer(b, view, which, slot, &p, &sz) != GRIS_OK || bytes != sz)
        return ctx_fail(ctx, GRIS_ERR_INVALID_ARGUMENT, "bad download request");
    return ctx_download_async(ctx, p, host, sz, "grisBatchDownloadAsync");
}

}  /* extern "C" */
