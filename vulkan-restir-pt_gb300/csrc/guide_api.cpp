/* guide_api.cpp — the guiding network's C ABI: creation (Glorot-uniform initialisation from a
 * seed), parameter upload / download, inference, the loss gradient and Adam steps on a batch
 * of samples, and the training-record buffers the path tracer fills while it renders. */
#include <cuda_runtime.h>
#include <math.h>
#include <string.h>

#include <string>
#include <vector>

#include "../../include/grisrt.h"
#include "grisrt_internal.h"
#include "guide.cuh"
#include "guide_kernels.h"

using namespace grisrt;

#define GUIDE_CK(ctx, call)                                                                                  \
    do {                                                                                                     \
        cudaError_t e_ = (call);                                                                             \
        if (e_ != cudaSuccess) return ctx_fail(ctx, GRIS_ERR_CUDA, std::string(#call ": ") + cudaGetErrorString(e_)); \
    } while (0)

struct GrisGuide {
    GrisContext* ctx = nullptr;
    int device = 0;
    GrisGuideConfig cfg{};
    void* block = nullptr;          /* one allocation for everything below */
    float* params = nullptr;        /* FP32 master parameters (flat: W0 b0 ... W4 b4) */
    float* grad = nullptr;
    float* m = nullptr;
    float* v = nullptr;
    __nv_bfloat16* wPacked = nullptr;
    float* bias = nullptr;
    uint32_t* step = nullptr;
    float* invSum = nullptr;
    /* training batch: records gathered from the rendered paths */
    float* tFeat = nullptr;
    float* tDir = nullptr;
    float* tWeight = nullptr;
    uint32_t* tCount = nullptr;
    uint32_t cap = 0;
};

namespace grisrt {
guide::GuideDevice guide_device(const GrisGuide* g) {
    guide::GuideDevice d;
    d.wPacked = g->wPacked; d.bias = g->bias;
    d.tFeat = g->tFeat; d.tDir = g->tDir; d.tWeight = g->tWeight; d.tCount = g->tCount; d.cap = g->cap;
    d.tensorCores = g->cfg.tensorCores != 0;
    d.mix = g->cfg.mix;
    return d;
}
const GrisGuideConfig& guide_config(const GrisGuide* g) { return g->cfg; }

/* The training steps of one frame on the gathered records (enqueued; capturable). */
cudaError_t guide_train_frame(GrisGuide* g, cudaStream_t st) {
    const uint32_t steps = g->cfg.stepsPerFrame ? g->cfg.stepsPerFrame : 1u;
    const uint32_t per = g->cap / steps;
    for (uint32_t s = 0; s < steps; s++) {
        guide::GradArgs a;
        a.wPacked = g->wPacked; a.bias = g->bias;
        a.feat = g->tFeat + (size_t)s * per * 9;
        a.dir = g->tDir + (size_t)s * per * 3;
        a.weight = g->tWeight + (size_t)s * per;
        a.count = g->tCount;
        a.base = s * per;
        a.n = per;
        a.invWeightSum = g->invSum;
        a.grad = g->grad;
        a.tensorCores = g->cfg.trainKernel == 0u;
        a.err = ctx_counters(g->ctx) + GRIS_COUNTER_ERROR;
        cudaError_t e = guide::launch_grad(a, st);
        if (e != cudaSuccess) return e;
        e = guide::launch_adam(g->params, g->grad, g->m, g->v, g->step, g->cfg.learningRate, st);
        if (e != cudaSuccess) return e;
        e = guide::launch_pack(g->params, g->wPacked, g->bias, st);
        if (e != cudaSuccess) return e;
    }
    return cudaSuccess;
}
}  // namespace grisrt

static void glorot(uint64_t seed, std::vector<float>& p) {
    uint64_t s = seed * 0x9e3779b97f4a7c15ull + 0x632be59bd9b4e019ull;
    auto next = [&]() {
        uint64_t z = (s += 0x9e3779b97f4a7c15ull);
        z = (z ^ (z >> 30)) * 0xbf58476d1ce4e5b9ull;
        z = (z ^ (z >> 27)) * 0x94d049bb133111ebull;
        return (double)((z ^ (z >> 31)) >> 11) * (1.0 / 9007199254740992.0);
    };
    p.assign(guide::kParams, 0.0f);
    for (int l = 0; l < guide::kLayers; l++) {
        int in = guide::layer_in(l), out = guide::layer_out(l);
        double lim = sqrt(6.0 / (in + out));
        for (int i = 0; i < in * out; i++) p[guide::param_w(l) + i] = (float)((2.0 * next() - 1.0) * lim);
    }
}

static int upload_params(GrisGuide* g, const float* host) {
    GrisContext* ctx = g->ctx;
    cudaStream_t st = ctx_stream(ctx);
    GUIDE_CK(ctx, cudaMemcpyAsync(g->params, host, guide::kParams * sizeof(float), cudaMemcpyHostToDevice, st));
    GUIDE_CK(ctx, cudaMemsetAsync(g->grad, 0, 3 * guide::kParams * sizeof(float), st));   /* grad, m, v */
    GUIDE_CK(ctx, cudaMemsetAsync(g->step, 0, sizeof(uint32_t), st));
    GUIDE_CK(ctx, guide::launch_pack(g->params, g->wPacked, g->bias, st));
    GUIDE_CK(ctx, cudaStreamSynchronize(st));
    return GRIS_OK;
}

extern "C" {

int grisGuideCreate(GrisContext* ctx, const GrisGuideConfig* cfg, GrisGuide** out) {
    if (!ctx || !cfg || !out) return ctx_fail(ctx, GRIS_ERR_INVALID_ARGUMENT, "null argument");
    if (!(cfg->mix >= 0.0f && cfg->mix < 1.0f) || !(cfg->learningRate >= 0.0f) || cfg->samplesPerFrame > (1u << 24))
        return ctx_fail(ctx, GRIS_ERR_INVALID_ARGUMENT, "bad guide configuration");
    cudaSetDevice(ctx_device(ctx));
    GrisGuide* g = new GrisGuide();
    g->ctx = ctx;
    g->cfg = *cfg;
    if (g->cfg.stepsPerFrame == 0) g->cfg.stepsPerFrame = 1;
    g->cap = (cfg->samplesPerFrame / g->cfg.stepsPerFrame) * g->cfg.stepsPerFrame;
    const size_t P = guide::kParams;
    /* one allocation: each part at a 256-byte boundary */
    auto up = [](size_t n) { return (n + 255) & ~(size_t)255; };
    const size_t parts[] = {P * 4, P * 4 * 3, (size_t)guide::kPackedW * 2, (size_t)guide::kBiases * 4, 16, 16, 16,
                            (size_t)g->cap * 9 * 4, (size_t)g->cap * 3 * 4, (size_t)g->cap * 4};
    size_t bytes = 0;
    for (size_t n : parts) bytes += up(n);
    if (cudaMalloc(&g->block, bytes) != cudaSuccess) {
        delete g;
        return ctx_fail(ctx, GRIS_ERR_OUT_OF_MEMORY, "guide allocation");
    }
    char* p = (char*)g->block;
    int part = 0;
    auto take = [&]() { char* r = p; p += up(parts[part++]); return r; };
    g->params = (float*)take();
    g->grad = (float*)take();   /* grad, m, v contiguous */
    g->m = g->grad + P;
    g->v = g->grad + 2 * P;
    g->wPacked = (__nv_bfloat16*)take();
    g->bias = (float*)take();
    g->step = (uint32_t*)take();
    g->invSum = (float*)take();
    g->tCount = (uint32_t*)take();
    g->tFeat = (float*)take();
    g->tDir = (float*)take();
    g->tWeight = (float*)take();
    g->device = ctx_device(ctx);
    std::vector<float> host;
    glorot(cfg->seed, host);
    int rc = upload_params(g, host.data());
    if (rc == GRIS_OK) {
        cudaMemsetAsync(g->tCount, 0, 16, ctx_stream(ctx));
        if (g->cap) {
            cudaMemsetAsync(g->tWeight, 0, (size_t)g->cap * 4, ctx_stream(ctx));
            cudaMemsetAsync(g->tFeat, 0, (size_t)g->cap * 9 * 4, ctx_stream(ctx));
            cudaMemsetAsync(g->tDir, 0, (size_t)g->cap * 3 * 4, ctx_stream(ctx));
        }
        if (cudaStreamSynchronize(ctx_stream(ctx)) != cudaSuccess) rc = ctx_fail(ctx, GRIS_ERR_CUDA, "guide init");
    }
    if (rc != GRIS_OK) {
        cudaFree(g->block);
        delete g;
        return rc;
    }
    *out = g;
    return GRIS_OK;
}

int grisGuideDestroy(GrisGuide* g) {
    if (!g) return GRIS_ERR_INVALID_ARGUMENT;
    cudaSetDevice(g->device);
    cudaFree(g->block);   /* waits for the device's work that may still use it */
    delete g;
    return GRIS_OK;
}

int grisGuideParamCount(void) { return guide::kParams; }

int grisGuideSetTraining(GrisGuide* g, int enable) {
    if (!g) return GRIS_ERR_INVALID_ARGUMENT;
    g->cfg.train = enable != 0;
    return GRIS_OK;
}

int grisGuideSetParams(GrisGuide* g, const float* params, size_t count) {
    if (!g || !params || count != (size_t)guide::kParams) return GRIS_ERR_INVALID_ARGUMENT;
    cudaSetDevice(ctx_device(g->ctx));
    return upload_params(g, params);
}

int grisGuideGetParams(GrisGuide* g, float* params, size_t count) {
    if (!g || !params || count != (size_t)guide::kParams) return GRIS_ERR_INVALID_ARGUMENT;
    GrisContext* ctx = g->ctx;
    cudaSetDevice(ctx_device(ctx));
    GUIDE_CK(ctx, cudaMemcpyAsync(params, g->params, count * sizeof(float), cudaMemcpyDeviceToHost, ctx_stream(ctx)));
    GUIDE_CK(ctx, cudaStreamSynchronize(ctx_stream(ctx)));
    return GRIS_OK;
}

int grisGuideForward(GrisContext* ctx, GrisGuide* g, const float* feat, uint32_t n, float* out) {
    if (!ctx || !g || (n && (!feat || !out))) return ctx_fail(ctx, GRIS_ERR_INVALID_ARGUMENT, "bad guide forward");
    if (n == 0) return GRIS_OK;
    cudaSetDevice(ctx_device(ctx));
    guide::FwdArgs a;
    a.wPacked = g->wPacked; a.bias = g->bias; a.feat = feat; a.count = nullptr; a.n = n; a.out = out;
    a.tensorCores = g->cfg.tensorCores != 0; a.err = ctx_counters(ctx) + GRIS_COUNTER_ERROR;
    GUIDE_CK(ctx, guide::launch_forward(a, ctx_stream(ctx)));
    return GRIS_OK;
}

int grisDebugGuideForwardStall(GrisContext* ctx, GrisGuide* g, const float* feat, uint32_t n, float* out) {
    if (!ctx || !g || !n || !feat || !out) return ctx_fail(ctx, GRIS_ERR_INVALID_ARGUMENT, "bad guide forward");
    cudaSetDevice(ctx_device(ctx));
    guide::FwdArgs a;
    a.wPacked = g->wPacked; a.bias = g->bias; a.feat = feat; a.count = nullptr; a.n = n; a.out = out;
    a.tensorCores = 1; a.err = ctx_counters(ctx) + GRIS_COUNTER_ERROR; a.withholdCommit = 1;
    GUIDE_CK(ctx, guide::launch_forward(a, ctx_stream(ctx)));
    return GRIS_OK;
}

int grisGuideGradient(GrisContext* ctx, GrisGuide* g, const float* feat, const float* dir, const float* weight, uint32_t n,
                      float* gradOut) {
    if (!ctx || !g || !gradOut || (n && (!feat || !dir || !weight)))
        return ctx_fail(ctx, GRIS_ERR_INVALID_ARGUMENT, "bad guide gradient");
    cudaSetDevice(ctx_device(ctx));
    cudaStream_t st = ctx_stream(ctx);
    GUIDE_CK(ctx, cudaMemsetAsync(gradOut, 0, guide::kParams * sizeof(float), st));
    if (n == 0) return GRIS_OK;
    guide::GradArgs a;
    a.wPacked = g->wPacked; a.bias = g->bias; a.feat = feat; a.dir = dir; a.weight = weight;
    a.count = nullptr; a.base = 0; a.n = n; a.invWeightSum = g->invSum; a.grad = gradOut;
    a.tensorCores = g->cfg.trainKernel == 0u; a.err = ctx_counters(ctx) + GRIS_COUNTER_ERROR;
    GUIDE_CK(ctx, guide::launch_grad(a, st));
    return GRIS_OK;
}

int grisGuideTrainStep(GrisContext* ctx, GrisGuide* g, const float* feat, const float* dir, const float* weight, uint32_t n) {
    if (!ctx || !g || (n && (!feat || !dir || !weight))) return ctx_fail(ctx, GRIS_ERR_INVALID_ARGUMENT, "bad guide step");
    cudaSetDevice(ctx_device(ctx));
    cudaStream_t st = ctx_stream(ctx);
    if (n) {
        guide::GradArgs a;
        a.wPacked = g->wPacked; a.bias = g->bias; a.feat = feat; a.dir = dir; a.weight = weight;
        a.count = nullptr; a.base = 0; a.n = n; a.invWeightSum = g->invSum; a.grad = g->grad;
        a.tensorCores = g->cfg.trainKernel == 0u; a.err = ctx_counters(ctx) + GRIS_COUNTER_ERROR;
        GUIDE_CK(ctx, guide::launch_grad(a, st));
    }
    GUIDE_CK(ctx, guide::launch_adam(g->params, g->grad, g->m, g->v, g->step, g->cfg.learningRate, st));
    GUIDE_CK(ctx, guide::launch_pack(g->params, g->wPacked, g->bias, st));
    return GRIS_OK;
}

}  // extern "C"
