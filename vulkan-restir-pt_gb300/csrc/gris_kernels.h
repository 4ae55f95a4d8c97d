/*
 * gris_kernels.h — host-side launch interface of the grisrt kernels.
 */
#ifndef GRISRT_GRIS_KERNELS_H
#define GRISRT_GRIS_KERNELS_H

#include <cuda_runtime.h>
#include <stdint.h>

#include "../../include/grisrt.h"
#include "guide_kernels.h"

namespace grisrt {

/* Device pointers of an uploaded scene (DeviceScene's buffers + the BVH). */
struct DeviceSceneView {
    const GrisMeshVertex* vertices; uint64_t nVertices;
    const uint32_t* indices; uint64_t nIndices;
    const GrisObjectInstance* instances; uint64_t nInstances;
    const GrisMaterial* materials; uint64_t nMaterials;
    const int32_t* matIndices; uint64_t nMatIndices;
    const GrisTriangleLight* lights; uint64_t nLights;
    const GrisLightTableEntry* table; uint64_t nTable;
    const uint32_t* nodes;
    const float* tris;
    float boxMin[3], boxMax[3];   /* bounds of the world-space triangles */
};

/* Receives a mark before (begin = true) and after each kernel launch, on the launch stream. */
struct KernelTimer {
    virtual void mark(int kernel, bool begin, cudaStream_t stream) = 0;
    virtual ~KernelTimer() {}
};

/* kernels: 0 G-buffer, 1 path trace, 2 temporal reuse, 3 spatial reuse */
cudaError_t launch_gbuffer(const DeviceSceneView& scene, const GrisGBufferBindings& b, const GrisCamera& cam,
                           unsigned long long* counters, int countWork, KernelTimer* timer, cudaStream_t stream);
cudaError_t launch_gris(const DeviceSceneView& scene, const GrisPassBindings& b, const GrisCamera& cam,
                        const GrisCamera& prevCam, const GrisSettings& set, int passes, unsigned long long* counters,
                        int countWork, KernelTimer* timer, cudaStream_t stream, int launchMode = GRIS_LAUNCH_PERSISTENT);
/* ReSTIR DI (TestReSTIR::render): passes bit 0 candidates, bit 1 temporal, bit 2 spatial */
/* split: scratch of di_split_bytes_per_pixel() * splitPixels + 256 bytes for the candidates and
 * spatial passes in three launches (null or too small: their single kernels). side: a second
 * stream and two events of the caller's, on which the candidates pass walks its shadow queries
 * beside its closest-hit queries (null, or a kernel timer: both on `stream`, in order) */
struct DISide {
    cudaStream_t aux;
    cudaEvent_t evFork, evJoin;
};
cudaError_t launch_di(const DeviceSceneView& scene, const GrisDIBindings& b, const GrisCamera& cam,
                      const GrisCamera& prevCam, const GrisDISettings& set, int passes, unsigned long long* counters,
                      int countWork, KernelTimer* timer, cudaStream_t stream, void* split = nullptr,
                      uint64_t splitPixels = 0, const DISide* side = nullptr);
size_t di_split_bytes_per_pixel();
/* presentation pass (post_proc.frag): composition, tone mapping, gamma, UNORM8 */
cudaError_t launch_post(const GrisPostBindings& b, const GrisPostSettings& set, cudaStream_t stream);
/* converged image: FP64 sums of independent paths per pixel; relMSE / MSE reduction */
cudaError_t launch_converged(const DeviceSceneView& scene, const GrisConvergedBindings& b, const GrisCamera& cam,
                             const GrisSettings& set, uint32_t sppBegin, uint32_t sppCount, int estimator,
                             unsigned long long* counters, cudaStream_t stream);
cudaError_t launch_relmse(const float* image, const double* refSum, double refScale, uint64_t pixels, double eps,
                          double* scratch, cudaStream_t stream);
size_t relmse_scratch_doubles();
/* One view of a batch for one frame: its scene, this frame's buffers (ping-pong resolved),
 * cameras and settings. */
struct BatchView {
    DeviceSceneView scene;
    GrisPassBindings b;
    GrisGBufferBindings gb;
    GrisCamera cam, prev;
    GrisSettings set;
};

/* Device buffers of the reuse passes' three-launch form (prepare, visibility walk, finish) for up
 * to `capacity` pixels with `slots` neighbour slots each; slots = 0: not allocated, the reuse
 * passes then run as one per-pixel kernel each. One allocation (`block`, reuse_bytes bytes) carved
 * by reuse_carve. */
struct ReuseBuffers {
    void* block;
    void* pa;            /* float4 per slot */
    void* pb;            /* float4 per slot */
    uint32_t* pn;        /* per slot */
    unsigned char* ps;   /* per slot */
    void* q;             /* 32 B per query, a query per slot at most */
    uint32_t* counts;    /* 4 words */
    uint32_t slots;
    uint64_t capacity;
};
constexpr uint32_t kReuseMaxSlots = 16;   /* views with more spatial neighbours use the per-pixel kernels */
size_t reuse_bytes(uint64_t pixels, uint32_t slots);
void reuse_carve(ReuseBuffers& r, void* block, uint64_t pixels, uint32_t slots);

/* Device buffers of the wavefront path tracer, for up to `capacity` paths (pixels of a batch). */
/* bytes per path of the wavefront's path record and NEE record */
constexpr size_t kWaveStateBytes = 256, kWaveNeeBytes = 96;

struct WaveBuffers {
    void* state;
    void* nee;
    void* hit;
    unsigned char* blocked;
    uint32_t* queue[2];
    uint32_t* shadowQueue;
    void* ray;          /* 32 B per path: the next closest-hit ray */
    uint32_t* counts;   /* 1536 words */
    uint64_t capacity;
    /* two more streams and their events (null: the frame's kernels run in order on one stream):
     * aux for a bounce's shadow queries beside the next bounce's closest hits, aux2 for the
     * temporal pass's shifts and visibility walk beside the path tracer */
    cudaStream_t aux, aux2;
    cudaEvent_t evFork, evJoin, evTemporal, evTemporalDone;
    /* guided batches only (null otherwise): post queue, guide inputs / outputs per guided
     * vertex, training record per path, frame state (4 words) */
    uint32_t* postQueue;
    float* gFeat;
    float* gOut;
    float* gRec;
    uint32_t* gFrame;
    float* gPrimFeat;   /* the guide's inputs / raw outputs at every path's primary vertex */
    float* gPrimOut;
    ReuseBuffers reuse;  /* the reuse passes' three-launch form (slots = 0: not used) */
};
/* the side streams and events of WaveBuffers (destroy waits for the streams' work) */
cudaError_t wave_streams_create(WaveBuffers& wb);
void wave_streams_destroy(WaveBuffers& wb);
size_t view_entry_bytes();

/* Grid sizes of the wavefront kernels, in blocks of 128 threads per SM. */
struct WaveLaunch {
    int traceBlocksPerSM = 16;
    int shadeBlocksPerSM = 8;
    int refill = 0;   /* 1: the resident traversal kernels (lanes take new rays while others walk) */
};

struct BatchShape {
    int n;
    uint32_t tiles, pixels;
    int maxDepth;
    bool pairwise = false;   /* some view uses the pairwise MIS weights */
    uint32_t maxNeighbours = 0;   /* largest spatialNeighbors of the views */
};

/* Writes the view table of a frame into hViews (pinned host memory). */
BatchShape fill_view_table(const BatchView* views, int n, void* hViews, unsigned long long* counters, int countWork,
                           const float* gPrim = nullptr, float gMix = 0.0f);
/* Enqueues one batch frame: copy of the view table, then the kernels. passes: bit 3 G-buffer,
 * bit 0 path trace, bit 1 temporal, bit 2 spatial. pathForm: GRIS_PATH_MEGAKERNEL or
 * GRIS_PATH_WAVEFRONT. Only stream operations: it can be captured into a CUDA graph. */
cudaError_t enqueue_batch(const BatchShape& sh, void* dViews, const void* hViews, const WaveBuffers& wb,
                          unsigned long long* counters, int countWork, KernelTimer* timer, cudaStream_t stream,
                          int pathForm, int passes, const WaveLaunch& wl,
                          const guide::GuideDevice* guide = nullptr);
cudaError_t launch_batch(const BatchView* views, int n, void* dViews, void* hViews, const WaveBuffers& wb,
                         unsigned long long* counters, int countWork, KernelTimer* timer, cudaStream_t stream,
                         int pathForm, int passes, const WaveLaunch& wl);

cudaError_t launch_debug_trace(const uint32_t* nodes, const float* tris, const float* rays, uint64_t n, int anyHit,
                               float* hitTUV, uint32_t* hitInst, uint32_t* hitTri, unsigned long long* counters,
                               cudaStream_t stream);

}  // namespace grisrt

#endif
