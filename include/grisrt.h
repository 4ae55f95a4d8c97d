/*
 * grisrt.h — C ABI of the GB300-native ReSTIR PT (GRIS) pass.
 *
 * Drop-in boundary for the reference's GRISReSTIR pass (src/GRISReSTIR.h:24-26):
 *   GRISReSTIR::createPipeline(ShaderManager*, descLayouts)      -> grisCreate / grisSceneCreate
 *   GRISReSTIR::render(cmd, extent, DescriptorSetBindingMap)     -> grisPassRender (caller-owned
 *                                                                    device buffers, like the
 *                                                                    descriptor sets) or
 *                                                                    grisFrameRender (library-owned
 *                                                                    frame buffers with the
 *                                                                    renderer's ping-pong)
 * and for its input producers:
 *   GBufferPass::render (src/GBufferPass.cpp:22-55, raster)      -> grisPassGBuffer / grisFrameGBuffer
 *   DeviceScene ctor + createAccelerationStructure
 *     (src/Scene.cpp:324-330, 448-547)                           -> grisSceneCreate (8-wide BVH)
 *   Scene::buildLightDataStructure (src/Scene.cpp:309-322)       -> grisBuildLightTable
 *   Camera::update (src/Camera.cpp:78-98)                        -> grisCameraSetup
 *
 * Conventions: every call returns GRIS_OK (0) or a negative GRIS_ERR_* code and never
 * throws; grisGetError() gives the context's last message. Work is enqueued on the
 * context's CUDA stream and the call returns after enqueue; grisSync() waits. A context
 * is used by one host thread at a time. All structs below are the reference's std430
 * layouts, byte for byte (sizes are checked at compile time in the library).
 */
#ifndef GRISRT_H
#define GRISRT_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define GRIS_OK 0
#define GRIS_ERR_INVALID_ARGUMENT (-1)
#define GRIS_ERR_CUDA (-2)
#define GRIS_ERR_OUT_OF_MEMORY (-3)
#define GRIS_ERR_UNSUPPORTED (-4)
#define GRIS_ERR_DEVICE_FAULT (-5)   /* a kernel raised its error word: bit 0 the traversal stack limit,
                                        bit 1 a bounded tensor-core wait ran out, bit 2 the drain wait
                                        after it ran out too, bit 3 the wavefront's post() disagreed
                                        with the next ray shade() queued ahead of it */
#define GRIS_ERR_TOO_LARGE (-6)

/* ---------------------------------------------------------------- layouts */

/* reference: Material, src/shader/layouts.glsl:6-25 (RESTIR_PT_MATERIAL = 1, 32 B).
 * type: 1 Lambert, 2 MetallicWorkflow, 3 Metal, 4 Dielectric, 6 Fake (material.glsl:13-20). */
typedef struct GrisMaterial {
    float baseColor[3];
    uint32_t type;
    uint32_t textureIdx;     /* 0xffffffff: no texture (textures are not supported) */
    float metallic;
    float roughness;
    float ior;
} GrisMaterial;

/* reference: MeshVertex, layouts.glsl:53-58 (32 B) */
typedef struct GrisMeshVertex {
    float pos[3];
    float uvx;
    float norm[3];
    float uvy;
} GrisMeshVertex;

/* reference: ObjectInstance, layouts.glsl:60-72 (224 B). Matrices are column-major. */
typedef struct GrisObjectInstance {
    float transform[16];
    float transformInv[16];
    float transformInvT[16];
    float radiance[3];
    float pad0;
    uint32_t indexOffset;
    uint32_t indexCount;
    uint32_t matIndex;
    float pad2;
} GrisObjectInstance;

/* reference: TriangleLight, layouts.glsl:74-83 (64 B) */
typedef struct GrisTriangleLight {
    float v0[3]; float nx;
    float v1[3]; float ny;
    float v2[3]; float nz;
    float radiance[3]; float area;
} GrisTriangleLight;

/* reference: LightSampleTableElement, layouts.glsl:85-88 (8 B). Entry 0 = {sumPower, count};
 * entry i+1 = {prob, failId (1-based)} (src/util/AliasTable.h:26-71). */
typedef struct GrisLightTableEntry {
    float prob;
    uint32_t failId;
} GrisLightTableEntry;

/* reference: Camera, layouts.glsl:27-51 (352 B, the camera UBO element) */
typedef struct GrisCamera {
    float view[16];
    float proj[16];
    float projView[16];
    float lastProjView[16];
    float pos[3]; float FOV;
    float angle[3]; float nearZ;
    float front[3]; float farZ;
    float right[3]; float lensRadius;
    float up[3]; float focalDist;
    uint32_t filmSize[2];
    uint32_t frameIndex;     /* bit 31: clear flag (camera.glsl:6-7) */
    uint32_t seed;
} GrisCamera;

/* reference: Intersection, layouts.glsl:90-94 (16 B) */
typedef struct GrisIntersection {
    float bary[2];
    uint32_t instanceIdx;    /* 0: light instance; 0xffffffff: miss; 0xfffffffe: primary (bary = uv) */
    uint32_t triangleIdx;
} GrisIntersection;

/* reference: GRISPathSample + GRISReservoir, layouts.glsl:132-156 (96 B) */
typedef struct GrisReservoir {
    GrisIntersection rcIsec;
    float rcLi[3]; uint32_t rcRng;
    float rcWi[3]; uint32_t flags;   /* bits 0-7 rcVertexId, 8-15 pathLength, 16-23 rcVertexType */
    float pad[2]; float rcPrevSamplePdf; float rcJacobian;
    float F[3]; uint32_t primaryRng;
    float sampleCount;
    float resampleWeight;
    float contribWeight;
    float pad0;
} GrisReservoir;

/* reference: GRISReSTIR::Settings (src/GRISReSTIR.h:11-17, the 20-byte push constant) followed by
 * the constants the reference hard-codes, as parameters (defaults = reference values). */
typedef struct GrisSettings {
    uint32_t shiftType;         /* 0 Reconnection, 1 Replay, 2 Hybrid (GRISReSTIR.h:9) */
    float rrScale;              /* 1.0 */
    uint32_t temporalReuse;     /* bool */
    uint32_t spatialReuse;      /* bool */
    uint32_t cap;               /* M cap, 20 */
    uint32_t maxDepth;          /* MaxTracingDepth, gris_path_trace.glsl:46 (15) */
    uint32_t spatialNeighbors;  /* ResampleNum, gris_resample_spatial.glsl:65 (3) */
    float spatialRadius;        /* ResampleRadius in pixels, gris_resample_spatial.glsl:66 (20) */
    float envRadiance[3];       /* reserved, must be 0 (a miss ends the path, as in the reference) */
    uint32_t misWeights;        /* extension: 0 = the reference's merge (M-proportional weights); 1 = pairwise
                                   generalised balance heuristic (each reused sample and the canonical one are
                                   weighed against each other through shifts in both directions) */
    uint32_t reserved[4];
} GrisSettings;

/* Host-side scene arrays (what DeviceScene uploads, src/Scene.cpp:368-446). */
typedef struct GrisSceneDesc {
    const GrisMeshVertex* vertices; uint64_t vertexCount;
    const uint32_t* indices; uint64_t indexCount;
    const GrisObjectInstance* instances; uint64_t instanceCount;
    const GrisMaterial* materials; uint64_t materialCount;
    const int32_t* materialIndices; uint64_t materialIndexCount;   /* one per triangle: [indexOffset/3 + tri] */
    const GrisTriangleLight* lights; uint64_t lightCount;
    const GrisLightTableEntry* lightTable; uint64_t lightTableCount;  /* lightCount + 1 */
} GrisSceneDesc;

/* Device buffers of one GRISReSTIR::render call: descriptor set 2 of the reference
 * (layouts.glsl:180-195, bound per frame by Renderer.cpp:329-347). W x H pixels, row-major. */
typedef struct GrisPassBindings {
    uint32_t width, height;
    const float* depthNormal;        /* float4: depth, normal.xyz (RGBA32F) */
    const float* depthNormalPrev;
    const uint32_t* albedoMatId;     /* uint2: unorm4x8 albedo, matIndex<<16 | instanceIdx (RG32UI) */
    const uint32_t* albedoMatIdPrev;
    const uint16_t* motion;          /* half2 (RG16F) */
    GrisReservoir* reservoirThis;
    const GrisReservoir* reservoirPrev;
    GrisReservoir* reservoirTemp;
    float* output;                   /* float4 RGBA32F, running mean (indirect output) */
} GrisPassBindings;

/* Device buffers written by the G-buffer pass (GBufferPass.h:23-26 formats). */
typedef struct GrisGBufferBindings {
    uint32_t width, height;
    float* depthNormal;
    uint32_t* albedoMatId;
    uint16_t* motion;
} GrisGBufferBindings;

typedef struct GrisSceneStats {
    uint64_t triangleCount;          /* light + object triangles in the BVH */
    uint64_t nodeCount;              /* 8-wide nodes (80 B each) */
    uint64_t nodeBytes, triangleBytes;
    uint32_t maxDepth;               /* deepest 8-wide level */
    uint32_t reserved;
    double buildSeconds;
} GrisSceneStats;

/* Ray counters (device-side, exact): index 0 closest-hit rays, 1 shadow/visibility rays,
 * 2 G-buffer primary rays, 3 error word (0 = none). */
#define GRIS_COUNTER_CLOSEST 0
#define GRIS_COUNTER_SHADOW 1
#define GRIS_COUNTER_PRIMARY 2
#define GRIS_COUNTER_ERROR 3

typedef struct GrisContext GrisContext;
typedef struct GrisScene GrisScene;
typedef struct GrisFrame GrisFrame;
typedef struct GrisHostScene GrisHostScene;

/* ---------------------------------------------------------------- context */
int grisCreate(int device, GrisContext** out);
int grisDestroy(GrisContext* ctx);
const char* grisGetError(const GrisContext* ctx);
int grisSync(GrisContext* ctx);
void* grisGetStream(GrisContext* ctx);                    /* cudaStream_t */
int grisReadCounters(GrisContext* ctx, uint64_t out[4], int reset);
int grisGetVersion(void);
/* Per-kernel timing (CUDA events around every launch on the context stream while enabled).
 * Kernels: 0 G-buffer, 1 path trace, 2 temporal reuse, 3 spatial reuse + final shading. */
int grisSetProfiling(GrisContext* ctx, int enable);
int grisReadProfile(GrisContext* ctx, double msTotal[4], uint64_t launches[4], int reset);
/* Traversal work per kernel while enabled: BVH nodes intersected, triangles tested and
 * closest-hit rays (primary rays for the G-buffer); shadow rays are in grisReadCounters. */
int grisSetWorkCounting(GrisContext* ctx, int enable);
/* Launch form of the three GRIS passes: GRIS_LAUNCH_GRID (default: one thread per pixel of a
 * 16 x 8 tile) or GRIS_LAUNCH_PERSISTENT (resident warps take 16 x 16 pixel tiles and refill
 * idle lanes pixel by pixel). Results are identical; only speed differs. */
#define GRIS_LAUNCH_GRID 0
#define GRIS_LAUNCH_PERSISTENT 1
int grisSetLaunchMode(GrisContext* ctx, int mode);
int grisReadWorkCounters(GrisContext* ctx, uint64_t nodes[4], uint64_t tris[4], uint64_t closestRays[4], int reset);
/* Per-kernel profile with the wavefront stages on their own: slots 0-3 as grisReadProfile (slot 1
 * spans the whole path tracer), then the wavefront's begin, extension (closest hits), shading,
 * shadow and post stages, then the guide's inference and training, then the three ReSTIR DI
 * kernels, then the visibility walks of the temporal and the spatial pass (batches, where a pass
 * runs as prepare -> walk -> finish; slots 2 and 3 span the whole pass, walk included).
 * ms/launches while profiling is on; nodes/tris/rays while work counting is on, for the slots
 * that traverse (rays: closest-hit rays, shadow rays for the shadow stage and the walks). */
#define GRIS_PROFILE_SLOTS 16
#define GRIS_SLOT_WAVE_BEGIN 4
#define GRIS_SLOT_WAVE_EXTEND 5
#define GRIS_SLOT_WAVE_SHADE 6
#define GRIS_SLOT_WAVE_SHADOW 7
#define GRIS_SLOT_WAVE_POST 8
#define GRIS_SLOT_GUIDE_INFER 9     /* guided batches: the network's inference per level */
#define GRIS_SLOT_GUIDE_TRAIN 10    /* guided batches: the frame's training steps */
#define GRIS_SLOT_DI_CANDIDATES 11  /* ReSTIR DI (rays: closest-hit and shadow rays together) */
#define GRIS_SLOT_DI_TEMPORAL 12
#define GRIS_SLOT_DI_SPATIAL 13
#define GRIS_SLOT_REUSE_VIS_TEMPORAL 14
#define GRIS_SLOT_REUSE_VIS_SPATIAL 15
typedef struct GrisKernelProfile {
    double ms;
    uint64_t launches;
    uint64_t nodes, tris, rays;
} GrisKernelProfile;
int grisReadKernelProfile(GrisContext* ctx, GrisKernelProfile out[GRIS_PROFILE_SLOTS], int reset);
/* No counterpart in the reference. The GPU's L2 read bandwidth in GB/s: a plain read kernel
 * (16-B loads that bypass L1) over a buffer of `bytes` (1 to 256 MiB; choose one that fits in L2)
 * read `reps` times per launch, best of five launches timed with CUDA events on the context's
 * stream. Allocates and frees its buffer. The roofline denominator of the kernels whose working
 * set (the BVH, the queues) stays in L2. */
int grisMeasureL2Bandwidth(GrisContext* ctx, uint64_t bytes, int reps, double* gbs);
size_t grisSizeof(int which);   /* 0 camera, 1 reservoir, 2 material, 3 vertex, 4 instance, 5 light, 6 table entry,
                                   7 settings, 8 DI reservoir, 9 DI settings */

/* ---------------------------------------------------------------- host helpers (no GPU) */
/* reference: DiscreteSampler1D::build, src/util/AliasTable.h:26-71 (table of n+1 entries). */
int grisBuildLightTable(const float* distribution, uint32_t n, GrisLightTableEntry* out);
/* reference: Camera::update (src/Camera.cpp:78-98) + the per-frame fields; angle in degrees
 * (yaw, pitch, roll), FOV in degrees; frameIndex = 0, seed = 0, lastProjView = projView. */
int grisCameraSetup(GrisCamera* cam, const float pos[3], const float angle[3], float fovDeg,
                    uint32_t width, uint32_t height);
/* reference: Camera::setDir (src/Camera.cpp:39-48) then update(). */
int grisCameraLookAt(GrisCamera* cam, const float pos[3], const float target[3], float fovDeg,
                     uint32_t width, uint32_t height);
/* Synthetic scenes. kind 0: closed box of 12 quads + ceiling quad light (radiance 15, 1/16 of the
 * ceiling area), Lambertian walls with albedo ~ U[0.2,0.8]^3; kind 1: fBm heightfield (gridN x gridN
 * vertices) + `spheres` instanced icospheres (subdivision 2) with radii log-uniform [0.1, 2], GGX
 * MetallicWorkflow materials, 4 quad lights; kind 2: glossy variant of kind 1 (roughness U[0.02,0.3],
 * 70% metallic, the lights facing up under white Lambertian bounce panels: no direct light on the
 * ground); kind 3: the kind 0 box furnished with `spheres`
 * instanced icospheres (320 triangles each, radii U[0.02,0.12], Lambertian or GGX). The camera for
 * frame f of the scene's orbit comes from grisHostSceneCamera. */
int grisHostSceneCreate(int kind, uint64_t seed, uint32_t gridN, uint32_t spheres, GrisHostScene** out);
int grisHostSceneDesc(const GrisHostScene* hs, GrisSceneDesc* out);
int grisHostSceneCamera(const GrisHostScene* hs, uint32_t frame, uint32_t frames, uint32_t width,
                        uint32_t height, GrisCamera* out);
int grisHostSceneDestroy(GrisHostScene* hs);
/* A scene in the reference's XML scene format (src/Scene.cpp:131-303) with Wavefront OBJ meshes:
 * integrator size, camera (position + angle or lookAt, fov), model instances with transforms,
 * light radiance (power over the light's area) and material overrides. errBuf (optional)
 * receives a message on failure. The camera comes from grisHostSceneCamera; the film size
 * given by the file from grisHostSceneFilmSize (0 x 0 when absent). */
int grisHostSceneLoad(const char* path, GrisHostScene** out, char* errBuf, size_t errLen);
int grisHostSceneFilmSize(const GrisHostScene* hs, uint32_t* width, uint32_t* height);

/* ---------------------------------------------------------------- converged image */
/* The converged image the GRIS path converges to, for quality measurement (relMSE): per pixel,
 * FP64 sums over independent samples of the path tracer (FP32 path arithmetic, as the GRIS
 * passes) from the pixel's G-buffer surface. Estimator GRIS_ESTIMATOR_CANDIDATES sums the
 * contributions the path tracer gives its reservoir stream as candidates (what ReSTIR PT's
 * output converges to); GRIS_ESTIMATOR_INDIRECT sums every NEE and light-hit contribution
 * (gi_naive.glsl:28-149's indirect illumination, with the GRIS path's MIS weights). Each
 * sample is clamped as clampColor before it is added. No counterpart in the reference's GRIS
 * pass; it replaces the reference's accumulation of many frames. */
#define GRIS_ESTIMATOR_CANDIDATES 0
#define GRIS_ESTIMATOR_INDIRECT 1
typedef struct GrisConvergedBindings {
    uint32_t width, height;
    const float* depthNormal;     /* the G-buffer of `cam` (grisPassGBuffer) */
    const uint32_t* albedoMatId;
    double* sum;                  /* 3 doubles per pixel, added to */
    double* sumSq;                /* optional (NULL): per-channel sums of squares, added to */
} GrisConvergedBindings;
/* Adds samples [sppBegin, sppBegin + sppCount) of every pixel (enqueued on the context stream). */
int grisConvergedAccumulate(GrisContext* ctx, const GrisScene* scene, const GrisConvergedBindings* b,
                            const GrisCamera* cam, const GrisSettings* settings, uint32_t sppBegin, uint32_t sppCount,
                            int estimator);
/* relMSE = mean over pixels and RGB of (image - ref)^2 / (ref^2 + eps) and MSE = mean of
 * (image - ref)^2 with ref = refSum * refScale (device pointers: RGBA32F image, 3 doubles per
 * pixel), reduced in FP64 on the device in a fixed order; waits and writes {relMSE, MSE}. */
int grisRelMSE(GrisContext* ctx, const float* image, const double* refSum, double refScale, uint64_t pixels,
               double eps, double out[2]);

/* ---------------------------------------------------------------- guiding network */
/* A directional proposal learned online: an MLP (80 -> 64 x4 -> 48, BF16 tensor-core matrix
 * products with FP32 accumulation) predicts per path vertex an 8-lobe von Mises-Fisher mixture
 * over world directions from the vertex position (12-frequency sin/cos encoding in the scene
 * box), shading normal and direction towards the previous vertex. A guided batch draws the
 * directions of the vertices after a path's reconnection vertex (which the hybrid shift never
 * replays) from the mixture with probability `mix` and from the BSDF otherwise, with the
 * one-sample MIS pdf of both, and trains the network on the radiance those paths carry
 * (Adam on -sum w log p / sum w, w = luminance(f cos L) / pdf). No counterpart in the
 * reference; guiding off reproduces the reference's sampling exactly. */
typedef struct GrisGuide GrisGuide;
typedef struct GrisGuideConfig {
    uint64_t seed;              /* Glorot-uniform initialisation */
    float learningRate;         /* Adam (1e-3) */
    float mix;                  /* probability of drawing from the guide at a guided vertex (0.5) */
    uint32_t samplesPerFrame;   /* training records gathered per frame (2^18) */
    uint32_t stepsPerFrame;     /* Adam steps per frame, each on samplesPerFrame / stepsPerFrame records */
    uint32_t train;             /* train while rendering */
    uint32_t tensorCores;       /* inference on the 5th-generation tensor cores (tcgen05, tensor-memory
                                   accumulators) when 1; warp-level mma.sync when 0 */
    uint32_t trainKernel;       /* the loss gradient (training): 0 tcgen05 — 128-record tiles, the weight
                                   gradients accumulated in tensor memory across the tiles — 1 warp-level
                                   mma.sync */
    uint32_t reserved;
} GrisGuideConfig;
int grisGuideCreate(GrisContext* ctx, const GrisGuideConfig* cfg, GrisGuide** out);
int grisGuideDestroy(GrisGuide* guide);
int grisGuideParamCount(void);                                   /* 20784 FP32 values: W0 b0 ... W4 b4 */
int grisGuideSetParams(GrisGuide* guide, const float* params, size_t count);   /* host; resets Adam */
int grisGuideGetParams(GrisGuide* guide, float* params, size_t count);         /* host */
int grisGuideSetTraining(GrisGuide* guide, int enable);
/* device pointers: feat 9 floats per sample (position in [0,1]^3, normal, wo), out 40 raw
 * outputs per sample (lobe j: direction 5j..5j+2, log-concentration 5j+3, logit 5j+4) */
int grisGuideForward(GrisContext* ctx, GrisGuide* guide, const float* feat, uint32_t n, float* out);
/* Test of the tcgen05 kernel's bounded waits: the inference with the completion of its matrix
 * products never signalled. Every wait gives up after its poll limit (well under a second), the
 * kernel raises bit 1 of the error word (grisSync then returns GRIS_ERR_DEVICE_FAULT), frees its
 * tensor memory and returns; the context stays usable (reset the word with grisReadCounters). */
int grisDebugGuideForwardStall(GrisContext* ctx, GrisGuide* guide, const float* feat, uint32_t n, float* out);
/* gradient of -sum_i weight_i log p(dir_i) / sum_i weight_i with respect to the FP32 parameters
 * (device; overwritten) at the current weights */
int grisGuideGradient(GrisContext* ctx, GrisGuide* guide, const float* feat, const float* dir, const float* weight,
                      uint32_t n, float* grad);
/* one Adam step on that loss */
int grisGuideTrainStep(GrisContext* ctx, GrisGuide* guide, const float* feat, const float* dir, const float* weight,
                       uint32_t n);

/* ---------------------------------------------------------------- scene */
/* Copies the arrays to the device and builds the 8-wide BVH over lights (instance 0) and every
 * instance's world-space triangles. */
int grisSceneCreate(GrisContext* ctx, const GrisSceneDesc* desc, GrisScene** out);
/* Synchronizes the context's stream, then frees the scene's device buffers. Work that reads the
 * scene on other streams (grisPassRenderNoAlloc on a caller's stream) must be synchronized by the
 * caller first. */
int grisSceneDestroy(GrisScene* scene);
int grisSceneGetStats(const GrisScene* scene, GrisSceneStats* out);
/* Builder check: closest-hit / any-hit of n rays (float[8] each: org.xyz, tmin, dir.xyz, tmax)
 * through the BVH on the host or on the device (dev pointers). hits: float[4] per ray
 * {t, u, v, bitcast instanceIdx} and uint triangleIdx in a second array. anyHit != 0: shadow query. */
/* Builder check without a GPU: builds the BVH on the host only (no context, no upload); the
 * result serves grisDebugTraceHost / grisSceneGetStats and is freed by grisSceneDestroy. */
int grisDebugHostSceneCreate(const GrisSceneDesc* desc, GrisScene** out);
int grisDebugTraceHost(const GrisScene* scene, const float* rays, uint64_t n, int anyHit,
                       float* hitTUV, uint32_t* hitInst, uint32_t* hitTri);
int grisDebugTraceDevice(GrisContext* ctx, const GrisScene* scene, const float* dRays, uint64_t n,
                         int anyHit, float* dHitTUV, uint32_t* dHitInst, uint32_t* dHitTri);

/* ---------------------------------------------------------------- passes on caller buffers */
int grisPassGBuffer(GrisContext* ctx, const GrisScene* scene, const GrisGBufferBindings* b,
                    const GrisCamera* cam);
/* GRISReSTIR::render: path trace -> temporal reuse -> spatial reuse + final shading. passes:
 * bit 0 path trace, bit 1 temporal, bit 2 spatial (7 = the full pass). */
int grisPassRender(GrisContext* ctx, const GrisScene* scene, const GrisPassBindings* b,
                   const GrisCamera* cam, const GrisCamera* prevCam, const GrisSettings* settings,
                   int passes);

/* No counterpart in the reference. The GRIS pass for callers that cannot allocate device memory
 * while they render (for example a host callback or plugin that must not call cudaMalloc, or a
 * process whose device allocator belongs to another framework). The temporary reservoirs that
 * carry the temporal result to the spatial kernel, and the ray-counter words, live in one static
 * device array of GRIS_NOALLOC_MAX_PIXELS x 96 B + 256 B (about 6.3 MB) that every GPU loading
 * the library holds until exit. The caller passes inputs and outputs as for grisPassRender, with
 * reservoirTemp = NULL, and a CUDA stream (NULL = the default stream); all three passes run.
 * Frames larger than GRIS_NOALLOC_MAX_PIXELS return GRIS_ERR_TOO_LARGE before any work. The
 * call allocates nothing: it clears the part of the array it uses (so its result equals
 * grisPassRender's with a zero-filled reservoirTemp), then launches. The first call on a device
 * looks up the array's device address (cudaGetSymbolAddress, with that device current); make
 * that first call before any stream capture. Every call shares the one array: calls that overlap
 * on the GPU (other streams, other threads) race on it. The call makes the scene's device current
 * for its launches and gives the caller's current device back before it returns. Errors the
 * kernels raise on the device (bit 0: the traversal stack limit) accumulate in the array's error
 * word across calls; grisNoAllocReadError reads and clears it. The scene must outlive the work:
 * synchronize `stream` before grisSceneDestroy. */
#define GRIS_NOALLOC_MAX_PIXELS 65536
int grisPassRenderNoAlloc(const GrisScene* scene, const GrisPassBindings* b, const GrisCamera* cam,
                          const GrisCamera* prevCam, const GrisSettings* settings, void* stream);
/* No counterpart in the reference. The device error word of grisPassRenderNoAlloc on `device`,
 * read after the work queued on `stream` (the call synchronizes `stream`) and then cleared.
 * Returns GRIS_OK with *errorWord = 0, or GRIS_ERR_DEVICE_FAULT with the bits in *errorWord.
 * Allocates nothing; restores the caller's current device. */
int grisNoAllocReadError(int device, void* stream, uint64_t* errorWord);

/* ---------------------------------------------------------------- batches of views */
/* A batch renders many independent views per frame — each with its own scene, resolution,
 * cameras and settings (depth, reuse, ...) — with one launch per pass for all of them (the
 * per-frame view table lives in device memory). Buffers are library-owned per view, with the
 * renderer's ping-pong, as for grisFrame*. The path tracer runs either as one kernel per frame
 * (GRIS_PATH_MEGAKERNEL) or as wavefront stages per bounce — closest hits, shading, shadow
 * queries, NEE + BSDF sampling — over queues of live paths compacted at every bounce
 * (GRIS_PATH_WAVEFRONT, default). Results are identical either way. */
#define GRIS_PATH_MEGAKERNEL 0
#define GRIS_PATH_WAVEFRONT 1
typedef struct GrisBatch GrisBatch;
int grisSetPathForm(GrisContext* ctx, int form);
/* Batch frames are captured once into a CUDA graph (per staging slot and frame shape) and
 * replayed (default on; off while per-kernel profiling is on). */
int grisSetGraphs(GrisContext* ctx, int enable);
/* Grid sizes of the wavefront kernels, in 128-thread blocks per SM (defaults 16 and 8). */
int grisSetWaveLaunch(GrisContext* ctx, int traceBlocksPerSM, int shadeBlocksPerSM);
/* 1: the wavefront's traversal kernels keep every lane busy (a lane whose ray is finished takes
 * the next ray while the others of its warp still walk), and a bounce level with fewer than 8,192
 * rays is walked one ray per warp (each round 4 nodes and up to 32 triangles); same results. */
int grisSetWaveRefill(GrisContext* ctx, int enable);
/* Times candidate configurations — the megakernel path tracer, the wavefront one with trace
 * grids of 8/16/32 and shading grids of 4/8/16 blocks per SM, and the wavefront one with the
 * refilling traversal kernels at 4/8/16 blocks per SM — over `frames` frames each on the given
 * views (those frames are rendered: reservoirs and output change), keeps the fastest in the
 * context and reports it. */
typedef struct GrisTuneResult {
    int pathForm;
    int traceBlocksPerSM, shadeBlocksPerSM;
    int candidates;
    double msPerFrame;            /* of the chosen configuration */
    double candidateMs[16];       /* per candidate, in the order above */
    int refill;                   /* the chosen wavefront uses the refilling traversal kernels */
} GrisTuneResult;
int grisBatchCreate(GrisContext* ctx, uint32_t nViews, const GrisScene* const* scenes, const uint32_t* widths,
                    const uint32_t* heights, GrisBatch** out);
int grisBatchDestroy(GrisBatch* batch);
/* cams, prevCams, settings: nViews entries each (filmSize must match the view's size). */
int grisBatchRender(GrisContext* ctx, GrisBatch* batch, const GrisCamera* cams, const GrisCamera* prevCams,
                    const GrisSettings* settings);
/* which / slot as in grisFrameGetBuffer, for one view; view = GRIS_BATCH_ALL_VIEWS gives the
 * buffer of every view at once (the views' pixels one after another, in view order). */
#define GRIS_BATCH_ALL_VIEWS 0xffffffffu
int grisBatchGetBuffer(const GrisBatch* batch, uint32_t view, int which, int slot, void** devPtr, size_t* bytes);
/* Copies one view's buffer to host memory on the context stream and waits for it. */
int grisBatchDownload(GrisContext* ctx, const GrisBatch* batch, uint32_t view, int which, int slot, void* host,
                      size_t bytes);
/* The pipelined form (grisFrameDownloadAsync): returns at once, complete after grisDownloadWait. */
int grisBatchDownloadAsync(GrisContext* ctx, const GrisBatch* batch, uint32_t view, int which, int slot, void* host,
                           size_t bytes);
/* Attaches a guide (NULL detaches it): the batch's path tracing then guides the vertices after
 * each path's reconnection vertex and, when the guide trains, runs its Adam steps on the
 * frame's records after each frame (wavefront path form only). */
int grisBatchSetGuide(GrisBatch* batch, GrisGuide* guide);
int grisBatchAutotune(GrisContext* ctx, GrisBatch* batch, const GrisCamera* cams, const GrisCamera* prevCams,
                      const GrisSettings* settings, int frames, GrisTuneResult* out);

/* ---------------------------------------------------------------- frames (library-owned buffers) */
/* G-buffer cur/prev, reservoirs This[2]/Temp, output: the renderer's per-frame resources
 * (src/Renderer.cpp:193-257) with its ping-pong (Renderer.cpp:329-347, 567). */
int grisFrameCreate(GrisContext* ctx, uint32_t width, uint32_t height, GrisFrame** out);
int grisFrameDestroy(GrisFrame* frame);
/* G-buffer into the current slot, then GRISReSTIR::render on the current slot, then swap. */
int grisFrameRender(GrisContext* ctx, const GrisScene* scene, GrisFrame* frame, const GrisCamera* cam,
                    const GrisCamera* prevCam, const GrisSettings* settings);
/* which: 0 depthNormal, 1 albedoMatId, 2 motion, 3 reservoir, 4 temp reservoir, 5 output,
 * 6 DI reservoir, 7 DI temp reservoir, 8 direct output (6-8 once grisFrameRenderDI ran).
 * slot: 0 = the slot the last grisFrameRender wrote (current), 1 = the other one. */
int grisFrameGetBuffer(const GrisFrame* frame, int which, int slot, void** devPtr, size_t* bytes);
int grisFrameDownload(GrisContext* ctx, const GrisFrame* frame, int which, int slot, void* host, size_t bytes);
/* Pipelined downloads (no counterpart in the reference, which presents its image on the GPU):
 * the buffer is copied on the context stream into a library-owned device staging area (a
 * device-to-device copy after the work queued so far), and from there to `host` on a separate
 * copy stream, so that the next frame's kernels, queued right after, run while the copy to host
 * proceeds. Returns at once; `host` holds the data after grisDownloadWait. Any number of
 * downloads may be queued between two waits (the staging area grows; growing waits for the
 * downloads in flight). `host` should be pinned (page-locked) for the copy to overlap. */
int grisFrameDownloadAsync(GrisContext* ctx, const GrisFrame* frame, int which, int slot, void* host, size_t bytes);
/* Waits for every download queued by grisFrameDownloadAsync / grisBatchDownloadAsync. */
int grisDownloadWait(GrisContext* ctx);
int grisFrameUpload(GrisContext* ctx, GrisFrame* frame, int which, int slot, const void* host, size_t bytes);

/* ---------------------------------------------------------------- ReSTIR DI (direct lighting)
 * The reference's ReSTIR DI pass (TestReSTIR::render, src/TestReSTIR.cpp:9-35), which the
 * renderer runs for directMethod = ReSTIR DI before the indirect pass (src/Renderer.cpp:449-476):
 *   candidates  di_path_gen.glsl:9-40 + sampleLi (di_reservoir.glsl:78-174): one light sample
 *               (power-proportional, shadow-tested) and/or one BSDF sample that hits a light,
 *               streamed into a reservoir at the primary vertex
 *   temporal    di_temporal.glsl:9-90: the previous frame's reservoir at the reprojected pixel
 *               (same mat/mesh id, normal >= 0.95, distance <= 0.5), shifted and merged, the
 *               final sample's visibility tested, M capped at 40
 *   spatial     di_spatial.glsl:9-121: 10 neighbours in a 20-pixel disk (normal >= 0.9,
 *               distance <= 0.4), shifted and merged, visibility, cap 40, then the final
 *               shading Li / lum(Li) * W / M into the running mean of the direct output
 *               (di_spatial.comp:14-27)
 * Shifts (di_reservoir.glsl:176-296): reconnection (the light vertex seen from the destination,
 * one visibility ray) or random replay (the source's candidates drawn again at the destination
 * from the source's seed); the reference merges nothing for its third value (hybrid). */
#define GRIS_DI_SHIFT_RECONNECTION 0
#define GRIS_DI_SHIFT_REPLAY 1
#define GRIS_DI_SHIFT_HYBRID 2
#define GRIS_DI_SAMPLE_LIGHT 0
#define GRIS_DI_SAMPLE_BSDF 1
#define GRIS_DI_SAMPLE_BOTH 2
/* TestReSTIR::Settings (src/TestReSTIR.h:12-17), the pass's 16-byte push constant; the
 * reference's defaults are {RECONNECTION, LIGHT, 0, 1} (TestReSTIR.h:29). */
typedef struct GrisDISettings {
    uint32_t shiftType;
    uint32_t sampleType;
    uint32_t temporalReuse;
    uint32_t spatialReuse;
} GrisDISettings;
/* DIReservoir (layouts.glsl:96-115), 64 B std430 (DIReservoirData, src/Renderer.cpp:33). */
typedef struct GrisDIReservoir {
    float bary[2];
    uint32_t instanceIdx, triangleIdx;   /* instance 0: a light triangle */
    float Li[3];
    float pad0;
    float jacobian;                      /* |cos| / d^2 at the light vertex */
    float samplePdf;
    uint32_t rng;                        /* the candidates' seed (random replay) */
    uint32_t isLightSample;              /* GLSL bool: 0 / 1 */
    uint32_t sampleCount;
    float resampleWeight, contribWeight, weight;
} GrisDIReservoir;
typedef struct GrisDIBindings {
    uint32_t width, height;
    const float* depthNormal;        /* the G-buffer of grisPassGBuffer, as for GrisPassBindings */
    const float* depthNormalPrev;
    const uint32_t* albedoMatId;
    const uint32_t* albedoMatIdPrev;
    const uint16_t* motion;
    GrisDIReservoir* reservoirThis;
    const GrisDIReservoir* reservoirPrev;
    GrisDIReservoir* reservoirTemp;
    float* directOutput;             /* float4 RGBA32F, running mean */
} GrisDIBindings;
/* passes: bit 0 candidates, bit 1 temporal, bit 2 spatial (7 = TestReSTIR::render). */
int grisPassDI(GrisContext* ctx, const GrisScene* scene, const GrisDIBindings* b, const GrisCamera* cam,
               const GrisCamera* prevCam, const GrisDISettings* settings, int passes);
/* The renderer's frame with directMethod = ReSTIR DI: G-buffer into the current slot, the DI pass
 * on the frame's DI buffers (allocated on first use, zeroed: two reservoirs per pixel
 * ping-ponged with the frame's slots, a temporary one and the direct output), then
 * GRISReSTIR::render unless `settings` is NULL (indirectMethod = None), then swap. */
int grisFrameRenderDI(GrisContext* ctx, const GrisScene* scene, GrisFrame* frame, const GrisCamera* cam,
                      const GrisCamera* prevCam, const GrisSettings* settings, const GrisDISettings* di);

/* ---------------------------------------------------------------- post-processing (headless)
 * The reference's presentation pass (PostProcessFrag, src/shader/post_proc.frag:30-44, push
 * constant src/PostProcessFrag.h:7-12) as a kernel: direct + indirect output (each unless its
 * flag is set), tone mapping (0 none, 1 filmic, 2 ACES), gamma 1/2.2, then the B8G8R8A8_UNORM
 * swapchain conversion (NaN -> 0, clamp to [0, 1], round(255 c)). The full-screen quad samples
 * texel ivec2((size - 1) * uv) at uv = pixel centre / size, as the fragment shader does. The
 * renderer's defaults are filmic + gamma (src/Renderer.h:32-33). pow is the library's
 * deterministic x^y = 2^(y log2 x). */
#define GRIS_TONEMAP_NONE 0
#define GRIS_TONEMAP_FILMIC 1
#define GRIS_TONEMAP_ACES 2
typedef struct GrisPostSettings {   /* PostProcessFrag::PushConstant, 16 B */
    uint32_t toneMapping;
    uint32_t correctGamma;
    uint32_t noDirect;
    uint32_t noIndirect;
} GrisPostSettings;
typedef struct GrisPostBindings {
    uint32_t width, height;
    const float* directOutput;       /* float4 RGBA32F (may be NULL when noDirect) */
    const float* indirectOutput;     /* float4 RGBA32F (may be NULL when noIndirect) */
    float* color;                    /* float4: the fragment shader's output, NaN as 0x7fc00000 (may be NULL) */
    uint8_t* rgba8;                  /* 4 bytes per pixel, R G B A, row 0 at the top (may be NULL) */
} GrisPostBindings;
int grisPostProcess(GrisContext* ctx, const GrisPostBindings* b, const GrisPostSettings* settings);
/* Host: writes 8-bit RGBA pixels (row 0 at the top) as a PNG file (zlib stored blocks, no
 * compression). Returns GRIS_OK or GRIS_ERR_INVALID_ARGUMENT with a message in errBuf. */
int grisWritePNG(const char* path, const uint8_t* rgba, uint32_t width, uint32_t height, char* errBuf, size_t errLen);

#ifdef __cplusplus
}
#endif

#endif
