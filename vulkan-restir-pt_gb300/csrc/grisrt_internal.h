/*
 * grisrt_internal.h — internal declarations shared by the grisrt translation units.
 */
#ifndef GRISRT_INTERNAL_H
#define GRISRT_INTERNAL_H

#include <cuda_runtime.h>
#include <stdint.h>

#include <string>
#include <vector>

#include "../../include/grisrt.h"

namespace grisrt {

/* Host copy of the 8-wide BVH (layout in bvh_traverse.h). */
struct BvhHost {
    std::vector<uint32_t> nodes;   /* GRIS_NODE_WORDS per node */
    std::vector<float> tris;       /* GRIS_TRI_FLOATS per triangle, in leaf order */
    uint32_t maxDepth = 0;
    uint64_t triangleCount = 0;
    double buildSeconds = 0.0;
};

/* World-space triangles of the scene as every ray query sees them: light triangles
 * (instance 0, index = light index) then each object instance k (instance k+1, index = local
 * triangle), vertex = vec3(transform * vec4(pos, 1)) evaluated column by column. */
void world_triangles(const GrisSceneDesc& d, std::vector<float>& v012, std::vector<uint32_t>& ids);

/* Builds the BVH; returns false with a message on failure. */
bool build_bvh(const GrisSceneDesc& d, BvhHost& out, std::string& err);

struct DeviceSceneView;
struct KernelTimer;
int ctx_device(GrisContext* ctx);
cudaStream_t ctx_stream(GrisContext* ctx);
unsigned long long* ctx_counters(GrisContext* ctx);
int ctx_count_work(GrisContext* ctx);
int ctx_path_form(GrisContext* ctx);
KernelTimer* ctx_timer(GrisContext* ctx);
int ctx_fail(GrisContext* ctx, int code, const std::string& msg);
/* a pipelined download (grisFrameDownloadAsync): device-to-device into the staging area on the
 * context stream, then to host on the copy stream */
int ctx_download_async(GrisContext* ctx, const void* dev, void* host, size_t bytes, const char* what);
struct WaveLaunch;
namespace guide { struct GuideDevice; }
guide::GuideDevice guide_device(const GrisGuide* g);
const GrisGuideConfig& guide_config(const GrisGuide* g);
cudaError_t guide_train_frame(GrisGuide* g, cudaStream_t st);
bool ctx_graphs(GrisContext* ctx);            /* graphs enabled and per-kernel profiling off */
bool ctx_profiling(GrisContext* ctx);         /* per-kernel profiling on (kernels then run in order) */
WaveLaunch ctx_wave_launch(GrisContext* ctx);
void ctx_set_tuning(GrisContext* ctx, int pathForm, WaveLaunch wl);
/* Device view and device ordinal of an uploaded scene; false for a host-only scene. */
bool scene_device(const GrisScene* s, DeviceSceneView* view, int* device);

/* Values looked up once per device and cached for every later launch on that device: SM counts,
 * occupancies, kernel attributes. once_per_device(key, f) runs f() with the calling thread's
 * current device, under a lock shared by all threads, the first time `key` is asked for on that
 * device, and returns its result then and afterwards; a negative result (an error) is returned
 * but not cached, so the next call tries again. Keys are the kDeviceKey* values below. */
constexpr int kDeviceKeys = 16;
enum {
    kDeviceKeySMs = 0,              /* multiprocessor count */
    kDeviceKeyOccPath = 1,          /* resident blocks per SM of the persistent pass kernels */
    kDeviceKeyOccTemporal = 2,
    kDeviceKeyOccSpatial = 3,
    kDeviceKeyGuideTcAttr = 4,      /* dynamic shared memory attribute of the tcgen05 inference kernel */
    kDeviceKeyGuideGradAttr = 5,    /* ... of the gradient kernel */
    kDeviceKeyGuideGradTcAttr = 6,  /* ... of the tcgen05 gradient kernel */
    kDeviceKeyWalkCarveout = 7,     /* shared-memory carveout of the resident traversal kernels */
};
int once_per_device(int key, int (*f)());
/* SM count of the current device (cached; 1 if it cannot be read). */
int current_sm_count();

}  // namespace grisrt

#endif
