/*
 * gris_kernels.h — host-side launch interface of the grisrt kernels.
 */
#ifndef GRISRT_GRIS_KERNELS_H
#define GRISRT_GRIS_KERNELS_H

#include <cuda_runtime.h>
#include <stdint.h>

#include "../../include/grisrt.h"

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
cudaError_t launch_debug_trace(const uint32_t* nodes, const float* tris, const float* rays, uint64_t n, int anyHit,
                               float* hitTUV, uint32_t* hitInst, uint32_t* hitTri, unsigned long long* counters,
                               cudaStream_t stream);

}  // namespace grisrt

#endif
