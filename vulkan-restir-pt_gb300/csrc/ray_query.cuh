/*
 * ray_query.cuh — the ray queries of the passes (ray_query.glsl:6-70 over the 8-wide BVH of
 * bvh_traverse.h), their per-thread counts and the per-warp flush into the context counters,
 * and the host-side conversions of cameras and scene views into kernel arguments. Shared by
 * the GRIS kernels (gris_kernels.cu) and the ReSTIR DI kernels (di_kernels.cu).
 */
#ifndef GRISRT_RAY_QUERY_CUH
#define GRISRT_RAY_QUERY_CUH

#include "gris_device.cuh"
#include "gris_kernels.h"

namespace grisrt {

/* ------------------------------------------------------------------ ray queries */
/* Per-thread ray counts, plus traversal work when the pass counts it (ctx work counting). */
struct RayCount { uint32_t closest, shadow; GrisWork work; };

GD RayCount ray_count() {
    RayCount rc;
    rc.closest = 0u; rc.shadow = 0u; rc.work.nodes = 0u; rc.work.tris = 0u;
    return rc;
}

GD Isec traceClosestHit(const DevScene& sc, V3 o, V3 d, float tmin, float tmax, RayCount& rc, int& err) {
    rc.closest++;
    GrisRayHit h;
    Isec r;
    if (gris_bvh_trace<false>(sc.nodes, sc.tris, o.x, o.y, o.z, d.x, d.y, d.z, tmin, tmax, false, &h, &err, &rc.work)) {
        r.bx = h.u; r.by = h.v; r.inst = h.inst; r.tri = h.tri;
    } else {
        r.bx = 0.0f; r.by = 0.0f; r.inst = kInvalidHit; r.tri = 0u;
    }
    return r;
}
GD bool traceShadow(const DevScene& sc, V3 o, float tmin, V3 d, float tmax, RayCount& rc, int& err) {
    rc.shadow++;
    GrisRayHit h;
    return gris_bvh_trace<true>(sc.nodes, sc.tris, o.x, o.y, o.z, d.x, d.y, d.z, tmin, tmax, false, &h, &err, &rc.work);
}
/* The same queries as out-of-line calls, for the reuse passes: there the traversal loop would be
 * inlined at three call sites of one kernel, and the one shared copy runs faster (fewer
 * instruction-fetch stalls); the path tracer keeps the inlined form. */
static __device__ __noinline__ Isec traceClosestHitCall(const DevScene& sc, V3 o, V3 d, float tmin, float tmax, RayCount& rc, int& err) {
    return traceClosestHit(sc, o, d, tmin, tmax, rc, err);
}
static __device__ __noinline__ bool traceShadowCall(const DevScene& sc, V3 o, float tmin, V3 d, float tmax, RayCount& rc, int& err) {
    return traceShadow(sc, o, tmin, d, tmax, rc, err);
}
/* ray_query.glsl:29-39 */
GD bool traceVisibility(const DevScene& sc, V3 from, V3 to, RayCount& rc, int& err) {
    return !traceShadowCall(sc, from, kMinRayDistance, normalize3(to - from), distance3(to, from) - kMinRayDistance, rc, err);
}

/* counters: [0] closest, [1] shadow, [2] primary, [3] error word,
 * [8+2k] nodes and [9+2k] triangles of kernel k, [16+k] closest-hit rays of kernel k
 * (k: 0 G-buffer, 1 path trace, 2 temporal, 3 spatial); the wavefront's traversal stages also
 * count on their own: [26+3s] nodes, [27+3s] triangles, [28+3s] rays (closest for s = 0, the
 * extension stage; shadow for s = 1, the shadow stage), and so do the visibility walks of the
 * reuse passes' three-launch form: [41+3r] nodes, [42+3r] triangles, [43+3r] rays (stage s = 2 + r,
 * r = 0 temporal, 1 spatial); words 24-25 hold the persistent form's
 * tile cursors; the ReSTIR DI kernels (k = 4, 5, 6: candidates, temporal, spatial) count their
 * work in [32+3d] nodes, [33+3d] triangles, [34+3d] rays of both kinds (d = k - 4). */
GD void flush_counts(unsigned long long* counters, const RayCount& rc, int err, int kernel, int countWork,
                     int stage = -1) {
    unsigned int c = __reduce_add_sync(0xffffffffu, rc.closest);
    unsigned int s = __reduce_add_sync(0xffffffffu, rc.shadow);
    unsigned int e = __reduce_or_sync(0xffffffffu, (unsigned)err);
    unsigned long long nodes = 0, tris = 0;
    if (countWork) {
        nodes = __reduce_add_sync(0xffffffffu, rc.work.nodes);
        tris = __reduce_add_sync(0xffffffffu, rc.work.tris);
    }
    if (((threadIdx.y * blockDim.x + threadIdx.x) & 31u) == 0u) {
        if (c) atomicAdd(counters + GRIS_COUNTER_CLOSEST, (unsigned long long)c);
        if (s) atomicAdd(counters + GRIS_COUNTER_SHADOW, (unsigned long long)s);
        if (e) atomicOr(counters + GRIS_COUNTER_ERROR, (unsigned long long)e);
        if (countWork && kernel >= 4) {
            atomicAdd(counters + 32 + 3 * (kernel - 4), nodes);
            atomicAdd(counters + 33 + 3 * (kernel - 4), tris);
            atomicAdd(counters + 34 + 3 * (kernel - 4), (unsigned long long)(c + s));
        } else if (countWork) {
            atomicAdd(counters + 8 + 2 * kernel, nodes);
            atomicAdd(counters + 9 + 2 * kernel, tris);
            atomicAdd(counters + 16 + kernel, (unsigned long long)c);
            if (stage >= 0) {
                const int w = stage < 2 ? 26 + 3 * stage : 41 + 3 * (stage - 2);
                atomicAdd(counters + w, nodes);
                atomicAdd(counters + w + 1, tris);
                atomicAdd(counters + w + 2, (unsigned long long)(stage == 0 ? c : s));
            }
        }
    }
}

/* ------------------------------------------------------------------ kernel arguments */
inline CamD make_cam(const GrisCamera& c) {
    CamD d;
    d.pos.x = c.pos[0]; d.pos.y = c.pos[1]; d.pos.z = c.pos[2];
    d.front.x = c.front[0]; d.front.y = c.front[1]; d.front.z = c.front[2];
    d.right.x = c.right[0]; d.right.y = c.right[1]; d.right.z = c.right[2];
    d.up.x = c.up[0]; d.up.y = c.up[1]; d.up.z = c.up[2];
    d.FOV = c.FOV;
    d.w = c.filmSize[0]; d.h = c.filmSize[1];
    d.frameIndex = c.frameIndex; d.seed = c.seed;
    d.aspect = (float)d.w / (float)d.h;
    d.tanHalfFov = gris_det_tanf(c.FOV * 0.5f * 0.01745329251994329577f);
    return d;
}

inline DevScene to_dev(const DeviceSceneView& v) {
    DevScene s;
    s.vertices = v.vertices; s.nVertices = v.nVertices;
    s.indices = v.indices; s.nIndices = v.nIndices;
    s.instances = v.instances; s.nInstances = v.nInstances;
    s.materials = v.materials; s.nMaterials = v.nMaterials;
    s.matIndices = v.matIndices; s.nMatIndices = v.nMatIndices;
    s.lights = v.lights; s.nLights = v.nLights;
    s.table = v.table; s.nTable = v.nTable;
    s.nodes = v.nodes; s.tris = v.tris;
    return s;
}

}  // namespace grisrt

#endif
