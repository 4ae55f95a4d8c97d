/*
 * ref_common.h — what the GPU supplied to the reference's shaders, for the two harnesses that
 * run those shaders on the CPU (ref_harness.cpp: the GRIS pass; ref_harness_di.cpp: the ReSTIR
 * DI pass).
 *
 * TEST INFRASTRUCTURE (oracle); only tests/ use the libraries built from it.
 *
 *   - traceClosestHit / traceShadow / traceVisibility (reference: src/shader/ray_query.glsl:6-70,
 *     hardware ray queries) as a brute-force loop over every triangle of the scene with
 *     the project's ray/triangle test (Moller-Trumbore with its cross and dot products fused,
 *     two-sided, t in [tmin, tmax]) and a
 *     deterministic tie-break: smallest t, then smallest (instanceIdx, triangleIdx).
 *     Instance 0 is the light geometry (src/Scene.cpp:455-479, 525-541).
 *   - the scene's storage buffers bound to caller arrays, and binary16 conversions for the
 *     RG16F motion vectors (src/GBufferPass.h:23-26).
 */
#ifndef GREF_COMMON_H
#define GREF_COMMON_H
#include <stdint.h>
#include <stdlib.h>
#include <string.h>
#include <vector>
#include "glsl_compat.h"

namespace glsl {

static int gref_max_depth = 15;
static uint gref_resample_num = 3;
static float gref_resample_radius = 20.0f;
#define GREF_MAX_DEPTH gref_max_depth
#define GREF_RESAMPLE_NUM gref_resample_num
#define GREF_RESAMPLE_RADIUS gref_resample_radius

#include "HostDevice.h"
#include "ray_layouts.glsl"

}  /* namespace glsl */
/* HostDevice.h maps the fixed-width names onto GLSL types for shader code. */
#undef int32_t
#undef uint32_t
namespace glsl {

/* ------------------------------------------------------------------ traversal */
struct WTri { vec3 v0, e1, e2; uint inst, tri; };
static std::vector<WTri> g_tris;
static unsigned long long g_ray_counts[4];   /* closest, shadow, gbuffer, unused */

/* cross and dot products with one rounding per fused step: a*b - c*d = fma(a, b, -(c*d)),
 * a.b = fma(a.z, b.z, fma(a.y, b.y, a.x*b.x)) */
static inline vec3 gref_cross(const vec3& a, const vec3& b) {
    return vec3(__builtin_fmaf(a.y, b.z, -(a.z * b.y)), __builtin_fmaf(a.z, b.x, -(a.x * b.z)), __builtin_fmaf(a.x, b.y, -(a.y * b.x)));
}
static inline float gref_dot(const vec3& a, const vec3& b) { return __builtin_fmaf(a.z, b.z, __builtin_fmaf(a.y, b.y, a.x * b.x)); }
static inline bool gref_tri_hit(const WTri& T, const vec3& o, const vec3& d, float tmin, float tmax,
                                float& t, float& u, float& v) {
    vec3 pv = gref_cross(d, T.e2);
    float det = gref_dot(T.e1, pv);
    if (det == 0.0f) return false;
    float inv = 1.0f / det;
    vec3 tv = o - T.v0;
    u = gref_dot(tv, pv) * inv;
    if (!(u >= 0.0f) || !(u <= 1.0f)) return false;
    vec3 qv = gref_cross(tv, T.e1);
    v = gref_dot(d, qv) * inv;
    if (!(v >= 0.0f) || !(u + v <= 1.0f)) return false;
    t = gref_dot(T.e2, qv) * inv;
    if (!(t >= tmin) || !(t <= tmax)) return false;
    return true;
}

static Intersection gref_closest(vec3 o, vec3 d, float tmin, float tmax, bool skipLights) {
    float bestT = tmax;
    unsigned long long bestKey = ~0ull;
    Intersection isec;
    isec.bary = vec2(0.0f);
    isec.instanceIdx = InvalidHitIndex;
    isec.triangleIdx = 0;
    for (const WTri& T : g_tris) {
        if (skipLights && T.inst == 0) continue;
        float t, u, v;
        if (!gref_tri_hit(T, o, d, tmin, tmax, t, u, v)) continue;
        unsigned long long key = ((unsigned long long)T.inst << 32) | T.tri;
        if (t < bestT || (t == bestT && key < bestKey)) {
            bestT = t; bestKey = key;
            isec.bary = vec2(u, v); isec.instanceIdx = T.inst; isec.triangleIdx = T.tri;
        }
    }
    return isec;
}

Intersection traceClosestHit(accelerationStructureEXT, uint, uint, vec3 origin, float minDist, vec3 direction, float maxDist) {
#pragma omp atomic
    g_ray_counts[0]++;
    return gref_closest(origin, direction, minDist, maxDist, false);
}

bool traceShadow(accelerationStructureEXT, uint, uint, vec3 origin, float minDist, vec3 direction, float maxDist) {
#pragma omp atomic
    g_ray_counts[1]++;
    for (const WTri& T : g_tris) {
        float t, u, v;
        if (gref_tri_hit(T, origin, direction, minDist, maxDist, t, u, v)) return true;
    }
    return false;
}

/* reference: src/shader/ray_query.glsl:29-39 */
bool traceVisibility(accelerationStructureEXT as, uint rayFlags, uint rayMask, vec3 from, vec3 to) {
    return !traceShadow(as, rayFlags, rayMask, from, MinRayDistance, normalize(to - from), distance(to, from) - MinRayDistance);
}


/* ------------------------------------------------------------------ binary16 */
static uint16_t gref_f32_to_f16(float f) {
    uint32_t x; memcpy(&x, &f, 4);
    uint32_t sign = (x >> 16) & 0x8000u, ex = (x >> 23) & 0xffu, mant = x & 0x7fffffu;
    if (ex == 0xffu) return (uint16_t)(sign | 0x7c00u | (mant ? (0x200u | (mant >> 13)) : 0u));
    int e = (int)ex - 112;
    if (e >= 31) return (uint16_t)(sign | 0x7c00u);
    if (e <= 0) {
        if (e < -10) return (uint16_t)sign;
        mant |= 0x800000u;
        int shift = 14 - e;
        uint32_t hm = mant >> shift, rem = mant & ((1u << shift) - 1u), half = 1u << (shift - 1);
        if (rem > half || (rem == half && (hm & 1u))) hm++;
        return (uint16_t)(sign | hm);
    }
    uint32_t hm = mant >> 13, rem = mant & 0x1fffu;
    uint32_t h = sign | ((uint32_t)e << 10) | hm;
    if (rem > 0x1000u || (rem == 0x1000u && (hm & 1u))) h++;
    return (uint16_t)h;
}
static float gref_f16_to_f32(uint16_t h) {
    uint32_t sign = (uint32_t)(h & 0x8000u) << 16, ex = (h >> 10) & 0x1fu, mant = h & 0x3ffu, x;
    if (ex == 0) {
        if (mant == 0) x = sign;
        else { int e = -1; do { mant <<= 1; e++; } while (!(mant & 0x400u)); x = sign | ((uint32_t)(112 - e) << 23) | ((mant & 0x3ffu) << 13); }
    } else if (ex == 31) x = sign | 0x7f800000u | (mant << 13);
    else x = sign | ((ex + 112) << 23) | (mant << 13);
    float f; memcpy(&f, &x, 4); return f;
}


/* Binds the scene arrays (the caller keeps them alive) and builds the world-space triangle list. */
static int gref_bind_scene(void* vertices, unsigned long long nv, void* indices, unsigned long long ni,
                           void* instances, unsigned long long ninst, void* materials, unsigned long long nmat,
                           void* matIndices, unsigned long long nmi, void* lights, unsigned long long nl,
                           void* table, unsigned long long nt) {
    uVertices.data = (MeshVertex*)vertices; uVertices.n = nv;
    uIndices.data = (uint*)indices; uIndices.n = ni;
    uObjectInstances.data = (ObjectInstance*)instances; uObjectInstances.n = ninst;
    uMaterials.data = (Material*)materials; uMaterials.n = nmat;
    uMaterialIndices.data = (int*)matIndices; uMaterialIndices.n = nmi;
    uTriangleLights.data = (TriangleLight*)lights; uTriangleLights.n = nl;
    uLightSampleTable.data = (LightSampleTableElement*)table; uLightSampleTable.n = nt;
    g_tris.clear();
    for (uint i = 0; i < (uint)nl; i++) {
        TriangleLight L = uTriangleLights[i];
        WTri T; T.v0 = L.v0; T.e1 = L.v1 - L.v0; T.e2 = L.v2 - L.v0; T.inst = 0; T.tri = i;
        g_tris.push_back(T);
    }
    for (uint k = 0; k < (uint)ninst; k++) {
        ObjectInstance I = uObjectInstances[k];
        for (uint t = 0; t < I.indexCount / 3; t++) {
            vec3 w[3];
            for (int j = 0; j < 3; j++) {
                MeshVertex mv = uVertices[uIndices[I.indexOffset + t * 3 + j]];
                w[j] = vec3(I.transform * vec4(mv.pos, 1.0f));
            }
            WTri T; T.v0 = w[0]; T.e1 = w[1] - w[0]; T.e2 = w[2] - w[0]; T.inst = k + 1; T.tri = t;
            g_tris.push_back(T);
        }
    }
    return (int)g_tris.size();
}

}  /* namespace glsl */

#endif
