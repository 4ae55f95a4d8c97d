/*
 * ref_harness.cpp — runs the reference's own GRIS shader code (compiled as C++ by
 * oracle/ref/make_ref.py) on the CPU, to pin the oracle restatement.
 *
 * TEST INFRASTRUCTURE (oracle). Built into oracle/_ref/libgrisref.so; only tests/ use it.
 *
 * The shader library is the reference's; ref_common.h supplies the ray queries and the scene
 * buffers, and this file the rest of what the GPU supplied:
 *   - the G-buffer (reference: src/shader/GBuffer.vert:16-28 and GBuffer.frag:21-54, a raster
 *     pass) as one primary ray per pixel centre that ignores the light instance, with the
 *     vertex shader's per-vertex transform and the fragment shader's outputs; the motion
 *     vector is rounded to binary16 (RG16F target, src/GBufferPass.h:23-26).
 *   - the three compute wrappers gris_path_trace.comp:14-28, gris_resample_temporal.comp:14-28
 *     and gris_resample_spatial.comp:14-28 (the last one accumulates into the RGBA32F output).
 */
#include "ref_common.h"

namespace glsl {

#include "gris_path_trace.glsl"
#include "gris_resample_temporal.glsl"
#include "gris_resample_spatial.glsl"
#include "gi_naive.glsl"

/* ------------------------------------------------------------------ C API */
struct GrefSettings {
    uint shiftType; float rrScale; uint temporalReuse; uint spatialReuse; uint cap;
    uint maxDepth; uint spatialNeighbors; float spatialRadius;
};

extern "C" {

int gref_sizeof(int which) {
    switch (which) {
    case 0: return (int)sizeof(Camera);
    case 1: return (int)sizeof(GRISReservoir);
    case 2: return (int)sizeof(Material);
    case 3: return (int)sizeof(MeshVertex);
    case 4: return (int)sizeof(ObjectInstance);
    case 5: return (int)sizeof(TriangleLight);
    case 6: return (int)sizeof(LightSampleTableElement);
    }
    return -1;
}

/* Binds the scene (caller keeps the arrays alive) and builds the world-space triangle list. */
int gref_scene_set(void* vertices, unsigned long long nv, void* indices, unsigned long long ni,
                   void* instances, unsigned long long ninst, void* materials, unsigned long long nmat,
                   void* matIndices, unsigned long long nmi, void* lights, unsigned long long nl,
                   void* table, unsigned long long nt) {
    return gref_bind_scene(vertices, nv, indices, ni, instances, ninst, materials, nmat, matIndices, nmi, lights, nl,
                           table, nt);
}

void gref_counters(unsigned long long* out, int reset) {
    for (int i = 0; i < 4; i++) { out[i] = g_ray_counts[i]; if (reset) g_ray_counts[i] = 0; }
}

/* G-buffer of one frame: depthNormal RGBA32F, albedoMatId RG32UI, motion RG16F (bits). */
void gref_gbuffer(const void* camera, uint W, uint H, float* depthNormal, uint* albedoMatId, uint16_t* motion) {
    Camera cam; memcpy(&cam, camera, sizeof(Camera));
#pragma omp parallel for schedule(dynamic, 4)
    for (int y = 0; y < (int)H; y++) {
        for (uint x = 0; x < W; x++) {
            size_t p = (size_t)y * W + x;
            vec2 uv = (vec2(uvec2(x, (uint)y)) + 0.5f) / vec2(uvec2(W, H));
            Ray ray = pinholeCameraSampleRay(cam, vec2(uv.x, 1.0f - uv.y), vec2(0.0f));
#pragma omp atomic
            g_ray_counts[2]++;
            Intersection h = gref_closest(ray.ori, ray.dir, MinRayDistance, MaxRayDistance, true);
            if (h.instanceIdx == InvalidHitIndex) {
                for (int c = 0; c < 4; c++) depthNormal[p * 4 + c] = 0.0f;
                albedoMatId[p * 2] = 0; albedoMatId[p * 2 + 1] = 0;
                motion[p * 2] = 0; motion[p * 2 + 1] = 0;
                continue;
            }
            uint k = h.instanceIdx - 1;
            ObjectInstance inst = uObjectInstances[k];
            vec3 b = vec3(1.0f - h.bary.x - h.bary.y, h.bary.x, h.bary.y);
            mat3 nrm = mat3(vec3(inst.transformInvT[0]), vec3(inst.transformInvT[1]), vec3(inst.transformInvT[2]));
            vec3 P[3], N[3];
            for (int j = 0; j < 3; j++) {
                MeshVertex mv = uVertices[uIndices[inst.indexOffset + h.triangleIdx * 3 + j]];
                P[j] = vec3(inst.transform * vec4(mv.pos, 1.0f));
                N[j] = normalize(nrm * mv.norm);
            }
            vec3 pos = (P[0] * b.x + P[1] * b.y) + P[2] * b.z;
            vec3 nor = normalize((N[0] * b.x + N[1] * b.y) + N[2] * b.z);
            uint matIndex = (uint)uMaterialIndices[inst.indexOffset / 3 + h.triangleIdx];
            vec3 albedo = uMaterials[matIndex].baseColor;
            vec4 last = cam.lastProjView * vec4(pos, 1.0f);
            last = last / last.w;
            last = last * 0.5f + 0.5f;
            vec2 thisCoord = vec2((float)x + 0.5f, (float)y + 0.5f) / vec2(uvec2(W, H));
            vec2 mvec = last.xy() - thisCoord;
            depthNormal[p * 4 + 0] = length(cam.pos - pos);
            depthNormal[p * 4 + 1] = nor.x; depthNormal[p * 4 + 2] = nor.y; depthNormal[p * 4 + 3] = nor.z;
            albedoMatId[p * 2] = packAlbedo(albedo);
            albedoMatId[p * 2 + 1] = (matIndex << 16) | k;
            motion[p * 2] = gref_f32_to_f16(mvec.x); motion[p * 2 + 1] = gref_f32_to_f16(mvec.y);
        }
    }
}

/* One GRISReSTIR::render (src/GRISReSTIR.cpp:9-53): path trace, temporal reuse, spatial reuse.
 * passes: bit 0 PT, bit 1 temporal, bit 2 spatial. */
void gref_gris_frame(const void* camera, const void* prevCamera, const void* settings,
                     const float* dnCur, const float* dnPrev, const uint* amCur, const uint* amPrev,
                     const uint16_t* motion, void* resvThis, void* resvPrev, void* resvTemp,
                     float* output, int passes) {
    memcpy(&uCamera, camera, sizeof(Camera));
    memcpy(&uPrevCamera, prevCamera, sizeof(Camera));
    GrefSettings s; memcpy(&s, settings, sizeof(s));
    uSettings.shiftMode = s.shiftType; uSettings.rrScale = s.rrScale;
    uSettings.temporalReuse = s.temporalReuse != 0; uSettings.spatialReuse = s.spatialReuse != 0;
    uSettings.cap = s.cap;
    gref_max_depth = (int)s.maxDepth; gref_resample_num = s.spatialNeighbors; gref_resample_radius = s.spatialRadius;
    int W = (int)uCamera.filmSize.x, H = (int)uCamera.filmSize.y;
    size_t n = (size_t)W * H;
    std::vector<float> mvf(n * 2);
    for (size_t i = 0; i < n * 2; i++) mvf[i] = gref_f16_to_f32(motion[i]);
    uDepthNormal.data = dnCur; uDepthNormal.w = W; uDepthNormal.h = H; uDepthNormal.ch = 4;
    uDepthNormalPrev.data = dnPrev; uDepthNormalPrev.w = W; uDepthNormalPrev.h = H; uDepthNormalPrev.ch = 4;
    uAlbedoMatId.data = amCur; uAlbedoMatId.w = W; uAlbedoMatId.h = H;
    uAlbedoMatIdPrev.data = amPrev; uAlbedoMatIdPrev.w = W; uAlbedoMatIdPrev.h = H;
    uMotionVector.data = mvf.data(); uMotionVector.w = W; uMotionVector.h = H; uMotionVector.ch = 2;
    uGRISReservoir.data = (GRISReservoir*)resvThis; uGRISReservoir.n = n;
    uGRISReservoirPrev.data = (GRISReservoir*)resvPrev; uGRISReservoirPrev.n = n;
    uGRISReservoirTemp.data = (GRISReservoir*)resvTemp; uGRISReservoirTemp.n = n;

    if (passes & 1) {
#pragma omp parallel for schedule(dynamic, 2)
        for (int y = 0; y < H; y++)
            for (int x = 0; x < W; x++) { vec3 c = clampColor(tracePath(uvec2(x, y), uCamera.filmSize)); (void)c; }
    }
    if (passes & 2) {
#pragma omp parallel for schedule(dynamic, 2)
        for (int y = 0; y < H; y++)
            for (int x = 0; x < W; x++) { vec3 c = temporalReuse(uvec2(x, y), uCamera.filmSize); (void)c; }
    }
    if (passes & 4) {
        float frameCount = float(uCamera.frameIndex & CameraFrameIndexMask);
#pragma omp parallel for schedule(dynamic, 2)
        for (int y = 0; y < H; y++)
            for (int x = 0; x < W; x++) {
                vec3 color = spatialReuse(uvec2(x, y), uCamera.filmSize);
                float* o = output + ((size_t)y * W + x) * 4;
                vec3 acc = vec3(o[0], o[1], o[2]);
                acc = (acc * frameCount + color) / (frameCount + 1.0f);
                o[0] = acc.x; o[1] = acc.y; o[2] = acc.z; o[3] = 1.0f;
            }
    }
}

/* The reference's naive indirect path tracer (gi_naive.comp:14-28), for convergence checks. */
void gref_naive_frame(const void* camera, const float* dnCur, const uint* amCur, float* output) {
    memcpy(&uCamera, camera, sizeof(Camera));
    int W = (int)uCamera.filmSize.x, H = (int)uCamera.filmSize.y;
    uDepthNormal.data = dnCur; uDepthNormal.w = W; uDepthNormal.h = H; uDepthNormal.ch = 4;
    uAlbedoMatId.data = amCur; uAlbedoMatId.w = W; uAlbedoMatId.h = H;
    float frameCount = float(uCamera.frameIndex & CameraFrameIndexMask);
#pragma omp parallel for schedule(dynamic, 2)
    for (int y = 0; y < H; y++)
        for (int x = 0; x < W; x++) {
            vec3 radiance = indirectIllumination(uvec2(x, y), uCamera.filmSize);
            float* o = output + ((size_t)y * W + x) * 4;
            vec3 acc = vec3(o[0], o[1], o[2]);
            acc = (acc * frameCount + radiance) / (frameCount + 1.0f);
            o[0] = acc.x; o[1] = acc.y; o[2] = acc.z; o[3] = 1.0f;
        }
}

uint16_t gref_f16(float f) { return gref_f32_to_f16(f); }

/* Brute-force ray queries: rays float[8] (org, tmin, dir, tmax); out float[4] {t,u,v,-} + inst + tri. */
void gref_trace(const float* rays, unsigned long long n, int anyHit, float* tuv, uint* inst, uint* tri) {
#pragma omp parallel for schedule(dynamic, 64)
    for (long long i = 0; i < (long long)n; i++) {
        const float* r = rays + i * 8;
        vec3 o = vec3(r[0], r[1], r[2]), d = vec3(r[4], r[5], r[6]);
        tuv[i * 4 + 3] = 0.0f;
        if (anyHit) {
            bool hit = false;
            for (const WTri& T : g_tris) {
                float t, u, v;
                if (gref_tri_hit(T, o, d, r[3], r[7], t, u, v)) { hit = true; break; }
            }
            tuv[i * 4] = hit ? 1.0f : -1.0f; tuv[i * 4 + 1] = 0.0f; tuv[i * 4 + 2] = 0.0f;
            inst[i] = hit ? 0u : InvalidHitIndex; tri[i] = hit ? 0u : InvalidHitIndex;
            continue;
        }
        float bestT = r[7];
        unsigned long long bestKey = ~0ull;
        bool found = false;
        float bu = 0.0f, bv = 0.0f;
        for (const WTri& T : g_tris) {
            float t, u, v;
            if (!gref_tri_hit(T, o, d, r[3], r[7], t, u, v)) continue;
            unsigned long long key = ((unsigned long long)T.inst << 32) | T.tri;
            if (t < bestT || (t == bestT && key < bestKey)) { bestT = t; bestKey = key; bu = u; bv = v; found = true; }
        }
        tuv[i * 4] = found ? bestT : -1.0f; tuv[i * 4 + 1] = bu; tuv[i * 4 + 2] = bv;
        inst[i] = found ? (uint)(bestKey >> 32) : InvalidHitIndex;
        tri[i] = found ? (uint)(bestKey & 0xffffffffu) : InvalidHitIndex;
    }
}

}  /* extern "C" */

}  /* namespace glsl */
