/*
 * ref_harness_di.cpp — runs the reference's own ReSTIR DI shader code (di_path_gen.glsl,
 * di_temporal.glsl, di_spatial.glsl, di_reservoir.glsl; compiled as C++ by
 * oracle/ref/make_ref.py) on the CPU, to pin the oracle's restatement of that pass.
 *
 * TEST INFRASTRUCTURE (oracle). Built into oracle/_ref/libdiref.so; only tests/ use it.
 *
 * ref_common.h supplies the ray queries and the scene buffers; this file supplies the three
 * compute wrappers di_path_gen.comp:14-26, di_temporal.comp:14-26 (neither stores its colour)
 * and di_spatial.comp:14-27 (running mean into the RGBA32F direct output), in the order of
 * TestReSTIR::render (src/TestReSTIR.cpp:9-35). The G-buffer comes from the caller.
 *
 * DIPathSample ends in a GLSL bool (4 bytes in std430); here it is a 1-byte C++ bool followed
 * by 3 padding bytes, which every pass clears so that the buffers compare byte for byte with
 * the std430 layout (bool as 0 / 1 in a 32-bit word).
 */
#include "ref_common.h"

namespace glsl {

#include "di_path_gen.glsl"
#include "di_temporal.glsl"
#include "di_spatial.glsl"

static void dref_clear_padding(DIReservoir* r, size_t n) {
    static_assert(sizeof(DIReservoir) == 64, "DIReservoir is 64 bytes in std430");
    for (size_t i = 0; i < n; i++) {
        unsigned char* p = reinterpret_cast<unsigned char*>(r + i) + 44;
        p[0] = p[0] ? 1 : 0;
        p[1] = p[2] = p[3] = 0;
    }
}

extern "C" {

int dref_sizeof(void) { return (int)sizeof(DIReservoir); }

int dref_scene_set(void* vertices, unsigned long long nv, void* indices, unsigned long long ni,
                   void* instances, unsigned long long ninst, void* materials, unsigned long long nmat,
                   void* matIndices, unsigned long long nmi, void* lights, unsigned long long nl,
                   void* table, unsigned long long nt) {
    return gref_bind_scene(vertices, nv, indices, ni, instances, ninst, materials, nmat, matIndices, nmi, lights, nl,
                           table, nt);
}

void dref_counters(unsigned long long* out, int reset) {
    for (int i = 0; i < 4; i++) { out[i] = g_ray_counts[i]; if (reset) g_ray_counts[i] = 0; }
}

/* One TestReSTIR::render. settings: {shiftType, sampleType, temporalReuse, spatialReuse}
 * (TestReSTIR::Settings). passes: bit 0 candidates, bit 1 temporal, bit 2 spatial. */
void dref_di_frame(const void* camera, const void* prevCamera, const uint* settings,
                   const float* dnCur, const float* dnPrev, const uint* amCur, const uint* amPrev,
                   const uint16_t* motion, void* resvThis, void* resvPrev, void* resvTemp,
                   float* output, int passes) {
    memcpy(&uCamera, camera, sizeof(Camera));
    memcpy(&uPrevCamera, prevCamera, sizeof(Camera));
    uSettings.shiftMode = settings[0];
    uSettings.sampleMode = settings[1];
    uSettings.temporalReuse = settings[2] != 0;
    uSettings.spatialReuse = settings[3] != 0;
    int W = (int)uCamera.filmSize.x, H = (int)uCamera.filmSize.y;
    size_t n = (size_t)W * H;
    std::vector<float> mvf(n * 2);
    for (size_t i = 0; i < n * 2; i++) mvf[i] = gref_f16_to_f32(motion[i]);
    uDepthNormal.data = dnCur; uDepthNormal.w = W; uDepthNormal.h = H; uDepthNormal.ch = 4;
    uDepthNormalPrev.data = dnPrev; uDepthNormalPrev.w = W; uDepthNormalPrev.h = H; uDepthNormalPrev.ch = 4;
    uAlbedoMatId.data = amCur; uAlbedoMatId.w = W; uAlbedoMatId.h = H;
    uAlbedoMatIdPrev.data = amPrev; uAlbedoMatIdPrev.w = W; uAlbedoMatIdPrev.h = H;
    uMotionVector.data = mvf.data(); uMotionVector.w = W; uMotionVector.h = H; uMotionVector.ch = 2;
    uDIReservoir.data = (DIReservoir*)resvThis; uDIReservoir.n = n;
    uDIReservoirPrev.data = (DIReservoir*)resvPrev; uDIReservoirPrev.n = n;
    uDIReservoirTemp.data = (DIReservoir*)resvTemp; uDIReservoirTemp.n = n;

    if (passes & 1) {
#pragma omp parallel for schedule(dynamic, 2)
        for (int y = 0; y < H; y++)
            for (int x = 0; x < W; x++) { vec3 c = generatePath(uvec2(x, y), uCamera.filmSize); (void)c; }
        dref_clear_padding((DIReservoir*)resvThis, n);
    }
    if (passes & 2) {
#pragma omp parallel for schedule(dynamic, 2)
        for (int y = 0; y < H; y++)
            for (int x = 0; x < W; x++) { vec3 c = temporalReuse(uvec2(x, y), uCamera.filmSize); (void)c; }
        dref_clear_padding((DIReservoir*)resvTemp, n);
    }
    if (passes & 4) {
        float frameCount = float(uCamera.frameIndex & CameraFrameIndexMask);
#pragma omp parallel for schedule(dynamic, 2)
        for (int y = 0; y < H; y++)
            for (int x = 0; x < W; x++) {
                vec3 radiance = spatialReuse(uvec2(x, y), uCamera.filmSize);
                float* o = output + ((size_t)y * W + x) * 4;
                vec3 acc = vec3(o[0], o[1], o[2]);
                acc = (acc * frameCount + radiance) / (frameCount + 1.0f);
                o[0] = acc.x; o[1] = acc.y; o[2] = acc.z; o[3] = 1.0f;
            }
        dref_clear_padding((DIReservoir*)resvThis, n);
    }
}

}  /* extern "C" */

}  /* namespace glsl */
