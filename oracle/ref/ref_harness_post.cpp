/*
 * ref_harness_post.cpp — runs the reference's own presentation shader (post_proc.frag, compiled
 * as C++ by oracle/ref/make_ref.py) on the CPU, to pin the oracle's restatement of that pass.
 *
 * TEST INFRASTRUCTURE (oracle). Built into oracle/_ref/libpostref.so; only tests/ use it.
 *
 * What the graphics pipeline supplied around the fragment shader (PostProcessFrag.cpp) is
 * supplied here:
 *   - the full-screen quad (PostProcessFrag.cpp:20-27: positions = texture coordinates in
 *     [0,1]^2, post_proc.vert: gl_Position = aPos * 2 - 1) rasterised over a viewport of the
 *     image's size: one fragment per pixel, its interpolated vTexUV taken at the pixel centre as
 *     ((x + 0.5) / W, (y + 0.5) / H);
 *   - the images the shader reads: uDirectOutput and uIndirectOutput (RGBA32F, as the renderer
 *     allocates them, Renderer.cpp:194) and uDepthNormal, of which it reads only the size;
 *   - the push constant {uToneMapping, uCorrectGamma, noDirect, noIndirect}
 *     (PostProcessFrag.h:7-12);
 *   - the B8G8R8A8_UNORM swapchain's conversion of FragColor: NaN -> 0, clamp to [0, 1], then
 *     round(c * 255) with ties up.
 */
#include "ref_common.h"

namespace glsl {

#define main post_proc_main
#include "post_proc.frag"
#undef main

static uint8_t pref_unorm8(float c) {
    if (!(c > 0.0f)) return 0;
    if (c >= 1.0f) return 255;
    return (uint8_t)__builtin_floorf(c * 255.0f + 0.5f);
}

extern "C" {

/* settings: {toneMapping, correctGamma, noDirect, noIndirect}. color: the fragment colours
 * (float4 per pixel, NaN channels as the canonical quiet NaN); rgba8: their UNORM8 conversion
 * (R, G, B, A bytes per pixel). Either output may be null. */
void pref_post(uint W, uint H, const float* direct, const float* indirect, const uint* settings, float* color,
               uint8_t* rgba8) {
    uToneMapping = settings[0];
    uCorrectGamma = settings[1];
    noDirect = settings[2];
    noIndirect = settings[3];
    uDepthNormal.data = nullptr; uDepthNormal.w = (int)W; uDepthNormal.h = (int)H; uDepthNormal.ch = 4;
    uDirectOutput.data = const_cast<float*>(direct); uDirectOutput.w = (int)W; uDirectOutput.h = (int)H;
    uIndirectOutput.data = const_cast<float*>(indirect); uIndirectOutput.w = (int)W; uIndirectOutput.h = (int)H;
    for (uint y = 0; y < H; y++)
        for (uint x = 0; x < W; x++) {
            vTexUV = vec2(((float)x + 0.5f) / (float)W, ((float)y + 0.5f) / (float)H);
            post_proc_main();
            const size_t i = (size_t)y * W + x;
            const float c[4] = {FragColor.x, FragColor.y, FragColor.z, FragColor.w};
            if (color)
                for (int k = 0; k < 4; k++) {
                    uint32_t qnan = 0x7fc00000u;
                    float q;
                    memcpy(&q, &qnan, 4);
                    color[i * 4 + k] = __builtin_isnan(c[k]) ? q : c[k];
                }
            if (rgba8)
                for (int k = 0; k < 4; k++) rgba8[i * 4 + k] = pref_unorm8(c[k]);
        }
}

}  /* extern "C" */

}  /* namespace glsl */
