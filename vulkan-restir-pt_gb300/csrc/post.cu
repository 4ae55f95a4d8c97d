/*
 * post.cu — the presentation pass of the reference (post_proc.frag:16-44) as a CUDA kernel:
 * composition of the direct and indirect outputs, filmic or ACES tone mapping, gamma, and the
 * UNORM8 conversion of the B8G8R8A8_UNORM swapchain, one thread per pixel. HBM-bound: 32 B read
 * and up to 20 B written per pixel.
 */
#include <cuda_runtime.h>

#include "detmath.h"
#include "gris_kernels.h"

namespace grisrt {

struct PostCtx {
    GrisPostBindings b;
    GrisPostSettings set;
};

/* calcFilmic / filmic / ACES (post_proc.frag:16-28), per channel */
__device__ __forceinline__ float calc_filmic(float c) {
    return (c * (c * 0.22f + 0.03f) + 0.002f) / (c * (c * 0.22f + 0.3f) + 0.06f) - 1.0f / 30.0f;
}
__device__ __forceinline__ float filmic(float c) { return calc_filmic(c * 1.6f) / calc_filmic(11.2f); }
__device__ __forceinline__ float aces(float c) { return (c * (c * 2.51f + 0.03f)) / (c * (c * 2.43f + 0.59f) + 0.14f); }
__device__ __forceinline__ float tonemap(float c, uint32_t mode) {
    return mode == 0u ? c : (mode == 1u ? filmic(c) : aces(c));
}
/* UNORM conversion of a colour attachment: NaN -> 0, clamp, round to nearest */
__device__ __forceinline__ uint32_t unorm8(float c) {
    if (!(c > 0.0f)) return 0u;
    if (c >= 1.0f) return 255u;
    return (uint32_t)floorf(c * 255.0f + 0.5f);
}

__global__ void __launch_bounds__(256) k_post(PostCtx P) {
    uint32_t x = blockIdx.x * blockDim.x + threadIdx.x, y = blockIdx.y;
    const uint32_t W = P.b.width, H = P.b.height;
    if (x >= W) return;
    /* vTexUV at the pixel centre; texel ivec2(vec2(textureSize - 1) * vTexUV) (post_proc.frag:31) */
    float u = ((float)x + 0.5f) / (float)W, v = ((float)y + 0.5f) / (float)H;
    uint32_t cx = (uint32_t)((float)(W - 1u) * u), cy = (uint32_t)((float)(H - 1u) * v);
    uint64_t src = (uint64_t)cy * W + cx, dst = (uint64_t)y * W + x;
    float r = 0.0f, g = 0.0f, bl = 0.0f;
    if (P.set.noDirect == 0u) {
        float4 d = __ldg(reinterpret_cast<const float4*>(P.b.directOutput) + src);
        r = r + d.x; g = g + d.y; bl = bl + d.z;
    }
    if (P.set.noIndirect == 0u) {
        float4 d = __ldg(reinterpret_cast<const float4*>(P.b.indirectOutput) + src);
        r = r + d.x; g = g + d.y; bl = bl + d.z;
    }
    r = tonemap(r, P.set.toneMapping); g = tonemap(g, P.set.toneMapping); bl = tonemap(bl, P.set.toneMapping);
    if (P.set.correctGamma != 0u) {
        const float e = 1.0f / 2.2f;
        r = gris_det_powf(r, e); g = gris_det_powf(g, e); bl = gris_det_powf(bl, e);
    }
    if (P.b.color) {   /* a NaN channel is written as the canonical quiet NaN 0x7fc00000 */
        const float qnan = __uint_as_float(0x7fc00000u);
        reinterpret_cast<float4*>(P.b.color)[dst] = make_float4(isnan(r) ? qnan : r, isnan(g) ? qnan : g,
                                                                isnan(bl) ? qnan : bl, 1.0f);
    }
    if (P.b.rgba8)
        reinterpret_cast<uint32_t*>(P.b.rgba8)[dst] = unorm8(r) | (unorm8(g) << 8) | (unorm8(bl) << 16) | (255u << 24);
}

cudaError_t launch_post(const GrisPostBindings& b, const GrisPostSettings& set, cudaStream_t stream) {
    PostCtx P;
    P.b = b;
    P.set = set;
    dim3 block(256), grid((b.width + 255) / 256, b.height);
    k_post<<<grid, block, 0, stream>>>(P);
    return cudaGetLastError();
}

}  // namespace grisrt
