/* guide.cuh — the guiding network's device side: layout of its parameters, the input encoding,
 * BF16 tensor-core fragments (mma.sync m16n8k16, FP32 accumulation) and the 8-lobe von
 * Mises-Fisher mixture it predicts (density, sampling).
 *
 * Network: 80 -> 64 -> 64 -> 64 -> 64 (ReLU) -> 48 (linear, the first 40 used).
 * Input (78 values, zero-padded to 80): the vertex position p normalised to the scene box, as
 * sin(2^k pi p), cos(2^k pi p), k = 0..11 per coordinate (x: 12 sines then 12 cosines, then y,
 * then z), the shading normal and the direction towards the previous vertex.
 * Output per lobe j (values 5j..5j+4): a direction m (mu = m / |m|), a log-concentration
 * (kappa = exp(clamp(k, -4, 7))) and a logit (weights = softmax over the lobes).
 * vMF density: kappa / (2 pi (1 - exp(-2 kappa))) exp(kappa (mu . w - 1)).
 */
#pragma once
#include <cuda_bf16.h>
#include <stdint.h>

namespace grisrt {
namespace guide {

constexpr int kIn = 80, kHid = 64, kOut = 48, kLobes = 8, kRaw = 40, kLayers = 5;
constexpr float kKappaMin = -4.0f, kKappaMax = 7.0f;
/* per layer: inputs, outputs, offset of W (out x in, row-major) and b in the flat FP32 parameters */
__host__ __device__ constexpr int layer_in(int l) { return l == 0 ? kIn : kHid; }
__host__ __device__ constexpr int layer_out(int l) { return l == 4 ? kOut : kHid; }
__host__ __device__ constexpr int param_w(int l) {
    return l == 0 ? 0 : param_w(l - 1) + layer_in(l - 1) * layer_out(l - 1) + layer_out(l - 1);
}
__host__ __device__ constexpr int param_b(int l) { return param_w(l) + layer_in(l) * layer_out(l); }
constexpr int kParams = param_b(4) + layer_out(4);   /* 20784 */
/* BF16 copy for the tensor cores: rows padded to in + 8 elements (conflict-free fragment loads) */
__host__ __device__ constexpr int stride_w(int l) { return layer_in(l) + 8; }
__host__ __device__ constexpr int packed_w(int l) { return l == 0 ? 0 : packed_w(l - 1) + layer_out(l - 1) * stride_w(l - 1); }
constexpr int kPackedW = packed_w(4) + layer_out(4) * stride_w(4);   /* 22912 BF16 */
__host__ __device__ constexpr int bias_off(int l) { return l == 0 ? 0 : bias_off(l - 1) + layer_out(l - 1); }
constexpr int kBiases = bias_off(4) + layer_out(4);    /* 304 */
static_assert(kParams == 20784, "parameter count");
static_assert((kPackedW * 2) % 16 == 0, "16-byte copies of the packed weights");

#if defined(__CUDACC__)
/* ---------------------------------------------------------------- tensor-core fragments */
/* D(16x8, FP32) += A(16x16, BF16, row) * B(16x8, BF16, col). Fragment ownership (g = lane/4,
 * t = lane%4): a[0] (g, 2t..2t+1), a[1] (g+8, 2t..), a[2] (g, 2t+8..), a[3] (g+8, 2t+8..);
 * b[0] (k 2t..2t+1, n g), b[1] (k 2t+8.., n g); c[0..1] (g, 2t..2t+1), c[2..3] (g+8, 2t..). */
__device__ __forceinline__ void mma16816(float c[4], const uint32_t a[4], uint32_t b0, uint32_t b1) {
    asm volatile("mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, {%0,%1,%2,%3};\n"
                 : "+f"(c[0]), "+f"(c[1]), "+f"(c[2]), "+f"(c[3])
                 : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(b0), "r"(b1));
}
__device__ __forceinline__ uint32_t pack_bf16(float lo, float hi) {
    __nv_bfloat162 v = __floats2bfloat162_rn(lo, hi);
    return *reinterpret_cast<uint32_t*>(&v);
}
__device__ __forceinline__ uint32_t ld_u32(const __nv_bfloat16* p) { return *reinterpret_cast<const uint32_t*>(p); }
__device__ __forceinline__ uint32_t pack_pair(const __nv_bfloat16* lo, const __nv_bfloat16* hi) {
    uint32_t a = *reinterpret_cast<const uint16_t*>(lo), b = *reinterpret_cast<const uint16_t*>(hi);
    return a | (b << 16);
}

/* ---------------------------------------------------------------- encoding */
/* Input value `col` (0..79) of a vertex: f[0..2] position in [0,1], f[3..5] normal, f[6..8] wo. */
__device__ __forceinline__ float encode(const float f[9], int col) {
    if (col < 72) {
        int c = col / 24, j = col % 24;
        float x = f[c] * (float)(1 << (j % 12));   /* exact: a power of two */
        float s, co;
        sincospif(x, &s, &co);
        return j < 12 ? s : co;
    }
    if (col < 78) return f[col - 69];
    return 0.0f;
}

/* ---------------------------------------------------------------- the mixture */
struct Lobes {
    float mu[kLobes][3];
    float kappa[kLobes];
    float w[kLobes];       /* softmax weights */
    float norm[kLobes];    /* kappa / (2 pi (1 - exp(-2 kappa))) */
};

__device__ __forceinline__ void make_lobes(const float* raw, Lobes& L) {
    float mx = -3.0e38f;
    for (int j = 0; j < kLobes; j++) mx = fmaxf(mx, raw[5 * j + 4]);
    float sum = 0.0f;
    for (int j = 0; j < kLobes; j++) {
        float m0 = raw[5 * j], m1 = raw[5 * j + 1], m2 = raw[5 * j + 2];
        float len = sqrtf(m0 * m0 + m1 * m1 + m2 * m2);
        float inv = len > 1e-12f ? 1.0f / len : 0.0f;
        L.mu[j][0] = m0 * inv; L.mu[j][1] = m1 * inv; L.mu[j][2] = m2 * inv;
        if (len <= 1e-12f) { L.mu[j][0] = 0.0f; L.mu[j][1] = 0.0f; L.mu[j][2] = 1.0f; }
        float k = expf(fminf(fmaxf(raw[5 * j + 3], kKappaMin), kKappaMax));
        L.kappa[j] = k;
        L.norm[j] = k / (6.283185307179586f * (-expm1f(-2.0f * k)));
        float e = expf(raw[5 * j + 4] - mx);
        L.w[j] = e;
        sum += e;
    }
    float inv = 1.0f / sum;
    for (int j = 0; j < kLobes; j++) L.w[j] *= inv;
}

__device__ __forceinline__ float lobes_pdf(const Lobes& L, float x, float y, float z) {
    float p = 0.0f;
    for (int j = 0; j < kLobes; j++) {
        float c = L.mu[j][0] * x + L.mu[j][1] * y + L.mu[j][2] * z;
        p += L.w[j] * L.norm[j] * expf(L.kappa[j] * (c - 1.0f));
    }
    return p;
}

/* Direction from the mixture: a lobe by u0 over the weights, then the vMF by (u1, u2)
 * (Jakob 2012: cos = 1 + log(u1 + (1 - u1) exp(-2 kappa)) / kappa, phi = 2 pi u2). */
__device__ __forceinline__ void lobes_sample(const Lobes& L, float u0, float u1, float u2, float d[3]) {
    int j = 0;
    float acc = L.w[0];
    while (j < kLobes - 1 && u0 >= acc) { j++; acc += L.w[j]; }
    float k = L.kappa[j];
    float cz = 1.0f + logf(u1 + (1.0f - u1) * expf(-2.0f * k)) / k;
    cz = fminf(fmaxf(cz, -1.0f), 1.0f);
    float s = sqrtf(fmaxf(0.0f, 1.0f - cz * cz));
    float sp, cp;
    sincospif(2.0f * u2, &sp, &cp);
    const float* m = L.mu[j];
    float tx, ty, tz;
    if (fabsf(m[2]) > 0.999f) { tx = 0.0f; ty = 1.0f; tz = 0.0f; } else { tx = 0.0f; ty = 0.0f; tz = 1.0f; }
    /* b = normalize(m x t), t' = b x m */
    float bx = m[1] * tz - m[2] * ty, by = m[2] * tx - m[0] * tz, bz = m[0] * ty - m[1] * tx;
    float bl = rsqrtf(bx * bx + by * by + bz * bz);
    bx *= bl; by *= bl; bz *= bl;
    float ux = by * m[2] - bz * m[1], uy = bz * m[0] - bx * m[2], uz = bx * m[1] - by * m[0];
    d[0] = ux * (s * cp) + bx * (s * sp) + m[0] * cz;
    d[1] = uy * (s * cp) + by * (s * sp) + m[1] * cz;
    d[2] = uz * (s * cp) + bz * (s * sp) + m[2] * cz;
    float inv = rsqrtf(d[0] * d[0] + d[1] * d[1] + d[2] * d[2]);
    d[0] *= inv; d[1] *= inv; d[2] *= inv;
}

/* d loss_i / d raw for loss_i = -wn_i log p(w_i) (wn: the sample's normalised weight); raw[40] in,
 * g[40] out. */
__device__ __forceinline__ void lobes_loss_grad(const float* raw, const float w[3], float wn, float* g) {
    Lobes L;
    make_lobes(raw, L);
    float lp[kLobes], mx = -3.0e38f;
    for (int j = 0; j < kLobes; j++) {
        float c = L.mu[j][0] * w[0] + L.mu[j][1] * w[1] + L.mu[j][2] * w[2];
        lp[j] = logf(L.w[j]) + logf(L.norm[j]) + L.kappa[j] * (c - 1.0f);
        mx = fmaxf(mx, lp[j]);
    }
    float s = 0.0f;
    for (int j = 0; j < kLobes; j++) s += expf(lp[j] - mx);
    float logp = mx + logf(s);
    for (int j = 0; j < kLobes; j++) {
        float r = expf(lp[j] - logp);
        float gl = -wn;                                   /* d loss / d log p */
        g[5 * j + 4] = gl * (r - L.w[j]);
        float k = L.kappa[j];
        float c = L.mu[j][0] * w[0] + L.mu[j][1] * w[1] + L.mu[j][2] * w[2];
        float e2 = expf(-2.0f * k);
        float dk = 1.0f / k - 2.0f * e2 / (-expm1f(-2.0f * k)) + (c - 1.0f);
        float kr = raw[5 * j + 3];
        g[5 * j + 3] = (kr > kKappaMin && kr < kKappaMax) ? gl * r * dk * k : 0.0f;
        float m0 = raw[5 * j], m1 = raw[5 * j + 1], m2 = raw[5 * j + 2];
        float len = sqrtf(m0 * m0 + m1 * m1 + m2 * m2);
        float il = len > 1e-12f ? 1.0f / len : 0.0f;
        /* d lv / d m = kappa (w - (mu.w) mu) / |m| */
        for (int a = 0; a < 3; a++) g[5 * j + a] = gl * r * k * (w[a] - c * L.mu[j][a]) * il;
    }
}

#endif  // __CUDACC__

}  // namespace guide
}  // namespace grisrt
