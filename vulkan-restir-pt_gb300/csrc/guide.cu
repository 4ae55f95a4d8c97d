/* guide.cu — the guiding network's kernels: inference (features -> raw mixture parameters),
 * the loss gradient (forward, per-sample vMF-mixture gradient, backward through the MLP, weight
 * gradients), Adam, and the packing of the FP32 master weights into the BF16 copy the tensor
 * cores read. Matrix products are mma.sync m16n8k16 BF16 with FP32 accumulation; a warp keeps
 * 16 samples' activations in registers through the whole network (the accumulator fragments of
 * one layer are the A fragments of the next). */
#include <cuda_bf16.h>
#include <cuda_runtime.h>
#include <stdint.h>

#include "guide.cuh"
#include "guide_kernels.h"
#include "grisrt_internal.h"

namespace grisrt {
namespace guide {

/* ---------------------------------------------------------------- shared helpers */
template <int K, int N>
__device__ __forceinline__ void layer_mma(float C[N / 8][4], const uint32_t A[K / 16][4], const __nv_bfloat16* W, int S,
                                          const float* bias, int g, int t) {
#pragma unroll
    for (int nt = 0; nt < N / 8; nt++) {
        float b0 = bias[8 * nt + 2 * t], b1 = bias[8 * nt + 2 * t + 1];
        C[nt][0] = b0; C[nt][1] = b1; C[nt][2] = b0; C[nt][3] = b1;
        const __nv_bfloat16* row = W + (8 * nt + g) * S + 2 * t;
#pragma unroll
        for (int kt = 0; kt < K / 16; kt++) mma16816(C[nt], A[kt], ld_u32(row + 16 * kt), ld_u32(row + 16 * kt + 8));
    }
}

/* ReLU of the accumulators, rounded to BF16, as the A fragments of the next layer */
template <int N>
__device__ __forceinline__ void relu_to_a(const float C[N / 8][4], uint32_t A[N / 16][4]) {
#pragma unroll
    for (int kt = 0; kt < N / 16; kt++) {
        A[kt][0] = pack_bf16(fmaxf(C[2 * kt][0], 0.0f), fmaxf(C[2 * kt][1], 0.0f));
        A[kt][1] = pack_bf16(fmaxf(C[2 * kt][2], 0.0f), fmaxf(C[2 * kt][3], 0.0f));
        A[kt][2] = pack_bf16(fmaxf(C[2 * kt + 1][0], 0.0f), fmaxf(C[2 * kt + 1][1], 0.0f));
        A[kt][3] = pack_bf16(fmaxf(C[2 * kt + 1][2], 0.0f), fmaxf(C[2 * kt + 1][3], 0.0f));
    }
}

__device__ __forceinline__ void load_features(const float* feat, uint32_t r, uint32_t n, float f[9]) {
#pragma unroll
    for (int i = 0; i < 9; i++) f[i] = r < n ? feat[(size_t)r * 9 + i] : 0.0f;
}

__device__ __forceinline__ void encode_a(const float f0[9], const float f1[9], int t, uint32_t A[kIn / 16][4]) {
#pragma unroll
    for (int kt = 0; kt < kIn / 16; kt++) {
        int c = 16 * kt + 2 * t;
        A[kt][0] = pack_bf16(encode(f0, c), encode(f0, c + 1));
        A[kt][1] = pack_bf16(encode(f1, c), encode(f1, c + 1));
        A[kt][2] = pack_bf16(encode(f0, c + 8), encode(f0, c + 9));
        A[kt][3] = pack_bf16(encode(f1, c + 8), encode(f1, c + 9));
    }
}

/* ---------------------------------------------------------------- inference */
__global__ void __launch_bounds__(128) k_guide_forward(FwdArgs a) {
    __shared__ __align__(16) __nv_bfloat16 sW[kPackedW];
    __shared__ float sB[kBiases];
    for (int i = threadIdx.x; i < kPackedW / 8; i += blockDim.x)
        reinterpret_cast<uint4*>(sW)[i] = reinterpret_cast<const uint4*>(a.wPacked)[i];
    for (int i = threadIdx.x; i < kBiases; i += blockDim.x) sB[i] = a.bias[i];
    __syncthreads();
    uint32_t n = a.count ? min(*a.count, a.n) : a.n;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, g = lane >> 2, t = lane & 3;
    const uint32_t warps = gridDim.x * (blockDim.x >> 5);
    for (uint32_t tile = blockIdx.x * (blockDim.x >> 5) + warp; tile * 16u < n; tile += warps) {
        const uint32_t r0 = tile * 16u + g, r1 = r0 + 8u;
        float f0[9], f1[9];
        load_features(a.feat, r0, n, f0);
        load_features(a.feat, r1, n, f1);
        uint32_t A0[kIn / 16][4];
        encode_a(f0, f1, t, A0);
        float C[8][4];
        uint32_t A[4][4];
        layer_mma<kIn, kHid>(C, A0, sW + packed_w(0), stride_w(0), sB + bias_off(0), g, t);
        relu_to_a<kHid>(C, A);
#pragma unroll
        for (int l = 1; l < 4; l++) {
            layer_mma<kHid, kHid>(C, A, sW + packed_w(l), stride_w(l), sB + bias_off(l), g, t);
            relu_to_a<kHid>(C, A);
        }
        float O[kOut / 8][4];
        layer_mma<kHid, kOut>(O, A, sW + packed_w(4), stride_w(4), sB + bias_off(4), g, t);
#pragma unroll
        for (int nt = 0; nt < kRaw / 8; nt++) {
            int c = 8 * nt + 2 * t;
            if (r0 < n) { a.out[(size_t)r0 * kRaw + c] = O[nt][0]; a.out[(size_t)r0 * kRaw + c + 1] = O[nt][1]; }
            if (r1 < n) { a.out[(size_t)r1 * kRaw + c] = O[nt][2]; a.out[(size_t)r1 * kRaw + c + 1] = O[nt][3]; }
        }
    }
}

/* ---------------------------------------------------------------- loss gradient */
/* Dynamic shared memory of k_guide_grad (bytes): packed weights, biases, the CTA's gradient
 * sums (flat FP32 parameter layout) and per warp the transposed layer inputs hT[l][in_l][24],
 * the transposed pre-activation gradient dzT[64][24] and the outputs / their gradient ob[16][49]. */
constexpr int kHtStride = 24;
constexpr int kHtElems = (kIn + 4 * kHid) * kHtStride;
constexpr int kDzElems = kHid * kHtStride;
constexpr int kObStride = 49;
constexpr int kWarpBytes = (kHtElems + kDzElems) * 2 + 16 * kObStride * 4;
constexpr int kGradWarps = 4;
constexpr size_t kGradSmem = (size_t)kPackedW * 2 + kBiases * 4 + (size_t)kParams * 4 + (size_t)kGradWarps * kWarpBytes;
size_t grad_smem_bytes() { return kGradSmem; }

__device__ __forceinline__ int ht_off(int l) { return l == 0 ? 0 : (kIn + (l - 1) * kHid) * kHtStride; }

__device__ __forceinline__ void store_ht(__nv_bfloat16* hT, int col, int row, float v) {
    hT[col * kHtStride + row] = __float2bfloat16_rn(v);
}

__global__ void __launch_bounds__(kGradWarps * 32, 1) k_guide_grad(GradArgs a) {
    extern __shared__ __align__(16) unsigned char smem[];
    __nv_bfloat16* sW = reinterpret_cast<__nv_bfloat16*>(smem);
    float* sB = reinterpret_cast<float*>(smem + kPackedW * 2);
    float* sG = sB + kBiases;
    unsigned char* warpBase = reinterpret_cast<unsigned char*>(sG + kParams);
    for (int i = threadIdx.x; i < kPackedW / 8; i += blockDim.x)
        reinterpret_cast<uint4*>(sW)[i] = reinterpret_cast<const uint4*>(a.wPacked)[i];
    for (int i = threadIdx.x; i < kBiases; i += blockDim.x) sB[i] = a.bias[i];
    for (int i = threadIdx.x; i < kParams; i += blockDim.x) sG[i] = 0.0f;
    __syncthreads();

    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, g = lane >> 2, t = lane & 3;
    __nv_bfloat16* hT = reinterpret_cast<__nv_bfloat16*>(warpBase + (size_t)warp * kWarpBytes);
    __nv_bfloat16* dzT = hT + kHtElems;
    float* ob = reinterpret_cast<float*>(dzT + kDzElems);
    const uint32_t n = a.count ? min(max(*a.count, a.base) - a.base, a.n) : a.n;
    const float invSum = *a.invWeightSum;
    const uint32_t warps = gridDim.x * kGradWarps;

    for (uint32_t tile = blockIdx.x * kGradWarps + warp; tile * 16u < n; tile += warps) {
        const uint32_t r0 = tile * 16u + g, r1 = r0 + 8u;
        /* ---- forward, keeping every layer's input (transposed) */
        float f0[9], f1[9];
        load_features(a.feat, r0, n, f0);
        load_features(a.feat, r1, n, f1);
        uint32_t A0[kIn / 16][4];
#pragma unroll
        for (int kt = 0; kt < kIn / 16; kt++) {
            int c = 16 * kt + 2 * t;
            float v[8] = {encode(f0, c), encode(f0, c + 1), encode(f1, c), encode(f1, c + 1),
                          encode(f0, c + 8), encode(f0, c + 9), encode(f1, c + 8), encode(f1, c + 9)};
            A0[kt][0] = pack_bf16(v[0], v[1]); A0[kt][1] = pack_bf16(v[2], v[3]);
            A0[kt][2] = pack_bf16(v[4], v[5]); A0[kt][3] = pack_bf16(v[6], v[7]);
            store_ht(hT, c, g, v[0]); store_ht(hT, c + 1, g, v[1]);
            store_ht(hT, c, g + 8, v[2]); store_ht(hT, c + 1, g + 8, v[3]);
            store_ht(hT, c + 8, g, v[4]); store_ht(hT, c + 9, g, v[5]);
            store_ht(hT, c + 8, g + 8, v[6]); store_ht(hT, c + 9, g + 8, v[7]);
        }
        float C[8][4];
        uint32_t A[4][4];
        layer_mma<kIn, kHid>(C, A0, sW + packed_w(0), stride_w(0), sB + bias_off(0), g, t);
#pragma unroll
        for (int l = 1; l < 5; l++) {
            __nv_bfloat16* h = hT + ht_off(l);
#pragma unroll
            for (int nt = 0; nt < 8; nt++) {
                int c = 8 * nt + 2 * t;
                store_ht(h, c, g, fmaxf(C[nt][0], 0.0f)); store_ht(h, c + 1, g, fmaxf(C[nt][1], 0.0f));
                store_ht(h, c, g + 8, fmaxf(C[nt][2], 0.0f)); store_ht(h, c + 1, g + 8, fmaxf(C[nt][3], 0.0f));
            }
            relu_to_a<kHid>(C, A);
            if (l < 4) layer_mma<kHid, kHid>(C, A, sW + packed_w(l), stride_w(l), sB + bias_off(l), g, t);
        }
        float O[kOut / 8][4];
        layer_mma<kHid, kOut>(O, A, sW + packed_w(4), stride_w(4), sB + bias_off(4), g, t);
#pragma unroll
        for (int nt = 0; nt < kOut / 8; nt++) {
            int c = 8 * nt + 2 * t;
            ob[g * kObStride + c] = O[nt][0]; ob[g * kObStride + c + 1] = O[nt][1];
            ob[(g + 8) * kObStride + c] = O[nt][2]; ob[(g + 8) * kObStride + c + 1] = O[nt][3];
        }
        __syncwarp();
        /* ---- per-sample gradient of the loss with respect to the outputs */
        if (lane < 16) {
            uint32_t r = tile * 16u + lane;
            float gr[kRaw];
            if (r < n) {
                float raw[kRaw];
                for (int i = 0; i < kRaw; i++) raw[i] = ob[lane * kObStride + i];
                float d[3] = {a.dir[(size_t)r * 3], a.dir[(size_t)r * 3 + 1], a.dir[(size_t)r * 3 + 2]};
                lobes_loss_grad(raw, d, a.weight[r] * invSum, gr);
            } else {
                for (int i = 0; i < kRaw; i++) gr[i] = 0.0f;
            }
            for (int i = 0; i < kRaw; i++) ob[lane * kObStride + i] = gr[i];
            for (int i = kRaw; i < kOut; i++) ob[lane * kObStride + i] = 0.0f;
        }
        __syncwarp();
        /* ---- output layer: db4, dW4 = dz4^T h4, dh4 = dz4 W4 */
        for (int c = lane; c < kOut; c += 32) {
            float s = 0.0f;
            for (int r = 0; r < 16; r++) s += ob[r * kObStride + c];
            if (s != 0.0f) atomicAdd(&sG[param_b(4) + c], s);
        }
        {
            const __nv_bfloat16* h = hT + ht_off(4);
#pragma unroll
            for (int mt = 0; mt < kOut / 16; mt++) {
                int n0 = 16 * mt + g;
                uint32_t Af[4] = {pack_bf16(ob[(2 * t) * kObStride + n0], ob[(2 * t + 1) * kObStride + n0]),
                                  pack_bf16(ob[(2 * t) * kObStride + n0 + 8], ob[(2 * t + 1) * kObStride + n0 + 8]),
                                  pack_bf16(ob[(2 * t + 8) * kObStride + n0], ob[(2 * t + 9) * kObStride + n0]),
                                  pack_bf16(ob[(2 * t + 8) * kObStride + n0 + 8], ob[(2 * t + 9) * kObStride + n0 + 8])};
#pragma unroll
                for (int nt = 0; nt < kHid / 8; nt++) {
                    float D[4] = {0.0f, 0.0f, 0.0f, 0.0f};
                    mma16816(D, Af, ld_u32(h + (8 * nt + g) * kHtStride + 2 * t), ld_u32(h + (8 * nt + g) * kHtStride + 2 * t + 8));
                    float* gw = sG + param_w(4);
                    int c = 8 * nt + 2 * t;
                    atomicAdd(&gw[n0 * kHid + c], D[0]); atomicAdd(&gw[n0 * kHid + c + 1], D[1]);
                    atomicAdd(&gw[(n0 + 8) * kHid + c], D[2]); atomicAdd(&gw[(n0 + 8) * kHid + c + 1], D[3]);
                }
            }
        }
        float dz[8][4];
        {
            uint32_t Ad[kOut / 16][4];
#pragma unroll
            for (int kt = 0; kt < kOut / 16; kt++) {
                int c = 16 * kt + 2 * t;
                Ad[kt][0] = pack_bf16(ob[g * kObStride + c], ob[g * kObStride + c + 1]);
                Ad[kt][1] = pack_bf16(ob[(g + 8) * kObStride + c], ob[(g + 8) * kObStride + c + 1]);
                Ad[kt][2] = pack_bf16(ob[g * kObStride + c + 8], ob[g * kObStride + c + 9]);
                Ad[kt][3] = pack_bf16(ob[(g + 8) * kObStride + c + 8], ob[(g + 8) * kObStride + c + 9]);
            }
            const __nv_bfloat16* W = sW + packed_w(4);
            const int S = stride_w(4);
#pragma unroll
            for (int nt = 0; nt < kHid / 8; nt++) {
                dz[nt][0] = dz[nt][1] = dz[nt][2] = dz[nt][3] = 0.0f;
                int col = 8 * nt + g;
#pragma unroll
                for (int kt = 0; kt < kOut / 16; kt++) {
                    int k = 16 * kt + 2 * t;
                    mma16816(dz[nt], Ad[kt], pack_pair(W + k * S + col, W + (k + 1) * S + col),
                             pack_pair(W + (k + 8) * S + col, W + (k + 9) * S + col));
                }
            }
        }
        /* ---- hidden layers 3..0 */
#pragma unroll
        for (int l = 3; l >= 0; l--) {
            /* dz_l = dh_{l+1} * relu'(input of layer l+1) */
            const __nv_bfloat16* hin = hT + ht_off(l + 1);
#pragma unroll
            for (int nt = 0; nt < 8; nt++) {
                int c = 8 * nt + 2 * t;
                if (!(__bfloat162float(hin[c * kHtStride + g]) > 0.0f)) dz[nt][0] = 0.0f;
                if (!(__bfloat162float(hin[(c + 1) * kHtStride + g]) > 0.0f)) dz[nt][1] = 0.0f;
                if (!(__bfloat162float(hin[c * kHtStride + g + 8]) > 0.0f)) dz[nt][2] = 0.0f;
                if (!(__bfloat162float(hin[(c + 1) * kHtStride + g + 8]) > 0.0f)) dz[nt][3] = 0.0f;
            }
            /* db_l: column sums over the 16 rows */
#pragma unroll
            for (int nt = 0; nt < 8; nt++) {
                float s0 = dz[nt][0] + dz[nt][2], s1 = dz[nt][1] + dz[nt][3];
                s0 += __shfl_xor_sync(0xffffffffu, s0, 4); s1 += __shfl_xor_sync(0xffffffffu, s1, 4);
                s0 += __shfl_xor_sync(0xffffffffu, s0, 8); s1 += __shfl_xor_sync(0xffffffffu, s1, 8);
                s0 += __shfl_xor_sync(0xffffffffu, s0, 16); s1 += __shfl_xor_sync(0xffffffffu, s1, 16);
                if (g == 0) {
                    atomicAdd(&sG[param_b(l) + 8 * nt + 2 * t], s0);
                    atomicAdd(&sG[param_b(l) + 8 * nt + 2 * t + 1], s1);
                }
            }
            /* dzT (BF16) for the weight gradient */
#pragma unroll
            for (int nt = 0; nt < 8; nt++) {
                int c = 8 * nt + 2 * t;
                store_ht(dzT, c, g, dz[nt][0]); store_ht(dzT, c + 1, g, dz[nt][1]);
                store_ht(dzT, c, g + 8, dz[nt][2]); store_ht(dzT, c + 1, g + 8, dz[nt][3]);
            }
            __syncwarp();
            /* dW_l = dz_l^T h_l */
            {
                const __nv_bfloat16* h = hT + ht_off(l);
                const int inl = layer_in(l);
                float* gw = sG + param_w(l);
#pragma unroll
                for (int mt = 0; mt < 4; mt++) {
                    int n0 = 16 * mt + g;
                    uint32_t Af[4] = {ld_u32(dzT + n0 * kHtStride + 2 * t), ld_u32(dzT + (n0 + 8) * kHtStride + 2 * t),
                                      ld_u32(dzT + n0 * kHtStride + 2 * t + 8), ld_u32(dzT + (n0 + 8) * kHtStride + 2 * t + 8)};
                    for (int nt = 0; nt < inl / 8; nt++) {
                        float D[4] = {0.0f, 0.0f, 0.0f, 0.0f};
                        mma16816(D, Af, ld_u32(h + (8 * nt + g) * kHtStride + 2 * t), ld_u32(h + (8 * nt + g) * kHtStride + 2 * t + 8));
                        int c = 8 * nt + 2 * t;
                        atomicAdd(&gw[n0 * inl + c], D[0]); atomicAdd(&gw[n0 * inl + c + 1], D[1]);
                        atomicAdd(&gw[(n0 + 8) * inl + c], D[2]); atomicAdd(&gw[(n0 + 8) * inl + c + 1], D[3]);
                    }
                }
            }
            /* dh_l = dz_l W_l (not needed below the first layer) */
            if (l > 0) {
                uint32_t Ad[4][4];
#pragma unroll
                for (int kt = 0; kt < 4; kt++) {
                    Ad[kt][0] = pack_bf16(dz[2 * kt][0], dz[2 * kt][1]);
                    Ad[kt][1] = pack_bf16(dz[2 * kt][2], dz[2 * kt][3]);
                    Ad[kt][2] = pack_bf16(dz[2 * kt + 1][0], dz[2 * kt + 1][1]);
                    Ad[kt][3] = pack_bf16(dz[2 * kt + 1][2], dz[2 * kt + 1][3]);
                }
                const __nv_bfloat16* W = sW + packed_w(l);
                const int S = stride_w(l);
#pragma unroll
                for (int nt = 0; nt < 8; nt++) {
                    dz[nt][0] = dz[nt][1] = dz[nt][2] = dz[nt][3] = 0.0f;
                    int col = 8 * nt + g;
#pragma unroll
                    for (int kt = 0; kt < 4; kt++) {
                        int k = 16 * kt + 2 * t;
                        mma16816(dz[nt], Ad[kt], pack_pair(W + k * S + col, W + (k + 1) * S + col),
                                 pack_pair(W + (k + 8) * S + col, W + (k + 9) * S + col));
                    }
                }
            }
            __syncwarp();
        }
    }
    __syncthreads();
    for (int i = threadIdx.x; i < kParams; i += blockDim.x) {
        float v = sG[i];
        if (v != 0.0f) atomicAdd(&a.grad[i], v);
    }
}

/* ---------------------------------------------------------------- weights */
__global__ void k_guide_pack(const float* __restrict__ params, __nv_bfloat16* __restrict__ wPacked, float* __restrict__ bias) {
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < kPackedW; i += gridDim.x * blockDim.x) {
        int l = 0;
        while (l < 4 && i >= packed_w(l + 1)) l++;
        int j = i - packed_w(l), row = j / stride_w(l), col = j % stride_w(l);
        float v = col < layer_in(l) ? params[param_w(l) + row * layer_in(l) + col] : 0.0f;
        wPacked[i] = __float2bfloat16_rn(v);
    }
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < kBiases; i += gridDim.x * blockDim.x) {
        int l = 0;
        while (l < 4 && i >= bias_off(l + 1)) l++;
        bias[i] = params[param_b(l) + (i - bias_off(l))];
    }
}

/* One Adam step (bias-corrected; the 1-based step count at *step) on every parameter; the
 * gradient is cleared for the next accumulation. */
__global__ void k_guide_adam(float* __restrict__ params, float* __restrict__ grad, float* __restrict__ m, float* __restrict__ v,
                             const uint32_t* step, float lr, float b1, float b2, float eps) {
    const float tt = (float)*step;
    const float c1 = 1.0f / (1.0f - powf(b1, tt)), c2 = 1.0f / (1.0f - powf(b2, tt));
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < kParams; i += gridDim.x * blockDim.x) {
        float gr = grad[i];
        float mm = b1 * m[i] + (1.0f - b1) * gr;
        float vv = b2 * v[i] + (1.0f - b2) * gr * gr;
        m[i] = mm;
        v[i] = vv;
        params[i] -= lr * (mm * c1) / (sqrtf(vv * c2) + eps);
        grad[i] = 0.0f;
    }
}
__global__ void k_guide_step(uint32_t* step) { *step += 1u; }

/* 1 / sum of the batch's sample weights (a fixed-order FP64 reduction in one block) */
__global__ void __launch_bounds__(256) k_guide_weight_sum(const float* weight, const uint32_t* count, uint32_t base, uint32_t n,
                                                          float* invSum) {
    __shared__ double part[256];
    uint32_t m = count ? min(max(*count, base) - base, n) : n;
    double s = 0.0;
    for (uint32_t i = threadIdx.x; i < m; i += 256) s += (double)weight[i];
    part[threadIdx.x] = s;
    __syncthreads();
    for (int o = 128; o > 0; o >>= 1) {
        if ((int)threadIdx.x < o) part[threadIdx.x] += part[threadIdx.x + o];
        __syncthreads();
    }
    if (threadIdx.x == 0) *invSum = part[0] > 0.0 ? (float)(1.0 / part[0]) : 0.0f;
}

/* ---------------------------------------------------------------- launchers */
cudaError_t launch_forward(const FwdArgs& a, cudaStream_t stream) {
    if (a.tensorCores) return launch_forward_tc(a, stream);
    const int sm = current_sm_count();
    k_guide_forward<<<sm * 4, 128, 0, stream>>>(a);
    return cudaGetLastError();
}

cudaError_t launch_grad(const GradArgs& a, cudaStream_t stream) {
    const int sm = current_sm_count();
    /* the shared-memory attribute is a per-device property of the kernel: set once per device */
    const int attr = once_per_device(kDeviceKeyGuideGradAttr, []() {
        cudaError_t e = cudaFuncSetAttribute(k_guide_grad, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kGradSmem);
        return e == cudaSuccess ? 1 : -(int)e;
    });
    if (attr < 0) return (cudaError_t)(-attr);
    if (!a.invWeightSum) return cudaErrorInvalidValue;
    k_guide_weight_sum<<<1, 256, 0, stream>>>(a.weight, a.count, a.base, a.n, a.invWeightSum);
    if (a.tensorCores) return launch_grad_tc(a, stream);
    k_guide_grad<<<sm, kGradWarps * 32, kGradSmem, stream>>>(a);
    return cudaGetLastError();
}

cudaError_t launch_pack(const float* params, __nv_bfloat16* wPacked, float* bias, cudaStream_t stream) {
    k_guide_pack<<<48, 256, 0, stream>>>(params, wPacked, bias);
    return cudaGetLastError();
}

cudaError_t launch_adam(float* params, float* grad, float* m, float* v, uint32_t* step, float lr, cudaStream_t stream) {
    k_guide_step<<<1, 1, 0, stream>>>(step);
    k_guide_adam<<<(kParams + 255) / 256, 256, 0, stream>>>(params, grad, m, v, step, lr, 0.9f, 0.99f, 1e-8f);
    return cudaGetLastError();
}

}  // namespace guide
}  // namespace grisrt
