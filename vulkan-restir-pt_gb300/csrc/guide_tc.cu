/* guide_tc.cu — the guiding network's inference on the 5th-generation tensor cores (tcgen05).
 *
 * A CTA holds the weights of all layers in shared memory and runs two independent groups of 128
 * threads; a group carries 128 vertices (one per thread, one accumulator row each) through the
 * five layers: the layer input sits in shared memory as a 128 x K BF16 tile, one elected thread
 * of the group issues the layer's K/16 `tcgen05.mma.cta_group::1.kind::f16` (M = 128, N = 64 or
 * 48, K = 16 each, FP32 accumulation in the group's 64 tensor-memory columns), a
 * `tcgen05.commit` arrives on the group's mbarrier when they are done, and each warp reads its 32
 * accumulator rows back with `tcgen05.ld` (32x32b shape), adds the bias, applies ReLU and writes
 * the next layer's input tile as BF16. The groups synchronise on their own named barriers, so
 * one group's epilogue overlaps the other's matrix products.
 *
 * Shared-memory operand layout (no swizzle, K-major): 8 x 8 BF16 core matrices of 128
 * contiguous bytes (8 rows of 16 B); for a tile of R rows and K columns, core matrix
 * (r / 8, k / 8) starts at ((r / 8) * (K / 8) + k / 8) * 128 B, so the descriptor's leading byte
 * offset (between the two core matrices of a 16-wide K slice) is 128 B and its stride byte
 * offset (between 8-row groups) is K / 8 * 128 B. An MMA's K slice s starts 2 s core matrices in.
 *
 * Every wait on the mbarrier is bounded: on timeout the kernel sets the error word, commits once
 * more and waits (bounded) on that commit, so that no MMA it issued is still running, then frees
 * its tensor memory and returns.
 */
#include <cuda_bf16.h>
#include <cuda_runtime.h>
#include <stdint.h>

#include "guide.cuh"
#include "guide_kernels.h"
#include "grisrt_internal.h"

namespace grisrt {
namespace guide {

#if defined(__CUDA_ARCH__) && (__CUDA_ARCH__ >= 1000)
#define GRIS_TC_DEVICE 1
#endif

constexpr int kTcRows = 128;                 /* vertices per group tile = MMA M */
constexpr int kTcGroups = 2;                 /* independent groups (tiles in flight) per CTA */
constexpr uint32_t kTmemCols = 64 * kTcGroups;   /* accumulator columns: 64 per group (N <= 64) */
constexpr uint64_t kWaitNs = 200000000ull;   /* a wait on the mbarrier gives up after 0.2 s */
constexpr uint32_t kWaitPolls = 1u << 26;    /* and after this many polls in any case */

/* byte offset of core matrix (row, k) inside a tile of K columns */
__host__ __device__ constexpr uint32_t core_off(uint32_t row, uint32_t k, uint32_t K) {
    return ((row >> 3) * (K >> 3) + (k >> 3)) * 128u + (row & 7u) * 16u;
}
/* shared memory: weights of the five layers (tile of layer_out x layer_in), the layer-input
 * tile (128 x 80 at most), biases, mbarrier, tensor-memory address slot */
__host__ __device__ constexpr uint32_t tc_w_off(int l) {
    return l == 0 ? 0u : tc_w_off(l - 1) + (uint32_t)(layer_out(l - 1) * layer_in(l - 1)) * 2u;
}
constexpr uint32_t kTcA = tc_w_off(5);                                  /* 40960 */
constexpr uint32_t kTcATile = (uint32_t)(kTcRows * kIn) * 2u;           /* 20480 per group */
constexpr uint32_t kTcBias = kTcA + kTcATile * (uint32_t)kTcGroups;
constexpr uint32_t kTcBar = kTcBias + (uint32_t)kBiases * 4u;           /* one mbarrier per group */
constexpr uint32_t kTcSlot = kTcBar + 8u * (uint32_t)kTcGroups;
constexpr uint32_t kTcSmem = kTcSlot + 8u + 1024u;                      /* + alignment slack */
static_assert(kTcA % 1024u == 0u && kTcBar % 8u == 0u, "operand tiles 1024-B aligned, mbarrier 8-B aligned");

size_t tc_smem_bytes() { return kTcSmem; }

/* instruction descriptor of kind::f16: D FP32, A and B BF16, both K-major, M = 128, N = n */
__host__ __device__ constexpr uint32_t tc_idesc(uint32_t n) {
    return (1u << 4) | (1u << 7) | (1u << 10) | ((n >> 3) << 17) | ((uint32_t)(kTcRows >> 4) << 24);
}

#ifdef GRIS_TC_DEVICE
__device__ __forceinline__ uint32_t smem_u32(const void* p) { return (uint32_t)__cvta_generic_to_shared(p); }

/* shared-memory matrix descriptor: start address, leading / stride byte offsets (16-B units),
 * descriptor version 1, no swizzle */
__device__ __forceinline__ uint64_t tc_sdesc(uint32_t addr, uint32_t lbo, uint32_t sbo) {
    return (uint64_t)((addr & 0x3ffffu) >> 4) | ((uint64_t)((lbo >> 4) & 0x3fffu) << 16) |
           ((uint64_t)((sbo >> 4) & 0x3fffu) << 32) | (1ull << 46);
}

__device__ __forceinline__ void tc_mma(uint32_t tmem, uint64_t a, uint64_t b, uint32_t idesc, uint32_t acc) {
    asm volatile(
        "{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n"
        " tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}\n"
        :: "r"(tmem), "l"(a), "l"(b), "r"(idesc), "r"(acc) : "memory");
}
__device__ __forceinline__ void tc_commit(uint32_t bar) {
    asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" :: "r"(bar) : "memory");
}
__device__ __forceinline__ bool bar_try(uint32_t bar, uint32_t parity) {
    uint32_t ok;
    asm volatile("{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}\n"
                 : "=r"(ok) : "r"(bar), "r"(parity) : "memory");
    return ok != 0u;
}
__device__ __forceinline__ uint64_t global_ns() {
    uint64_t t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    return t;
}
/* bounded wait for the phase `parity` of the mbarrier (0.2 s of the global timer, or the poll
 * limit); false: gave up */
__device__ __forceinline__ bool bar_wait(uint32_t bar, uint32_t parity) {
    if (bar_try(bar, parity)) return true;
    const uint64_t t0 = global_ns();
    for (uint32_t i = 1; i < kWaitPolls; i++) {
        if (bar_try(bar, parity)) return true;
        if ((i & 255u) == 0u && global_ns() - t0 > kWaitNs) return false;
    }
    return false;
}
__device__ __forceinline__ void tc_ld16(uint32_t taddr, uint32_t r[16]) {
    asm volatile("tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, [%16];"
                 : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
                   "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
                 : "r"(taddr));
}
__device__ __forceinline__ void tc_wait_ld() { asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory"); }
__device__ __forceinline__ void tc_fence_before() { asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void tc_fence_after() { asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void fence_async_smem() { asm volatile("fence.proxy.async.shared::cta;" ::: "memory"); }
/* barrier of one group's 128 threads (named barrier 1 + group) */
__device__ __forceinline__ void group_sync(uint32_t g) { asm volatile("bar.sync %0, %1;" :: "r"(1u + g), "r"(kTcRows) : "memory"); }

/* ReLU(acc + bias) of 16 columns [c, c + 16) of this thread's row, as BF16 into the next tile */
__device__ __forceinline__ void store_hidden16(unsigned char* tile, uint32_t row, uint32_t c, const uint32_t r[16],
                                               const float* bias) {
    uint32_t w[8];
#pragma unroll
    for (int i = 0; i < 8; i++) {
        float a = fmaxf(__uint_as_float(r[2 * i]) + bias[c + 2 * i], 0.0f);
        float b = fmaxf(__uint_as_float(r[2 * i + 1]) + bias[c + 2 * i + 1], 0.0f);
        w[i] = pack_bf16(a, b);
    }
    *reinterpret_cast<uint4*>(tile + core_off(row, c, kHid)) = make_uint4(w[0], w[1], w[2], w[3]);
    *reinterpret_cast<uint4*>(tile + core_off(row, c + 8, kHid)) = make_uint4(w[4], w[5], w[6], w[7]);
}
#endif

__global__ void __launch_bounds__(kTcRows * kTcGroups, 2) k_guide_forward_tc(FwdArgs a) {
#ifdef GRIS_TC_DEVICE
    extern __shared__ unsigned char smemRaw[];
    unsigned char* smem = reinterpret_cast<unsigned char*>((reinterpret_cast<uintptr_t>(smemRaw) + 1023u) & ~(uintptr_t)1023u);
    const uint32_t ctaThreads = (uint32_t)(kTcRows * kTcGroups);
    const uint32_t grp = threadIdx.x / (uint32_t)kTcRows;     /* this thread's group */
    const uint32_t tid = threadIdx.x % (uint32_t)kTcRows;     /* = its row in the group's tile */
    const uint32_t warp = tid >> 5;                           /* warp within the group: TMEM lanes 32 warp.. */
    unsigned char* sA = smem + kTcA + grp * kTcATile;
    float* sBias = reinterpret_cast<float*>(smem + kTcBias);
    const uint32_t bar = smem_u32(smem + kTcBar + 8u * grp);
    uint32_t* slot = reinterpret_cast<uint32_t*>(smem + kTcSlot);
    __shared__ uint32_t sFail[kTcGroups];

    /* weights into the core-matrix layout (16-B chunks: row n, columns 8kg..8kg+7) and biases */
    for (int l = 0; l < 5; l++) {
        const int K = layer_in(l), N = layer_out(l), chunks = N * (K / 8);
        for (int i = (int)threadIdx.x; i < chunks; i += (int)ctaThreads) {
            int n = i / (K / 8), kg = i % (K / 8);
            uint4 v = *reinterpret_cast<const uint4*>(a.wPacked + packed_w(l) + n * stride_w(l) + 8 * kg);
            *reinterpret_cast<uint4*>(smem + tc_w_off(l) + core_off((uint32_t)n, (uint32_t)(8 * kg), (uint32_t)K)) = v;
        }
    }
    for (int i = (int)threadIdx.x; i < kBiases; i += (int)ctaThreads) sBias[i] = a.bias[i];
    if (tid == 0) {
        sFail[grp] = 0u;
        asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" :: "r"(bar) : "memory");
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    if (threadIdx.x < 32u) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" :: "r"(smem_u32(slot)), "r"(kTmemCols)
                     : "memory");
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
    }
    fence_async_smem();
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    const uint32_t tmemBase = *slot;
    const uint32_t tmem = tmemBase + 64u * grp;                 /* the group's accumulator columns */
    const uint32_t myLanes = tmem + ((warp * 32u) << 16);
    uint32_t phase = 0u;
    const uint32_t n = a.count ? min(*a.count, a.n) : a.n;

    for (uint32_t tile = blockIdx.x * kTcGroups + grp; tile * (uint32_t)kTcRows < n; tile += gridDim.x * kTcGroups) {
        const uint32_t row = tid, v = tile * (uint32_t)kTcRows + tid;
        /* layer-0 input: the encoding of this thread's vertex (zeros past the end) */
        float f[9];
#pragma unroll
        for (int i = 0; i < 9; i++) f[i] = v < n ? a.feat[(size_t)v * 9 + i] : 0.0f;
        /* position encoding per coordinate: 12 sines then 12 cosines = three 8-column chunks */
#pragma unroll
        for (int c = 0; c < 3; c++) {
            float sv[12], cv[12];
#pragma unroll
            for (int j = 0; j < 12; j++) sincospif(f[c] * (float)(1 << j), &sv[j], &cv[j]);
            unsigned char* base = sA + core_off(row, (uint32_t)(24 * c), kIn);
            *reinterpret_cast<uint4*>(base) =
                make_uint4(pack_bf16(sv[0], sv[1]), pack_bf16(sv[2], sv[3]), pack_bf16(sv[4], sv[5]), pack_bf16(sv[6], sv[7]));
            *reinterpret_cast<uint4*>(base + 128) =
                make_uint4(pack_bf16(sv[8], sv[9]), pack_bf16(sv[10], sv[11]), pack_bf16(cv[0], cv[1]), pack_bf16(cv[2], cv[3]));
            *reinterpret_cast<uint4*>(base + 256) =
                make_uint4(pack_bf16(cv[4], cv[5]), pack_bf16(cv[6], cv[7]), pack_bf16(cv[8], cv[9]), pack_bf16(cv[10], cv[11]));
        }
        /* normal, direction towards the previous vertex, two zeros */
        *reinterpret_cast<uint4*>(sA + core_off(row, 72u, kIn)) =
            make_uint4(pack_bf16(f[3], f[4]), pack_bf16(f[5], f[6]), pack_bf16(f[7], f[8]), pack_bf16(0.0f, 0.0f));
        fence_async_smem();
        tc_fence_before();
        group_sync(grp);
        bool ok = sFail[grp] == 0u;
        for (int l = 0; l < 5 && ok; l++) {
            const uint32_t K = (uint32_t)layer_in(l), N = (uint32_t)layer_out(l);
            if (tid == 0) {
                tc_fence_after();
                const uint32_t aBase = smem_u32(sA), bBase = smem_u32(smem + tc_w_off(l));
                for (uint32_t s = 0; s < K / 16u; s++)
                    tc_mma(tmem, tc_sdesc(aBase + s * 256u, 128u, (K / 8u) * 128u),
                           tc_sdesc(bBase + s * 256u, 128u, (K / 8u) * 128u), tc_idesc(N), s > 0u ? 1u : 0u);
                if (!a.withholdCommit) tc_commit(bar);
            }
            if (!bar_wait(bar, phase)) {
                sFail[grp] = 1u;
                if (a.err) atomicOr(a.err, 2ull);
            }
            phase ^= 1u;
            tc_fence_after();
            group_sync(grp);
            ok = sFail[grp] == 0u;
            if (!ok) break;
            const float* bias = sBias + bias_off(l);
            if (l < 4) {
#pragma unroll
                for (uint32_t c = 0; c < (uint32_t)kHid; c += 16u) {
                    uint32_t r[16];
                    tc_ld16(myLanes + c, r);
                    tc_wait_ld();
                    store_hidden16(sA, row, c, r, bias);
                }
                fence_async_smem();
                tc_fence_before();
                group_sync(grp);
            } else {
#pragma unroll
                for (uint32_t c = 0; c < 48u; c += 16u) {
                    uint32_t r[16];
                    tc_ld16(myLanes + c, r);
                    tc_wait_ld();
                    if (v < n) {
#pragma unroll
                        for (uint32_t i = 0; i < 16u; i++)
                            if (c + i < (uint32_t)kRaw) a.out[(size_t)v * kRaw + c + i] = __uint_as_float(r[i]) + bias[c + i];
                    }
                }
                tc_fence_before();
                group_sync(grp);
            }
        }
        if (!ok) break;
    }
    /* After a timeout the phase waited on (parity phase ^ 1, `phase` having been flipped since) is
     * still open: a commit now arrives on it once every matrix product this thread issued has
     * completed, and one more bounded wait on that phase drains them before the tensor memory is
     * freed. Bit 2 of the error word records a drain that did not finish either. */
    if (sFail[grp] && tid == 0) {
        tc_commit(bar);
        if (!bar_wait(bar, phase ^ 1u) && a.err) atomicOr(a.err, 4ull);
    }
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    if (threadIdx.x < 32u)
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" :: "r"(tmemBase), "r"(kTmemCols) : "memory");
#endif
}

cudaError_t launch_forward_tc(const FwdArgs& a, cudaStream_t stream) {
    const int sm = current_sm_count();
    /* the shared-memory attribute is a per-device property of the kernel: set once per device */
    const int attr = once_per_device(kDeviceKeyGuideTcAttr, []() {
        cudaError_t e = cudaFuncSetAttribute(k_guide_forward_tc, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kTcSmem);
        return e == cudaSuccess ? 1 : -(int)e;
    });
    if (attr < 0) return (cudaError_t)(-attr);
    k_guide_forward_tc<<<sm * 2, kTcRows * kTcGroups, kTcSmem, stream>>>(a);
    return cudaGetLastError();
}

}  // namespace guide
}  // namespace grisrt
