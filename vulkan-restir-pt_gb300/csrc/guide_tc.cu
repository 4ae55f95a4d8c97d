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

/* ================================================================ loss gradient on tcgen05 */
/* One CTA of 128 threads per SM walks 128-record tiles (one thread per record = one accumulator
 * row). Per tile:
 *   forward   five layers as in k_guide_forward_tc, every layer's input tile kept in shared
 *             memory (the backward pass needs them);
 *   loss      each thread turns its record's 40 outputs into d loss / d outputs (lobes_loss_grad);
 *   backward  per layer l = 4..0 one elected thread issues
 *               dW_l^T += H_l^T dZ_l   (M = 128 input rows, N = out_l, K = the tile's 128 records)
 *             into the layer's own tensor-memory accumulator, which stays resident across all
 *             the CTA's tiles (this replaces the per-warp shared-memory atomic fold), and for l > 0
 *               dH_l = dZ_l W_l        (M = 128 records, N = in_l = 64, K = out_l),
 *             whose rows the threads read back to form dZ_{l-1} = dH_l * [H_l > 0].
 * H_l^T and dZ_l^T (K = records) are written transposed into two scratch tiles; row in_l of H_l^T
 * holds ones, so that row of the accumulator is the bias gradient sum_r dZ_l[r]. At the end each
 * thread reads its accumulator rows and adds them to the gradient (one atomic per parameter and
 * CTA). Operands: K-major, no swizzle, the core-matrix layout of k_guide_forward_tc; all MMAs are
 * cta_group::1 kind::f16 with M = 128. Every mbarrier wait is bounded as in the inference kernel.
 *
 * Shared memory (from a 1024-B aligned base; every tile 1024-B aligned):
 *   [0, 40960)        W_l, forward B operands (N = out_l rows, K = in_l)          tc_w_off(l)
 *   [40960, 71680)    W_l^T, l = 1..4, dH B operands (N = in_l rows, K = out_l)   kGtWT + gt_wt_off(l)
 *   [71680, 92160)    H_0: layer-0 inputs, 128 records x 80
 *   [92160, 157696)   H_1..H_4: inputs of layers 1..4, 128 records x 64 each
 *   [157696, 174080)  dZ_l, 128 records x out_l (A of dH)
 *   [174080, 206848)  H_l^T: 128 rows (inputs; row in_l = ones) x 128 records (A of dW^T)
 *   [206848, 223232)  dZ_l^T: out_l rows x 128 records (B of dW^T)
 *   then biases (304 floats), the mbarrier and the tensor-memory address slot.
 * Tensor memory: 512 columns; [0, 64) the forward / dH accumulator, 64 + 64 l the dW_l^T
 * accumulator (N = out_l columns). */
__host__ __device__ constexpr uint32_t gt_wt_off(int l) { return l <= 1 ? 0u : gt_wt_off(l - 1) + (uint32_t)(layer_in(l - 1) * layer_out(l - 1)) * 2u; }
constexpr uint32_t kGtWT = tc_w_off(5);                                 /* 40960 */
constexpr uint32_t kGtH0 = kGtWT + gt_wt_off(5);                        /* 71680 */
constexpr uint32_t kGtH = kGtH0 + (uint32_t)(kTcRows * kIn) * 2u;       /* 92160 */
constexpr uint32_t kGtHTile = (uint32_t)(kTcRows * kHid) * 2u;          /* 16384 */
constexpr uint32_t kGtDZ = kGtH + 4u * kGtHTile;                        /* 157696 */
constexpr uint32_t kGtHT = kGtDZ + kGtHTile;                            /* 174080 */
constexpr uint32_t kGtDZT = kGtHT + 128u * 128u * 2u;                   /* 206848 */
constexpr uint32_t kGtBias = kGtDZT + 64u * 128u * 2u;                  /* 223232 */
constexpr uint32_t kGtBar = kGtBias + (uint32_t)kBiases * 4u;
constexpr uint32_t kGtSlot = kGtBar + 8u;
constexpr uint32_t kGtSmem = kGtSlot + 8u + 1024u;
constexpr uint32_t kGtTmemCols = 512u;
static_assert(kGtWT == 40960u && kGtH0 == 71680u && kGtDZT == 206848u, "gradient kernel layout");
static_assert(kGtH0 % 1024u == 0u && kGtH % 1024u == 0u && kGtDZ % 1024u == 0u && kGtHT % 1024u == 0u &&
              kGtDZT % 1024u == 0u && kGtBar % 8u == 0u, "operand tiles 1024-B aligned, mbarrier 8-B aligned");
static_assert(kGtSmem <= 232448u, "fits the 227 KB a CTA may opt in to");

size_t tc_grad_smem_bytes() { return kGtSmem; }

#ifdef GRIS_TC_DEVICE
/* one BF16 element (row, k) of a K-major no-swizzle tile of K columns */
__device__ __forceinline__ void st_bf16(unsigned char* tile, uint32_t row, uint32_t k, uint32_t K, float v) {
    *reinterpret_cast<__nv_bfloat16*>(tile + core_off(row, k, K) + (k & 7u) * 2u) = __float2bfloat16_rn(v);
}
__device__ __forceinline__ float ld_bf16(const unsigned char* tile, uint32_t row, uint32_t k, uint32_t K) {
    return __bfloat162float(*reinterpret_cast<const __nv_bfloat16*>(tile + core_off(row, k, K) + (k & 7u) * 2u));
}
/* 8 BF16 values (columns c..c+7, c a multiple of 8) of one row as one 16-B store */
__device__ __forceinline__ void st_row8(unsigned char* tile, uint32_t row, uint32_t c, uint32_t K, const float* v) {
    *reinterpret_cast<uint4*>(tile + core_off(row, c, K)) =
        make_uint4(pack_bf16(v[0], v[1]), pack_bf16(v[2], v[3]), pack_bf16(v[4], v[5]), pack_bf16(v[6], v[7]));
}
#endif

__global__ void __launch_bounds__(kTcRows, 1) k_guide_grad_tc(GradArgs a) {
#ifdef GRIS_TC_DEVICE
    extern __shared__ unsigned char smemRaw[];
    unsigned char* smem = reinterpret_cast<unsigned char*>((reinterpret_cast<uintptr_t>(smemRaw) + 1023u) & ~(uintptr_t)1023u);
    const uint32_t tid = threadIdx.x, warp = tid >> 5;
    float* sBias = reinterpret_cast<float*>(smem + kGtBias);
    const uint32_t bar = smem_u32(smem + kGtBar);
    uint32_t* slot = reinterpret_cast<uint32_t*>(smem + kGtSlot);
    unsigned char* sH0 = smem + kGtH0;
    unsigned char* sDZ = smem + kGtDZ;
    unsigned char* sHT = smem + kGtHT;
    unsigned char* sDZT = smem + kGtDZT;
    __shared__ uint32_t sFail;

    /* forward weights (as the inference kernel), transposed weights, biases; H^T's rows past the
     * inputs start at zero */
    for (int l = 0; l < 5; l++) {
        const int K = layer_in(l), N = layer_out(l), chunks = N * (K / 8);
        for (int i = (int)tid; i < chunks; i += kTcRows) {
            int nn = i / (K / 8), kg = i % (K / 8);
            uint4 v = *reinterpret_cast<const uint4*>(a.wPacked + packed_w(l) + nn * stride_w(l) + 8 * kg);
            *reinterpret_cast<uint4*>(smem + tc_w_off(l) + core_off((uint32_t)nn, (uint32_t)(8 * kg), (uint32_t)K)) = v;
        }
    }
    for (int l = 1; l < 5; l++) {
        const int I = layer_in(l), O = layer_out(l);
        unsigned char* wt = smem + kGtWT + gt_wt_off(l);
        for (int i = (int)tid; i < I * O; i += kTcRows) {
            const int in = i / O, o = i % O;   /* element (row in, column o) = W_l[o][in] */
            *reinterpret_cast<__nv_bfloat16*>(wt + core_off((uint32_t)in, (uint32_t)o, (uint32_t)O) + (uint32_t)(o & 7) * 2u) =
                a.wPacked[packed_w(l) + o * stride_w(l) + in];
        }
    }
    for (int i = (int)tid; i < kBiases; i += kTcRows) sBias[i] = a.bias[i];
    for (uint32_t i = tid; i < 128u * 128u * 2u / 16u; i += (uint32_t)kTcRows)
        reinterpret_cast<uint4*>(sHT)[i] = make_uint4(0u, 0u, 0u, 0u);
    if (tid == 0) {
        sFail = 0u;
        asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" :: "r"(bar) : "memory");
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    if (warp == 0) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" :: "r"(smem_u32(slot)), "r"(kGtTmemCols)
                     : "memory");
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
    }
    fence_async_smem();
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    const uint32_t tmem = *slot;
    const uint32_t myLanes = tmem + ((warp * 32u) << 16);
    uint32_t phase = 0u;
    bool ok = true, any = false;
    const uint32_t n = a.count ? min(max(*a.count, a.base) - a.base, a.n) : a.n;
    const float invSum = *a.invWeightSum;

    /* the elected thread issues, commits; every thread waits (bounded) for the phase */
    auto wait_all = [&]() -> bool {
        if (!bar_wait(bar, phase)) {
            sFail = 1u;
            if (a.err) atomicOr(a.err, 2ull);
        }
        phase ^= 1u;
        tc_fence_after();
        __syncthreads();
        return sFail == 0u;
    };

    for (uint32_t tile = blockIdx.x; ok && tile * (uint32_t)kTcRows < n; tile += gridDim.x) {
        const uint32_t r = tile * (uint32_t)kTcRows + tid;
        const bool valid = r < n;
        /* layer-0 input: the encoding of this thread's record (zeros past the end) */
        float f[9];
#pragma unroll
        for (int i = 0; i < 9; i++) f[i] = valid ? a.feat[(size_t)r * 9 + i] : 0.0f;
#pragma unroll
        for (int c = 0; c < 3; c++) {
            float sv[12], cv[12];
#pragma unroll
            for (int j = 0; j < 12; j++) sincospif(f[c] * (float)(1 << j), &sv[j], &cv[j]);
            unsigned char* base = sH0 + core_off(tid, (uint32_t)(24 * c), kIn);
            *reinterpret_cast<uint4*>(base) =
                make_uint4(pack_bf16(sv[0], sv[1]), pack_bf16(sv[2], sv[3]), pack_bf16(sv[4], sv[5]), pack_bf16(sv[6], sv[7]));
            *reinterpret_cast<uint4*>(base + 128) =
                make_uint4(pack_bf16(sv[8], sv[9]), pack_bf16(sv[10], sv[11]), pack_bf16(cv[0], cv[1]), pack_bf16(cv[2], cv[3]));
            *reinterpret_cast<uint4*>(base + 256) =
                make_uint4(pack_bf16(cv[4], cv[5]), pack_bf16(cv[6], cv[7]), pack_bf16(cv[8], cv[9]), pack_bf16(cv[10], cv[11]));
        }
        *reinterpret_cast<uint4*>(sH0 + core_off(tid, 72u, kIn)) =
            make_uint4(pack_bf16(f[3], f[4]), pack_bf16(f[5], f[6]), pack_bf16(f[7], f[8]), pack_bf16(0.0f, 0.0f));
        fence_async_smem();
        tc_fence_before();
        __syncthreads();

        /* ---- forward; raw: this record's 48 outputs */
        float raw[kOut];
        for (int l = 0; l < 5 && ok; l++) {
            const uint32_t K = (uint32_t)layer_in(l), N = (uint32_t)layer_out(l);
            if (tid == 0) {
                tc_fence_after();
                const uint32_t aBase = smem_u32(l == 0 ? sH0 : smem + kGtH + (uint32_t)(l - 1) * kGtHTile);
                const uint32_t bBase = smem_u32(smem + tc_w_off(l));
                for (uint32_t s = 0; s < K / 16u; s++)
                    tc_mma(tmem, tc_sdesc(aBase + s * 256u, 128u, (K / 8u) * 128u),
                           tc_sdesc(bBase + s * 256u, 128u, (K / 8u) * 128u), tc_idesc(N), s > 0u ? 1u : 0u);
                if (!a.withholdCommit) tc_commit(bar);
            }
            ok = wait_all();
            if (!ok) break;
            const float* bias = sBias + bias_off(l);
            if (l < 4) {
                unsigned char* next = smem + kGtH + (uint32_t)l * kGtHTile;
#pragma unroll
                for (uint32_t c = 0; c < (uint32_t)kHid; c += 16u) {
                    uint32_t q[16];
                    tc_ld16(myLanes + c, q);
                    tc_wait_ld();
                    store_hidden16(next, tid, c, q, bias);
                }
            } else {
#pragma unroll
                for (uint32_t c = 0; c < (uint32_t)kOut; c += 16u) {
                    uint32_t q[16];
                    tc_ld16(myLanes + c, q);
                    tc_wait_ld();
#pragma unroll
                    for (uint32_t i = 0; i < 16u; i++) raw[c + i] = __uint_as_float(q[i]) + bias[c + i];
                }
            }
            fence_async_smem();
            tc_fence_before();
            __syncthreads();
        }
        if (!ok) break;

        /* ---- d loss / d outputs of this record: dZ_4 (40 used of 48), with H_4^T */
        {
            float g[kRaw];
            if (valid) {
                const float d[3] = {a.dir[(size_t)r * 3], a.dir[(size_t)r * 3 + 1], a.dir[(size_t)r * 3 + 2]};
                lobes_loss_grad(raw, d, a.weight[r] * invSum, g);
            } else {
#pragma unroll
                for (int i = 0; i < kRaw; i++) g[i] = 0.0f;
            }
            float z8[8] = {0.0f, 0.0f, 0.0f, 0.0f, 0.0f, 0.0f, 0.0f, 0.0f};
#pragma unroll
            for (uint32_t c = 0; c < (uint32_t)kRaw; c += 8u) st_row8(sDZ, tid, c, (uint32_t)kOut, g + c);
            st_row8(sDZ, tid, (uint32_t)kRaw, (uint32_t)kOut, z8);
            for (uint32_t o = 0; o < (uint32_t)kOut; o++) st_bf16(sDZT, o, tid, 128u, o < (uint32_t)kRaw ? g[o] : 0.0f);
            const unsigned char* h4 = smem + kGtH + 3u * kGtHTile;
            for (uint32_t m = 0; m < (uint32_t)kHid; m++) st_bf16(sHT, m, tid, 128u, ld_bf16(h4, tid, m, (uint32_t)kHid));
            st_bf16(sHT, (uint32_t)kHid, tid, 128u, 1.0f);
        }
        fence_async_smem();
        tc_fence_before();
        __syncthreads();

        /* ---- backward */
        for (int l = 4; l >= 0 && ok; l--) {
            const uint32_t I = (uint32_t)layer_in(l), O = (uint32_t)layer_out(l);
            if (tid == 0) {
                tc_fence_after();
                const uint32_t aT = smem_u32(sHT), bT = smem_u32(sDZT);
                const uint32_t acc = tmem + 64u + 64u * (uint32_t)l;
                for (uint32_t s = 0; s < 8u; s++)   /* K = 128 records */
                    tc_mma(acc, tc_sdesc(aT + s * 256u, 128u, 16u * 128u), tc_sdesc(bT + s * 256u, 128u, 16u * 128u),
                           tc_idesc(O), (any || s > 0u) ? 1u : 0u);
                if (l > 0) {
                    const uint32_t aD = smem_u32(sDZ), bW = smem_u32(smem + kGtWT + gt_wt_off(l));
                    for (uint32_t s = 0; s < O / 16u; s++)
                        tc_mma(tmem, tc_sdesc(aD + s * 256u, 128u, (O / 8u) * 128u),
                               tc_sdesc(bW + s * 256u, 128u, (O / 8u) * 128u), tc_idesc(I), s > 0u ? 1u : 0u);
                }
                tc_commit(bar);
            }
            ok = wait_all();
            if (!ok || l == 0) break;
            /* dZ_{l-1} = dH_l * [H_l > 0]; H_l = the input of layer l; then H_{l-1}^T */
            const unsigned char* hl = smem + kGtH + (uint32_t)(l - 1) * kGtHTile;
#pragma unroll
            for (uint32_t c = 0; c < (uint32_t)kHid; c += 16u) {
                uint32_t q[16];
                tc_ld16(myLanes + c, q);
                tc_wait_ld();
                float dz[16];
#pragma unroll
                for (uint32_t i = 0; i < 16u; i++) dz[i] = ld_bf16(hl, tid, c + i, (uint32_t)kHid) > 0.0f ? __uint_as_float(q[i]) : 0.0f;
                st_row8(sDZ, tid, c, (uint32_t)kHid, dz);
                st_row8(sDZ, tid, c + 8u, (uint32_t)kHid, dz + 8);
#pragma unroll
                for (uint32_t i = 0; i < 16u; i++) st_bf16(sDZT, c + i, tid, 128u, dz[i]);
            }
            const uint32_t In = (uint32_t)layer_in(l - 1);
            const unsigned char* hin = l - 1 == 0 ? sH0 : smem + kGtH + (uint32_t)(l - 2) * kGtHTile;
            for (uint32_t m = 0; m < In; m++) st_bf16(sHT, m, tid, 128u, ld_bf16(hin, tid, m, In));
            st_bf16(sHT, In, tid, 128u, 1.0f);
            fence_async_smem();
            tc_fence_before();
            __syncthreads();
        }
        any = true;
    }

    /* ---- the CTA's weight and bias gradients: row m of dW_l^T is input m (m = in_l: the bias) */
    if (ok && any) {
        const uint32_t m = tid;
        for (int l = 0; l < 5; l++) {
            const uint32_t I = (uint32_t)layer_in(l), O = (uint32_t)layer_out(l);
            for (uint32_t c = 0; c < O; c += 16u) {
                uint32_t q[16];
                tc_ld16(myLanes + 64u + 64u * (uint32_t)l + c, q);
                tc_wait_ld();
                if (m < I) {
                    float* gw = a.grad + param_w(l);
#pragma unroll
                    for (uint32_t i = 0; i < 16u; i++) {
                        const float v = __uint_as_float(q[i]);
                        if (v != 0.0f) atomicAdd(gw + (c + i) * I + m, v);
                    }
                } else if (m == I) {
                    float* gb = a.grad + param_b(l);
#pragma unroll
                    for (uint32_t i = 0; i < 16u; i++) {
                        const float v = __uint_as_float(q[i]);
                        if (v != 0.0f) atomicAdd(gb + c + i, v);
                    }
                }
            }
        }
    }
    /* after a timeout: a commit drains the products in flight (see k_guide_forward_tc) */
    if (sFail && tid == 0) {
        tc_commit(bar);
        if (!bar_wait(bar, phase ^ 1u) && a.err) atomicOr(a.err, 4ull);
    }
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    if (warp == 0)
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" :: "r"(tmem), "r"(kGtTmemCols) : "memory");
#endif
}

cudaError_t launch_grad_tc(const GradArgs& a, cudaStream_t stream) {
    const int sm = current_sm_count();
    const int attr = once_per_device(kDeviceKeyGuideGradTcAttr, []() {
        cudaError_t e = cudaFuncSetAttribute(k_guide_grad_tc, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kGtSmem);
        return e == cudaSuccess ? 1 : -(int)e;
    });
    if (attr < 0) return (cudaError_t)(-attr);
    const uint32_t tiles = (a.n + (uint32_t)kTcRows - 1u) / (uint32_t)kTcRows;
    const int grid = (int)(tiles < (uint32_t)sm ? (tiles > 0u ? tiles : 1u) : (uint32_t)sm);
    k_guide_grad_tc<<<grid, kTcRows, kGtSmem, stream>>>(a);
    return cudaGetLastError();
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
