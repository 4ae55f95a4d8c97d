/* Host-side declarations of the guiding network's kernels (guide.cu). */
#pragma once
#include <cuda_bf16.h>
#include <cuda_runtime.h>
#include <stddef.h>
#include <stdint.h>

namespace grisrt {
namespace guide {

/* features: per sample 9 floats (position in [0,1]^3, normal, wo); out: 40 raw values per sample */
struct FwdArgs {
    const __nv_bfloat16* wPacked;
    const float* bias;
    const float* feat;
    const uint32_t* count;     /* optional device count (samples = min(*count, n)) */
    uint32_t n;
    float* out;
    int tensorCores = 0;                /* 1: the tcgen05 kernel (guide_tc.cu), 0: mma.sync */
    unsigned long long* err = nullptr;  /* error word (bit 1: a tensor-core wait gave up) */
    int withholdCommit = 0;             /* test of the bounded waits: the MMAs' completion is never signalled */
};

/* gradient of loss = -sum_i weight_i log p(dir_i | feat_i) / sum_i weight_i, added to grad */
struct GradArgs {
    const __nv_bfloat16* wPacked;
    const float* bias;
    const float* feat;
    const float* dir;
    const float* weight;
    const uint32_t* count;     /* optional device count of the whole record array: samples = */
    uint32_t base;             /* min(max(*count, base) - base, n), from feat/dir/weight (already offset) */
    uint32_t n;
    float* invWeightSum;       /* device scalar: written here from the weights, then read */
    float* grad;
    int tensorCores = 0;                /* 1: the tcgen05 kernel (guide_tc.cu), 0: mma.sync */
    unsigned long long* err = nullptr;  /* error word (bit 1: a tensor-core wait gave up) */
    int withholdCommit = 0;             /* test of the bounded waits: a forward layer's completion is never signalled */
};

/* what the path tracer needs of a guide: the network and the training-record batch */
struct GuideDevice {
    const __nv_bfloat16* wPacked;
    const float* bias;
    float* tFeat;
    float* tDir;
    float* tWeight;
    uint32_t* tCount;
    uint32_t cap;
    float mix;
    int tensorCores;   /* inference kernel: 1 tcgen05, 0 mma.sync */
};

cudaError_t launch_forward(const FwdArgs& a, cudaStream_t stream);
cudaError_t launch_forward_tc(const FwdArgs& a, cudaStream_t stream);
size_t tc_smem_bytes();
cudaError_t launch_grad(const GradArgs& a, cudaStream_t stream);
cudaError_t launch_grad_tc(const GradArgs& a, cudaStream_t stream);
size_t tc_grad_smem_bytes();
cudaError_t launch_pack(const float* params, __nv_bfloat16* wPacked, float* bias, cudaStream_t stream);
cudaError_t launch_adam(float* params, float* grad, float* m, float* v, uint32_t* step, float lr, cudaStream_t stream);
size_t grad_smem_bytes();

}  // namespace guide
}  // namespace grisrt
