// mlp.h -- host interface of the charging network kernels (mlp.cu).
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

namespace shark {

struct MlpArgs {
    const float* feat;       // raw features: sample s at feat[s * feat_stride + 0 .. NFEAT-1]
    const float* target;     // training: t of sample s at target[s * feat_stride + NFEAT]
    int feat_stride;
    const int32_t* index;    // sample of tile slot i: index[i] (nullptr: i)
    int n;                   // samples in this launch
    const float* blob;       // FP32 parameters + normalisation (SHARK_MLP_NBLOB)
    const uint8_t* packed;   // BF16 operand packs (mlp_packed_bytes())
    float* out;              // inference: t per sample (nullptr: none)
    float* seed;             // inference: psi0 (1 + t) per sample (nullptr: none)
    double psi0;
    float* grad;             // training: gradient accumulator (SHARK_MLP_NPARAM)
    float* loss;             // training: sum of squared normalised errors
    float inv_n;             // training: 1 / batch size
    unsigned int* err;       // set to 1 if an mbarrier wait gave up
};

size_t mlp_packed_bytes();
cudaError_t mlp_pack(const float* blob, uint8_t* packed, cudaStream_t st);
cudaError_t mlp_forward(const MlpArgs& a, cudaStream_t st);
cudaError_t mlp_backward(const MlpArgs& a, cudaStream_t st);
cudaError_t mlp_adam(float* blob, const float* grad, float* m, float* v, float lr, int step, cudaStream_t st);

}  // namespace shark
