// Types and kernel launchers of the learned warm start (k_unet.cu, unet.cu).
#pragma once

#include <cuda_bf16.h>
#include <cuda_runtime.h>
#include <stdint.h>

namespace ib3d {
namespace unet {

using bf16 = __nv_bfloat16;

// B x D x H x W voxels, x fastest.
struct Vol {
  int B, D, H, W;
  __host__ __device__ __forceinline__ long long voxels() const { return (long long)B * D * H * W; }
};

// A channels-last tensor or a channel slice of one: element (v, c) is p[v*cs + co + c].
struct Act {
  bf16* p;
  int cs, co;
};

// err (device int) is set when a tensor-core wait gives up (it does not, unless the
// device misbehaves); the host checks it after synchronising
void conv(cudaStream_t st, const Vol& vol, Act X, int K, const bf16* W, const float* bias, int relu, int sign, Act Y,
          int N, int* err);
// weight gradients on the tensor cores (k_wgrad_tc; err as for conv), and the FP32
// CUDA-core form kept as its reference
void wgrad(cudaStream_t st, const Vol& vol, Act dZ, int N, Act X, int K, float* dW, int* err);
void wgrad_cuda_cores(cudaStream_t st, const Vol& vol, Act dZ, int N, Act X, int K, float* dW);
void bias_grad(cudaStream_t st, long long M, Act dZ, int N, float* db);
void relu_bwd(cudaStream_t st, long long M, int C, Act dY, Act Y);
void pool_fwd(cudaStream_t st, const Vol& out, int C, Act in, Act o);
void pool_bwd(cudaStream_t st, const Vol& out, int C, Act gout, Act gin, int accumulate);
void up_fwd(cudaStream_t st, const Vol& fine, int C, Act in, Act o);
void up_bwd(cudaStream_t st, const Vol& coarse, int C, Act gfine, Act gout);
void head_fwd(cudaStream_t st, long long M, int C, Act in, const float* w, float* out);
void head_bwd(cudaStream_t st, long long M, int C, Act in, const float* w, const float* gout, Act gin, float* dw);
void mse(cudaStream_t st, long long M, const float* out, const float* t, float* g, double* loss);
void adam(cudaStream_t st, int n, float* p, const float* g, float* m1, float* m2, float lr, int step);
void cast_conv_weights(cudaStream_t st, int N, int K, const float* w, bf16* wf, bf16* wt);

}  // namespace unet
}  // namespace ib3d
