// conv.cuh -- 3x3 and 3x3x3 convolutions on the tensor cores (conv.cu).
#pragma once

#include <cuda_bf16.h>

#include "common.cuh"

namespace scihpc {

// one-time setup of the kernels' shared-memory limits (the argument is unused: every channel
// count fits the same two-stage budget)
int conv3x3_init(int max_n);
// dynamic shared memory of a convolution launch with n output channels
size_t conv_smem(int n);

// out[p][n] = bias[n] + sum_{t, ci} X[p + off(t)][ci] * Wk[n][t][ci], optional ReLU; out is
// BF16 or FP32 [H*W][N].  Ci and N multiples of 16, N <= 256.  *err is set to 1 if an
// mbarrier wait times out.
int conv3x3_forward(const __nv_bfloat16 *X, const __nv_bfloat16 *Wk, const float *bias, void *out, bool out_bf16,
                    int H, int W, int Ci, int N, bool relu, int *err, cudaStream_t s);
// the same over a D x H x W grid with 27 taps, Wk [N][27][Ci]
int conv3x3x3_forward(const __nv_bfloat16 *X, const __nv_bfloat16 *Wk, const float *bias, void *out, bool out_bf16,
                      int D, int H, int W, int Ci, int N, bool relu, int *err, cudaStream_t s);

// dW[n][t][ci] = sum_p X[p + off(t)][ci] * dZ[p][n] (FP32), split over `splits` pixel ranges;
// partial holds splits * taps * Ci * N floats (taps = 9 in 2D, 27 in 3D)
int conv3x3_wgrad(const __nv_bfloat16 *X, const __nv_bfloat16 *dZ, float *partial, float *dW, int H, int W, int Ci,
                  int N, int splits, int *err, cudaStream_t s);
int conv3x3x3_wgrad(const __nv_bfloat16 *X, const __nv_bfloat16 *dZ, float *partial, float *dW, int D, int H, int W,
                    int Ci, int N, int splits, int *err, cudaStream_t s);

}  // namespace scihpc
