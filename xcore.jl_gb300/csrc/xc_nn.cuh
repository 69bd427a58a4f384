// Internal declarations of the learned preconditioner's network (the U-Net
// and its BF16 tensor-core convolutions).
#pragma once

#include <cuda_runtime.h>

// y (NHWC BF16, or y_f32 FP32, either may be null) = relu?(conv3x3(x, w) + bias)
// x: NHWC BF16 [B][H][W][Cin]; w: BF16 [Cout][9][Cin]; bias: FP32 [Cout] or null.
// Cin, Cout in {16, 32, 64, 128}; W a multiple of 128 or a power of two below
// 128 with H divisible by 128 / W.  err: device int set nonzero when a bounded
// wait inside the kernel ran out.
int nn_conv3x3_fwd(const void* x, const void* w, const float* bias, void* y, float* y_f32, int B, int H, int W,
                   int Cin, int Cout, int relu, int* err, cudaStream_t s);
// dw (FP32 [Cout][9][Cin]) = scale * sum_p dy[p] (x) x[p + off] (+ dw when
// accumulate); partial: FP32 scratch of partial_blocks * 9 * Cout * Cin
int nn_conv3x3_wgrad(const void* x, const void* dy, float* dw, float* partial, int partial_blocks, int B, int H,
                     int W, int Cin, int Cout, float scale, int accumulate, int* err, cudaStream_t s);

// the network on the stream without synchronising (graph capture allowed):
// the FP32 result [npix][16] (first out_ch channels used) is nn_out16(n)
struct xc_nn;
int nn_forward_async(xc_nn* n, const float* in, cudaStream_t s);
const float* nn_out16(const xc_nn* n);
// wait for the stream and report a bounded wait that ran out inside a
// convolution as XC_TIMEOUT
int nn_check(xc_nn* n, cudaStream_t s);
