// lb_mlp.cuh -- the closure network, 19 -> 64 -> 64 -> 1 with ReLU: its
// sizes, the layout of its packed FP32 parameter vector and the device-side
// view the tensor-core kernels (lb_closure.cu) read.
//
// Rounding points (the numpy oracle in oracle/mlp_oracle.py applies the same
// ones): inputs and the first hidden layer enter the MMAs as BF16, W1 and W2
// as BF16 copies of the FP32 master weights; biases, the last layer and all
// accumulation stay FP32.
#pragma once

#include <cuda_bf16.h>

namespace lb {

constexpr int MLP_IN = 19;      // non-equilibrium moments (18) + |S|
constexpr int MLP_IN_PAD = 32;  // K of the first layer (two k16 steps)
constexpr int MLP_H = 64;
// packed FP32 parameter vector: W1[64][19], b1[64], W2[64][64], b2[64], w3[64], b3
constexpr int MLP_OFF_W1 = 0;
constexpr int MLP_OFF_B1 = MLP_OFF_W1 + MLP_H * MLP_IN;
constexpr int MLP_OFF_W2 = MLP_OFF_B1 + MLP_H;
constexpr int MLP_OFF_B2 = MLP_OFF_W2 + MLP_H * MLP_H;
constexpr int MLP_OFF_W3 = MLP_OFF_B2 + MLP_H;
constexpr int MLP_OFF_B3 = MLP_OFF_W3 + MLP_H;
constexpr int MLP_NPARAM = MLP_OFF_B3 + 1;  // 5505

// device-side network: BF16 copies of W1 (padded to 32 inputs) and W2, FP32 rest
struct MlpDev {
    const __nv_bfloat16 *w1;  // [64][32]
    const __nv_bfloat16 *w2;  // [64][64]
    const __nv_bfloat16 *w2t; // [64][64]: W2 transposed (the backward pass)
    const float *b1, *b2, *w3, *b3;
};

}  // namespace lb
