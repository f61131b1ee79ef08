// lb_mlp.cuh -- the closure network, 19 -> 64 -> 64 -> 1 with ReLU, evaluated
// by one warp for 32 samples at a time on the tensor cores
// (mma.sync.m16n8k16, BF16 operands, FP32 accumulate).
//
// Rounding points (the numpy oracle in oracle/mlp_oracle.py applies the same
// ones): inputs and the first hidden layer enter the MMAs as BF16, W1 and W2
// as BF16 copies of the FP32 master weights; biases, the last layer and all
// accumulation stay FP32.
//
// Fragment layouts are those of the PTX ISA for m16n8k16 with row-major A
// and column-major B: with g = lane/4 and t = lane%4, A register j holds
// (row g + 8*(j&1), cols 2t + 8*(j>>1) .. +1), B register j holds
// (k 2t + 8j .. +1, n g), and C holds (row g + 8*(j>>1), col 2t + (j&1)).
#pragma once

#include <cuda_bf16.h>
#include <stdint.h>

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

// shared-memory row strides (in bf16 elements), padded so that the eight
// rows a fragment load touches fall in distinct banks
constexpr int SX_STRIDE = MLP_IN_PAD + 8;  // 40
constexpr int SH_STRIDE = MLP_H + 8;       // 72
constexpr int SW1_STRIDE = MLP_IN_PAD + 8; // 40
constexpr int SW2_STRIDE = MLP_H + 8;      // 72

// device-side network: BF16 copies of W1 (padded to 32 inputs) and W2, FP32 rest
struct MlpDev {
    const __nv_bfloat16 *w1;  // [64][32]
    const __nv_bfloat16 *w2;  // [64][64]
    const float *b1, *b2, *w3, *b3;
};

// per-block shared weights + per-warp activation tiles
struct MlpSmemWeights {
    __nv_bfloat16 w1[MLP_H * SW1_STRIDE];
    __nv_bfloat16 w2[MLP_H * SW2_STRIDE];
    float b1[MLP_H], b2[MLP_H], w3[MLP_H], b3;
};
struct MlpSmemWarp {
    __nv_bfloat16 x[32 * SX_STRIDE];
    __nv_bfloat16 h1[32 * SH_STRIDE];
    float y[32];
};

__device__ __forceinline__ void mma_bf16_16816(float (&d)[4], const uint32_t (&a)[4],
                                               const uint32_t (&b)[2]) {
    asm volatile(
        "mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 "
        "{%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, {%0,%1,%2,%3};\n"
        : "+f"(d[0]), "+f"(d[1]), "+f"(d[2]), "+f"(d[3])
        : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(b[0]), "r"(b[1]));
}

__device__ __forceinline__ uint32_t ld_b32(const __nv_bfloat16 *p) {
    return *reinterpret_cast<const uint32_t *>(p);
}

// Four 8x8 bf16 matrices from shared memory, each transposed on the way
// (ldmatrix .trans): lane l gives the address of row l % 8 of matrix l / 8
// (16 contiguous bytes, 16-byte aligned); register q receives matrix q in the
// fragment layout of an mma operand whose rows are the stored columns.
__device__ __forceinline__ void ldsm_x4_trans(uint32_t (&r)[4], const __nv_bfloat16 *row) {
    const uint32_t a = (uint32_t)__cvta_generic_to_shared(row);
    asm volatile("ldmatrix.sync.aligned.m8n8.x4.trans.shared.b16 {%0,%1,%2,%3}, [%4];\n"
                 : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3])
                 : "r"(a)
                 : "memory");
}

// all threads of the block: stage the network in shared memory
__device__ __forceinline__ void mlp_load_weights(MlpSmemWeights &s, const MlpDev &m) {
    for (int i = threadIdx.x + blockDim.x * threadIdx.y; i < MLP_H * MLP_IN_PAD;
         i += blockDim.x * blockDim.y)
        s.w1[(i / MLP_IN_PAD) * SW1_STRIDE + i % MLP_IN_PAD] = m.w1[i];
    for (int i = threadIdx.x + blockDim.x * threadIdx.y; i < MLP_H * MLP_H;
         i += blockDim.x * blockDim.y)
        s.w2[(i / MLP_H) * SW2_STRIDE + i % MLP_H] = m.w2[i];
    for (int i = threadIdx.x + blockDim.x * threadIdx.y; i < MLP_H; i += blockDim.x * blockDim.y) {
        s.b1[i] = m.b1[i];
        s.b2[i] = m.b2[i];
        s.w3[i] = m.w3[i];
    }
    if (threadIdx.x == 0 && threadIdx.y == 0) s.b3 = m.b3[0];
}

// One warp, rows 16*mt .. 16*mt+15 of its 32 samples (the input rows are in
// sw.x, written and __syncwarp'ed by the caller).  Writes those rows of the
// first hidden layer into sw.h1 (BF16, after ReLU), returns this lane's
// C-fragment values of the second hidden layer (after ReLU, FP32) in
// h2[nt][j], and -- if want_y -- the network output of the 16 rows in sw.y.
// One m-tile at a time keeps 32 accumulators live instead of 64.
__device__ __forceinline__ void mlp_forward_tile(const MlpSmemWeights &s, MlpSmemWarp &sw,
                                                 int mt, float (&h2)[8][4], bool want_y) {
    const int lane = threadIdx.x & 31, g = lane >> 2, t = lane & 3;
    {
        float acc[8][4];
#pragma unroll
        for (int nt = 0; nt < 8; nt++) acc[nt][0] = acc[nt][1] = acc[nt][2] = acc[nt][3] = 0.f;
#pragma unroll
        for (int kt = 0; kt < 2; kt++) {
            const __nv_bfloat16 *xa = sw.x + (mt * 16 + g) * SX_STRIDE + kt * 16 + 2 * t;
            const uint32_t a[4] = {ld_b32(xa), ld_b32(xa + 8 * SX_STRIDE), ld_b32(xa + 8),
                                   ld_b32(xa + 8 * SX_STRIDE + 8)};
#pragma unroll
            for (int nt = 0; nt < 8; nt++) {
                const __nv_bfloat16 *wb = s.w1 + (nt * 8 + g) * SW1_STRIDE + kt * 16 + 2 * t;
                const uint32_t b[2] = {ld_b32(wb), ld_b32(wb + 8)};
                mma_bf16_16816(acc[nt], a, b);
            }
        }
#pragma unroll
        for (int nt = 0; nt < 8; nt++) {
            const int c0 = nt * 8 + 2 * t, r0 = mt * 16 + g;
            const __nv_bfloat162 lo = __floats2bfloat162_rn(fmaxf(acc[nt][0] + s.b1[c0], 0.f),
                                                            fmaxf(acc[nt][1] + s.b1[c0 + 1], 0.f));
            const __nv_bfloat162 hi = __floats2bfloat162_rn(fmaxf(acc[nt][2] + s.b1[c0], 0.f),
                                                            fmaxf(acc[nt][3] + s.b1[c0 + 1], 0.f));
            *reinterpret_cast<__nv_bfloat162 *>(sw.h1 + r0 * SH_STRIDE + c0) = lo;
            *reinterpret_cast<__nv_bfloat162 *>(sw.h1 + (r0 + 8) * SH_STRIDE + c0) = hi;
        }
    }
    __syncwarp();
#pragma unroll
    for (int nt = 0; nt < 8; nt++) h2[nt][0] = h2[nt][1] = h2[nt][2] = h2[nt][3] = 0.f;
#pragma unroll
    for (int kt = 0; kt < 4; kt++) {
        const __nv_bfloat16 *ha = sw.h1 + (mt * 16 + g) * SH_STRIDE + kt * 16 + 2 * t;
        const uint32_t a[4] = {ld_b32(ha), ld_b32(ha + 8 * SH_STRIDE), ld_b32(ha + 8),
                               ld_b32(ha + 8 * SH_STRIDE + 8)};
#pragma unroll
        for (int nt = 0; nt < 8; nt++) {
            const __nv_bfloat16 *wb = s.w2 + (nt * 8 + g) * SW2_STRIDE + kt * 16 + 2 * t;
            const uint32_t b[2] = {ld_b32(wb), ld_b32(wb + 8)};
            mma_bf16_16816(h2[nt], a, b);
        }
    }
#pragma unroll
    for (int nt = 0; nt < 8; nt++) {
        const int c0 = nt * 8 + 2 * t;
        h2[nt][0] = fmaxf(h2[nt][0] + s.b2[c0], 0.f);
        h2[nt][1] = fmaxf(h2[nt][1] + s.b2[c0 + 1], 0.f);
        h2[nt][2] = fmaxf(h2[nt][2] + s.b2[c0], 0.f);
        h2[nt][3] = fmaxf(h2[nt][3] + s.b2[c0 + 1], 0.f);
    }
    if (!want_y) return;
    float p0 = 0.f, p1 = 0.f;  // rows mt*16+g and mt*16+g+8
#pragma unroll
    for (int nt = 0; nt < 8; nt++) {
        const int c0 = nt * 8 + 2 * t;
        p0 = p0 + h2[nt][0] * s.w3[c0];
        p0 = p0 + h2[nt][1] * s.w3[c0 + 1];
        p1 = p1 + h2[nt][2] * s.w3[c0];
        p1 = p1 + h2[nt][3] * s.w3[c0 + 1];
    }
    p0 = p0 + __shfl_xor_sync(0xffffffffu, p0, 1);
    p0 = p0 + __shfl_xor_sync(0xffffffffu, p0, 2);
    p1 = p1 + __shfl_xor_sync(0xffffffffu, p1, 1);
    p1 = p1 + __shfl_xor_sync(0xffffffffu, p1, 2);
    if (t == 0) {
        sw.y[mt * 16 + g] = p0 + s.b3;
        sw.y[mt * 16 + g + 8] = p1 + s.b3;
    }
}

// The whole warp tile (32 rows): h2 of both m-tiles and, if want_y, sw.y.
__device__ __forceinline__ void mlp_forward_warp(const MlpSmemWeights &s, MlpSmemWarp &sw,
                                                 float (&h2)[2][8][4], bool want_y) {
    __syncwarp();
    mlp_forward_tile(s, sw, 0, h2[0], want_y);
    mlp_forward_tile(s, sw, 1, h2[1], want_y);
    __syncwarp();
}

// Only the outputs: sw.y for the 32 rows, one m-tile at a time.
__device__ __forceinline__ void mlp_output_warp(const MlpSmemWeights &s, MlpSmemWarp &sw) {
    __syncwarp();
#pragma unroll 1
    for (int mt = 0; mt < 2; mt++) {
        float h2[8][4];
        mlp_forward_tile(s, sw, mt, h2, true);
    }
    __syncwarp();
}

}  // namespace lb
