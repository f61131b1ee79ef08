// lb_tc05.cu -- a self-check of the tcgen05 pattern the closure kernel uses,
// in one CTA of 128 threads: per round, the A tile (128 x 32 BF16) is
// written, D = A W1^T is computed (two k16 MMAs, FP32 in 64 tensor-memory
// columns) and read back, a hidden tile H (128 x 64 BF16, K = 64) is written
// over A, D = H W2^T is computed into the same columns and read back.  Three
// rounds reuse the columns and cycle the mbarrier phases as consecutive
// cell runs do.  The operands are small integers, so every product is exact.
#include <cuda_bf16.h>

#include "../../include/lbgb300.h"
#include "lb_kernels.cuh"
#include "lb_tc05.cuh"

namespace lb {

constexpr int ST_ROUNDS = 3;
__host__ __device__ constexpr int selftest_x(int r, int k, int round) {
    return ((r * 7 + k * 3) % 9 - 4) * (round + 1);
}
__host__ __device__ constexpr int selftest_w1(int n, int k) { return (n * 5 + k) % 7 - 3; }
__host__ __device__ constexpr int selftest_h(int r, int k, int round) {
    return (r + 3 * k + round) % 5 - 2;
}
__host__ __device__ constexpr int selftest_w2(int n, int k) { return (n + 2 * k) % 5 - 2; }

__global__ void __launch_bounds__(128) tc05_selftest_kernel(float *out, int *status) {
    __shared__ __align__(1024) uint8_t sa[128 * 64 * 2];
    __shared__ __align__(1024) uint8_t sw1[64 * 32 * 2];
    __shared__ __align__(1024) uint8_t sw2[64 * 64 * 2];
    __shared__ uint64_t mbar;
    __shared__ uint32_t tslot;
    const int t = threadIdx.x, warp = t >> 5;
    for (int i = t; i < 64 * 32; i += 128)
        *reinterpret_cast<__nv_bfloat16 *>(sw1 + kmajor_offset(i / 32, i % 32, 32)) =
            __float2bfloat16((float)selftest_w1(i / 32, i % 32));
    for (int i = t; i < 64 * 64; i += 128)
        *reinterpret_cast<__nv_bfloat16 *>(sw2 + kmajor_offset(i / 64, i % 64, 64)) =
            __float2bfloat16((float)selftest_w2(i / 64, i % 64));
    if (warp == 0) tc_alloc(&tslot, 64);
    if (t == 0) mbar_init(&mbar, 1);
    fence_proxy_async();
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    const uint32_t tmem = tslot, lane_base = tmem + ((uint32_t)(warp * 32) << 16);
    const uint32_t idesc = tc_idesc_bf16(128, 64);
    uint32_t phase = 0;
    bool ok = true;
    for (int round = 0; round < ST_ROUNDS && ok; round++) {
        for (int k = 0; k < 32; k++)  // row t of A
            *reinterpret_cast<__nv_bfloat16 *>(sa + kmajor_offset(t, k, 32)) =
                __float2bfloat16((float)selftest_x(t, k, round));
        fence_proxy_async();
        tc_fence_before();
        __syncthreads();
        if (t == 0) {
            tc_fence_after();
            for (int s = 0; s < 2; s++)
                tc_mma_bf16(tmem, tc_desc(smem_u32(sa) + 256 * s, 128, 512),
                            tc_desc(smem_u32(sw1) + 256 * s, 128, 512), idesc, s > 0);
            tc_commit(&mbar);
        }
        ok = __syncthreads_and(mbar_wait(&mbar, phase, 1 << 20));
        phase ^= 1;
        if (!ok) {
            if (t == 0) atomicOr(status, 1 << (2 * round));
            break;
        }
        tc_fence_after();
        float v[32];
        for (int c = 0; c < 64; c += 32) {
            tc_ld32(lane_base + (uint32_t)c, v);
#pragma unroll
            for (int j = 0; j < 32; j++) out[(round * 2 * 128 + t) * 64 + c + j] = v[j];
        }
        for (int k = 0; k < 64; k++)  // row t of H over A
            *reinterpret_cast<__nv_bfloat16 *>(sa + kmajor_offset(t, k, 64)) =
                __float2bfloat16((float)selftest_h(t, k, round));
        fence_proxy_async();
        tc_fence_before();
        __syncthreads();
        if (t == 0) {
            tc_fence_after();
            for (int s = 0; s < 4; s++)
                tc_mma_bf16(tmem, tc_desc(smem_u32(sa) + 256 * s, 128, 1024),
                            tc_desc(smem_u32(sw2) + 256 * s, 128, 1024), idesc, s > 0);
            tc_commit(&mbar);
        }
        ok = __syncthreads_and(mbar_wait(&mbar, phase, 1 << 20));
        phase ^= 1;
        if (!ok) {
            if (t == 0) atomicOr(status, 2 << (2 * round));
            break;
        }
        tc_fence_after();
        for (int c = 0; c < 64; c += 32) {
            tc_ld32(lane_base + (uint32_t)c, v);
#pragma unroll
            for (int j = 0; j < 32; j++) out[((round * 2 + 1) * 128 + t) * 64 + c + j] = v[j];
        }
        tc_fence_before();
    }
    if (!ok) mbar_wait(&mbar, phase ^ 1, 1 << 20);
    tc_fence_before();
    __syncthreads();
    if (warp == 0) tc_dealloc(tmem, 64);
    if (t == 0) mbar_inval(&mbar);
}

// self-check of the bounded mbarrier wait: nothing is committed to the
// barrier, so the wait must give up after `limit` attempts; the block then
// releases its tensor memory and reports
__global__ void __launch_bounds__(128) tc05_wait_selftest_kernel(int *status, int limit) {
    __shared__ uint64_t mbar;
    __shared__ uint32_t tslot;
    const int t = threadIdx.x, warp = t >> 5;
    if (warp == 0) tc_alloc(&tslot, 32);
    if (t == 0) mbar_init(&mbar, 1);
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    const bool ok = __syncthreads_and(mbar_wait(&mbar, 0, limit));
    if (!ok && t == 0) atomicExch(status, 1);
    tc_fence_before();
    __syncthreads();
    if (warp == 0) tc_dealloc(tslot, 32);
    if (t == 0) mbar_inval(&mbar);
}

}  // namespace lb

extern "C" int lb_wait_selftest(int which, int *status_host) {
    if (!status_host || which < 1 || which > 2) return LB_ERR_ARG;
    int *dev = nullptr;
    cudaError_t e = cudaMalloc(&dev, 2 * sizeof(int));
    if (e == cudaSuccess) e = cudaMemset(dev, 0, 2 * sizeof(int));
    if (e == cudaSuccess) {
        if (which == 2) {
            e = lb::sc_stage_wait_selftest(dev);
        } else {
            lb::tc05_wait_selftest_kernel<<<1, 128>>>(dev, 1 << 10);
            e = cudaGetLastError();
        }
    }
    if (e == cudaSuccess) e = cudaMemcpy(status_host, dev, sizeof(int), cudaMemcpyDeviceToHost);
    cudaFree(dev);
    if (e != cudaSuccess) {
        lb::abi_record_error("lb_wait_selftest", cudaGetErrorString(e));
        return LB_ERR_CUDA;
    }
    return LB_OK;
}

extern "C" int lb_tcgen05_selftest(float *out_host, int *status_host) {
    if (!out_host || !status_host) return LB_ERR_ARG;
    const size_t n = (size_t)lb::ST_ROUNDS * 2 * 128 * 64;
    float *out = nullptr;
    int *status = nullptr;
    cudaError_t e = cudaMalloc(&out, sizeof(float) * n);
    if (e == cudaSuccess) e = cudaMalloc(&status, sizeof(int));
    if (e == cudaSuccess) e = cudaMemset(status, 0, sizeof(int));
    if (e == cudaSuccess) e = cudaMemset(out, 0, sizeof(float) * n);
    if (e == cudaSuccess) {
        lb::tc05_selftest_kernel<<<1, 128>>>(out, status);
        e = cudaGetLastError();
    }
    if (e == cudaSuccess) e = cudaMemcpy(out_host, out, sizeof(float) * n, cudaMemcpyDeviceToHost);
    if (e == cudaSuccess) e = cudaMemcpy(status_host, status, sizeof(int), cudaMemcpyDeviceToHost);
    cudaFree(out);
    cudaFree(status);
    if (e != cudaSuccess) {
        lb::abi_record_error("lb_tcgen05_selftest", cudaGetErrorString(e));
        return LB_ERR_CUDA;
    }
    return LB_OK;
}
