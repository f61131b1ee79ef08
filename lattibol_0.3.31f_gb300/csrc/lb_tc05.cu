// lb_tc05.cu -- a self-check of the tcgen05 operand layout the closure kernel
// uses: one CTA multiplies a 128x32 BF16 tile by a 64x32 BF16 tile
// (D = X W^T, FP32 accumulator in tensor memory, two k16 MMAs) and writes D.
// The operands are small integers, so the product is exact and comparable
// bit for bit with a host product.
#include <cuda_bf16.h>

#include "../../include/lbgb300.h"
#include "lb_kernels.cuh"
#include "lb_tc05.cuh"

namespace lb {

__host__ __device__ constexpr int selftest_x(int r, int k) { return (r * 7 + k * 3) % 9 - 4; }
__host__ __device__ constexpr int selftest_w(int n, int k) { return (n * 5 + k) % 7 - 3; }

__global__ void __launch_bounds__(128) tc05_selftest_kernel(float *out, int *status) {
    __shared__ __align__(1024) uint8_t sx[128 * 32 * 2];
    __shared__ __align__(1024) uint8_t sw[64 * 32 * 2];
    __shared__ uint64_t mbar;
    __shared__ uint32_t tslot;
    const int t = threadIdx.x, warp = t >> 5;
    for (int i = t; i < 128 * 32; i += 128)
        *reinterpret_cast<__nv_bfloat16 *>(sx + kmajor_offset(i / 32, i % 32, 32)) =
            __float2bfloat16((float)selftest_x(i / 32, i % 32));
    for (int i = t; i < 64 * 32; i += 128)
        *reinterpret_cast<__nv_bfloat16 *>(sw + kmajor_offset(i / 32, i % 32, 32)) =
            __float2bfloat16((float)selftest_w(i / 32, i % 32));
    if (warp == 0) tc_alloc(&tslot, 64);
    if (t == 0) mbar_init(&mbar, 1);
    fence_proxy_async();
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    const uint32_t tmem = tslot;
    if (t == 0) {
        const uint32_t idesc = tc_idesc_bf16(128, 64);
        for (int s = 0; s < 2; s++)
            tc_mma_bf16(tmem, tc_desc(smem_u32(sx) + 256 * s, 128, 512),
                        tc_desc(smem_u32(sw) + 256 * s, 128, 512), idesc, s > 0);
        tc_commit(&mbar);
    }
    const bool ok = __all_sync(0xffffffffu, mbar_wait(&mbar, 0, 1 << 20));
    tc_fence_after();
    if (ok) {
        float v[32];
        for (int c = 0; c < 64; c += 32) {
            tc_ld32(tmem + ((uint32_t)(warp * 32) << 16) + (uint32_t)c, v);
#pragma unroll
            for (int j = 0; j < 32; j++) out[t * 64 + c + j] = v[j];
        }
    } else if ((t & 31) == 0) {
        atomicExch(status, 1);
    }
    tc_fence_before();
    __syncthreads();
    if (warp == 0) tc_dealloc(tmem, 64);
    if (t == 0) mbar_inval(&mbar);
}

}  // namespace lb

extern "C" int lb_tcgen05_selftest(float *out_host) {
    if (!out_host) return LB_ERR_ARG;
    float *out = nullptr;
    int *status = nullptr;
    cudaError_t e = cudaMalloc(&out, sizeof(float) * 128 * 64);
    if (e == cudaSuccess) e = cudaMalloc(&status, sizeof(int));
    if (e == cudaSuccess) e = cudaMemset(status, 0, sizeof(int));
    if (e == cudaSuccess) {
        lb::tc05_selftest_kernel<<<1, 128>>>(out, status);
        e = cudaGetLastError();
    }
    int st = 0;
    if (e == cudaSuccess) e = cudaMemcpy(out_host, out, sizeof(float) * 128 * 64,
                                         cudaMemcpyDeviceToHost);
    if (e == cudaSuccess) e = cudaMemcpy(&st, status, sizeof(int), cudaMemcpyDeviceToHost);
    cudaFree(out);
    cudaFree(status);
    if (e != cudaSuccess) {
        lb::abi_record_error("lb_tcgen05_selftest", cudaGetErrorString(e));
        return LB_ERR_CUDA;
    }
    if (st) {
        lb::abi_record_error("lb_tcgen05_selftest", "the MMA did not complete in time");
        return LB_ERR_DEVICE;
    }
    return LB_OK;
}
