// lb_reduce.cu -- the cursor probe (read_value) and the global conservation
// sums.  The sums accumulate in FP64 (the only FP64 arithmetic of the native
// path): per thread over a grid-stride range, then warp shuffles, then one
// partial per block; a single-block second pass folds the partials in a fixed
// order, so the result is reproducible run to run.
#include "lb_kernels.cuh"

namespace lb {

constexpr int RED_BLOCKS = 608;  // 4 blocks on each of the 152 SMs
constexpr int RED_THREADS = 256;
constexpr int RED_FIELDS = 7;

int reduce_partials_size() { return RED_BLOCKS * RED_FIELDS; }

// reference src/read_value.cu:27-34 (plot float4 at the cursor); without a
// plot buffer the probe reads the moment arrays
__global__ void read_value_kernel(const float4 *plot, const float *ux, const float *uy,
                                  const float *uz, const float *rho, float *value, long o) {
    if (plot) {
        const float4 v = plot[o];
        value[0] = v.x; value[1] = v.y; value[2] = v.z; value[3] = v.w;
    } else {
        value[0] = ux[o]; value[1] = uy[o]; value[2] = uz ? uz[o] : 0.f; value[3] = rho[o];
    }
}

cudaError_t launch_read_value(const float *plot, const float *ux, const float *uy,
                             const float *uz, const float *rho, float *value, long o,
                             cudaStream_t s) {
    read_value_kernel<<<1, 32, 0, s>>>(reinterpret_cast<const float4 *>(plot), ux, uy, uz, rho,
                                       value, o);
    return cudaGetLastError();
}

__device__ __forceinline__ double warp_sum(double v) {
#pragma unroll
    for (int d = 16; d > 0; d >>= 1) v += __shfl_down_sync(0xffffffffu, v, d);
    return v;
}
__device__ __forceinline__ double warp_max(double v) {
#pragma unroll
    for (int d = 16; d > 0; d >>= 1) v = fmax(v, __shfl_down_sync(0xffffffffu, v, d));
    return v;
}

// folds acc[RED_FIELDS] of every thread of the block into out[RED_FIELDS]
// (field 5 is a maximum, the others sums); valid in thread 0
__device__ void block_fold(double (&acc)[RED_FIELDS], double *out) {
    __shared__ double sh[RED_THREADS / 32][RED_FIELDS];
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
#pragma unroll
    for (int i = 0; i < RED_FIELDS; i++) acc[i] = i == 5 ? warp_max(acc[i]) : warp_sum(acc[i]);
    if (lane == 0)
#pragma unroll
        for (int i = 0; i < RED_FIELDS; i++) sh[wid][i] = acc[i];
    __syncthreads();
    if (threadIdx.x == 0) {
        for (int i = 0; i < RED_FIELDS; i++) {
            double v = sh[0][i];
            for (int w = 1; w < RED_THREADS / 32; w++) v = i == 5 ? fmax(v, sh[w][i]) : v + sh[w][i];
            out[i] = v;
        }
    }
}

__global__ void __launch_bounds__(RED_THREADS) reduce_pass1(const float *rho, const float *ux,
                                                            const float *uy, const float *uz,
                                                            const uint8_t *solid, uint8_t mask,
                                                            long N, double *partials) {
    double acc[RED_FIELDS] = {0, 0, 0, 0, 0, 0, 0};
    for (long o = blockIdx.x * (long)blockDim.x + threadIdx.x; o < N;
         o += (long)gridDim.x * blockDim.x) {
        if (solid && (solid[o] & mask)) continue;
        const double r = rho[o], vx = ux[o], vy = uy[o], vz = uz ? uz[o] : 0.0;
        const double u2 = vx * vx + vy * vy + vz * vz;
        acc[0] += r;
        acc[1] += r * vx;
        acc[2] += r * vy;
        acc[3] += r * vz;
        acc[4] += 0.5 * r * u2;
        acc[5] = fmax(acc[5], sqrt(u2));
        acc[6] += 1.0;
    }
    block_fold(acc, partials + blockIdx.x * RED_FIELDS);
}

__global__ void __launch_bounds__(RED_THREADS) reduce_pass2(const double *partials, int nblocks,
                                                            double *out) {
    double acc[RED_FIELDS] = {0, 0, 0, 0, 0, 0, 0};
    for (int b = threadIdx.x; b < nblocks; b += blockDim.x)
#pragma unroll
        for (int i = 0; i < RED_FIELDS; i++) {
            const double v = partials[b * RED_FIELDS + i];
            acc[i] = i == 5 ? fmax(acc[i], v) : acc[i] + v;
        }
    block_fold(acc, out);
}

cudaError_t launch_reduce(const float *rho, const float *ux, const float *uy, const float *uz,
                          const uint8_t *solid, uint8_t mask, long N, double *partials,
                          double *out_dev, cudaStream_t s) {
    reduce_pass1<<<RED_BLOCKS, RED_THREADS, 0, s>>>(rho, ux, uy, uz, solid, mask, N, partials);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return e;
    reduce_pass2<<<1, RED_THREADS, 0, s>>>(partials, RED_BLOCKS, out_dev);
    return cudaGetLastError();
}

cudaError_t launch_reduce_blocks(const float *rho, const float *ux, const float *uy,
                                 const float *uz, const uint8_t *solid, uint8_t mask, long N,
                                 int nblocks, double *partials, double *out_dev,
                                 cudaStream_t s) {
    if (nblocks < 1) return cudaErrorInvalidValue;
    reduce_pass1<<<nblocks, RED_THREADS, 0, s>>>(rho, ux, uy, uz, solid, mask, N, partials);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return e;
    reduce_pass2<<<1, RED_THREADS, 0, s>>>(partials, nblocks, out_dev);
    return cudaGetLastError();
}

}  // namespace lb
