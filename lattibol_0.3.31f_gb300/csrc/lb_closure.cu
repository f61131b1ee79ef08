// lb_closure.cu -- learned sub-grid closure for under-resolved D3Q19 flow.
//
// * d3q19_closure_kernel: the fused native D3Q19 step in which every cell's
//   relaxation time comes from the closure network.  Per cell it forms 19
//   features from the pre-collision populations -- the 18 non-conserved
//   non-equilibrium moments (momentum 3, stress 6, third/fourth order 9 in
//   the raw basis c_x c_y^2, ..., c_y^2 c_z^2) scaled by 1/(rho c_s^2 tau0
//   s_ref), and |S| / s_ref with S = -Pi_neq / (2 rho c_s^2 tau0) -- and the
//   warp evaluates the network for its 32 cells on the tensor cores.  The
//   output y gives nu_t = nu0 * clamp(y, 0, z_max) and tau = 0.5 + 3 (nu0 +
//   nu_t).
// * filter / feature kernels: box-filter a fine lattice's moments onto a
//   coarse grid (Favre averages), and from the filtered fields build the
//   same 19 features (stress features -2 S/s_ref from central differences of
//   the filtered velocity; the other moments are zero at first order) and
//   the target z = nu_t/nu0 of the local least-squares eddy viscosity of the
//   filtered sub-grid stress, nu_t = max(0, -(T_dev : S) / (2 S : S)).
// * training: the forward pass of the closure kernel (tensor cores), an FP32
//   backward pass per sample, per-block weight-gradient sums in shared
//   memory, a fixed-order reduction of the block partials, and Adam.
#include <algorithm>
#include <cstddef>
#include <cmath>
#include <cstring>
#include <string>
#include <vector>

#include "../../include/lbgb300.h"
#include "lb_d3q19.cuh"
#include "lb_tc05.cuh"

using namespace lb;

namespace lb {

// ------------------------------------------------------------------ features
// The 18 raw non-equilibrium moments sum_k P(c_k) (g_k - feq_k) as raw
// moments of g minus the moments of the D3Q19 second-order equilibrium in
// closed form (exact identities of the lattice: sum c_a feq = rho u_a,
// sum c_a^2 feq = rho/3 + rho u_a^2, sum c_a c_b feq = rho u_a u_b,
// sum c_a c_b^2 feq = rho u_a / 3, sum c_a^2 c_b^2 feq = rho (1/9 - u^2/6 +
// (u_a^2 + u_b^2)/2)).  The raw moments come from the four edge velocities of
// each coordinate plane: with g_pp, g_pm, g_mp, g_mm the plane's (+,+), (+,-),
// (-,+), (-,-) populations, sum c_a c_b = (pp + mm) - (pm + mp), sum c_a c_b^2
// = (pp + pm) - (mp + mm) (also the plane's part of sum c_a), sum c_b c_a^2 =
// (pp + mp) - (pm + mm), sum c_a^2 c_b^2 = (pp + pm) + (mp + mm).
struct PlaneSums {
    float ab, a_b2, b_a2, a2b2;
    __device__ __forceinline__ PlaneSums(float pp, float pm, float mp, float mm) {
        ab = (pp + mm) - (pm + mp);
        a_b2 = (pp + pm) - (mp + mm);
        b_a2 = (pp + mp) - (pm + mm);
        a2b2 = (pp + pm) + (mp + mm);
    }
};

__device__ __forceinline__ void closure_features(const float (&g)[19], float rho, float ux,
                                                 float uy, float uz, float tau0, float s_ref,
                                                 float (&feat)[MLP_IN]) {
    // planes (a, b): xy = (7, 8, 11, 12), xz = (9, 10, 13, 14), yz = (15, 16, 17, 18)
    const PlaneSums xy(g[7], g[8], g[11], g[12]);
    const PlaneSums xz(g[9], g[10], g[13], g[14]);
    const PlaneSums yz(g[15], g[16], g[17], g[18]);
    const float third = 1.f / 3.f;
    const float rx = rho * ux, ry = rho * uy, rz = rho * uz;
    const float uxx = ux * ux, uyy = uy * uy, uzz = uz * uz;
    const float e4 = 1.f / 9.f - (uxx + uyy + uzz) * (1.f / 6.f);
    float m[18];
    m[0] = ((g[1] - g[2]) + (xy.a_b2 + xz.a_b2)) - rx;
    m[1] = ((g[3] - g[4]) + (xy.b_a2 + yz.a_b2)) - ry;
    m[2] = ((g[5] - g[6]) + (xz.b_a2 + yz.b_a2)) - rz;
    m[3] = ((g[1] + g[2]) + (xy.a2b2 + xz.a2b2)) - (rho * third + rx * ux);
    m[4] = ((g[3] + g[4]) + (xy.a2b2 + yz.a2b2)) - (rho * third + ry * uy);
    m[5] = ((g[5] + g[6]) + (xz.a2b2 + yz.a2b2)) - (rho * third + rz * uz);
    m[6] = xy.ab - rx * uy;
    m[7] = xz.ab - rx * uz;
    m[8] = yz.ab - ry * uz;
    m[9] = xy.a_b2 - rx * third;
    m[10] = xz.a_b2 - rx * third;
    m[11] = xy.b_a2 - ry * third;
    m[12] = yz.a_b2 - ry * third;
    m[13] = xz.b_a2 - rz * third;
    m[14] = yz.b_a2 - rz * third;
    m[15] = xy.a2b2 - rho * (e4 + 0.5f * (uxx + uyy));
    m[16] = xz.a2b2 - rho * (e4 + 0.5f * (uxx + uzz));
    m[17] = yz.a2b2 - rho * (e4 + 0.5f * (uyy + uzz));
    const float scale = 1.f / (rho * (1.f / 3.f) * tau0 * s_ref);
#pragma unroll
    for (int i = 0; i < 18; i++) feat[i] = m[i] * scale;
    // S = -Pi / (2 rho cs2 tau0): |S| = sqrt(2 S:S) with the off-diagonals twice
    const float h = -0.5f * scale;  // S/s_ref = h * Pi
    const float sxx = h * m[3], syy = h * m[4], szz = h * m[5];
    const float sxy = h * m[6], sxz = h * m[7], syz = h * m[8];
    feat[18] = sqrtf(2.f * (sxx * sxx + syy * syy + szz * szz +
                            2.f * (sxy * sxy + sxz * sxz + syz * syz)));
}

// fused native D3Q19 step with the closure (F32 storage)
// Persistent: each block stages the network once and then walks row-blocks
// of D3_BLOCK cells (x-run at fixed y, z) with a stride of the grid size.
template <bool MOM>
__global__ void __launch_bounds__(D3_BLOCK) d3q19_closure_kernel(const D3Args a,
                                                                 const ClosureArgs ca) {
    __shared__ MlpSmemWeights sW;
    __shared__ MlpSmemWarp sWarp[D3_BLOCK / 32];
    mlp_load_weights(sW, ca.mlp);
    __syncthreads();
    const int lane = threadIdx.x & 31;
    MlpSmemWarp &sw = sWarp[threadIdx.x >> 5];
    const int nbx = (a.W + D3_BLOCK - 1) / D3_BLOCK;
    const long nrows = (long)nbx * a.H * a.D;
    for (long r = blockIdx.x; r < nrows; r += gridDim.x) {
        const long rr = a.reverse ? nrows - 1 - r : r;
        const int bx = (int)(rr % nbx);
        const long yz = rr / nbx;
        const int y = (int)(yz % a.H), z = (int)(yz / a.H);
        const int x = bx * D3_BLOCK + threadIdx.x;
        const bool inside = x < a.W;
        const int o = inside ? x + a.W * (y + a.H * z) : 0;
        const uint8_t fl = inside ? a.flags[o] : CELL_WALL;
        const bool fluid = !(fl & CELL_WALL);
        float g[19], rho = 1.f, ux = 0.f, uy = 0.f, uz = 0.f;
        float feat[MLP_IN];
#pragma unroll
        for (int i = 0; i < MLP_IN; i++) feat[i] = 0.f;
        if (fluid) {
            const Nbr3 n(x, y, z, a.W, a.H, a.D);
            pull_native<float>(a, o, n, fl, g);
            d3q19_moments_native(g, rho, ux, uy, uz);
            closure_features(g, rho, ux, uy, uz, ca.tau0, ca.s_ref, feat);
        }
        __nv_bfloat162 *row = reinterpret_cast<__nv_bfloat162 *>(sw.x + lane * SX_STRIDE);
#pragma unroll
        for (int i = 0; i < MLP_IN_PAD / 2; i++)
            row[i] = __floats2bfloat162_rn(2 * i < MLP_IN ? feat[2 * i] : 0.f,
                                           2 * i + 1 < MLP_IN ? feat[2 * i + 1] : 0.f);
        mlp_output_warp(sW, sw);
        const float yv = sw.y[lane];
        if (!inside) continue;
        if (!fluid) {
            if (MOM) { a.ux[o] = 0.f; a.uy[o] = 0.f; a.uz[o] = 0.f; a.rho[o] = 0.f; }
            if (a.probe && o == a.probe_o) *a.probe = make_float4(0.f, 0.f, 0.f, 0.f);
            continue;
        }
        if (ca.y_out) ca.y_out[o] = yv;
        const float zt = fminf(fmaxf(yv, 0.f), ca.z_max);
        const float tau_inv = 1.f / (0.5f + 3.f * (ca.nu0 + ca.nu0 * zt));
        if (MOM) { a.ux[o] = ux; a.uy[o] = uy; a.uz[o] = uz; a.rho[o] = rho; }
        if (a.probe && o == a.probe_o) *a.probe = make_float4(ux, uy, uz, rho);
        float ex = ux, ey = uy, ez = uz;
        if (a.Fx != 0.f || a.Fy != 0.f || a.Fz != 0.f) {
            const float inv_rt = 1.f / (rho * tau_inv);
            if (a.Fx != 0.f) ex = __fmaf_rn(a.Fx, inv_rt, ux);
            if (a.Fy != 0.f) ey = __fmaf_rn(a.Fy, inv_rt, uy);
            if (a.Fz != 0.f) ez = __fmaf_rn(a.Fz, inv_rt, uz);
        }
        d3q19_bgk_native(g, ex, ey, ez, rho, a.w0, a.w1, a.w7, tau_inv);
#pragma unroll
        for (int k = 0; k < 19; k++) a.dst.f[k][o] = g[k];
    }
}

// ---------------------------------------------------------------------------
// The same step with the network on the 5th-generation tensor cores.  A block
// of 128 threads takes a run of 128 cells; thread t owns cell t, row t of the
// MMA tiles and lane t of tensor memory.  Per run:
//   1. every thread writes its 19 BF16 features (padded to 32) as row t of A
//      (K-major 8x8 core matrices, lb_tc05.cuh);
//   2. thread 0 issues D = A W1^T (M 128, N 64, two k16 MMAs, FP32 in 64
//      tensor-memory columns) and commits to an mbarrier;
//   3. each warp loads its 32 lanes of D, adds b1 and writes the hidden row,
//      ReLU and BF16 rounding in one conversion, over A (now K = 64);
//   4. thread 0 issues D = H W2^T (four k16 MMAs) into the same columns;
//   5. each thread loads its row, adds b2, applies ReLU and sums w3 h + b3
//      (fused multiply-adds).
// Rounding points are the warp-level kernel's (BF16 inputs, weights and
// first hidden layer; FP32 accumulation, biases and last layer) except that
// the last layer's products are fused into the sum (one rounding each, not
// two).
// ---------------------------------------------------------------------------
// ReLU and round-to-nearest BF16 of two floats in one conversion, lo in the
// low half (the PTX packs its first source into the high half)
__device__ __forceinline__ uint32_t bf16x2_relu(float lo, float hi) {
    uint32_t d;
    asm("cvt.rn.relu.bf16x2.f32 %0, %1, %2;" : "=r"(d) : "f"(hi), "f"(lo));
    return d;
}

constexpr int TC_COLS = 64;             // tensor-memory columns per block (D is 128 x 64)
constexpr int TC_WAIT = 1 << 22;        // mbarrier polls before a block gives up

struct TcSmem {
    uint8_t a[128 * MLP_H * 2];         // A: features (K 32) then the hidden layer (K 64)
    uint8_t w1[MLP_H * MLP_IN_PAD * 2]; // W1 [64][32], K-major core matrices
    uint8_t w2[MLP_H * MLP_H * 2];      // W2 [64][64]
    uint64_t mbar;
    uint32_t tslot;
};

template <bool MOM>
__global__ void __launch_bounds__(D3_BLOCK) d3q19_closure_tc_kernel(const D3Args a,
                                                                    const ClosureArgs ca) {
    __shared__ __align__(1024) TcSmem sm;
    const int t = threadIdx.x, warp = t >> 5;
    for (int i = t; i < MLP_H * MLP_IN_PAD; i += D3_BLOCK)
        *reinterpret_cast<__nv_bfloat16 *>(sm.w1 + kmajor_offset(i / MLP_IN_PAD, i % MLP_IN_PAD,
                                                                 MLP_IN_PAD)) = ca.mlp.w1[i];
    for (int i = t; i < MLP_H * MLP_H; i += D3_BLOCK)
        *reinterpret_cast<__nv_bfloat16 *>(sm.w2 + kmajor_offset(i / MLP_H, i % MLP_H, MLP_H)) =
            ca.mlp.w2[i];
    if (t == 0) mbar_init(&sm.mbar, 1);
    if (warp == 0) tc_alloc(&sm.tslot, TC_COLS);
    fence_proxy_async();
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    const uint32_t tmem = sm.tslot;
    const uint32_t lane_base = tmem + ((uint32_t)(warp * 32) << 16);
    const uint32_t a_addr = smem_u32(sm.a), w1_addr = smem_u32(sm.w1), w2_addr = smem_u32(sm.w2);
    constexpr uint32_t id = tc_idesc_bf16(128, MLP_H);
    uint32_t phase = 0;
    bool ok = true;

    // runs of 128 consecutive nodes r * 128 .. r * 128 + 127 (row after row, so
    // a lattice narrower than 128 nodes still fills every row of the MMA tile);
    // 32-bit: the node count is below 2^31
    const int WH = a.W * a.H, ncell = WH * a.D;
    const int nrows = (ncell + D3_BLOCK - 1) / D3_BLOCK;
    // a run of 128 cells: this thread's cell, its flags and pulled populations
    struct Run {
        int o;
        bool inside, fluid;
        float g[19];
    };
    auto load = [&](int r, Run &u) {
        const int rr = a.reverse ? nrows - 1 - r : r;
        const int oo = rr * D3_BLOCK + t;
        u.inside = oo < ncell;
        u.o = u.inside ? oo : 0;
        const int z = u.o / WH, rem = u.o - z * WH;
        const int y = rem / a.W, x = rem - y * a.W;
        const uint8_t fl = u.inside ? a.flags[u.o] : CELL_WALL;
        u.fluid = !(fl & CELL_WALL);
        if (u.fluid) {
            const Nbr3 n(x, y, z, a.W, a.H, a.D);
            pull_native<float>(a, u.o, n, fl, u.g);
        }
    };
    // The next run's populations are loaded while this run's network runs on
    // the tensor core: their DRAM latency overlaps the two MMAs and epilogues.
    Run cur, nxt;
    if (blockIdx.x < nrows) load(blockIdx.x, cur);
    for (int r = blockIdx.x; r < nrows && ok; r += gridDim.x) {
        const int o = cur.o;
        const bool inside = cur.inside, fluid = cur.fluid;
        float(&g)[19] = cur.g;
        float rho = 1.f, ux = 0.f, uy = 0.f, uz = 0.f;
        float feat[MLP_IN];
#pragma unroll
        for (int i = 0; i < MLP_IN; i++) feat[i] = 0.f;
        if (fluid) {
            d3q19_moments_native(g, rho, ux, uy, uz);
            closure_features(g, rho, ux, uy, uz, ca.tau0, ca.s_ref, feat);
        }
        // 1. features -> row t of A (four 16-byte column groups, K = 32)
#pragma unroll
        for (int h = 0; h < MLP_IN_PAD / 8; h++) {
            __nv_bfloat162 p[4];
#pragma unroll
            for (int j = 0; j < 4; j++) {
                const int k0 = 8 * h + 2 * j;
                p[j] = __floats2bfloat162_rn(k0 < MLP_IN ? feat[k0] : 0.f,
                                             k0 + 1 < MLP_IN ? feat[k0 + 1] : 0.f);
            }
            *reinterpret_cast<uint4 *>(sm.a + kmajor_offset(t, 8 * h, MLP_IN_PAD)) =
                *reinterpret_cast<const uint4 *>(p);
        }
        if (r + (int)gridDim.x < nrows) load(r + gridDim.x, nxt);
        fence_proxy_async();
        tc_fence_before();
        __syncthreads();
        // 2. layer 1
        if (t == 0) {
            tc_fence_after();
#pragma unroll
            for (int s = 0; s < MLP_IN_PAD / 16; s++)
                tc_mma_bf16(tmem, tc_desc(a_addr + 256 * s, 128, MLP_IN_PAD / 8 * 128),
                            tc_desc(w1_addr + 256 * s, 128, MLP_IN_PAD / 8 * 128), id, s > 0);
            tc_commit(&sm.mbar);
        }
        // thread 0 polls the mbarrier; the others wait at the block barrier
        // (no issue slots), which with tcgen05.fence::after_thread_sync
        // orders their tensor-memory loads after the MMA's completion
        ok = __syncthreads_and(t == 0 ? mbar_wait(&sm.mbar, phase, TC_WAIT) : true);
        phase ^= 1;
        if (!ok) break;
        tc_fence_after();
        // 3. hidden layer: + b1, ReLU, BF16 -> row t of A (K = 64)
#pragma unroll
        for (int c = 0; c < MLP_H; c += 32) {
            float v[32];
            tc_ld32(lane_base + (uint32_t)c, v);
#pragma unroll
            for (int h = 0; h < 4; h++) {
                uint32_t p[4];
#pragma unroll
                for (int j = 0; j < 4; j++) {
                    const int q = 8 * h + 2 * j;
                    const float2 h = __fadd2_rn(make_float2(v[q], v[q + 1]),
                                                make_float2(ca.head_b1[c + q], ca.head_b1[c + q + 1]));
                    p[j] = bf16x2_relu(h.x, h.y);
                }
                *reinterpret_cast<uint4 *>(sm.a + kmajor_offset(t, c + 8 * h, MLP_H)) =
                    make_uint4(p[0], p[1], p[2], p[3]);
            }
        }
        fence_proxy_async();
        tc_fence_before();
        __syncthreads();
        // 4. layer 2
        if (t == 0) {
            tc_fence_after();
#pragma unroll
            for (int s = 0; s < MLP_H / 16; s++)
                tc_mma_bf16(tmem, tc_desc(a_addr + 256 * s, 128, MLP_H / 8 * 128),
                            tc_desc(w2_addr + 256 * s, 128, MLP_H / 8 * 128), id, s > 0);
            tc_commit(&sm.mbar);
        }
        ok = __syncthreads_and(t == 0 ? mbar_wait(&sm.mbar, phase, TC_WAIT) : true);
        phase ^= 1;
        if (!ok) break;
        tc_fence_after();
        // 5. output: b3 + sum_j w3_j ReLU(D_j + b2_j), even and odd j in the two
        // lanes of paired FP32 instructions (two accumulation chains)
        float2 y2 = make_float2(0.f, 0.f);
#pragma unroll
        for (int c = 0; c < MLP_H; c += 32) {
            float v[32];
            tc_ld32(lane_base + (uint32_t)c, v);
#pragma unroll
            for (int j = 0; j < 32; j += 2) {
                float2 h = __fadd2_rn(make_float2(v[j], v[j + 1]),
                                      make_float2(ca.head_b2[c + j], ca.head_b2[c + j + 1]));
                h.x = fmaxf(h.x, 0.f);
                h.y = fmaxf(h.y, 0.f);
                y2 = __ffma2_rn(make_float2(ca.head_w3[c + j], ca.head_w3[c + j + 1]), h, y2);
            }
        }
        const float yv = (y2.x + y2.y) + ca.head_b3;
        tc_fence_before();  // the next run's MMA overwrites these columns after a barrier
        if (inside && !fluid) {
            if (MOM) { a.ux[o] = 0.f; a.uy[o] = 0.f; a.uz[o] = 0.f; a.rho[o] = 0.f; }
            if (a.probe && o == a.probe_o) *a.probe = make_float4(0.f, 0.f, 0.f, 0.f);
        } else if (inside) {
            if (ca.y_out) ca.y_out[o] = yv;
            const float zt = fminf(fmaxf(yv, 0.f), ca.z_max);
            const float tau_inv = 1.f / (0.5f + 3.f * (ca.nu0 + ca.nu0 * zt));
            if (MOM) { a.ux[o] = ux; a.uy[o] = uy; a.uz[o] = uz; a.rho[o] = rho; }
            if (a.probe && o == a.probe_o) *a.probe = make_float4(ux, uy, uz, rho);
            float ex = ux, ey = uy, ez = uz;
            if (a.Fx != 0.f || a.Fy != 0.f || a.Fz != 0.f) {
                const float inv_rt = 1.f / (rho * tau_inv);
                if (a.Fx != 0.f) ex = __fmaf_rn(a.Fx, inv_rt, ux);
                if (a.Fy != 0.f) ey = __fmaf_rn(a.Fy, inv_rt, uy);
                if (a.Fz != 0.f) ez = __fmaf_rn(a.Fz, inv_rt, uz);
            }
            d3q19_bgk_native(g, ex, ey, ez, rho, a.w0, a.w1, a.w7, tau_inv);
#pragma unroll
            for (int k = 0; k < 19; k++) a.dst.f[k][o] = g[k];
        }
        cur = nxt;
    }
    if (!ok) {
        // an MMA did not complete: record it, give it one more bounded wait so
        // that no MMA is writing the columns when they are released
        if (t == 0 && ca.err) atomicExch(ca.err, 1);
        mbar_wait(&sm.mbar, phase ^ 1, TC_WAIT);
    }
    tc_fence_before();
    __syncthreads();
    if (warp == 0) tc_dealloc(tmem, TC_COLS);
    if (t == 0) mbar_inval(&sm.mbar);
}

cudaError_t launch_d3q19_closure(const D3Args &a, const ClosureArgs &ca, bool mom,
                                 cudaStream_t s) {
    if (!ca.legacy_mma) {
        // SMs x resident blocks.  The occupancy query reports one block per SM
        // for a kernel that allocates tensor memory, so the residency is
        // computed from the kernel's registers and shared memory, and capped
        // at 8 blocks (8 x 64 of the SM's 512 tensor-memory columns).
        static int tc_cap = 0;
        if (!tc_cap) {
            int dev = 0, sms = 1, smem_sm = 0, thr_sm = 2048;
            cudaGetDevice(&dev);
            cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
            cudaDeviceGetAttribute(&smem_sm, cudaDevAttrMaxSharedMemoryPerMultiprocessor, dev);
            cudaDeviceGetAttribute(&thr_sm, cudaDevAttrMaxThreadsPerMultiProcessor, dev);
            cudaFuncAttributes fa{};
            cudaFuncGetAttributes(&fa, d3q19_closure_tc_kernel<false>);
            const int regs = std::max(1, (fa.numRegs + 7) / 8 * 8 * D3_BLOCK);
            int occ = std::min({65536 / regs, thr_sm / D3_BLOCK,
                                smem_sm / (int)(fa.sharedSizeBytes + 1024), 512 / TC_COLS});
            tc_cap = sms * std::max(occ, 1);
        }
        const long nrows = ((long)a.W * a.H * a.D + D3_BLOCK - 1) / D3_BLOCK;
        const unsigned g = (unsigned)(nrows < tc_cap ? nrows : tc_cap);
        if (mom) d3q19_closure_tc_kernel<true><<<g, D3_BLOCK, 0, s>>>(a, ca);
        else d3q19_closure_tc_kernel<false><<<g, D3_BLOCK, 0, s>>>(a, ca);
        return cudaGetLastError();
    }
    static int grid_cap = 0;  // SMs x resident blocks of the kernel, computed once
    if (!grid_cap) {
        int dev = 0, sms = 1, occ = 1;
        cudaGetDevice(&dev);
        cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, d3q19_closure_kernel<false>,
                                                      D3_BLOCK, 0);
        grid_cap = sms * (occ > 0 ? occ : 1);
    }
    const long nrows = (long)((a.W + D3_BLOCK - 1) / D3_BLOCK) * a.H * a.D;
    const unsigned g = (unsigned)(nrows < grid_cap ? nrows : grid_cap);
    if (mom) d3q19_closure_kernel<true><<<g, D3_BLOCK, 0, s>>>(a, ca);
    else d3q19_closure_kernel<false><<<g, D3_BLOCK, 0, s>>>(a, ca);
    return cudaGetLastError();
}

}  // namespace lb

namespace {

// ------------------------------------------------------------------ filter
// Favre box filter of factor^3 fine cells onto each coarse cell: rho_bar,
// u_bar = sum(rho u)/sum(rho), T_ab = sum(rho u_a u_b)/sum(rho) - u_a u_b.
// out: [0] rho, [1..3] u, [4..9] T (xx, yy, zz, xy, xz, yz), each Nc floats
__global__ void filter_kernel(const float *rho, const float *ux, const float *uy,
                              const float *uz, int W, int H, int D, int f, float *out, long Nc) {
    const long c = blockIdx.x * (long)blockDim.x + threadIdx.x;
    if (c >= Nc) return;
    const int Wc = W / f, Hc = H / f;
    const int I = (int)(c % Wc), J = (int)((c / Wc) % Hc), K = (int)(c / ((long)Wc * Hc));
    double sr = 0, sx = 0, sy = 0, sz = 0, sxx = 0, syy = 0, szz = 0, sxy = 0, sxz = 0, syz = 0;
    for (int k = 0; k < f; k++)
        for (int j = 0; j < f; j++)
            for (int i = 0; i < f; i++) {
                const long o = (I * f + i) + (long)W * ((J * f + j) + (long)H * (K * f + k));
                const double r = rho[o], vx = ux[o], vy = uy[o], vz = uz[o];
                sr += r; sx += r * vx; sy += r * vy; sz += r * vz;
                sxx += r * vx * vx; syy += r * vy * vy; szz += r * vz * vz;
                sxy += r * vx * vy; sxz += r * vx * vz; syz += r * vy * vz;
            }
    const double bx = sx / sr, by = sy / sr, bz = sz / sr;
    out[c] = (float)(sr / ((double)f * f * f));
    out[Nc + c] = (float)bx;
    out[2 * Nc + c] = (float)by;
    out[3 * Nc + c] = (float)bz;
    out[4 * Nc + c] = (float)(sxx / sr - bx * bx);
    out[5 * Nc + c] = (float)(syy / sr - by * by);
    out[6 * Nc + c] = (float)(szz / sr - bz * bz);
    out[7 * Nc + c] = (float)(sxy / sr - bx * by);
    out[8 * Nc + c] = (float)(sxz / sr - bx * bz);
    out[9 * Nc + c] = (float)(syz / sr - by * bz);
}

// strain rate of the filtered velocity at coarse cell (I, J, K) (periodic
// central differences) and the two contractions of the eddy-viscosity fit,
// T_dev : S and S : S
struct FilteredCell {
    float S[3][3], TS, SS;
    __device__ FilteredCell(const float *fl, int Wc, int Hc, int Dc, int I, int J, int K) {
        const long Nc = (long)Wc * Hc * Dc;
        auto at = [&](int i, int j, int k) -> long {
            i = (i + Wc) % Wc; j = (j + Hc) % Hc; k = (k + Dc) % Dc;
            return i + (long)Wc * (j + (long)Hc * k);
        };
        const long c = at(I, J, K);
        const float *u[3] = {fl + Nc, fl + 2 * Nc, fl + 3 * Nc};
        float du[3][3];  // du[a][b] = d u_b / d x_a
        const long pa[3] = {at(I + 1, J, K), at(I, J + 1, K), at(I, J, K + 1)};
        const long ma[3] = {at(I - 1, J, K), at(I, J - 1, K), at(I, J, K - 1)};
        for (int aa = 0; aa < 3; aa++)
            for (int b = 0; b < 3; b++) du[aa][b] = 0.5f * (u[b][pa[aa]] - u[b][ma[aa]]);
        for (int aa = 0; aa < 3; aa++)
            for (int b = 0; b < 3; b++) S[aa][b] = 0.5f * (du[aa][b] + du[b][aa]);
        const float T[6] = {fl[4 * Nc + c], fl[5 * Nc + c], fl[6 * Nc + c],
                            fl[7 * Nc + c], fl[8 * Nc + c], fl[9 * Nc + c]};
        const float tr = (T[0] + T[1] + T[2]) / 3.f;
        TS = (T[0] - tr) * S[0][0] + (T[1] - tr) * S[1][1] + (T[2] - tr) * S[2][2] +
             2.f * (T[3] * S[0][1] + T[4] * S[0][2] + T[5] * S[1][2]);
        SS = S[0][0] * S[0][0] + S[1][1] * S[1][1] + S[2][2] * S[2][2] +
             2.f * (S[0][1] * S[0][1] + S[0][2] * S[0][2] + S[1][2] * S[1][2]);
    }
};

// T_dev : S and S : S of every coarse cell (for the averaged fit)
__global__ void ts_ss_kernel(const float *fl, int Wc, int Hc, int Dc, float *ts, float *ss) {
    const long Nc = (long)Wc * Hc * Dc;
    const long c = blockIdx.x * (long)blockDim.x + threadIdx.x;
    if (c >= Nc) return;
    const FilteredCell fc(fl, Wc, Hc, Dc, (int)(c % Wc), (int)((c / Wc) % Hc),
                          (int)(c / ((long)Wc * Hc)));
    ts[c] = fc.TS;
    ss[c] = fc.SS;
}

// features and targets from the filtered fields.  The target is the eddy
// viscosity of the least-squares fit of the sub-grid stress, nu_t =
// max(0, -(T_dev : S) / (2 S : S)), either per cell (rad 0) or with both
// contractions summed over the (2 rad + 1)^3 cells around it (periodic) before
// the ratio is formed -- the averaging of the dynamic procedure, which leaves
// far fewer cells clipped at zero and so does not bias the fit upward.
__global__ void features_kernel(const float *fl, int Wc, int Hc, int Dc, float nu0, float s_ref,
                                float z_max, const float *ts, const float *ss, int rad,
                                float *feat, float *target) {
    const long Nc = (long)Wc * Hc * Dc;
    const long c = blockIdx.x * (long)blockDim.x + threadIdx.x;
    if (c >= Nc) return;
    const int I = (int)(c % Wc), J = (int)((c / Wc) % Hc), K = (int)(c / ((long)Wc * Hc));
    const FilteredCell fc(fl, Wc, Hc, Dc, I, J, K);
    float TS = fc.TS, SS = fc.SS;
    if (rad > 0) {
        double sts = 0.0, sss = 0.0;
        for (int k = -rad; k <= rad; k++)
            for (int j = -rad; j <= rad; j++)
                for (int i = -rad; i <= rad; i++) {
                    const long o = (I + i + Wc) % Wc +
                                   (long)Wc * ((J + j + Hc) % Hc + (long)Hc * ((K + k + Dc) % Dc));
                    sts += ts[o];
                    sss += ss[o];
                }
        TS = (float)sts;
        SS = (float)sss;
    }
    const float nut = fmaxf(0.f, -TS / (2.f * SS + 1e-30f));
    target[c] = fminf(nut / nu0, z_max);
    float *fo = feat + c * MLP_IN;
    const float q = -2.f / s_ref;
    for (int i = 0; i < MLP_IN; i++) fo[i] = 0.f;
    fo[3] = q * fc.S[0][0]; fo[4] = q * fc.S[1][1]; fo[5] = q * fc.S[2][2];
    fo[6] = q * fc.S[0][1]; fo[7] = q * fc.S[0][2]; fo[8] = q * fc.S[1][2];
    fo[18] = sqrtf(2.f * fc.SS) / s_ref;
}

// ------------------------------------------------------------------ training
constexpr int HROW = MLP_H + 1;
struct TrainSmemWarp {
    MlpSmemWarp m;                         // x and the first hidden layer (BF16), y
    float h2[32 * HROW];                   // row stride 65: a warp walking its rows hits 32 banks
    float dh2[32 * HROW];
    float dh1[32 * HROW];
    __nv_bfloat16 dh2b[32 * SH_STRIDE];    // BF16 copies: operands of the gradient MMAs
    __nv_bfloat16 dh1b[32 * SH_STRIDE];
    float dy[32];
};
constexpr int TRAIN_WARPS = 4;
constexpr int NGRAD = MLP_NPARAM + 1;  // + loss
// the per-warp tiles start on a 128-byte boundary after the weights
constexpr size_t TRAIN_WARP_OFF = (sizeof(MlpSmemWeights) + 127) / 128 * 128;
constexpr size_t TRAIN_SMEM =
    TRAIN_WARP_OFF + TRAIN_WARPS * sizeof(TrainSmemWarp) + NGRAD * sizeof(float);
static_assert(offsetof(MlpSmemWeights, w2) % 16 == 0 && sizeof(MlpSmemWarp) % 16 == 0 &&
                  (32 * HROW * sizeof(float)) % 16 == 0 && sizeof(TrainSmemWarp) % 16 == 0,
              "ldmatrix rows stay 16-byte aligned");

// Forward (mma.sync, as mlp_forward_warp) and backward over the samples
// [0, n) of a batch, every contraction on the tensor cores (mma.sync
// m16n8k16, BF16 operands, FP32 accumulate).  A block takes 128 samples at a
// time, 32 per warp:
//  * per warp: dy = 2 (y - z) / n per sample, dH2 = dy w3 (h2 > 0) from the
//    second layer's accumulator fragments, dH1 = (dH2 W2) (h1 > 0) -- dH2 and
//    W2 as BF16 operands (W2 read transposed by ldmatrix .trans);
//  * per block (after a barrier): warp w owns rows 16w .. 16w+15 of dW2 =
//    dH2^T H1 and of dW1 = dH1^T X, contracting over all 128 samples in a
//    fixed order (both operands read transposed by ldmatrix .trans), and adds
//    them into the block's gradient sums, every element owned by one thread;
//  * the bias and output-layer gradients (db1, db2, dw3, db3) are FP32 sums
//    over the samples, each parameter owned by one thread.
// Rounding points (restated by the numpy oracle): dH2 and dH1 enter the MMAs
// as BF16; everything is accumulated in FP32.  Each block leaves its gradient
// sums (already divided by n) and its loss sum in partial[block][NGRAD].
__global__ void __launch_bounds__(32 * TRAIN_WARPS) mlp_train_kernel(
    MlpDev mlp, const float *X, const float *Z, long n, float *partial) {
    extern __shared__ __align__(128) unsigned char smem[];
    MlpSmemWeights &sW = *reinterpret_cast<MlpSmemWeights *>(smem);
    TrainSmemWarp *sWarp = reinterpret_cast<TrainSmemWarp *>(smem + TRAIN_WARP_OFF);
    float *sG = reinterpret_cast<float *>(smem + TRAIN_WARP_OFF +
                                          TRAIN_WARPS * sizeof(TrainSmemWarp));
    mlp_load_weights(sW, mlp);
    for (int i = threadIdx.x; i < NGRAD; i += blockDim.x) sG[i] = 0.f;
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    TrainSmemWarp &tw = sWarp[wid];
    const int g = lane >> 2, t = lane & 3;
    const float inv_n = 1.f / (float)n;
    // ldmatrix row addresses: (row, column) of this lane in the four 8x8 matrices
    // of a 16x16 tile read as [k-rows 0-7 | 8-15] x [n-columns 0-7 | 8-15]
    const int lr_b = (lane & 7) + 8 * ((lane >> 3) & 1), lc_b = 8 * (lane >> 4);
    //   ... and as [m-columns 0-7 | 8-15] x [k-rows 0-7 | 8-15] (A from a stored
    //   [k][m] matrix)
    const int lr_a = (lane & 7) + 8 * (lane >> 4), lc_a = 8 * ((lane >> 3) & 1);
    __syncthreads();
    for (long base = (long)blockIdx.x * 32 * TRAIN_WARPS; base < n;
         base += (long)gridDim.x * 32 * TRAIN_WARPS) {
        const long s = base + wid * 32 + lane;
        const bool valid = s < n;
        for (int i = 0; i < MLP_IN_PAD; i++)
            tw.m.x[lane * SX_STRIDE + i] =
                __float2bfloat16_rn((valid && i < MLP_IN) ? X[s * MLP_IN + i] : 0.f);
        float h2[2][8][4];
        mlp_forward_warp(sW, tw.m, h2, true);
        const float err = valid ? tw.m.y[lane] - Z[s] : 0.f;
        tw.dy[lane] = 2.f * err * inv_n;
        __syncwarp();
        // dH2 = dy w3 (h2 > 0), from the accumulator fragments
#pragma unroll
        for (int mt = 0; mt < 2; mt++) {
            const int r0 = mt * 16 + g, r1 = r0 + 8;
            const float dy0 = tw.dy[r0], dy1 = tw.dy[r1];
#pragma unroll
            for (int nt = 0; nt < 8; nt++) {
                const int c0 = nt * 8 + 2 * t;
                const float *q = h2[mt][nt];
                const float d00 = q[0] > 0.f ? dy0 * sW.w3[c0] : 0.f;
                const float d01 = q[1] > 0.f ? dy0 * sW.w3[c0 + 1] : 0.f;
                const float d10 = q[2] > 0.f ? dy1 * sW.w3[c0] : 0.f;
                const float d11 = q[3] > 0.f ? dy1 * sW.w3[c0 + 1] : 0.f;
                tw.h2[r0 * HROW + c0] = q[0];
                tw.h2[r0 * HROW + c0 + 1] = q[1];
                tw.h2[r1 * HROW + c0] = q[2];
                tw.h2[r1 * HROW + c0 + 1] = q[3];
                tw.dh2[r0 * HROW + c0] = d00;
                tw.dh2[r0 * HROW + c0 + 1] = d01;
                tw.dh2[r1 * HROW + c0] = d10;
                tw.dh2[r1 * HROW + c0 + 1] = d11;
                *reinterpret_cast<__nv_bfloat162 *>(tw.dh2b + r0 * SH_STRIDE + c0) =
                    __floats2bfloat162_rn(d00, d01);
                *reinterpret_cast<__nv_bfloat162 *>(tw.dh2b + r1 * SH_STRIDE + c0) =
                    __floats2bfloat162_rn(d10, d11);
            }
        }
        __syncwarp();
        // dH1 = (dH2 W2) (h1 > 0): A = dH2 [samples x 64], B[k = j][n = i] = W2[j][i]
#pragma unroll 1
        for (int mt = 0; mt < 2; mt++) {
            float acc[8][4];
#pragma unroll
            for (int nt = 0; nt < 8; nt++) acc[nt][0] = acc[nt][1] = acc[nt][2] = acc[nt][3] = 0.f;
#pragma unroll
            for (int kt = 0; kt < 4; kt++) {
                const __nv_bfloat16 *da = tw.dh2b + (mt * 16 + g) * SH_STRIDE + kt * 16 + 2 * t;
                const uint32_t a[4] = {ld_b32(da), ld_b32(da + 8 * SH_STRIDE), ld_b32(da + 8),
                                       ld_b32(da + 8 * SH_STRIDE + 8)};
#pragma unroll
                for (int np = 0; np < 4; np++) {
                    uint32_t b[4];
                    ldsm_x4_trans(b, sW.w2 + (kt * 16 + lr_b) * SW2_STRIDE + np * 16 + lc_b);
                    const uint32_t b0[2] = {b[0], b[1]}, b1[2] = {b[2], b[3]};
                    mma_bf16_16816(acc[2 * np], a, b0);
                    mma_bf16_16816(acc[2 * np + 1], a, b1);
                }
            }
            const int r0 = mt * 16 + g, r1 = r0 + 8;
#pragma unroll
            for (int nt = 0; nt < 8; nt++) {
                const int c0 = nt * 8 + 2 * t;
                const __nv_bfloat16 *h1r0 = tw.m.h1 + r0 * SH_STRIDE + c0;
                const __nv_bfloat16 *h1r1 = tw.m.h1 + r1 * SH_STRIDE + c0;
                const float d00 = __bfloat162float(h1r0[0]) > 0.f ? acc[nt][0] : 0.f;
                const float d01 = __bfloat162float(h1r0[1]) > 0.f ? acc[nt][1] : 0.f;
                const float d10 = __bfloat162float(h1r1[0]) > 0.f ? acc[nt][2] : 0.f;
                const float d11 = __bfloat162float(h1r1[1]) > 0.f ? acc[nt][3] : 0.f;
                tw.dh1[r0 * HROW + c0] = d00;
                tw.dh1[r0 * HROW + c0 + 1] = d01;
                tw.dh1[r1 * HROW + c0] = d10;
                tw.dh1[r1 * HROW + c0 + 1] = d11;
                *reinterpret_cast<__nv_bfloat162 *>(tw.dh1b + r0 * SH_STRIDE + c0) =
                    __floats2bfloat162_rn(d00, d01);
                *reinterpret_cast<__nv_bfloat162 *>(tw.dh1b + r1 * SH_STRIDE + c0) =
                    __floats2bfloat162_rn(d10, d11);
            }
        }
        // block loss: sum over the warp, one atomic per warp into shared memory
        float e2 = err * err;
        for (int d = 16; d > 0; d >>= 1) e2 += __shfl_xor_sync(0xffffffffu, e2, d);
        if (lane == 0) atomicAdd(&sG[MLP_NPARAM], e2 * inv_n);
        __syncthreads();
        // dW2 rows j = 16 wid .. 16 wid + 15 (all 64 columns) and dW1 rows
        // i = 16 wid .. (inputs 0..31) over the block's 128 samples: k-step kk
        // is samples 16 kk .. 16 kk + 15, rows 16 (kk & 1) .. of warp kk / 2's tiles
        {
            float a2[8][4], a1[4][4];
#pragma unroll
            for (int nt = 0; nt < 8; nt++) a2[nt][0] = a2[nt][1] = a2[nt][2] = a2[nt][3] = 0.f;
#pragma unroll
            for (int nt = 0; nt < 4; nt++) a1[nt][0] = a1[nt][1] = a1[nt][2] = a1[nt][3] = 0.f;
#pragma unroll 1
            for (int kk = 0; kk < 2 * TRAIN_WARPS; kk++) {
                const TrainSmemWarp &u = sWarp[kk >> 1];
                const int sr = (kk & 1) * 16;
                uint32_t a[4];
                // A[m = j][k = sample] = dH2[sample][j]
                ldsm_x4_trans(a, u.dh2b + (sr + lr_a) * SH_STRIDE + wid * 16 + lc_a);
#pragma unroll
                for (int np = 0; np < 4; np++) {
                    uint32_t b[4];  // B[k = sample][n = i] = h1[sample][i]
                    ldsm_x4_trans(b, u.m.h1 + (sr + lr_b) * SH_STRIDE + np * 16 + lc_b);
                    const uint32_t b0[2] = {b[0], b[1]}, b1[2] = {b[2], b[3]};
                    mma_bf16_16816(a2[2 * np], a, b0);
                    mma_bf16_16816(a2[2 * np + 1], a, b1);
                }
                // A[m = i][k = sample] = dH1[sample][i]
                ldsm_x4_trans(a, u.dh1b + (sr + lr_a) * SH_STRIDE + wid * 16 + lc_a);
#pragma unroll
                for (int np = 0; np < 2; np++) {
                    uint32_t b[4];  // B[k = sample][n = input] = x[sample][input]
                    ldsm_x4_trans(b, u.m.x + (sr + lr_b) * SX_STRIDE + np * 16 + lc_b);
                    const uint32_t b0[2] = {b[0], b[1]}, b1[2] = {b[2], b[3]};
                    mma_bf16_16816(a1[2 * np], a, b0);
                    mma_bf16_16816(a1[2 * np + 1], a, b1);
                }
            }
            const int j0 = wid * 16 + g, j1 = j0 + 8;
#pragma unroll
            for (int nt = 0; nt < 8; nt++) {
                const int c0 = nt * 8 + 2 * t;
                sG[MLP_OFF_W2 + j0 * MLP_H + c0] += a2[nt][0];
                sG[MLP_OFF_W2 + j0 * MLP_H + c0 + 1] += a2[nt][1];
                sG[MLP_OFF_W2 + j1 * MLP_H + c0] += a2[nt][2];
                sG[MLP_OFF_W2 + j1 * MLP_H + c0 + 1] += a2[nt][3];
            }
#pragma unroll
            for (int nt = 0; nt < 4; nt++) {
                const int f0 = nt * 8 + 2 * t;
                if (f0 < MLP_IN) {
                    sG[MLP_OFF_W1 + j0 * MLP_IN + f0] += a1[nt][0];
                    sG[MLP_OFF_W1 + j1 * MLP_IN + f0] += a1[nt][2];
                }
                if (f0 + 1 < MLP_IN) {
                    sG[MLP_OFF_W1 + j0 * MLP_IN + f0 + 1] += a1[nt][1];
                    sG[MLP_OFF_W1 + j1 * MLP_IN + f0 + 1] += a1[nt][3];
                }
            }
        }
        // db1, db2, dw3, db3: FP32 sums over the 128 samples, one owner each
        for (int q = threadIdx.x; q < 3 * MLP_H + 1; q += blockDim.x) {
            float acc = 0.f;
            for (int w = 0; w < TRAIN_WARPS; w++) {
                const TrainSmemWarp &u = sWarp[w];
                for (int r = 0; r < 32; r++) {
                    if (q < MLP_H) acc = acc + u.dh1[r * HROW + q];
                    else if (q < 2 * MLP_H) acc = acc + u.dh2[r * HROW + q - MLP_H];
                    else if (q < 3 * MLP_H) acc = acc + u.dy[r] * u.h2[r * HROW + q - 2 * MLP_H];
                    else acc = acc + u.dy[r];
                }
            }
            const int p = q < MLP_H ? MLP_OFF_B1 + q
                        : q < 2 * MLP_H ? MLP_OFF_B2 + q - MLP_H
                        : q < 3 * MLP_H ? MLP_OFF_W3 + q - 2 * MLP_H
                                        : MLP_OFF_B3;
            sG[p] = sG[p] + acc;
        }
        __syncthreads();
    }
    for (int i = threadIdx.x; i < NGRAD; i += blockDim.x) partial[(long)blockIdx.x * NGRAD + i] = sG[i];
}

__global__ void grad_reduce_kernel(const float *partial, int nblocks, float *grad) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= NGRAD) return;
    float s = 0.f;
    for (int b = 0; b < nblocks; b++) s = s + partial[(long)b * NGRAD + i];
    grad[i] = s;
}

// Adam step on the FP32 master parameters, refreshing the BF16 copies
__global__ void adam_kernel(float *p, float *m1, float *m2, const float *grad, float lr,
                            float b1c, float b2c, __nv_bfloat16 *w1b, __nv_bfloat16 *w2b) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= MLP_NPARAM) return;
    const float gr = grad[i];
    const float a = 0.9f * m1[i] + 0.1f * gr;
    const float b = 0.999f * m2[i] + 0.001f * gr * gr;
    m1[i] = a;
    m2[i] = b;
    const float v = p[i] - lr * (a / b1c) / (sqrtf(b / b2c) + 1e-8f);
    p[i] = v;
    if (i < MLP_OFF_B1) w1b[(i / MLP_IN) * MLP_IN_PAD + i % MLP_IN] = __float2bfloat16_rn(v);
    else if (i >= MLP_OFF_W2 && i < MLP_OFF_B2) w2b[i - MLP_OFF_W2] = __float2bfloat16_rn(v);
}

__global__ void refresh_bf16_kernel(const float *p, __nv_bfloat16 *w1b, __nv_bfloat16 *w2b) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < MLP_H * MLP_IN_PAD) {
        const int j = i / MLP_IN_PAD, f = i % MLP_IN_PAD;
        w1b[i] = __float2bfloat16_rn(f < MLP_IN ? p[MLP_OFF_W1 + j * MLP_IN + f] : 0.f);
    }
    if (i < MLP_H * MLP_H) w2b[i] = __float2bfloat16_rn(p[MLP_OFF_W2 + i]);
}

// inference of the network on rows of features (the closure kernel's forward)
__global__ void __launch_bounds__(128) mlp_forward_kernel(MlpDev mlp, const float *X, long n,
                                                          float *Y) {
    __shared__ MlpSmemWeights sW;
    __shared__ MlpSmemWarp sWarp[4];
    mlp_load_weights(sW, mlp);
    __syncthreads();
    const int lane = threadIdx.x & 31;
    MlpSmemWarp &sw = sWarp[threadIdx.x >> 5];
    for (long base = (long)blockIdx.x * 128; base < n; base += (long)gridDim.x * 128) {
        const long s = base + threadIdx.x;
        for (int i = 0; i < MLP_IN_PAD; i++)
            sw.x[lane * SX_STRIDE + i] =
                __float2bfloat16_rn((s < n && i < MLP_IN) ? X[s * MLP_IN + i] : 0.f);
        float h2[2][8][4];
        mlp_forward_warp(sW, sw, h2, true);
        if (s < n) Y[s] = sw.y[lane];
        __syncwarp();
    }
}

}  // namespace

struct lb_mlp {
    float *p = nullptr, *m1 = nullptr, *m2 = nullptr, *grad = nullptr, *partial = nullptr;
    __nv_bfloat16 *w1b = nullptr, *w2b = nullptr;
    int nblocks = 304;
    long step = 0;
    cudaStream_t stream = nullptr;
    std::string err;
};

namespace {

MlpDev mlp_dev(const lb_mlp *m) {
    MlpDev d;
    d.w1 = m->w1b;
    d.w2 = m->w2b;
    d.b1 = m->p + MLP_OFF_B1;
    d.b2 = m->p + MLP_OFF_B2;
    d.w3 = m->p + MLP_OFF_W3;
    d.b3 = m->p + MLP_OFF_B3;
    return d;
}

int mfail(lb_mlp *m, cudaError_t e, const char *where) {
    if (m) m->err = std::string(where) + ": " + cudaGetErrorString(e);
    return LB_ERR_CUDA;
}
#define LB_MTRY(m, where, call)                                   \
    do {                                                          \
        cudaError_t e_ = (call);                                  \
        if (e_ != cudaSuccess) return mfail(m, e_, where);        \
    } while (0)

int mlp_gradient(lb_mlp *m, const float *X, const float *Z, long n) {
    static bool attr = false;
    if (!attr) {
        LB_MTRY(m, "cudaFuncSetAttribute",
                cudaFuncSetAttribute(mlp_train_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                     (int)TRAIN_SMEM));
        attr = true;
    }
    const long chunks = (n + 127) / 128;
    const int nb = (int)std::min<long>(m->nblocks, chunks);
    mlp_train_kernel<<<nb, 32 * TRAIN_WARPS, TRAIN_SMEM, m->stream>>>(mlp_dev(m), X, Z, n,
                                                                      m->partial);
    LB_MTRY(m, "mlp_train_kernel", cudaGetLastError());
    grad_reduce_kernel<<<(NGRAD + 255) / 256, 256, 0, m->stream>>>(m->partial, nb, m->grad);
    LB_MTRY(m, "grad_reduce_kernel", cudaGetLastError());
    return LB_OK;
}

}  // namespace

extern "C" {

int lb_mlp_create(uint64_t seed, lb_mlp **out) {
    if (!out) return LB_ERR_ARG;
    lb_mlp *m = new lb_mlp;
    cudaError_t e = cudaSuccess;
    if (e == cudaSuccess) e = cudaMalloc(&m->p, sizeof(float) * MLP_NPARAM);
    if (e == cudaSuccess) e = cudaMalloc(&m->m1, sizeof(float) * MLP_NPARAM);
    if (e == cudaSuccess) e = cudaMalloc(&m->m2, sizeof(float) * MLP_NPARAM);
    if (e == cudaSuccess) e = cudaMalloc(&m->grad, sizeof(float) * NGRAD);
    if (e == cudaSuccess) e = cudaMalloc(&m->partial, sizeof(float) * NGRAD * m->nblocks);
    if (e == cudaSuccess) e = cudaMalloc(&m->w1b, sizeof(__nv_bfloat16) * MLP_H * MLP_IN_PAD);
    if (e == cudaSuccess) e = cudaMalloc(&m->w2b, sizeof(__nv_bfloat16) * MLP_H * MLP_H);
    if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&m->stream, cudaStreamNonBlocking);
    if (e != cudaSuccess) {
        lb_mlp_destroy(m);
        return LB_ERR_NOMEM;
    }
    // He-uniform initialisation from a 64-bit LCG (host side, deterministic)
    std::vector<float> p(MLP_NPARAM, 0.f);
    uint64_t st = seed * 6364136223846793005ULL + 1442695040888963407ULL;
    auto uni = [&]() {
        st = st * 6364136223846793005ULL + 1442695040888963407ULL;
        return (float)((st >> 11) * (1.0 / 9007199254740992.0)) * 2.f - 1.f;
    };
    const float a1 = sqrtf(6.f / MLP_IN), a2 = sqrtf(6.f / MLP_H), a3 = sqrtf(3.f / MLP_H);
    for (int i = 0; i < MLP_H * MLP_IN; i++) p[MLP_OFF_W1 + i] = a1 * uni();
    for (int i = 0; i < MLP_H * MLP_H; i++) p[MLP_OFF_W2 + i] = a2 * uni();
    for (int i = 0; i < MLP_H; i++) p[MLP_OFF_W3 + i] = a3 * uni();
    const int rc = lb_mlp_set_params(m, p.data());
    if (rc != LB_OK) {
        lb_mlp_destroy(m);
        return rc;
    }
    *out = m;
    return LB_OK;
}

int lb_mlp_destroy(lb_mlp *m) {
    if (!m) return LB_ERR_ARG;
    if (m->stream) cudaStreamSynchronize(m->stream);
    cudaFree(m->p); cudaFree(m->m1); cudaFree(m->m2); cudaFree(m->grad); cudaFree(m->partial);
    cudaFree(m->w1b); cudaFree(m->w2b);
    if (m->stream) cudaStreamDestroy(m->stream);
    delete m;
    return LB_OK;
}

const char *lb_mlp_error(const lb_mlp *m) { return m ? m->err.c_str() : "null network"; }
int lb_mlp_num_params(void) { return MLP_NPARAM; }

int lb_mlp_set_params(lb_mlp *m, const float *p) {
    if (!m || !p) return LB_ERR_ARG;
    LB_MTRY(m, "set_params", cudaMemcpyAsync(m->p, p, sizeof(float) * MLP_NPARAM,
                                             cudaMemcpyHostToDevice, m->stream));
    LB_MTRY(m, "set_params", cudaMemsetAsync(m->m1, 0, sizeof(float) * MLP_NPARAM, m->stream));
    LB_MTRY(m, "set_params", cudaMemsetAsync(m->m2, 0, sizeof(float) * MLP_NPARAM, m->stream));
    refresh_bf16_kernel<<<(MLP_H * MLP_H + 255) / 256, 256, 0, m->stream>>>(m->p, m->w1b, m->w2b);
    LB_MTRY(m, "refresh_bf16", cudaGetLastError());
    m->step = 0;
    LB_MTRY(m, "set_params", cudaStreamSynchronize(m->stream));
    return LB_OK;
}

int lb_mlp_get_params(lb_mlp *m, float *p) {
    if (!m || !p) return LB_ERR_ARG;
    LB_MTRY(m, "get_params", cudaMemcpyAsync(p, m->p, sizeof(float) * MLP_NPARAM,
                                             cudaMemcpyDeviceToHost, m->stream));
    LB_MTRY(m, "get_params", cudaStreamSynchronize(m->stream));
    return LB_OK;
}

int lb_mlp_forward(lb_mlp *m, const float *x_dev, float *y_dev, long n) {
    if (!m || !x_dev || !y_dev || n < 0) return LB_ERR_ARG;
    const int nb = (int)std::min<long>(1216, (n + 127) / 128);
    if (nb > 0) mlp_forward_kernel<<<nb, 128, 0, m->stream>>>(mlp_dev(m), x_dev, n, y_dev);
    LB_MTRY(m, "mlp_forward_kernel", cudaGetLastError());
    LB_MTRY(m, "mlp_forward", cudaStreamSynchronize(m->stream));
    return LB_OK;
}

int lb_mlp_grad(lb_mlp *m, const float *x_dev, const float *z_dev, long n, float *grad,
                double *loss) {
    if (!m || !x_dev || !z_dev || n < 1) return LB_ERR_ARG;
    const int rc = mlp_gradient(m, x_dev, z_dev, n);
    if (rc != LB_OK) return rc;
    std::vector<float> h(NGRAD);
    LB_MTRY(m, "grad", cudaMemcpyAsync(h.data(), m->grad, sizeof(float) * NGRAD,
                                       cudaMemcpyDeviceToHost, m->stream));
    LB_MTRY(m, "grad", cudaStreamSynchronize(m->stream));
    if (grad) memcpy(grad, h.data(), sizeof(float) * MLP_NPARAM);
    if (loss) *loss = h[MLP_NPARAM];
    return LB_OK;
}

// Adam over random contiguous windows of `batch` samples (a 64-bit LCG
// picks the window starts); loss_log[i] = loss of step i (optional)
int lb_mlp_train(lb_mlp *m, const float *x_dev, const float *z_dev, long n, int steps,
                 int batch, float lr, uint64_t seed, float *loss_log) {
    if (!m || !x_dev || !z_dev || n < 1 || steps < 0 || batch < 1) return LB_ERR_ARG;
    if (batch > n) batch = (int)n;
    uint64_t st = seed * 2862933555777941757ULL + 3037000493ULL;
    for (int it = 0; it < steps; it++) {
        st = st * 6364136223846793005ULL + 1442695040888963407ULL;
        const long start = (long)((st >> 17) % (uint64_t)(n - batch + 1));
        int rc = mlp_gradient(m, x_dev + start * MLP_IN, z_dev + start, batch);
        if (rc != LB_OK) return rc;
        m->step++;
        const float b1c = 1.f - powf(0.9f, (float)m->step), b2c = 1.f - powf(0.999f, (float)m->step);
        adam_kernel<<<(MLP_NPARAM + 255) / 256, 256, 0, m->stream>>>(m->p, m->m1, m->m2, m->grad,
                                                                     lr, b1c, b2c, m->w1b, m->w2b);
        LB_MTRY(m, "adam_kernel", cudaGetLastError());
        if (loss_log) {
            float l;
            LB_MTRY(m, "loss", cudaMemcpyAsync(&l, m->grad + MLP_NPARAM, sizeof(float),
                                               cudaMemcpyDeviceToHost, m->stream));
            LB_MTRY(m, "loss", cudaStreamSynchronize(m->stream));
            loss_log[it] = l;
        }
    }
    LB_MTRY(m, "train", cudaStreamSynchronize(m->stream));
    return LB_OK;
}

int lb_closure_enable(lb_ctx *ctx, const lb_mlp *m, float nu0, float s_ref, float z_max,
                      float *y_out_dev) {
    if (!ctx) return LB_ERR_ARG;
    if (!m) return context_set_closure(ctx, nullptr);
    if (!(nu0 > 0.f) || !(s_ref > 0.f) || !(z_max >= 0.f)) return LB_ERR_ARG;
    ClosureArgs ca{};
    ca.mlp = mlp_dev(m);
    cudaError_t e = cudaSuccess;
    const std::pair<float *, int> head[4] = {{ca.head_b1, MLP_OFF_B1}, {ca.head_b2, MLP_OFF_B2},
                                             {ca.head_w3, MLP_OFF_W3}, {&ca.head_b3, MLP_OFF_B3}};
    for (int i = 0; i < 4 && e == cudaSuccess; i++)
        e = cudaMemcpy(head[i].first, m->p + head[i].second,
                       sizeof(float) * (i == 3 ? 1 : MLP_H), cudaMemcpyDeviceToHost);
    if (e != cudaSuccess) return LB_ERR_CUDA;
    ca.nu0 = nu0;
    ca.tau0 = 0.5f + 3.f * nu0;
    ca.s_ref = s_ref;
    ca.z_max = z_max;
    ca.y_out = y_out_dev;
    return context_set_closure(ctx, &ca);
}

// training data from a fine lattice: filter its last-step moment fields by
// `factor` and write features [Nc][19] and targets [Nc] (device buffers, Nc =
// nodes / factor^3) and the mean resolved kinetic energy of the filtered field
int lb_closure_sample(lb_ctx *fine, int factor, float nu0, float s_ref, float z_max,
                      float *features_dev, float *targets_dev, double *ke_mean) {
    return lb_closure_sample_avg(fine, factor, nu0, s_ref, z_max, 0, features_dev, targets_dev,
                                 ke_mean);
}

int lb_closure_sample_avg(lb_ctx *fine, int factor, float nu0, float s_ref, float z_max,
                          int avg_radius, float *features_dev, float *targets_dev,
                          double *ke_mean) {
    if (!fine || factor < 1 || avg_radius < 0) return LB_ERR_ARG;
    float *f[4];
    int rc = lb_device_fields(fine, &f[0], &f[1], &f[2], &f[3]);
    if (rc != LB_OK) return rc;
    int W, H, D;
    rc = lb_extents(fine, &W, &H, &D);
    if (rc != LB_OK) return rc;
    if (W % factor || H % factor || D % factor) return LB_ERR_ARG;
    const int Wc = W / factor, Hc = H / factor, Dc = D / factor;
    const long Nc = (long)Wc * Hc * Dc;
    float *fl = nullptr;
    if (cudaMalloc(&fl, sizeof(float) * 12 * Nc) != cudaSuccess) return LB_ERR_NOMEM;
    cudaError_t e = cudaDeviceSynchronize();
    if (e == cudaSuccess) {
        filter_kernel<<<(unsigned)((Nc + 255) / 256), 256>>>(f[0], f[1], f[2], f[3], W, H, D,
                                                             factor, fl, Nc);
        e = cudaGetLastError();
    }
    float *ts = fl + 10 * Nc, *ss = fl + 11 * Nc;
    if (e == cudaSuccess && features_dev && targets_dev && avg_radius > 0) {
        ts_ss_kernel<<<(unsigned)((Nc + 255) / 256), 256>>>(fl, Wc, Hc, Dc, ts, ss);
        e = cudaGetLastError();
    }
    if (e == cudaSuccess && features_dev && targets_dev) {
        features_kernel<<<(unsigned)((Nc + 255) / 256), 256>>>(fl, Wc, Hc, Dc, nu0, s_ref, z_max,
                                                               ts, ss, avg_radius, features_dev,
                                                               targets_dev);
        e = cudaGetLastError();
    }
    if (e == cudaSuccess && ke_mean) {
        std::vector<float> h(4 * Nc);
        e = cudaMemcpy(h.data(), fl, sizeof(float) * 4 * Nc, cudaMemcpyDeviceToHost);
        double ke = 0.0;
        for (long c = 0; c < Nc; c++) {
            const double ux = h[Nc + c], uy = h[2 * Nc + c], uz = h[3 * Nc + c];
            ke += 0.5 * h[c] * (ux * ux + uy * uy + uz * uz);
        }
        *ke_mean = ke / (double)Nc;
    }
    if (e == cudaSuccess) e = cudaDeviceSynchronize();
    cudaFree(fl);
    return e == cudaSuccess ? LB_OK : LB_ERR_CUDA;
}

}  // extern "C"
