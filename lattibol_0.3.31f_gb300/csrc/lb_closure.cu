// lb_closure.cu -- learned sub-grid closure for under-resolved D3Q19 flow.
//
// * d3q19_closure_tc_kernel: the fused native D3Q19 step in which every cell's
//   relaxation time comes from the closure network.  Per cell it forms 19
//   features from the pre-collision populations -- the 18 non-conserved
//   non-equilibrium moments (momentum 3, stress 6, third/fourth order 9 in
//   the raw basis c_x c_y^2, ..., c_y^2 c_z^2) scaled by 1/(rho c_s^2 tau0
//   s_ref), and |S| / s_ref with S = -Pi_neq / (2 rho c_s^2 tau0) -- and the
//   block evaluates the network for its 128 cells on the tensor cores.  The
//   output y gives nu_t = nu0 * clamp(y, 0, z_max) and tau = 0.5 + 3 (nu0 +
//   nu_t).
// * filter / feature kernels: box-filter a fine lattice's moments onto a
//   coarse grid (Favre averages), and from the filtered fields build the
//   same 19 features (stress features -2 S/s_ref from central differences of
//   the filtered velocity; the other moments are zero at first order) and
//   the target z = nu_t/nu0 of the local least-squares eddy viscosity of the
//   filtered sub-grid stress, nu_t = max(0, -(T_dev : S) / (2 S : S)).
// * training: forward and backward passes over 128-sample tiles with every
//   contraction on the tensor cores (mlp_tc_kernel), per-block gradient sums
//   accumulated in tensor memory, a fixed-order reduction of the block
//   partials, and Adam.
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

// ---------------------------------------------------------------------------
// The fused native D3Q19 step (F32 storage) with the network on the
// 5th-generation tensor cores.  A block of 128 threads takes a run of 128
// cells; thread t owns cell t, row t of the
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
// Rounding points (restated by the numpy oracle): BF16 inputs, weights and
// first hidden layer; FP32 accumulation, biases and last layer, whose
// products are fused into the sum.
// ---------------------------------------------------------------------------
// ReLU and round-to-nearest BF16 of two floats in one conversion, lo in the
// low half (the PTX packs its first source into the high half)
__device__ __forceinline__ uint32_t bf16x2_relu(float lo, float hi) {
    uint32_t d;
    asm("cvt.rn.relu.bf16x2.f32 %0, %1, %2;" : "=r"(d) : "f"(hi), "f"(lo));
    return d;
}

// n / d for 32-bit n and d by one multiply-high with c = floor((2^64 - 1) / d)
// + 1 (exact for every 32-bit n and d >= 2: Lemire, Kaser and Kurz, "Faster
// remainder by direct computation", 2019); d = 1 is n itself
__host__ __device__ __forceinline__ uint64_t div_constant(uint32_t d) {
    return d > 1 ? ~0ull / d + 1 : 0;
}
__device__ __forceinline__ uint32_t div_u32(uint32_t n, uint64_t c, uint32_t d) {
    return d > 1 ? (uint32_t)__umul64hi(c, (uint64_t)n) : n;
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
        const int z = (int)div_u32((uint32_t)u.o, ca.div_wh, (uint32_t)WH), rem = u.o - z * WH;
        const int y = (int)div_u32((uint32_t)rem, ca.div_w, (uint32_t)a.W), x = rem - y * a.W;
        const uint8_t fl = u.inside ? a.flags[u.o] : CELL_WALL;
        u.fluid = !(fl & CELL_WALL);
        if (u.fluid) {
            const Nbr3 n(x, y, z, a.W, a.H, a.D);
            pull_native<float, true>(a, u.o, n, fl, u.g);
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
    ClosureArgs c = ca;
    c.div_wh = div_constant((uint32_t)(a.W * a.H));
    c.div_w = div_constant((uint32_t)a.W);
    if (mom) d3q19_closure_tc_kernel<true><<<g, D3_BLOCK, 0, s>>>(a, c);
    else d3q19_closure_tc_kernel<false><<<g, D3_BLOCK, 0, s>>>(a, c);
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

// ------------------------------------------------------------------ network
// The network's forward pass and, for training, its backward pass over tiles
// of 128 samples on the 5th-generation tensor cores.  Thread t owns sample t
// of a tile, row t of the sample-major MMA tiles, column t of the transposed
// (sample-contracted) tiles and lane t of tensor memory.  Thread 0 issues
// every MMA (BF16 operands in shared memory, K-major core matrices,
// lb_tc05.cuh; FP32 accumulators in tensor memory) and commits it to one
// mbarrier.  Per tile:
//   1. x (19 features, padded to 32) -> row t of A; D_h1 = A W1^T;
//   2. h1 = ReLU(D_h1 + b1) as BF16 -> row t of A (K 64) and column t of
//      H1^T; D_h2 = A W2^T;
//   3. h2 = ReLU(D_h2 + b2), y = b3 + sum_j w3_j h2_j (paired FP32, as the
//      closure kernel).  Forward only: y is the output.  Training:
//      dy = 2 (y - z) / n, dH2 = dy w3 (h2 > 0) as BF16 -> row t of A and
//      column t of dH2^T; h2 and dy as BF16 -> column t of H2^T and of dY;
//      D_dh1 = dH2 W2 (B = W2^T);
//   4. dH1 = D_dh1 (h1 > 0) as BF16 -> column t of dH1^T; then two MMAs
//      contract over the tile's samples into accumulators that persist
//      across the block's tiles:
//        G  = [dH2^T; dH1^T] [H1^T; X^T; 1]^T  (M 128, N 96): dW2 = G[0:64,
//             0:64], dW1 = G[64:128, 64:83], db2 = G[0:64, 83], db1 =
//             G[64:128, 83] (the other blocks of G are not read);
//        G3 = [H2^T; 1] dY^T  (M 128, N 16): dw3 = G3[0:64, 0], db3 = G3[64, 0].
// After its last tile each block writes its sums, already divided by n, and
// its loss sum to partial[block][NGRAD].
// Rounding points (restated by the numpy oracle): x, W1, W2, h1 enter the
// forward MMAs as BF16; dH2, dH1, h1, x, h2 and dy enter the gradient MMAs
// as BF16; every accumulation is FP32.
namespace net {
constexpr int OFF_W1 = 0;                               // W1 [64][32]: B of layer 1
constexpr int OFF_W2 = OFF_W1 + MLP_H * MLP_IN_PAD * 2; // W2 [j][i]: B of layer 2
constexpr int OFF_A = OFF_W2 + MLP_H * MLP_H * 2;       // x (K 32), h1, then dH2 (K 64)
constexpr int OFF_F = OFF_A + 128 * MLP_H * 2;          // b1, b2, w3, b3, loss, mbarrier, slot
constexpr int FWD_SMEM = OFF_F + 1024;
constexpr int OFF_W2T = FWD_SMEM;                       // W2^T [i][j]: B of dH1 = dH2 W2
constexpr int OFF_GA = OFF_W2T + MLP_H * MLP_H * 2;     // [dH2^T; dH1^T] [128][128 samples]
constexpr int OFF_GB = OFF_GA + 128 * 128 * 2;          // [H1^T; X^T; 1; 0] [96][128]
constexpr int OFF_HA = OFF_GB + 96 * 128 * 2;           // [H2^T; 1; 0] [128][128]
constexpr int OFF_DY = OFF_HA + 128 * 128 * 2;          // [dY; 0] [16][128]
constexpr int TRAIN_SMEM = OFF_DY + 16 * 128 * 2;
// tensor-memory columns
constexpr uint32_t COL_H1 = 0, COL_H2 = 64, COL_G = 128, COL_G3 = 224;
constexpr int ROW_ONES = 64 + MLP_IN;  // the row of ones in [H1^T; X^T; 1; 0]
static_assert(OFF_F % 16 == 0 && OFF_GA % 16 == 0 && OFF_GB % 16 == 0 && OFF_HA % 16 == 0 &&
                  OFF_DY % 16 == 0 && TRAIN_SMEM <= 227 * 1024,
              "descriptor start addresses on 16 bytes; one block fits the SM");
static_assert(COL_G3 + 16 <= 256 && ROW_ONES < 96, "tensor-memory and tile extents");
}  // namespace net
constexpr int NGRAD = MLP_NPARAM + 1;  // + loss
constexpr int NET_FWD_SMEM = 50 * 1024;  // at most 4 blocks (4 x 128 columns) per SM

__device__ __forceinline__ void st_b16(uint8_t *base, uint32_t off, uint32_t bits) {
    *reinterpret_cast<uint16_t *>(base + off) = (uint16_t)bits;
}
__device__ __forceinline__ uint32_t bf16x2_bits(float lo, float hi) {
    const __nv_bfloat162 p = __floats2bfloat162_rn(lo, hi);
    return *reinterpret_cast<const uint32_t *>(&p);
}
// Rows r0 .. r0+3 (r0 a multiple of 4) of column t of a sample-contracted
// tile (K = 128 samples), from w01 (rows r0, r0+1 in its low, high half) and
// w23.  The four 8-lane groups of a warp start at different rows, so the four
// 16-byte pieces of each store instruction fall in different banks.
__device__ __forceinline__ void st_col4(uint8_t *tile, int r0, int t, uint32_t w01,
                                        uint32_t w23) {
    const int g = (t >> 3) & 3;
    const uint32_t off = kmajor_offset(r0, t, 128);
#pragma unroll
    for (int u = 0; u < 4; u++) {
        const int k = (g + u) & 3;  // row r0 + k: 16 k bytes further in the core matrix
        const uint32_t w = (k & 2) ? w23 : w01;
        st_b16(tile, off + 16 * k, (k & 1) ? w >> 16 : w);
    }
}

template <bool TRAIN>
__global__ void __launch_bounds__(128, 1) mlp_tc_kernel(const MlpDev mlp, const float *X,
                                                     const float *Z, long n, float *out,
                                                     int *err) {
    using namespace net;
    extern __shared__ __align__(1024) uint8_t smem[];
    constexpr uint32_t NCOLS = TRAIN ? 256 : 128;
    uint8_t *sA = smem + OFF_A, *sGA = smem + OFF_GA, *sGB = smem + OFF_GB;
    uint8_t *sHA = smem + OFF_HA, *sDY = smem + OFF_DY;
    float *sb1 = reinterpret_cast<float *>(smem + OFF_F), *sb2 = sb1 + MLP_H, *sw3 = sb2 + MLP_H;
    float *sloss = sw3 + MLP_H + 1;  // after b3: one sum per warp
    uint64_t *mbar = reinterpret_cast<uint64_t *>(smem + OFF_F + 800);
    uint32_t *tslot = reinterpret_cast<uint32_t *>(smem + OFF_F + 808);
    const int t = threadIdx.x, warp = t >> 5, lane = t & 31;

    // the first tile's inputs are loaded before the weights are staged, every
    // later tile's while the MMAs of the one before run
    float x[MLP_IN], zn = 0.f;
    auto load_inputs = [&](long b) {
        const long s = b + t;
        const bool v = s < n;
#pragma unroll
        for (int i = 0; i < MLP_IN; i++) x[i] = v ? X[s * MLP_IN + i] : 0.f;
        if (TRAIN) zn = v ? Z[s] : 0.f;
    };
    load_inputs((long)blockIdx.x * 128);
    // the weights in 16-byte pieces (8 BF16 of a row), all loads issued first:
    // W1 2 pieces per thread, W2 4 and, for training, W2^T 4
    {
        const uint4 *w1v = reinterpret_cast<const uint4 *>(mlp.w1);
        const uint4 *w2v = reinterpret_cast<const uint4 *>(mlp.w2);
        const uint4 *w2tv = reinterpret_cast<const uint4 *>(mlp.w2t);
        uint4 p1[2], p2[4], p3[4];
#pragma unroll
        for (int u = 0; u < 2; u++) p1[u] = w1v[t + 128 * u];
#pragma unroll
        for (int u = 0; u < 4; u++) p2[u] = w2v[t + 128 * u];
        if (TRAIN) {
#pragma unroll
            for (int u = 0; u < 4; u++) p3[u] = w2tv[t + 128 * u];
        }
        const float bv1 = t < MLP_H ? mlp.b1[t] : 0.f, bv2 = t < MLP_H ? mlp.b2[t] : 0.f;
        const float wv3 = t < MLP_H ? mlp.w3[t] : 0.f, bv3 = mlp.b3[0];
#pragma unroll
        for (int u = 0; u < 2; u++) {
            const int q = t + 128 * u;  // row q / 4, columns 8 (q % 4) ..
            *reinterpret_cast<uint4 *>(smem + OFF_W1 +
                                       kmajor_offset(q / 4, 8 * (q % 4), MLP_IN_PAD)) = p1[u];
        }
#pragma unroll
        for (int u = 0; u < 4; u++) {
            const int q = t + 128 * u, j = q / 8, k0 = 8 * (q % 8);  // row j, columns k0 ..
            *reinterpret_cast<uint4 *>(smem + OFF_W2 + kmajor_offset(j, k0, MLP_H)) = p2[u];
            if (TRAIN)
                *reinterpret_cast<uint4 *>(smem + OFF_W2T + kmajor_offset(j, k0, MLP_H)) = p3[u];
        }
        if (t < MLP_H) {
            sb1[t] = bv1;
            sb2[t] = bv2;
            sw3[t] = wv3;
        }
        if (t == 0) sw3[MLP_H] = bv3;
    }
    if (TRAIN) {
        // the constant rows: ones (bias gradients) and zeros (padding)
        constexpr uint32_t ONE = 0x3F80u;  // 1.0 in BF16
        for (int r = ROW_ONES; r < 96; r++) st_b16(sGB, kmajor_offset(r, t, 128), r == ROW_ONES ? ONE : 0u);
        for (int r = MLP_H; r < 128; r++) st_b16(sHA, kmajor_offset(r, t, 128), r == MLP_H ? ONE : 0u);
        for (int r = 1; r < 16; r++) st_b16(sDY, kmajor_offset(r, t, 128), 0u);
        if (t < 4) sloss[t] = 0.f;
    }
    if (t == 0) mbar_init(mbar, 1);
    if (warp == 0) tc_alloc(tslot, NCOLS);
    fence_proxy_async();
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    const uint32_t tmem = *tslot;
    const uint32_t lane_base = tmem + ((uint32_t)(warp * 32) << 16);
    const uint32_t a_addr = smem_u32(sA), w1_addr = smem_u32(smem + OFF_W1);
    const uint32_t w2_addr = smem_u32(smem + OFF_W2), w2t_addr = smem_u32(smem + OFF_W2T);
    const uint32_t ga_addr = smem_u32(sGA), gb_addr = smem_u32(sGB);
    const uint32_t ha_addr = smem_u32(sHA), dy_addr = smem_u32(sDY);
    constexpr uint32_t ID64 = tc_idesc_bf16(128, MLP_H), ID96 = tc_idesc_bf16(128, 96),
                       ID16 = tc_idesc_bf16(128, 16);
    uint32_t phase = 0;
    bool ok = true;
    // every thread's shared-memory writes are made visible to the tensor core,
    // thread 0 issues the MMAs and waits (bounded) for their commit while the
    // others wait at the block barrier
    auto run_mma = [&](auto issue) -> bool {
        fence_proxy_async();
        tc_fence_before();
        __syncthreads();
        if (t == 0) {
            tc_fence_after();
            issue();
            tc_commit(mbar);
        }
        const bool done = __syncthreads_and(t == 0 ? mbar_wait(mbar, phase, TC_WAIT) : true);
        phase ^= 1;
        tc_fence_after();
        return done;
    };

    const float inv_n = 1.f / (float)n;
    int ntile = 0;
    for (long base = (long)blockIdx.x * 128; base < n; base += (long)gridDim.x * 128, ntile++) {
        const long s = base + t;
        const bool valid = s < n;
        const float zv = zn;
        // 1. x -> row t of A (K 32); training: column t of X^T
#pragma unroll
        for (int h = 0; h < MLP_IN_PAD / 8; h++) {
            uint32_t p[4];
#pragma unroll
            for (int j = 0; j < 4; j++) {
                const int k0 = 8 * h + 2 * j;
                p[j] = bf16x2_bits(k0 < MLP_IN ? x[k0] : 0.f, k0 + 1 < MLP_IN ? x[k0 + 1] : 0.f);
            }
            // rows 64 + k of [H1^T; X^T; 1; 0]: features 0-18, then the row of ones
            constexpr uint32_t ONE_HI = 0x3F800000u;  // BF16 1.0 in the high half
            static_assert(MLP_IN % 4 == 3, "the row of ones closes the features' last group of 4");
            if (TRAIN && 8 * h < MLP_IN)
                st_col4(sGB, MLP_H + 8 * h, t, p[0], 8 * h + 3 == MLP_IN ? p[1] | ONE_HI : p[1]);
            if (TRAIN && 8 * h + 4 < MLP_IN)
                st_col4(sGB, MLP_H + 8 * h + 4, t, p[2], 8 * h + 7 == MLP_IN ? p[3] | ONE_HI : p[3]);
            *reinterpret_cast<uint4 *>(sA + kmajor_offset(t, 8 * h, MLP_IN_PAD)) =
                make_uint4(p[0], p[1], p[2], p[3]);
        }
        if (base + (long)gridDim.x * 128 < n) load_inputs(base + (long)gridDim.x * 128);
        ok = run_mma([&] {
#pragma unroll
            for (int k = 0; k < MLP_IN_PAD / 16; k++)
                tc_mma_bf16(tmem + COL_H1, tc_desc(a_addr + 256 * k, 128, MLP_IN_PAD / 8 * 128),
                            tc_desc(w1_addr + 256 * k, 128, MLP_IN_PAD / 8 * 128), ID64, k > 0);
        });
        if (!ok) break;
        // 2. h1 = ReLU(D + b1) as BF16 -> row t of A (K 64); training: column t
        // of H1^T and the mask h1 > 0
        uint64_t m1 = 0;
#pragma unroll
        for (int c = 0; c < MLP_H; c += 32) {
            float v[32];
            tc_ld32(lane_base + COL_H1 + (uint32_t)c, v);
#pragma unroll
            for (int h = 0; h < 4; h++) {
                uint32_t p[4];
#pragma unroll
                for (int j = 0; j < 4; j++) {
                    const int q = 8 * h + 2 * j;
                    const float2 hv = __fadd2_rn(make_float2(v[q], v[q + 1]),
                                                 make_float2(sb1[c + q], sb1[c + q + 1]));
                    p[j] = bf16x2_relu(hv.x, hv.y);
                    if (TRAIN) {
                        m1 |= (uint64_t)((p[j] & 0xFFFFu) != 0u) << (c + q);
                        m1 |= (uint64_t)((p[j] >> 16) != 0u) << (c + q + 1);
                    }
                }
                if (TRAIN) {
                    st_col4(sGB, c + 8 * h, t, p[0], p[1]);
                    st_col4(sGB, c + 8 * h + 4, t, p[2], p[3]);
                }
                *reinterpret_cast<uint4 *>(sA + kmajor_offset(t, c + 8 * h, MLP_H)) =
                    make_uint4(p[0], p[1], p[2], p[3]);
            }
        }
        ok = run_mma([&] {
#pragma unroll
            for (int k = 0; k < MLP_H / 16; k++)
                tc_mma_bf16(tmem + COL_H2, tc_desc(a_addr + 256 * k, 128, MLP_H / 8 * 128),
                            tc_desc(w2_addr + 256 * k, 128, MLP_H / 8 * 128), ID64, k > 0);
        });
        if (!ok) break;
        // 3. y = b3 + sum_j w3_j ReLU(D_j + b2_j), even and odd j in the two
        // lanes of paired FP32 instructions
        float2 y2 = make_float2(0.f, 0.f);
#pragma unroll
        for (int c = 0; c < MLP_H; c += 32) {
            float v[32];
            tc_ld32(lane_base + COL_H2 + (uint32_t)c, v);
#pragma unroll
            for (int j = 0; j < 32; j += 2) {
                float2 h = __fadd2_rn(make_float2(v[j], v[j + 1]),
                                      make_float2(sb2[c + j], sb2[c + j + 1]));
                h.x = fmaxf(h.x, 0.f);
                h.y = fmaxf(h.y, 0.f);
                y2 = __ffma2_rn(make_float2(sw3[c + j], sw3[c + j + 1]), h, y2);
            }
        }
        const float yv = (y2.x + y2.y) + sw3[MLP_H];
        if (!TRAIN) {
            if (valid) out[s] = yv;
            continue;
        }
        const float e = valid ? yv - zv : 0.f;
        const float dy = 2.f * e * inv_n;
        float e2 = e * e;
#pragma unroll
        for (int d = 16; d > 0; d >>= 1) e2 += __shfl_xor_sync(0xffffffffu, e2, d);
        if (lane == 0) sloss[warp] += e2;
        st_b16(sDY, kmajor_offset(0, t, 128), bf16x2_bits(dy, 0.f));
        // dH2 = dy w3 (h2 > 0) as BF16 -> row t of A and column t of dH2^T;
        // h2 as BF16 -> column t of H2^T
#pragma unroll
        for (int c = 0; c < MLP_H; c += 32) {
            float v[32];
            tc_ld32(lane_base + COL_H2 + (uint32_t)c, v);
#pragma unroll
            for (int h = 0; h < 4; h++) {
                uint32_t p[4], hb[4];
#pragma unroll
                for (int j = 0; j < 4; j++) {
                    const int q = 8 * h + 2 * j;
                    float2 hv = __fadd2_rn(make_float2(v[q], v[q + 1]),
                                           make_float2(sb2[c + q], sb2[c + q + 1]));
                    hv.x = fmaxf(hv.x, 0.f);
                    hv.y = fmaxf(hv.y, 0.f);
                    p[j] = bf16x2_bits(hv.x > 0.f ? dy * sw3[c + q] : 0.f,
                                       hv.y > 0.f ? dy * sw3[c + q + 1] : 0.f);
                    hb[j] = bf16x2_bits(hv.x, hv.y);
                }
                st_col4(sGA, c + 8 * h, t, p[0], p[1]);
                st_col4(sGA, c + 8 * h + 4, t, p[2], p[3]);
                st_col4(sHA, c + 8 * h, t, hb[0], hb[1]);
                st_col4(sHA, c + 8 * h + 4, t, hb[2], hb[3]);
                *reinterpret_cast<uint4 *>(sA + kmajor_offset(t, c + 8 * h, MLP_H)) =
                    make_uint4(p[0], p[1], p[2], p[3]);
            }
        }
        ok = run_mma([&] {
#pragma unroll
            for (int k = 0; k < MLP_H / 16; k++)
                tc_mma_bf16(tmem + COL_H1, tc_desc(a_addr + 256 * k, 128, MLP_H / 8 * 128),
                            tc_desc(w2t_addr + 256 * k, 128, MLP_H / 8 * 128), ID64, k > 0);
        });
        if (!ok) break;
        // 4. dH1 = D (h1 > 0) as BF16 -> column t of dH1^T
#pragma unroll
        for (int c = 0; c < MLP_H; c += 32) {
            float v[32];
            tc_ld32(lane_base + COL_H1 + (uint32_t)c, v);
#pragma unroll
            for (int j = 0; j < 32; j += 4) {
                const uint32_t p01 = bf16x2_bits((m1 >> (c + j)) & 1 ? v[j] : 0.f,
                                                 (m1 >> (c + j + 1)) & 1 ? v[j + 1] : 0.f);
                const uint32_t p23 = bf16x2_bits((m1 >> (c + j + 2)) & 1 ? v[j + 2] : 0.f,
                                                 (m1 >> (c + j + 3)) & 1 ? v[j + 3] : 0.f);
                st_col4(sGA, MLP_H + c + j, t, p01, p23);
            }
        }
        const uint32_t acc = ntile > 0 ? 1u : 0u;
        ok = run_mma([&] {
#pragma unroll
            for (int k = 0; k < 128 / 16; k++)
                tc_mma_bf16(tmem + COL_G, tc_desc(ga_addr + 256 * k, 128, 128 / 8 * 128),
                            tc_desc(gb_addr + 256 * k, 128, 128 / 8 * 128), ID96, acc | (k > 0));
#pragma unroll
            for (int k = 0; k < 128 / 16; k++)
                tc_mma_bf16(tmem + COL_G3, tc_desc(ha_addr + 256 * k, 128, 128 / 8 * 128),
                            tc_desc(dy_addr + 256 * k, 128, 128 / 8 * 128), ID16, acc | (k > 0));
        });
        if (!ok) break;
    }
    if (TRAIN && ok) {
        // the block's sums: warps 0-1 hold rows j of dW2, db2 and dw3, warps
        // 2-3 rows i of dW1 and db1, lane 64 db3
        float *pb = out + (long)blockIdx.x * NGRAD;
        float v[32];
        if (ntile == 0) {
            for (int i = t; i < NGRAD; i += 128) pb[i] = 0.f;
        } else {
            if (warp < 2) {
#pragma unroll
                for (int c = 0; c < MLP_H; c += 32) {
                    tc_ld32(lane_base + COL_G + (uint32_t)c, v);
#pragma unroll
                    for (int i = 0; i < 32; i++) pb[MLP_OFF_W2 + t * MLP_H + c + i] = v[i];
                }
            }
            tc_ld32(lane_base + COL_G + MLP_H, v);
            if (warp < 2) {
                pb[MLP_OFF_B2 + t] = v[MLP_IN];
            } else {
#pragma unroll
                for (int f = 0; f < MLP_IN; f++) pb[MLP_OFF_W1 + (t - MLP_H) * MLP_IN + f] = v[f];
                pb[MLP_OFF_B1 + t - MLP_H] = v[MLP_IN];
            }
            tc_ld32(lane_base + COL_G3, v);
            if (t < MLP_H) pb[MLP_OFF_W3 + t] = v[0];
            else if (t == MLP_H) pb[MLP_OFF_B3] = v[0];
            if (t == 0) pb[MLP_NPARAM] = ((sloss[0] + sloss[1]) + (sloss[2] + sloss[3])) * inv_n;
        }
    }
    if (!ok) {
        // an MMA did not complete: record it, give it one more bounded wait so
        // that no MMA is writing the columns when they are released
        if (t == 0 && err) atomicExch(err, 1);
        mbar_wait(mbar, phase ^ 1, TC_WAIT);
    }
    tc_fence_before();
    __syncthreads();
    if (warp == 0) tc_dealloc(tmem, NCOLS);
    if (t == 0) mbar_inval(mbar);
}

// one Adam step of the FP32 master parameters (p == nullptr: none)
struct AdamStep {
    float *p = nullptr, *m1 = nullptr, *m2 = nullptr;
    __nv_bfloat16 *w1b = nullptr, *w2b = nullptr;
    float lr = 0.f, b1c = 1.f, b2c = 1.f;  // rate, bias corrections 1 - beta^step
};

// Sums of the block partials: a block of 256 threads takes 32 parameters, 8
// threads per parameter each sum a run of consecutive partials (16 loads in
// flight, additions in block order), and the runs' sums are added in run
// order -- a fixed order for a given block count.  The loss also goes into
// *loss_slot (a step's entry of a device-side loss log) when given.  With
// ad.p, the parameter's thread then takes its Adam step and refreshes the
// parameter's BF16 copies.
constexpr int RED_PAR = 32, RED_RUNS = 8;
__global__ void __launch_bounds__(RED_PAR * RED_RUNS)
    grad_reduce_kernel(const float *partial, int nblocks, float *grad, float *loss_slot,
                       const AdamStep ad) {
    __shared__ float run_sum[RED_RUNS][RED_PAR];
    const int pl = threadIdx.x % RED_PAR, run = threadIdx.x / RED_PAR;
    const int i = blockIdx.x * RED_PAR + pl;
    const int per = (nblocks + RED_RUNS - 1) / RED_RUNS;
    const int b0 = min(run * per, nblocks), b1 = min(b0 + per, nblocks);
    float s = 0.f;
    if (i < NGRAD) {
        int b = b0;
        for (; b + 16 <= b1; b += 16) {
            float v[16];
#pragma unroll
            for (int u = 0; u < 16; u++) v[u] = partial[(long)(b + u) * NGRAD + i];
#pragma unroll
            for (int u = 0; u < 16; u++) s = s + v[u];
        }
        for (; b < b1; b++) s = s + partial[(long)b * NGRAD + i];
    }
    run_sum[run][pl] = s;
    __syncthreads();
    if (run != 0 || i >= NGRAD) return;
    s = run_sum[0][pl];
#pragma unroll
    for (int r = 1; r < RED_RUNS; r++) s = s + run_sum[r][pl];
    grad[i] = s;
    if (i == MLP_NPARAM) {
        if (loss_slot) *loss_slot = s;
        return;
    }
    if (!ad.p) return;
    const float a = 0.9f * ad.m1[i] + 0.1f * s;
    const float q = 0.999f * ad.m2[i] + 0.001f * s * s;
    ad.m1[i] = a;
    ad.m2[i] = q;
    const float v = ad.p[i] - ad.lr * (a / ad.b1c) / (sqrtf(q / ad.b2c) + 1e-8f);
    ad.p[i] = v;
    if (i < MLP_OFF_B1)
        ad.w1b[(i / MLP_IN) * MLP_IN_PAD + i % MLP_IN] = __float2bfloat16_rn(v);
    else if (i >= MLP_OFF_W2 && i < MLP_OFF_B2) {
        const int e = i - MLP_OFF_W2;  // W2[e / 64][e % 64], then its transposed copy
        ad.w2b[e] = __float2bfloat16_rn(v);
        ad.w2b[MLP_H * MLP_H + (e % MLP_H) * MLP_H + e / MLP_H] = __float2bfloat16_rn(v);
    }
}

__global__ void refresh_bf16_kernel(const float *p, __nv_bfloat16 *w1b, __nv_bfloat16 *w2b) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < MLP_H * MLP_IN_PAD) {
        const int j = i / MLP_IN_PAD, f = i % MLP_IN_PAD;
        w1b[i] = __float2bfloat16_rn(f < MLP_IN ? p[MLP_OFF_W1 + j * MLP_IN + f] : 0.f);
    }
    if (i < MLP_H * MLP_H) {
        w2b[i] = __float2bfloat16_rn(p[MLP_OFF_W2 + i]);
        w2b[MLP_H * MLP_H + (i % MLP_H) * MLP_H + i / MLP_H] = w2b[i];
    }
}

}  // namespace

struct lb_mlp {
    float *p = nullptr, *m1 = nullptr, *m2 = nullptr, *grad = nullptr, *partial = nullptr;
    __nv_bfloat16 *w1b = nullptr, *w2b = nullptr;  // w2b: W2 [64][64], then W2^T
    int *err_dev = nullptr;  // device word: a tensor-core MMA of the network never completed
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
    d.w2t = m->w2b + MLP_H * MLP_H;
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

// the network kernels' dynamic shared memory above the default 48 KB
cudaError_t mlp_kernel_attributes() {
    static cudaError_t done = cudaErrorNotReady;
    if (done == cudaErrorNotReady) {
        done = cudaFuncSetAttribute(mlp_tc_kernel<true>,
                                    cudaFuncAttributeMaxDynamicSharedMemorySize, net::TRAIN_SMEM);
        if (done == cudaSuccess)
            done = cudaFuncSetAttribute(mlp_tc_kernel<false>,
                                        cudaFuncAttributeMaxDynamicSharedMemorySize, NET_FWD_SMEM);
    }
    return done;
}

// the kernels' error word: nonzero when an MMA never completed
int mlp_check(lb_mlp *m) {
    int h = 0;
    LB_MTRY(m, "mlp error word", cudaMemcpyAsync(&h, m->err_dev, sizeof(int),
                                                 cudaMemcpyDeviceToHost, m->stream));
    LB_MTRY(m, "mlp error word", cudaStreamSynchronize(m->stream));
    if (h) {
        m->err = "a tensor-core MMA of the network did not complete (bounded wait ran out)";
        return LB_ERR_CUDA;
    }
    return LB_OK;
}

// the gradient over n samples into m->grad, then (ad.p) the Adam step
int mlp_gradient(lb_mlp *m, const float *X, const float *Z, long n, float *loss_slot = nullptr,
                 const AdamStep &ad = AdamStep()) {
    LB_MTRY(m, "cudaFuncSetAttribute", mlp_kernel_attributes());
    const long chunks = (n + 127) / 128;
    const int nb = (int)std::min<long>(m->nblocks, chunks);
    mlp_tc_kernel<true><<<nb, 128, net::TRAIN_SMEM, m->stream>>>(mlp_dev(m), X, Z, n, m->partial,
                                                                 m->err_dev);
    LB_MTRY(m, "mlp_tc_kernel", cudaGetLastError());
    grad_reduce_kernel<<<(NGRAD + RED_PAR - 1) / RED_PAR, RED_PAR * RED_RUNS, 0, m->stream>>>(
        m->partial, nb, m->grad, loss_slot, ad);
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
    if (e == cudaSuccess) e = cudaMalloc(&m->w2b, sizeof(__nv_bfloat16) * 2 * MLP_H * MLP_H);
    if (e == cudaSuccess) e = cudaMalloc(&m->err_dev, sizeof(int));
    if (e == cudaSuccess) e = cudaMemset(m->err_dev, 0, sizeof(int));
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
    cudaFree(m->w1b); cudaFree(m->w2b); cudaFree(m->err_dev);
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
    LB_MTRY(m, "cudaFuncSetAttribute", mlp_kernel_attributes());
    static int cap = 0;  // SMs x 4: the blocks whose tensor memory (128 columns) fits at once
    if (!cap) {
        int dev = 0, sms = 1;
        cudaGetDevice(&dev);
        cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
        cap = 4 * sms;
    }
    const int nb = (int)std::min<long>(cap, (n + 127) / 128);
    if (nb > 0)
        mlp_tc_kernel<false><<<nb, 128, NET_FWD_SMEM, m->stream>>>(mlp_dev(m), x_dev, nullptr, n,
                                                                   y_dev, m->err_dev);
    LB_MTRY(m, "mlp_tc_kernel", cudaGetLastError());
    return mlp_check(m);
}

int lb_mlp_grad(lb_mlp *m, const float *x_dev, const float *z_dev, long n, float *grad,
                double *loss) {
    if (!m || !x_dev || !z_dev || n < 1) return LB_ERR_ARG;
    const int rc = mlp_gradient(m, x_dev, z_dev, n);
    if (rc != LB_OK) return rc;
    std::vector<float> h(NGRAD);
    LB_MTRY(m, "grad", cudaMemcpyAsync(h.data(), m->grad, sizeof(float) * NGRAD,
                                       cudaMemcpyDeviceToHost, m->stream));
    const int crc = mlp_check(m);
    if (crc != LB_OK) return crc;
    if (grad) memcpy(grad, h.data(), sizeof(float) * MLP_NPARAM);
    if (loss) *loss = h[MLP_NPARAM];
    return LB_OK;
}

// Adam over random contiguous windows of `batch` samples (a 64-bit LCG
// picks the window starts); loss_log[i] = loss of step i (optional).  The
// steps are queued without a host round trip: the losses go to a device log
// that is copied back once.
int lb_mlp_train(lb_mlp *m, const float *x_dev, const float *z_dev, long n, int steps,
                 int batch, float lr, uint64_t seed, float *loss_log) {
    if (!m || !x_dev || !z_dev || n < 1 || steps < 0 || batch < 1) return LB_ERR_ARG;
    if (batch > n) batch = (int)n;
    float *log_dev = nullptr;
    if (loss_log && steps > 0)
        LB_MTRY(m, "loss log", cudaMalloc(&log_dev, sizeof(float) * steps));
    struct Free {
        float *p;
        ~Free() { cudaFree(p); }
    } free_log{log_dev};
    uint64_t st = seed * 2862933555777941757ULL + 3037000493ULL;
    for (int it = 0; it < steps; it++) {
        st = st * 6364136223846793005ULL + 1442695040888963407ULL;
        const long start = (long)((st >> 17) % (uint64_t)(n - batch + 1));
        m->step++;
        AdamStep ad;
        ad.p = m->p;
        ad.m1 = m->m1;
        ad.m2 = m->m2;
        ad.w1b = m->w1b;
        ad.w2b = m->w2b;
        ad.lr = lr;
        ad.b1c = 1.f - powf(0.9f, (float)m->step);
        ad.b2c = 1.f - powf(0.999f, (float)m->step);
        const int rc = mlp_gradient(m, x_dev + start * MLP_IN, z_dev + start, batch,
                                    log_dev ? log_dev + it : nullptr, ad);
        if (rc != LB_OK) return rc;
    }
    if (log_dev)
        LB_MTRY(m, "loss log", cudaMemcpyAsync(loss_log, log_dev, sizeof(float) * steps,
                                               cudaMemcpyDeviceToHost, m->stream));
    return mlp_check(m);
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
