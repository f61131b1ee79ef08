// lb_tblock.cu -- D2Q9 temporal blocking for lattices whose state lives in
// L2 (the 256^2 lid-driven cavity and smaller): one launch advances TS steps.
//
// A block owns a BX x BY tile.  It loads the tile and a halo of TS nodes on
// every side (periodic wrap) into shared memory, then advances the whole
// region one step at a time between two shared-memory buffers; the region
// whose result is still exact shrinks by one node per step, so after TS steps
// the tile itself is exact and goes back to global memory.  The halo nodes
// are recomputed by every block that needs them: for TS = 4 and 16 x 16
// tiles that is 1.43 node updates per lattice update, paid in shared-memory
// arithmetic instead of a launch and an L2 round trip per step.
//
// The per-node update is the native-mode fused step of lb_d2q9.cu (pull,
// half-way bounce-back with the moving-wall term, moments, velocity-shift
// force, BGK), built from the same device functions, so every population is
// bit-identical to TS launches of d2q9_fused_kernel.  Shan-Chen (whose force
// needs psi of the whole neighbourhood at the same time level) and the
// reference mode (Zou-He on the inlet and outlet columns) keep the per-step
// kernels.
#include "lb_kernels.cuh"

namespace lb {

namespace {

// pulls the nine populations of region node i from buffer `cur` (SoA, RN
// nodes per population, rows of RX nodes); near-wall nodes take their own
// opposite population where the upstream node is a wall (half-way
// bounce-back), minus the moving-wall term.  Same rule as the fused kernel.
// The choice is made per warp (the near-wall form is exact for every node),
// so warps away from walls run the plain pull with constant offsets only.
template <int RX, int RN>
__device__ __forceinline__ void tb_pull(const float *cur, const uint8_t *fl, int i, uint8_t f,
                                        const float *corr, float (&g)[9]) {
    if (__any_sync(__activemask(), f & CELL_NEAR_WALL)) {
#pragma unroll
        for (int k = 0; k < 9; k++) {
            const int up = i - d2_cx(k) - RX * d2_cr(k);
            const uint8_t fu = k == 0 ? 0 : fl[up];
            if (fu & CELL_WALL) {
                const float v = cur[d2_opp(k) * RN + i];
                g[k] = (fu & CELL_MOVING) ? v - corr[d2_opp(k)] : v;
            } else {
                g[k] = cur[k * RN + up];
            }
        }
    } else {
#pragma unroll
        for (int k = 0; k < 9; k++) g[k] = cur[k * RN + i - d2_cx(k) - RX * d2_cr(k)];
    }
}

// collision of the fused native step: moments, force shift, BGK
__device__ __forceinline__ void tb_collide(const D2Args &a, float (&g)[9], float &rho, float &ux,
                                           float &uy) {
    d2q9_collide_native(g, a.Fx, a.Fy, a.w0, a.w1, a.w5, a.tau_inv, rho, ux, uy);
}

// one inner step s (1 <= s < TS): region nodes [s, R - s) in both axes,
// shared buffer `cur` -> `nxt`
template <int RX, int RY, int NT, int S>
__device__ __forceinline__ void tb_inner_step(const D2Args &a, const float *cur, float *nxt,
                                              const uint8_t *fl, const float *corr) {
    constexpr int RN = RX * RY;
    constexpr int NX = RX - 2 * S, NY = RY - 2 * S, N = NX * NY;
    // the active nodes are dealt out to the threads in order, so only the
    // last warp of a step has idle lanes
    for (int j = threadIdx.x; j < N; j += NT) {
        const int i = (S + j % NX) + RX * (S + j / NX);
        const uint8_t f = fl[i];
        if (f & CELL_WALL) continue;  // never read by a fluid node
        float g[9], rho, ux, uy;
        tb_pull<RX, RN>(cur, fl, i, f, corr, g);
        tb_collide(a, g, rho, ux, uy);
#pragma unroll
        for (int k = 0; k < 9; k++) nxt[k * RN + i] = g[k];
    }
}

template <int RX, int RY, int NT, int TS, int S>
struct TbSteps {
    __device__ __forceinline__ static void run(const D2Args &a, float *b0, float *b1,
                                               const uint8_t *fl, const float *corr) {
        tb_inner_step<RX, RY, NT, S>(a, (S & 1) ? b0 : b1, (S & 1) ? b1 : b0, fl, corr);
        __syncthreads();
        TbSteps<RX, RY, NT, TS, S + 1>::run(a, b0, b1, fl, corr);
    }
};
template <int RX, int RY, int NT, int TS>
struct TbSteps<RX, RY, NT, TS, TS> {
    __device__ __forceinline__ static void run(const D2Args &, float *, float *, const uint8_t *,
                                               const float *) {}
};

}  // namespace

template <int TS, int BX, int BY, int NT>
constexpr size_t tblock_smem() {
    return (size_t)(BX + 2 * TS) * (BY + 2 * TS) * (2 * 9 * sizeof(float) + 1);
}

// TS steps of the native D2Q9 fused update, set src -> set dst.  Launched as
// a programmatic dependent of the previous launch (griddepcontrol.wait
// before the first load).
template <int TS, int BX, int BY, int NT, bool MOM>
__global__ void __launch_bounds__(NT) d2q9_tblock_kernel(const D2Args a) {
    constexpr int RX = BX + 2 * TS, RY = BY + 2 * TS, RN = RX * RY;
    extern __shared__ float4 tb_smem4[];
    float *b0 = reinterpret_cast<float *>(tb_smem4);
    float *b1 = b0 + 9 * RN;
    uint8_t *fl = reinterpret_cast<uint8_t *>(b1 + 9 * RN);
    __shared__ float corr[9];

    asm volatile("griddepcontrol.wait;" ::: "memory");
    asm volatile("griddepcontrol.launch_dependents;" ::: "memory");

    const int W = a.W, H = a.H;
    const int x0 = blockIdx.x * BX, y0 = blockIdx.y * BY;
    if (threadIdx.x < 9) corr[threadIdx.x] = a.corr[threadIdx.x];
    // region node (rx, ry) is lattice node (x0 - TS + rx, y0 - TS + ry),
    // wrapped: one conditional add or subtract when the lattice is at least a
    // tile and its halo wide and high (every coordinate then lies within one
    // period of the lattice), the remainder otherwise
    const bool one_wrap = W >= BX + TS && H >= BY + TS;
    for (int i = threadIdx.x; i < RN; i += NT) {
        int gx = x0 - TS + i % RX, gy = y0 - TS + i / RX;
        if (one_wrap) {
            gx = gx < 0 ? gx + W : (gx >= W ? gx - W : gx);
            gy = gy < 0 ? gy + H : (gy >= H ? gy - H : gy);
        } else {
            gx %= W;
            gy %= H;
            gx += gx < 0 ? W : 0;
            gy += gy < 0 ? H : 0;
        }
        const int o = gx + W * gy;
        fl[i] = a.flags[o];
#pragma unroll
        for (int k = 0; k < 9; k++) b0[k * RN + i] = ld_stream(a.src.f[k] + o);
    }
    __syncthreads();
    TbSteps<RX, RY, NT, TS, 1>::run(a, b0, b1, fl, corr);

    // step TS: the tile itself, from shared memory straight to set dst
    const float *cur = (TS & 1) ? b0 : b1;
    for (int j = threadIdx.x; j < BX * BY; j += NT) {
        const int tx = j % BX, ty = j / BX;
        const int gx = x0 + tx, gy = y0 + ty;
        if (gx >= W || gy >= H) continue;
        const int o = gx + W * gy;
        const int i = (TS + tx) + RX * (TS + ty);
        const uint8_t f = fl[i];
        if (f & CELL_WALL) {
            if (MOM) { a.ux[o] = 0.f; a.uy[o] = 0.f; a.rho[o] = 0.f; }
            if (a.probe && o == a.probe_o) *a.probe = make_float4(0.f, 0.f, 0.f, 0.f);
            continue;
        }
        float g[9], rho, ux, uy;
        tb_pull<RX, RN>(cur, fl, i, f, corr, g);
        tb_collide(a, g, rho, ux, uy);
        if (MOM) { a.ux[o] = ux; a.uy[o] = uy; a.rho[o] = rho; }
        if (a.probe && o == a.probe_o) *a.probe = make_float4(ux, uy, 0.f, rho);
#pragma unroll
        for (int k = 0; k < 9; k++) a.dst.f[k][o] = g[k];
    }
}

namespace {

template <int TS, int BX, int BY, int NT>
cudaError_t tb_launch(const D2Args &a, bool mom, cudaStream_t s) {
    constexpr size_t smem = tblock_smem<TS, BX, BY, NT>();
    static_assert(smem <= 227 * 1024, "temporal block region does not fit in shared memory");
    void (*kern)(const D2Args) = mom ? d2q9_tblock_kernel<TS, BX, BY, NT, true>
                                     : d2q9_tblock_kernel<TS, BX, BY, NT, false>;
    // once per instantiation
    static const cudaError_t attr_e[2] = {
        cudaFuncSetAttribute(d2q9_tblock_kernel<TS, BX, BY, NT, false>,
                             cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem),
        cudaFuncSetAttribute(d2q9_tblock_kernel<TS, BX, BY, NT, true>,
                             cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem)};
    if (attr_e[mom ? 1 : 0] != cudaSuccess) return attr_e[mom ? 1 : 0];
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3((a.W + BX - 1) / BX, (a.H + BY - 1) / BY);
    cfg.blockDim = dim3(NT);
    cfg.dynamicSmemBytes = smem;
    cfg.stream = s;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
    attr[0].val.programmaticStreamSerializationAllowed = 1;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    return cudaLaunchKernelEx(&cfg, kern, a);
}

}  // namespace

// block shapes by variant: (variant, steps per launch, tile x, tile y, threads)
#define LB_TBLOCK_SHAPES(X)     \
    X(1, 4, 32, 16, 960)        \
    X(2, 4, 32, 14, 896)        \
    X(3, 3, 32, 14, 768)        \
    X(4, 2, 32, 16, 736)        \
    X(5, 5, 32, 14, 1024)       \
    X(6, 4, 16, 16, 576)        \
    X(7, 3, 16, 16, 512)        \
    X(8, 8, 16, 16, 1024)       \
    X(9, 6, 16, 16, 800)        \
    X(10, 4, 16, 16, 256)

int tblock_steps(int variant) {
    switch (variant) {
#define LB_TB_STEPS(V, TS, BX, BY, NT) \
    case V: return TS;
        LB_TBLOCK_SHAPES(LB_TB_STEPS)
#undef LB_TB_STEPS
        default: return 0;
    }
}

cudaError_t launch_d2q9_tblock(const D2Args &a, int variant, bool mom, cudaStream_t s) {
    if (a.G != 0.f) return cudaErrorInvalidValue;  // no Shan-Chen here
    switch (variant) {
#define LB_TB_LAUNCH(V, TS, BX, BY, NT) \
    case V: return tb_launch<TS, BX, BY, NT>(a, mom, s);
        LB_TBLOCK_SHAPES(LB_TB_LAUNCH)
#undef LB_TB_LAUNCH
        default: return cudaErrorInvalidValue;
    }
}

}  // namespace lb
