// lb_sc_stage.cu -- single-pass D3Q19 Shan-Chen step for lattices without
// wall nodes (the periodic spinodal case), fed by asynchronous copies into
// shared memory.
//
// A block of 256 threads owns a 32 x 8 column tile and marches through a
// chunk of z planes.  The populations reach shared memory as "stages": stage
// z holds, for every population k, exactly what the pulls of plane z read for
// the tile and the ring around it -- rows y0-1-c_y .. y0+8-c_y of plane
// z - c_z(k), columns x0-1-c_x .. x0+32-c_x rounded out to 16-byte chunks
// (28.8 KB per FP32 stage, 16.6 KB per 16-bit stage: 3 blocks fit per SM).
// The threads copy a stage in 16-byte cp.async chunks (each warp instruction
// moves 512 contiguous bytes; periodic wrap is folded into each thread's chunk
// addresses, formed once per block) and report on the slot's mbarrier when
// their copies have landed.  Stages are issued two (FP32) or three (16-bit)
// steps ahead of their use, so DRAM latency is covered by copies in flight
// rather than by warps waiting on loads, and no global address is formed per
// population and node.
//
// Step j of the march takes stage z = z0 - 1 + j: every thread pulls its own
// node from it (kept in registers for the relaxation one step later) and the
// first 84 threads also pull one node of the ring around the tile; each forms
// psi(rho) into a four-plane psi buffer.  One barrier later the slot is
// refilled with the stage SLOTS planes ahead and plane z - 1 is relaxed from
// the kept populations and the psi stencil of planes z - 2 .. z.  Four psi
// slots make that one barrier per plane enough (a warp writing psi of plane
// z + 1 has passed the barrier of plane z, reached only after every warp
// relaxed plane z - 2, the last reader of that slot).
//
// Arithmetic: the pulls read the same stored values as the two-pass step,
// widened the same way; rho, the stencil sum and the relaxation are the same
// device functions in the same order (d3q19_rho_native, d3q19_moments_native,
// d3q19_sc_sum_native, d3q19_bgk_native), so the result is bit-identical to
// the density pass + fused step.
//
// Every mbarrier wait is bounded (wait_limit polls of about a microsecond for
// a stage; ST_WAIT in the library's launches); a block that gives up raises
// the device error word, waits (bounded by ST_WAIT) for the stages it still
// has in flight, drains its threads' own copies (cp.async.wait_all) and
// returns.  sc_stage_wait_selftest makes the first wait run
// out (wait_limit 0) to exercise that path.  (A first form copied each stage row with one cp.async.bulk per
// population and row, 228 copies per stage: 20.9 GLUPS for FP32 and 16-bit
// alike at 256^3, bound by the number of copies, not their bytes.)
#include <cuda_bf16.h>
#include <cuda_fp16.h>

#include "lb_d3q19.cuh"
#include "lb_tc05.cuh"

namespace lb {

namespace {

constexpr int ST_TX = 32, ST_TY = 8;
constexpr int ST_THREADS = ST_TX * ST_TY;             // 256
constexpr int ST_PX = ST_TX + 2, ST_PY = ST_TY + 2;   // psi region: tile + ring
constexpr int ST_HALO = ST_PX * ST_PY - ST_THREADS;   // 84 ring nodes
constexpr int ST_WAIT = 1 << 22;                      // mbarrier polls before giving up

// Stage layout.  Population k of a stage holds the 10 rows its pulls read for
// the tile and its ring (rows y0-1-c_y .. y0+8-c_y of plane z - c_z) over the
// columns they read (x0-1-c_x .. x0+32-c_x) rounded out to whole 16-byte
// chunks: 32 + 2E columns for c_x = 0, 32 + E otherwise (E elements per
// chunk).  The populations follow one another, row by row.
template <typename S>
struct StageShape {
    static constexpr int E = 16 / (int)sizeof(S);      // elements per 16-byte chunk
    static constexpr int ROWS = ST_TY + 2;             // rows of every population
    // first column relative to x0, and width, of population k
    static constexpr int col0(int k) { return d3_cx(k) < 0 ? 0 : -E; }
    static constexpr int width(int k) { return d3_cx(k) == 0 ? ST_TX + 2 * E : ST_TX + E; }
    static constexpr int chunks(int k) { return ROWS * width(k) / E; }
    static constexpr int first_chunk(int k) {
        int c = 0;
        for (int j = 0; j < k; j++) c += chunks(j);
        return c;
    }
    static constexpr int CHUNKS = first_chunk(19);       // 1800 (FP32) / 1040 (16-bit)
    static constexpr int ELEMS = CHUNKS * E;
    static constexpr int BYTES = CHUNKS * 16;            // 28 800 / 16 640
    static constexpr int SLOTS = sizeof(S) == 4 ? 2 : 3;
    static constexpr int MIN_BLOCKS = 3;                  // resident blocks per SM
    static constexpr int PSI_BYTES = 4 * ST_PY * ST_PX * (int)sizeof(float);
    static constexpr int SMEM = SLOTS * BYTES + PSI_BYTES + SLOTS * 8;
    static_assert(BYTES % 128 == 0 && PSI_BYTES % 16 == 0, "stage alignment");
};

// the stored value of population k, widened as Store<S>::load does
__device__ __forceinline__ float widen(float v, float) { return v; }
__device__ __forceinline__ float widen(__half v, float wr) { return wr + __half2float(v); }
__device__ __forceinline__ float widen(__nv_bfloat16 v, float wr) {
    return wr + __bfloat162float(v);
}

// v in [-n, 2n): its periodic image in [0, n)
__device__ __forceinline__ int wrap1(int v, int n) { return v < 0 ? v + n : (v >= n ? v - n : v); }

// 16 bytes from global memory into shared memory (L2 only), asynchronously
__device__ __forceinline__ void cp16(void *dst, const void *src) {
    asm volatile("cp.async.cg.shared.global [%0], [%1], 16;\n" ::"r"(smem_u32(dst)), "l"(src)
                 : "memory");
}
// one arrival on mbar once every cp.async this thread issued so far has landed
__device__ __forceinline__ void cp_arrive(uint64_t *mbar) {
    asm volatile("cp.async.mbarrier.arrive.noinc.shared::cta.b64 [%0];\n" ::"r"(smem_u32(mbar))
                 : "memory");
}

// populations with c_z (c_y) = +1 / -1 as bit masks over k
constexpr unsigned cz_mask(int sign) {
    unsigned m = 0;
    for (int k = 0; k < 19; k++) m |= (d3_cz(k) == sign ? 1u : 0u) << k;
    return m;
}
constexpr unsigned kCzPos = cz_mask(1), kCzNeg = cz_mask(-1);
static_assert(kCzPos == 0x2A220u && kCzNeg == 0x54440u, "D3Q19 z classes");
constexpr unsigned cy_mask(int sign) {
    unsigned m = 0;
    for (int k = 0; k < 19; k++) m |= (d3_cy(k) == sign ? 1u : 0u) << k;
    return m;
}
constexpr unsigned kCyPos = cy_mask(1), kCyNeg = cy_mask(-1);

// A stage is copied in 16-byte chunks: chunk c of a slot is bytes 16c .. 16c+15,
// element (k, row, col) of the stage layout.  Thread t copies chunks t, t + 256,
// ...; which global row and column each of its chunks reads does not change
// from plane to plane, so the thread forms those offsets once: the element
// offset from population 0's array in plane 0 (the populations lie at
// f[0] + k * stride, and the launch guarantees 19 strides fit in 32 bits),
// with the chunk's z class -- plane z - c_z read for plane z -- in the two low
// bits, free because every chunk starts on a 16-byte boundary.
template <typename S>
struct StageCopy {
    using SS = StageShape<S>;
    static constexpr int E = SS::E;
    static constexpr int CHUNKS = SS::CHUNKS;
    static constexpr int PER_T = (CHUNKS + ST_THREADS - 1) / ST_THREADS;  // 8 / 5
    uint32_t off[PER_T];

    __device__ __forceinline__ StageCopy(const D3Args &a, int x0, int y0) {
        const long stride = (reinterpret_cast<const char *>(a.src.f[1]) -
                             reinterpret_cast<const char *>(a.src.f[0])) / (long)sizeof(S);
#pragma unroll
        for (int i = 0; i < PER_T; i++) {
            const int c = min((int)threadIdx.x + ST_THREADS * i, CHUNKS - 1);
            // population k of chunk c, its first chunk, chunks per row, first column
            int k = 0, c0 = 0, cpr = SS::width(0) / E, x_0 = SS::col0(0);
#pragma unroll
            for (int j = 1; j < 19; j++)
                if (c >= SS::first_chunk(j)) {
                    k = j;
                    c0 = SS::first_chunk(j);
                    cpr = SS::width(j) / E;
                    x_0 = SS::col0(j);
                }
            const int r = (c - c0) / cpr, q = c - c0 - r * cpr;
            const int cy = (kCyPos >> k & 1) ? 1 : ((kCyNeg >> k & 1) ? -1 : 0);
            const int cls = (kCzPos >> k & 1) ? 0 : ((kCzNeg >> k & 1) ? 2 : 1);  // c_z +1, 0, -1
            const int yr = wrap1(y0 - 1 - cy + r, a.H);
            const int xm = wrap1(x0 + x_0 + q * E, a.W);
            off[i] = (uint32_t)(k * stride + (long)yr * a.W + xm) | (uint32_t)cls;
        }
    }

    // stage of plane zs into slot; one arrival per thread on mbar
    __device__ __forceinline__ void issue(const D3Args &a, S *slot, uint64_t *mbar, int zs) const {
        const S *base = reinterpret_cast<const S *>(a.src.f[0]);
        const uint32_t plane = (uint32_t)a.W * (uint32_t)a.H;
        // element offset of the plane read by each z class, minus the class tag
        const uint32_t o0 = (uint32_t)wrap1(zs - 1, a.D) * plane,
                       o1 = (uint32_t)wrap1(zs, a.D) * plane - 1u,
                       o2 = (uint32_t)wrap1(zs + 1, a.D) * plane - 2u;
        char *dst = reinterpret_cast<char *>(slot) + 16 * threadIdx.x;
#pragma unroll
        for (int i = 0; i < PER_T; i++) {
            if (i == PER_T - 1 && (int)threadIdx.x + ST_THREADS * i >= CHUNKS) break;
            const uint32_t e = off[i], cls = e & 3u;
            cp16(dst + 16 * ST_THREADS * i, base + (e + (cls == 0 ? o0 : (cls == 1 ? o1 : o2))));
        }
        cp_arrive(mbar);
    }
};

// the 19 post-stream populations of the ring node (rx, ry) relative to the
// tile origin (rx in -1..32, ry in -1..8): population k comes from row
// ry - c_y (local row ry + 1 of its rows) and column rx - c_x
template <typename S>
__device__ __forceinline__ void pull_stage(const S *st, int rx, int ry, const float *wr,
                                           float (&g)[19]) {
    using SS = StageShape<S>;
#pragma unroll
    for (int k = 0; k < 19; k++)
        g[k] = widen(st[SS::first_chunk(k) * SS::E + (ry + 1) * SS::width(k) + rx - d3_cx(k) -
                        SS::col0(k)],
                     wr[k]);
}

// the pseudo-potential of the configured form (LB_PSI_REF = 0: the
// reference's 4 exp(-200/rho); LB_PSI_EXP1: 1 - exp(-rho)), a compile-time
// choice so that each kernel carries the code of one form only
template <int PSI>
__device__ __forceinline__ float psi_of(float rho) {
    return PSI == 0 ? psi_ref(rho) : psi_exp1(rho);
}

}  // namespace

template <typename S, bool MOM, int PSI>
__global__ void __launch_bounds__(ST_THREADS, StageShape<S>::MIN_BLOCKS)
    d3q19_sc_stage_kernel(const __grid_constant__ D3Args a, int zc, int wait_limit) {
    using SS = StageShape<S>;
    extern __shared__ __align__(128) unsigned char smem[];
    S *stage = reinterpret_cast<S *>(smem);
    float(*sp)[ST_PY][ST_PX] = reinterpret_cast<float(*)[ST_PY][ST_PX]>(smem + SS::SLOTS * SS::BYTES);
    uint64_t *full = reinterpret_cast<uint64_t *>(smem + SS::SLOTS * SS::BYTES + SS::PSI_BYTES);

    const int tid = threadIdx.x, tx = tid % ST_TX, ty = tid / ST_TX;
    const int x0 = blockIdx.x * ST_TX, y0 = blockIdx.y * ST_TY, z0 = blockIdx.z * zc;
    const int x = x0 + tx, y = y0 + ty;
    // the ring node this thread also handles (tid < 84), relative to the tile:
    // the two rows of 34, then the two side columns of 8
    int hx = 0, hy = 0;
    if (tid < 2 * ST_PX) {
        hx = tid % ST_PX - 1;
        hy = tid < ST_PX ? -1 : ST_TY;
    } else if (tid < ST_HALO) {
        hx = (tid - 2 * ST_PX) < ST_TY ? -1 : ST_TX;
        hy = (tid - 2 * ST_PX) % ST_TY;
    }

    if (tid == 0)
        for (int s = 0; s < SS::SLOTS; s++) mbar_init(&full[s], ST_THREADS);
    __syncthreads();
    const StageCopy<S> cp(a, x0, y0);
    const int nst = zc + 2;  // stages z0 - 1 .. z0 + zc
    for (int j = 0; j < SS::SLOTS && j < nst; j++)
        cp.issue(a, stage + j * SS::ELEMS, &full[j], z0 - 1 + j);

    // step j: psi of plane z0 - 1 + j from its stage (the own node's populations
    // into gn), then the relaxation of the plane before it from gs, pulled one
    // step earlier; false when the block gave up waiting for its copies
    auto step = [&](int j, float(&gs)[19], float(&gn)[19]) -> bool {
        const int slot = j % SS::SLOTS;
        const int zs = z0 - 1 + j;
        const S *st = stage + slot * SS::ELEMS;
        const bool ok = mbar_wait(&full[slot], (uint32_t)((j / SS::SLOTS) & 1), wait_limit);
        float(*ps)[ST_PX] = sp[(zs + 4) & 3];
        if (ok) {
            pull_stage<S>(st, tx, ty, a.wr, gn);
            ps[ty + 1][tx + 1] = psi_of<PSI>(d3q19_rho_native(gn));
            if (tid < ST_HALO) {
                float gh[19];
                pull_stage<S>(st, hx, hy, a.wr, gh);
                ps[hy + 1][hx + 1] = psi_of<PSI>(d3q19_rho_native(gh));
            }
        }
        if (__syncthreads_or(!ok)) {
            // give up: report, then wait (bounded) for the stages still in flight
            if (tid == 0 && a.err) atomicExch(a.err, 1);
            for (int i = j; i < j + SS::SLOTS && i < nst; i++)
                mbar_wait(&full[i % SS::SLOTS], (uint32_t)((i / SS::SLOTS) & 1), ST_WAIT);
            // then drain this thread's own copies whatever those waits saw, so
            // that none can land in shared memory that the next block resident
            // on this SM reuses (memory copies always complete; no other party
            // has to act for this wait to end)
            asm volatile("cp.async.wait_all;\n" ::: "memory");
            return false;
        }
        if (j + SS::SLOTS < nst) cp.issue(a, stage + slot * SS::ELEMS, &full[slot], zs + SS::SLOTS);
        if (j >= 2) {
            const int z = zs - 1;
            const int o = x + a.W * (y + a.H * z);
            float rho, ux, uy, uz;
            d3q19_moments_native(gs, rho, ux, uy, uz);
            if (MOM) { a.ux[o] = ux; a.uy[o] = uy; a.uz[o] = uz; a.rho[o] = rho; }
            if (a.probe && o == a.probe_o) *a.probe = make_float4(ux, uy, uz, rho);
            const float inv_rt = 1.f / (rho * a.tau_inv);
            float ex = ux, ey = uy, ez = uz;
            if (a.Fx != 0.f) ex = __fmaf_rn(a.Fx, inv_rt, ux);
            if (a.Fy != 0.f) ey = __fmaf_rn(a.Fy, inv_rt, uy);
            if (a.Fz != 0.f) ez = __fmaf_rn(a.Fz, inv_rt, uz);
            float pz[19];
#pragma unroll
            for (int k = 0; k < 19; k++)
                pz[k] = sp[(z + d3_cz(k) + 4) & 3][ty + 1 + d3_cy(k)][tx + 1 + d3_cx(k)];
            float IFx, IFy, IFz;
            d3q19_sc_sum_native(pz, a.w1, a.w7, IFx, IFy, IFz);
            const float c = (-a.G * pz[0]) * inv_rt;
            ex = __fmaf_rn(c, IFx, ex);
            ey = __fmaf_rn(c, IFy, ey);
            ez = __fmaf_rn(c, IFz, ez);
            d3q19_bgk_native(gs, ex, ey, ez, rho, a.w0, a.w1, a.w7, a.tau_inv);
            S *const *dst = reinterpret_cast<S *const *>(a.dst.f);
#pragma unroll
            for (int k = 0; k < 19; k++) Store<S>::store(dst[k] + o, gs[k], a.wr[k]);
        }
        return true;
    };
    // two steps per iteration with the population arrays swapped, so that no
    // step copies the pulled populations from one array to the other
    float ga[19], gb[19];
#pragma unroll
    for (int k = 0; k < 19; k++) ga[k] = gb[k] = 0.f;
    int j = 0;
    for (; j + 1 < nst; j += 2) {
        if (!step(j, ga, gb)) return;
        if (!step(j + 1, gb, ga)) return;
    }
    if (j < nst && !step(j, ga, gb)) return;
    // every wait has completed and no copy is in flight
    if (tid == 0)
        for (int s = 0; s < SS::SLOTS; s++) mbar_inval(&full[s]);
}

// z-chunk of the staged kernel, 0 if the lattice does not tile: the longest
// march that still gives at least 1216 blocks (eight per SM on 152 SMs, about
// three waves of 3 resident blocks), else the shortest that divides D.  At
// 256^3 that is 32 planes (2048 blocks); 16 planes measured slower (more
// halo planes per plane).
int sc_stage_chunk(int W, int H, int D) {
    if (W % ST_TX || H % ST_TY) return 0;
    int pick = 0;
    for (int zc : {32, 16, 8, 4}) {
        if (D % zc) continue;
        pick = zc;
        if ((long)(W / ST_TX) * (H / ST_TY) * (D / zc) >= 1216) return zc;
    }
    return pick;
}

namespace {

template <typename S, bool MOM, int PSI>
cudaError_t stage_launch(const D3Args &a, int zc, cudaStream_t s) {
    using SS = StageShape<S>;
    static_assert(SS::MIN_BLOCKS * (SS::SMEM + 1024) <= 228 * 1024, "resident blocks per SM");
    // once per instantiation
    static const cudaError_t attr_e = cudaFuncSetAttribute(
        d3q19_sc_stage_kernel<S, MOM, PSI>, cudaFuncAttributeMaxDynamicSharedMemorySize, SS::SMEM);
    if (attr_e != cudaSuccess) return attr_e;
    const dim3 g(a.W / ST_TX, a.H / ST_TY, a.D / zc);
    d3q19_sc_stage_kernel<S, MOM, PSI><<<g, ST_THREADS, SS::SMEM, s>>>(a, zc, ST_WAIT);
    return cudaGetLastError();
}

template <typename S>
cudaError_t stage_launch(const D3Args &a, bool mom, int zc, cudaStream_t s) {
    if (a.psi_form == 0)
        return mom ? stage_launch<S, true, 0>(a, zc, s) : stage_launch<S, false, 0>(a, zc, s);
    return mom ? stage_launch<S, true, 1>(a, zc, s) : stage_launch<S, false, 1>(a, zc, s);
}

}  // namespace

// The give-up path of the staged step on a 32 x 8 x 4 FP32 lattice: every
// first stage wait is given no polls, so each block reports through *err,
// waits for the stages its prologue issued and returns.
cudaError_t sc_stage_wait_selftest(int *err) {
    constexpr int W = ST_TX, H = ST_TY, D = 4, N = W * H * D;
    using SS = StageShape<float>;
    float *buf = nullptr;
    cudaError_t e = cudaMalloc(&buf, sizeof(float) * 2 * 19 * N);
    if (e != cudaSuccess) return e;
    e = cudaMemset(buf, 0, sizeof(float) * 2 * 19 * N);
    D3Args a{};
    for (int k = 0; k < 19; k++) {
        a.src.f[k] = buf + (long)k * N;
        a.dst.f[k] = buf + (long)(19 + k) * N;
    }
    a.W = W; a.H = H; a.D = D; a.ndev = 1;
    a.tau_inv = 1.f; a.G = -5.f; a.psi_form = 1;
    a.err = err;
    static const cudaError_t attr_e = cudaFuncSetAttribute(
        d3q19_sc_stage_kernel<float, false, 1>, cudaFuncAttributeMaxDynamicSharedMemorySize,
        SS::SMEM);
    if (e == cudaSuccess) e = attr_e;
    if (e == cudaSuccess) {
        d3q19_sc_stage_kernel<float, false, 1><<<dim3(1, 1, 1), ST_THREADS, SS::SMEM>>>(a, D, 0);
        e = cudaGetLastError();
    }
    if (e == cudaSuccess) e = cudaDeviceSynchronize();
    cudaFree(buf);
    return e;
}

cudaError_t launch_d3q19_sc_stage(const D3Args &a, int storage, bool mom, cudaStream_t s) {
    const int zc = sc_stage_chunk(a.W, a.H, a.D);
    if (!zc) return cudaErrorInvalidValue;
    switch (storage) {
    case 0: return stage_launch<float>(a, mom, zc, s);
    case 1: return stage_launch<__half>(a, mom, zc, s);
    case 2: return stage_launch<__nv_bfloat16>(a, mom, zc, s);
    }
    return cudaErrorInvalidValue;
}

}  // namespace lb
