// lb_sc_stage.cu -- single-pass D3Q19 Shan-Chen step for lattices without
// wall nodes (the periodic spinodal case), fed by asynchronous copies into
// shared memory.
//
// A block of 256 threads owns a 32 x 8 column tile and marches through a
// chunk of z planes.  The populations reach shared memory as "stages": stage
// z holds, for every population k, what the pulls of plane z read for the
// tile and the ring around it -- rows y0-1-c_y .. y0+8-c_y of plane z - c_z(k),
// columns x0-E .. x0+32+E-1 (E elements = 16 bytes on each side), one
// 128-byte-aligned box per population (31.6 KB per FP32 stage, 19.5 KB per
// 16-bit stage: 3 blocks fit per SM).
//
// Copies.  A block whose boxes all lie inside the lattice (not in the first
// or last column of tiles, nor the first or last row) gets each stage as 19
// TMA tensor copies (cp.async.bulk.tensor.4d over the populations' own
// arrays, one tensor map of dims (W, H, D, population)) issued by one thread
// and completed on the slot's mbarrier by transaction count: the other 255
// threads issue no copy instructions at all.  (The 19 boxes issued by one
// warp, a lane each, measured slower: 38.0 against 41.9 GLUPS.)  TMA does
// not wrap, so the edge blocks (periodic wrap in x or y) copy the same layout
// in 16-byte cp.async chunks instead (each warp instruction moves 512
// contiguous bytes; the wrap is folded into each thread's chunk addresses,
// formed once per block) and report on the mbarrier when their copies have
// landed.  Stages are issued two
// (FP32) or three (16-bit) steps ahead of their use, so DRAM latency is
// covered by copies in flight rather than by warps waiting on loads, and no
// global address is formed per population and node.
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
// device functions in the same order (StepArith<S>: the native FP32 forms or,
// in 16-bit storage, their deviation forms; d3q19_sc_sum_native), so the
// result is bit-identical to the density pass + fused step.
//
// Every mbarrier wait is bounded (wait_limit polls for a stage; ST_WAIT in the
// library's launches); a block that gives up raises
// the device error word, waits (bounded by ST_WAIT) for the stages it still
// has in flight, drains its threads' own copies (cp.async.wait_all) and
// returns.  sc_stage_wait_selftest makes the first wait run out (wait_limit
// 0) to exercise that path.  (A first form copied each stage row with one
// cp.async.bulk per population and row, 228 copies per stage: 20.9 GLUPS for
// FP32 and 16-bit alike at 256^3, bound by the number of copies, not their
// bytes.)
#include <cuda.h>
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

// Stage layouts.  Population k of a stage holds the 10 rows its pulls read for
// the tile and its ring (rows y0-1-c_y .. y0+8-c_y of plane z - c_z), row after
// row, over the columns they read:
//  * compact (U = false, the cp.async-only kernel): x0-1-c_x .. x0+32-c_x
//    rounded out to 16-byte chunks, 32 + 2E columns for c_x = 0 and 32 + E
//    otherwise, the populations packed one after another (28.8 KB per FP32
//    stage, 16.6 KB per 16-bit stage);
//  * uniform (U = true, the kernel with TMA copies): x0-E .. x0+32+E-1 for
//    every population, one box of (32 + 2E) x 10 elements padded to 128 bytes
//    (a TMA destination's alignment) per population (31.6 / 19.5 KB).
// Column c below counts from x0 - E in both.
template <typename S, bool U>
struct StageShape {
    static constexpr int E = 16 / (int)sizeof(S);      // elements per 16-byte chunk
    static constexpr int ROWS = ST_TY + 2;             // rows of every population
    static constexpr int BW = ST_TX + 2 * E;           // columns of a uniform box (40 / 48)
    static constexpr int BOX_BYTES = BW * ROWS * (int)sizeof(S);     // 1600 / 960
    static constexpr int POP_BYTES = (BOX_BYTES + 127) / 128 * 128;  // 1664 / 1024
    static constexpr int PAD = POP_BYTES - BOX_BYTES;                // 64 / 64
    // first column (relative to x0) and width of population k
    static constexpr int col0(int k) { return U ? -E : (d3_cx(k) < 0 ? 0 : -E); }
    static constexpr int width(int k) {
        return U ? BW : (d3_cx(k) == 0 ? ST_TX + 2 * E : ST_TX + E);
    }
    static constexpr int chunks(int k) { return ROWS * width(k) / E; }
    static constexpr int first_chunk(int k) {
        int c = 0;
        for (int j = 0; j < k; j++) c += chunks(j);
        return c;
    }
    static constexpr int first_byte(int k) { return U ? k * POP_BYTES : first_chunk(k) * 16; }
    static constexpr int CPP = U ? ROWS * BW / E : 0;    // chunks per population (uniform)
    static constexpr int CHUNKS = first_chunk(19);      // 1800 / 1040 compact, 1900 / 1140 uniform
    static constexpr int BYTES = U ? 19 * POP_BYTES : CHUNKS * 16;
    static constexpr int ELEMS = BYTES / (int)sizeof(S);
    static constexpr int SLOTS = sizeof(S) == 4 ? 2 : 3;
    static constexpr int MIN_BLOCKS = 3;                // resident blocks per SM
    static constexpr int PSI_BYTES = 4 * ST_PY * ST_PX * (int)sizeof(float);
    static constexpr int SMEM = SLOTS * BYTES + PSI_BYTES + SLOTS * 8;
    // element of population k, stage row r, column c (0 = x0 - E)
    static constexpr int elem(int k, int r, int c) {
        return first_byte(k) / (int)sizeof(S) + r * width(k) + c - E - col0(k);
    }
    // shared-memory byte of chunk c (chunks in population order)
    __device__ static constexpr int chunk_byte(int c) {
        return U ? 16 * c + PAD * (c / CPP) : 16 * c;
    }
    static_assert(BYTES % 128 == 0 && PSI_BYTES % 16 == 0, "stage alignment");
    static_assert((BW * (int)sizeof(S)) % 16 == 0, "a TMA box row is a multiple of 16 bytes");
};

// the stored value of population k as the step works on it (Store<S>::load_dev:
// f_k in FP32, the deviation d_k in 16-bit storage)
__device__ __forceinline__ float widen(float v) { return v; }
__device__ __forceinline__ float widen(__half v) { return __half2float(v); }
__device__ __forceinline__ float widen(__nv_bfloat16 v) { return __bfloat162float(v); }

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

// cp.async copies of a stage (the compact kernel's every block, the uniform
// kernel's edge blocks): chunk c is 16 bytes of population k (the last
// population whose first chunk is at most c), at shared byte chunk_byte(c) of
// the slot.  Thread t copies chunks t, t + 256, ...; which global row and
// column each of its chunks reads does not change from plane to plane, so the
// thread forms those offsets once: the element offset from population 0's
// array in plane 0 (the populations lie at f[0] + k * stride, and the launch
// guarantees 19 strides fit in 32 bits), with the chunk's z class -- plane
// z - c_z read for plane z -- in the two low bits, free because every chunk
// starts on a 16-byte boundary.
template <typename S, bool U>
struct StageCopy {
    using SS = StageShape<S, U>;
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
        char *dst = reinterpret_cast<char *>(slot);
#pragma unroll
        for (int i = 0; i < PER_T; i++) {
            const int c = (int)threadIdx.x + ST_THREADS * i;
            if (i == PER_T - 1 && c >= CHUNKS) break;
            const uint32_t e = off[i], cls = e & 3u;
            cp16(dst + SS::chunk_byte(c), base + (e + (cls == 0 ? o0 : (cls == 1 ? o1 : o2))));
        }
        cp_arrive(mbar);
    }
};

// mbarrier arrival that also announces `bytes` of asynchronous copies
__device__ __forceinline__ void mbar_expect_tx(uint64_t *mbar, uint32_t bytes) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;\n" ::"r"(
                     smem_u32(mbar)),
                 "r"(bytes)
                 : "memory");
}

// Interior blocks: one thread copies a stage as 19 tensor boxes (BW x ROWS x
// 1 x 1 of the map over (W, H, D, population)), completing on mbar by bytes.
// Coordinates: x0 - E is a multiple of 16 bytes (x0 of 32 elements, E of 16
// bytes) and every box lies inside the lattice.
template <typename S>
__device__ __forceinline__ void tma_issue(const CUtensorMap &tmap, S *slot, uint64_t *mbar,
                                          int x0, int y0, int zs, int D) {
    using SS = StageShape<S, true>;
    mbar_expect_tx(mbar, 19 * SS::BOX_BYTES);
    const uint64_t map = reinterpret_cast<uint64_t>(&tmap);
    const uint32_t bar = smem_u32(mbar);
    const uint32_t dst = smem_u32(slot);
#pragma unroll
    for (int k = 0; k < 19; k++) {
        const int yc = y0 - 1 - d3_cy(k), zc = wrap1(zs - d3_cz(k), D);
        asm volatile(
            "cp.async.bulk.tensor.4d.shared::cluster.global.mbarrier::complete_tx::bytes "
            "[%0], [%1, {%2, %3, %4, %5}], [%6];\n" ::"r"(dst + k * SS::POP_BYTES),
            "l"(map), "r"(x0 - SS::E), "r"(yc), "r"(zc), "r"(k), "r"(bar)
            : "memory");
    }
}

// the 19 post-stream populations of the ring node (rx, ry) relative to the
// tile origin (rx in -1..32, ry in -1..8): population k comes from row
// ry - c_y (local row ry + 1 of its rows) and column rx - c_x
template <typename S, bool U>
__device__ __forceinline__ void pull_stage(const S *st, int rx, int ry, float (&g)[19]) {
    using SS = StageShape<S, U>;
#pragma unroll
    for (int k = 0; k < 19; k++) g[k] = widen(st[SS::elem(k, ry + 1, rx - d3_cx(k) + SS::E)]);
}

// the pseudo-potential of the configured form (LB_PSI_REF = 0: the
// reference's 4 exp(-200/rho); LB_PSI_EXP1: 1 - exp(-rho)), a compile-time
// choice so that each kernel carries the code of one form only
template <int PSI>
__device__ __forceinline__ float psi_of(float rho) {
    return PSI == 0 ? psi_ref(rho) : psi_exp1(rho);
}

}  // namespace

template <typename S, bool MOM, int PSI, bool U>
__global__ void __launch_bounds__(ST_THREADS, (StageShape<S, U>::MIN_BLOCKS))
    d3q19_sc_stage_kernel(const __grid_constant__ D3Args a, const __grid_constant__ CUtensorMap tmap,
                          int use_tma, int zc, int wait_limit) {
    using SS = StageShape<S, U>;
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

    // TMA for a block whose boxes lie inside the lattice (and whose shared
    // memory has the 128-byte alignment the boxes need); cp.async chunks else
    const bool tma = U && use_tma && blockIdx.x > 0 && blockIdx.x + 1 < gridDim.x &&
                     blockIdx.y > 0 && blockIdx.y + 1 < gridDim.y && (smem_u32(smem) & 127u) == 0;
    if (tid == 0)
        for (int s = 0; s < SS::SLOTS; s++) mbar_init(&full[s], tma ? 1 : ST_THREADS);
    __syncthreads();
    const StageCopy<S, U> cp(a, x0, y0);
    const int nst = zc + 2;  // stages z0 - 1 .. z0 + zc
    auto issue = [&](int slot, int zs) {
        if (!tma) cp.issue(a, stage + slot * SS::ELEMS, &full[slot], zs);
        else if (tid == 0) tma_issue<S>(tmap, stage + slot * SS::ELEMS, &full[slot], x0, y0, zs, a.D);
    };
    for (int j = 0; j < SS::SLOTS && j < nst; j++) issue(j, z0 - 1 + j);

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
            pull_stage<S, U>(st, tx, ty, gn);
            ps[ty + 1][tx + 1] = psi_of<PSI>(StepArith<S>::rho(gn, a));
            if (tid < ST_HALO) {
                float gh[19];
                pull_stage<S, U>(st, hx, hy, gh);
                ps[hy + 1][hx + 1] = psi_of<PSI>(StepArith<S>::rho(gh, a));
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
        if (j + SS::SLOTS < nst) {
            // the barrier above ordered every thread's reads of this slot
            // before the copy that overwrites it; the tensor copies write
            // through the async proxy
            if (tma && tid == 0) fence_proxy_async();
            issue(slot, zs + SS::SLOTS);
        }
        if (j >= 2) {
            const int z = zs - 1;
            const int o = x + a.W * (y + a.H * z);
            float rho, ux, uy, uz;
            StepArith<S>::moments(gs, a, rho, ux, uy, uz);
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
            StepArith<S>::bgk(gs, ex, ey, ez, rho, a, a.tau_inv);
            S *const *dst = reinterpret_cast<S *const *>(a.dst.f);
#pragma unroll
            for (int k = 0; k < 19; k++) Store<S>::store_dev(dst[k] + o, gs[k]);
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

template <typename S, bool MOM, int PSI, bool U>
cudaError_t stage_launch(const D3Args &a, const CUtensorMap *tmap, int zc, cudaStream_t s) {
    using SS = StageShape<S, U>;
    static_assert(SS::MIN_BLOCKS * (SS::SMEM + 1024) <= 228 * 1024, "resident blocks per SM");
    // once per instantiation
    static const cudaError_t attr_e =
        cudaFuncSetAttribute(d3q19_sc_stage_kernel<S, MOM, PSI, U>,
                             cudaFuncAttributeMaxDynamicSharedMemorySize, SS::SMEM);
    if (attr_e != cudaSuccess) return attr_e;
    const dim3 g(a.W / ST_TX, a.H / ST_TY, a.D / zc);
    CUtensorMap none{};
    d3q19_sc_stage_kernel<S, MOM, PSI, U><<<g, ST_THREADS, SS::SMEM, s>>>(
        a, tmap ? *tmap : none, tmap ? 1 : 0, zc, ST_WAIT);
    return cudaGetLastError();
}

// with a tensor map: the uniform layout, TMA copies for the interior tiles;
// without: the compact layout, every stage by cp.async.  FP32 steps always
// take the compact layout (the context builds tensor maps for 16-bit storage
// only), so its uniform form is not instantiated.
template <typename S, bool MOM, int PSI>
cudaError_t stage_launch(const D3Args &a, const CUtensorMap *tmap, int zc, cudaStream_t s) {
    if constexpr (sizeof(S) == 2) {
        if (tmap) return stage_launch<S, MOM, PSI, true>(a, tmap, zc, s);
    } else if (tmap) {
        return cudaErrorInvalidValue;
    }
    return stage_launch<S, MOM, PSI, false>(a, nullptr, zc, s);
}

template <typename S>
cudaError_t stage_launch(const D3Args &a, const CUtensorMap *tmap, bool mom, int zc,
                         cudaStream_t s) {
    if (a.psi_form == 0)
        return mom ? stage_launch<S, true, 0>(a, tmap, zc, s)
                   : stage_launch<S, false, 0>(a, tmap, zc, s);
    return mom ? stage_launch<S, true, 1>(a, tmap, zc, s)
               : stage_launch<S, false, 1>(a, tmap, zc, s);
}

using EncodeTiled = CUresult (*)(CUtensorMap *, CUtensorMapDataType, cuuint32_t, void *,
                                 const cuuint64_t *, const cuuint64_t *, const cuuint32_t *,
                                 const cuuint32_t *, CUtensorMapInterleave, CUtensorMapSwizzle,
                                 CUtensorMapL2promotion, CUtensorMapFloatOOBfill);

// the driver's cuTensorMapEncodeTiled, looked up once through the runtime
EncodeTiled encode_tiled() {
    static EncodeTiled fn = [] {
        void *p = nullptr;
        cudaDriverEntryPointQueryResult q{};
        if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000,
                                             cudaEnableDefault, &q) != cudaSuccess ||
            q != cudaDriverEntryPointSuccess)
            p = nullptr;
        return reinterpret_cast<EncodeTiled>(p);
    }();
    return fn;
}

}  // namespace

// The tensor map of the populations a step reads (a.src): dims (W, H, D, 19)
// over population 0's array with the populations' stride as the fourth, box
// (32 + 2E) x 10 x 1 x 1 with E = 8 halo columns per side.  16-bit storage
// only; false for FP32 or when the driver cannot encode it (the step then
// copies every stage with cp.async).
bool sc_stage_tensor_map(const D3Args &a, int storage, CUtensorMap *out) {
    const EncodeTiled enc = encode_tiled();
    if (!enc || (storage != 1 && storage != 2) || !sc_stage_chunk(a.W, a.H, a.D)) return false;
    const int es = 2;
    const long stride = (reinterpret_cast<const char *>(a.src.f[1]) -
                         reinterpret_cast<const char *>(a.src.f[0]));
    const int bw = ST_TX + 2 * (16 / es);
    const cuuint64_t dims[4] = {(cuuint64_t)a.W, (cuuint64_t)a.H, (cuuint64_t)a.D, 19};
    const cuuint64_t strides[3] = {(cuuint64_t)a.W * es, (cuuint64_t)a.W * a.H * es,
                                   (cuuint64_t)stride};
    const cuuint32_t box[4] = {(cuuint32_t)bw, ST_TY + 2, 1, 1};
    const cuuint32_t estr[4] = {1, 1, 1, 1};
    if (stride <= 0 || stride % 16) return false;
    const CUtensorMapDataType dt =
        storage == 1 ? CU_TENSOR_MAP_DATA_TYPE_FLOAT16 : CU_TENSOR_MAP_DATA_TYPE_BFLOAT16;
    return enc(out, dt, 4, const_cast<float *>(a.src.f[0]), dims, strides, box, estr,
               CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE,
               CU_TENSOR_MAP_L2_PROMOTION_L2_256B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) ==
           CUDA_SUCCESS;
}

// The give-up path of the staged step on a 32 x 8 x 4 FP32 lattice: every
// first stage wait is given no polls, so each block reports through *err,
// waits for the stages its prologue issued and returns.
cudaError_t sc_stage_wait_selftest(int *err) {
    constexpr int W = ST_TX, H = ST_TY, D = 4, N = W * H * D;
    using SS = StageShape<float, false>;
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
        d3q19_sc_stage_kernel<float, false, 1, false>, cudaFuncAttributeMaxDynamicSharedMemorySize,
        SS::SMEM);
    if (e == cudaSuccess) e = attr_e;
    if (e == cudaSuccess) {
        CUtensorMap none{};
        d3q19_sc_stage_kernel<float, false, 1, false><<<dim3(1, 1, 1), ST_THREADS, SS::SMEM>>>(
            a, none, 0, D, 0);
        e = cudaGetLastError();
    }
    if (e == cudaSuccess) e = cudaDeviceSynchronize();
    cudaFree(buf);
    return e;
}

cudaError_t launch_d3q19_sc_stage(const D3Args &a, int storage, bool mom,
                                  const CUtensorMap *tmap, cudaStream_t s) {
    const int zc = sc_stage_chunk(a.W, a.H, a.D);
    if (!zc) return cudaErrorInvalidValue;
    switch (storage) {
    case 0: return stage_launch<float>(a, tmap, mom, zc, s);
    case 1: return stage_launch<__half>(a, tmap, mom, zc, s);
    case 2: return stage_launch<__nv_bfloat16>(a, tmap, mom, zc, s);
    }
    return cudaErrorInvalidValue;
}

}  // namespace lb
