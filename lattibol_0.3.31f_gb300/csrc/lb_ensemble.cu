// lb_ensemble.cu -- many independent periodic D2Q9 Shan-Chen domains of
// different sizes advanced together (include/lbgb300.h, ensemble API).
//
// All domains live in one packed structure-of-arrays slab (domain d occupies
// nodes [off_d, off_d + W_d*H_d), node x + W_d*y inside it), in two
// population sets that alternate like the single-lattice context.  A step is
// two persistent launches over a host-built work list of row groups (a
// domain's extents and physics and a first row): the density pass writes psi = psi(rho) of every node,
// the fused pass pulls the populations, adds the Shan-Chen shift from the
// 3x3 psi stencil and relaxes.  Each block walks the work list with a stride
// of the grid size, and the grid is a multiple of the SM count, so uneven
// domain sizes do not leave SMs idle.  Batches of steps are replayed from a
// captured CUDA graph.  The launch shape (threads along x, rows per item,
// blocks per SM) is chosen by lb_ensemble_autotune, which times each
// candidate on the ensemble itself.
//
// The per-node arithmetic is the single-domain native D2Q9 Shan-Chen step's
// (same device functions, same order: d2q9_moments_native,
// d2q9_sc_shift_native, d2q9_bgk_native), so a domain of the ensemble evolves
// bit for bit like the same domain run alone through the context API.
#include <algorithm>
#include <cstring>
#include <string>
#include <vector>

#include "../../include/lbgb300.h"
#include "lb_kernels.cuh"

using namespace lb;

namespace {

struct EnsDomain {
    int W, H, off;
    float G, tau_inv;
};

// one work item: a group of rows of one domain, with the domain's extents
// and physics copied in, so that a block needs one load (not two dependent
// ones) before it can address its populations
struct EnsItem {
    int off, W, H, y;
    float G, tau_inv;
    int x;  // single-pass tiles: first column of the tile (0 for row groups)
};

struct EnsArgs {
    const float *src[9];
    float *dst[9];
    float *psi;
    float *rho, *ux, *uy;
    const EnsItem *items;
    int nitems;
    int psi_form;
    float w0, w1, w5;
};

// pull of node (x, y) of a periodic domain starting at node `off`
__device__ __forceinline__ void ens_pull(const EnsArgs &a, const EnsItem &dm, int x, int y,
                                         float (&g)[9]) {
    const int xm = x == 0 ? dm.W - 1 : x - 1, xp = x == dm.W - 1 ? 0 : x + 1;
    const int rm = y == 0 ? dm.H - 1 : y - 1, rp = y == dm.H - 1 ? 0 : y + 1;
#pragma unroll
    for (int k = 0; k < 9; k++) {
        // upstream node x - c_k (row offset -cr_k)
        const int ux = d2_cx(k) > 0 ? xm : (d2_cx(k) < 0 ? xp : x);
        const int uy = d2_cr(k) > 0 ? rm : (d2_cr(k) < 0 ? rp : y);
        g[k] = __ldg(a.src[k] + dm.off + ux + dm.W * uy);
    }
}

// Both passes walk the work list with a stride of the grid size and load the
// next item while they work on the current one.
__global__ void ens_density_kernel(const EnsArgs a) {
    int it = blockIdx.x;
    if (it >= a.nitems) return;
    EnsItem dm = a.items[it];
    for (; it < a.nitems; it += gridDim.x) {
        const int nit = it + gridDim.x;
        const EnsItem next = nit < a.nitems ? a.items[nit] : dm;
        const int y = dm.y + threadIdx.y;
        if (y < dm.H) {
            for (int x = threadIdx.x; x < dm.W; x += blockDim.x) {
                float g[9];
                ens_pull(a, dm, x, y, g);
                const float rho = d2q9_rho_native(g);
                a.psi[dm.off + x + dm.W * y] = a.psi_form == 0 ? psi_ref(rho) : psi_exp1(rho);
            }
        }
        dm = next;
    }
}

template <bool MOM>
__global__ void ens_fused_kernel(const EnsArgs a) {
    int it = blockIdx.x;
    if (it >= a.nitems) return;
    EnsItem next = a.items[it];
    for (; it < a.nitems; it += gridDim.x) {
        const EnsItem dm = next;
        const int nit = it + gridDim.x;
        if (nit < a.nitems) next = a.items[nit];
        const int y = dm.y + threadIdx.y;
        if (y >= dm.H) continue;
        const int rm = y == 0 ? dm.H - 1 : y - 1, rp = y == dm.H - 1 ? 0 : y + 1;
        const float *psi = a.psi + dm.off;
        for (int x = threadIdx.x; x < dm.W; x += blockDim.x) {
            float g[9];
            ens_pull(a, dm, x, y, g);
            float rho, ux, uy;
            d2q9_moments_native(g, rho, ux, uy);
            const int xm = x == 0 ? dm.W - 1 : x - 1, xp = x == dm.W - 1 ? 0 : x + 1;
            const int W = dm.W;
            const float ps[9] = {__ldg(psi + x + W * y),   __ldg(psi + xp + W * y),
                                 __ldg(psi + x + W * rp),  __ldg(psi + xm + W * y),
                                 __ldg(psi + x + W * rm),  __ldg(psi + xp + W * rp),
                                 __ldg(psi + xm + W * rp), __ldg(psi + xm + W * rm),
                                 __ldg(psi + xp + W * rm)};
            float ex = ux, ey = uy;
            d2q9_sc_shift_native(ps, a.w1, a.w5, dm.G, 1.f / (dm.tau_inv * rho), ex, ey);
            d2q9_bgk_native(g, ex, ey, rho, a.w0, a.w1, a.w5, dm.tau_inv);
            const int o = dm.off + x + W * y;
            if (MOM) { a.rho[o] = rho; a.ux[o] = ux; a.uy[o] = uy; }
#pragma unroll
            for (int k = 0; k < 9; k++) a.dst[k][o] = g[k];
        }
    }
}

// ---------------------------------------------------------------------------
// Single-pass step over tiles of 32 x BY nodes (the default launch).  A
// block pulls its tile nodes (one per thread) and the ring of nodes around
// them (84 for 32 x 8 tiles), forms psi of all of them in shared memory, and then relaxes
// its tile nodes with the Shan-Chen shift from the shared psi tile.  psi never
// goes through DRAM and a step is one launch: 72 B per node update moved
// (populations read and written once; the ring's pulls are L2 hits of the
// neighbouring tiles) instead of the two passes' 116.  The arithmetic is the
// two-pass path's (same pulls, moments, psi, stencil order, BGK).
// ---------------------------------------------------------------------------
constexpr int ET_BX = 32, ET_PX = ET_BX + 2;  // tile width; psi tile width with its ring

// v modulo n for v in [-n, 2n) (fast) or any v (small domains)
__device__ __forceinline__ int ens_wrap(int v, int n, bool small) {
    if (small) {
        v %= n;
        return v < 0 ? v + n : v;
    }
    return v < 0 ? v + n : (v >= n ? v - n : v);
}

// tiles of ET_BX x BY nodes, one thread per tile node; MINB resident blocks
// per SM bound the registers
template <int BY, int MINB, bool MOM>
__global__ void __launch_bounds__(ET_BX * BY, MINB) ens_tile_kernel(const EnsArgs a) {
    constexpr int PY = BY + 2, RING = 2 * ET_PX + 2 * BY;
    // two psi tiles used by alternate items: a block passes one barrier per
    // item (a warp writing tile b for item i + 2 has passed the barrier of
    // item i + 1, which every warp reaches only after its reads of item i)
    __shared__ float sp2[2][PY][ET_PX];
    const int tx = threadIdx.x % ET_BX, ty = threadIdx.x / ET_BX;
    // this thread's ring node, as a position in the psi tile
    int rx = 0, ry = 0;
    {
        const int r = threadIdx.x;
        if (r < ET_PX) { rx = r; ry = 0; }
        else if (r < 2 * ET_PX) { rx = r - ET_PX; ry = PY - 1; }
        else if (r < 2 * ET_PX + BY) { rx = 0; ry = 1 + r - 2 * ET_PX; }
        else { rx = ET_PX - 1; ry = 1 + r - 2 * ET_PX - BY; }
    }
    int it = blockIdx.x;
    if (it >= a.nitems) return;
    EnsItem next = a.items[it];
    for (int b = 0; it < a.nitems; it += gridDim.x, b ^= 1) {
        float (*sp)[ET_PX] = sp2[b];
        const EnsItem dm = next;
        const int nit = it + gridDim.x;
        if (nit < a.nitems) next = a.items[nit];
        const bool small = dm.W < ET_PX || dm.H < PY;
        // the tile node (a wrapped copy where the tile overhangs the domain);
        // the ring node's loads are issued before either density is formed
        const int xt = ens_wrap(dm.x + tx, dm.W, small), yt = ens_wrap(dm.y + ty, dm.H, small);
        const bool ring = threadIdx.x < RING;
        float g[9], g2[9];
        ens_pull(a, dm, xt, yt, g);
        if (ring)
            ens_pull(a, dm, ens_wrap(dm.x - 1 + rx, dm.W, small),
                     ens_wrap(dm.y - 1 + ry, dm.H, small), g2);
        float rho, ux, uy;
        d2q9_moments_native(g, rho, ux, uy);
        sp[ty + 1][tx + 1] = a.psi_form == 0 ? psi_ref(rho) : psi_exp1(rho);
        if (ring) {
            const float r2 = d2q9_rho_native(g2);
            sp[ry][rx] = a.psi_form == 0 ? psi_ref(r2) : psi_exp1(r2);
        }
        __syncthreads();
        if (dm.x + tx < dm.W && dm.y + ty < dm.H) {
            // psi(x), psi(x+1,y), psi(x,row+1), psi(x-1,y), psi(x,row-1), then
            // the diagonals: the fused pass's order
            const float ps[9] = {sp[ty + 1][tx + 1], sp[ty + 1][tx + 2], sp[ty + 2][tx + 1],
                                 sp[ty + 1][tx],     sp[ty][tx + 1],     sp[ty + 2][tx + 2],
                                 sp[ty + 2][tx],     sp[ty][tx],         sp[ty][tx + 2]};
            float ex = ux, ey = uy;
            d2q9_sc_shift_native(ps, a.w1, a.w5, dm.G, 1.f / (dm.tau_inv * rho), ex, ey);
            d2q9_bgk_native(g, ex, ey, rho, a.w0, a.w1, a.w5, dm.tau_inv);
            const int o = dm.off + xt + dm.W * yt;
            if (MOM) { a.rho[o] = rho; a.ux[o] = ux; a.uy[o] = uy; }
#pragma unroll
            for (int k = 0; k < 9; k++) a.dst[k][o] = g[k];
        }
    }
}

// ---------------------------------------------------------------------------
// Single pass by warps marching down 32-column strips: no block barrier.  A
// work item is a strip of 32 columns and R rows of one domain, and lane l owns
// column x0 + l (a wrapped copy where the strip overhangs the domain).  For
// each row r the warp pulls row r + 1 and forms its psi (lanes 0 and 31 also
// psi of the columns x0 - 1 and x0 + 32), then relaxes row r with the psi
// stencil of rows r - 1, r, r + 1 from its registers and its neighbour lanes.
// Per node update that is 1 + 2/R + 2/32 pulls instead of the tiles' 1.33.
// Same arithmetic and stencil order as the two-pass step.
// ---------------------------------------------------------------------------
constexpr int ENS_MARCH_THREADS = 256;

__device__ __forceinline__ float ens_psi(const EnsArgs &a, float rho) {
    return a.psi_form == 0 ? psi_ref(rho) : psi_exp1(rho);
}

// one strip item (march of R rows of 32 columns) by one warp, plain loads
template <int R, bool MOM>
__device__ __forceinline__ void ens_march_item(const EnsArgs &a, const EnsItem dm, int lane) {
    constexpr unsigned FULL = 0xffffffffu;
    const bool edge = lane == 0 || lane == 31;
    const bool small = dm.W < ET_PX;
    const int x = ens_wrap(dm.x + lane, dm.W, small);
    const int xh = ens_wrap(lane == 0 ? dm.x - 1 : dm.x + ET_BX, dm.W, small);
    const bool own = dm.x + lane < dm.W;
    const int y_end = min(dm.y + R, dm.H);
    float gc[9], rc, uxc, uyc;  // row r: pulled populations and moments at x
    float pm, pc, hm = 0.f, hc = 0.f;  // psi of rows r - 1, r (h: the halo column)
    {
        float g[9];
        const int ym = ens_wrap(dm.y - 1, dm.H, false);
        ens_pull(a, dm, x, ym, g);
        pm = ens_psi(a, d2q9_rho_native(g));
        ens_pull(a, dm, x, dm.y, gc);
        d2q9_moments_native(gc, rc, uxc, uyc);
        pc = ens_psi(a, rc);
        if (edge) {
            ens_pull(a, dm, xh, ym, g);
            hm = ens_psi(a, d2q9_rho_native(g));
            ens_pull(a, dm, xh, dm.y, g);
            hc = ens_psi(a, d2q9_rho_native(g));
        }
    }
    for (int r = dm.y; r < y_end; r++) {
        const int yp = ens_wrap(r + 1, dm.H, false);
        float gn[9], rn, uxn, uyn, hn = 0.f;
        ens_pull(a, dm, x, yp, gn);
        if (edge) {
            float g[9];
            ens_pull(a, dm, xh, yp, g);
            hn = ens_psi(a, d2q9_rho_native(g));
        }
        d2q9_moments_native(gn, rn, uxn, uyn);
        const float pn = ens_psi(a, rn);
        // x - 1 and x + 1 from the neighbour lanes, the halo at the strip ends
        float lm = __shfl_up_sync(FULL, pm, 1), lc = __shfl_up_sync(FULL, pc, 1);
        float ln = __shfl_up_sync(FULL, pn, 1);
        float qm = __shfl_down_sync(FULL, pm, 1), qc = __shfl_down_sync(FULL, pc, 1);
        float qn = __shfl_down_sync(FULL, pn, 1);
        if (lane == 0) { lm = hm; lc = hc; ln = hn; }
        if (lane == 31) { qm = hm; qc = hc; qn = hn; }
        if (own) {
            // the fused pass's order: psi(x), psi(x+1,y), psi(x,row+1),
            // psi(x-1,y), psi(x,row-1), then the diagonals
            const float ps[9] = {pc, qc, pn, lc, pm, qn, ln, lm, qm};
            float ex = uxc, ey = uyc;
            d2q9_sc_shift_native(ps, a.w1, a.w5, dm.G, 1.f / (dm.tau_inv * rc), ex, ey);
            d2q9_bgk_native(gc, ex, ey, rc, a.w0, a.w1, a.w5, dm.tau_inv);
            const int o = dm.off + x + dm.W * r;
            if (MOM) { a.rho[o] = rc; a.ux[o] = uxc; a.uy[o] = uyc; }
#pragma unroll
            for (int k = 0; k < 9; k++) a.dst[k][o] = gc[k];
        }
#pragma unroll
        for (int k = 0; k < 9; k++) gc[k] = gn[k];
        rc = rn; uxc = uxn; uyc = uyn;
        pm = pc; pc = pn; hm = hc; hc = hn;
    }
}

template <int R, int MINB, bool MOM>
__global__ void __launch_bounds__(ENS_MARCH_THREADS, MINB) ens_march_kernel(const EnsArgs a) {
    const int lane = threadIdx.x & 31;
    const int warps_per_block = ENS_MARCH_THREADS / 32;
    const int nwarps = gridDim.x * warps_per_block;
    for (int it = blockIdx.x * warps_per_block + (threadIdx.x >> 5); it < a.nitems;
         it += nwarps)
        ens_march_item<R, MOM>(a, a.items[it], lane);
}

// ---------------------------------------------------------------------------
// Strips with a shared-memory row ring.  The march above must wait for the
// loads of row r + 1 before it can relax row r: a DRAM latency per row for
// every warp.  Here each warp keeps the source rows its pulls read in a ring
// of ENS_RING slots in shared memory (9 populations x 40 columns: the strip,
// the two halo columns and their outer neighbours, rounded out to 16-byte
// chunks) and copies source row r + 4 with 16-byte cp.async (one commit group
// per row) before it pulls row r + 1, so rows land two rows ahead of their
// use and the pulls are shared-memory loads.  A lane waits for its own groups
// (cp.async.wait_group) and a warp barrier makes every lane's copies visible;
// no block barrier.  An item qualifies when its domain's rows start on 16
// bytes and no chunk straddles its periodic x edge (W a multiple of 32, first
// node a multiple of 4); the work list puts those first, and the other items
// take the plain march in a second launch (kept out of this kernel, whose
// registers it would crowd).  Same pulls and arithmetic as the march, so the
// same bits.
// ---------------------------------------------------------------------------
constexpr int ENS_RING = 6;                    // source-row slots per warp
constexpr int ENS_RCOLS = ET_BX + 8;           // columns x0 - 4 .. x0 + 35
constexpr int ENS_RROW = 9 * ENS_RCOLS;        // floats per slot (90 chunks of 16 bytes)
constexpr int ENS_RING_SMEM = ENS_RING * ENS_RROW * 4 * (ENS_MARCH_THREADS / 32);  // 69 120 B

__device__ __forceinline__ void ens_cp16(float *dst, const float *src) {
    asm volatile("cp.async.cg.shared.global [%0], [%1], 16;\n" ::"r"(
                     (uint32_t)__cvta_generic_to_shared(dst)),
                 "l"(src)
                 : "memory");
}
__device__ __forceinline__ void ens_cp_commit() {
    asm volatile("cp.async.commit_group;\n" ::: "memory");
}
// this lane's commit groups except the newest N have landed
template <int N>
__device__ __forceinline__ void ens_cp_wait() {
    asm volatile("cp.async.wait_group %0;\n" ::"n"(N) : "memory");
}

template <int R, int MINB, bool MOM>
__global__ void __launch_bounds__(ENS_MARCH_THREADS, MINB) ens_ring_kernel(const EnsArgs a) {
    constexpr unsigned FULL = 0xffffffffu;
    extern __shared__ __align__(16) float ens_ring_smem[];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    float *const ring = ens_ring_smem + warp * ENS_RING * ENS_RROW;
    const int warps_per_block = ENS_MARCH_THREADS / 32;
    const int nwarps = gridDim.x * warps_per_block;
    const bool edge = lane == 0 || lane == 31;
    const int col = 4 + lane, hcol = lane == 0 ? 3 : 4 + ET_BX;  // ring columns of x, xh
    for (int it = blockIdx.x * warps_per_block + warp; it < a.nitems; it += nwarps) {
        const EnsItem dm = a.items[it];
        if ((dm.W & 31) || (dm.off & 3)) continue;  // the work list gives this kernel none
        const int y_end = min(dm.y + R, dm.H);
        const bool small_h = dm.H < 4;
        // this lane's chunks of a source row (chunk c = 10 k + q: population k,
        // columns x0 - 4 + 4q .. + 3), addresses in row 0 of the domain
        const float *cs[3];
#pragma unroll
        for (int i = 0; i < 3; i++) {
            const int c = min(lane + 32 * i, 89);
            const int k = c / 10, q = c - 10 * k;
            cs[i] = a.src[k] + dm.off + ens_wrap(dm.x - 4 + 4 * q, dm.W, false);
        }
        // source row sr of the item lives in slot (sr - (y - 2)) % ENS_RING
        auto slot = [&](int i) { return ring + i * ENS_RROW; };
        // source row sr into slot i as one commit group (empty past the item)
        auto issue = [&](int sr, int i) {
            if (sr <= y_end + 1) {
                const long row = (long)dm.W * ens_wrap(sr, dm.H, small_h);
                float *sl = slot(i);
#pragma unroll
                for (int j = 0; j < 3; j++)
                    if (lane + 32 * j < 90) ens_cp16(sl + 4 * (lane + 32 * j), cs[j] + row);
            }
            ens_cp_commit();
        };
        // pull of ring column cl of the row whose upstream rows (row - 1, row,
        // row + 1) sit in slots im, i0, ip: population k from row - cr_k,
        // column cl - cx_k
        auto pull = [&](int cl, int im, int i0, int ip, float(&g)[9]) {
            const float *sm = slot(im), *s0 = slot(i0), *sp = slot(ip);
#pragma unroll
            for (int k = 0; k < 9; k++) {
                const float *sl = d2_cr(k) > 0 ? sm : (d2_cr(k) < 0 ? sp : s0);
                g[k] = sl[k * ENS_RCOLS + cl - d2_cx(k)];
            }
        };
#pragma unroll
        for (int i = 0; i < ENS_RING; i++) issue(dm.y - 2 + i, i);  // source rows y - 2 .. y + 3
        ens_cp_wait<ENS_RING - 4>();  // rows y - 2 .. y + 1 have landed
        __syncwarp();
        float gc[9], rc, uxc, uyc;  // row r: pulled populations and moments at x
        float pm, pc, hm = 0.f, hc = 0.f;  // psi of rows r - 1, r (h: the halo column)
        {
            float g[9];
            pull(col, 0, 1, 2, g);
            pm = ens_psi(a, d2q9_rho_native(g));
            pull(col, 1, 2, 3, gc);
            d2q9_moments_native(gc, rc, uxc, uyc);
            pc = ens_psi(a, rc);
            if (edge) {
                pull(hcol, 0, 1, 2, g);
                hm = ens_psi(a, d2q9_rho_native(g));
                pull(hcol, 1, 2, 3, g);
                hc = ens_psi(a, d2q9_rho_native(g));
            }
        }
        auto next = [](int i) { return i == ENS_RING - 1 ? 0 : i + 1; };
        int i0 = 2;  // slot of source row r
        const int x = dm.x + lane;
        for (int r = dm.y; r < y_end; r++) {
            const int i1 = next(i0), i2 = next(i1);
            __syncwarp();  // every lane is done with the slot of source row r - 2
            issue(r + ENS_RING - 2, i0 >= 2 ? i0 - 2 : i0 + ENS_RING - 2);
            ens_cp_wait<ENS_RING - 4>();  // source row r + 2 has landed
            __syncwarp();
            float gn[9], rn, uxn, uyn, hn = 0.f;
            pull(col, i0, i1, i2, gn);
            if (edge) {
                float g[9];
                pull(hcol, i0, i1, i2, g);
                hn = ens_psi(a, d2q9_rho_native(g));
            }
            i0 = i1;
            d2q9_moments_native(gn, rn, uxn, uyn);
            const float pn = ens_psi(a, rn);
            // x - 1 and x + 1 from the neighbour lanes, the halo at the strip ends
            float lm = __shfl_up_sync(FULL, pm, 1), lc = __shfl_up_sync(FULL, pc, 1);
            float ln = __shfl_up_sync(FULL, pn, 1);
            float qm = __shfl_down_sync(FULL, pm, 1), qc = __shfl_down_sync(FULL, pc, 1);
            float qn = __shfl_down_sync(FULL, pn, 1);
            if (lane == 0) { lm = hm; lc = hc; ln = hn; }
            if (lane == 31) { qm = hm; qc = hc; qn = hn; }
            const float ps[9] = {pc, qc, pn, lc, pm, qn, ln, lm, qm};
            float ex = uxc, ey = uyc;
            d2q9_sc_shift_native(ps, a.w1, a.w5, dm.G, 1.f / (dm.tau_inv * rc), ex, ey);
            d2q9_bgk_native(gc, ex, ey, rc, a.w0, a.w1, a.w5, dm.tau_inv);
            const int o = dm.off + x + dm.W * r;
            if (MOM) { a.rho[o] = rc; a.ux[o] = uxc; a.uy[o] = uyc; }
#pragma unroll
            for (int k = 0; k < 9; k++) a.dst[k][o] = gc[k];
#pragma unroll
            for (int k = 0; k < 9; k++) gc[k] = gn[k];
            rc = rn; uxc = uxn; uyc = uyn;
            pm = pc; pc = pn; hm = hc; hc = hn;
        }
        __syncwarp();  // the next item's copies overwrite slots this item read
    }
}

// ring strip shapes: rows per item and the register bound (resident blocks per SM)
#define LB_ENS_RING(X) \
    X(10, 32, 3)       \
    X(11, 64, 3)       \
    X(12, 16, 3)

int ens_ring_rows(int shape) {
    switch (shape) {
#define LB_ENS_RROWS(S, R, MINB) \
    case S: return R;
        LB_ENS_RING(LB_ENS_RROWS)
#undef LB_ENS_RROWS
        default: return 0;
    }
}

template <int R, int MINB>
cudaError_t ens_ring_launch(const EnsArgs &a, bool mom, unsigned grid, cudaStream_t s) {
    // once per instantiation
    static const cudaError_t attr_e[2] = {
        cudaFuncSetAttribute(ens_ring_kernel<R, MINB, false>,
                             cudaFuncAttributeMaxDynamicSharedMemorySize, ENS_RING_SMEM),
        cudaFuncSetAttribute(ens_ring_kernel<R, MINB, true>,
                             cudaFuncAttributeMaxDynamicSharedMemorySize, ENS_RING_SMEM)};
    if (attr_e[mom ? 1 : 0] != cudaSuccess) return attr_e[mom ? 1 : 0];
    if (mom) ens_ring_kernel<R, MINB, true><<<grid, ENS_MARCH_THREADS, ENS_RING_SMEM, s>>>(a);
    else ens_ring_kernel<R, MINB, false><<<grid, ENS_MARCH_THREADS, ENS_RING_SMEM, s>>>(a);
    return cudaGetLastError();
}

// march shapes: rows per item and the register bound (resident blocks per SM)
#define LB_ENS_MARCH(X) \
    X(6, 32, 3)         \
    X(7, 32, 4)         \
    X(8, 64, 3)         \
    X(9, 16, 3)

int ens_march_rows(int shape) {
    switch (shape) {
#define LB_ENS_MROWS(S, R, MINB) \
    case S: return R;
        LB_ENS_MARCH(LB_ENS_MROWS)
#undef LB_ENS_MROWS
        default: return 0;
    }
}

// tile shapes: rows per tile and the register bound (resident blocks per SM)
#define LB_ENS_TILES(X) \
    X(1, 8, 5)          \
    X(2, 8, 6)          \
    X(3, 16, 2)         \
    X(4, 16, 3)         \
    X(5, 32, 1)

int ens_tile_rows(int shape) {
    switch (shape) {
#define LB_ENS_ROWS(S, BY, MINB) \
    case S: return BY;
        LB_ENS_TILES(LB_ENS_ROWS)
#undef LB_ENS_ROWS
        default: return 0;
    }
}

struct LaunchShape {
    int bx, ry, bps;  // threads along x, rows per work item (= blockDim.y), blocks per SM;
                      // bx = 0: the single-pass tile kernel of tile shape ry
};

}  // namespace

struct lb_ensemble {
    int nd = 0;
    std::vector<EnsDomain> dom;
    long NT = 0, stride = 0;
    float *pop[2] = {nullptr, nullptr};
    float *psi = nullptr, *mom = nullptr;
    EnsItem *items_d = nullptr;
    int nitems = 0, items_cap = 0;
    int nring = 0;  // ring strip shapes: the leading items the ring kernel takes
    int cur = 0, psi_form = LB_PSI_EXP1, sms = 1, graph_steps = 32;
    // single-pass warp strips of 32 rows with the shared-memory row ring, 3
    // blocks per SM: 72.4 GLUPS on 512 droplet domains, against 63.2 for the
    // strips with plain loads (shape 6)
    LaunchShape shape{0, 10, 3};
    cudaStream_t stream = nullptr;
    cudaEvent_t ev0 = nullptr, ev1 = nullptr;
    cudaGraphExec_t graph[2] = {nullptr, nullptr};
    int64_t launches = 0;
    std::string err;
};

namespace {

int efail(lb_ensemble *e, int code, const std::string &m) {
    if (e) e->err = m;
    return code;
}
#define LB_ETRY(e, where, call)                                                      \
    do {                                                                             \
        cudaError_t c_ = (call);                                                     \
        if (c_ != cudaSuccess)                                                       \
            return efail(e, LB_ERR_CUDA, std::string(where) + ": " + cudaGetErrorString(c_)); \
    } while (0)

const float W2F[3] = {(float)(4.0 / 9.0), (float)(1.0 / 9.0), (float)(1.0 / 36.0)};

float *pk(lb_ensemble *e, int set, int k) { return e->pop[set] + (long)k * e->stride; }

EnsArgs args_for(lb_ensemble *e, int from) {
    EnsArgs a{};
    for (int k = 0; k < 9; k++) {
        a.src[k] = pk(e, from, k);
        a.dst[k] = pk(e, 1 - from, k);
    }
    a.psi = e->psi;
    a.rho = e->mom; a.ux = e->mom + e->stride; a.uy = e->mom + 2 * e->stride;
    a.items = e->items_d;
    a.nitems = e->nitems;
    a.psi_form = e->psi_form;
    a.w0 = W2F[0]; a.w1 = W2F[1]; a.w5 = W2F[2];
    return a;
}

int launches_per_step(const lb_ensemble *e) {
    if (e->shape.bx != 0) return 2;
    if (ens_ring_rows(e->shape.ry)) return (e->nring > 0) + (e->nitems > e->nring);
    return 1;
}

// ring strip shapes: the ring kernel over the leading qualifying items, the
// plain march over the rest
template <int R, int MINB>
cudaError_t ens_ring_step(lb_ensemble *e, const EnsArgs &a, bool mom) {
    const auto grid_for = [e](int n) {
        return (unsigned)std::max(1, std::min(n, e->sms * e->shape.bps));
    };
    EnsArgs ar = a, am = a;
    ar.nitems = e->nring;
    am.items = a.items + e->nring;
    am.nitems = a.nitems - e->nring;
    if (ar.nitems > 0) {
        const cudaError_t c = ens_ring_launch<R, MINB>(ar, mom, grid_for(ar.nitems), e->stream);
        if (c != cudaSuccess) return c;
        e->launches += 1;
    }
    if (am.nitems > 0) {
        const unsigned g = grid_for(am.nitems);
        if (mom) ens_march_kernel<R, MINB, true><<<g, ENS_MARCH_THREADS, 0, e->stream>>>(am);
        else ens_march_kernel<R, MINB, false><<<g, ENS_MARCH_THREADS, 0, e->stream>>>(am);
        e->launches += 1;
        return cudaGetLastError();
    }
    return cudaSuccess;
}

cudaError_t ens_step(lb_ensemble *e, int from, bool mom) {
    const EnsArgs a = args_for(e, from);
    const unsigned grid = (unsigned)std::max(1, std::min(e->nitems, e->sms * e->shape.bps));
    if (e->shape.bx == 0) {
        switch (e->shape.ry) {
#define LB_ENS_LAUNCH(S, BY, MINB)                                                            \
    case S:                                                                                   \
        if (mom) ens_tile_kernel<BY, MINB, true><<<grid, ET_BX * BY, 0, e->stream>>>(a);    \
        else ens_tile_kernel<BY, MINB, false><<<grid, ET_BX * BY, 0, e->stream>>>(a);       \
        break;
            LB_ENS_TILES(LB_ENS_LAUNCH)
#undef LB_ENS_LAUNCH
#define LB_ENS_MLAUNCH(S, R, MINB)                                                             \
    case S:                                                                                    \
        if (mom) ens_march_kernel<R, MINB, true><<<grid, ENS_MARCH_THREADS, 0, e->stream>>>(a); \
        else ens_march_kernel<R, MINB, false><<<grid, ENS_MARCH_THREADS, 0, e->stream>>>(a);    \
        break;
            LB_ENS_MARCH(LB_ENS_MLAUNCH)
#undef LB_ENS_MLAUNCH
#define LB_ENS_RLAUNCH(S, R, MINB)                                                             \
    case S:                                                                                    \
        return ens_ring_step<R, MINB>(e, a, mom);
            LB_ENS_RING(LB_ENS_RLAUNCH)
#undef LB_ENS_RLAUNCH
            default: return cudaErrorInvalidValue;
        }
        e->launches += 1;
        return cudaGetLastError();
    }
    const dim3 block(e->shape.bx, e->shape.ry);
    ens_density_kernel<<<grid, block, 0, e->stream>>>(a);
    cudaError_t c = cudaGetLastError();
    if (c != cudaSuccess) return c;
    if (mom) ens_fused_kernel<true><<<grid, block, 0, e->stream>>>(a);
    else ens_fused_kernel<false><<<grid, block, 0, e->stream>>>(a);
    e->launches += 2;
    return cudaGetLastError();
}

void drop_graphs(lb_ensemble *e) {
    for (int i = 0; i < 2; i++)
        if (e->graph[i]) {
            cudaGraphExecDestroy(e->graph[i]);
            e->graph[i] = nullptr;
        }
}

// work list of row groups for the current shape
int build_items(lb_ensemble *e) {
    std::vector<EnsItem> items, rest;
    for (int d = 0; d < e->nd; d++) {
        const EnsDomain &m = e->dom[d];
        if (e->shape.bx == 0) {  // tiles or strips, row by row
            const int rows = ens_tile_rows(e->shape.ry) + ens_march_rows(e->shape.ry) +
                             ens_ring_rows(e->shape.ry);
            // ring strips: the items the ring kernel takes first, the rest after
            const bool ring = ens_ring_rows(e->shape.ry) > 0;
            std::vector<EnsItem> &to = ring && ((m.W & 31) || (m.off & 3)) ? rest : items;
            for (int y = 0; y < m.H; y += rows)
                for (int x = 0; x < m.W; x += ET_BX)
                    to.push_back(EnsItem{m.off, m.W, m.H, y, m.G, m.tau_inv, x});
        } else {  // groups of ry rows
            for (int y = 0; y < m.H; y += e->shape.ry)
                items.push_back(EnsItem{m.off, m.W, m.H, y, m.G, m.tau_inv, 0});
        }
    }
    e->nring = (int)items.size();
    items.insert(items.end(), rest.begin(), rest.end());
    if ((int)items.size() > e->items_cap) {
        if (e->items_d) cudaFree(e->items_d);
        e->items_d = nullptr;
        LB_ETRY(e, "work list", cudaMalloc(&e->items_d, sizeof(EnsItem) * items.size()));
        e->items_cap = (int)items.size();
    }
    LB_ETRY(e, "work list", cudaMemcpy(e->items_d, items.data(), sizeof(EnsItem) * items.size(),
                                       cudaMemcpyHostToDevice));
    e->nitems = (int)items.size();
    drop_graphs(e);
    return LB_OK;
}

int egraph(lb_ensemble *e, int from, cudaGraphExec_t *out) {
    if (e->graph[from]) { *out = e->graph[from]; return LB_OK; }
    const int64_t before = e->launches;
    LB_ETRY(e, "capture", cudaStreamBeginCapture(e->stream, cudaStreamCaptureModeThreadLocal));
    cudaError_t c = cudaSuccess;
    int set = from;
    for (int i = 0; i < e->graph_steps && c == cudaSuccess; i++) {
        c = ens_step(e, set, false);
        set = 1 - set;
    }
    cudaGraph_t g;
    cudaError_t c2 = cudaStreamEndCapture(e->stream, &g);
    e->launches = before;
    LB_ETRY(e, "capture", c);
    LB_ETRY(e, "capture", c2);
    c = cudaGraphInstantiate(&e->graph[from], g, 0);
    cudaGraphDestroy(g);
    LB_ETRY(e, "cudaGraphInstantiate", c);
    *out = e->graph[from];
    return LB_OK;
}

}  // namespace

extern "C" {

int lb_ensemble_create(int nd, const int *nx, const int *ny, const float *G, const float *tau_inv,
                       int psi_form, lb_ensemble **out) {
    if (!out || nd < 1 || !nx || !ny || !G || !tau_inv) return LB_ERR_ARG;
    *out = nullptr;
    if (psi_form != LB_PSI_REF && psi_form != LB_PSI_EXP1) return LB_ERR_ARG;
    lb_ensemble *e = new lb_ensemble;
    e->nd = nd;
    e->psi_form = psi_form;
    long off = 0;
    for (int d = 0; d < nd; d++) {
        if (nx[d] < 1 || ny[d] < 1) { delete e; return LB_ERR_ARG; }
        e->dom.push_back(EnsDomain{nx[d], ny[d], (int)off, G[d], tau_inv[d]});
        off += (long)nx[d] * ny[d];
        if (off > (1L << 31) - 256) { delete e; return LB_ERR_ARG; }
    }
    e->NT = off;
    e->stride = (off + 127) / 128 * 128;
    int dev = 0;
    cudaError_t c = cudaGetDevice(&dev);
    if (c == cudaSuccess) c = cudaDeviceGetAttribute(&e->sms, cudaDevAttrMultiProcessorCount, dev);
    if (c == cudaSuccess) c = cudaMalloc(&e->pop[0], sizeof(float) * 9 * e->stride);
    if (c == cudaSuccess) c = cudaMalloc(&e->pop[1], sizeof(float) * 9 * e->stride);
    if (c == cudaSuccess) c = cudaMalloc(&e->psi, sizeof(float) * e->stride);
    if (c == cudaSuccess) c = cudaMalloc(&e->mom, sizeof(float) * 3 * e->stride);
    if (c == cudaSuccess) c = cudaMemset(e->mom, 0, sizeof(float) * 3 * e->stride);
    if (c == cudaSuccess) c = cudaStreamCreateWithFlags(&e->stream, cudaStreamNonBlocking);
    if (c == cudaSuccess) c = cudaEventCreate(&e->ev0);
    if (c == cudaSuccess) c = cudaEventCreate(&e->ev1);
    if (c != cudaSuccess) {
        lb_ensemble_destroy(e);
        return c == cudaErrorMemoryAllocation ? LB_ERR_NOMEM : LB_ERR_CUDA;
    }
    if (build_items(e) != LB_OK) {
        lb_ensemble_destroy(e);
        return LB_ERR_CUDA;
    }
    *out = e;
    return LB_OK;
}

int lb_ensemble_destroy(lb_ensemble *e) {
    if (!e) return LB_ERR_ARG;
    if (e->stream) cudaStreamSynchronize(e->stream);
    drop_graphs(e);
    for (int i = 0; i < 2; i++)
        if (e->pop[i]) cudaFree(e->pop[i]);
    if (e->psi) cudaFree(e->psi);
    if (e->mom) cudaFree(e->mom);
    if (e->items_d) cudaFree(e->items_d);
    if (e->ev0) cudaEventDestroy(e->ev0);
    if (e->ev1) cudaEventDestroy(e->ev1);
    if (e->stream) cudaStreamDestroy(e->stream);
    delete e;
    return LB_OK;
}

const char *lb_ensemble_error(const lb_ensemble *e) { return e ? e->err.c_str() : "null ensemble"; }
long lb_ensemble_nodes(const lb_ensemble *e) { return e ? e->NT : -1; }
long lb_ensemble_offset(const lb_ensemble *e, int d) {
    return (e && d >= 0 && d < e->nd) ? e->dom[d].off : -1;
}
int64_t lb_ensemble_launch_count(const lb_ensemble *e) { return e ? e->launches : -1; }

int lb_ensemble_set_populations(lb_ensemble *e, const float *f) {
    if (!e || !f) return LB_ERR_ARG;
    for (int k = 0; k < 9; k++)
        LB_ETRY(e, "lb_ensemble_set_populations",
                cudaMemcpyAsync(pk(e, e->cur, k), f + (long)k * e->NT, sizeof(float) * e->NT,
                                cudaMemcpyHostToDevice, e->stream));
    LB_ETRY(e, "lb_ensemble_set_populations", cudaStreamSynchronize(e->stream));
    return LB_OK;
}

int lb_ensemble_get_populations(lb_ensemble *e, float *f) {
    if (!e || !f) return LB_ERR_ARG;
    for (int k = 0; k < 9; k++)
        LB_ETRY(e, "lb_ensemble_get_populations",
                cudaMemcpyAsync(f + (long)k * e->NT, pk(e, e->cur, k), sizeof(float) * e->NT,
                                cudaMemcpyDeviceToHost, e->stream));
    LB_ETRY(e, "lb_ensemble_get_populations", cudaStreamSynchronize(e->stream));
    return LB_OK;
}

int lb_ensemble_init_equilibrium(lb_ensemble *e, const float *rho) {
    if (!e || !rho) return LB_ERR_ARG;
    LB_ETRY(e, "lb_ensemble_init_equilibrium",
            cudaMemcpyAsync(e->mom, rho, sizeof(float) * e->NT, cudaMemcpyHostToDevice, e->stream));
    Pop<9> p;
    for (int k = 0; k < 9; k++) p.f[k] = pk(e, e->cur, k);
    LB_ETRY(e, "lb_ensemble_init_equilibrium",
            launch_d2q9_equilibrium(p, e->mom, nullptr, nullptr, (int)e->NT, W2F[0], W2F[1],
                                    W2F[2], e->stream));
    e->launches += 1;
    LB_ETRY(e, "lb_ensemble_init_equilibrium", cudaStreamSynchronize(e->stream));
    return LB_OK;
}

int lb_ensemble_step(lb_ensemble *e, int nsteps) {
    if (!e || nsteps < 0) return LB_ERR_ARG;
    if (nsteps == 0) return LB_OK;
    int rest = nsteps - 1;
    while (rest >= e->graph_steps) {
        cudaGraphExec_t g;
        const int rc = egraph(e, e->cur, &g);
        if (rc != LB_OK) return rc;
        LB_ETRY(e, "cudaGraphLaunch", cudaGraphLaunch(g, e->stream));
        e->launches += (int64_t)launches_per_step(e) * e->graph_steps;
        rest -= e->graph_steps;
    }
    for (; rest > 0; rest--) {
        LB_ETRY(e, "lb_ensemble_step", ens_step(e, e->cur, false));
        e->cur = 1 - e->cur;
    }
    LB_ETRY(e, "lb_ensemble_step", ens_step(e, e->cur, true));
    e->cur = 1 - e->cur;
    return LB_OK;
}

int lb_ensemble_time_steps(lb_ensemble *e, int nsteps, float *ms) {
    if (!e || !ms) return LB_ERR_ARG;
    LB_ETRY(e, "lb_ensemble_time_steps", cudaEventRecord(e->ev0, e->stream));
    const int rc = lb_ensemble_step(e, nsteps);
    if (rc != LB_OK) return rc;
    LB_ETRY(e, "lb_ensemble_time_steps", cudaEventRecord(e->ev1, e->stream));
    LB_ETRY(e, "lb_ensemble_time_steps", cudaEventSynchronize(e->ev1));
    LB_ETRY(e, "lb_ensemble_time_steps", cudaEventElapsedTime(ms, e->ev0, e->ev1));
    return LB_OK;
}

int lb_ensemble_get_moments(lb_ensemble *e, float *rho, float *ux, float *uy) {
    if (!e) return LB_ERR_ARG;
    float *dst[3] = {rho, ux, uy};
    for (int i = 0; i < 3; i++)
        if (dst[i])
            LB_ETRY(e, "lb_ensemble_get_moments",
                    cudaMemcpyAsync(dst[i], e->mom + (long)i * e->stride, sizeof(float) * e->NT,
                                    cudaMemcpyDeviceToHost, e->stream));
    LB_ETRY(e, "lb_ensemble_get_moments", cudaStreamSynchronize(e->stream));
    return LB_OK;
}

int lb_ensemble_set_launch(lb_ensemble *e, int threads_x, int rows, int blocks_per_sm) {
    const bool tiles = threads_x == 0;
    if (!e || blocks_per_sm < 1 || blocks_per_sm > 32 ||
        (tiles && ens_tile_rows(rows) + ens_march_rows(rows) + ens_ring_rows(rows) == 0) ||
        (!tiles && (threads_x < 32 || threads_x % 32 || rows < 1 || threads_x * rows > 1024)))
        return LB_ERR_ARG;
    LB_ETRY(e, "lb_ensemble_set_launch", cudaStreamSynchronize(e->stream));
    e->shape = LaunchShape{threads_x, rows, blocks_per_sm};
    return build_items(e);
}

int lb_ensemble_get_launch(const lb_ensemble *e, int out[3]) {
    if (!e || !out) return LB_ERR_ARG;
    out[0] = e->shape.bx; out[1] = e->shape.ry; out[2] = e->shape.bps;
    return LB_OK;
}

// Times every candidate shape for trial_steps steps (after one untimed step)
// on the ensemble's current state and keeps the fastest.  The state advances
// by (trial_steps + 1) steps per candidate: tune before setting the initial
// state.
int lb_ensemble_autotune(lb_ensemble *e, int trial_steps, int out[3]) {
    if (!e || trial_steps < 1) return LB_ERR_ARG;
    // the single-pass tiles, then the two-pass row groups {64, 128, 256
    // threads} x {1, 2, 4 rows} x {2, 4, 8 blocks}
    static const int BX[3] = {64, 128, 256}, RY[3] = {1, 2, 4}, BPS[3] = {2, 4, 8};
    // (tile or strip shape, blocks per SM): each shape at its register-bound
    // residency and at twice it
    static const int TILES[][2] = {{1, 5}, {1, 10}, {2, 6}, {2, 12}, {3, 2}, {3, 4}, {4, 3},
                                   {5, 1}, {6, 3}, {6, 6}, {7, 4}, {7, 8}, {8, 3}, {9, 3},
                                   {10, 3}, {11, 3}, {12, 3}};
    std::vector<LaunchShape> cand;
    for (const auto &t : TILES) cand.push_back(LaunchShape{0, t[0], t[1]});
    for (int i = 0; i < 3; i++)
        for (int j = 0; j < 3; j++)
            for (int k = 0; k < 3; k++)
                if (BX[i] * RY[j] <= 512) cand.push_back(LaunchShape{BX[i], RY[j], BPS[k]});
    float best = 1e30f;
    LaunchShape pick = e->shape;
    for (const LaunchShape &c : cand) {
        int rc = lb_ensemble_set_launch(e, c.bx, c.ry, c.bps);
        if (rc != LB_OK) return rc;
        LB_ETRY(e, "autotune", ens_step(e, e->cur, false));  // one untimed step
        e->cur = 1 - e->cur;
        LB_ETRY(e, "autotune", cudaEventRecord(e->ev0, e->stream));
        for (int s = 0; s < trial_steps; s++) {
            LB_ETRY(e, "autotune", ens_step(e, e->cur, false));
            e->cur = 1 - e->cur;
        }
        LB_ETRY(e, "autotune", cudaEventRecord(e->ev1, e->stream));
        LB_ETRY(e, "autotune", cudaEventSynchronize(e->ev1));
        float ms = 0.f;
        LB_ETRY(e, "autotune", cudaEventElapsedTime(&ms, e->ev0, e->ev1));
        if (ms < best) {
            best = ms;
            pick = e->shape;
        }
    }
    const int rc = lb_ensemble_set_launch(e, pick.bx, pick.ry, pick.bps);
    if (rc != LB_OK) return rc;
    if (out) lb_ensemble_get_launch(e, out);
    return LB_OK;
}

}  // extern "C"
