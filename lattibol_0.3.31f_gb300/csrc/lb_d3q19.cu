// lb_d3q19.cu -- D3Q19 kernels: the fused pull-stream + collide step (the hot
// path) with FP32 or 16-bit deviation storage and an optional Shan-Chen
// force, the density (psi) pass of the Shan-Chen step, and the
// reference-exact standalone streaming / collision / border kernels behind
// the drop-in entry points.
//
// Layout: structure of arrays, one array per population, node index
// o = x + W*(y + H*z) (reference src/streaming.cu:98).  A thread owns one
// node; a block covers a run of x at fixed (y, z), so every population load
// and store of a warp is one coalesced row (shifted by one element for
// populations with c_x != 0).
#include "lb_d3q19.cuh"

namespace lb {

// ---------------------------------------------------------------------------
// Fused step.  Pull: population k of node o comes from o - c_k.
//  * fluid node: pull all 18, (reference mode) Zou-He on the x faces,
//    moments, (native) force shift and Shan-Chen shift, BGK, store to dst.
//  * reference mode, solid node: reproduces the reference's full-way
//    bounce-back storage.  Slot m of a solid node receives, by the swap
//    streaming of src/streaming.cu, the population opp(m) leaving
//    o + c_m, i.e. src[opp(m)][o + c_m] -- unless the node that owns that
//    swap pair is solid_bound (o itself for the positive slots, o + c_m for
//    the others), in which case the slot keeps its value.
//  * native mode: a fluid node whose upstream neighbour is a wall takes its
//    own outgoing opposite population (half-way bounce-back), minus the
//    moving-wall term corr[opp(k)].  Wall nodes are not updated.
// Shan-Chen (native): F = -G psi(x) sum_k w_k psi(x + c_k) c_k with psi from
// the density pass of this step, applied as a velocity shift F/(tau_inv rho)
// like the reference's force (src/collision.cu:92-96).
// ---------------------------------------------------------------------------
// 16-bit storage without Shan-Chen waits on its loads, not on issue.  Two
// things put more of them in flight:
//  * at least 12 blocks per SM (40 registers, a 24-byte spill; 64.0 vs 62.4
//    GLUPS on the 256x128x128 channel, FP16); FP32 keeps its own register
//    count (46.0 vs 44.2 GLUPS when held to 12 blocks);
//  * an L2 prefetch of the populations the block FUSED_PF_BLOCKS later in the
//    sweep pulls: its two 128-byte lines of each of the 19 arrays (66.8 vs
//    63.4 GLUPS; 608 to 1520 blocks ahead measured alike, 3648 lost the gain;
//    prefetching that block's flags as well, or pulling before testing the
//    node's flags, measured no faster).
constexpr long FUSED_PF_BLOCKS = 912;
static_assert(D3_BLOCK * 2 == 256, "two 128-byte lines per 16-bit population run");

template <int MODE, bool MOM, bool PLOT, typename S, bool SC>
__global__ void __launch_bounds__(D3_BLOCK, (sizeof(S) == 2 && !SC) ? 12 : 0)
    d3q19_fused_kernel(const D3Args a) {
    const Coord3 c(a);
    const int x = c.x, y = c.y, z = c.z;
    if (x >= a.W) return;
    const int o = x + a.W * (y + a.H * z);
    if (sizeof(S) == 2 && MODE == MODE_NATIVE && !SC && threadIdx.x < 19 * 2) {
        // L2 prefetch: line (threadIdx.x & 1) of population threadIdx.x / 2's
        // run of the block FUSED_PF_BLOCKS later in the sweep
        const int k = threadIdx.x >> 1, l = threadIdx.x & 1;
        const long po = ((long)o - threadIdx.x) +
                        (a.reverse ? -1L : 1L) * FUSED_PF_BLOCKS * blockDim.x + l * 64;
        if (po >= 0 && po < (long)a.W * a.H * a.D)
            asm volatile("prefetch.global.L2 [%0];" ::"l"(reinterpret_cast<const S *>(a.src.f[k]) +
                                                           po));
    }
    const uint8_t fl = a.flags[o];
    const Nbr3 n(x, y, z, a.W, a.H, a.D);

    if (MODE == MODE_REF && (fl & CELL_WALL)) {
        const bool sb_self = a.sb[o] != 0;
#pragma unroll
        for (int m = 0; m < 19; m++) {
            float v;
            if (m == 0) {
                v = ld_stream(a.src.f[0] + o);
            } else {
                const int on = o + n.off(d3_cx(m), d3_cy(m), d3_cz(m));
                const bool resp_sb = d3_pos(m) ? sb_self : (a.sb[on] != 0);
                v = resp_sb ? ld_stream(a.src.f[m] + o) : ld_stream(a.src.f[d3_opp(m)] + on);
            }
            a.dst.f[m][o] = v;
        }
        if (MOM) { a.ux[o] = 0.f; a.uy[o] = 0.f; a.uz[o] = 0.f; a.rho[o] = 0.f; }
        if (PLOT) a.plot[o] = make_float4(0.f, 0.f, 0.f, 0.f);
        if (a.probe && o == a.probe_o) *a.probe = make_float4(0.f, 0.f, 0.f, 0.f);
        return;
    }
    if (MODE == MODE_NATIVE && (fl & CELL_WALL)) {
        if (MOM) { a.ux[o] = 0.f; a.uy[o] = 0.f; a.uz[o] = 0.f; a.rho[o] = 0.f; }
        if (a.probe && o == a.probe_o) *a.probe = make_float4(0.f, 0.f, 0.f, 0.f);
        return;
    }

    float g[19];
    if (MODE == MODE_NATIVE) {
        pull_native<S>(a, o, n, fl, g);
    } else {
#pragma unroll
        for (int k = 0; k < 19; k++)
            g[k] = ld_stream(a.src.f[k] + o + n.off(-d3_cx(k), -d3_cy(k), -d3_cz(k)));
        if (x == 0 && a.dev == 0)
            d3q19_zou_he_west(g, a.ux_in);
        else if (x == a.W - 1 && a.dev == a.ndev - 1)
            d3q19_zou_he_east(g, a.rho_out);
    }
    float rho, ux, uy, uz;
    if (MODE == MODE_NATIVE) StepArith<S>::moments(g, a, rho, ux, uy, uz);
    else d3q19_moments(g, rho, ux, uy, uz);
    if (MOM) { a.ux[o] = ux; a.uy[o] = uy; a.uz[o] = uz; a.rho[o] = rho; }
    if (PLOT) a.plot[o] = make_float4(ux, uy, uz, rho);
    if (a.probe && o == a.probe_o) *a.probe = make_float4(ux, uy, uz, rho);
    if (MODE == MODE_NATIVE) {
        float ex = ux, ey = uy, ez = uz;
        // velocity-shift forcing (the form of reference src/collision.cu:280-284)
        // and the Shan-Chen shift share one division, 1 / (rho tau_inv)
        if (SC || a.Fx != 0.f || a.Fy != 0.f || a.Fz != 0.f) {
            const float inv_rt = 1.f / (rho * a.tau_inv);
            if (a.Fx != 0.f) ex = __fmaf_rn(a.Fx, inv_rt, ux);
            if (a.Fy != 0.f) ey = __fmaf_rn(a.Fy, inv_rt, uy);
            if (a.Fz != 0.f) ez = __fmaf_rn(a.Fz, inv_rt, uz);
            if (SC) {
                float ps[19];
                ps[0] = a.psi[o];
#pragma unroll
                for (int k = 1; k < 19; k++)
                    ps[k] = __ldg(a.psi + o + n.off(d3_cx(k), d3_cy(k), d3_cz(k)));
                float IFx, IFy, IFz;
                d3q19_sc_sum_native(ps, a.w1, a.w7, IFx, IFy, IFz);
                const float c = (-a.G * ps[0]) * inv_rt;
                ex = __fmaf_rn(c, IFx, ex);
                ey = __fmaf_rn(c, IFy, ey);
                ez = __fmaf_rn(c, IFz, ez);
            }
        }
        StepArith<S>::bgk(g, ex, ey, ez, rho, a, a.tau_inv);
    } else {
        d3q19_bgk(g, ux, uy, uz, rho, a.w0, a.w1, a.w7, a.tau_inv);
    }
    S *const *dst = reinterpret_cast<S *const *>(a.dst.f);
#pragma unroll
    for (int k = 0; k < 19; k++) Store<S>::store_dev(dst[k] + o, g[k]);
}

// Density pass of the Shan-Chen step: psi(rho) of the post-stream density of
// every fluid node (the native moments' sum, so rho is the same float the
// fused kernel computes), 0 at walls.
template <typename S>
__global__ void __launch_bounds__(D3_BLOCK) d3q19_density_kernel(const D3Args a) {
    const Coord3 c(a);
    if (c.x >= a.W) return;
    const int o = c.x + a.W * (c.y + a.H * c.z);
    const uint8_t fl = a.flags[o];
    if (fl & CELL_WALL) {
        a.psi[o] = 0.f;
        return;
    }
    const Nbr3 n(c.x, c.y, c.z, a.W, a.H, a.D);
    float g[19];
    pull_native<S>(a, o, n, fl, g);
    const float rho = StepArith<S>::rho(g, a);
    a.psi[o] = a.psi_form == 0 ? psi_ref(rho) : psi_exp1(rho);
}


// ---------------------------------------------------------------------------
// Reference-exact standalone streaming, src/streaming.cu:84-163: in-place
// swap of f_k(o) and f_opp(k)(o + c_k) for the nine owned slots.  Every
// (node, slot) belongs to exactly one pair and each pair to exactly one
// thread, so the in-place update has no race.
// ---------------------------------------------------------------------------
__global__ void __launch_bounds__(D3_BLOCK) d3q19_stream_swap_kernel(Pop<19> p,
                                                                    const uint8_t *sb, int W,
                                                                    int H, int D) {
    const int x = blockIdx.x * blockDim.x + threadIdx.x;
    const int y = blockIdx.y, z = blockIdx.z;
    if (x >= W) return;
    const int o = x + W * (y + H * z);
    if (sb[o]) return;
    const Nbr3 n(x, y, z, W, H, D);
#pragma unroll
    for (int k = 1; k < 19; k++) {
        if (!d3_pos(k)) continue;
        const int on = o + n.off(d3_cx(k), d3_cy(k), d3_cz(k));
        const float t = p.f[k][o];
        p.f[k][o] = p.f[d3_opp(k)][on];
        p.f[d3_opp(k)][on] = t;
    }
}

// Reference-exact standalone collision, src/collision.cu:357-552.
template <bool PLOT>
__global__ void __launch_bounds__(D3_BLOCK) d3q19_collide_kernel(const D3Args a) {
    const int x = blockIdx.x * blockDim.x + threadIdx.x;
    const int y = blockIdx.y, z = blockIdx.z;
    if (x >= a.W) return;
    const int o = x + a.W * (y + a.H * z);
    if (a.flags[o]) {
        a.ux[o] = 0.f; a.uy[o] = 0.f; a.uz[o] = 0.f; a.rho[o] = 0.f;
        if (PLOT) a.plot[o] = make_float4(0.f, 0.f, 0.f, 0.f);
        return;
    }
    float g[19];
    // local swap back to natural slot order ("bounce-back" in the reference)
#pragma unroll
    for (int k = 0; k < 19; k++) g[k] = a.dst.f[d3_opp(k)][o];
    if (x == 0 && a.dev == 0)
        d3q19_zou_he_west(g, a.ux_in);
    else if (x == a.W - 1 && a.dev == a.ndev - 1)
        d3q19_zou_he_east(g, a.rho_out);
    float rho, ux, uy, uz;
    d3q19_moments(g, rho, ux, uy, uz);
    a.ux[o] = ux; a.uy[o] = uy; a.uz[o] = uz; a.rho[o] = rho;
    if (PLOT) a.plot[o] = make_float4(ux, uy, uz, rho);
    d3q19_bgk(g, ux, uy, uz, rho, a.w0, a.w1, a.w7, a.tau_inv);
#pragma unroll
    for (int k = 0; k < 19; k++) a.dst.f[k][o] = g[k];
}

// x-face pack / unpack, src/get_border.cu:59-98 and src/apply_border.cu:58-97;
// one thread per face node instead of a full-grid launch
__global__ void d3q19_get_border_kernel(CPop<19> p, Pop<10> border, int W, int H, int D) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;  // y + z*H
    if (i >= H * D) return;
    const int y = i % H, z = i / H;
    const int oe = (W - 1) + W * (y + H * z), ow = W * (y + H * z);
    border.f[0][i] = p.f[1][oe];  border.f[1][i] = p.f[7][oe];  border.f[2][i] = p.f[8][oe];
    border.f[3][i] = p.f[9][oe];  border.f[4][i] = p.f[10][oe];
    border.f[5][i] = p.f[2][ow];  border.f[6][i] = p.f[11][ow]; border.f[7][i] = p.f[12][ow];
    border.f[8][i] = p.f[13][ow]; border.f[9][i] = p.f[14][ow];
}

__global__ void d3q19_apply_border_kernel(Pop<19> p, CPop<10> nb, int W, int H, int D) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= H * D) return;
    const int y = i % H, z = i / H;
    const int oe = (W - 1) + W * (y + H * z), ow = W * (y + H * z);
    p.f[2][ow] = nb.f[5][i];  p.f[11][ow] = nb.f[6][i]; p.f[12][ow] = nb.f[7][i];
    p.f[13][ow] = nb.f[8][i]; p.f[14][ow] = nb.f[9][i];
    p.f[1][oe] = nb.f[0][i];  p.f[7][oe] = nb.f[1][i];  p.f[8][oe] = nb.f[2][i];
    p.f[9][oe] = nb.f[3][i];  p.f[10][oe] = nb.f[4][i];
}

// equilibrium from moment fields (BGK with tau_inv = 1 from zero populations
// yields the equilibrium in the BGK's own operation order)
__global__ void d3q19_equilibrium_kernel(Pop<19> p, const float *rho, const float *ux,
                                         const float *uy, const float *uz, int N, float w0,
                                         float w1, float w7) {
    const int o = blockIdx.x * blockDim.x + threadIdx.x;
    if (o >= N) return;
    float g[19];
#pragma unroll
    for (int k = 0; k < 19; k++) g[k] = 0.f;
    d3q19_bgk(g, ux ? ux[o] : 0.f, uy ? uy[o] : 0.f, uz ? uz[o] : 0.f, rho ? rho[o] : 1.f, w0,
              w1, w7, 1.f);
#pragma unroll
    for (int k = 0; k < 19; k++) p.f[k][o] = g[k];
}

struct Wr19 {
    float v[19];
};

// the same equilibrium, stored in 16-bit deviation form
template <typename S>
__global__ void d3q19_equilibrium_store_kernel(Pop<19> p, const float *rho, const float *ux,
                                               const float *uy, const float *uz, int N,
                                               float w0, float w1, float w7, Wr19 wr) {
    const int o = blockIdx.x * blockDim.x + threadIdx.x;
    if (o >= N) return;
    float g[19];
#pragma unroll
    for (int k = 0; k < 19; k++) g[k] = 0.f;
    d3q19_bgk(g, ux ? ux[o] : 0.f, uy ? uy[o] : 0.f, uz ? uz[o] : 0.f, rho ? rho[o] : 1.f, w0,
              w1, w7, 1.f);
    S *const *dst = reinterpret_cast<S *const *>(p.f);
#pragma unroll
    for (int k = 0; k < 19; k++) Store<S>::store(dst[k] + o, g[k], wr.v[k]);
}

cudaError_t launch_d3q19_equilibrium_storage(const Pop<19> &p, const float *rho, const float *ux,
                                             const float *uy, const float *uz, int N, float w0,
                                             float w1, float w7, const float *wr, int storage,
                                             cudaStream_t s) {
    Wr19 w;
    for (int k = 0; k < 19; k++) w.v[k] = wr[k];
    const unsigned blocks = (unsigned)((N + 255) / 256);
    if (storage == 1)
        d3q19_equilibrium_store_kernel<__half><<<blocks, 256, 0, s>>>(p, rho, ux, uy, uz, N, w0,
                                                                      w1, w7, w);
    else if (storage == 2)
        d3q19_equilibrium_store_kernel<__nv_bfloat16><<<blocks, 256, 0, s>>>(p, rho, ux, uy, uz,
                                                                             N, w0, w1, w7, w);
    else
        return cudaErrorInvalidValue;
    return cudaGetLastError();
}

template <typename S>
__global__ void to_storage_kernel(const float *src, S *dst, long n, float wr) {
    const long i = blockIdx.x * (long)blockDim.x + threadIdx.x;
    if (i < n) Store<S>::store(dst + i, src[i], wr);
}
template <typename S>
__global__ void from_storage_kernel(const S *src, float *dst, long n, float wr) {
    const long i = blockIdx.x * (long)blockDim.x + threadIdx.x;
    if (i < n) dst[i] = Store<S>::load(src + i, wr);
}

// ---------------------------------------------------------------- launchers
static dim3 grid_of(int W, int H, int D) { return dim3((W + D3_BLOCK - 1) / D3_BLOCK, H, D); }

cudaError_t launch_d3q19_fused(const D3Args &a, int mode, bool mom, bool plot, cudaStream_t s) {
    const dim3 g = grid_of(a.W, a.H, a.D), b(D3_BLOCK);
#define LB_D3_CASE(M, MO, PL)                                                    \
    if (mode == M && mom == MO && plot == PL) {                                  \
        d3q19_fused_kernel<M, MO, PL, float, false><<<g, b, 0, s>>>(a);         \
        return cudaGetLastError();                                               \
    }
    LB_D3_CASE(MODE_REF, true, true)
    LB_D3_CASE(MODE_REF, true, false)
    LB_D3_CASE(MODE_REF, false, false)
    LB_D3_CASE(MODE_NATIVE, true, false)
    LB_D3_CASE(MODE_NATIVE, false, false)
#undef LB_D3_CASE
    return cudaErrorInvalidValue;
}

template <typename S>
static cudaError_t native_launch(const D3Args &a, bool mom, bool sc, cudaStream_t s) {
    const dim3 g = grid_of(a.W, a.H, a.D), b(D3_BLOCK);
    if (sc) {
        d3q19_density_kernel<S><<<g, b, 0, s>>>(a);
        cudaError_t e = cudaGetLastError();
        if (e != cudaSuccess) return e;
        if (mom) d3q19_fused_kernel<MODE_NATIVE, true, false, S, true><<<g, b, 0, s>>>(a);
        else d3q19_fused_kernel<MODE_NATIVE, false, false, S, true><<<g, b, 0, s>>>(a);
    } else {
        if (mom) d3q19_fused_kernel<MODE_NATIVE, true, false, S, false><<<g, b, 0, s>>>(a);
        else d3q19_fused_kernel<MODE_NATIVE, false, false, S, false><<<g, b, 0, s>>>(a);
    }
    return cudaGetLastError();
}

template <typename S>
static cudaError_t native_planes(const D3Args &a0, bool mom, int z_lo, int z_skip, int nplanes,
                                 cudaStream_t s) {
    D3Args a = a0;
    a.reverse = 0;
    a.z_lo = z_lo;
    a.z_skip = z_skip;
    const dim3 g((a.W + D3_BLOCK - 1) / D3_BLOCK, a.H, nplanes), b(D3_BLOCK);
    if (mom) d3q19_fused_kernel<MODE_NATIVE, true, false, S, false><<<g, b, 0, s>>>(a);
    else d3q19_fused_kernel<MODE_NATIVE, false, false, S, false><<<g, b, 0, s>>>(a);
    return cudaGetLastError();
}

cudaError_t launch_d3q19_native_planes(const D3Args &a, int storage, bool mom, int z_lo,
                                       int z_skip, int nplanes, cudaStream_t s) {
    if (nplanes <= 0) return cudaSuccess;
    switch (storage) {
    case 0: return native_planes<float>(a, mom, z_lo, z_skip, nplanes, s);
    case 1: return native_planes<__half>(a, mom, z_lo, z_skip, nplanes, s);
    case 2: return native_planes<__nv_bfloat16>(a, mom, z_lo, z_skip, nplanes, s);
    }
    return cudaErrorInvalidValue;
}

// ---------------------------------------------------------------------------
// Plane copies of the z-slab exchange: up to 10 planes (the 5 populations
// crossing each of a slab's two faces) in one launch; blockIdx.y picks the
// plane, the x blocks stride through its bytes.  The pointers may lie on
// another device the calling one reaches (peer loads or stores).
// ---------------------------------------------------------------------------
constexpr int PC_MAX = 10;
struct PlaneCopyArgs {
    const char *src[PC_MAX];
    char *dst[PC_MAX];
    long n;  // elements of T per plane
};

template <typename T>
__global__ void __launch_bounds__(256) plane_copy_kernel(const PlaneCopyArgs p) {
    const T *src = reinterpret_cast<const T *>(p.src[blockIdx.y]);
    T *dst = reinterpret_cast<T *>(p.dst[blockIdx.y]);
    for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < p.n;
         i += (long)gridDim.x * blockDim.x)
        dst[i] = src[i];
}

cudaError_t launch_plane_copy(const void *const *src, void *const *dst, int n, long bytes,
                              cudaStream_t s) {
    if (n <= 0 || bytes <= 0) return cudaSuccess;
    if (n > PC_MAX) return cudaErrorInvalidValue;
    PlaneCopyArgs p{};
    uintptr_t align = (uintptr_t)bytes;
    for (int i = 0; i < n; i++) {
        p.src[i] = static_cast<const char *>(src[i]);
        p.dst[i] = static_cast<char *>(dst[i]);
        align |= (uintptr_t)src[i] | (uintptr_t)dst[i];
    }
    const int w = (align & 15) == 0 ? 16 : (align & 3) == 0 ? 4 : (align & 1) == 0 ? 2 : 1;
    p.n = bytes / w;
    const long per = (p.n + 255) / 256;
    const dim3 g((unsigned)(per < 64 ? (per > 0 ? per : 1) : 64), n);
    switch (w) {
    case 16: plane_copy_kernel<uint4><<<g, 256, 0, s>>>(p); break;
    case 4: plane_copy_kernel<uint32_t><<<g, 256, 0, s>>>(p); break;
    case 2: plane_copy_kernel<uint16_t><<<g, 256, 0, s>>>(p); break;
    default: plane_copy_kernel<uint8_t><<<g, 256, 0, s>>>(p); break;
    }
    return cudaGetLastError();
}

cudaError_t launch_d3q19_native(const D3Args &a, int storage, bool mom, bool sc, cudaStream_t s) {
    switch (storage) {
    case 0: return native_launch<float>(a, mom, sc, s);
    case 1: return native_launch<__half>(a, mom, sc, s);
    case 2: return native_launch<__nv_bfloat16>(a, mom, sc, s);
    }
    return cudaErrorInvalidValue;
}

cudaError_t launch_to_storage(const float *src, void *dst, long n, float wr, int storage,
                              cudaStream_t s) {
    const unsigned blocks = (unsigned)((n + 255) / 256);
    if (storage == 1) to_storage_kernel<__half><<<blocks, 256, 0, s>>>(src, (__half *)dst, n, wr);
    else if (storage == 2)
        to_storage_kernel<__nv_bfloat16><<<blocks, 256, 0, s>>>(src, (__nv_bfloat16 *)dst, n, wr);
    else to_storage_kernel<float><<<blocks, 256, 0, s>>>(src, (float *)dst, n, wr);
    return cudaGetLastError();
}

cudaError_t launch_from_storage(const void *src, float *dst, long n, float wr, int storage,
                                cudaStream_t s) {
    const unsigned blocks = (unsigned)((n + 255) / 256);
    if (storage == 1)
        from_storage_kernel<__half><<<blocks, 256, 0, s>>>((const __half *)src, dst, n, wr);
    else if (storage == 2)
        from_storage_kernel<__nv_bfloat16><<<blocks, 256, 0, s>>>((const __nv_bfloat16 *)src,
                                                                  dst, n, wr);
    else from_storage_kernel<float><<<blocks, 256, 0, s>>>((const float *)src, dst, n, wr);
    return cudaGetLastError();
}

cudaError_t launch_d3q19_stream_swap(const Pop<19> &p, const uint8_t *sb, int W, int H, int D,
                                     cudaStream_t s) {
    d3q19_stream_swap_kernel<<<grid_of(W, H, D), D3_BLOCK, 0, s>>>(p, sb, W, H, D);
    return cudaGetLastError();
}

cudaError_t launch_d3q19_collide(const D3Args &a, bool plot, cudaStream_t s) {
    if (plot)
        d3q19_collide_kernel<true><<<grid_of(a.W, a.H, a.D), D3_BLOCK, 0, s>>>(a);
    else
        d3q19_collide_kernel<false><<<grid_of(a.W, a.H, a.D), D3_BLOCK, 0, s>>>(a);
    return cudaGetLastError();
}

cudaError_t launch_d3q19_get_border(const CPop<19> &p, const Pop<10> &b, int W, int H, int D,
                                    cudaStream_t s) {
    const int n = H * D;
    d3q19_get_border_kernel<<<(n + 255) / 256, 256, 0, s>>>(p, b, W, H, D);
    return cudaGetLastError();
}

cudaError_t launch_d3q19_apply_border(const Pop<19> &p, const CPop<10> &nb, int W, int H, int D,
                                      cudaStream_t s) {
    const int n = H * D;
    d3q19_apply_border_kernel<<<(n + 255) / 256, 256, 0, s>>>(p, nb, W, H, D);
    return cudaGetLastError();
}

cudaError_t launch_d3q19_equilibrium(const Pop<19> &p, const float *rho, const float *ux,
                                     const float *uy, const float *uz, int N, float w0, float w1,
                                     float w7, cudaStream_t s) {
    d3q19_equilibrium_kernel<<<(N + 255) / 256, 256, 0, s>>>(p, rho, ux, uy, uz, N, w0, w1, w7);
    return cudaGetLastError();
}

}  // namespace lb
