// lb_d2q9.cu -- D2Q9 kernels: fused pull-stream + collide (first pass), the
// Shan-Chen force step (second pass), and the reference-exact standalone
// streaming / collision / border kernels behind the drop-in entry points.
//
// Layout: one float array per population, node o = x + W*y, row y+1 is
// physical -y (reference src/streaming.cu:44-54).
#include <algorithm>

#include "lb_kernels.cuh"

namespace lb {

struct Nbr2 {
    int xm, xp, rm, rp;  // offsets to x-1, x+1, row-1, row+1 (periodic)
    __device__ __forceinline__ Nbr2(int x, int y, int W, int H) {
        xm = x == 0 ? W - 1 : -1;
        xp = x == W - 1 ? -(W - 1) : 1;
        rm = y == 0 ? (H - 1) * W : -W;
        rp = y == H - 1 ? -(H - 1) * W : W;
    }
    __device__ __forceinline__ int off(int cx, int cr) const {
        return (cx > 0 ? xp : (cx < 0 ? xm : 0)) + (cr > 0 ? rp : (cr < 0 ? rm : 0));
    }
};

// ---------------------------------------------------------------------------
// Fused first pass (see lb_d3q19.cu for the pull / wall conventions).  With
// SC the pass ends like the reference's first kernel for G != 0
// (src/collision.cu:290-296): psi, u_eq and the moments are stored and the
// populations are stored post-stream and unrelaxed; the Shan-Chen pass then
// relaxes them in place.
// ---------------------------------------------------------------------------
// PDL: launched as a programmatic dependent of the previous step, the grid
// may start while that step drains; it waits for it (griddepcontrol.wait,
// which also makes that step's stores visible) before touching memory.
template <int MODE, bool MOM, bool PLOT, bool SC, bool PDL = false>
__global__ void __launch_bounds__(D2_BLOCK) d2q9_fused_kernel(const D2Args a) {
    if (PDL) {
        asm volatile("griddepcontrol.wait;" ::: "memory");
        asm volatile("griddepcontrol.launch_dependents;" ::: "memory");
    }
    const int bx = a.reverse ? gridDim.x - 1 - blockIdx.x : blockIdx.x;
    const int x = bx * blockDim.x + threadIdx.x;
    const int y = a.reverse ? a.H - 1 - (int)blockIdx.y : (int)blockIdx.y;
    if (x >= a.W) return;
    const int o = x + a.W * y;
    const uint8_t fl = a.flags[o];
    const Nbr2 n(x, y, a.W, a.H);

    if (fl & CELL_WALL) {
        if (MODE == MODE_REF) {
            const bool sb_self = a.sb[o] != 0;
#pragma unroll
            for (int m = 0; m < 9; m++) {
                float v;
                if (m == 0) {
                    v = ld_stream(a.src.f[0] + o);
                } else {
                    const int on = o + n.off(d2_cx(m), d2_cr(m));
                    const bool resp_sb = d2_pos(m) ? sb_self : (a.sb[on] != 0);
                    v = resp_sb ? ld_stream(a.src.f[m] + o) : ld_stream(a.src.f[d2_opp(m)] + on);
                }
                a.dst.f[m][o] = v;
            }
            if (PLOT) a.plot[o] = make_float4(0.f, 0.f, 0.f, 0.f);
        } else if (SC) {
            a.psi[o] = 0.f;
        }
        if (MOM) { a.ux[o] = 0.f; a.uy[o] = 0.f; a.rho[o] = 0.f; }
        if (a.probe && o == a.probe_o) *a.probe = make_float4(0.f, 0.f, 0.f, 0.f);
        return;
    }

    float g[9];
    if (MODE == MODE_NATIVE && (fl & CELL_NEAR_WALL)) {
#pragma unroll
        for (int k = 0; k < 9; k++) {
            const int up = o + n.off(-d2_cx(k), -d2_cr(k));
            const uint8_t fu = k == 0 ? 0 : a.flags[up];
            if (fu & CELL_WALL) {
                const float v = ld_stream(a.src.f[d2_opp(k)] + o);
                g[k] = (fu & CELL_MOVING) ? v - a.corr[d2_opp(k)] : v;
            } else {
                g[k] = ld_stream(a.src.f[k] + up);
            }
        }
    } else {
#pragma unroll
        for (int k = 0; k < 9; k++) g[k] = ld_stream(a.src.f[k] + o + n.off(-d2_cx(k), -d2_cr(k)));
    }
    if (MODE == MODE_NATIVE) {
        // native arithmetic (d2q9_*_native); with Shan-Chen the pass stores
        // psi, u_eq and the unrelaxed populations for the Shan-Chen pass
        float rho, ux, uy;
        if (!SC) {
            d2q9_collide_native(g, a.Fx, a.Fy, a.w0, a.w1, a.w5, a.tau_inv, rho, ux, uy);
            if (PLOT) a.plot[o] = make_float4(ux, uy, 0.f, rho);
        } else {
            d2q9_moments_native(g, rho, ux, uy);
            float ex = ux, ey = uy;
            if (a.Fx != 0.f || a.Fy != 0.f) {
                const float inv_rt = 1.f / (rho * a.tau_inv);
                if (a.Fx != 0.f) ex = __fmaf_rn(a.Fx, inv_rt, ux);
                if (a.Fy != 0.f) ey = __fmaf_rn(a.Fy, inv_rt, uy);
            }
            a.psi[o] = a.psi_form == 0 ? psi_ref(rho) : psi_exp1(rho);
            a.ueq_x[o] = ex;
            a.ueq_y[o] = ey;
        }
        if (MOM) { a.ux[o] = ux; a.uy[o] = uy; a.rho[o] = rho; }
        if (a.probe && o == a.probe_o) *a.probe = make_float4(ux, uy, 0.f, rho);
#pragma unroll
        for (int k = 0; k < 9; k++) a.dst.f[k][o] = g[k];
        return;
    }
    if (MODE == MODE_REF) {
        if (x == 0 && a.dev == 0)
            d2q9_zou_he_west(g, a.ux_in);
        else if (x == a.W - 1 && a.dev == a.ndev - 1)
            d2q9_zou_he_east(g, a.rho_out);
    }
    float rho, ux, uy;
    d2q9_moments(g, rho, ux, uy);
    float ex = ux, ey = uy;
    if (a.Fx != 0.f) ex = ux + a.Fx / (rho * a.tau_inv);
    if (a.Fy != 0.f) ey = uy + a.Fy / (rho * a.tau_inv);
    if (MOM) { a.ux[o] = ux; a.uy[o] = uy; a.rho[o] = rho; }
    if (a.probe && o == a.probe_o) *a.probe = make_float4(ux, uy, 0.f, rho);
    if (SC) {
        a.psi[o] = (MODE == MODE_REF || a.psi_form == 0) ? psi_ref(rho) : psi_exp1(rho);
        a.ueq_x[o] = ex;
        a.ueq_y[o] = ey;
    } else {
        if (PLOT) a.plot[o] = make_float4(ux, uy, 0.f, rho);
        d2q9_bgk(g, ex, ey, rho, a.w0, a.w1, a.w5, a.tau_inv);
    }
#pragma unroll
    for (int k = 0; k < 9; k++) a.dst.f[k][o] = g[k];
}

// ---------------------------------------------------------------------------
// Shan-Chen force step, reference src/collision.cu:35-166: interaction force
// -G psi(x) sum_k w_k psi(x + c_k) c_k and adhesion -G_ads psi(x) sum_k w_k
// s(x + c_k) c_k shift u_eq, then BGK in place.  Reference mode: the
// reference's accumulation order; native mode: d2q9_sc_shift_native, one
// division and d2q9_bgk_native.  psi and the wall flags of the 3x3 stencil
// come through L1.
// ---------------------------------------------------------------------------
// adhesion sums s = sum_k w_k [x + c_k is a wall] c_k in the reference's
// order (src/collision.cu:105-140); m1..m8 are the stencil's node indices
__device__ __forceinline__ void d2q9_adhesion_sums(const uint8_t *s, int m1, int m2, int m3,
                                                   int m4, int m5, int m6, int m7, int m8,
                                                   float w1, float w5, float &Fsx, float &Fsy) {
    Fsx = 0.f;
    Fsy = 0.f;
    if (s[m1] & CELL_WALL) Fsx = Fsx + w1;
    if (s[m2] & CELL_WALL) Fsy = Fsy - w1;
    if (s[m3] & CELL_WALL) Fsx = Fsx - w1;
    if (s[m4] & CELL_WALL) Fsy = Fsy + w1;
    if (s[m5] & CELL_WALL) { Fsx = Fsx + w5; Fsy = Fsy - w5; }
    if (s[m6] & CELL_WALL) { Fsx = Fsx - w5; Fsy = Fsy - w5; }
    if (s[m7] & CELL_WALL) { Fsx = Fsx - w5; Fsy = Fsy + w5; }
    if (s[m8] & CELL_WALL) { Fsx = Fsx + w5; Fsy = Fsy + w5; }
}

template <int MODE, bool PLOT>
__global__ void __launch_bounds__(D2_BLOCK) d2q9_sc_kernel(const D2Args a) {
    const int x = blockIdx.x * blockDim.x + threadIdx.x;
    const int y = blockIdx.y;
    if (x >= a.W) return;
    const int o = x + a.W * y;
    if (a.flags[o] & CELL_WALL) return;
    const int W = a.W, H = a.H;
    const int xn = x > 0 ? x - 1 : W - 1, xp = x < W - 1 ? x + 1 : 0;
    const int yn = y > 0 ? y - 1 : H - 1, yp = y < H - 1 ? y + 1 : 0;
    const int m1 = y * W + xp, m2 = yp * W + x, m3 = y * W + xn, m4 = yn * W + x;
    const int m5 = yp * W + xp, m6 = yp * W + xn, m7 = yn * W + xn, m8 = yn * W + xp;
    const float *psi = a.psi;
    const float w1 = a.w1, w5 = a.w5;
    const float ps[9] = {psi[o],           __ldg(psi + m1), __ldg(psi + m2),
                         __ldg(psi + m3),  __ldg(psi + m4), __ldg(psi + m5),
                         __ldg(psi + m6),  __ldg(psi + m7), __ldg(psi + m8)};
    const float p0 = ps[0], rho = a.rho[o];
    float ex = a.ueq_x[o], ey = a.ueq_y[o];
    if (MODE == MODE_NATIVE) {
        // one division 1/(tau_inv rho) for the interaction and the adhesion
        const float inv_rt = 1.f / (a.tau_inv * rho);
        d2q9_sc_shift_native(ps, w1, w5, a.G, inv_rt, ex, ey);
        if (a.Gads != 0.f) {
            float Fsx, Fsy;
            d2q9_adhesion_sums(a.flags, m1, m2, m3, m4, m5, m6, m7, m8, w1, w5, Fsx, Fsy);
            const float c = (-a.Gads * p0) * inv_rt;
            ex = __fmaf_rn(c, Fsx, ex);
            ey = __fmaf_rn(c, Fsy, ey);
        }
        if (PLOT) a.plot[o] = make_float4(a.ux[o], a.uy[o], 0.f, rho);
        float g[9];
#pragma unroll
        for (int k = 0; k < 9; k++) g[k] = a.dst.f[k][o];
        d2q9_bgk_native(g, ex, ey, rho, a.w0, a.w1, a.w5, a.tau_inv);
#pragma unroll
        for (int k = 0; k < 9; k++) a.dst.f[k][o] = g[k];
        return;
    }
    d2q9_sc_shift(ps, w1, w5, a.G, a.tau_inv, rho, ex, ey);
    if (a.Gads != 0.f) {
        float Fsx, Fsy;
        d2q9_adhesion_sums(a.flags, m1, m2, m3, m4, m5, m6, m7, m8, w1, w5, Fsx, Fsy);
        Fsx = -a.Gads * p0 * Fsx;
        Fsy = -a.Gads * p0 * Fsy;
        ex = ex + (Fsx / (a.tau_inv * rho));
        ey = ey + (Fsy / (a.tau_inv * rho));
    }
    if (PLOT) a.plot[o] = make_float4(a.ux[o], a.uy[o], 0.f, rho);
    float g[9];
#pragma unroll
    for (int k = 0; k < 9; k++) g[k] = a.dst.f[k][o];
    d2q9_bgk(g, ex, ey, rho, a.w0, a.w1, a.w5, a.tau_inv);
#pragma unroll
    for (int k = 0; k < 9; k++) a.dst.f[k][o] = g[k];
}

// Reference-exact standalone streaming, src/streaming.cu:24-74.
__global__ void __launch_bounds__(D2_BLOCK) d2q9_stream_swap_kernel(Pop<9> p, const uint8_t *sb,
                                                                   int W, int H) {
    const int x = blockIdx.x * blockDim.x + threadIdx.x;
    const int y = blockIdx.y;
    if (x >= W) return;
    const int o = x + W * y;
    if (sb[o]) return;
    const Nbr2 n(x, y, W, H);
#pragma unroll
    for (int k = 1; k < 9; k++) {
        if (!d2_pos(k)) continue;
        const int on = o + n.off(d2_cx(k), d2_cr(k));
        const float t = p.f[k][o];
        p.f[k][o] = p.f[d2_opp(k)][on];
        p.f[d2_opp(k)][on] = t;
    }
}

// Reference-exact standalone first collision pass, src/collision.cu:168-341
// (the Shan-Chen pass is d2q9_sc_kernel, launched after it when G < 0).
template <bool PLOT>
__global__ void __launch_bounds__(D2_BLOCK) d2q9_collide_kernel(const D2Args a) {
    const int x = blockIdx.x * blockDim.x + threadIdx.x;
    const int y = blockIdx.y;
    if (x >= a.W) return;
    const int o = x + a.W * y;
    if (a.flags[o]) {
        if (PLOT) a.plot[o] = make_float4(0.f, 0.f, 0.f, 0.f);
        a.ux[o] = 0.f; a.uy[o] = 0.f; a.rho[o] = 0.f;
        return;
    }
    float g[9];
#pragma unroll
    for (int k = 0; k < 9; k++) g[k] = a.dst.f[d2_opp(k)][o];
    if (x == 0 && a.dev == 0)
        d2q9_zou_he_west(g, a.ux_in);
    else if (x == a.W - 1 && a.dev == a.ndev - 1)
        d2q9_zou_he_east(g, a.rho_out);
    float rho, ux, uy;
    d2q9_moments(g, rho, ux, uy);
    float ex = ux, ey = uy;
    if (a.Fx != 0.f) ex = ux + a.Fx / (rho * a.tau_inv);
    if (a.Fy != 0.f) ey = uy + a.Fy / (rho * a.tau_inv);
    a.ux[o] = ux; a.uy[o] = uy; a.rho[o] = rho;
    if (a.G != 0.f) {
        a.psi[o] = psi_ref(rho);
        a.ueq_x[o] = ex;
        a.ueq_y[o] = ey;
    } else {
        if (PLOT) a.plot[o] = make_float4(ux, uy, 0.f, rho);
        d2q9_bgk(g, ex, ey, rho, a.w0, a.w1, a.w5, a.tau_inv);
    }
#pragma unroll
    for (int k = 0; k < 9; k++) a.dst.f[k][o] = g[k];
}

__global__ void d2q9_get_border_kernel(CPop<9> p, Pop<6> b, int W, int H) {
    const int y = blockIdx.x * blockDim.x + threadIdx.x;
    if (y >= H) return;
    const int oe = (W - 1) + W * y, ow = W * y;
    b.f[0][y] = p.f[1][oe]; b.f[1][y] = p.f[5][oe]; b.f[2][y] = p.f[8][oe];
    b.f[3][y] = p.f[3][ow]; b.f[4][y] = p.f[6][ow]; b.f[5][y] = p.f[7][ow];
}

__global__ void d2q9_apply_border_kernel(Pop<9> p, CPop<6> nb, int W, int H) {
    const int y = blockIdx.x * blockDim.x + threadIdx.x;
    if (y >= H) return;
    const int oe = (W - 1) + W * y, ow = W * y;
    p.f[3][ow] = nb.f[3][y]; p.f[7][ow] = nb.f[5][y]; p.f[6][ow] = nb.f[4][y];
    p.f[1][oe] = nb.f[0][y]; p.f[8][oe] = nb.f[2][y]; p.f[5][oe] = nb.f[1][y];
}

__global__ void d2q9_equilibrium_kernel(Pop<9> p, const float *rho, const float *ux,
                                        const float *uy, int N, float w0, float w1, float w5) {
    const int o = blockIdx.x * blockDim.x + threadIdx.x;
    if (o >= N) return;
    float g[9];
#pragma unroll
    for (int k = 0; k < 9; k++) g[k] = 0.f;
    d2q9_bgk(g, ux ? ux[o] : 0.f, uy ? uy[o] : 0.f, rho ? rho[o] : 1.f, w0, w1, w5, 1.f);
#pragma unroll
    for (int k = 0; k < 9; k++) p.f[k][o] = g[k];
}

// ---------------------------------------------------------------- launchers
static dim3 grid2(int W, int H) { return dim3((W + D2_BLOCK - 1) / D2_BLOCK, H); }

cudaError_t launch_d2q9_fused(const D2Args &a, int mode, bool mom, bool plot, cudaStream_t s) {
    const dim3 g = grid2(a.W, a.H), b(D2_BLOCK);
    // the Shan-Chen pass runs for G < 0 in reference mode (src/collision.cu:352)
    // and for any G != 0 in native mode
    const bool sc = a.G != 0.f;
    const bool sc_pass = mode == MODE_REF ? a.G < 0.f : sc;
    if (sc) mom = true;  // the second pass reads rho
#define LB_D2_CASE(M, MO, PL, SC)                                                 \
    if (mode == M && mom == MO && plot == PL && sc == SC) {                       \
        d2q9_fused_kernel<M, MO, PL, SC><<<g, b, 0, s>>>(a);                     \
        ok = true;                                                                \
    }
    bool ok = false;
    LB_D2_CASE(MODE_REF, true, true, false)
    LB_D2_CASE(MODE_REF, true, false, false)
    LB_D2_CASE(MODE_REF, false, false, false)
    LB_D2_CASE(MODE_REF, true, true, true)
    LB_D2_CASE(MODE_REF, true, false, true)
    LB_D2_CASE(MODE_NATIVE, true, false, false)
    LB_D2_CASE(MODE_NATIVE, false, false, false)
    LB_D2_CASE(MODE_NATIVE, true, true, false)
    LB_D2_CASE(MODE_NATIVE, true, false, true)
    LB_D2_CASE(MODE_NATIVE, true, true, true)
#undef LB_D2_CASE
    if (!ok) return cudaErrorInvalidValue;
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess || !sc_pass) return e;
    if (mode == MODE_REF) {
        if (plot) d2q9_sc_kernel<MODE_REF, true><<<g, b, 0, s>>>(a);
        else d2q9_sc_kernel<MODE_REF, false><<<g, b, 0, s>>>(a);
    } else {
        if (plot) d2q9_sc_kernel<MODE_NATIVE, true><<<g, b, 0, s>>>(a);
        else d2q9_sc_kernel<MODE_NATIVE, false><<<g, b, 0, s>>>(a);
    }
    return cudaGetLastError();
}

cudaError_t launch_d2q9_fused_pdl(const D2Args &a, int mode, bool mom, cudaStream_t s) {
    if (a.G != 0.f) return cudaErrorInvalidValue;  // no Shan-Chen pass here
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = grid2(a.W, a.H);
    cfg.blockDim = dim3(D2_BLOCK);
    cfg.stream = s;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
    attr[0].val.programmaticStreamSerializationAllowed = 1;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    if (mode == MODE_REF)
        return mom ? cudaLaunchKernelEx(&cfg, d2q9_fused_kernel<MODE_REF, true, false, false, true>, a)
                   : cudaLaunchKernelEx(&cfg, d2q9_fused_kernel<MODE_REF, false, false, false, true>, a);
    return mom ? cudaLaunchKernelEx(&cfg, d2q9_fused_kernel<MODE_NATIVE, true, false, false, true>, a)
               : cudaLaunchKernelEx(&cfg, d2q9_fused_kernel<MODE_NATIVE, false, false, false, true>, a);
}

cudaError_t launch_d2q9_stream_swap(const Pop<9> &p, const uint8_t *sb, int W, int H,
                                    cudaStream_t s) {
    d2q9_stream_swap_kernel<<<grid2(W, H), D2_BLOCK, 0, s>>>(p, sb, W, H);
    return cudaGetLastError();
}

cudaError_t launch_d2q9_collide(const D2Args &a, bool plot, cudaStream_t s) {
    const dim3 g = grid2(a.W, a.H), b(D2_BLOCK);
    if (plot) d2q9_collide_kernel<true><<<g, b, 0, s>>>(a);
    else d2q9_collide_kernel<false><<<g, b, 0, s>>>(a);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess || !(a.G < 0.f)) return e;
    if (plot) d2q9_sc_kernel<MODE_REF, true><<<g, b, 0, s>>>(a);
    else d2q9_sc_kernel<MODE_REF, false><<<g, b, 0, s>>>(a);
    return cudaGetLastError();
}

cudaError_t launch_d2q9_get_border(const CPop<9> &p, const Pop<6> &b, int W, int H,
                                   cudaStream_t s) {
    d2q9_get_border_kernel<<<(H + 255) / 256, 256, 0, s>>>(p, b, W, H);
    return cudaGetLastError();
}

cudaError_t launch_d2q9_apply_border(const Pop<9> &p, const CPop<6> &nb, int W, int H,
                                     cudaStream_t s) {
    d2q9_apply_border_kernel<<<(H + 255) / 256, 256, 0, s>>>(p, nb, W, H);
    return cudaGetLastError();
}

cudaError_t launch_d2q9_equilibrium(const Pop<9> &p, const float *rho, const float *ux,
                                    const float *uy, int N, float w0, float w1, float w5,
                                    cudaStream_t s) {
    d2q9_equilibrium_kernel<<<(N + 255) / 256, 256, 0, s>>>(p, rho, ux, uy, N, w0, w1, w5);
    return cudaGetLastError();
}

}  // namespace lb
