// lb_common.cuh -- lattice tables, pointer bundles and the per-node math that
// every lattice Boltzmann kernel of the library shares.
//
// The library is compiled with -fmad=false: each float operation below rounds
// once, in the order written, which is the order of the reference kernels
// (reference src/collision.cu).  Together with IEEE division (nvcc's default
// -prec-div=true) this makes the GPU results bit-identical to the reference's
// float arithmetic, which is what the parity tests check.
#pragma once

#include <cuda_bf16.h>
#include <cuda_fp16.h>
#include <cuda_runtime.h>
#include <stdint.h>

namespace lb {

// ---------------------------------------------------------------- D3Q19 table
// velocity set and order of the reference, src/collision.cu:463-478 and the
// streaming pairs of src/streaming.cu:116-161
__host__ __device__ constexpr int d3_cx(int k) {
    return (k == 1 || (k >= 7 && k <= 10)) ? 1 : ((k == 2 || (k >= 11 && k <= 14)) ? -1 : 0);
}
__host__ __device__ constexpr int d3_cy(int k) {
    return (k == 3 || k == 7 || k == 11 || k == 15 || k == 16) ? 1
         : ((k == 4 || k == 8 || k == 12 || k == 17 || k == 18) ? -1 : 0);
}
__host__ __device__ constexpr int d3_cz(int k) {
    return (k == 5 || k == 9 || k == 13 || k == 15 || k == 17) ? 1
         : ((k == 6 || k == 10 || k == 14 || k == 16 || k == 18) ? -1 : 0);
}
__host__ __device__ constexpr int d3_opp(int k) {
    return k == 0 ? 0 : (k <= 6 ? ((k & 1) ? k + 1 : k - 1)
         : (k == 7 ? 12 : k == 8 ? 11 : k == 9 ? 14 : k == 10 ? 13 : k == 11 ? 8 : k == 12 ? 7
         : k == 13 ? 10 : k == 14 ? 9 : k == 15 ? 18 : k == 16 ? 17 : k == 17 ? 16 : 15));
}
// slot of a streaming pair owned by the node itself (src/streaming.cu:127-161)
__host__ __device__ constexpr bool d3_pos(int k) {
    return k == 1 || k == 3 || k == 5 || k == 7 || k == 8 || k == 9 || k == 10 || k == 15 ||
           k == 16;
}

// ---------------------------------------------------------------- D2Q9 table
// x offset and ROW offset (physical +y is row-1), src/streaming.cu:44-68
__host__ __device__ constexpr int d2_cx(int k) {
    return (k == 1 || k == 5 || k == 8) ? 1 : ((k == 3 || k == 6 || k == 7) ? -1 : 0);
}
__host__ __device__ constexpr int d2_cr(int k) {
    return (k == 2 || k == 5 || k == 6) ? -1 : ((k == 4 || k == 7 || k == 8) ? 1 : 0);
}
__host__ __device__ constexpr int d2_opp(int k) {
    return k == 0 ? 0 : (k <= 4 ? ((k + 1) % 4 + 1) : ((k - 5 + 2) % 4 + 5));
}
__host__ __device__ constexpr bool d2_pos(int k) { return k == 1 || k == 2 || k == 5 || k == 6; }

static_assert(d2_opp(1) == 3 && d2_opp(2) == 4 && d2_opp(3) == 1 && d2_opp(4) == 2, "d2 opp");
static_assert(d2_opp(5) == 7 && d2_opp(6) == 8 && d2_opp(7) == 5 && d2_opp(8) == 6, "d2 opp");
static_assert(d3_opp(7) == 12 && d3_opp(16) == 17 && d3_opp(5) == 6 && d3_opp(6) == 5, "d3 opp");

// ---------------------------------------------------------------- bundles
template <int Q> struct Pop {
    float *f[Q];
};
template <int Q> struct CPop {
    const float *__restrict__ f[Q];
};

// cell flag bits used by the kernels (the low two are the public LB_CELL_*)
enum : uint8_t {
    CELL_WALL = 0x01,
    CELL_MOVING = 0x02,
    CELL_NEAR_WALL = 0x04,   // fluid cell with at least one wall neighbour
    CELL_SOLID_BOUND = 0x08, // reference mode: wall cell surrounded by walls
};

__device__ __forceinline__ int wrap_dec(int v, int n) { return v == 0 ? n - 1 : v - 1; }
__device__ __forceinline__ int wrap_inc(int v, int n) { return v == n - 1 ? 0 : v + 1; }
__device__ __forceinline__ int wrap_add(int v, int c, int n) {
    return c > 0 ? wrap_inc(v, n) : (c < 0 ? wrap_dec(v, n) : v);
}

// streaming loads: read-only for the kernel's lifetime, touched once per step
__device__ __forceinline__ float ld_stream(const float *p) { return __ldg(p); }

// Population storage.  FP32 stores f_k itself.  The 16-bit forms store the
// deviation d_k = f_k - wr_k from an offset wr_k = w_k * rho_ref (rounded to
// float once on the host), widened to FP32 for the arithmetic.  load/store
// convert between f and the stored form (f = wr_k + widen(h), h =
// narrow_rne(f - wr_k): lb_set/get_populations, equilibrium initialisation).
// The step kernels keep the value their arithmetic works on: f itself in
// FP32, the widened deviation d_k in 16-bit storage (load_dev / store_dev,
// no offset added or taken off; the d3q19_*_dev arithmetic below).
template <typename S> struct Store;
template <> struct Store<float> {
    static constexpr int kind = 0;
    __device__ __forceinline__ static float load(const float *p, float) { return __ldg(p); }
    __device__ __forceinline__ static void store(float *p, float v, float) { *p = v; }
    __device__ __forceinline__ static float load_dev(const float *p) { return __ldg(p); }
    __device__ __forceinline__ static void store_dev(float *p, float v) { *p = v; }
};
template <> struct Store<__half> {
    static constexpr int kind = 1;
    __device__ __forceinline__ static float load(const __half *p, float wr) {
        return wr + __half2float(__ldg(p));
    }
    __device__ __forceinline__ static void store(__half *p, float v, float wr) {
        *p = __float2half_rn(v - wr);
    }
    __device__ __forceinline__ static float load_dev(const __half *p) {
        return __half2float(__ldg(p));
    }
    __device__ __forceinline__ static void store_dev(__half *p, float d) {
        *p = __float2half_rn(d);
    }
};
template <> struct Store<__nv_bfloat16> {
    static constexpr int kind = 2;
    __device__ __forceinline__ static float load(const __nv_bfloat16 *p, float wr) {
        return wr + __bfloat162float(__ldg(p));
    }
    __device__ __forceinline__ static void store(__nv_bfloat16 *p, float v, float wr) {
        *p = __float2bfloat16_rn(v - wr);
    }
    __device__ __forceinline__ static float load_dev(const __nv_bfloat16 *p) {
        return __bfloat162float(__ldg(p));
    }
    __device__ __forceinline__ static void store_dev(__nv_bfloat16 *p, float d) {
        *p = __float2bfloat16_rn(d);
    }
};

// ---------------------------------------------------------------- BGK, D3Q19
// relaxation towards the equilibrium at velocity (ux,uy,uz), reference
// src/collision.cu:480-541 (same association of every term)
__device__ __forceinline__ void d3q19_bgk(float (&g)[19], float ux, float uy, float uz,
                                          float rho, float w0, float w1, float w7,
                                          float tau_inv) {
    const float uxsq = ux * ux, uysq = uy * uy, uzsq = uz * uz;
    const float usq = uxsq + uysq + uzsq;
    const float a0 = w0 * rho, a1 = w1 * rho, a7 = w7 * rho;
    const float p7 = +ux + uy, p8 = +ux - uy, p9 = +ux + uz;
    const float p10 = +ux - uz, p15 = +uy + uz, p16 = +uy - uz;
    g[0]  = g[0]  - tau_inv * (g[0]  - a0 * (1.f - 1.5f * usq));
    g[1]  = g[1]  - tau_inv * (g[1]  - a1 * (1.f + 3.f * ux + 4.5f * uxsq - 1.5f * usq));
    g[2]  = g[2]  - tau_inv * (g[2]  - a1 * (1.f - 3.f * ux + 4.5f * uxsq - 1.5f * usq));
    g[3]  = g[3]  - tau_inv * (g[3]  - a1 * (1.f + 3.f * uy + 4.5f * uysq - 1.5f * usq));
    g[4]  = g[4]  - tau_inv * (g[4]  - a1 * (1.f - 3.f * uy + 4.5f * uysq - 1.5f * usq));
    g[5]  = g[5]  - tau_inv * (g[5]  - a1 * (1.f + 3.f * uz + 4.5f * uzsq - 1.5f * usq));
    g[6]  = g[6]  - tau_inv * (g[6]  - a1 * (1.f - 3.f * uz + 4.5f * uzsq - 1.5f * usq));
    g[7]  = g[7]  - tau_inv * (g[7]  - a7 * (1.f + 3.f * p7  + 4.5f * p7  * p7  - 1.5f * usq));
    g[8]  = g[8]  - tau_inv * (g[8]  - a7 * (1.f + 3.f * p8  + 4.5f * p8  * p8  - 1.5f * usq));
    g[9]  = g[9]  - tau_inv * (g[9]  - a7 * (1.f + 3.f * p9  + 4.5f * p9  * p9  - 1.5f * usq));
    g[10] = g[10] - tau_inv * (g[10] - a7 * (1.f + 3.f * p10 + 4.5f * p10 * p10 - 1.5f * usq));
    g[11] = g[11] - tau_inv * (g[11] - a7 * (1.f - 3.f * p8  + 4.5f * p8  * p8  - 1.5f * usq));
    g[12] = g[12] - tau_inv * (g[12] - a7 * (1.f - 3.f * p7  + 4.5f * p7  * p7  - 1.5f * usq));
    g[13] = g[13] - tau_inv * (g[13] - a7 * (1.f - 3.f * p10 + 4.5f * p10 * p10 - 1.5f * usq));
    g[14] = g[14] - tau_inv * (g[14] - a7 * (1.f - 3.f * p9  + 4.5f * p9  * p9  - 1.5f * usq));
    g[15] = g[15] - tau_inv * (g[15] - a7 * (1.f + 3.f * p15 + 4.5f * p15 * p15 - 1.5f * usq));
    g[16] = g[16] - tau_inv * (g[16] - a7 * (1.f + 3.f * p16 + 4.5f * p16 * p16 - 1.5f * usq));
    g[17] = g[17] - tau_inv * (g[17] - a7 * (1.f - 3.f * p16 + 4.5f * p16 * p16 - 1.5f * usq));
    g[18] = g[18] - tau_inv * (g[18] - a7 * (1.f - 3.f * p15 + 4.5f * p15 * p15 - 1.5f * usq));
}

// density and bare velocity, reference src/collision.cu:453-478
__device__ __forceinline__ void d3q19_moments(const float (&g)[19], float &rho, float &ux,
                                              float &uy, float &uz) {
    rho = g[0] + g[1] + g[2] + g[3] + g[4] + g[5] + g[6] + g[7] + g[8] + g[9] + g[10] + g[11] +
          g[12] + g[13] + g[14] + g[15] + g[16] + g[17] + g[18];
    ux = (g[1] + g[7] + g[8] + g[9] + g[10] - g[2] - g[11] - g[12] - g[13] - g[14]) / rho;
    uy = (g[3] + g[7] + g[11] + g[15] + g[16] - g[4] - g[8] - g[12] - g[17] - g[18]) / rho;
    uz = (g[5] + g[9] + g[13] + g[15] + g[17] - g[6] - g[10] - g[14] - g[16] - g[18]) / rho;
}

// ------------------------------------------------ native-mode D3Q19 arithmetic
// The native mode (no reference counterpart) is free to associate its
// arithmetic for fewer instructions; the oracle restates the same order and
// the same fused multiply-adds (fmaf), so the results stay bit-identical.

// density as the sum of the cx = +1, -1 and 0 partial sums (shared with j_x)
__device__ __forceinline__ void d3q19_xsums_native(const float (&g)[19], float &px, float &mx,
                                                   float &zx) {
    px = (g[1] + g[7]) + (g[8] + g[9]) + g[10];
    mx = (g[2] + g[11]) + (g[12] + g[13]) + g[14];
    zx = ((g[0] + g[3]) + (g[4] + g[5])) + ((g[6] + g[15]) + (g[16] + g[17])) + g[18];
}
__device__ __forceinline__ float d3q19_rho_native(const float (&g)[19]) {
    float px, mx, zx;
    d3q19_xsums_native(g, px, mx, zx);
    return (px + mx) + zx;
}

// density and bare velocity: one division gives 1/rho
__device__ __forceinline__ void d3q19_moments_native(const float (&g)[19], float &rho,
                                                     float &ux, float &uy, float &uz) {
    float px, mx, zx;
    d3q19_xsums_native(g, px, mx, zx);
    rho = (px + mx) + zx;
    const float jy = ((g[3] + g[7]) + (g[11] + g[15]) + g[16]) -
                     ((g[4] + g[8]) + (g[12] + g[17]) + g[18]);
    const float jz = ((g[5] + g[9]) + (g[13] + g[15]) + g[17]) -
                     ((g[6] + g[10]) + (g[14] + g[16]) + g[18]);
    const float inv = 1.f / rho;
    ux = (px - mx) * inv;
    uy = jy * inv;
    uz = jz * inv;
}

// One opposite pair (g+, g-) of the native BGK for projection p, every step
// a fused multiply-add: t = fma(4.5p, p, base), q+- = fma(+-3, p, t),
// d+- = fma(a, q+-, -g+-) (f_eq - g in one rounding), g+- = fma(tau_inv, d+-,
// g+-).  The two lanes run as paired FP32 FMAs (.f32x2, sm_100 and later),
// each lane the scalar IEEE fma: the oracle's scalar fmaf gives the same bits.
__device__ __forceinline__ void bgk_pair_native(float2 &gg, float a, float p, float base,
                                                float tau_inv) {
    const float t = __fmaf_rn(4.5f * p, p, base);
    const float2 q = __ffma2_rn(make_float2(3.f, -3.f), make_float2(p, p), make_float2(t, t));
    const float2 d = __ffma2_rn(make_float2(a, a), q, make_float2(-gg.x, -gg.y));
    gg = __ffma2_rn(make_float2(tau_inv, tau_inv), d, gg);
}

// BGK at velocity (ux, uy, uz): per opposite pair with projection p,
// t = 1 - 1.5 u^2 + 4.5 p^2 once, f_eq = w rho (t +- 3 p), f += tau_inv (f_eq - f)
// (bgk_pair_native)
__device__ __forceinline__ void d3q19_bgk_native(float (&g)[19], float ux, float uy, float uz,
                                                 float rho, float w0, float w1, float w7,
                                                 float tau_inv) {
    const float usq = __fmaf_rn(uz, uz, __fmaf_rn(uy, uy, ux * ux));
    const float base = __fmaf_rn(-1.5f, usq, 1.f);
    const float a0 = w0 * rho, a1 = w1 * rho, a7 = w7 * rho;
    g[0] = __fmaf_rn(tau_inv, __fmaf_rn(a0, base, -g[0]), g[0]);
    auto pair = [&](int kp, int km, float a, float p) {
        float2 gg = make_float2(g[kp], g[km]);
        bgk_pair_native(gg, a, p, base, tau_inv);
        g[kp] = gg.x;
        g[km] = gg.y;
    };
    pair(1, 2, a1, ux);
    pair(3, 4, a1, uy);
    pair(5, 6, a1, uz);
    pair(7, 12, a7, ux + uy);
    pair(8, 11, a7, ux - uy);
    pair(9, 14, a7, ux + uz);
    pair(10, 13, a7, ux - uz);
    pair(15, 18, a7, uy + uz);
    pair(16, 17, a7, uy - uz);
}

// ----------------------------------- 16-bit storage: arithmetic on deviations
// The state is d_k = f_k - wr_k with wr_k = w_k rho_ref.  Density: rho =
// rho_ref + sum_k d_k (the native moments' association over d; rho_ref here
// is sum_k wr_k, the density the offsets carry, rounded once); momentum
// sum_k c_k d_k (the offsets cancel pairwise: wr_k = wr_opp(k) exactly).
// Relaxation: d_k' = (1 - tau_inv) d_k + tau_inv (f_eq,k - wr_k), evaluated
// per opposite pair as x = fma(tau_inv w rho, q, -tau_inv wr), d' =
// fma(1 - tau_inv, d, x): as many instructions as the FP32 form, no offset
// added on load or taken off on store, and f_eq - wr formed with one
// rounding (no cancellation against wr).
__device__ __forceinline__ float d3q19_rho_dev(const float (&d)[19], float rho_ref) {
    return rho_ref + d3q19_rho_native(d);
}

__device__ __forceinline__ void d3q19_moments_dev(const float (&d)[19], float rho_ref,
                                                  float &rho, float &ux, float &uy, float &uz) {
    float px, mx, zx;
    d3q19_xsums_native(d, px, mx, zx);
    rho = rho_ref + ((px + mx) + zx);
    const float jy = ((d[3] + d[7]) + (d[11] + d[15]) + d[16]) -
                     ((d[4] + d[8]) + (d[12] + d[17]) + d[18]);
    const float jz = ((d[5] + d[9]) + (d[13] + d[15]) + d[17]) -
                     ((d[6] + d[10]) + (d[14] + d[16]) + d[18]);
    const float inv = 1.f / rho;
    ux = (px - mx) * inv;
    uy = jy * inv;
    uz = jz * inv;
}

// one opposite pair of the deviation BGK: t = fma(4.5p, p, base), q+- =
// fma(+-3, p, t), x+- = fma(oa, q+-, -owr), d+- = fma(om, d+-, x+-), the pair
// in paired FP32 FMAs (each lane the scalar IEEE fma)
__device__ __forceinline__ void bgk_pair_dev(float2 &dd, float oa, float owr, float p, float base,
                                             float om) {
    const float t = __fmaf_rn(4.5f * p, p, base);
    const float2 q = __ffma2_rn(make_float2(3.f, -3.f), make_float2(p, p), make_float2(t, t));
    const float2 x = __ffma2_rn(make_float2(oa, oa), q, make_float2(-owr, -owr));
    dd = __ffma2_rn(make_float2(om, om), dd, x);
}

// deviation BGK at velocity (ux, uy, uz); wr0, wr1, wr7: the offsets of the
// three weight classes
__device__ __forceinline__ void d3q19_bgk_dev(float (&d)[19], float ux, float uy, float uz,
                                              float rho, float w0, float w1, float w7,
                                              float tau_inv, float wr0, float wr1, float wr7) {
    const float usq = __fmaf_rn(uz, uz, __fmaf_rn(uy, uy, ux * ux));
    const float base = __fmaf_rn(-1.5f, usq, 1.f);
    const float om = 1.f - tau_inv;
    const float oa0 = tau_inv * (w0 * rho), oa1 = tau_inv * (w1 * rho), oa7 = tau_inv * (w7 * rho);
    const float owr0 = tau_inv * wr0, owr1 = tau_inv * wr1, owr7 = tau_inv * wr7;
    d[0] = __fmaf_rn(om, d[0], __fmaf_rn(oa0, base, -owr0));
    auto pair = [&](int kp, int km, float oa, float owr, float p) {
        float2 dd = make_float2(d[kp], d[km]);
        bgk_pair_dev(dd, oa, owr, p, base, om);
        d[kp] = dd.x;
        d[km] = dd.y;
    };
    pair(1, 2, oa1, owr1, ux);
    pair(3, 4, oa1, owr1, uy);
    pair(5, 6, oa1, owr1, uz);
    pair(7, 12, oa7, owr7, ux + uy);
    pair(8, 11, oa7, owr7, ux - uy);
    pair(9, 14, oa7, owr7, ux + uz);
    pair(10, 13, oa7, owr7, ux - uz);
    pair(15, 18, oa7, owr7, uy + uz);
    pair(16, 17, oa7, owr7, uy - uz);
}

// Shan-Chen interaction sum over the 18 neighbours, ps[k] = psi(x + c_k):
// IF = sum_k w_k psi(x + c_k) c_k, grouped by the sign of each component
__device__ __forceinline__ void d3q19_sc_sum_native(const float (&ps)[19], float w1, float w7,
                                                    float &IFx, float &IFy, float &IFz) {
    IFx = __fmaf_rn(w1, ps[1] - ps[2],
                    w7 * (((ps[7] + ps[8]) + (ps[9] + ps[10])) -
                          ((ps[11] + ps[12]) + (ps[13] + ps[14]))));
    IFy = __fmaf_rn(w1, ps[3] - ps[4],
                    w7 * (((ps[7] + ps[11]) + (ps[15] + ps[16])) -
                          ((ps[8] + ps[12]) + (ps[17] + ps[18]))));
    IFz = __fmaf_rn(w1, ps[5] - ps[6],
                    w7 * (((ps[9] + ps[13]) + (ps[15] + ps[17])) -
                          ((ps[10] + ps[14]) + (ps[16] + ps[18]))));
}

// Zou-He velocity inlet at the west face, reference src/collision.cu:412-430
// (the reference's double literals promote these lines to FP64)
__device__ __forceinline__ void d3q19_zou_he_west(float (&g)[19], float ux_in) {
    const float a = g[0] + g[3] + g[4] + g[5] + g[6] + g[15] + g[16] + g[17] + g[18];
    const float b = g[2] + g[11] + g[12] + g[13] + g[14];
    const float rho = (float)(((double)a + 2. * (double)b) / (1. - (double)ux_in));
    const float ru = rho * ux_in;
    const float ty = g[3] + g[15] + g[16] - g[4] - g[17] - g[18];
    const float tz = g[5] + g[11] + g[15] - g[6] - g[16] - g[18];
    g[1]  = (float)((double)g[2]  + (1. / 3.) * (double)ru);
    g[8]  = (float)((double)g[11] + (1. / 6.) * (double)ru + 0.5 * (double)ty);
    g[7]  = (float)((double)g[12] + (1. / 6.) * (double)ru - 0.5 * (double)ty);
    g[9]  = (float)((double)g[14] + (1. / 6.) * (double)ru - 0.5 * (double)tz);
    g[10] = (float)((double)g[13] + (1. / 6.) * (double)ru + 0.5 * (double)tz);
}

// Zou-He pressure outlet at the east face, reference src/collision.cu:432-451;
// the last two lines read the f11 written just before, as the reference does
__device__ __forceinline__ void d3q19_zou_he_east(float (&g)[19], float rho_out) {
    const float a = g[0] + g[3] + g[4] + g[5] + g[6] + g[15] + g[16] + g[17] + g[18];
    const float b = g[1] + g[7] + g[8] + g[9] + g[10];
    const float ux = (float)(-1. + ((double)a + 2. * (double)b) / (double)rho_out);
    const float ru = rho_out * ux;
    const float ty = g[3] + g[15] + g[16] - g[4] - g[17] - g[18];
    g[2]  = (float)((double)g[1] - (1. / 3.) * (double)ru);
    g[11] = (float)((double)g[8] - (1. / 6.) * (double)ru - 0.5 * (double)ty);
    g[12] = (float)((double)g[7] - (1. / 6.) * (double)ru + 0.5 * (double)ty);
    const float tz = g[5] + g[11] + g[15] - g[6] - g[16] - g[18];
    g[14] = (float)((double)g[9]  - (1. / 6.) * (double)ru + 0.5 * (double)tz);
    g[13] = (float)((double)g[10] - (1. / 6.) * (double)ru - 0.5 * (double)tz);
}

// ---------------------------------------------------------------- BGK, D2Q9
// reference src/collision.cu:298-330
__device__ __forceinline__ void d2q9_bgk(float (&g)[9], float ex, float ey, float rho, float w0,
                                         float w1, float w5, float tau_inv) {
    const float exsq = ex * ex, eysq = ey * ey;
    const float esq = exsq + eysq;
    const float a0 = w0 * rho, a1 = w1 * rho, a5 = w5 * rho;
    const float u5 = +ex + ey, u6 = -ex + ey;
    g[0] = g[0] - tau_inv * (g[0] - a0 * (1.f - 1.5f * esq));
    g[1] = g[1] - tau_inv * (g[1] - a1 * (1.f + 3.f * ex + 4.5f * exsq - 1.5f * esq));
    g[2] = g[2] - tau_inv * (g[2] - a1 * (1.f + 3.f * ey + 4.5f * eysq - 1.5f * esq));
    g[3] = g[3] - tau_inv * (g[3] - a1 * (1.f - 3.f * ex + 4.5f * exsq - 1.5f * esq));
    g[4] = g[4] - tau_inv * (g[4] - a1 * (1.f - 3.f * ey + 4.5f * eysq - 1.5f * esq));
    g[5] = g[5] - tau_inv * (g[5] - a5 * (1.f + 3.f * u5 + 4.5f * u5 * u5 - 1.5f * esq));
    g[6] = g[6] - tau_inv * (g[6] - a5 * (1.f + 3.f * u6 + 4.5f * u6 * u6 - 1.5f * esq));
    g[7] = g[7] - tau_inv * (g[7] - a5 * (1.f - 3.f * u5 + 4.5f * u5 * u5 - 1.5f * esq));
    g[8] = g[8] - tau_inv * (g[8] - a5 * (1.f - 3.f * u6 + 4.5f * u6 * u6 - 1.5f * esq));
}

__device__ __forceinline__ void d2q9_moments(const float (&g)[9], float &rho, float &ux,
                                             float &uy) {
    rho = g[0] + g[1] + g[2] + g[3] + g[4] + g[5] + g[6] + g[7] + g[8];
    ux = (g[1] - g[3] + g[5] - g[6] - g[7] + g[8]) / rho;
    uy = (g[2] - g[4] + g[5] + g[6] - g[7] - g[8]) / rho;
}

// ------------------------------------------- native-mode D2Q9 arithmetic
// The same quantities as above in the library's own association (partial
// sums by c_x shared between rho and j_x, one division for 1/rho) and with
// fused multiply-adds in the BGK, as d3q19_*_native.  Native mode only; the
// oracle performs the same operations (oracle/lb_oracle_body.h,
// d2q9_*_native).
__device__ __forceinline__ void d2q9_moments_native(const float (&g)[9], float &rho, float &ux,
                                                    float &uy) {
    const float px = (g[1] + g[5]) + g[8];  // c_x = +1
    const float mx = (g[3] + g[6]) + g[7];  // c_x = -1
    const float zx = (g[0] + g[2]) + g[4];  // c_x = 0
    const float r = (px + mx) + zx;
    const float jy = ((g[2] + g[5]) + g[6]) - ((g[4] + g[7]) + g[8]);
    const float inv = 1.f / r;
    rho = r;
    ux = (px - mx) * inv;
    uy = jy * inv;
}

__device__ __forceinline__ void d2q9_bgk_native(float (&g)[9], float ux, float uy, float rho,
                                                float w0, float w1, float w5, float tau_inv) {
    const float usq = __fmaf_rn(uy, uy, ux * ux);
    const float base = __fmaf_rn(-1.5f, usq, 1.f);
    const float a0 = w0 * rho, a1 = w1 * rho, a5 = w5 * rho;
    g[0] = __fmaf_rn(tau_inv, __fmaf_rn(a0, base, -g[0]), g[0]);
    auto pair = [&](int kp, int km, float a, float p) {
        float2 gg = make_float2(g[kp], g[km]);
        bgk_pair_native(gg, a, p, base, tau_inv);
        g[kp] = gg.x;
        g[km] = gg.y;
    };
    pair(1, 3, a1, ux);
    pair(2, 4, a1, uy);
    pair(5, 7, a5, ux + uy);
    pair(6, 8, a5, uy - ux);
}

// native Shan-Chen shift of (ex, ey): IF = sum_k w_k psi(x + c_k) c_k grouped
// by the sign of each component (ps in the order psi(x), psi(x+1,y),
// psi(x,row+1), psi(x-1,y), psi(x,row-1), then the diagonals (x+1,row+1),
// (x-1,row+1), (x-1,row-1), (x+1,row-1); row+1 is physical -y), applied as
// (-G psi(x)) inv_rt IF with inv_rt = 1/(tau_inv rho)
__device__ __forceinline__ void d2q9_sc_shift_native(const float (&ps)[9], float w1, float w5,
                                                     float G, float inv_rt, float &ex,
                                                     float &ey) {
    const float IFx = __fmaf_rn(w1, ps[1] - ps[3], w5 * ((ps[5] + ps[8]) - (ps[6] + ps[7])));
    const float IFy = __fmaf_rn(w1, ps[4] - ps[2], w5 * ((ps[7] + ps[8]) - (ps[5] + ps[6])));
    const float c = (-G * ps[0]) * inv_rt;
    ex = __fmaf_rn(c, IFx, ex);
    ey = __fmaf_rn(c, IFy, ey);
}

__device__ __forceinline__ float d2q9_rho_native(const float (&g)[9]) {
    return (((g[1] + g[5]) + g[8]) + ((g[3] + g[6]) + g[7])) + ((g[0] + g[2]) + g[4]);
}

// native collision after the pull: moments, velocity-shift force with one
// division 1/(rho tau_inv) (the form of reference src/collision.cu:280-284),
// BGK; rho, ux, uy are the moments before the shift
__device__ __forceinline__ void d2q9_collide_native(float (&g)[9], float Fx, float Fy, float w0,
                                                    float w1, float w5, float tau_inv,
                                                    float &rho, float &ux, float &uy) {
    d2q9_moments_native(g, rho, ux, uy);
    float ex = ux, ey = uy;
    if (Fx != 0.f || Fy != 0.f) {
        const float inv_rt = 1.f / (rho * tau_inv);
        if (Fx != 0.f) ex = __fmaf_rn(Fx, inv_rt, ux);
        if (Fy != 0.f) ey = __fmaf_rn(Fy, inv_rt, uy);
    }
    d2q9_bgk_native(g, ex, ey, rho, w0, w1, w5, tau_inv);
}

// Zou-He west inlet / east outlet, reference src/collision.cu:210-262
__device__ __forceinline__ void d2q9_zou_he_west(float (&g)[9], float ux_in) {
    const float a = g[0] + g[2] + g[4], b = g[3] + g[7] + g[6];
    const float r = (float)(((double)a + 2. * (double)b) / (1. - (double)ux_in));
    const float ru = r * ux_in;
    g[1] = (float)((double)g[3] + (2. / 3.) * (double)ru);
    g[5] = (float)((double)g[7] + (1. / 6.) * (double)ru - 0.5 * (double)(g[2] - g[4]));
    g[8] = (float)((double)g[6] + (1. / 6.) * (double)ru - 0.5 * (double)(g[4] - g[2]));
}
__device__ __forceinline__ void d2q9_zou_he_east(float (&g)[9], float rho_out) {
    const float a = g[0] + g[2] + g[4], b = g[1] + g[5] + g[8];
    const float vx = (float)(-1. + ((double)a + 2. * (double)b) / (double)rho_out);
    const float ru = rho_out * vx;
    g[3] = (float)((double)g[1] - (2. / 3.) * (double)ru);
    g[7] = (float)((double)g[5] - (1. / 6.) * (double)ru + 0.5 * (double)(g[2] - g[4]));
    g[6] = (float)((double)g[8] - (1. / 6.) * (double)ru + 0.5 * (double)(g[4] - g[2]));
}

// Shan-Chen interaction of the D2Q9 step, reference src/collision.cu:78-96:
// F = -G psi(x) sum_k w_k psi(x + c_k) c_k accumulated in the reference's
// order, then u_eq += F / (tau_inv rho).  ps[m] is psi at the reference's
// stencil slot m (0 centre, 1 x+1, 2 row+1, 3 x-1, 4 row-1, 5 (x+1,row+1),
// 6 (x-1,row+1), 7 (x-1,row-1), 8 (x+1,row-1)).
__device__ __forceinline__ void d2q9_sc_shift(const float (&ps)[9], float w1, float w5, float G,
                                              float tau_inv, float rho, float &ex, float &ey) {
    float IFx = 0.f, IFy = 0.f;
    IFx = IFx + w1 * ps[1];
    IFx = IFx - w1 * ps[3];
    IFx = IFx + w5 * ps[5];
    IFx = IFx - w5 * ps[6];
    IFx = IFx - w5 * ps[7];
    IFx = IFx + w5 * ps[8];
    IFy = IFy - w1 * ps[2];
    IFy = IFy + w1 * ps[4];
    IFy = IFy - w5 * ps[5];
    IFy = IFy - w5 * ps[6];
    IFy = IFy + w5 * ps[7];
    IFy = IFy + w5 * ps[8];
    IFx = -G * ps[0] * IFx;
    IFy = -G * ps[0] * IFy;
    ex = ex + (IFx / (tau_inv * rho));
    ey = ey + (IFy / (tau_inv * rho));
}

// exp(x) in float, this library's own: Cody-Waite range reduction
// x = k ln2 + r with ln2 split into a 12-bit head (k*head exact) and a tail,
// |r| <= ln2/2, then the degree-7 Taylor polynomial of exp(r) (coefficients
// 1/n! rounded to float) by Horner, scaled by 2^k.  Error at most 1.12 ulp
// on [-87, 88].  Every operation rounds once (the library builds with
// -fmad=false), so the oracle's copy of the same steps gives the same bits.
__device__ __forceinline__ float lb_expf(float x) {
    if (x < -103.f) return 0.f;
    if (x > 88.7f) return __int_as_float(0x7f800000);
    const float k = rintf(x * 0x1.715476p+0f);
    const float r = (x - k * 0x1.62ep-1f) - k * 0x1.0bfbe8p-15f;
    float p = 0x1.a01a02p-13f;
    p = p * r + 0x1.6c16c2p-10f;
    p = p * r + 0x1.111112p-7f;
    p = p * r + 0x1.555556p-5f;
    p = p * r + 0x1.555556p-3f;
    p = p * r + 0.5f;
    p = p * r + 1.0f;
    p = p * r + 1.0f;
    const int ki = (int)k;
    if (ki >= -126) return p * __int_as_float((ki + 127) << 23);
    return (p * __int_as_float((ki + 64 + 127) << 23)) * 0x1p-64f;
}

// psi(rho) forms of the Shan-Chen pseudo-potential
__device__ __forceinline__ float psi_ref(float rho) {  // src/collision.cu:293
    return (float)(4. * exp(-200. / (double)rho));
}
__device__ __forceinline__ float psi_exp1(float rho) { return 1.f - lb_expf(-rho); }

}  // namespace lb
