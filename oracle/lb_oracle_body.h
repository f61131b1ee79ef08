/*
 * lb_oracle_body.h -- precision-generic body of the CPU oracle (test
 * infrastructure only).  lb_oracle.c includes it twice: R=float/S=f32 and
 * R=double/S=f64.  Where the reference promotes to double (double literals in
 * the Zou-He lines and exp() in psi) the code promotes explicitly, so the f32
 * instantiation reproduces the reference's float arithmetic operation by
 * operation; expressions keep the reference's left-to-right association.
 */

#define CAT2_(a, b) a##_##b
#define CAT_(a, b) CAT2_(a, b)
#define FN(n) CAT_(n, S)

/* ======================================================================== */
/* D3Q19, reference semantics                                               */
/* ======================================================================== */

/* In-place swap streaming, src/streaming.cu:84-163: every node that is not
 * solid_bound swaps f_k(x) with f_opp(k)(x+c_k) for the nine "positive"
 * directions, periodic in x, y and z.  Each (node, slot) belongs to exactly one
 * pair and each pair to one node, so the z planes can run in parallel. */
void FN(lbo_d3q19_stream)(R *f, const uint8_t *solid_bound, int W, int H, int D)
{
    const long N = (long)W * H * D;
#pragma omp parallel for schedule(static)
    for (int z = 0; z < D; z++)
        for (int y = 0; y < H; y++)
            for (int x = 0; x < W; x++) {
                const long o = x + (long)y * W + (long)z * W * H;
                if (solid_bound[o]) continue;
                for (int p = 0; p < 9; p++) {
                    const int k = D3_POS[p], q = D3_OPP[k];
                    const int xn = wrapi(x + D3_CX[k], W);
                    const int yn = wrapi(y + D3_CY[k], H);
                    const int zn = wrapi(z + D3_CZ[k], D);
                    const long on = xn + (long)yn * W + (long)zn * W * H;
                    R t = f[k * N + o];
                    f[k * N + o] = f[q * N + on];
                    f[q * N + on] = t;
                }
            }
}

/* BGK relaxation of the 19 populations at one node, src/collision.cu:480-541
 * (velocity argument = u, or u_eq when a force shift is applied).  The
 * association of every expression is the reference's. */
static inline void FN(d3q19_bgk)(R *g, R ux, R uy, R uz, R rho, R w0, R w1, R w7, R tau_inv)
{
    const R uxsq = ux * ux, uysq = uy * uy, uzsq = uz * uz;
    const R usq = uxsq + uysq + uzsq;
    const R a0 = w0 * rho, a1 = w1 * rho, a7 = w7 * rho;
    const R uxuy7 = +ux + uy, uxuy8 = +ux - uy, uxuz9 = +ux + uz;
    const R uxuz10 = +ux - uz, uyuz15 = +uy + uz, uyuz16 = +uy - uz;
    const R c1 = (R)1.f, c3 = (R)3.f, c45 = (R)4.5f, c15 = (R)1.5f;
    g[0]  = g[0]  - tau_inv * (g[0]  - a0 * (c1 - c15 * usq));
    g[1]  = g[1]  - tau_inv * (g[1]  - a1 * (c1 + c3 * ux + c45 * uxsq - c15 * usq));
    g[2]  = g[2]  - tau_inv * (g[2]  - a1 * (c1 - c3 * ux + c45 * uxsq - c15 * usq));
    g[3]  = g[3]  - tau_inv * (g[3]  - a1 * (c1 + c3 * uy + c45 * uysq - c15 * usq));
    g[4]  = g[4]  - tau_inv * (g[4]  - a1 * (c1 - c3 * uy + c45 * uysq - c15 * usq));
    g[5]  = g[5]  - tau_inv * (g[5]  - a1 * (c1 + c3 * uz + c45 * uzsq - c15 * usq));
    g[6]  = g[6]  - tau_inv * (g[6]  - a1 * (c1 - c3 * uz + c45 * uzsq - c15 * usq));
    g[7]  = g[7]  - tau_inv * (g[7]  - a7 * (c1 + c3 * uxuy7  + c45 * uxuy7  * uxuy7  - c15 * usq));
    g[8]  = g[8]  - tau_inv * (g[8]  - a7 * (c1 + c3 * uxuy8  + c45 * uxuy8  * uxuy8  - c15 * usq));
    g[9]  = g[9]  - tau_inv * (g[9]  - a7 * (c1 + c3 * uxuz9  + c45 * uxuz9  * uxuz9  - c15 * usq));
    g[10] = g[10] - tau_inv * (g[10] - a7 * (c1 + c3 * uxuz10 + c45 * uxuz10 * uxuz10 - c15 * usq));
    g[11] = g[11] - tau_inv * (g[11] - a7 * (c1 - c3 * uxuy8  + c45 * uxuy8  * uxuy8  - c15 * usq));
    g[12] = g[12] - tau_inv * (g[12] - a7 * (c1 - c3 * uxuy7  + c45 * uxuy7  * uxuy7  - c15 * usq));
    g[13] = g[13] - tau_inv * (g[13] - a7 * (c1 - c3 * uxuz10 + c45 * uxuz10 * uxuz10 - c15 * usq));
    g[14] = g[14] - tau_inv * (g[14] - a7 * (c1 - c3 * uxuz9  + c45 * uxuz9  * uxuz9  - c15 * usq));
    g[15] = g[15] - tau_inv * (g[15] - a7 * (c1 + c3 * uyuz15 + c45 * uyuz15 * uyuz15 - c15 * usq));
    g[16] = g[16] - tau_inv * (g[16] - a7 * (c1 + c3 * uyuz16 + c45 * uyuz16 * uyuz16 - c15 * usq));
    g[17] = g[17] - tau_inv * (g[17] - a7 * (c1 - c3 * uyuz16 + c45 * uyuz16 * uyuz16 - c15 * usq));
    g[18] = g[18] - tau_inv * (g[18] - a7 * (c1 - c3 * uyuz15 + c45 * uyuz15 * uyuz15 - c15 * usq));
}

/* density and bare velocity, src/collision.cu:453-478 */
static inline void FN(d3q19_moments)(const R *g, R *rho, R *ux, R *uy, R *uz)
{
    const R r = g[0] + g[1] + g[2] + g[3] + g[4] + g[5] + g[6] + g[7] + g[8] + g[9] + g[10] +
                g[11] + g[12] + g[13] + g[14] + g[15] + g[16] + g[17] + g[18];
    *rho = r;
    *ux = (g[1] + g[7] + g[8] + g[9] + g[10] - g[2] - g[11] - g[12] - g[13] - g[14]) / r;
    *uy = (g[3] + g[7] + g[11] + g[15] + g[16] - g[4] - g[8] - g[12] - g[17] - g[18]) / r;
    *uz = (g[5] + g[9] + g[13] + g[15] + g[17] - g[6] - g[10] - g[14] - g[16] - g[18]) / r;
}

/* ---- native mode (no reference counterpart): the library's association and
 * fused multiply-adds (FMA_R = fmaf / fma, one rounding like the GPU's)
 * lattibol_0.3.31f_gb300/csrc/lb_common.cuh, d3q19_*_native */
static inline void FN(d3q19_xsums_native)(const R *g, R *px, R *mx, R *zx)
{
    *px = (g[1] + g[7]) + (g[8] + g[9]) + g[10];
    *mx = (g[2] + g[11]) + (g[12] + g[13]) + g[14];
    *zx = ((g[0] + g[3]) + (g[4] + g[5])) + ((g[6] + g[15]) + (g[16] + g[17])) + g[18];
}
static inline R FN(d3q19_rho_native)(const R *g)
{
    R px, mx, zx;
    FN(d3q19_xsums_native)(g, &px, &mx, &zx);
    return (px + mx) + zx;
}
static inline void FN(d3q19_moments_native)(const R *g, R *rho, R *ux, R *uy, R *uz)
{
    R px, mx, zx;
    FN(d3q19_xsums_native)(g, &px, &mx, &zx);
    const R r = (px + mx) + zx;
    const R jy = ((g[3] + g[7]) + (g[11] + g[15]) + g[16]) -
                 ((g[4] + g[8]) + (g[12] + g[17]) + g[18]);
    const R jz = ((g[5] + g[9]) + (g[13] + g[15]) + g[17]) -
                 ((g[6] + g[10]) + (g[14] + g[16]) + g[18]);
    const R inv = (R)1 / r;
    *rho = r;
    *ux = (px - mx) * inv;
    *uy = jy * inv;
    *uz = jz * inv;
}
static inline void FN(bgk_pair_native)(R *g, int kp, int km, R a, R p, R base, R tau_inv)
{
    /* every step a fused multiply-add; f_eq - g in one rounding */
    const R t = FMA_R((R)4.5f * p, p, base);
    const R dp = FMA_R(a, FMA_R((R)3.f, p, t), -g[kp]);
    const R dm = FMA_R(a, FMA_R((R)-3.f, p, t), -g[km]);
    g[kp] = FMA_R(tau_inv, dp, g[kp]);
    g[km] = FMA_R(tau_inv, dm, g[km]);
}
static inline void FN(d3q19_bgk_native)(R *g, R ux, R uy, R uz, R rho, R w0, R w1, R w7,
                                        R tau_inv)
{
    const R usq = FMA_R(uz, uz, FMA_R(uy, uy, ux * ux));
    const R base = FMA_R((R)-1.5f, usq, (R)1.f);
    const R a0 = w0 * rho, a1 = w1 * rho, a7 = w7 * rho;
    g[0] = FMA_R(tau_inv, FMA_R(a0, base, -g[0]), g[0]);
    FN(bgk_pair_native)(g, 1, 2, a1, ux, base, tau_inv);
    FN(bgk_pair_native)(g, 3, 4, a1, uy, base, tau_inv);
    FN(bgk_pair_native)(g, 5, 6, a1, uz, base, tau_inv);
    FN(bgk_pair_native)(g, 7, 12, a7, ux + uy, base, tau_inv);
    FN(bgk_pair_native)(g, 8, 11, a7, ux - uy, base, tau_inv);
    FN(bgk_pair_native)(g, 9, 14, a7, ux + uz, base, tau_inv);
    FN(bgk_pair_native)(g, 10, 13, a7, ux - uz, base, tau_inv);
    FN(bgk_pair_native)(g, 15, 18, a7, uy + uz, base, tau_inv);
    FN(bgk_pair_native)(g, 16, 17, a7, uy - uz, base, tau_inv);
}
/* 16-bit storage: the step on the deviations d_k = f_k - wr_k
 * (lattibol_0.3.31f_gb300/csrc/lb_common.cuh, d3q19_*_dev): density
 * rho_off + sum d (rho_off = sum_k wr_k), momentum sum c d, relaxation
 * d' = fma(1 - tau_inv, d, fma(tau_inv w rho, q, -tau_inv wr)) */
static inline void FN(d3q19_moments_dev)(const R *d, R rho_off, R *rho, R *ux, R *uy, R *uz)
{
    R px, mx, zx;
    FN(d3q19_xsums_native)(d, &px, &mx, &zx);
    const R r = rho_off + ((px + mx) + zx);
    const R jy = ((d[3] + d[7]) + (d[11] + d[15]) + d[16]) -
                 ((d[4] + d[8]) + (d[12] + d[17]) + d[18]);
    const R jz = ((d[5] + d[9]) + (d[13] + d[15]) + d[17]) -
                 ((d[6] + d[10]) + (d[14] + d[16]) + d[18]);
    const R inv = (R)1 / r;
    *rho = r;
    *ux = (px - mx) * inv;
    *uy = jy * inv;
    *uz = jz * inv;
}
static inline void FN(bgk_pair_dev)(R *d, int kp, int km, R oa, R owr, R p, R base, R om)
{
    const R t = FMA_R((R)4.5f * p, p, base);
    const R xp = FMA_R(oa, FMA_R((R)3.f, p, t), -owr);
    const R xm = FMA_R(oa, FMA_R((R)-3.f, p, t), -owr);
    d[kp] = FMA_R(om, d[kp], xp);
    d[km] = FMA_R(om, d[km], xm);
}
static inline void FN(d3q19_bgk_dev)(R *d, R ux, R uy, R uz, R rho, R w0, R w1, R w7,
                                     R tau_inv, R wr0, R wr1, R wr7)
{
    const R usq = FMA_R(uz, uz, FMA_R(uy, uy, ux * ux));
    const R base = FMA_R((R)-1.5f, usq, (R)1.f);
    const R om = (R)1.f - tau_inv;
    const R oa0 = tau_inv * (w0 * rho), oa1 = tau_inv * (w1 * rho), oa7 = tau_inv * (w7 * rho);
    const R owr0 = tau_inv * wr0, owr1 = tau_inv * wr1, owr7 = tau_inv * wr7;
    d[0] = FMA_R(om, d[0], FMA_R(oa0, base, -owr0));
    FN(bgk_pair_dev)(d, 1, 2, oa1, owr1, ux, base, om);
    FN(bgk_pair_dev)(d, 3, 4, oa1, owr1, uy, base, om);
    FN(bgk_pair_dev)(d, 5, 6, oa1, owr1, uz, base, om);
    FN(bgk_pair_dev)(d, 7, 12, oa7, owr7, ux + uy, base, om);
    FN(bgk_pair_dev)(d, 8, 11, oa7, owr7, ux - uy, base, om);
    FN(bgk_pair_dev)(d, 9, 14, oa7, owr7, ux + uz, base, om);
    FN(bgk_pair_dev)(d, 10, 13, oa7, owr7, ux - uz, base, om);
    FN(bgk_pair_dev)(d, 15, 18, oa7, owr7, uy + uz, base, om);
    FN(bgk_pair_dev)(d, 16, 17, oa7, owr7, uy - uz, base, om);
}
/* native D2Q9 (lattibol_0.3.31f_gb300/csrc/lb_common.cuh, d2q9_*_native):
 * partial sums by c_x, one division for 1/rho, the BGK pairs above */
static inline void FN(d2q9_moments_native)(const R *g, R *rho, R *ux, R *uy)
{
    const R px = (g[1] + g[5]) + g[8];
    const R mx = (g[3] + g[6]) + g[7];
    const R zx = (g[0] + g[2]) + g[4];
    const R r = (px + mx) + zx;
    const R jy = ((g[2] + g[5]) + g[6]) - ((g[4] + g[7]) + g[8]);
    const R inv = (R)1 / r;
    *rho = r;
    *ux = (px - mx) * inv;
    *uy = jy * inv;
}
static inline void FN(d2q9_bgk_native)(R *g, R ux, R uy, R rho, R w0, R w1, R w5, R tau_inv)
{
    const R usq = FMA_R(uy, uy, ux * ux);
    const R base = FMA_R((R)-1.5f, usq, (R)1.f);
    const R a0 = w0 * rho, a1 = w1 * rho, a5 = w5 * rho;
    g[0] = FMA_R(tau_inv, FMA_R(a0, base, -g[0]), g[0]);
    FN(bgk_pair_native)(g, 1, 3, a1, ux, base, tau_inv);
    FN(bgk_pair_native)(g, 2, 4, a1, uy, base, tau_inv);
    FN(bgk_pair_native)(g, 5, 7, a5, ux + uy, base, tau_inv);
    FN(bgk_pair_native)(g, 6, 8, a5, uy - ux, base, tau_inv);
}
/* ps[k] = psi(x + c_k) */
static inline void FN(d3q19_sc_sum_native)(const R *ps, R w1, R w7, R *IFx, R *IFy, R *IFz)
{
    *IFx = FMA_R(w1, ps[1] - ps[2],
                 w7 * (((ps[7] + ps[8]) + (ps[9] + ps[10])) - ((ps[11] + ps[12]) + (ps[13] + ps[14]))));
    *IFy = FMA_R(w1, ps[3] - ps[4],
                 w7 * (((ps[7] + ps[11]) + (ps[15] + ps[16])) - ((ps[8] + ps[12]) + (ps[17] + ps[18]))));
    *IFz = FMA_R(w1, ps[5] - ps[6],
                 w7 * (((ps[9] + ps[13]) + (ps[15] + ps[17])) - ((ps[10] + ps[14]) + (ps[16] + ps[18]))));
}

/* Zou-He velocity inlet (west), src/collision.cu:412-430 */
static inline void FN(d3q19_zou_he_west)(R *g, R ux_in)
{
    const R a = g[0] + g[3] + g[4] + g[5] + g[6] + g[15] + g[16] + g[17] + g[18];
    const R b = g[2] + g[11] + g[12] + g[13] + g[14];
    const R rho = (R)(((double)a + 2. * (double)b) / (1. - (double)ux_in));
    const R ru = rho * ux_in;
    const R ty = g[3] + g[15] + g[16] - g[4] - g[17] - g[18];
    const R tz = g[5] + g[11] + g[15] - g[6] - g[16] - g[18];
    g[1]  = (R)((double)g[2]  + (1. / 3.) * (double)ru);
    g[8]  = (R)((double)g[11] + (1. / 6.) * (double)ru + 0.5 * (double)ty);
    g[7]  = (R)((double)g[12] + (1. / 6.) * (double)ru - 0.5 * (double)ty);
    g[9]  = (R)((double)g[14] + (1. / 6.) * (double)ru - 0.5 * (double)tz);
    g[10] = (R)((double)g[13] + (1. / 6.) * (double)ru + 0.5 * (double)tz);
}

/* Zou-He pressure outlet (east), src/collision.cu:432-451.  The writes are
 * sequential: f14 and f13 read the f11 written two lines earlier. */
static inline void FN(d3q19_zou_he_east)(R *g, R rho_out)
{
    const R a = g[0] + g[3] + g[4] + g[5] + g[6] + g[15] + g[16] + g[17] + g[18];
    const R b = g[1] + g[7] + g[8] + g[9] + g[10];
    const R ux = (R)(-1. + ((double)a + 2. * (double)b) / (double)rho_out);
    const R ru = rho_out * ux;
    const R ty = g[3] + g[15] + g[16] - g[4] - g[17] - g[18];
    g[2]  = (R)((double)g[1] - (1. / 3.) * (double)ru);
    g[11] = (R)((double)g[8] - (1. / 6.) * (double)ru - 0.5 * (double)ty);
    g[12] = (R)((double)g[7] - (1. / 6.) * (double)ru + 0.5 * (double)ty);
    {
        const R tz = g[5] + g[11] + g[15] - g[6] - g[16] - g[18];
        g[14] = (R)((double)g[9] - (1. / 6.) * (double)ru + 0.5 * (double)tz);
    }
    {
        const R tz = g[5] + g[11] + g[15] - g[6] - g[16] - g[18];
        g[13] = (R)((double)g[10] - (1. / 6.) * (double)ru - 0.5 * (double)tz);
    }
}

/* Collision, src/collision.cu:357-552: local swap back to natural order,
 * Zou-He x boundaries (always on for non-solid nodes of the first/last
 * device), moments, plot float4, BGK.  Solid nodes get zero moments/plot and
 * keep their populations. */
void FN(lbo_d3q19_collide)(float *plot, R *f, const uint8_t *solid, R *ux, R *uy, R *uz,
                           R *rho, int W, int H, int D, int dev, int ndev, R w0, R w1,
                           R w7, R tau_inv, R ux_in, R uy_in, R uz_in, R rho_out)
{
    (void)uy_in; (void)uz_in;
    const long N = (long)W * H * D;
#pragma omp parallel for schedule(static)
    for (long o = 0; o < N; o++) {
        const int x = (int)(o % W);
        if (solid[o]) {
            if (plot) { plot[4 * o] = 0.f; plot[4 * o + 1] = 0.f; plot[4 * o + 2] = 0.f; plot[4 * o + 3] = 0.f; }
            ux[o] = 0; uy[o] = 0; uz[o] = 0; rho[o] = 0;
            continue;
        }
        R g[19];
        for (int k = 0; k < 19; k++) g[k] = f[k * N + o];
        for (int p = 0; p < 9; p++) {
            const int k = D3_POS[p], q = D3_OPP[k];
            R t = g[k]; g[k] = g[q]; g[q] = t;
        }
        if (x == 0 && dev == 0)
            FN(d3q19_zou_he_west)(g, ux_in);
        else if (x == W - 1 && dev == ndev - 1)
            FN(d3q19_zou_he_east)(g, rho_out);
        R r, vx, vy, vz;
        FN(d3q19_moments)(g, &r, &vx, &vy, &vz);
        ux[o] = vx; uy[o] = vy; uz[o] = vz; rho[o] = r;
        if (plot) { plot[4 * o] = (float)vx; plot[4 * o + 1] = (float)vy; plot[4 * o + 2] = (float)vz; plot[4 * o + 3] = (float)r; }
        FN(d3q19_bgk)(g, vx, vy, vz, r, w0, w1, w7, tau_inv);
        for (int k = 0; k < 19; k++) f[k * N + o] = g[k];
    }
}

/* ======================================================================== */
/* D2Q9, reference semantics                                                */
/* ======================================================================== */

/* In-place swap streaming, src/streaming.cu:24-74 (+y is row-1). */
void FN(lbo_d2q9_stream)(R *f, const uint8_t *solid_bound, int W, int H)
{
    const long N = (long)W * H;
#pragma omp parallel for schedule(static)
    for (int y = 0; y < H; y++)
        for (int x = 0; x < W; x++) {
            const long o = x + (long)y * W;
            if (solid_bound[o]) continue;
            for (int p = 0; p < 4; p++) {
                const int k = D2_POS[p], q = D2_OPP[k];
                const long on = wrapi(x + D2_CX[k], W) + (long)wrapi(y + D2_CR[k], H) * W;
                R t = f[k * N + o];
                f[k * N + o] = f[q * N + on];
                f[q * N + on] = t;
            }
        }
}

static inline void FN(d2q9_bgk)(R *g, R ueq_x, R ueq_y, R rho, R w0, R w1, R w5, R tau_inv)
{
    const R ueq_xsq = ueq_x * ueq_x, ueq_ysq = ueq_y * ueq_y;
    const R ueq_sq = ueq_xsq + ueq_ysq;
    const R a0 = w0 * rho, a1 = w1 * rho, a5 = w5 * rho;
    const R u5 = +ueq_x + ueq_y, u6 = -ueq_x + ueq_y;
    const R c1 = (R)1.f, c3 = (R)3.f, c45 = (R)4.5f, c15 = (R)1.5f;
    g[0] = g[0] - tau_inv * (g[0] - a0 * (c1 - c15 * ueq_sq));
    g[1] = g[1] - tau_inv * (g[1] - a1 * (c1 + c3 * ueq_x + c45 * ueq_xsq - c15 * ueq_sq));
    g[2] = g[2] - tau_inv * (g[2] - a1 * (c1 + c3 * ueq_y + c45 * ueq_ysq - c15 * ueq_sq));
    g[3] = g[3] - tau_inv * (g[3] - a1 * (c1 - c3 * ueq_x + c45 * ueq_xsq - c15 * ueq_sq));
    g[4] = g[4] - tau_inv * (g[4] - a1 * (c1 - c3 * ueq_y + c45 * ueq_ysq - c15 * ueq_sq));
    g[5] = g[5] - tau_inv * (g[5] - a5 * (c1 + c3 * u5 + c45 * u5 * u5 - c15 * ueq_sq));
    g[6] = g[6] - tau_inv * (g[6] - a5 * (c1 + c3 * u6 + c45 * u6 * u6 - c15 * ueq_sq));
    g[7] = g[7] - tau_inv * (g[7] - a5 * (c1 - c3 * u5 + c45 * u5 * u5 - c15 * ueq_sq));
    g[8] = g[8] - tau_inv * (g[8] - a5 * (c1 - c3 * u6 + c45 * u6 * u6 - c15 * ueq_sq));
}

static inline void FN(d2q9_moments)(const R *g, R *rho, R *ux, R *uy)
{
    const R r = g[0] + g[1] + g[2] + g[3] + g[4] + g[5] + g[6] + g[7] + g[8];
    *rho = r;
    *ux = (g[1] - g[3] + g[5] - g[6] - g[7] + g[8]) / r;
    *uy = (g[2] - g[4] + g[5] + g[6] - g[7] - g[8]) / r;
}

static inline R FN(psi_of)(R rho, int form)
{
    if (form == LBO_PSI_REF) return (R)(4. * exp(-200. / (double)rho));
    return (R)1 - (sizeof(R) == sizeof(float) ? (R)lbo_expf((float)-rho) : (R)exp((double)-rho));
}

/* Shan-Chen interaction + adhesion force and BGK, the second launch of the
 * reference's D2Q9 collision (src/collision.cu:35-166).  The 3x3 psi and
 * solid stencils wrap periodically; row y+1 is physical -y. */
static void FN(d2q9_sc_pass)(float *plot, R *f, const uint8_t *solid, const R *ux,
                             const R *uy, const R *rho, const R *psi, const R *ueq_x,
                             const R *ueq_y, int W, int H, R w0, R w1, R w5, R tau_inv,
                             R G, R Gads)
{
    const long N = (long)W * H;
#pragma omp parallel for schedule(static)
    for (long o = 0; o < N; o++) {
        if (solid[o]) continue;
        const int x = (int)(o % W), y = (int)(o / W);
        const int xn = x > 0 ? x - 1 : W - 1, xp = x < W - 1 ? x + 1 : 0;
        const int yn = y > 0 ? y - 1 : H - 1, yp = y < H - 1 ? y + 1 : 0;
        long m[9];
        m[0] = (long)y * W + x;   m[1] = (long)y * W + xp;  m[2] = (long)yp * W + x;
        m[3] = (long)y * W + xn;  m[4] = (long)yn * W + x;  m[5] = (long)yp * W + xp;
        m[6] = (long)yp * W + xn; m[7] = (long)yn * W + xn; m[8] = (long)yn * W + xp;
        R IFx = 0, IFy = 0;
        IFx = IFx + w1 * psi[m[1]];
        IFx = IFx - w1 * psi[m[3]];
        IFx = IFx + w5 * psi[m[5]];
        IFx = IFx - w5 * psi[m[6]];
        IFx = IFx - w5 * psi[m[7]];
        IFx = IFx + w5 * psi[m[8]];
        IFy = IFy - w1 * psi[m[2]];
        IFy = IFy + w1 * psi[m[4]];
        IFy = IFy - w5 * psi[m[5]];
        IFy = IFy - w5 * psi[m[6]];
        IFy = IFy + w5 * psi[m[7]];
        IFy = IFy + w5 * psi[m[8]];
        IFx = -G * psi[o] * IFx;
        IFy = -G * psi[o] * IFy;
        R vx = ueq_x[o] + (IFx / (tau_inv * rho[o]));
        R vy = ueq_y[o] + (IFy / (tau_inv * rho[o]));
        if (Gads != 0) {
            R Fsx = 0, Fsy = 0;
            if (solid[m[1]]) Fsx = Fsx + w1;
            if (solid[m[2]]) Fsy = Fsy - w1;
            if (solid[m[3]]) Fsx = Fsx - w1;
            if (solid[m[4]]) Fsy = Fsy + w1;
            if (solid[m[5]]) { Fsx = Fsx + w5; Fsy = Fsy - w5; }
            if (solid[m[6]]) { Fsx = Fsx - w5; Fsy = Fsy - w5; }
            if (solid[m[7]]) { Fsx = Fsx - w5; Fsy = Fsy + w5; }
            if (solid[m[8]]) { Fsx = Fsx + w5; Fsy = Fsy + w5; }
            Fsx = -Gads * psi[o] * Fsx;
            Fsy = -Gads * psi[o] * Fsy;
            vx = vx + (Fsx / (tau_inv * rho[o]));
            vy = vy + (Fsy / (tau_inv * rho[o]));
        }
        if (plot) { plot[4 * o] = (float)ux[o]; plot[4 * o + 1] = (float)uy[o]; plot[4 * o + 2] = 0.f; plot[4 * o + 3] = (float)rho[o]; }
        R g[9];
        for (int k = 0; k < 9; k++) g[k] = f[k * N + o];
        FN(d2q9_bgk)(g, vx, vy, rho[o], w0, w1, w5, tau_inv);
        for (int k = 0; k < 9; k++) f[k * N + o] = g[k];
    }
}

/* The Shan-Chen pass in native mode (lattibol_0.3.31f_gb300/csrc/lb_d2q9.cu,
 * d2q9_sc_kernel<MODE_NATIVE>): the stencil sums grouped by sign
 * (d2q9_sc_shift_native), one division 1/(tau_inv rho) shared by the
 * interaction and the adhesion, FMA shifts, the native BGK. */
static void FN(d2q9_sc_pass_native)(R *f, const uint8_t *solid, const R *rho, const R *psi,
                                    const R *ueq_x, const R *ueq_y, int W, int H, R w0, R w1,
                                    R w5, R tau_inv, R G, R Gads)
{
    const long N = (long)W * H;
#pragma omp parallel for schedule(static)
    for (long o = 0; o < N; o++) {
        if (solid[o]) continue;
        const int x = (int)(o % W), y = (int)(o / W);
        const int xn = x > 0 ? x - 1 : W - 1, xp = x < W - 1 ? x + 1 : 0;
        const int yn = y > 0 ? y - 1 : H - 1, yp = y < H - 1 ? y + 1 : 0;
        long m[9];
        m[0] = (long)y * W + x;   m[1] = (long)y * W + xp;  m[2] = (long)yp * W + x;
        m[3] = (long)y * W + xn;  m[4] = (long)yn * W + x;  m[5] = (long)yp * W + xp;
        m[6] = (long)yp * W + xn; m[7] = (long)yn * W + xn; m[8] = (long)yn * W + xp;
        R ps[9];
        for (int k = 0; k < 9; k++) ps[k] = psi[m[k]];
        const R IFx = FMA_R(w1, ps[1] - ps[3], w5 * ((ps[5] + ps[8]) - (ps[6] + ps[7])));
        const R IFy = FMA_R(w1, ps[4] - ps[2], w5 * ((ps[7] + ps[8]) - (ps[5] + ps[6])));
        const R inv_rt = (R)1 / (tau_inv * rho[o]);
        const R c = (-G * ps[0]) * inv_rt;
        R vx = FMA_R(c, IFx, ueq_x[o]);
        R vy = FMA_R(c, IFy, ueq_y[o]);
        if (Gads != 0) {
            R Fsx = 0, Fsy = 0;
            if (solid[m[1]]) Fsx = Fsx + w1;
            if (solid[m[2]]) Fsy = Fsy - w1;
            if (solid[m[3]]) Fsx = Fsx - w1;
            if (solid[m[4]]) Fsy = Fsy + w1;
            if (solid[m[5]]) { Fsx = Fsx + w5; Fsy = Fsy - w5; }
            if (solid[m[6]]) { Fsx = Fsx - w5; Fsy = Fsy - w5; }
            if (solid[m[7]]) { Fsx = Fsx - w5; Fsy = Fsy + w5; }
            if (solid[m[8]]) { Fsx = Fsx + w5; Fsy = Fsy + w5; }
            const R ca = (-Gads * ps[0]) * inv_rt;
            vx = FMA_R(ca, Fsx, vx);
            vy = FMA_R(ca, Fsy, vy);
        }
        R g[9];
        for (int k = 0; k < 9; k++) g[k] = f[k * N + o];
        FN(d2q9_bgk_native)(g, vx, vy, rho[o], w0, w1, w5, tau_inv);
        for (int k = 0; k < 9; k++) f[k * N + o] = g[k];
    }
}

/* Collision launcher, src/collision.cu:168-355: first kernel (local swap,
 * Zou-He west inlet / east outlet, moments, force shift, BGK or -- if G != 0 --
 * psi/u_eq output without relaxation), then the Shan-Chen pass when G < 0. */
void FN(lbo_d2q9_collide)(float *plot, R *f, const uint8_t *solid, R *ux, R *uy, R *rho,
                          R *psi, R *ueq_x, R *ueq_y, int W, int H, int dev, int ndev, R w0,
                          R w1, R w5, R tau_inv, R ux_in, R uy_in, R rho_out, R Fx, R Fy,
                          R G, R Gads)
{
    (void)uy_in;
    const long N = (long)W * H;
#pragma omp parallel for schedule(static)
    for (long o = 0; o < N; o++) {
        const int x = (int)(o % W);
        if (solid[o]) {
            if (plot) { plot[4 * o] = 0.f; plot[4 * o + 1] = 0.f; plot[4 * o + 2] = 0.f; plot[4 * o + 3] = 0.f; }
            ux[o] = 0; uy[o] = 0; rho[o] = 0;
            continue;
        }
        R g[9];
        for (int k = 0; k < 9; k++) g[k] = f[k * N + o];
        for (int p = 0; p < 4; p++) {
            const int k = D2_POS[p], q = D2_OPP[k];
            R t = g[k]; g[k] = g[q]; g[q] = t;
        }
        if (x == 0 && dev == 0) {
            const R a = g[0] + g[2] + g[4], b = g[3] + g[7] + g[6];
            const R r = (R)(((double)a + 2. * (double)b) / (1. - (double)ux_in));
            const R ru = r * ux_in;
            g[1] = (R)((double)g[3] + (2. / 3.) * (double)ru);
            g[5] = (R)((double)g[7] + (1. / 6.) * (double)ru - 0.5 * (double)(g[2] - g[4]));
            g[8] = (R)((double)g[6] + (1. / 6.) * (double)ru - 0.5 * (double)(g[4] - g[2]));
        } else if (x == W - 1 && dev == ndev - 1) {
            const R a = g[0] + g[2] + g[4], b = g[1] + g[5] + g[8];
            const R vx = (R)(-1. + ((double)a + 2. * (double)b) / (double)rho_out);
            const R ru = rho_out * vx;
            g[3] = (R)((double)g[1] - (2. / 3.) * (double)ru);
            g[7] = (R)((double)g[5] - (1. / 6.) * (double)ru + 0.5 * (double)(g[2] - g[4]));
            g[6] = (R)((double)g[8] - (1. / 6.) * (double)ru + 0.5 * (double)(g[4] - g[2]));
        }
        R r, vx, vy;
        FN(d2q9_moments)(g, &r, &vx, &vy);
        R ex = vx, ey = vy;
        if (Fx != 0) ex = vx + Fx / (r * tau_inv);
        if (Fy != 0) ey = vy + Fy / (r * tau_inv);
        ux[o] = vx; uy[o] = vy; rho[o] = r;
        if (G != 0) {
            psi[o] = FN(psi_of)(r, LBO_PSI_REF);
            ueq_x[o] = ex;
            ueq_y[o] = ey;
        } else {
            if (plot) { plot[4 * o] = (float)vx; plot[4 * o + 1] = (float)vy; plot[4 * o + 2] = 0.f; plot[4 * o + 3] = (float)r; }
            FN(d2q9_bgk)(g, ex, ey, r, w0, w1, w5, tau_inv);
        }
        for (int k = 0; k < 9; k++) f[k * N + o] = g[k];
    }
    if (G < 0)
        FN(d2q9_sc_pass)(plot, f, solid, ux, uy, rho, psi, ueq_x, ueq_y, W, H, w0, w1, w5,
                         tau_inv, G, Gads);
}

/* ======================================================================== */
/* Native mode (no reference counterpart for the boundary handling):       */
/* periodic in every axis, half-way bounce-back at LBO_SOLID cells with the */
/* moving-wall momentum term corr[k] = 6 w_k (c_k . u_wall) at LBO_MOVING   */
/* cells, body force by the reference's velocity shift, optional Shan-Chen. */
/* Streaming keeps the reference's swap scheme: a pair that crosses a       */
/* fluid/wall link is not swapped, so the outgoing population stays in its */
/* slot and the collision's local swap turns it around (half-way BB).       */
/* ======================================================================== */

void FN(lbo_d3q19_stream_native)(R *f, const uint8_t *flags, const R *corr, int W, int H, int D)
{
    const long N = (long)W * H * D;
#pragma omp parallel for schedule(static)
    for (int z = 0; z < D; z++)
        for (int y = 0; y < H; y++)
            for (int x = 0; x < W; x++) {
                const long o = x + (long)y * W + (long)z * W * H;
                const int so = flags[o] & LBO_SOLID;
                for (int p = 0; p < 9; p++) {
                    const int k = D3_POS[p], q = D3_OPP[k];
                    const long on = wrapi(x + D3_CX[k], W) + (long)wrapi(y + D3_CY[k], H) * W +
                                    (long)wrapi(z + D3_CZ[k], D) * W * H;
                    const int sn = flags[on] & LBO_SOLID;
                    if (!so && !sn) {
                        R t = f[k * N + o];
                        f[k * N + o] = f[q * N + on];
                        f[q * N + on] = t;
                    } else if (!so) {
                        if (flags[on] & LBO_MOVING) f[k * N + o] = f[k * N + o] - corr[k];
                    } else if (!sn) {
                        if (flags[o] & LBO_MOVING) f[q * N + on] = f[q * N + on] - corr[q];
                    }
                }
            }
}

/* Native collision: local swap, moments, body-force velocity shift (the form
 * of src/collision.cu:280-284), optional Shan-Chen force on the 18-neighbour
 * stencil (psi of the post-stream density), BGK.  Moment pointers may be NULL. */
/* dev != 0: f holds the deviations d_k = f_k - wr_k of 16-bit storage and the
 * step uses the deviation arithmetic (wr: per-direction offsets, rho_off =
 * their sum) */
static void FN(d3q19_collide_native_impl)(R *f, const uint8_t *flags, R *ux, R *uy, R *uz,
                                          R *rho, R *psi, int W, int H, int D, R w0, R w1,
                                          R w7, R tau_inv, R Fx, R Fy, R Fz, R G, int psi_form,
                                          int dev, R rho_off, const R *wr)
{
    const long N = (long)W * H * D;
    const int sc = (G != 0) && psi;
    if (sc) {
#pragma omp parallel for schedule(static)
        for (long o = 0; o < N; o++) {
            if (flags[o] & LBO_SOLID) { psi[o] = 0; continue; }
            /* post-stream populations sit in the opposite slots before the
             * local swap; the density in the native moments' association */
            R g[19];
            g[0] = f[o];
            for (int k = 1; k < 19; k++) g[k] = f[D3_OPP[k] * N + o];
            const R r = dev ? rho_off + FN(d3q19_rho_native)(g) : FN(d3q19_rho_native)(g);
            psi[o] = FN(psi_of)(r, psi_form);
        }
    }
#pragma omp parallel for schedule(static)
    for (long o = 0; o < N; o++) {
        if (flags[o] & LBO_SOLID) {
            if (rho) { ux[o] = 0; uy[o] = 0; uz[o] = 0; rho[o] = 0; }
            continue;
        }
        R g[19];
        for (int k = 0; k < 19; k++) g[k] = f[k * N + o];
        for (int p = 0; p < 9; p++) {
            const int k = D3_POS[p], q = D3_OPP[k];
            R t = g[k]; g[k] = g[q]; g[q] = t;
        }
        R r, vx, vy, vz;
        if (dev) FN(d3q19_moments_dev)(g, rho_off, &r, &vx, &vy, &vz);
        else FN(d3q19_moments_native)(g, &r, &vx, &vy, &vz);
        R ex = vx, ey = vy, ez = vz;
        if (sc || Fx != 0 || Fy != 0 || Fz != 0) {
            const R inv_rt = (R)1 / (r * tau_inv);
            if (Fx != 0) ex = FMA_R(Fx, inv_rt, vx);
            if (Fy != 0) ey = FMA_R(Fy, inv_rt, vy);
            if (Fz != 0) ez = FMA_R(Fz, inv_rt, vz);
            if (sc) {
                const int x = (int)(o % W), y = (int)((o / W) % H), z = (int)(o / ((long)W * H));
                R ps[19];
                for (int k = 0; k < 19; k++)
                    ps[k] = psi[wrapi(x + D3_CX[k], W) + (long)wrapi(y + D3_CY[k], H) * W +
                                (long)wrapi(z + D3_CZ[k], D) * W * H];
                R IFx, IFy, IFz;
                FN(d3q19_sc_sum_native)(ps, w1, w7, &IFx, &IFy, &IFz);
                const R c = (-G * ps[0]) * inv_rt;
                ex = FMA_R(c, IFx, ex);
                ey = FMA_R(c, IFy, ey);
                ez = FMA_R(c, IFz, ez);
            }
        }
        if (rho) { ux[o] = vx; uy[o] = vy; uz[o] = vz; rho[o] = r; }
        if (dev) FN(d3q19_bgk_dev)(g, ex, ey, ez, r, w0, w1, w7, tau_inv, wr[0], wr[1], wr[7]);
        else FN(d3q19_bgk_native)(g, ex, ey, ez, r, w0, w1, w7, tau_inv);
        for (int k = 0; k < 19; k++) f[k * N + o] = g[k];
    }
}

void FN(lbo_d3q19_collide_native)(R *f, const uint8_t *flags, R *ux, R *uy, R *uz, R *rho,
                                  R *psi, int W, int H, int D, R w0, R w1, R w7, R tau_inv,
                                  R Fx, R Fy, R Fz, R G, int psi_form)
{
    FN(d3q19_collide_native_impl)(f, flags, ux, uy, uz, rho, psi, W, H, D, w0, w1, w7, tau_inv,
                                  Fx, Fy, Fz, G, psi_form, 0, (R)0, NULL);
}

void FN(lbo_d3q19_collide_native_dev)(R *d, const uint8_t *flags, R *ux, R *uy, R *uz, R *rho,
                                      R *psi, int W, int H, int D, R w0, R w1, R w7, R tau_inv,
                                      R Fx, R Fy, R Fz, R G, int psi_form, R rho_off,
                                      const R *wr)
{
    FN(d3q19_collide_native_impl)(d, flags, ux, uy, uz, rho, psi, W, H, D, w0, w1, w7, tau_inv,
                                  Fx, Fy, Fz, G, psi_form, 1, rho_off, wr);
}

void FN(lbo_d2q9_stream_native)(R *f, const uint8_t *flags, const R *corr, int W, int H)
{
    const long N = (long)W * H;
#pragma omp parallel for schedule(static)
    for (int y = 0; y < H; y++)
        for (int x = 0; x < W; x++) {
            const long o = x + (long)y * W;
            const int so = flags[o] & LBO_SOLID;
            for (int p = 0; p < 4; p++) {
                const int k = D2_POS[p], q = D2_OPP[k];
                const long on = wrapi(x + D2_CX[k], W) + (long)wrapi(y + D2_CR[k], H) * W;
                const int sn = flags[on] & LBO_SOLID;
                if (!so && !sn) {
                    R t = f[k * N + o];
                    f[k * N + o] = f[q * N + on];
                    f[q * N + on] = t;
                } else if (!so) {
                    if (flags[on] & LBO_MOVING) f[k * N + o] = f[k * N + o] - corr[k];
                } else if (!sn) {
                    if (flags[o] & LBO_MOVING) f[q * N + on] = f[q * N + on] - corr[q];
                }
            }
        }
}

/* Native D2Q9 collision, in the native arithmetic (d2q9_moments_native,
 * d2q9_bgk_native).  With Shan-Chen: the reference's two-pass structure
 * (moments, psi, u_eq; then the Shan-Chen pass, d2q9_sc_pass_native) without
 * Zou-He, with psi defined (0) at wall cells, the psi form selectable, and
 * the interaction applied for any G != 0. */
void FN(lbo_d2q9_collide_native)(R *f, const uint8_t *flags, R *ux, R *uy, R *rho, R *psi,
                                 int W, int H, R w0, R w1, R w5, R tau_inv, R Fx, R Fy, R G,
                                 R Gads, int psi_form)
{
    const long N = (long)W * H;
    const int sc = (G != 0);
    R *ex_buf = NULL, *ey_buf = NULL, *r_buf = NULL;
    uint8_t *solid = NULL;
    if (sc) {
        ex_buf = (R *)malloc(sizeof(R) * N);
        ey_buf = (R *)malloc(sizeof(R) * N);
        r_buf = (R *)malloc(sizeof(R) * N);
        solid = (uint8_t *)malloc(N);
        for (long o = 0; o < N; o++) solid[o] = (flags[o] & LBO_SOLID) ? 1 : 0;
    }
#pragma omp parallel for schedule(static)
    for (long o = 0; o < N; o++) {
        if (flags[o] & LBO_SOLID) {
            if (rho) { ux[o] = 0; uy[o] = 0; rho[o] = 0; }
            if (sc) { psi[o] = 0; r_buf[o] = 0; ex_buf[o] = 0; ey_buf[o] = 0; }
            continue;
        }
        R g[9];
        for (int k = 0; k < 9; k++) g[k] = f[k * N + o];
        for (int p = 0; p < 4; p++) {
            const int k = D2_POS[p], q = D2_OPP[k];
            R t = g[k]; g[k] = g[q]; g[q] = t;
        }
        R r, vx, vy;
        if (!sc) {
            /* without Shan-Chen: the native arithmetic, one division for
             * 1/(rho tau_inv) in the force shift */
            FN(d2q9_moments_native)(g, &r, &vx, &vy);
            R ex = vx, ey = vy;
            if (Fx != 0 || Fy != 0) {
                const R inv_rt = (R)1 / (r * tau_inv);
                if (Fx != 0) ex = FMA_R(Fx, inv_rt, vx);
                if (Fy != 0) ey = FMA_R(Fy, inv_rt, vy);
            }
            if (rho) { ux[o] = vx; uy[o] = vy; rho[o] = r; }
            FN(d2q9_bgk_native)(g, ex, ey, r, w0, w1, w5, tau_inv);
            for (int k = 0; k < 9; k++) f[k * N + o] = g[k];
            continue;
        }
        /* with Shan-Chen: the native moments and force shift, then psi and
         * u_eq for the native Shan-Chen pass */
        FN(d2q9_moments_native)(g, &r, &vx, &vy);
        R ex = vx, ey = vy;
        if (Fx != 0 || Fy != 0) {
            const R inv_rt = (R)1 / (r * tau_inv);
            if (Fx != 0) ex = FMA_R(Fx, inv_rt, vx);
            if (Fy != 0) ey = FMA_R(Fy, inv_rt, vy);
        }
        if (rho) { ux[o] = vx; uy[o] = vy; rho[o] = r; }
        psi[o] = FN(psi_of)(r, psi_form);
        r_buf[o] = r; ex_buf[o] = ex; ey_buf[o] = ey;
        for (int k = 0; k < 9; k++) f[k * N + o] = g[k];
    }
    if (sc) {
        FN(d2q9_sc_pass_native)(f, solid, r_buf, psi, ex_buf, ey_buf, W, H, w0, w1, w5, tau_inv,
                                G, Gads);
        free(ex_buf); free(ey_buf); free(r_buf); free(solid);
    }
}

/* Equilibrium populations from (rho, u), in the operation order of the BGK
 * equilibrium above (src/simulation_d3q19.cu:104-122 for the uniform case). */
void FN(lbo_d3q19_equilibrium)(R *f, const R *rho, const R *ux, const R *uy, const R *uz,
                               long N, R w0, R w1, R w7)
{
#pragma omp parallel for schedule(static)
    for (long o = 0; o < N; o++) {
        R g[19];
        /* BGK with tau_inv = 1 from zero populations gives f_eq exactly:
         * 0 - 1*(0 - feq) = feq */
        for (int k = 0; k < 19; k++) g[k] = 0;
        FN(d3q19_bgk)(g, ux[o], uy[o], uz[o], rho[o], w0, w1, w7, (R)1);
        for (int k = 0; k < 19; k++) f[k * N + o] = g[k];
    }
}

void FN(lbo_d2q9_equilibrium)(R *f, const R *rho, const R *ux, const R *uy, long N, R w0,
                              R w1, R w5)
{
#pragma omp parallel for schedule(static)
    for (long o = 0; o < N; o++) {
        R g[9];
        for (int k = 0; k < 9; k++) g[k] = 0;
        FN(d2q9_bgk)(g, ux[o], uy[o], rho[o], w0, w1, w5, (R)1);
        for (int k = 0; k < 9; k++) f[k * N + o] = g[k];
    }
}

#undef FN
#undef CAT_
#undef CAT2_
