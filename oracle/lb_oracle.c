/*
 * lb_oracle.c -- CPU oracle for the lattice Boltzmann hot path (TEST
 * INFRASTRUCTURE ONLY: loaded by tests/, __graft_entry__.smoke() and the CPU
 * baseline leg of bench.py to verify results against or to time the
 * reference's loop, never by the GPU library).
 *
 * Build: oracle/Makefile (gcc -O2 -fopenmp -ffp-contract=off).  FP
 * contraction must stay off so that the float instantiation performs the
 * reference kernels' float operations one by one.
 *
 * Lattice tables follow the reference:
 *   D3Q19 velocities: src/collision.cu:463-478 (moments) and the streaming
 *   pairs of src/streaming.cu:116-161.
 *   D2Q9 velocities (row index grows downwards, +y = row-1):
 *   src/streaming.cu:44-68 and src/collision.cu:264-275.
 */
#include "lb_oracle.h"

#include <math.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

/* D3Q19: k = 0..18 */
static const int D3_CX[19] = {0, 1, -1, 0, 0, 0, 0, 1, 1, 1, 1, -1, -1, -1, -1, 0, 0, 0, 0};
static const int D3_CY[19] = {0, 0, 0, 1, -1, 0, 0, 1, -1, 0, 0, 1, -1, 0, 0, 1, 1, -1, -1};
static const int D3_CZ[19] = {0, 0, 0, 0, 0, 1, -1, 0, 0, 1, -1, 0, 0, 1, -1, 1, -1, 1, -1};
static const int D3_OPP[19] = {0, 2, 1, 4, 3, 6, 5, 12, 11, 14, 13, 8, 7, 10, 9, 18, 17, 16, 15};
/* the slot of each swap pair that the owning node holds (src/streaming.cu:127-161) */
static const int D3_POS[9] = {1, 3, 5, 7, 8, 9, 10, 15, 16};

/* D2Q9: x offset and ROW offset of each velocity (physical c_y = -row offset) */
static const int D2_CX[9] = {0, 1, 0, -1, 0, 1, -1, -1, 1};
static const int D2_CR[9] = {0, 0, -1, 0, 1, -1, -1, 1, 1};
static const int D2_OPP[9] = {0, 3, 4, 1, 2, 7, 8, 5, 6};
static const int D2_POS[4] = {1, 2, 5, 6};

static inline int wrapi(int v, int n) { return v < 0 ? v + n : (v >= n ? v - n : v); }

static inline float bits_to_float(uint32_t u) { float v; memcpy(&v, &u, 4); return v; }

/* exp in float by the GPU library's method (Cody-Waite reduction by ln 2 with
 * a 12-bit head, degree-7 Taylor polynomial by Horner, scaling by 2^k): the
 * same operations in the same order, one rounding each, so that psi =
 * 1 - exp(-rho) is bit-identical on both sides.  Accuracy is checked against
 * libm by tests/test_oracle_storage.py. */
float lbo_expf(float x)
{
    if (x < -103.f) return 0.f;
    if (x > 88.7f) return bits_to_float(0x7f800000u);
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
    if (ki >= -126) return p * bits_to_float((uint32_t)(ki + 127) << 23);
    return (p * bits_to_float((uint32_t)(ki + 64 + 127) << 23)) * 0x1p-64f;
}

#define R float
#define S f32
#define FMA_R fmaf
#include "lb_oracle_body.h"
#undef R
#undef S
#undef FMA_R

#define R double
#define S f64
#define FMA_R fma
#include "lb_oracle_body.h"
#undef R
#undef S
#undef FMA_R

/* solid_bound = node and all 8 neighbours solid, for x in 1..W-2 only and
 * periodic in y (src/simulation_d2q9.cu:318-334) */
void lbo_d2q9_solid_bound(const uint8_t *solid, uint8_t *sb, int W, int H)
{
    memset(sb, 0, (size_t)W * H);
    for (int y = 0; y < H; y++)
        for (int x = 1; x < W - 1; x++) {
            const int yn = y > 0 ? y - 1 : H - 1, yp = y < H - 1 ? y + 1 : 0;
            int all = 1;
            for (int dy = 0; dy < 3 && all; dy++)
                for (int dx = -1; dx <= 1 && all; dx++) {
                    const int yy = dy == 0 ? y : (dy == 1 ? yp : yn);
                    if (!solid[(x + dx) + (long)yy * W]) all = 0;
                }
            sb[x + (long)y * W] = (uint8_t)all;
        }
}

/* solid_bound = node and all 18 neighbours solid, x in 1..W-2, periodic in y
 * and z (src/simulation_d3q19.cu:167-204) */
void lbo_d3q19_solid_bound(const uint8_t *solid, uint8_t *sb, int W, int H, int D)
{
    memset(sb, 0, (size_t)W * H * D);
    for (int z = 0; z < D; z++)
        for (int y = 0; y < H; y++)
            for (int x = 1; x < W - 1; x++) {
                int all = 1;
                for (int k = 0; k < 19 && all; k++) {
                    const long on = (x + D3_CX[k]) + (long)wrapi(y + D3_CY[k], H) * W +
                                    (long)wrapi(z + D3_CZ[k], D) * W * H;
                    if (!solid[on]) all = 0;
                }
                sb[x + (long)y * W + (long)z * W * H] = (uint8_t)all;
            }
}

/* border pack, src/get_border.cu:26-50: border = {f1, f5, f8 at x=W-1; f3, f6, f7 at x=0} */
void lbo_d2q9_get_border(const float *f, float *const border[6], int W, int H)
{
    const long N = (long)W * H;
    static const int kk[6] = {1, 5, 8, 3, 6, 7};
    for (int y = 0; y < H; y++)
        for (int j = 0; j < 6; j++) {
            const int x = j < 3 ? W - 1 : 0;
            border[j][y] = f[kk[j] * N + x + (long)y * W];
        }
}

/* border unpack, src/apply_border.cu:25-48: x=0 gets f3,f6,f7; x=W-1 gets f1,f5,f8 */
void lbo_d2q9_apply_border(float *f, const float *const nb[6], int W, int H)
{
    const long N = (long)W * H;
    static const int kk[6] = {1, 5, 8, 3, 6, 7};
    for (int y = 0; y < H; y++) {
        for (int j = 3; j < 6; j++) f[kk[j] * N + 0 + (long)y * W] = nb[j][y];
        if (W >= 1)
            for (int j = 0; j < 3; j++) f[kk[j] * N + (W - 1) + (long)y * W] = nb[j][y];
    }
}

/* border pack, src/get_border.cu:59-98: {f1,f7,f8,f9,f10 at x=W-1; f2,f11,f12,f13,f14 at x=0},
 * face index y + z*H */
void lbo_d3q19_get_border(const float *f, float *const border[10], int W, int H, int D)
{
    const long N = (long)W * H * D;
    static const int kk[10] = {1, 7, 8, 9, 10, 2, 11, 12, 13, 14};
    for (int z = 0; z < D; z++)
        for (int y = 0; y < H; y++)
            for (int j = 0; j < 10; j++) {
                const int x = j < 5 ? W - 1 : 0;
                border[j][y + (long)z * H] = f[kk[j] * N + x + (long)y * W + (long)z * W * H];
            }
}

/* border unpack, src/apply_border.cu:58-97 */
void lbo_d3q19_apply_border(float *f, const float *const nb[10], int W, int H, int D)
{
    const long N = (long)W * H * D;
    static const int kk[10] = {1, 7, 8, 9, 10, 2, 11, 12, 13, 14};
    for (int z = 0; z < D; z++)
        for (int y = 0; y < H; y++) {
            for (int j = 5; j < 10; j++)
                f[kk[j] * N + 0 + (long)y * W + (long)z * W * H] = nb[j][y + (long)z * H];
            for (int j = 0; j < 5; j++)
                f[kk[j] * N + (W - 1) + (long)y * W + (long)z * W * H] = nb[j][y + (long)z * H];
        }
}

/* cursor probe, src/read_value.cu:27-34 */
void lbo_read_value(const float *plot, float value[4], int W, int H, int x, int y, int z)
{
    const long o = x + (long)y * W + (long)z * W * H;
    for (int i = 0; i < 4; i++) value[i] = plot[4 * o + i];
}

void lbo_reduce_f32(const float *rho, const float *ux, const float *uy, const float *uz,
                    const uint8_t *solid, long N, double out[7])
{
    double m = 0, px = 0, py = 0, pz = 0, ke = 0, umax = 0, nf = 0;
    for (long o = 0; o < N; o++) {
        if (solid && solid[o]) continue;
        const double r = rho[o], vx = ux[o], vy = uy[o], vz = uz ? uz[o] : 0.0;
        const double u2 = vx * vx + vy * vy + vz * vz;
        m += r; px += r * vx; py += r * vy; pz += r * vz; ke += 0.5 * r * u2;
        if (sqrt(u2) > umax) umax = sqrt(u2);
        nf += 1;
    }
    out[0] = m; out[1] = px; out[2] = py; out[3] = pz; out[4] = ke; out[5] = umax; out[6] = nf;
}

/* IEEE binary16 / bfloat16 conversions with round-to-nearest-even, written
 * from the format definitions (NaN inputs become a quiet NaN). */
uint16_t lbo_f32_to_f16(float v)
{
    uint32_t u; memcpy(&u, &v, 4);
    const uint32_t sign = (u >> 16) & 0x8000u;
    const uint32_t absu = u & 0x7fffffffu;
    if (absu >= 0x7f800000u) return (uint16_t)(sign | (absu > 0x7f800000u ? 0x7e00u : 0x7c00u));
    if (absu >= 0x477ff000u) return (uint16_t)(sign | 0x7c00u); /* rounds to >= 65520 -> inf */
    if (absu < 0x38800000u) {                                  /* result is subnormal or zero */
        if (absu < 0x33000000u) return (uint16_t)sign;         /* below half of the smallest subnormal */
        const uint32_t e = absu >> 23;                         /* biased exponent, 102..112 */
        const uint32_t mant = (absu & 0x7fffffu) | 0x800000u;
        const uint32_t shift = 126 - e;                        /* value = mant * 2^(e-150); unit = 2^-24 */
        uint32_t q = mant >> shift;
        const uint32_t rem = mant & ((1u << shift) - 1u), half = 1u << (shift - 1);
        if (rem > half || (rem == half && (q & 1u))) q++;
        return (uint16_t)(sign | q);
    }
    uint32_t r = absu - 0x38000000u;                           /* rebias 127 -> 15 (in place) */
    uint32_t q = r >> 13;
    const uint32_t rem = r & 0x1fffu;
    if (rem > 0x1000u || (rem == 0x1000u && (q & 1u))) q++;
    return (uint16_t)(sign | q);
}

float lbo_f16_to_f32(uint16_t h)
{
    const uint32_t sign = ((uint32_t)h & 0x8000u) << 16;
    uint32_t e = (h >> 10) & 0x1fu, m = h & 0x3ffu, u;
    if (e == 0x1f) u = sign | 0x7f800000u | (m << 13);
    else if (e == 0) {
        if (m == 0) u = sign;
        else {
            int sh = 0;
            while (!(m & 0x400u)) { m <<= 1; sh++; }
            m &= 0x3ffu;
            u = sign | ((uint32_t)(113 - sh) << 23) | (m << 13);
        }
    } else u = sign | ((e + 112u) << 23) | (m << 13);
    float v; memcpy(&v, &u, 4);
    return v;
}

uint16_t lbo_f32_to_bf16(float v)
{
    uint32_t u; memcpy(&u, &v, 4);
    if ((u & 0x7fffffffu) > 0x7f800000u) return (uint16_t)((u >> 16) | 0x40u);
    const uint32_t rem = u & 0xffffu;
    uint32_t q = u >> 16;
    if (rem > 0x8000u || (rem == 0x8000u && (q & 1u))) q++;
    return (uint16_t)q;
}

float lbo_bf16_to_f32(uint16_t h)
{
    uint32_t u = (uint32_t)h << 16;
    float v; memcpy(&v, &u, 4);
    return v;
}

void lbo_round_storage(float *f, long n, int kind)
{
    for (long i = 0; i < n; i++)
        f[i] = kind == 1 ? lbo_f16_to_f32(lbo_f32_to_f16(f[i])) : lbo_bf16_to_f32(lbo_f32_to_bf16(f[i]));
}

void lbo_quantize_dev(float *f, int Q, long N, const float *wr, const uint8_t *flags, int kind)
{
#pragma omp parallel for schedule(static)
    for (long o = 0; o < N; o++) {
        if (flags && (flags[o] & LBO_SOLID)) continue;
        for (int k = 0; k < Q; k++) {
            const float d = f[(long)k * N + o] - wr[k];
            const float q = kind == 1 ? lbo_f16_to_f32(lbo_f32_to_f16(d))
                                      : lbo_bf16_to_f32(lbo_f32_to_bf16(d));
            f[(long)k * N + o] = wr[k] + q;
        }
    }
}

int lbo_num_threads(void)
{
#ifdef _OPENMP
    return omp_get_max_threads();
#else
    return 1;
#endif
}

void lbo_set_threads(int n)
{
#ifdef _OPENMP
    if (n > 0) omp_set_num_threads(n);
#else
    (void)n;
#endif
}
