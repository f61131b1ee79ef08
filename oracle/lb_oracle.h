/*
 * lb_oracle.h -- CPU oracle for the lattice Boltzmann hot path.
 *
 * TEST INFRASTRUCTURE ONLY.  This is a plain-C restatement of the per-step
 * update of lattibol (streaming + collision + Shan-Chen force step + border
 * pack/unpack + cursor probe).  Only the tests, the smoke check and the CPU
 * baseline leg of the benchmark load it, only to verify results against or to
 * time the reference's loop.  The GPU
 * library never links against it.
 *
 * Every routine exists twice: *_f32 computes in float with the exact
 * operation order and float->double promotions of the reference kernels (so
 * it is bit-identical to them when compiled without FP contraction), *_f64 is
 * the same algorithm in double (the FP64 oracle used for error statements).
 *
 * Population layout: structure of arrays, f[k*N + node], node = x + y*W +
 * z*W*H (the reference's `offset`, src/streaming.cu:98).  D2Q9 uses the
 * reference's flipped y axis (+y = row-1, src/streaming.cu:48).
 *
 * Pinning: tests/test_oracle_pin.py checks *_f32 bit-exactly against the
 * reference's own kernels compiled for the host (oracle/_ref, recipe in
 * oracle/Makefile) and tests/test_golden.py against fixtures generated from
 * them (tests/golden/make_golden.py).
 */
#ifndef LB_ORACLE_H
#define LB_ORACLE_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* cell flags of the native (non-reference) mode */
#define LBO_SOLID  0x01u  /* wall cell: half-way bounce-back for its fluid neighbours */
#define LBO_MOVING 0x02u  /* wall cell that moves with the lid velocity (set with LBO_SOLID) */

/* psi(rho) forms of the Shan-Chen pseudo-potential */
#define LBO_PSI_REF  0    /* 4*exp(-200/rho) in double, src/collision.cu:293 */
#define LBO_PSI_EXP1 1    /* 1-exp(-rho), float */

/* ---- reference semantics ------------------------------------------------ */
void lbo_d2q9_solid_bound(const uint8_t *solid, uint8_t *solid_bound, int W, int H);
void lbo_d3q19_solid_bound(const uint8_t *solid, uint8_t *solid_bound, int W, int H, int D);

#define LBO_DECL(S, R)                                                                    \
void lbo_d3q19_stream_##S(R *f, const uint8_t *solid_bound, int W, int H, int D);         \
void lbo_d3q19_collide_##S(float *plot, R *f, const uint8_t *solid, R *ux, R *uy, R *uz,  \
    R *rho, int W, int H, int D, int dev, int ndev, R w0, R w1, R w7, R tau_inv,          \
    R ux_in, R uy_in, R uz_in, R rho_out);                                                \
void lbo_d2q9_stream_##S(R *f, const uint8_t *solid_bound, int W, int H);                 \
void lbo_d2q9_collide_##S(float *plot, R *f, const uint8_t *solid, R *ux, R *uy, R *rho,  \
    R *psi, R *ueq_x, R *ueq_y, int W, int H, int dev, int ndev, R w0, R w1, R w5,        \
    R tau_inv, R ux_in, R uy_in, R rho_out, R Fx, R Fy, R G, R Gads);                     \
/* ---- native mode: periodic, half-way bounce-back, moving walls, body force ---- */     \
void lbo_d3q19_stream_native_##S(R *f, const uint8_t *flags, const R *corr, int W,       \
    int H, int D);                                                                        \
void lbo_d3q19_collide_native_##S(R *f, const uint8_t *flags, R *ux, R *uy, R *uz,        \
    R *rho, R *psi, int W, int H, int D, R w0, R w1, R w7, R tau_inv, R Fx, R Fy, R Fz,   \
    R G, int psi_form);                                                                   \
/* 16-bit storage: the same step on the deviations d_k = f_k - wr_k */                  \
void lbo_d3q19_collide_native_dev_##S(R *d, const uint8_t *flags, R *ux, R *uy, R *uz,    \
    R *rho, R *psi, int W, int H, int D, R w0, R w1, R w7, R tau_inv, R Fx, R Fy, R Fz,   \
    R G, int psi_form, R rho_off, const R *wr);                                           \
void lbo_d2q9_stream_native_##S(R *f, const uint8_t *flags, const R *corr, int W, int H); \
void lbo_d2q9_collide_native_##S(R *f, const uint8_t *flags, R *ux, R *uy, R *rho,        \
    R *psi, int W, int H, R w0, R w1, R w5, R tau_inv, R Fx, R Fy, R G, R Gads,           \
    int psi_form);                                                                        \
void lbo_d3q19_equilibrium_##S(R *f, const R *rho, const R *ux, const R *uy,              \
    const R *uz, long N, R w0, R w1, R w7);                                               \
void lbo_d2q9_equilibrium_##S(R *f, const R *rho, const R *ux, const R *uy, long N,       \
    R w0, R w1, R w5);

LBO_DECL(f32, float)
LBO_DECL(f64, double)
#undef LBO_DECL

/* border pack/unpack and cursor probe (pure copies; float only) */
void lbo_d2q9_get_border(const float *f, float *const border[6], int W, int H);
void lbo_d2q9_apply_border(float *f, const float *const nb_border[6], int W, int H);
void lbo_d3q19_get_border(const float *f, float *const border[10], int W, int H, int D);
void lbo_d3q19_apply_border(float *f, const float *const nb_border[10], int W, int H, int D);
void lbo_read_value(const float *plot, float value[4], int W, int H, int x, int y, int z);

/* global sums over fluid cells (solid_or_flags != 0 excluded), accumulated in
 * double: out = {mass, mom_x, mom_y, mom_z, kinetic energy, max|u|, n_fluid} */
void lbo_reduce_f32(const float *rho, const float *ux, const float *uy, const float *uz,
                    const uint8_t *solid_or_flags, long N, double out[7]);

/* float <-> half / bfloat16, round to nearest even (storage emulation) */
uint16_t lbo_f32_to_f16(float v);
float lbo_f16_to_f32(uint16_t h);
uint16_t lbo_f32_to_bf16(float v);
float lbo_bf16_to_f32(uint16_t h);
void lbo_round_storage(float *f, long n, int kind /* 1 = f16, 2 = bf16 */);
/* emulate 16-bit deviation storage of a float population state: for every
 * node with (flags == NULL || !(flags[o] & LBO_SOLID)) and every k,
 * f[k][o] = wr[k] + widen(narrow_rne(f[k][o] - wr[k])), all in float */
void lbo_quantize_dev(float *f, int Q, long N, const float *wr, const uint8_t *flags, int kind);

/* exp in float by the GPU library's own method (same operations) */
float lbo_expf(float x);

int lbo_num_threads(void);
void lbo_set_threads(int n);

#ifdef __cplusplus
}
#endif
#endif
