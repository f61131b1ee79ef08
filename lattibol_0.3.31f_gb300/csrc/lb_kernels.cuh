// lb_kernels.cuh -- kernel argument bundles and launcher prototypes shared by
// the kernel files (lb_d3q19.cu, lb_d2q9.cu, lb_reduce.cu) and the host layers
// (lb_abi.cu, lb_context.cu).
#pragma once

#include <cuda.h>

#include "lb_common.cuh"
#include "lb_mlp.cuh"

namespace lb {

enum { MODE_REF = 0, MODE_NATIVE = 1 };

constexpr int D3_BLOCK = 128;  // threads per block along x (D3Q19)
constexpr int D2_BLOCK = 128;  // threads per block along x (D2Q9)

struct D3Args {
    CPop<19> src;           // populations at the start of the step
    Pop<19> dst;            // populations after the step (== src for in-place kernels)
    const uint8_t *flags;   // native: CELL_* bits; reference: the solid array (0/1)
    const uint8_t *sb;      // reference: solid_bound (0/1)
    float *ux, *uy, *uz, *rho;
    float4 *plot;
    int W, H, D, dev, ndev;
    int reverse;            // sweep the blocks in reverse order (L2 reuse across steps)
    float w0, w1, w7, tau_inv, ux_in, rho_out, Fx, Fy, Fz;
    float corr[19];         // moving-wall momentum term per direction
    float wr[19];           // 16-bit storage: offsets w_k * rho_ref of the stored deviations
    float *psi;             // Shan-Chen: pseudo-potential of the current step (density pass)
    float G;                // Shan-Chen interaction strength
    int psi_form;           // LB_PSI_REF or LB_PSI_EXP1
    float4 *probe;          // when set: (ux, uy, uz, rho) of node probe_o, every step
    int probe_o;            // (mapped host memory: the cursor read without a sync)
    int *err;               // device error word of a kernel that waits on the GPU (or null)
    int z_lo, z_skip;       // planes updated: z = z_lo + blockIdx.z * (1 + z_skip) (slabs;
                            // 0, 0 = every plane, blockIdx.z itself)
    float rho_ref;          // 16-bit storage: sum_k wr[k], the density the offsets carry
};

// The native step's arithmetic for storage type S: FP32 works on f itself,
// 16-bit storage on the deviations d_k = f_k - w_k rho_ref (lb_common.cuh).
template <typename S> struct StepArith {
    __device__ __forceinline__ static float rho(const float (&g)[19], const D3Args &) {
        return d3q19_rho_native(g);
    }
    __device__ __forceinline__ static void moments(const float (&g)[19], const D3Args &,
                                                   float &rho, float &ux, float &uy, float &uz) {
        d3q19_moments_native(g, rho, ux, uy, uz);
    }
    __device__ __forceinline__ static void bgk(float (&g)[19], float ux, float uy, float uz,
                                               float rho, const D3Args &a, float tau_inv) {
        d3q19_bgk_native(g, ux, uy, uz, rho, a.w0, a.w1, a.w7, tau_inv);
    }
};
template <typename S> struct StepArithDev {
    __device__ __forceinline__ static float rho(const float (&d)[19], const D3Args &a) {
        return d3q19_rho_dev(d, a.rho_ref);
    }
    __device__ __forceinline__ static void moments(const float (&d)[19], const D3Args &a,
                                                   float &rho, float &ux, float &uy, float &uz) {
        d3q19_moments_dev(d, a.rho_ref, rho, ux, uy, uz);
    }
    __device__ __forceinline__ static void bgk(float (&d)[19], float ux, float uy, float uz,
                                               float rho, const D3Args &a, float tau_inv) {
        d3q19_bgk_dev(d, ux, uy, uz, rho, a.w0, a.w1, a.w7, tau_inv, a.wr[0], a.wr[1], a.wr[7]);
    }
};
template <> struct StepArith<__half> : StepArithDev<__half> {};
template <> struct StepArith<__nv_bfloat16> : StepArithDev<__nv_bfloat16> {};

struct D2Args {
    CPop<9> src;
    Pop<9> dst;
    const uint8_t *flags;
    const uint8_t *sb;
    float *ux, *uy, *rho;
    float4 *plot;
    float *psi, *ueq_x, *ueq_y;
    int W, H, dev, ndev;
    int reverse;
    float w0, w1, w5, tau_inv, ux_in, rho_out, Fx, Fy, G, Gads;
    int psi_form;
    float corr[9];
    float4 *probe;          // as D3Args: (ux, uy, 0, rho) of node probe_o every step
    int probe_o;
};

// D3Q19
cudaError_t launch_d3q19_fused(const D3Args &a, int mode, bool mom, bool plot, cudaStream_t s);
// native mode with storage kind (0 f32, 1 f16, 2 bf16) and optional Shan-Chen
// (sc: the density pass writing a.psi, then the fused step reading it)
cudaError_t launch_d3q19_native(const D3Args &a, int storage, bool mom, bool sc, cudaStream_t s);
// the native step (no Shan-Chen) of `nplanes` planes z = z_lo + i * (1 + z_skip),
// i < nplanes, of a z-slab whose ghost planes hold the neighbours' faces
cudaError_t launch_d3q19_native_planes(const D3Args &a, int storage, bool mom, int z_lo,
                                       int z_skip, int nplanes, cudaStream_t s);
// copies n planes of `bytes` bytes each from src[i] to dst[i] (any devices the
// calling one can reach); 16-byte accesses when every pointer and `bytes` allow
cudaError_t launch_plane_copy(const void *const *src, void *const *dst, int n, long bytes,
                              cudaStream_t s);
// single-pass Shan-Chen step whose populations arrive by bulk asynchronous
// copies (lb_sc_stage.cu); lattices without wall nodes for which
// sc_stage_chunk(W, H, D) != 0.  A block that gives up waiting for its copies
// sets *a.err (when a.err is set).
int sc_stage_chunk(int W, int H, int D);
// tmap: the tensor map of a.src (sc_stage_tensor_map) for the blocks whose
// stages lie inside the lattice, or null (every stage by cp.async chunks)
cudaError_t launch_d3q19_sc_stage(const D3Args &a, int storage, bool mom,
                                  const CUtensorMap *tmap, cudaStream_t s);
// the tensor map the staged step reads a.src through; false if it cannot be
// encoded (no driver entry point, or a layout it does not describe)
bool sc_stage_tensor_map(const D3Args &a, int storage, CUtensorMap *out);
// self-check of the staged step's bounded wait: one block whose first stage
// waits get no polls gives up, sets *err (device memory) and returns
cudaError_t sc_stage_wait_selftest(int *err);
// equilibrium written in 16-bit deviation storage (storage 1 or 2; Pop holds
// the storage arrays reinterpreted as float*)
cudaError_t launch_d3q19_equilibrium_storage(const Pop<19> &p, const float *rho, const float *ux,
                                             const float *uy, const float *uz, int N, float w0,
                                             float w1, float w7, const float *wr, int storage,
                                             cudaStream_t s);
// float <-> storage conversion of one population array (deviation from wr)
cudaError_t launch_to_storage(const float *src, void *dst, long n, float wr, int storage,
                              cudaStream_t s);
cudaError_t launch_from_storage(const void *src, float *dst, long n, float wr, int storage,
                                cudaStream_t s);
cudaError_t launch_d3q19_stream_swap(const Pop<19> &p, const uint8_t *sb, int W, int H, int D,
                                     cudaStream_t s);
cudaError_t launch_d3q19_collide(const D3Args &a, bool plot, cudaStream_t s);
cudaError_t launch_d3q19_get_border(const CPop<19> &p, const Pop<10> &b, int W, int H, int D,
                                    cudaStream_t s);
cudaError_t launch_d3q19_apply_border(const Pop<19> &p, const CPop<10> &nb, int W, int H, int D,
                                      cudaStream_t s);
cudaError_t launch_d3q19_equilibrium(const Pop<19> &p, const float *rho, const float *ux,
                                     const float *uy, const float *uz, int N, float w0, float w1,
                                     float w7, cudaStream_t s);

// D2Q9
cudaError_t launch_d2q9_fused(const D2Args &a, int mode, bool mom, bool plot, cudaStream_t s);
// launch_d2q9_fused without Shan-Chen or plot, as a programmatic dependent
// launch (the grid may start while the previous kernel on s drains)
cudaError_t launch_d2q9_fused_pdl(const D2Args &a, int mode, bool mom, cudaStream_t s);
// temporal blocking (native mode, no Shan-Chen): one programmatic dependent
// launch advances tblock_steps(variant) steps from a.src to a.dst; mom writes
// the moments of the last one.  tblock_steps is 0 for an unknown variant.
int tblock_steps(int variant);
cudaError_t launch_d2q9_tblock(const D2Args &a, int variant, bool mom, cudaStream_t s);
cudaError_t launch_d2q9_stream_swap(const Pop<9> &p, const uint8_t *sb, int W, int H,
                                    cudaStream_t s);
cudaError_t launch_d2q9_collide(const D2Args &a, bool plot, cudaStream_t s);
cudaError_t launch_d2q9_get_border(const CPop<9> &p, const Pop<6> &b, int W, int H,
                                   cudaStream_t s);
cudaError_t launch_d2q9_apply_border(const Pop<9> &p, const CPop<6> &nb, int W, int H,
                                     cudaStream_t s);
cudaError_t launch_d2q9_equilibrium(const Pop<9> &p, const float *rho, const float *ux,
                                    const float *uy, int N, float w0, float w1, float w5,
                                    cudaStream_t s);

// probes and reductions
cudaError_t launch_read_value(const float *plot, const float *ux, const float *uy,
                             const float *uz, const float *rho, float *value, long o,
                             cudaStream_t s);
// out_dev[7] = {mass, mom_x, mom_y, mom_z, kinetic energy, max|u|, n_fluid};
// nodes with (solid[o] & mask) != 0 are skipped; partials must hold
// reduce_partials_size() doubles
int reduce_partials_size();
cudaError_t launch_reduce(const float *rho, const float *ux, const float *uy, const float *uz,
                          const uint8_t *solid, uint8_t mask, long N, double *partials,
                          double *out_dev, cudaStream_t s);
// the same two passes with a caller-chosen number of first-pass blocks
// (partials must hold 7 * nblocks doubles)
cudaError_t launch_reduce_blocks(const float *rho, const float *ux, const float *uy,
                                 const float *uz, const uint8_t *solid, uint8_t mask, long N,
                                 int nblocks, double *partials, double *out_dev,
                                 cudaStream_t s);

// records a message for lb_abi_last_error() on the calling thread
void abi_record_error(const char *where, const char *what);

// learned closure (lb_closure.cu): the network and its scalings
struct ClosureArgs {
    MlpDev mlp;
    // b1, b2, w3, b3 by value: the tensor-core kernel reads them as constant
    // operands of its epilogue instructions (a snapshot taken when the closure
    // is enabled)
    float head_b1[MLP_H], head_b2[MLP_H], head_w3[MLP_H], head_b3;
    float nu0, tau0, s_ref, z_max;
    float *y_out;     // optional: network output per cell (tests)
    int *err;         // device error word (tcgen05 kernel: an MMA that never completed)
    // division by W*H and by W as a multiply-high (set by launch_d3q19_closure)
    uint64_t div_wh, div_w;
};
cudaError_t launch_d3q19_closure(const D3Args &a, const ClosureArgs &ca, bool mom,
                                 cudaStream_t s);

}  // namespace lb

struct lb_ctx;
namespace lb {
// installs (ca != nullptr) or removes the closure of a context (lb_context.cu)
int context_set_closure(lb_ctx *c, const ClosureArgs *ca);

}  // namespace lb
