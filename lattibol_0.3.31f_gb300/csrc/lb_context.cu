// lb_context.cu -- the context API (include/lbgb300.h, part 2): one lattice
// per context, populations in two library-owned structure-of-arrays sets that
// the fused kernel ping-pongs between (FP32, or 16-bit deviations from
// w_k*rho_ref), batches of steps replayed from captured CUDA graphs, FP64
// reductions; plus the drop-in reductions and the small device helpers.
#include <algorithm>
#include <cstddef>
#include <cstdio>
#include <cstring>
#include <mutex>
#include <string>
#include <unordered_map>
#include <vector>

#include "../../include/lbgb300.h"
#include "lb_kernels.cuh"

using namespace lb;

struct lb_ctx {
    lb_config cfg{};
    int Q = 0;
    long N = 0, stride = 0;
    int esize = 4;                       // bytes per stored population value
    void *pop[2] = {nullptr, nullptr};   // two population sets, Q arrays of `stride` values each
    int cur = 0;                         // index of the set holding the current state
    uint8_t *flags = nullptr;            // CELL_* bits (native) or the solid array (reference)
    uint8_t *sb = nullptr;               // reference mode: solid_bound
    float *mom = nullptr;                // rho, ux, uy, uz (each `stride` floats)
    float *sc = nullptr;                 // psi (D3Q19, D2Q9) and ueq_x, ueq_y (D2Q9)
    float *stage = nullptr;              // 16-bit storage: one float array for conversions
    double *red = nullptr;               // reduction partials + result
    int *errw = nullptr;                 // device error word of the kernels that wait on the GPU
    float4 *probe_host = nullptr;        // lb_run_probe: mapped page-locked cursor value
    float4 *probe_dev = nullptr;         // its device address
    int probe_o = -1;                    // cursor node the captured graphs write (-1: none)
    bool err_pending = false;            // a launch whose error word is unread
    cudaStream_t stream = nullptr;
    cudaGraphExec_t graph[2] = {nullptr, nullptr};  // graph_steps steps starting from set 0 / 1
    cudaEvent_t ev0 = nullptr, ev1 = nullptr;
    float corr[19] = {0};
    float wr[19] = {0};                  // 16-bit storage offsets w_k * rho_ref
    int tune = 0;                        // LB_TUNE_* bits in effect
    bool closure_on = false;             // learned closure sets the local relaxation time
    ClosureArgs closure{};
    bool flags_set = false;
    bool any_wall = false;               // some node carries CELL_WALL (flags start all fluid)
    int64_t launches = 0;
    int64_t steps = 0;                   // time steps since lb_create (or the checkpoint's)
    std::string err;
    // z-slab of a larger lattice (lb_slab_create): planes 1..slab_nz are the
    // global planes slab_z0 .. slab_z0 + slab_nz - 1; planes 0 and slab_nz + 1
    // are ghost planes holding the neighbouring slabs' faces
    int slab_nz = 0;                     // 0: not a slab
    int slab_z0 = 0, slab_nz_global = 0;
    cudaStream_t side = nullptr;         // the interior planes of a slab step
    cudaEvent_t ev_in = nullptr, ev_done = nullptr, ev_pack = nullptr;
    bool interior_pending = false;       // `side` holds interior planes `stream` has not joined
    void *face[2][2] = {{nullptr, nullptr}, {nullptr, nullptr}};  // group exchange [parity][below/above]
    int parity = 0;
    // staged Shan-Chen step: tensor maps of the two population sets (TMA
    // copies of the interior tiles' stages); 0 unknown, 1 encoded, -1 not available
    CUtensorMap tmap[2];
    int tmap_state[2] = {0, 0};
    // lb_slab_group_step on this slab as the group's first: graph-captured
    // batches of steps of the group (key: the group's slab list), one graph
    // per starting (population set, face parity)
    std::vector<lb_ctx *> grp_key;
    cudaGraphExec_t grp_graph[2][2] = {{nullptr, nullptr}, {nullptr, nullptr}};
    cudaEvent_t ev_fork = nullptr;
};

namespace {

int fail(lb_ctx *c, int code, const std::string &msg) {
    if (c) c->err = msg;
    return code;
}
int cuda_fail(lb_ctx *c, const char *where, cudaError_t e) {
    return fail(c, LB_ERR_CUDA, std::string(where) + ": " + cudaGetErrorString(e));
}
#define LB_TRY(c, where, call)                                  \
    do {                                                        \
        cudaError_t e_ = (call);                                \
        if (e_ != cudaSuccess) return cuda_fail(c, where, e_);  \
    } while (0)

// launch tuning used when the caller leaves lb_config.tuning at LB_TUNE_DEFAULT.
// D3Q19: the alternating sweep measured 44.7 vs 43.8 GLUPS on the 256x128x128
// channel.  D2Q9: programmatic dependent launches measured 24.9 vs 22.7 GLUPS
// on the 256^2 cavity (the alternating sweep: 23.8 with them).  Temporal blocks of 5 steps on 32x14 tiles (native mode without
// Shan-Chen) measured 48.5 vs 24.1 GLUPS at 256^2, 11.1 vs 5.8 at 128^2 and
// 73.3 vs 60.9 at 512^2, but 94.7 vs 101.5 at 1024^2 (a step then streams
// from L2 faster than the blocks recompute their halos), so they are the
// default up to TBLOCK_DEFAULT_MAX_NODES.  D3Q19 Shan-Chen without walls: the
// staged single-pass step measured 28.6 / 34.1 / 34.2 GLUPS (FP32 / FP16 /
// BF16) at 256^3 against 26.4 / 31.5 / 31.5 for the density pass + fused step
// (34.9 / 40.3 / 40.4 with compact stages, two steps per loop iteration, 3
// blocks per SM and 32-bit chunk offsets).
constexpr int LB_TUNE_LIBRARY_DEFAULT_D3 = LB_TUNE_REVERSE | LB_TUNE_SC_STAGED;
constexpr int LB_TUNE_LIBRARY_DEFAULT_D2 = LB_TUNE_PDL;
constexpr int TBLOCK_DEFAULT_SHAPE = 5;
constexpr long TBLOCK_DEFAULT_MAX_NODES = 1L << 19;

const double W3[3] = {1.0 / 3.0, 1.0 / 18.0, 1.0 / 36.0};
const double W2[3] = {4.0 / 9.0, 1.0 / 9.0, 1.0 / 36.0};

double d3_weight(int k) { return k == 0 ? W3[0] : (k <= 6 ? W3[1] : W3[2]); }
double d2_weight(int k) { return k == 0 ? W2[0] : (k <= 4 ? W2[1] : W2[2]); }

// the moving-wall term 6 w_k (c_k . u_wall), evaluated in double and rounded
// to float (physical velocity components; for D2Q9 physical c_y = -row offset)
void wall_corr(const lb_config &cfg, float *corr) {
    if (cfg.lattice == LB_D3Q19) {
        for (int k = 0; k < 19; k++) {
            double dot = 0.0;
            dot = dot + d3_cx(k) * (double)cfg.wall_u[0];
            dot = dot + d3_cy(k) * (double)cfg.wall_u[1];
            dot = dot + d3_cz(k) * (double)cfg.wall_u[2];
            corr[k] = (float)(6.0 * d3_weight(k) * dot);
        }
    } else {
        for (int k = 0; k < 9; k++) {
            double dot = 0.0;
            dot = dot + d2_cx(k) * (double)cfg.wall_u[0];
            dot = dot + (-d2_cr(k)) * (double)cfg.wall_u[1];
            corr[k] = (float)(6.0 * d2_weight(k) * dot);
        }
    }
}

float *pop_k(lb_ctx *c, int set, int k) {
    return reinterpret_cast<float *>(static_cast<char *>(c->pop[set]) +
                                     (long)k * c->stride * c->esize);
}
float *mom_k(lb_ctx *c, int i) { return c->mom + (long)i * c->stride; }

// copies the current population set into the other one.  Native-mode wall
// nodes are never written by a step, so after the caller sets populations
// both sets must hold them: a wall node then reads the same at every step.
cudaError_t mirror_sets(lb_ctx *c) {
    return cudaMemcpyAsync(c->pop[1 - c->cur], c->pop[c->cur],
                           (size_t)c->esize * c->stride * c->Q, cudaMemcpyDeviceToDevice,
                           c->stream);
}

bool sc_on(const lb_ctx *c) {
    return c->cfg.mode == LB_MODE_REFERENCE ? (c->Q == 9 && c->cfg.G < 0.f) : c->cfg.G != 0.f;
}

// the D3Q19 Shan-Chen step runs as the single-pass kernel fed by bulk
// asynchronous copies: native mode, no wall node, a lattice it tiles, and the
// tuning asks for it
bool sc_stage_on(const lb_ctx *c) {
    // (the kernel addresses the populations as 32-bit element offsets from the
    // first array: all 19 must lie within 2^32 elements of it)
    return c->Q == 19 && c->cfg.mode == LB_MODE_NATIVE && sc_on(c) && !c->any_wall &&
           (c->tune & LB_TUNE_SC_STAGED) && sc_stage_chunk(c->cfg.nx, c->cfg.ny, c->cfg.nz) &&
           19L * c->stride < (1L << 32);
}

// the temporal-blocking shape in effect (0 = per-step launches): D2Q9 native
// mode without Shan-Chen, and the tuning asks for it
int tblock_variant(const lb_ctx *c) {
    if (c->Q != 9 || sc_on(c) || c->cfg.mode != LB_MODE_NATIVE || !(c->tune & LB_TUNE_TBLOCK))
        return 0;
    const int v = (c->tune >> 12) & 0x1f;
    return tblock_steps(v) > 0 ? v : TBLOCK_DEFAULT_SHAPE;
}

// launches of temporal blocks per captured graph: even, so that a graph
// returns to the set it started from
int tblock_graph_launches(const lb_ctx *c, int steps_per_launch) {
    return std::max(2, (c->cfg.graph_steps / steps_per_launch) & ~1);
}

// the step kernels write the cursor probe themselves (every step path does;
// the per-step fallback in lb_run_probe stays for paths that might not)
bool probe_in_step(const lb_ctx *) { return true; }

// forget the captured step graphs (their kernel arguments changed)
void drop_graphs(lb_ctx *c) {
    for (int i = 0; i < 2; i++)
        if (c->graph[i]) {
            cudaGraphExecDestroy(c->graph[i]);
            c->graph[i] = nullptr;
        }
}

// a slab whose interior planes still run on the side stream: make the main
// stream wait for them
cudaError_t slab_join(lb_ctx *c) {
    if (!c->interior_pending) return cudaSuccess;
    c->interior_pending = false;
    return cudaStreamWaitEvent(c->stream, c->ev_done, 0);
}

// after the stream has been synchronised: the device error word written by
// the kernels that wait on the GPU (a tcgen05 closure MMA that never
// completed; a staged Shan-Chen block whose copies never arrived)
int check_device_error(lb_ctx *c) {
    if (!c->err_pending) return LB_OK;
    int word = 0;
    LB_TRY(c, "device error word",
           cudaMemcpy(&word, c->errw, sizeof(int), cudaMemcpyDeviceToHost));
    c->err_pending = false;
    if (word != 0) {
        LB_TRY(c, "device error word", cudaMemset(c->errw, 0, sizeof(int)));
        return fail(c, LB_ERR_DEVICE,
                    "a kernel gave up waiting on the GPU (tensor-core MMA or staged copies)");
    }
    return LB_OK;
}

// the D2Q9 kernel arguments of a step from set `from` into set 1-from
D2Args d2_args(lb_ctx *c, int from) {
    const lb_config &g = c->cfg;
    D2Args a{};
    for (int k = 0; k < 9; k++) {
        a.src.f[k] = pop_k(c, from, k);
        a.dst.f[k] = pop_k(c, 1 - from, k);
    }
    a.flags = c->flags; a.sb = c->sb;
    a.reverse = (c->tune & LB_TUNE_REVERSE) && from == 1;
    a.rho = mom_k(c, 0); a.ux = mom_k(c, 1); a.uy = mom_k(c, 2);
    a.psi = c->sc; a.ueq_x = c->sc + c->stride; a.ueq_y = c->sc + 2 * c->stride;
    a.W = g.nx; a.H = g.ny; a.dev = 0; a.ndev = 1;
    a.w0 = (float)W2[0]; a.w1 = (float)W2[1]; a.w5 = (float)W2[2];
    a.tau_inv = g.tau_inv; a.ux_in = g.u_in[0]; a.rho_out = g.rho_out;
    a.Fx = g.force[0]; a.Fy = g.force[1]; a.G = g.G; a.Gads = g.G_ads;
    a.psi_form = g.psi_form;
    memcpy(a.corr, c->corr, sizeof(float) * 9);
    a.probe = c->probe_o >= 0 ? c->probe_dev : nullptr;
    a.probe_o = c->probe_o;
    return a;
}

// the D3Q19 kernel arguments of a step from set `from` into set 1-from
D3Args d3_args(lb_ctx *c, int from) {
    const lb_config &g = c->cfg;
    D3Args a{};
    for (int k = 0; k < 19; k++) {
        a.src.f[k] = pop_k(c, from, k);
        a.dst.f[k] = pop_k(c, 1 - from, k);
    }
    a.flags = c->flags; a.sb = c->sb;
    a.reverse = (c->tune & LB_TUNE_REVERSE) && from == 1;
    a.rho = mom_k(c, 0); a.ux = mom_k(c, 1); a.uy = mom_k(c, 2); a.uz = mom_k(c, 3);
    a.W = g.nx; a.H = g.ny; a.D = g.nz; a.dev = 0; a.ndev = 1;
    a.w0 = (float)W3[0]; a.w1 = (float)W3[1]; a.w7 = (float)W3[2];
    a.tau_inv = g.tau_inv; a.ux_in = g.u_in[0]; a.rho_out = g.rho_out;
    a.Fx = g.force[0]; a.Fy = g.force[1]; a.Fz = g.force[2];
    memcpy(a.corr, c->corr, sizeof(a.corr));
    memcpy(a.wr, c->wr, sizeof(a.wr));
    a.psi = c->sc; a.G = g.G; a.psi_form = g.psi_form;
    a.probe = c->probe_o >= 0 ? c->probe_dev : nullptr;
    a.probe_o = c->probe_o;
    // 16-bit storage: the density the offsets carry, sum_k wr_k (f_k = wr_k +
    // d_k, so rho = sum_k wr_k + sum_k d_k), summed in double, rounded once
    double wsum = 0.0;
    for (int k = 0; k < 19; k++) wsum += (double)c->wr[k];
    a.rho_ref = (float)wsum;
    return a;
}

// one time step from set `from` into set 1-from
cudaError_t step_once(lb_ctx *c, int from, bool moments) {
    const lb_config &g = c->cfg;
    if (c->Q == 19) {
        D3Args a = d3_args(c, from);
        if (g.mode == LB_MODE_REFERENCE) {
            c->launches += 1;
            return launch_d3q19_fused(a, MODE_REF, moments, false, c->stream);
        }
        if (c->closure_on) {
            c->launches += 1;
            ClosureArgs ca = c->closure;
            ca.err = c->errw;
            c->err_pending = true;  // the tcgen05 kernel reports through the error word
            return launch_d3q19_closure(a, ca, moments, c->stream);
        }
        const bool sc = sc_on(c);
        if (sc_stage_on(c)) {
            c->launches += 1;
            a.err = c->errw;
            c->err_pending = true;  // a block that gave up waiting reports through the error word
            // TMA copies for the 16-bit storage forms (42.0 vs 39.3 GLUPS at 256^3
            // against the same layout by cp.async); FP32 keeps the compact
            // cp.async stages (TMA measured 27.1 against 32.6 and 34.9 compact)
            if (!c->tmap_state[from])
                c->tmap_state[from] =
                    (c->tune & LB_TUNE_SC_NO_TMA) || g.storage == LB_STORE_F32 ? -1
                    : sc_stage_tensor_map(a, g.storage, &c->tmap[from]) ? 1 : -1;
            return launch_d3q19_sc_stage(a, g.storage, moments,
                                         c->tmap_state[from] > 0 ? &c->tmap[from] : nullptr,
                                         c->stream);
        }
        c->launches += sc ? 2 : 1;
        return launch_d3q19_native(a, g.storage, moments, sc, c->stream);
    }
    const D2Args a = d2_args(c, from);
    c->launches += sc_on(c) ? 2 : 1;
    if (!sc_on(c) && (c->tune & LB_TUNE_PDL))
        return launch_d2q9_fused_pdl(a, g.mode == LB_MODE_REFERENCE ? MODE_REF : MODE_NATIVE,
                                     moments, c->stream);
    return launch_d2q9_fused(a, g.mode == LB_MODE_REFERENCE ? MODE_REF : MODE_NATIVE, moments,
                             false, c->stream);
}

int graph_for(lb_ctx *c, int from, cudaGraphExec_t *out) {
    if (c->graph[from]) { *out = c->graph[from]; return LB_OK; }
    cudaGraph_t graph;
    const int64_t before = c->launches;
    LB_TRY(c, "cudaStreamBeginCapture",
           cudaStreamBeginCapture(c->stream, cudaStreamCaptureModeThreadLocal));
    int set = from;
    cudaError_t e = cudaSuccess;
    const int tv = tblock_variant(c);
    if (tv) {
        const int L = tblock_graph_launches(c, tblock_steps(tv));
        for (int i = 0; i < L && e == cudaSuccess; i++) {
            e = launch_d2q9_tblock(d2_args(c, set), tv, false, c->stream);
            set = 1 - set;
        }
    } else {
        for (int i = 0; i < c->cfg.graph_steps && e == cudaSuccess; i++) {
            e = step_once(c, set, false);
            set = 1 - set;
        }
    }
    cudaError_t e2 = cudaStreamEndCapture(c->stream, &graph);
    c->launches = before;  // capture launches nothing
    if (e != cudaSuccess) return cuda_fail(c, "graph capture", e);
    if (e2 != cudaSuccess) return cuda_fail(c, "cudaStreamEndCapture", e2);
    e = cudaGraphInstantiate(&c->graph[from], graph, 0);
    cudaGraphDestroy(graph);
    if (e != cudaSuccess) return cuda_fail(c, "cudaGraphInstantiate", e);
    *out = c->graph[from];
    return LB_OK;
}

int launches_per_step(const lb_ctx *c) {
    if (!sc_on(c)) return 1;
    if (sc_stage_on(c)) return 1;
    return 2;
}

// host-side flag preparation: native -> NEAR_WALL bits; reference -> 0/1
// solid plus the reference's solid_bound rule (src/simulation_d3q19.cu:167-204,
// src/simulation_d2q9.cu:318-334: x in 1..W-2 only, periodic in y and z)
void prepare_flags(const lb_ctx *c, const uint8_t *in, std::vector<uint8_t> &flags,
                   std::vector<uint8_t> &sb) {
    const int W = c->cfg.nx, H = c->cfg.ny, D = c->cfg.nz, Q = c->Q;
    const long N = c->N;
    flags.assign(N, 0);
    sb.assign(N, 0);
    auto wrap = [](int v, int n) { return v < 0 ? v + n : (v >= n ? v - n : v); };
    auto nb = [&](int x, int y, int z, int k, bool wrapx) -> long {
        int xx, yy, zz;
        if (Q == 19) { xx = x + d3_cx(k); yy = y + d3_cy(k); zz = z + d3_cz(k); }
        else { xx = x + d2_cx(k); yy = y + d2_cr(k); zz = z; }
        if (wrapx) xx = wrap(xx, W);
        return xx + (long)W * (wrap(yy, H) + (long)H * wrap(zz, D));
    };
    if (c->cfg.mode == LB_MODE_REFERENCE) {
        for (long o = 0; o < N; o++) flags[o] = in[o] ? 1 : 0;
        for (int z = 0; z < D; z++)
            for (int y = 0; y < H; y++)
                for (int x = 1; x < W - 1; x++) {
                    bool all = true;
                    for (int k = 0; k < Q && all; k++) all = flags[nb(x, y, z, k, false)] != 0;
                    sb[x + (long)W * (y + (long)H * z)] = all ? 1 : 0;
                }
        return;
    }
    bool any_wall = false;
    for (long o = 0; o < N; o++) {
        flags[o] = (in[o] & CELL_WALL) ? (in[o] & (CELL_WALL | CELL_MOVING)) : 0;
        any_wall = any_wall || flags[o];
    }
    if (!any_wall) return;  // fully periodic: no fluid cell is near a wall
    for (int z = 0; z < D; z++)
        for (int y = 0; y < H; y++)
            for (int x = 0; x < W; x++) {
                const long o = x + (long)W * (y + (long)H * z);
                if (flags[o] & CELL_WALL) continue;
                for (int k = 1; k < Q; k++)
                    if (flags[nb(x, y, z, k, true)] & CELL_WALL) {
                        flags[o] |= CELL_NEAR_WALL;
                        break;
                    }
            }
}

}  // namespace

extern "C" {

const char *lb_version(void) { return "lbgb300 0.2 (sm_103a)"; }

int lb_config_default(lb_config *cfg, int lattice, int nx, int ny, int nz) {
    if (!cfg) return LB_ERR_ARG;
    memset(cfg, 0, sizeof(*cfg));
    cfg->lattice = lattice;
    cfg->nx = nx; cfg->ny = ny; cfg->nz = lattice == LB_D2Q9 ? 1 : nz;
    cfg->mode = LB_MODE_NATIVE;
    cfg->storage = LB_STORE_F32;
    cfg->tau_inv = 1.f;
    cfg->rho_out = 1.f;
    cfg->psi_form = LB_PSI_EXP1;
    cfg->graph_steps = 64;
    cfg->rho_ref = 1.f;
    return LB_OK;
}

int lb_create(const lb_config *cfg, lb_ctx **out) {
    if (!cfg || !out) return LB_ERR_ARG;
    *out = nullptr;
    if (cfg->lattice != LB_D2Q9 && cfg->lattice != LB_D3Q19) return LB_ERR_ARG;
    if (cfg->nx < 1 || cfg->ny < 1 || cfg->nz < 1 || (cfg->lattice == LB_D2Q9 && cfg->nz != 1))
        return LB_ERR_ARG;
    if (cfg->mode != LB_MODE_REFERENCE && cfg->mode != LB_MODE_NATIVE) return LB_ERR_ARG;
    if (cfg->storage < LB_STORE_F32 || cfg->storage > LB_STORE_BF16) return LB_ERR_ARG;
    // 16-bit deviation storage: D3Q19 native mode only
    if (cfg->storage != LB_STORE_F32 &&
        (cfg->lattice != LB_D3Q19 || cfg->mode != LB_MODE_NATIVE))
        return LB_ERR_ARG;
    const long N = (long)cfg->nx * cfg->ny * cfg->nz;
    if (N > (1L << 31) - 64) return LB_ERR_ARG;  // 32-bit node offsets in the kernels
    lb_ctx *c = new lb_ctx;
    c->cfg = *cfg;
    if (c->cfg.graph_steps <= 0) c->cfg.graph_steps = 64;
    c->cfg.graph_steps += c->cfg.graph_steps & 1;  // even: a graph returns to its start set
    if (!(c->cfg.rho_ref > 0.f)) c->cfg.rho_ref = 1.f;
    // explicit: the bits the header defines (REVERSE, PDL, TBLOCK, SC_STAGED,
    // SC_NO_TMA, the block shape); any other bit is ignored
    constexpr int kTuneBits = LB_TUNE_REVERSE | LB_TUNE_PDL | LB_TUNE_TBLOCK | LB_TUNE_SC_STAGED |
                              LB_TUNE_SC_NO_TMA | LB_TUNE_TBLOCK_SHAPE(0x1f);
    static_assert(kTuneBits == 0x1f0e9, "tuning bits");
    c->tune = (cfg->tuning & LB_TUNE_EXPLICIT)
                  ? (cfg->tuning & kTuneBits)
                  : (cfg->lattice == LB_D2Q9 ? LB_TUNE_LIBRARY_DEFAULT_D2
                                             : LB_TUNE_LIBRARY_DEFAULT_D3);
    if (!(cfg->tuning & LB_TUNE_EXPLICIT) && cfg->lattice == LB_D2Q9 &&
        N <= TBLOCK_DEFAULT_MAX_NODES)
        c->tune |= LB_TUNE_TBLOCK | LB_TUNE_TBLOCK_SHAPE(TBLOCK_DEFAULT_SHAPE);
    c->Q = cfg->lattice;
    c->N = N;
    c->stride = (N + 127) / 128 * 128;  // every population array starts on a 256-byte boundary
    c->esize = cfg->storage == LB_STORE_F32 ? 4 : 2;
    wall_corr(c->cfg, c->corr);
    if (c->Q == 19)
        for (int k = 0; k < 19; k++) c->wr[k] = (float)(d3_weight(k) * (double)c->cfg.rho_ref);
    cudaError_t e = cudaSuccess;
    const size_t pbytes = (size_t)c->esize * c->stride * c->Q;
    const int nsc = c->Q == 9 ? 3 : (sc_on(c) ? 1 : 0);
    if (e == cudaSuccess) e = cudaMalloc(&c->pop[0], pbytes);
    if (e == cudaSuccess) e = cudaMalloc(&c->pop[1], pbytes);
    if (e == cudaSuccess) e = cudaMalloc(&c->flags, c->stride);
    if (e == cudaSuccess) e = cudaMalloc(&c->sb, c->stride);
    if (e == cudaSuccess) e = cudaMalloc(&c->mom, sizeof(float) * c->stride * 4);
    if (e == cudaSuccess && nsc) e = cudaMalloc(&c->sc, sizeof(float) * c->stride * nsc);
    if (e == cudaSuccess && c->esize != 4) e = cudaMalloc(&c->stage, sizeof(float) * c->stride);
    // reduction partials, 7 results, then 4 floats (2 doubles) for lb_probe
    if (e == cudaSuccess) e = cudaMalloc(&c->red, sizeof(double) * (reduce_partials_size() + 16));
    if (e == cudaSuccess)
        e = cudaMalloc(&c->errw, sizeof(int));
    if (e == cudaSuccess) e = cudaMemsetAsync(c->errw, 0, sizeof(int), c->stream);
    if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking);
    if (e == cudaSuccess) e = cudaEventCreate(&c->ev0);
    if (e == cudaSuccess) e = cudaEventCreate(&c->ev1);
    if (e == cudaSuccess) e = cudaMemsetAsync(c->flags, 0, c->stride, c->stream);
    if (e == cudaSuccess) e = cudaMemsetAsync(c->sb, 0, c->stride, c->stream);
    if (e == cudaSuccess) e = cudaMemsetAsync(c->mom, 0, sizeof(float) * c->stride * 4, c->stream);
    if (e == cudaSuccess && c->sc)
        e = cudaMemsetAsync(c->sc, 0, sizeof(float) * c->stride * nsc, c->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(c->stream);
    if (e != cudaSuccess) {
        lb_destroy(c);
        return e == cudaErrorMemoryAllocation ? LB_ERR_NOMEM : LB_ERR_CUDA;
    }
    *out = c;
    return LB_OK;
}

int lb_destroy(lb_ctx *c) {
    if (!c) return LB_ERR_ARG;
    if (c->stream) cudaStreamSynchronize(c->stream);
    for (int i = 0; i < 2; i++) {
        if (c->graph[i]) cudaGraphExecDestroy(c->graph[i]);
        if (c->pop[i]) cudaFree(c->pop[i]);
    }
    if (c->flags) cudaFree(c->flags);
    if (c->sb) cudaFree(c->sb);
    if (c->mom) cudaFree(c->mom);
    if (c->sc) cudaFree(c->sc);
    if (c->stage) cudaFree(c->stage);
    if (c->red) cudaFree(c->red);
    if (c->errw) cudaFree(c->errw);
    if (c->probe_host) cudaFreeHost(c->probe_host);
    if (c->side) cudaStreamSynchronize(c->side);
    for (int i = 0; i < 2; i++)
        for (int j = 0; j < 2; j++) {
            if (c->face[i][j]) cudaFree(c->face[i][j]);
            if (c->grp_graph[i][j]) cudaGraphExecDestroy(c->grp_graph[i][j]);
        }
    if (c->ev_fork) cudaEventDestroy(c->ev_fork);
    for (cudaEvent_t ev : {c->ev0, c->ev1, c->ev_in, c->ev_done, c->ev_pack})
        if (ev) cudaEventDestroy(ev);
    if (c->side) cudaStreamDestroy(c->side);
    if (c->stream) cudaStreamDestroy(c->stream);
    delete c;
    return LB_OK;
}

const char *lb_error(const lb_ctx *c) { return c ? c->err.c_str() : "null context"; }

int lb_set_flags(lb_ctx *c, const uint8_t *flags) {
    if (!c || !flags) return fail(c, LB_ERR_ARG, "lb_set_flags: null argument");
    std::vector<uint8_t> f, sb;
    prepare_flags(c, flags, f, sb);
    LB_TRY(c, "lb_set_flags", cudaMemcpyAsync(c->flags, f.data(), c->N, cudaMemcpyHostToDevice, c->stream));
    LB_TRY(c, "lb_set_flags", cudaMemcpyAsync(c->sb, sb.data(), c->N, cudaMemcpyHostToDevice, c->stream));
    LB_TRY(c, "lb_set_flags", cudaStreamSynchronize(c->stream));
    c->flags_set = true;
    bool any_wall = false;
    for (long o = 0; o < c->N && !any_wall; o++) any_wall = (f[o] & CELL_WALL) != 0;
    if (any_wall != c->any_wall) drop_graphs(c);  // the step kernel may change
    c->any_wall = any_wall;
    return LB_OK;
}

// populations cross the API as float; 16-bit storage converts on the device
// through a staging array of its own (the moment fields stay untouched)
int lb_set_populations(lb_ctx *c, const float *f) {
    if (!c || !f) return fail(c, LB_ERR_ARG, "lb_set_populations: null argument");
    for (int k = 0; k < c->Q; k++) {
        if (c->esize == 4) {
            LB_TRY(c, "lb_set_populations",
                   cudaMemcpyAsync(pop_k(c, c->cur, k), f + (long)k * c->N, sizeof(float) * c->N,
                                   cudaMemcpyHostToDevice, c->stream));
        } else {
            LB_TRY(c, "lb_set_populations",
                   cudaMemcpyAsync(c->stage, f + (long)k * c->N, sizeof(float) * c->N,
                                   cudaMemcpyHostToDevice, c->stream));
            LB_TRY(c, "lb_set_populations",
                   launch_to_storage(c->stage, pop_k(c, c->cur, k), c->N, c->wr[k],
                                     c->cfg.storage, c->stream));
            c->launches += 1;
        }
    }
    LB_TRY(c, "lb_set_populations", mirror_sets(c));
    LB_TRY(c, "lb_set_populations", cudaStreamSynchronize(c->stream));
    return LB_OK;
}

int lb_get_populations(lb_ctx *c, float *f) {
    if (!c || !f) return fail(c, LB_ERR_ARG, "lb_get_populations: null argument");
    LB_TRY(c, "lb_get_populations", slab_join(c));
    for (int k = 0; k < c->Q; k++) {
        const float *src = pop_k(c, c->cur, k);
        if (c->esize != 4) {
            LB_TRY(c, "lb_get_populations",
                   launch_from_storage(pop_k(c, c->cur, k), c->stage, c->N, c->wr[k],
                                       c->cfg.storage, c->stream));
            c->launches += 1;
            src = c->stage;
        }
        LB_TRY(c, "lb_get_populations",
               cudaMemcpyAsync(f + (long)k * c->N, src, sizeof(float) * c->N,
                               cudaMemcpyDeviceToHost, c->stream));
        // the staging array is reused by the next population
        LB_TRY(c, "lb_get_populations", cudaStreamSynchronize(c->stream));
    }
    return check_device_error(c);
}

int lb_init_equilibrium(lb_ctx *c, const float *rho, const float *ux, const float *uy,
                        const float *uz) {
    if (!c) return LB_ERR_ARG;
    const float *src[4] = {rho, ux, uy, uz};
    const float *dev[4] = {nullptr, nullptr, nullptr, nullptr};
    for (int i = 0; i < 4; i++) {
        if (!src[i] || (i == 3 && c->Q == 9)) continue;
        LB_TRY(c, "lb_init_equilibrium",
               cudaMemcpyAsync(mom_k(c, i), src[i], sizeof(float) * c->N, cudaMemcpyHostToDevice,
                               c->stream));
        dev[i] = mom_k(c, i);
    }
    cudaError_t e;
    if (c->Q == 19) {
        Pop<19> p;
        for (int k = 0; k < 19; k++) p.f[k] = pop_k(c, c->cur, k);
        if (c->esize == 4)
            e = launch_d3q19_equilibrium(p, dev[0], dev[1], dev[2], dev[3], (int)c->N,
                                         (float)W3[0], (float)W3[1], (float)W3[2], c->stream);
        else
            e = launch_d3q19_equilibrium_storage(p, dev[0], dev[1], dev[2], dev[3], (int)c->N,
                                                 (float)W3[0], (float)W3[1], (float)W3[2], c->wr,
                                                 c->cfg.storage, c->stream);
    } else {
        Pop<9> p;
        for (int k = 0; k < 9; k++) p.f[k] = pop_k(c, c->cur, k);
        e = launch_d2q9_equilibrium(p, dev[0], dev[1], dev[2], (int)c->N, (float)W2[0],
                                    (float)W2[1], (float)W2[2], c->stream);
    }
    LB_TRY(c, "lb_init_equilibrium", e);
    c->launches += 1;
    LB_TRY(c, "lb_init_equilibrium", mirror_sets(c));
    LB_TRY(c, "lb_init_equilibrium", cudaStreamSynchronize(c->stream));
    return LB_OK;
}

int lb_step(lb_ctx *c, int nsteps) {
    if (!c || nsteps < 0) return fail(c, LB_ERR_ARG, "lb_step: bad argument");
    if (c->slab_nz)
        return fail(c, LB_ERR_STATE, "lb_step: a slab steps with lb_slab_step or "
                                     "lb_slab_group_step (its ghost planes need the exchange)");
    if (nsteps == 0) return LB_OK;
    if (const int tv = tblock_variant(c)) {
        // temporal blocks of T steps (graphs of L blocks); the last block, or
        // the last per-step launch of a remainder, writes the moments
        const int T = tblock_steps(tv), L = tblock_graph_launches(c, T);
        int rest = nsteps;
        while (rest > L * T) {
            cudaGraphExec_t g;
            int rc = graph_for(c, c->cur, &g);
            if (rc != LB_OK) return rc;
            LB_TRY(c, "cudaGraphLaunch", cudaGraphLaunch(g, c->stream));
            c->launches += L;
            rest -= L * T;
        }
        for (; rest >= T; rest -= T) {
            LB_TRY(c, "lb_step", launch_d2q9_tblock(d2_args(c, c->cur), tv, rest == T, c->stream));
            c->launches += 1;
            c->cur = 1 - c->cur;
        }
        for (; rest > 0; rest--) {
            LB_TRY(c, "lb_step", step_once(c, c->cur, rest == 1));
            c->cur = 1 - c->cur;
        }
        c->steps += nsteps;
        return LB_OK;
    }
    int rest = nsteps - 1;  // the last step also writes the moment fields
    while (rest >= c->cfg.graph_steps) {
        cudaGraphExec_t g;
        int rc = graph_for(c, c->cur, &g);
        if (rc != LB_OK) return rc;
        LB_TRY(c, "cudaGraphLaunch", cudaGraphLaunch(g, c->stream));
        c->launches += (int64_t)c->cfg.graph_steps * launches_per_step(c);
        rest -= c->cfg.graph_steps;
    }
    for (; rest > 0; rest--) {
        LB_TRY(c, "lb_step", step_once(c, c->cur, false));
        c->cur = 1 - c->cur;
    }
    LB_TRY(c, "lb_step", step_once(c, c->cur, true));
    c->cur = 1 - c->cur;
    c->steps += nsteps;
    return LB_OK;
}

int lb_get_moments(lb_ctx *c, float *rho, float *ux, float *uy, float *uz) {
    if (!c) return LB_ERR_ARG;
    LB_TRY(c, "lb_get_moments", slab_join(c));
    float *dst[4] = {rho, ux, uy, uz};
    for (int i = 0; i < 4; i++) {
        if (!dst[i] || (i == 3 && c->Q == 9)) continue;
        LB_TRY(c, "lb_get_moments",
               cudaMemcpyAsync(dst[i], mom_k(c, i), sizeof(float) * c->N, cudaMemcpyDeviceToHost,
                               c->stream));
    }
    LB_TRY(c, "lb_get_moments", cudaStreamSynchronize(c->stream));
    return check_device_error(c);
}

int lb_reduce(lb_ctx *c, double out[7]) {
    if (!c || !out) return LB_ERR_ARG;
    LB_TRY(c, "lb_reduce", slab_join(c));
    double *res = c->red + reduce_partials_size();
    // a slab sums its own planes only (not the ghost planes)
    const long off = c->slab_nz ? (long)c->cfg.nx * c->cfg.ny : 0;
    const long n = c->slab_nz ? off * c->slab_nz : c->N;
    LB_TRY(c, "lb_reduce",
           launch_reduce(mom_k(c, 0) + off, mom_k(c, 1) + off, mom_k(c, 2) + off,
                         c->Q == 19 ? mom_k(c, 3) + off : nullptr, c->flags + off, CELL_WALL, n,
                         c->red, res, c->stream));
    c->launches += 2;
    LB_TRY(c, "lb_reduce", cudaMemcpyAsync(out, res, sizeof(double) * 7, cudaMemcpyDeviceToHost, c->stream));
    LB_TRY(c, "lb_reduce", cudaStreamSynchronize(c->stream));
    return check_device_error(c);
}

int lb_probe(lb_ctx *c, int x, int y, int z, float value[4]) {
    if (!c || !value) return LB_ERR_ARG;
    if (x < 0 || y < 0 || z < 0 || x >= c->cfg.nx || y >= c->cfg.ny || z >= c->cfg.nz)
        return fail(c, LB_ERR_ARG, "lb_probe: node outside the lattice");
    const long o = x + (long)c->cfg.nx * (y + (long)c->cfg.ny * z);
    // the 4 floats land in the reduction scratch, after partials and results
    float *dev = reinterpret_cast<float *>(c->red + reduce_partials_size() + 7);
    LB_TRY(c, "lb_probe",
           launch_read_value(nullptr, mom_k(c, 1), mom_k(c, 2), c->Q == 19 ? mom_k(c, 3) : nullptr,
                             mom_k(c, 0), dev, o, c->stream));
    c->launches += 1;
    LB_TRY(c, "lb_probe", cudaMemcpyAsync(value, dev, 4 * sizeof(float), cudaMemcpyDeviceToHost,
                                          c->stream));
    LB_TRY(c, "lb_probe", cudaStreamSynchronize(c->stream));
    return LB_OK;
}

int lb_run_probe(lb_ctx *c, int nsteps, int x, int y, int z, float value[4]) {
    if (!c || !value || nsteps < 0) return LB_ERR_ARG;
    if (x < 0 || y < 0 || z < 0 || x >= c->cfg.nx || y >= c->cfg.ny || z >= c->cfg.nz)
        return fail(c, LB_ERR_ARG, "lb_run_probe: node outside the lattice");
    if (c->slab_nz) return fail(c, LB_ERR_STATE, "lb_run_probe: not available on a slab");
    if (nsteps == 0) return LB_OK;
    if (probe_in_step(c)) {
        // every step's kernel writes the cursor node's moments into mapped
        // page-locked memory: the steps replay from graphs with no host
        // round trip between them
        if (!c->probe_host) {
            LB_TRY(c, "lb_run_probe",
                   cudaHostAlloc((void **)&c->probe_host, sizeof(float4), cudaHostAllocMapped));
            LB_TRY(c, "lb_run_probe",
                   cudaHostGetDevicePointer((void **)&c->probe_dev, c->probe_host, 0));
        }
        const int o = x + c->cfg.nx * (y + c->cfg.ny * z);
        if (o != c->probe_o) {
            LB_TRY(c, "lb_run_probe", cudaStreamSynchronize(c->stream));
            drop_graphs(c);  // the captured steps carry the probe node
            c->probe_o = o;
        }
        int rc = lb_step(c, nsteps);
        if (rc != LB_OK) return rc;
        LB_TRY(c, "lb_run_probe", cudaStreamSynchronize(c->stream));
        rc = check_device_error(c);
        if (rc != LB_OK) return rc;
        memcpy(value, (const void *)c->probe_host, 4 * sizeof(float));
        return LB_OK;
    }
    for (int i = 0; i < nsteps; i++) {
        LB_TRY(c, "lb_run_probe", step_once(c, c->cur, true));
        c->cur = 1 - c->cur;
        c->steps += 1;
        const int rc = lb_probe(c, x, y, z, value);
        if (rc != LB_OK) return rc;
    }
    return LB_OK;
}

int lb_device_fields(lb_ctx *c, float **rho, float **ux, float **uy, float **uz) {
    if (!c) return LB_ERR_ARG;
    if (rho) *rho = mom_k(c, 0);
    if (ux) *ux = mom_k(c, 1);
    if (uy) *uy = mom_k(c, 2);
    if (uz) *uz = c->Q == 19 ? mom_k(c, 3) : nullptr;
    return LB_OK;
}

int lb_extents(const lb_ctx *c, int *nx, int *ny, int *nz) {
    if (!c) return LB_ERR_ARG;
    if (nx) *nx = c->cfg.nx;
    if (ny) *ny = c->cfg.ny;
    if (nz) *nz = c->cfg.nz;
    return LB_OK;
}

int lb_synchronize(lb_ctx *c) {
    if (!c) return LB_ERR_ARG;
    LB_TRY(c, "lb_synchronize", slab_join(c));
    LB_TRY(c, "lb_synchronize", cudaStreamSynchronize(c->stream));
    return check_device_error(c);
}

int lb_time_steps(lb_ctx *c, int nsteps, float *ms) {
    if (!c || !ms) return LB_ERR_ARG;
    LB_TRY(c, "lb_time_steps", cudaEventRecord(c->ev0, c->stream));
    int rc = lb_step(c, nsteps);
    if (rc != LB_OK) return rc;
    LB_TRY(c, "lb_time_steps", cudaEventRecord(c->ev1, c->stream));
    LB_TRY(c, "lb_time_steps", cudaEventSynchronize(c->ev1));
    LB_TRY(c, "lb_time_steps", cudaEventElapsedTime(ms, c->ev0, c->ev1));
    return check_device_error(c);
}

int64_t lb_launch_count(const lb_ctx *c) { return c ? c->launches : -1; }

int lb_wall_correction(const lb_ctx *c, float *corr) {
    if (!c || !corr) return LB_ERR_ARG;
    memcpy(corr, c->corr, sizeof(float) * c->Q);
    return LB_OK;
}

int64_t lb_steps_done(const lb_ctx *c) { return c ? c->steps : -1; }

}  // extern "C"

// ----------------------------------------------------------------- checkpoints
//
// File layout (the host's byte order, marked in the header):
//   256-byte header (CkptHeader), then three sections:
//   flags        N bytes, the context's cell flags
//   populations  Q arrays of N values in the stored type (4 or 2 bytes)
//   moments      rho, ux, uy (, uz for D3Q19): N floats each
// Each section and the header carry a CRC-32 (reflected, polynomial
// 0xEDB88320).  A load checks every CRC before it changes the context.
namespace {

struct CkptHeader {
    char magic[8];
    uint32_t version, header_bytes, byte_order;
    int32_t lattice, nx, ny, nz, mode, storage, psi_form, graph_steps, tuning;
    float tau_inv, force[3], u_in[3], rho_out, wall_u[3], G, G_ads, rho_ref;
    int64_t steps;
    uint64_t flag_bytes, pop_bytes, mom_bytes;
    uint32_t crc_flags, crc_pop, crc_mom, crc_header;
    uint8_t pad[96];
};
static_assert(sizeof(CkptHeader) == 256, "checkpoint header is 256 bytes");
constexpr char CKPT_MAGIC[8] = {'L', 'B', 'G', 'B', 'C', 'K', 'P', 'T'};
constexpr uint32_t CKPT_BYTE_ORDER = 0x01020304u;

uint32_t crc32_update(uint32_t crc, const void *data, size_t n) {
    static uint32_t table[256];
    static std::once_flag once;
    std::call_once(once, [] {
        for (uint32_t i = 0; i < 256; i++) {
            uint32_t r = i;
            for (int j = 0; j < 8; j++) r = (r & 1) ? (r >> 1) ^ 0xEDB88320u : r >> 1;
            table[i] = r;
        }
    });
    const uint8_t *p = static_cast<const uint8_t *>(data);
    crc = ~crc;
    for (size_t i = 0; i < n; i++) crc = table[(crc ^ p[i]) & 0xff] ^ (crc >> 8);
    return ~crc;
}

int n_moments(const lb_ctx *c) { return c->Q == 19 ? 4 : 3; }

void header_from_config(const lb_config &g, CkptHeader &h) {
    memset(&h, 0, sizeof h);
    memcpy(h.magic, CKPT_MAGIC, 8);
    h.version = 1;
    h.header_bytes = sizeof(CkptHeader);
    h.byte_order = CKPT_BYTE_ORDER;
    h.lattice = g.lattice; h.nx = g.nx; h.ny = g.ny; h.nz = g.nz;
    h.mode = g.mode; h.storage = g.storage; h.psi_form = g.psi_form;
    h.graph_steps = g.graph_steps; h.tuning = g.tuning;
    h.tau_inv = g.tau_inv; h.rho_out = g.rho_out; h.G = g.G; h.G_ads = g.G_ads;
    h.rho_ref = g.rho_ref;
    for (int i = 0; i < 3; i++) {
        h.force[i] = g.force[i]; h.u_in[i] = g.u_in[i]; h.wall_u[i] = g.wall_u[i];
    }
}

void config_from_header(const CkptHeader &h, lb_config &g) {
    lb_config_default(&g, h.lattice, h.nx, h.ny, h.nz);
    g.mode = h.mode; g.storage = h.storage; g.psi_form = h.psi_form;
    g.graph_steps = h.graph_steps; g.tuning = h.tuning;
    g.tau_inv = h.tau_inv; g.rho_out = h.rho_out; g.G = h.G; g.G_ads = h.G_ads;
    g.rho_ref = h.rho_ref;
    for (int i = 0; i < 3; i++) {
        g.force[i] = h.force[i]; g.u_in[i] = h.u_in[i]; g.wall_u[i] = h.wall_u[i];
    }
}

// the header, checked for magic, version, byte order and its own CRC
std::string read_header(FILE *fp, CkptHeader &h) {
    if (fread(&h, sizeof h, 1, fp) != 1) return "not a checkpoint (short header)";
    if (memcmp(h.magic, CKPT_MAGIC, 8) != 0) return "not a checkpoint (magic)";
    if (h.byte_order != CKPT_BYTE_ORDER) return "checkpoint written with another byte order";
    if (h.version != 1 || h.header_bytes != sizeof(CkptHeader))
        return "unsupported checkpoint version";
    const uint32_t crc = crc32_update(0, &h, offsetof(CkptHeader, crc_header));
    if (crc != h.crc_header) return "checkpoint header damaged (CRC)";
    if ((h.lattice != LB_D2Q9 && h.lattice != LB_D3Q19) || h.nx < 1 || h.ny < 1 || h.nz < 1)
        return "checkpoint header has bad extents";
    return "";
}

// streams `bytes` bytes of the file through f(chunk, n) in pieces of at most
// `piece` bytes; false on a short read
template <class F>
bool stream_section(FILE *fp, uint64_t bytes, std::vector<uint8_t> &buf, F &&f) {
    while (bytes > 0) {
        const size_t n = (size_t)std::min<uint64_t>(bytes, buf.size());
        if (fread(buf.data(), 1, n, fp) != n) return false;
        f(buf.data(), n);
        bytes -= n;
    }
    return true;
}

}  // namespace

extern "C" {

int lb_checkpoint_save(lb_ctx *c, const char *path) {
    if (!c || !path) return fail(c, LB_ERR_ARG, "lb_checkpoint_save: null argument");
    if (c->slab_nz) return fail(c, LB_ERR_STATE, "lb_checkpoint_save: not available on a slab");
    const long N = c->N;
    const size_t pop_k_bytes = (size_t)N * c->esize;
    CkptHeader h;
    header_from_config(c->cfg, h);
    h.steps = c->steps;
    h.flag_bytes = (uint64_t)N;
    h.pop_bytes = (uint64_t)pop_k_bytes * c->Q;
    h.mom_bytes = (uint64_t)N * sizeof(float) * n_moments(c);
    const std::string tmp = std::string(path) + ".tmp";
    FILE *fp = fopen(tmp.c_str(), "wb");
    if (!fp) return fail(c, LB_ERR_IO, "lb_checkpoint_save: cannot create " + tmp);
    auto bail = [&](int code, const std::string &msg) {
        fclose(fp);
        remove(tmp.c_str());
        return fail(c, code, "lb_checkpoint_save: " + msg);
    };
    // the header goes first as a placeholder and is rewritten with the CRCs
    if (fwrite(&h, sizeof h, 1, fp) != 1) return bail(LB_ERR_IO, "write failed");
    std::vector<uint8_t> buf(std::max<size_t>(pop_k_bytes, (size_t)N * sizeof(float)));
    auto section = [&](const void *dev, size_t bytes, uint32_t &crc) -> int {
        cudaError_t e = cudaMemcpyAsync(buf.data(), dev, bytes, cudaMemcpyDeviceToHost, c->stream);
        if (e == cudaSuccess) e = cudaStreamSynchronize(c->stream);
        if (e != cudaSuccess) return cuda_fail(c, "lb_checkpoint_save", e);
        crc = crc32_update(crc, buf.data(), bytes);
        if (fwrite(buf.data(), 1, bytes, fp) != bytes) return LB_ERR_IO;
        return LB_OK;
    };
    int rc = LB_OK;
    LB_TRY(c, "lb_checkpoint_save", cudaStreamSynchronize(c->stream));
    rc = section(c->flags, (size_t)N, h.crc_flags);
    for (int k = 0; k < c->Q && rc == LB_OK; k++) rc = section(pop_k(c, c->cur, k), pop_k_bytes, h.crc_pop);
    for (int i = 0; i < n_moments(c) && rc == LB_OK; i++)
        rc = section(mom_k(c, i), (size_t)N * sizeof(float), h.crc_mom);
    if (rc == LB_ERR_CUDA) {
        fclose(fp);
        remove(tmp.c_str());
        return rc;
    }
    if (rc != LB_OK) return bail(LB_ERR_IO, "write failed");
    h.crc_header = crc32_update(0, &h, offsetof(CkptHeader, crc_header));
    if (fseek(fp, 0, SEEK_SET) != 0 || fwrite(&h, sizeof h, 1, fp) != 1)
        return bail(LB_ERR_IO, "write failed");
    if (fclose(fp) != 0) {
        remove(tmp.c_str());
        return fail(c, LB_ERR_IO, "lb_checkpoint_save: write failed");
    }
    if (rename(tmp.c_str(), path) != 0) {
        remove(tmp.c_str());
        return fail(c, LB_ERR_IO, std::string("lb_checkpoint_save: cannot rename to ") + path);
    }
    return LB_OK;
}

int lb_checkpoint_info(const char *path, lb_config *cfg, int64_t *steps) {
    if (!path) return LB_ERR_ARG;
    FILE *fp = fopen(path, "rb");
    if (!fp) {
        abi_record_error("lb_checkpoint_info", (std::string("cannot open ") + path).c_str());
        return LB_ERR_IO;
    }
    CkptHeader h;
    const std::string why = read_header(fp, h);
    fclose(fp);
    if (!why.empty()) {
        abi_record_error("lb_checkpoint_info", why.c_str());
        return LB_ERR_IO;
    }
    if (cfg) config_from_header(h, *cfg);
    if (steps) *steps = h.steps;
    return LB_OK;
}

int lb_checkpoint_load(lb_ctx *c, const char *path) {
    if (!c || !path) return fail(c, LB_ERR_ARG, "lb_checkpoint_load: null argument");
    FILE *fp = fopen(path, "rb");
    if (!fp) return fail(c, LB_ERR_IO, std::string("lb_checkpoint_load: cannot open ") + path);
    auto bail = [&](int code, const std::string &msg) {
        fclose(fp);
        return fail(c, code, "lb_checkpoint_load: " + msg);
    };
    CkptHeader h;
    std::string why = read_header(fp, h);
    if (!why.empty()) return bail(LB_ERR_IO, why);
    const lb_config &g = c->cfg;
    if (h.lattice != g.lattice || h.nx != g.nx || h.ny != g.ny || h.nz != g.nz ||
        h.mode != g.mode || h.storage != g.storage)
        return bail(LB_ERR_ARG, "lattice, extents, mode or storage differ from the context's");
    const long N = c->N;
    const size_t pop_k_bytes = (size_t)N * c->esize;
    const size_t mom_k_bytes = (size_t)N * sizeof(float);
    if (h.flag_bytes != (uint64_t)N || h.pop_bytes != (uint64_t)pop_k_bytes * c->Q ||
        h.mom_bytes != (uint64_t)mom_k_bytes * n_moments(c))
        return bail(LB_ERR_IO, "section sizes do not match the header");
    // pass 1: every CRC, before anything in the context changes
    std::vector<uint8_t> buf(std::max(pop_k_bytes, mom_k_bytes));
    uint32_t crc[3] = {0, 0, 0};
    const uint64_t sizes[3] = {h.flag_bytes, h.pop_bytes, h.mom_bytes};
    for (int s = 0; s < 3; s++)
        if (!stream_section(fp, sizes[s], buf, [&](const uint8_t *p, size_t n) {
                crc[s] = crc32_update(crc[s], p, n);
            }))
            return bail(LB_ERR_IO, "file is truncated");
    if (crc[0] != h.crc_flags || crc[1] != h.crc_pop || crc[2] != h.crc_mom)
        return bail(LB_ERR_IO, "checkpoint data damaged (CRC)");
    // pass 2: upload
    if (fseek(fp, (long)sizeof(CkptHeader), SEEK_SET) != 0) return bail(LB_ERR_IO, "seek failed");
    std::vector<uint8_t> flags((size_t)N);
    if (fread(flags.data(), 1, (size_t)N, fp) != (size_t)N) return bail(LB_ERR_IO, "read failed");
    auto upload = [&](void *dev, size_t bytes) -> int {
        if (fread(buf.data(), 1, bytes, fp) != bytes) return LB_ERR_IO;
        cudaError_t e = cudaMemcpyAsync(dev, buf.data(), bytes, cudaMemcpyHostToDevice, c->stream);
        if (e == cudaSuccess) e = cudaStreamSynchronize(c->stream);  // buf is reused
        return e == cudaSuccess ? LB_OK : LB_ERR_CUDA;
    };
    int rc = LB_OK;
    for (int k = 0; k < c->Q && rc == LB_OK; k++) rc = upload(pop_k(c, c->cur, k), pop_k_bytes);
    for (int i = 0; i < n_moments(c) && rc == LB_OK; i++) rc = upload(mom_k(c, i), mom_k_bytes);
    if (rc == LB_OK && mirror_sets(c) != cudaSuccess) rc = LB_ERR_CUDA;
    fclose(fp);
    if (rc == LB_ERR_IO) return fail(c, rc, "lb_checkpoint_load: read failed");
    if (rc != LB_OK) return fail(c, rc, "lb_checkpoint_load: copy to the device failed");
    rc = lb_set_flags(c, flags.data());  // re-derives the wall-neighbour bits and solid_bound
    if (rc != LB_OK) return rc;
    c->steps = h.steps;
    return LB_OK;
}

int lb_checkpoint_create(const char *path, lb_ctx **out) {
    if (!path || !out) return LB_ERR_ARG;
    *out = nullptr;
    lb_config cfg;
    int rc = lb_checkpoint_info(path, &cfg, nullptr);
    if (rc != LB_OK) return rc;
    lb_ctx *c = nullptr;
    rc = lb_create(&cfg, &c);
    if (rc != LB_OK) {
        abi_record_error("lb_checkpoint_create", "lb_create failed for the stored configuration");
        return rc;
    }
    rc = lb_checkpoint_load(c, path);
    if (rc != LB_OK) {
        abi_record_error("lb_checkpoint_create", c->err.c_str());
        lb_destroy(c);
        return rc;
    }
    *out = c;
    return LB_OK;
}

int lb_vtk_save_ctx(lb_ctx *c, const char *dir, int vtk_id) {
    if (!c) return LB_ERR_ARG;
    const long N = c->N;
    std::vector<float> m((size_t)N * 4, 0.f);
    int rc = lb_get_moments(c, m.data(), m.data() + N, m.data() + 2 * N,
                            c->Q == 19 ? m.data() + 3 * N : nullptr);
    if (rc != LB_OK) return rc;
    rc = lb_vtk_save(dir, vtk_id, 0, c->cfg.nx, c->cfg.ny, c->cfg.nz, m.data(), m.data() + N,
                     m.data() + 2 * N, c->Q == 19 ? m.data() + 3 * N : nullptr);
    if (rc != LB_OK) return fail(c, rc, lb_abi_last_error());
    return LB_OK;
}

}  // extern "C"

// ----------------------------------------------------------------- z-slabs
// The multi-device decomposition of a D3Q19 lattice (the reference's x-slab
// halo exchange get_border -> copy_border -> apply_border,
// src/get_border.cu:59-98, src/copy_border.cu:49-81, src/apply_border.cu:58-97,
// driven from src/simulation_d3q19.cu:363-406), here along z, the slowest
// axis, so that a face is contiguous: each of the 5 populations crossing a face
// is one plane of its array.  Populations leaving through the upper face have
// c_z = +1, through the lower face c_z = -1.
namespace {

const int kUp[5] = {5, 9, 13, 15, 17};     // c_z = +1
const int kDown[5] = {6, 10, 14, 16, 18};  // c_z = -1

long plane_of(const lb_ctx *c) { return (long)c->cfg.nx * c->cfg.ny; }

void *plane_ptr(lb_ctx *c, int set, int k, int z) {
    return static_cast<char *>((void *)pop_k(c, set, k)) + (size_t)z * plane_of(c) * c->esize;
}

// the faces of population set `set`: the c_z = -1 populations of plane 1 into
// to_below, the c_z = +1 populations of plane slab_nz into to_above, each a
// [5][nx * ny] array in the storage type
cudaError_t slab_pack(lb_ctx *c, int set, void *to_below, void *to_above, cudaStream_t s) {
    const void *src[10];
    void *dst[10];
    int n = 0;
    const size_t pb = (size_t)plane_of(c) * c->esize;
    for (int i = 0; i < 5; i++) {
        if (to_below) {
            src[n] = plane_ptr(c, set, kDown[i], 1);
            dst[n++] = static_cast<char *>(to_below) + i * pb;
        }
        if (to_above) {
            src[n] = plane_ptr(c, set, kUp[i], c->slab_nz);
            dst[n++] = static_cast<char *>(to_above) + i * pb;
        }
    }
    c->launches += n ? 1 : 0;
    return launch_plane_copy(src, dst, n, (long)pb, s);
}

// the neighbours' faces into the ghost planes of set `set`: the lower
// neighbour's upper face (c_z = +1) into plane 0, the upper neighbour's lower
// face (c_z = -1) into plane slab_nz + 1
cudaError_t slab_unpack(lb_ctx *c, int set, const void *from_below, const void *from_above,
                        cudaStream_t s) {
    const void *src[10];
    void *dst[10];
    int n = 0;
    const size_t pb = (size_t)plane_of(c) * c->esize;
    for (int i = 0; i < 5; i++) {
        if (from_below) {
            src[n] = static_cast<const char *>(from_below) + i * pb;
            dst[n++] = plane_ptr(c, set, kUp[i], 0);
        }
        if (from_above) {
            src[n] = static_cast<const char *>(from_above) + i * pb;
            dst[n++] = plane_ptr(c, set, kDown[i], c->slab_nz + 1);
        }
    }
    c->launches += n ? 1 : 0;
    return launch_plane_copy(src, dst, n, (long)pb, s);
}

}  // namespace

extern "C" {

int lb_slab_create(const lb_config *global, int z0, int nz, lb_ctx **out) {
    if (!global || !out) return LB_ERR_ARG;
    *out = nullptr;
    if (global->lattice != LB_D3Q19 || global->mode != LB_MODE_NATIVE || global->G != 0.f ||
        nz < 1 || z0 < 0 || z0 + nz > global->nz) {
        abi_record_error("lb_slab_create", "D3Q19 native mode without Shan-Chen, "
                                           "0 <= z0 and z0 + nz <= the global nz");
        return LB_ERR_ARG;
    }
    lb_config cfg = *global;
    cfg.nz = nz + 2;  // the own planes and one ghost plane on each side
    lb_ctx *c = nullptr;
    int rc = lb_create(&cfg, &c);
    if (rc != LB_OK) return rc;
    c->slab_nz = nz;
    c->slab_z0 = z0;
    c->slab_nz_global = global->nz;
    cudaError_t e = cudaStreamCreateWithFlags(&c->side, cudaStreamNonBlocking);
    for (cudaEvent_t *ev : {&c->ev_in, &c->ev_done, &c->ev_pack, &c->ev_fork})
        if (e == cudaSuccess) e = cudaEventCreateWithFlags(ev, cudaEventDisableTiming);
    const size_t fb = (size_t)5 * plane_of(c) * c->esize;
    for (int i = 0; i < 2; i++)
        for (int j = 0; j < 2; j++)
            if (e == cudaSuccess) e = cudaMalloc(&c->face[i][j], fb);
    if (e != cudaSuccess) {
        lb_destroy(c);
        return e == cudaErrorMemoryAllocation ? LB_ERR_NOMEM : LB_ERR_CUDA;
    }
    *out = c;
    return LB_OK;
}

int lb_slab_info(const lb_ctx *c, int *z0, int *nz, int *nz_global, size_t *face_bytes) {
    if (!c || !c->slab_nz) return LB_ERR_ARG;
    if (z0) *z0 = c->slab_z0;
    if (nz) *nz = c->slab_nz;
    if (nz_global) *nz_global = c->slab_nz_global;
    if (face_bytes) *face_bytes = (size_t)5 * plane_of(c) * c->esize;
    return LB_OK;
}

void *lb_stream(lb_ctx *c) { return c ? (void *)c->stream : nullptr; }

int lb_slab_pack(lb_ctx *c, void *to_below, void *to_above) {
    if (!c || !c->slab_nz) return fail(c, LB_ERR_ARG, "lb_slab_pack: not a slab");
    LB_TRY(c, "lb_slab_pack", slab_join(c));
    LB_TRY(c, "lb_slab_pack", slab_pack(c, c->cur, to_below, to_above, c->stream));
    return LB_OK;
}

int lb_slab_step(lb_ctx *c, int moments, void *to_below, void *to_above) {
    if (!c || !c->slab_nz) return fail(c, LB_ERR_ARG, "lb_slab_step: not a slab");
    LB_TRY(c, "lb_slab_step", slab_join(c));
    const int from = c->cur, to = 1 - from, nz = c->slab_nz;
    const D3Args a = d3_args(c, from);
    const bool mom = moments != 0;
    // interior planes 2 .. nz - 1 on the side stream, after everything queued so far
    if (nz > 2) {
        LB_TRY(c, "lb_slab_step", cudaEventRecord(c->ev_in, c->stream));
        LB_TRY(c, "lb_slab_step", cudaStreamWaitEvent(c->side, c->ev_in, 0));
    }
    // the two boundary planes 1 and nz first, then their faces, on the main stream
    LB_TRY(c, "lb_slab_step", launch_d3q19_native_planes(a, c->cfg.storage, mom, 1, nz - 2,
                                                         nz == 1 ? 1 : 2, c->stream));
    c->launches += 1;
    if (to_below || to_above)
        LB_TRY(c, "lb_slab_step", slab_pack(c, to, to_below, to_above, c->stream));
    if (nz > 2) {
        LB_TRY(c, "lb_slab_step",
               launch_d3q19_native_planes(a, c->cfg.storage, mom, 2, 0, nz - 2, c->side));
        c->launches += 1;
        LB_TRY(c, "lb_slab_step", cudaEventRecord(c->ev_done, c->side));
        c->interior_pending = true;
    }
    c->cur = to;
    c->steps += 1;
    return LB_OK;
}

int lb_slab_unpack(lb_ctx *c, const void *from_below, const void *from_above) {
    if (!c || !c->slab_nz) return fail(c, LB_ERR_ARG, "lb_slab_unpack: not a slab");
    LB_TRY(c, "lb_slab_unpack", slab_unpack(c, c->cur, from_below, from_above, c->stream));
    LB_TRY(c, "lb_slab_unpack", slab_join(c));
    return LB_OK;
}

}  // extern "C"

namespace {

// one step of every slab of a group, the faces moved by device copies (the
// unpack kernel of each slab reads its neighbours' packed faces); packs
// alternate between two buffers by step parity, so a slab's next pack never
// overwrites a face its neighbours may still be reading
int group_step_once(lb_ctx *const *slabs, int n, bool moments) {
    auto bad = [&](lb_ctx *c, cudaError_t e) {
        cuda_fail(c, "lb_slab_group_step", e);
        abi_record_error("lb_slab_group_step", c->err.c_str());
        return LB_ERR_CUDA;
    };
    for (int i = 0; i < n; i++) {
        lb_ctx *c = slabs[i];
        int rc = lb_slab_step(c, moments ? 1 : 0, c->face[c->parity][0], c->face[c->parity][1]);
        if (rc != LB_OK) {
            abi_record_error("lb_slab_group_step", c->err.c_str());
            return rc;
        }
        cudaError_t e = cudaEventRecord(c->ev_pack, c->stream);
        if (e != cudaSuccess) return bad(c, e);
    }
    for (int i = 0; i < n; i++) {
        lb_ctx *c = slabs[i], *lo = slabs[(i + n - 1) % n], *hi = slabs[(i + 1) % n];
        cudaError_t e = cudaSuccess;
        if (lo != c) e = cudaStreamWaitEvent(c->stream, lo->ev_pack, 0);
        if (e == cudaSuccess && hi != c && hi != lo)
            e = cudaStreamWaitEvent(c->stream, hi->ev_pack, 0);
        if (e != cudaSuccess) return bad(c, e);
        int rc = lb_slab_unpack(c, lo->face[lo->parity][1], hi->face[hi->parity][0]);
        if (rc != LB_OK) {
            abi_record_error("lb_slab_group_step", c->err.c_str());
            return rc;
        }
    }
    for (int i = 0; i < n; i++) slabs[i]->parity ^= 1;
    return LB_OK;
}

// slabs[1..] wait for the work queued so far on slabs[0]'s stream (or the
// reverse with `join`): the group's streams fork from and join into it
cudaError_t group_fork(lb_ctx *const *slabs, int n) {
    lb_ctx *c0 = slabs[0];
    cudaError_t e = cudaEventRecord(c0->ev_fork, c0->stream);
    for (int i = 1; i < n && e == cudaSuccess; i++)
        e = cudaStreamWaitEvent(slabs[i]->stream, c0->ev_fork, 0);
    return e;
}
cudaError_t group_join(lb_ctx *const *slabs, int n) {
    lb_ctx *c0 = slabs[0];
    cudaError_t e = cudaSuccess;
    for (int i = 1; i < n && e == cudaSuccess; i++) {
        e = cudaEventRecord(slabs[i]->ev_fork, slabs[i]->stream);
        if (e == cudaSuccess) e = cudaStreamWaitEvent(c0->stream, slabs[i]->ev_fork, 0);
    }
    return e;
}

// G steps of the group (G even: every slab returns to its population set and
// face parity) captured once as one graph on slabs[0]'s stream
int group_graph(lb_ctx *const *slabs, int n, int G, cudaGraphExec_t *out) {
    lb_ctx *c0 = slabs[0];
    const std::vector<lb_ctx *> key(slabs, slabs + n);
    if (c0->grp_key != key) {
        for (int i = 0; i < 2; i++)
            for (int j = 0; j < 2; j++)
                if (c0->grp_graph[i][j]) {
                    cudaGraphExecDestroy(c0->grp_graph[i][j]);
                    c0->grp_graph[i][j] = nullptr;
                }
        c0->grp_key = key;
    }
    cudaGraphExec_t &slot = c0->grp_graph[c0->cur][c0->parity];
    if (slot) { *out = slot; return LB_OK; }
    std::vector<int64_t> before(n), steps_before(n);
    for (int i = 0; i < n; i++) {
        before[i] = slabs[i]->launches;
        steps_before[i] = slabs[i]->steps;
    }
    cudaError_t e = cudaStreamBeginCapture(c0->stream, cudaStreamCaptureModeThreadLocal);
    int rc = LB_OK;
    if (e == cudaSuccess) e = group_fork(slabs, n);
    for (int t = 0; t < G && e == cudaSuccess && rc == LB_OK; t++)
        rc = group_step_once(slabs, n, false);
    if (e == cudaSuccess && rc == LB_OK) e = group_join(slabs, n);
    cudaGraph_t graph = nullptr;
    const cudaError_t e2 = cudaStreamEndCapture(c0->stream, &graph);
    for (int i = 0; i < n; i++) {  // capture launches nothing and advances no step
        slabs[i]->launches = before[i];
        slabs[i]->steps = steps_before[i];
    }
    if (rc != LB_OK) return rc;
    if (e == cudaSuccess) e = e2;
    if (e == cudaSuccess) e = cudaGraphInstantiate(&slot, graph, 0);
    if (graph) cudaGraphDestroy(graph);
    if (e != cudaSuccess) {
        slot = nullptr;
        abi_record_error("lb_slab_group_step (graph capture)", cudaGetErrorString(e));
        return LB_ERR_CUDA;
    }
    *out = slot;
    return LB_OK;
}

}  // namespace

extern "C" {

int lb_slab_group_step(lb_ctx *const *slabs, int n, int nsteps) {
    if (!slabs || n < 1 || nsteps < 0) return LB_ERR_ARG;
    int dev = -1;
    for (int i = 0; i < n; i++) {
        lb_ctx *c = slabs[i];
        const lb_ctx *p = slabs[(i + n - 1) % n];
        if (!c || !c->slab_nz || c->cfg.nx != slabs[0]->cfg.nx ||
            c->cfg.ny != slabs[0]->cfg.ny || c->esize != slabs[0]->esize ||
            c->slab_nz_global != slabs[0]->slab_nz_global ||
            (p->slab_z0 + p->slab_nz) % c->slab_nz_global != c->slab_z0) {
            abi_record_error("lb_slab_group_step", "slabs of one lattice, in z order, "
                                                   "covering it without gaps");
            return LB_ERR_ARG;
        }
    }
    if (cudaGetDevice(&dev) != cudaSuccess) return LB_ERR_CUDA;
    for (int i = 0; i < n; i++) {  // a caller's earlier steps may leave interior planes open
        if (slab_join(slabs[i]) != cudaSuccess) return LB_ERR_CUDA;
    }
    // all but the last step in graphs of G steps; the last writes the moments
    const int G = std::max(2, slabs[0]->cfg.graph_steps & ~1);
    int rest = nsteps - 1;
    if (rest >= G) {
        if (group_join(slabs, n) != cudaSuccess) return LB_ERR_CUDA;
        while (rest >= G) {
            cudaGraphExec_t gr;
            int rc = group_graph(slabs, n, G, &gr);
            if (rc != LB_OK) return rc;
            const cudaError_t e = cudaGraphLaunch(gr, slabs[0]->stream);
            if (e != cudaSuccess) {
                abi_record_error("lb_slab_group_step", cudaGetErrorString(e));
                return LB_ERR_CUDA;
            }
            for (int i = 0; i < n; i++) {
                lb_ctx *c = slabs[i];
                c->launches += (int64_t)G * (c->slab_nz > 2 ? 4 : 3);
                c->steps += G;  // G is even: every slab is back on its set and parity
            }
            rest -= G;
        }
        if (group_fork(slabs, n) != cudaSuccess) return LB_ERR_CUDA;
    }
    for (; rest > 0; rest--) {
        const int rc = group_step_once(slabs, n, false);
        if (rc != LB_OK) return rc;
    }
    return nsteps > 0 ? group_step_once(slabs, n, true) : LB_OK;
}

int lb_slab_group_time(lb_ctx *const *slabs, int n, int nsteps, float *ms) {
    if (!slabs || n < 1 || !ms || !slabs[0]) return LB_ERR_ARG;
    lb_ctx *c0 = slabs[0];
    // every slab starts after the start event and the stop event follows every slab
    cudaError_t e = cudaEventRecord(c0->ev0, c0->stream);
    for (int i = 1; i < n && e == cudaSuccess; i++)
        e = cudaStreamWaitEvent(slabs[i]->stream, c0->ev0, 0);
    if (e != cudaSuccess) {
        abi_record_error("lb_slab_group_time", cudaGetErrorString(e));
        return LB_ERR_CUDA;
    }
    int rc = lb_slab_group_step(slabs, n, nsteps);
    if (rc != LB_OK) return rc;
    for (int i = 1; i < n && e == cudaSuccess; i++) {
        e = cudaEventRecord(slabs[i]->ev1, slabs[i]->stream);
        if (e == cudaSuccess) e = cudaStreamWaitEvent(c0->stream, slabs[i]->ev1, 0);
    }
    if (e == cudaSuccess) e = cudaEventRecord(c0->ev1, c0->stream);
    if (e == cudaSuccess) e = cudaEventSynchronize(c0->ev1);
    if (e == cudaSuccess) e = cudaEventElapsedTime(ms, c0->ev0, c0->ev1);
    if (e != cudaSuccess) {
        abi_record_error("lb_slab_group_time", cudaGetErrorString(e));
        return LB_ERR_CUDA;
    }
    return LB_OK;
}

}  // extern "C"

extern "C" {

// ----------------------------------------------------------------- drop-in reductions
// Scratch (first-pass partials + the 7 results) of the drop-in reductions,
// one allocation per device ordinal, made on the first call with that device
// current: the caller may drive several devices (one DataD3Q19 per device,
// as the reference's host loop does), and each call sums on the device that
// is current when it is made.
static std::mutex g_red_mu;
static std::unordered_map<int, double *> g_red;  // device ordinal -> scratch

static int abi_reduce(const char *where, const float *rho, const float *ux, const float *uy,
                      const float *uz, const void *solid, long N, double out[7]) {
    std::lock_guard<std::mutex> l(g_red_mu);
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) {
        abi_record_error(where, cudaGetErrorString(e));
        return LB_ERR_CUDA;
    }
    double *&scratch = g_red[dev];
    if (!scratch) {
        e = cudaMalloc(&scratch, sizeof(double) * (reduce_partials_size() + 8));
        if (e != cudaSuccess) {
            scratch = nullptr;
            abi_record_error(where, cudaGetErrorString(e));
            return LB_ERR_NOMEM;
        }
    }
    double *res = scratch + reduce_partials_size();
    e = launch_reduce(rho, ux, uy, uz, reinterpret_cast<const uint8_t *>(solid), 0xff, N,
                      scratch, res, 0);
    if (e == cudaSuccess) e = cudaMemcpy(out, res, sizeof(double) * 7, cudaMemcpyDeviceToHost);
    if (e != cudaSuccess) {
        abi_record_error(where, cudaGetErrorString(e));
        return LB_ERR_CUDA;
    }
    return LB_OK;
}

int lb_reduce_d3q19(const DataD3Q19 *d, double out[7]) {
    if (!d || !out) {
        abi_record_error("lb_reduce_d3q19", "null data or output");
        return LB_ERR_ARG;
    }
    return abi_reduce("lb_reduce_d3q19", d->rho, d->ux, d->uy, d->uz, d->solid,
                      (long)d->width * d->height * d->depth, out);
}

int lb_reduce_d2q9(const DataD2Q9 *d, double out[7]) {
    if (!d || !out) {
        abi_record_error("lb_reduce_d2q9", "null data or output");
        return LB_ERR_ARG;
    }
    return abi_reduce("lb_reduce_d2q9", d->rho, d->ux, d->uy, nullptr, d->solid,
                      (long)d->width * d->height, out);
}

// ----------------------------------------------------------------- device helpers
int lb_device_count(int *n) {
    if (!n) return LB_ERR_ARG;
    return cudaGetDeviceCount(n) == cudaSuccess ? LB_OK : LB_ERR_CUDA;
}
int lb_set_device(int dev) {
    const cudaError_t e = cudaSetDevice(dev);
    if (e != cudaSuccess) {
        abi_record_error("lb_set_device", cudaGetErrorString(e));
        return e == cudaErrorInvalidDevice ? LB_ERR_ARG : LB_ERR_CUDA;
    }
    return LB_OK;
}
int lb_malloc(void **p, size_t bytes) {
    if (!p) return LB_ERR_ARG;
    return cudaMalloc(p, bytes) == cudaSuccess ? LB_OK : LB_ERR_NOMEM;
}
int lb_free(void *p) { return cudaFree(p) == cudaSuccess ? LB_OK : LB_ERR_CUDA; }
int lb_malloc_host(void **p, size_t bytes) {
    if (!p) return LB_ERR_ARG;
    return cudaMallocHost(p, bytes) == cudaSuccess ? LB_OK : LB_ERR_NOMEM;
}
int lb_free_host(void *p) { return cudaFreeHost(p) == cudaSuccess ? LB_OK : LB_ERR_CUDA; }
int lb_memcpy_h2d(void *dst, const void *src, size_t bytes) {
    return cudaMemcpy(dst, src, bytes, cudaMemcpyHostToDevice) == cudaSuccess ? LB_OK : LB_ERR_CUDA;
}
int lb_memcpy_d2h(void *dst, const void *src, size_t bytes) {
    return cudaMemcpy(dst, src, bytes, cudaMemcpyDeviceToHost) == cudaSuccess ? LB_OK : LB_ERR_CUDA;
}
int lb_memset(void *dst, int value, size_t bytes) {
    return cudaMemset(dst, value, bytes) == cudaSuccess ? LB_OK : LB_ERR_CUDA;
}
int lb_device_synchronize(void) {
    return cudaDeviceSynchronize() == cudaSuccess ? LB_OK : LB_ERR_CUDA;
}

}  // extern "C"

// installs (ca != nullptr) or removes the learned closure of a context; the
// closure kernel handles D3Q19 native mode with FP32 storage and no Shan-Chen
int lb::context_set_closure(lb_ctx *c, const ClosureArgs *ca) {
    if (!c) return LB_ERR_ARG;
    if (ca && (c->Q != 19 || c->cfg.mode != LB_MODE_NATIVE || c->cfg.storage != LB_STORE_F32 ||
               sc_on(c) || c->slab_nz))
        return fail(c, LB_ERR_ARG, "closure: D3Q19 native mode, FP32 storage, no Shan-Chen");
    LB_TRY(c, "closure", cudaStreamSynchronize(c->stream));
    drop_graphs(c);
    c->closure_on = ca != nullptr;
    if (ca) c->closure = *ca;
    return LB_OK;
}
