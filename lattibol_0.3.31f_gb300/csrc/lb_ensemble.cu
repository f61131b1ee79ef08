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
// (same device functions, same order), so a domain of the ensemble evolves
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
                float rho, ux, uy;
                d2q9_moments(g, rho, ux, uy);
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
            d2q9_moments(g, rho, ux, uy);
            const int xm = x == 0 ? dm.W - 1 : x - 1, xp = x == dm.W - 1 ? 0 : x + 1;
            const int W = dm.W;
            const float ps[9] = {__ldg(psi + x + W * y),   __ldg(psi + xp + W * y),
                                 __ldg(psi + x + W * rp),  __ldg(psi + xm + W * y),
                                 __ldg(psi + x + W * rm),  __ldg(psi + xp + W * rp),
                                 __ldg(psi + xm + W * rp), __ldg(psi + xm + W * rm),
                                 __ldg(psi + xp + W * rm)};
            float ex = ux, ey = uy;
            d2q9_sc_shift(ps, a.w1, a.w5, dm.G, dm.tau_inv, rho, ex, ey);
            d2q9_bgk(g, ex, ey, rho, a.w0, a.w1, a.w5, dm.tau_inv);
            const int o = dm.off + x + W * y;
            if (MOM) { a.rho[o] = rho; a.ux[o] = ux; a.uy[o] = uy; }
#pragma unroll
            for (int k = 0; k < 9; k++) a.dst[k][o] = g[k];
        }
    }
}

struct LaunchShape {
    int bx, ry, bps;  // threads along x, rows per work item (= blockDim.y), blocks per SM
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
    int cur = 0, psi_form = LB_PSI_EXP1, sms = 1, graph_steps = 32;
    LaunchShape shape{128, 1, 4};
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

cudaError_t ens_step(lb_ensemble *e, int from, bool mom) {
    const EnsArgs a = args_for(e, from);
    const dim3 block(e->shape.bx, e->shape.ry);
    const unsigned grid = (unsigned)std::max(1, std::min(e->nitems, e->sms * e->shape.bps));
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
    std::vector<EnsItem> items;
    for (int d = 0; d < e->nd; d++)
        for (int y = 0; y < e->dom[d].H; y += e->shape.ry) {
            const EnsDomain &m = e->dom[d];
            items.push_back(EnsItem{m.off, m.W, m.H, y, m.G, m.tau_inv});
        }
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
        e->launches += 2L * e->graph_steps;
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
    if (!e || threads_x < 32 || threads_x % 32 || rows < 1 || threads_x * rows > 1024 ||
        blocks_per_sm < 1 || blocks_per_sm > 32)
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
    static const int BX[3] = {64, 128, 256}, RY[3] = {1, 2, 4}, BPS[3] = {2, 4, 8};
    float best = 1e30f;
    LaunchShape pick = e->shape;
    for (int i = 0; i < 3; i++)
        for (int j = 0; j < 3; j++)
            for (int k = 0; k < 3; k++) {
                if (BX[i] * RY[j] > 512) continue;
                int rc = lb_ensemble_set_launch(e, BX[i], RY[j], BPS[k]);
                if (rc != LB_OK) return rc;
                for (int s = 0; s < 1; s++) {
                    LB_ETRY(e, "autotune", ens_step(e, e->cur, false));
                    e->cur = 1 - e->cur;
                }
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
