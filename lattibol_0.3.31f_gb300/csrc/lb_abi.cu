// lb_abi.cu -- the reference's extern "C" entry points (include/lbgb300.h,
// part 1), implemented on this library's kernels.
//
// Two modes (lb_abi_set_mode):
//  * standalone (default): streaming_* is the reference's in-place swap
//    streaming, collision_* the in-place collision; bit-identical to the
//    reference kernels, two passes over the populations per step.
//  * fused: streaming_* only records that a step has begun; collision_* runs
//    one pull-stream + collide pass from the caller's populations into a
//    second, library-owned set and then points data->f0..f18 at it (the next
//    step goes back).  One pass per step; the results are the same bits.
// Like the reference, everything runs on the legacy default stream.
#include <mutex>
#include <string>
#include <unordered_map>

#include "../../include/lbgb300.h"
#include "lb_kernels.cuh"

using namespace lb;

namespace {

thread_local std::string g_err;
int g_mode = LB_ABI_STANDALONE;
std::mutex g_mu;

void set_err(const char *where, cudaError_t e) {
    g_err = std::string(where) + ": " + cudaGetErrorString(e);
}
void set_err(const char *where, const char *what) { g_err = std::string(where) + ": " + what; }

template <int Q> struct Shadow {
    float *orig[Q];   // the caller's population pointers at registration
    float *lib[Q];    // the library's second set
    float *block;     // allocation backing lib[]
    long n;
    bool pending;     // streaming_* seen since the last collision_*
};
std::unordered_map<const void *, Shadow<19>> g_sh3;
std::unordered_map<const void *, Shadow<9>> g_sh2;

template <int Q> Pop<Q> pop_of(float *const *f) {
    Pop<Q> p;
    for (int k = 0; k < Q; k++) p.f[k] = f[k];
    return p;
}
template <int Q> CPop<Q> cpop_of(float *const *f) {
    CPop<Q> p;
    for (int k = 0; k < Q; k++) p.f[k] = f[k];
    return p;
}

float **d3_pops(DataD3Q19 *d) { return &d->f0; }
float **d2_pops(DataD2Q9 *d) { return &d->f0; }

// returns the shadow record of `key`, creating it (and allocating the second
// population set) if needed; nullptr on allocation failure
template <int Q>
Shadow<Q> *shadow_for(std::unordered_map<const void *, Shadow<Q>> &m, const void *key,
                      float **cur, long n) {
    auto it = m.find(key);
    if (it != m.end()) {
        Shadow<Q> &s = it->second;
        bool ours = true, theirs = true;
        for (int k = 0; k < Q; k++) {
            ours = ours && cur[k] == s.lib[k];
            theirs = theirs && cur[k] == s.orig[k];
        }
        if (s.n == n && (ours || theirs)) return &s;
        cudaFree(s.block);  // the caller swapped buffers or resized: start over
        m.erase(it);
    }
    Shadow<Q> s{};
    s.n = n;
    const long stride = (n + 63) / 64 * 64;
    if (cudaMalloc(&s.block, sizeof(float) * stride * Q) != cudaSuccess) return nullptr;
    for (int k = 0; k < Q; k++) {
        s.orig[k] = cur[k];
        s.lib[k] = s.block + stride * k;
    }
    return &(m[key] = s);
}

D3Args d3_args(DataD3Q19 *d) {
    D3Args a{};
    a.flags = reinterpret_cast<const uint8_t *>(d->solid);
    a.sb = reinterpret_cast<const uint8_t *>(d->solid_bound);
    a.ux = d->ux; a.uy = d->uy; a.uz = d->uz; a.rho = d->rho;
    a.W = d->width; a.H = d->height; a.D = d->depth;
    a.dev = d->dev; a.ndev = d->deviceCount;
    return a;
}

D2Args d2_args(DataD2Q9 *d) {
    D2Args a{};
    a.flags = reinterpret_cast<const uint8_t *>(d->solid);
    a.sb = reinterpret_cast<const uint8_t *>(d->solid_bound);
    a.ux = d->ux; a.uy = d->uy; a.rho = d->rho;
    a.psi = d->psi; a.ueq_x = d->ueq_x; a.ueq_y = d->ueq_y;
    a.W = d->width; a.H = d->height;
    a.dev = d->dev; a.ndev = d->deviceCount;
    return a;
}

bool bad_d3(const DataD3Q19 *d, const char *where) {
    if (!d || d->width <= 0 || d->height <= 0 || d->depth <= 0) {
        set_err(where, "null data or non-positive extent");
        return true;
    }
    return false;
}
bool bad_d2(const DataD2Q9 *d, const char *where) {
    if (!d || d->width <= 0 || d->height <= 0) {
        set_err(where, "null data or non-positive extent");
        return true;
    }
    return false;
}

}  // namespace

void lb::abi_record_error(const char *where, const char *what) { set_err(where, what); }

extern "C" {

int lb_abi_set_mode(int mode) {
    if (mode != LB_ABI_STANDALONE && mode != LB_ABI_FUSED) return LB_ERR_ARG;
    std::lock_guard<std::mutex> l(g_mu);
    g_mode = mode;
    return LB_OK;
}
int lb_abi_get_mode(void) { return g_mode; }
const char *lb_abi_last_error(void) { return g_err.c_str(); }
int lb_abi_clear_error(void) {
    g_err.clear();
    return LB_OK;
}

// ----------------------------------------------------------------- D3Q19
void streaming_d3q19(DataD3Q19 *data, dim3, dim3) {
    if (bad_d3(data, "streaming_d3q19")) return;
    std::lock_guard<std::mutex> l(g_mu);
    const long n = (long)data->width * data->height * data->depth;
    if (g_mode == LB_ABI_FUSED && data->deviceCount <= 1) {
        Shadow<19> *s = shadow_for(g_sh3, data, d3_pops(data), n);
        if (!s) { set_err("streaming_d3q19", "cannot allocate the second population set"); return; }
        s->pending = true;
        return;
    }
    cudaError_t e = launch_d3q19_stream_swap(pop_of<19>(d3_pops(data)),
                                             reinterpret_cast<const uint8_t *>(data->solid_bound),
                                             data->width, data->height, data->depth, 0);
    if (e != cudaSuccess) set_err("streaming_d3q19", e);
}

}  // extern "C"

namespace {
// collision_d3q19's work.  In fused mode a non-null probe (device-accessible,
// 16-byte aligned) receives the (ux, uy, uz, rho) that the pass writes into
// the plot buffer at node probe_o.  Returns true when the fused pass ran.
bool collide_d3q19(float *plot_data, DataD3Q19 *data, float w0, float w1, float w7,
                   float tau_inv, float ux_in, float rho_out, float4 *probe, int probe_o) {
    if (bad_d3(data, "collision_d3q19")) return false;
    std::lock_guard<std::mutex> l(g_mu);
    D3Args a = d3_args(data);
    a.w0 = w0; a.w1 = w1; a.w7 = w7; a.tau_inv = tau_inv; a.ux_in = ux_in; a.rho_out = rho_out;
    a.plot = reinterpret_cast<float4 *>(plot_data);
    float **cur = d3_pops(data);
    auto it = g_sh3.find(data);
    if (it != g_sh3.end() && it->second.pending) {
        Shadow<19> &s = it->second;
        bool ours = true;
        for (int k = 0; k < 19; k++) ours = ours && cur[k] == s.lib[k];
        float *const *dst = ours ? s.orig : s.lib;
        a.src = cpop_of<19>(cur);
        a.dst = pop_of<19>(dst);
        a.probe = probe;
        a.probe_o = probe_o;
        cudaError_t e = launch_d3q19_fused(a, MODE_REF, true, plot_data != nullptr, 0);
        s.pending = false;
        if (e != cudaSuccess) { set_err("collision_d3q19", e); return false; }
        for (int k = 0; k < 19; k++) cur[k] = dst[k];
        return true;
    }
    a.src = cpop_of<19>(cur);
    a.dst = pop_of<19>(cur);
    cudaError_t e = launch_d3q19_collide(a, plot_data != nullptr, 0);
    if (e != cudaSuccess) set_err("collision_d3q19", e);
    return false;
}
}  // namespace

extern "C" {

void collision_d3q19(float *plot_data, DataD3Q19 *data, float w0, float w1, float w7,
                     float tau_inv, float ux_in, float uy_in, float uz_in, float rho_out,
                     float u_min, float u_max, float rho_min, float rho_max, dim3, dim3) {
    (void)uy_in; (void)uz_in; (void)u_min; (void)u_max; (void)rho_min; (void)rho_max;
    collide_d3q19(plot_data, data, w0, w1, w7, tau_inv, ux_in, rho_out, nullptr, 0);
}

void get_border_d3q19(DataD3Q19 *data, dim3, dim3) {
    if (bad_d3(data, "get_border_d3q19")) return;
    Pop<10> b;
    float **bp = &data->border_f1;
    for (int j = 0; j < 10; j++) b.f[j] = bp[j];
    cudaError_t e = launch_d3q19_get_border(cpop_of<19>(d3_pops(data)), b, data->width,
                                            data->height, data->depth, 0);
    if (e != cudaSuccess) set_err("get_border_d3q19", e);
}

void apply_border_d3q19(DataD3Q19 *data, dim3, dim3) {
    if (bad_d3(data, "apply_border_d3q19")) return;
    CPop<10> nb;
    float **np = &data->nb_border_f1;
    for (int j = 0; j < 10; j++) nb.f[j] = np[j];
    cudaError_t e = launch_d3q19_apply_border(pop_of<19>(d3_pops(data)), nb, data->width,
                                              data->height, data->depth, 0);
    if (e != cudaSuccess) set_err("apply_border_d3q19", e);
}

void read_value_3d(float *plot_data, DataD3Q19 *data, int x, int y, int z) {
    if (bad_d3(data, "read_value_3d")) return;
    if (x < 0 || y < 0 || z < 0 || x >= data->width || y >= data->height || z >= data->depth) {
        set_err("read_value_3d", "cursor outside the lattice");
        return;
    }
    const long o = x + (long)y * data->width + (long)z * data->width * data->height;
    cudaError_t e = launch_read_value(plot_data, data->ux, data->uy, data->uz, data->rho,
                                      data->valueCur, o, 0);
    if (e == cudaSuccess) e = cudaDeviceSynchronize();  // as src/read_value.cu:57
    if (e != cudaSuccess) set_err("read_value_3d", e);
}

int lb_abi_release_d3q19(DataD3Q19 *data) {
    if (!data) return LB_ERR_ARG;
    std::lock_guard<std::mutex> l(g_mu);
    auto it = g_sh3.find(data);
    if (it == g_sh3.end()) return LB_OK;
    Shadow<19> &s = it->second;
    float **cur = d3_pops(data);
    bool ours = true;
    for (int k = 0; k < 19; k++) ours = ours && cur[k] == s.lib[k];
    if (ours) {
        for (int k = 0; k < 19; k++) {
            cudaError_t e = cudaMemcpy(s.orig[k], s.lib[k], sizeof(float) * s.n,
                                       cudaMemcpyDeviceToDevice);
            if (e != cudaSuccess) { set_err("lb_abi_release_d3q19", e); return LB_ERR_CUDA; }
            cur[k] = s.orig[k];
        }
    }
    cudaFree(s.block);
    g_sh3.erase(it);
    return LB_OK;
}

// ----------------------------------------------------------------- D2Q9
void streaming_d2q9(DataD2Q9 *data, dim3, dim3) {
    if (bad_d2(data, "streaming_d2q9")) return;
    std::lock_guard<std::mutex> l(g_mu);
    const long n = (long)data->width * data->height;
    if (g_mode == LB_ABI_FUSED && data->deviceCount <= 1) {
        Shadow<9> *s = shadow_for(g_sh2, data, d2_pops(data), n);
        if (!s) { set_err("streaming_d2q9", "cannot allocate the second population set"); return; }
        s->pending = true;
        return;
    }
    cudaError_t e = launch_d2q9_stream_swap(pop_of<9>(d2_pops(data)),
                                            reinterpret_cast<const uint8_t *>(data->solid_bound),
                                            data->width, data->height, 0);
    if (e != cudaSuccess) set_err("streaming_d2q9", e);
}

void collision_d2q9(float *plot_data, DataD2Q9 *data, float w0, float w1, float w5,
                    float tau_inv, float ux_in, float uy_in, float rho_out, float u_min,
                    float u_max, float rho_min, float rho_max, dim3, dim3, float Fx, float Fy,
                    float G, float Gads) {
    (void)uy_in; (void)u_min; (void)u_max; (void)rho_min; (void)rho_max;
    if (bad_d2(data, "collision_d2q9")) return;
    std::lock_guard<std::mutex> l(g_mu);
    D2Args a = d2_args(data);
    a.w0 = w0; a.w1 = w1; a.w5 = w5; a.tau_inv = tau_inv; a.ux_in = ux_in; a.rho_out = rho_out;
    a.Fx = Fx; a.Fy = Fy; a.G = G; a.Gads = Gads; a.psi_form = LB_PSI_REF;
    a.plot = reinterpret_cast<float4 *>(plot_data);
    float **cur = d2_pops(data);
    auto it = g_sh2.find(data);
    if (it != g_sh2.end() && it->second.pending) {
        Shadow<9> &s = it->second;
        bool ours = true;
        for (int k = 0; k < 9; k++) ours = ours && cur[k] == s.lib[k];
        float *const *dst = ours ? s.orig : s.lib;
        a.src = cpop_of<9>(cur);
        a.dst = pop_of<9>(dst);
        cudaError_t e = launch_d2q9_fused(a, MODE_REF, true, plot_data != nullptr, 0);
        s.pending = false;
        if (e != cudaSuccess) { set_err("collision_d2q9", e); return; }
        for (int k = 0; k < 9; k++) cur[k] = dst[k];
        return;
    }
    a.src = cpop_of<9>(cur);
    a.dst = pop_of<9>(cur);
    cudaError_t e = launch_d2q9_collide(a, plot_data != nullptr, 0);
    if (e != cudaSuccess) set_err("collision_d2q9", e);
}

void get_border_d2q9(DataD2Q9 *data, dim3, dim3) {
    if (bad_d2(data, "get_border_d2q9")) return;
    Pop<6> b;
    float **bp = &data->border_f1;
    for (int j = 0; j < 6; j++) b.f[j] = bp[j];
    cudaError_t e = launch_d2q9_get_border(cpop_of<9>(d2_pops(data)), b, data->width,
                                           data->height, 0);
    if (e != cudaSuccess) set_err("get_border_d2q9", e);
}

void apply_border_d2q9(DataD2Q9 *data, dim3, dim3) {
    if (bad_d2(data, "apply_border_d2q9")) return;
    CPop<6> nb;
    float **np = &data->nb_border_f1;
    for (int j = 0; j < 6; j++) nb.f[j] = np[j];
    cudaError_t e = launch_d2q9_apply_border(pop_of<9>(d2_pops(data)), nb, data->width,
                                             data->height, 0);
    if (e != cudaSuccess) set_err("apply_border_d2q9", e);
}

void read_value_2d(float *plot_data, DataD2Q9 *data, int x, int y, int z) {
    if (bad_d2(data, "read_value_2d")) return;
    if (x < 0 || y < 0 || x >= data->width || y >= data->height || z != 0) {
        set_err("read_value_2d", "cursor outside the lattice");
        return;
    }
    const long o = x + (long)y * data->width;
    cudaError_t e = launch_read_value(plot_data, data->ux, data->uy, nullptr, data->rho,
                                      data->valueCur, o, 0);
    if (e == cudaSuccess) e = cudaDeviceSynchronize();  // as src/read_value.cu:40
    if (e != cudaSuccess) set_err("read_value_2d", e);
}

int lb_abi_release_d2q9(DataD2Q9 *data) {
    if (!data) return LB_ERR_ARG;
    std::lock_guard<std::mutex> l(g_mu);
    auto it = g_sh2.find(data);
    if (it == g_sh2.end()) return LB_OK;
    Shadow<9> &s = it->second;
    float **cur = d2_pops(data);
    bool ours = true;
    for (int k = 0; k < 9; k++) ours = ours && cur[k] == s.lib[k];
    if (ours) {
        for (int k = 0; k < 9; k++) {
            cudaError_t e = cudaMemcpy(s.orig[k], s.lib[k], sizeof(float) * s.n,
                                       cudaMemcpyDeviceToDevice);
            if (e != cudaSuccess) { set_err("lb_abi_release_d2q9", e); return LB_ERR_CUDA; }
            cur[k] = s.orig[k];
        }
    }
    cudaFree(s.block);
    g_sh2.erase(it);
    return LB_OK;
}

int lb_run_lbm_d3q19(DataD3Q19 *data, float *plot_data, const lb_run_params_d3q19 *p, int steps,
                     float *value_host) {
    if (!data || !p || !value_host || steps < 0) return LB_ERR_ARG;
    const dim3 g(1, 1, 1), b(32, 4, 1);  // accepted and ignored, as by every entry point
    g_err.clear();
    if (bad_d3(data, "lb_run_lbm_d3q19")) return LB_ERR_ARG;
    const int cx = p->cursor[0], cy = p->cursor[1], cz = p->cursor[2];
    if (cx < 0 || cy < 0 || cz < 0 || cx >= data->width || cy >= data->height ||
        cz >= data->depth) {
        set_err("lb_run_lbm_d3q19", "cursor outside the lattice");
        return LB_ERR_ARG;
    }
    const long o = cx + (long)cy * data->width + (long)cz * data->width * data->height;
    // Each step's cursor value goes to value_host in stream order behind the
    // step, without read_value_3d's device-wide synchronisation, and the host
    // waits once, after the last step (as the per-step synchronous sequence
    // did, value_host then holds the last step's value):
    //  * page-locked, mapped value_host and the fused pass: the pass writes
    //    the cursor's plot value into it directly (its probe), and
    //    data->valueCur is filled once after the last step;
    //  * otherwise read_value_3d's kernel and a 16-byte copy per step.
    float4 *probe = nullptr;
    cudaPointerAttributes pa{};
    if (cudaPointerGetAttributes(&pa, value_host) == cudaSuccess &&
        pa.type == cudaMemoryTypeHost && pa.devicePointer &&
        reinterpret_cast<uintptr_t>(pa.devicePointer) % 16 == 0 && o < (1L << 31))
        probe = reinterpret_cast<float4 *>(pa.devicePointer);
    else
        (void)cudaGetLastError();
    bool probed = false;  // the last step's value went to value_host through the probe
    for (int i = 0; i < steps; i++) {
        streaming_d3q19(data, g, b);
        probed = collide_d3q19(plot_data, data, p->w0, p->w1, p->w7, p->tau_inv, p->ux_in,
                               p->rho_out, probe, (int)o) &&
                 probe && plot_data;
        if (!g_err.empty()) return LB_ERR_CUDA;
        if (probed) continue;
        cudaError_t e = launch_read_value(plot_data, data->ux, data->uy, data->uz, data->rho,
                                          data->valueCur, o, 0);
        if (e == cudaSuccess)
            e = cudaMemcpyAsync(value_host, data->valueCur, 4 * sizeof(float),
                                cudaMemcpyDeviceToHost, 0);
        if (e != cudaSuccess) { set_err("lb_run_lbm_d3q19", e); return LB_ERR_CUDA; }
    }
    cudaError_t e = probed ? launch_read_value(plot_data, data->ux, data->uy, data->uz,
                                               data->rho, data->valueCur, o, 0)
                           : cudaSuccess;
    if (e == cudaSuccess) e = cudaStreamSynchronize(0);
    if (e != cudaSuccess) { set_err("lb_run_lbm_d3q19", e); return LB_ERR_CUDA; }
    return LB_OK;
}

// ----------------------------------------------------------------- halo copies
// reference src/copy_border.cu:26-47: peer copies of the six D2Q9 face arrays
void copy_border_devices_d2q9(float *nb_border_f1, float *nb_border_f5, float *nb_border_f8,
                              float *nb_border_f3, float *nb_border_f6, float *nb_border_f7,
                              float *border_f1, float *border_f5, float *border_f8,
                              float *border_f3, float *border_f6, float *border_f7,
                              int height, cudaStream_t &s) {
    float *dst[6] = {nb_border_f1, nb_border_f5, nb_border_f8, nb_border_f3, nb_border_f6,
                     nb_border_f7};
    float *src[6] = {border_f1, border_f5, border_f8, border_f3, border_f6, border_f7};
    for (int j = 0; j < 6; j++) {
        cudaError_t e = cudaMemcpyAsync(dst[j], src[j], sizeof(float) * height,
                                        cudaMemcpyDefault, s);
        if (e != cudaSuccess) { set_err("copy_border_devices_d2q9", e); return; }
    }
}

void lb_copy_border_devices_d3q19(float *const dst[10], float *const src[10], int height,
                                  int depth, cudaStream_t s) {
    for (int j = 0; j < 10; j++) {
        cudaError_t e = cudaMemcpyAsync(dst[j], src[j], sizeof(float) * height * depth,
                                        cudaMemcpyDefault, s);
        if (e != cudaSuccess) { set_err("copy_border_devices_d3q19", e); return; }
    }
}

}  // extern "C"

// reference src/copy_border.cu:49-81, C++ linkage as in the reference
void copy_border_devices_d3q19(float *nb_border_f1, float *nb_border_f7, float *nb_border_f8,
                               float *nb_border_f9, float *nb_border_f10, float *nb_border_f2,
                               float *nb_border_f11, float *nb_border_f12,
                               float *nb_border_f13, float *nb_border_f14, float *border_f1,
                               float *border_f7, float *border_f8, float *border_f9,
                               float *border_f10, float *border_f2, float *border_f11,
                               float *border_f12, float *border_f13, float *border_f14,
                               int height, int depth, cudaStream_t &s) {
    float *dst[10] = {nb_border_f1, nb_border_f7, nb_border_f8, nb_border_f9, nb_border_f10,
                      nb_border_f2, nb_border_f11, nb_border_f12, nb_border_f13, nb_border_f14};
    float *src[10] = {border_f1, border_f7, border_f8, border_f9, border_f10,
                      border_f2, border_f11, border_f12, border_f13, border_f14};
    lb_copy_border_devices_d3q19(dst, src, height, depth, s);
}
