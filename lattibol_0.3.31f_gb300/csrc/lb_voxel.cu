// lb_voxel.cu -- STL reading and voxelisation of the solids of a 3-D case,
// the stand-in for the reference's Input::loadSolidsSTL (src/input.cpp:118-
// 142), which voxelises with cvmlcpp (not part of the reference tree).
//
// Grid: the geometry is scaled so that its longest bounding-box side spans
// max_dim voxels (the reference's geometry.scaleTo(1.0) with voxel size
// 1/maxDim); each axis gets ceil(extent / voxel) voxels; voxel (i, j, k) has
// its centre at the bounding-box corner + (i + 1/2, j + 1/2, k + 1/2) voxels.
// A voxel is solid when its centre lies inside the closed surface.
//
// Inside test, one GPU thread per (x, y) column: the vertices are snapped to
// a fixed-point grid of 2^-16 voxel; a triangle whose xy projection contains
// the column centre (exact 64-bit edge functions, a consistent tie rule on
// shared edges and vertices) crosses the column at the depth interpolated
// from those edge functions; the voxels of the column whose centres lie above
// an odd number of crossings are solid.
#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

#include "../../include/lbgb300.h"
#include "lb_kernels.cuh"

namespace {

int fail(int code, const char *where, const std::string &what) {
    lb::abi_record_error(where, what.c_str());
    return code;
}

constexpr int VOX_FRAC = 16;           // fixed point: 2^-16 voxel
constexpr int VOX_MAX_CROSS = 128;     // crossings kept per column

// a triangle in fixed-point voxel units, counter-clockwise in xy
struct TriFx {
    int x0, y0, z0, x1, y1, z1, x2, y2, z2;
    int bx0, by0, bx1, by1;  // column range its projection can touch
};

__device__ __forceinline__ long long edge_fn(int ax, int ay, int bx, int by, long long px,
                                             long long py) {
    return (long long)(bx - ax) * (py - ay) - (long long)(by - ay) * (px - ax);
}
// a point on edge a->b belongs to the triangle when the edge points "up", or
// is horizontal and points "left": of two triangles sharing the edge (in
// opposite directions) exactly one claims it
__device__ __forceinline__ bool edge_ok(long long e, int ax, int ay, int bx, int by) {
    if (e != 0) return e > 0;
    const int dx = bx - ax, dy = by - ay;
    return dy > 0 || (dy == 0 && dx < 0);
}

__global__ void voxelize_kernel(const TriFx *tri, long ntri, int W, int H, int D,
                                uint8_t *solids, int *status) {
    const int x = blockIdx.x * blockDim.x + threadIdx.x;
    const int y = blockIdx.y;
    if (x >= W) return;
    const long long px = ((long long)(2 * x + 1)) << (VOX_FRAC - 1);
    const long long py = ((long long)(2 * y + 1)) << (VOX_FRAC - 1);
    double zc[VOX_MAX_CROSS];
    int n = 0;
    bool overflow = false;
    for (long t = 0; t < ntri; t++) {
        const TriFx T = tri[t];
        if (x < T.bx0 || x > T.bx1 || y < T.by0 || y > T.by1) continue;
        const long long e0 = edge_fn(T.x1, T.y1, T.x2, T.y2, px, py);  // opposite vertex 0
        const long long e1 = edge_fn(T.x2, T.y2, T.x0, T.y0, px, py);
        const long long e2 = edge_fn(T.x0, T.y0, T.x1, T.y1, px, py);
        if (!edge_ok(e0, T.x1, T.y1, T.x2, T.y2) || !edge_ok(e1, T.x2, T.y2, T.x0, T.y0) ||
            !edge_ok(e2, T.x0, T.y0, T.x1, T.y1))
            continue;
        const double a = (double)e0 + (double)e1 + (double)e2;
        const double z = ((double)e0 * (double)T.z0 + (double)e1 * (double)T.z1 +
                          (double)e2 * (double)T.z2) / a;
        if (n < VOX_MAX_CROSS) zc[n++] = z;
        else overflow = true;
    }
    if (overflow) atomicOr(status, 1);
    if (n & 1) atomicOr(status, 2);
    // insertion sort of the crossing depths
    for (int i = 1; i < n; i++) {
        const double v = zc[i];
        int j = i - 1;
        while (j >= 0 && zc[j] > v) {
            zc[j + 1] = zc[j];
            j--;
        }
        zc[j + 1] = v;
    }
    int below = 0;
    for (int k = 0; k < D; k++) {
        const double centre = (double)(((long long)(2 * k + 1)) << (VOX_FRAC - 1));
        while (below < n && zc[below] < centre) below++;
        solids[x + (long)W * (y + (long)H * k)] = (uint8_t)(below & 1);
    }
}

// ------------------------------------------------------------------ STL files

bool is_ascii_stl(const std::vector<uint8_t> &b) {
    if (b.size() < 84) return true;
    if (std::memcmp(b.data(), "solid", 5) != 0) return false;
    uint32_t n;
    std::memcpy(&n, &b[80], 4);
    // a binary file whose header happens to start with "solid" has the size
    // its triangle count says
    return (uint64_t)84 + 50ull * n != b.size();
}

bool parse_ascii(const std::vector<uint8_t> &b, std::vector<float> &tri) {
    std::string s(b.begin(), b.end());
    size_t pos = 0;
    std::vector<float> v;
    while ((pos = s.find("vertex", pos)) != std::string::npos) {
        pos += 6;
        float xyz[3];
        const char *p = s.c_str() + pos;
        char *end = nullptr;
        for (int i = 0; i < 3; i++) {
            xyz[i] = (float)std::strtod(p, &end);  // via double, like the host tools
            if (end == p) return false;
            p = end;
        }
        pos = (size_t)(p - s.c_str());
        v.insert(v.end(), xyz, xyz + 3);
    }
    if (v.size() % 9 != 0) return false;
    tri.swap(v);
    return true;
}

int read_stl(const char *path, std::vector<float> &tri, const char *where) {
    FILE *fp = std::fopen(path, "rb");
    if (!fp) return fail(LB_ERR_IO, where, std::string("cannot open ") + path);
    std::vector<uint8_t> b;
    uint8_t buf[65536];
    size_t n;
    while ((n = std::fread(buf, 1, sizeof buf, fp)) > 0) b.insert(b.end(), buf, buf + n);
    std::fclose(fp);
    if (is_ascii_stl(b)) {
        if (!parse_ascii(b, tri)) return fail(LB_ERR_IO, where, std::string(path) + ": bad ASCII STL");
        return LB_OK;
    }
    uint32_t nt;
    std::memcpy(&nt, &b[80], 4);
    tri.resize((size_t)nt * 9);
    for (uint32_t t = 0; t < nt; t++)  // 12 bytes of normal, 3 vertices, 2 attribute bytes
        std::memcpy(&tri[(size_t)t * 9], &b[84 + 50 * (size_t)t + 12], 36);
    return LB_OK;
}

// the voxel grid of a triangle soup (see the file comment)
struct Grid {
    double lo[3], h;
    int dims[3];
};

int grid_of(const float *tri, int64_t ntri, int max_dim, Grid &g, const char *where) {
    if (ntri <= 0 || max_dim < 1 || max_dim > 4096)
        return fail(LB_ERR_ARG, where, "no triangles, or max_dim outside 1..4096");
    double lo[3] = {INFINITY, INFINITY, INFINITY}, hi[3] = {-INFINITY, -INFINITY, -INFINITY};
    for (int64_t i = 0; i < ntri * 3; i++)
        for (int a = 0; a < 3; a++) {
            const double v = tri[i * 3 + a];
            if (!std::isfinite(v)) return fail(LB_ERR_ARG, where, "non-finite vertex");
            lo[a] = std::min(lo[a], v);
            hi[a] = std::max(hi[a], v);
        }
    const double ext = std::max({hi[0] - lo[0], hi[1] - lo[1], hi[2] - lo[2]});
    if (!(ext > 0)) return fail(LB_ERR_ARG, where, "degenerate geometry");
    g.h = ext / max_dim;
    for (int a = 0; a < 3; a++) {
        g.lo[a] = lo[a];
        g.dims[a] = std::max(1, (int)std::ceil((hi[a] - lo[a]) / g.h - 1e-9));
    }
    return LB_OK;
}

}  // namespace

extern "C" {

int lb_stl_read(const char *path, int64_t *ntri, float *tri, size_t capacity) {
    const char *where = "lb_stl_read";
    if (!path || !ntri) return fail(LB_ERR_ARG, where, "null argument");
    std::vector<float> t;
    const int rc = read_stl(path, t, where);
    if (rc != LB_OK) return rc;
    *ntri = (int64_t)(t.size() / 9);
    if (!tri) return LB_OK;
    if (capacity < t.size()) return fail(LB_ERR_ARG, where, "triangle buffer too small");
    std::memcpy(tri, t.data(), t.size() * sizeof(float));
    return LB_OK;
}

int lb_voxelize(const float *tri, int64_t ntri, int max_dim, int dims[3], uint8_t *solids,
                size_t capacity, int *open_columns) {
    const char *where = "lb_voxelize";
    if (!tri || !dims) return fail(LB_ERR_ARG, where, "null argument");
    Grid g;
    int rc = grid_of(tri, ntri, max_dim, g, where);
    if (rc != LB_OK) return rc;
    for (int a = 0; a < 3; a++) dims[a] = g.dims[a];
    if (!solids) return LB_OK;
    const int W = g.dims[0], H = g.dims[1], D = g.dims[2];
    const size_t N = (size_t)W * H * D;
    if (capacity < N) return fail(LB_ERR_ARG, where, "solids buffer too small");
    // snap to the fixed-point voxel grid, orient counter-clockwise in xy, drop
    // triangles whose projection has no area
    std::vector<TriFx> fx;
    fx.reserve((size_t)ntri);
    const double sc = (double)(1 << VOX_FRAC) / g.h;
    for (int64_t t = 0; t < ntri; t++) {
        int q[9];
        for (int v = 0; v < 3; v++)
            for (int a = 0; a < 3; a++)
                q[3 * v + a] = (int)std::llround(((double)tri[t * 9 + 3 * v + a] - g.lo[a]) * sc);
        long long area = (long long)(q[3] - q[0]) * (q[7] - q[1]) -
                         (long long)(q[4] - q[1]) * (q[6] - q[0]);
        if (area == 0) continue;
        if (area < 0)
            for (int a = 0; a < 3; a++) std::swap(q[3 + a], q[6 + a]);
        TriFx T;
        T.x0 = q[0]; T.y0 = q[1]; T.z0 = q[2];
        T.x1 = q[3]; T.y1 = q[4]; T.z1 = q[5];
        T.x2 = q[6]; T.y2 = q[7]; T.z2 = q[8];
        // columns whose centre (i + 1/2) can fall inside [min, max]
        const double inv = 1.0 / (double)(1 << VOX_FRAC);
        const int xmn = std::min({q[0], q[3], q[6]}), xmx = std::max({q[0], q[3], q[6]});
        const int ymn = std::min({q[1], q[4], q[7]}), ymx = std::max({q[1], q[4], q[7]});
        T.bx0 = (int)std::floor(xmn * inv - 0.5) ; T.bx1 = (int)std::ceil(xmx * inv - 0.5);
        T.by0 = (int)std::floor(ymn * inv - 0.5) ; T.by1 = (int)std::ceil(ymx * inv - 0.5);
        fx.push_back(T);
    }
    TriFx *dtri = nullptr;
    uint8_t *dsol = nullptr;
    int *dst = nullptr;
    cudaError_t e = cudaMalloc(&dtri, sizeof(TriFx) * std::max<size_t>(fx.size(), 1));
    if (e == cudaSuccess) e = cudaMalloc(&dsol, N);
    if (e == cudaSuccess) e = cudaMalloc(&dst, sizeof(int));
    if (e == cudaSuccess) e = cudaMemset(dst, 0, sizeof(int));
    if (e == cudaSuccess && !fx.empty())
        e = cudaMemcpy(dtri, fx.data(), sizeof(TriFx) * fx.size(), cudaMemcpyHostToDevice);
    if (e == cudaSuccess) {
        voxelize_kernel<<<dim3((W + 127) / 128, H), 128>>>(dtri, (long)fx.size(), W, H, D, dsol,
                                                           dst);
        e = cudaGetLastError();
    }
    int st = 0;
    if (e == cudaSuccess) e = cudaMemcpy(solids, dsol, N, cudaMemcpyDeviceToHost);
    if (e == cudaSuccess) e = cudaMemcpy(&st, dst, sizeof(int), cudaMemcpyDeviceToHost);
    cudaFree(dtri);
    cudaFree(dsol);
    cudaFree(dst);
    if (e != cudaSuccess) return fail(LB_ERR_CUDA, where, cudaGetErrorString(e));
    if (st & 1) return fail(LB_ERR_ARG, where, "more than 128 surface crossings in a column");
    if (open_columns) *open_columns = (st & 2) ? 1 : 0;
    return LB_OK;
}

int lb_case_load_solids_stl(const char *path, int max_dim, int *width, int *height, int *depth,
                            uint8_t *solids, size_t capacity) {
    const char *where = "lb_case_load_solids_stl";
    if (!path || !width || !height || !depth) return fail(LB_ERR_ARG, where, "null argument");
    std::vector<float> t;
    int rc = read_stl(path, t, where);
    if (rc != LB_OK) return rc;
    int dims[3];
    rc = lb_voxelize(t.data(), (int64_t)(t.size() / 9), max_dim, dims, solids, capacity,
                     nullptr);
    if (rc != LB_OK) return rc;
    *width = dims[0];
    *height = dims[1];
    *depth = dims[2];
    return LB_OK;
}

}  // extern "C"
