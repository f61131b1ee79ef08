// lb_d3q19.cuh -- D3Q19 neighbour offsets, block-to-lattice mapping and the
// native pull shared by the D3Q19 kernels (lb_d3q19.cu) and the closure
// kernel (lb_closure.cu).
#pragma once

#include "lb_kernels.cuh"

namespace lb {

// offset from node o to its neighbour o + c for c in {-1, 0, +1}^3, periodic
struct Nbr3 {
    int xm, xp, ym, yp, zm, zp;  // offsets of the -/+ neighbour per axis
    __device__ __forceinline__ Nbr3(int x, int y, int z, int W, int H, int D) {
        const int WH = W * H;
        xm = x == 0 ? W - 1 : -1;
        xp = x == W - 1 ? -(W - 1) : 1;
        ym = y == 0 ? (H - 1) * W : -W;
        yp = y == H - 1 ? -(H - 1) * W : W;
        zm = z == 0 ? (D - 1) * WH : -WH;
        zp = z == D - 1 ? -(D - 1) * WH : WH;
    }
    // offset of o + (cx, cy, cz)
    __device__ __forceinline__ int off(int cx, int cy, int cz) const {
        return (cx > 0 ? xp : (cx < 0 ? xm : 0)) + (cy > 0 ? yp : (cy < 0 ? ym : 0)) +
               (cz > 0 ? zp : (cz < 0 ? zm : 0));
    }
};

// block -> lattice coordinates; a reversed step maps the linearly dispatched
// blocks back to front so that it begins where the previous step ended
struct Coord3 {
    int x, y, z;
    __device__ __forceinline__ Coord3(const D3Args &a) {
        const int bx = a.reverse ? gridDim.x - 1 - blockIdx.x : blockIdx.x;
        x = bx * blockDim.x + threadIdx.x;
        y = a.reverse ? a.H - 1 - (int)blockIdx.y : (int)blockIdx.y;
        z = a.reverse ? a.D - 1 - (int)blockIdx.z : a.z_lo + (int)blockIdx.z * (1 + a.z_skip);
    }
};

// Native pull of the 19 populations of fluid node o (see d3q19_fused_kernel):
// f_k in FP32 storage, the deviation d_k in 16-bit storage.  IDX32: each
// upstream index is summed in 32 bits before the one pointer addition (fewer
// instructions, a few more registers; for the issue-bound closure kernel).
template <typename S, bool IDX32 = false>
__device__ __forceinline__ void pull_native(const D3Args &a, int o, const Nbr3 &n, uint8_t fl,
                                            float (&g)[19]) {
    const S *const *src = (const S *const *)(a.src.f);  // storage arrays behind float*
    if (fl & CELL_NEAR_WALL) {
#pragma unroll
        for (int k = 0; k < 19; k++) {
            const int up = o + n.off(-d3_cx(k), -d3_cy(k), -d3_cz(k));
            const uint8_t fu = k == 0 ? 0 : a.flags[up];
            if (fu & CELL_WALL) {
                const float v = Store<S>::load_dev(src[d3_opp(k)] + o);
                g[k] = (fu & CELL_MOVING) ? v - a.corr[d3_opp(k)] : v;
            } else {
                g[k] = Store<S>::load_dev(src[k] + up);
            }
        }
    } else {
#pragma unroll
        for (int k = 0; k < 19; k++) {
            if (IDX32)
                g[k] = Store<S>::load_dev(src[k] + (o + n.off(-d3_cx(k), -d3_cy(k), -d3_cz(k))));
            else
                g[k] = Store<S>::load_dev(src[k] + o + n.off(-d3_cx(k), -d3_cy(k), -d3_cz(k)));
        }
    }
}

}  // namespace lb
