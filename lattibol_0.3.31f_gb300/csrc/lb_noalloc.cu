// lb_noalloc.cu -- lb_reduce_d3q19_noalloc: the conservation sums of
// lb_reduce_d3q19 without any device allocation, for callers that cannot
// allocate device memory.  Examples: a host that hands all of the GPU's memory
// to its own pool allocator when it starts, and a real-time loop (the
// reference runs its steps from a GUI timer) where cudaMalloc / cudaFree may
// synchronise the whole device.
//
// The scratch space (one FP64 partial per first-pass block plus the 7
// results) lives in a file-scope __device__ array of a fixed size instead of
// memory from cudaMalloc.  Every GPU that loads this library holds that array
// (128 KiB) until the process exits.
//
// In host code, the name g_reduce_scratch is a host-side stand-in for the
// array, not a device address: a kernel given it would fault or, where the GPU
// can reach host memory, silently use the wrong memory.  The device address is
// obtained once per device with cudaGetSymbolAddress, with that device current,
// on the first call made on that device.  Every call blocks the calling thread:
// it ends with a synchronous copy of the 7 results into the caller's host
// array, so no call may be made while a stream capture is in progress.
//
// All calls share the one array and each call leaves its partials in it.
// Nothing needs clearing between calls: every first-pass block overwrites its
// own partial slot, and the second pass reads only the slots of the current
// call.  Calls that overlap on the GPU (from several host threads or streams)
// race on the array and must not be issued.
#include <mutex>
#include <unordered_map>

#include "../../include/lbgb300.h"
#include "lb_kernels.cuh"

namespace {

constexpr int kScratchDoubles = 16384;                           // 128 KiB per device
constexpr long kNodesPerBlock = 65536;                           // first-pass block covers 64 Ki nodes
constexpr long kMaxBlocks = (kScratchDoubles - 8) / 7;           // 7 partials per block + 7 results
constexpr long kMaxNodes = kMaxBlocks * kNodesPerBlock;          // 153 288 704 nodes
// the largest lattice puts its 7 results in the array's last slots
static_assert(7 * kMaxBlocks + 7 <= kScratchDoubles, "scratch holds every partial and result");
static_assert(kMaxNodes == 153288704L, "the limit the error message and the header state");

static __device__ __align__(256) double g_reduce_scratch[kScratchDoubles];

std::mutex g_mu;
std::unordered_map<int, double *> g_scratch_addr;  // device ordinal -> device address

}  // namespace

extern "C" int lb_reduce_d3q19_noalloc(const DataD3Q19 *d, double out[7]) {
    if (!d || !out || d->width <= 0 || d->height <= 0 || d->depth <= 0) {
        lb::abi_record_error("lb_reduce_d3q19_noalloc", "null data or non-positive extent");
        return LB_ERR_ARG;
    }
    const long n = (long)d->width * d->height * d->depth;
    if (n > kMaxNodes) {
        lb::abi_record_error("lb_reduce_d3q19_noalloc",
                             "lattice has more than 153288704 nodes, the most its fixed "
                             "128 KiB scratch array supports; use lb_reduce_d3q19");
        return LB_ERR_ARG;
    }
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) {
        lb::abi_record_error("lb_reduce_d3q19_noalloc", cudaGetErrorString(e));
        return LB_ERR_CUDA;
    }
    double *scratch = nullptr;
    {
        std::lock_guard<std::mutex> l(g_mu);
        auto it = g_scratch_addr.find(dev);
        if (it == g_scratch_addr.end()) {
            e = cudaGetSymbolAddress((void **)&scratch, g_reduce_scratch);
            if (e != cudaSuccess || !scratch) {
                lb::abi_record_error("lb_reduce_d3q19_noalloc: cudaGetSymbolAddress",
                                     cudaGetErrorString(e));
                return LB_ERR_CUDA;
            }
            g_scratch_addr[dev] = scratch;
        } else {
            scratch = it->second;
        }
    }
    const int nblocks = (int)((n + kNodesPerBlock - 1) / kNodesPerBlock);
    double *result = scratch + 7L * nblocks;
    e = lb::launch_reduce_blocks(d->rho, d->ux, d->uy, d->uz,
                                 reinterpret_cast<const uint8_t *>(d->solid), 0xff, n, nblocks,
                                 scratch, result, 0);
    if (e == cudaSuccess) e = cudaMemcpy(out, result, 7 * sizeof(double), cudaMemcpyDeviceToHost);
    if (e != cudaSuccess) {
        lb::abi_record_error("lb_reduce_d3q19_noalloc", cudaGetErrorString(e));
        return LB_ERR_CUDA;
    }
    return LB_OK;
}
