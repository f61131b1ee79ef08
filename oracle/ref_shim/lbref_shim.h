/*
 * lbref_shim.h -- forced-include shim that lets the reference's CUDA kernel
 * sources compile as host C++ for the CPU pin of the oracle (test
 * infrastructure only).  A kernel launch `k<<<g, b>>>(args)` is rewritten by
 * the recipe in oracle/Makefile into `lbref_launch(g, b, k)(args)`, which runs
 * every (block, thread) index serially.  This is sound for the pinned kernels:
 * they use no shared memory, no barriers and no atomics, and each memory word
 * they write is owned by exactly one thread.
 */
#ifndef LBREF_SHIM_H
#define LBREF_SHIM_H
#include <math.h>
#include <stdio.h>
#include <stdlib.h>

#define __global__
#define __device__
#define __host__

struct dim3 {
    unsigned x, y, z;
    dim3(unsigned a = 1, unsigned b = 1, unsigned c = 1) : x(a), y(b), z(c) {}
};
typedef struct lbref_stream *cudaStream_t;
typedef int cudaError_t;

inline dim3 threadIdx, blockIdx, blockDim, gridDim;

template <class K> struct lbref_launcher {
    dim3 g, b;
    K k;
    template <class... A> void operator()(A... args) const {
        gridDim = g;
        blockDim = b;
        for (unsigned bz = 0; bz < g.z; bz++)
            for (unsigned by = 0; by < g.y; by++)
                for (unsigned bx = 0; bx < g.x; bx++)
                    for (unsigned tz = 0; tz < b.z; tz++)
                        for (unsigned ty = 0; ty < b.y; ty++)
                            for (unsigned tx = 0; tx < b.x; tx++) {
                                blockIdx = dim3(bx, by, bz);
                                threadIdx = dim3(tx, ty, tz);
                                k(args...);
                            }
    }
};
template <class K> lbref_launcher<K> lbref_launch(dim3 g, dim3 b, K k) { return lbref_launcher<K>{g, b, k}; }
#endif
