/*
 * lattibol.h -- per-device lattice state passed to every drop-in entry point.
 *
 * The two structs are the binary interface of the reference's kernels
 * (reference src/lattibol.h:29-97): the host loop fills them with device
 * pointers and passes them by address to collision_*, streaming_*,
 * get_border_*, apply_border_* and read_value_*.  The member order, types and
 * meaning are therefore kept exactly; only the comments are this project's.
 *
 * All arrays are structure-of-arrays over the sub-domain, node index
 * x + y*width (+ z*width*height), except the border arrays, which hold one x
 * face (height, or height*depth, floats; index y + z*height).
 */
#ifndef LATTIBOL_ABI_H
#define LATTIBOL_ABI_H

#include <cuda_runtime.h>
#include <stdbool.h>

typedef struct {
    float *ux, *uy, *rho;           /* moments written by collision_d2q9 (pre-collision) */
    bool *solid, *solid_bound;      /* wall flag; wall node whose 8 neighbours are walls too */
    float *f0, *f1, *f2, *f3, *f4;  /* populations, D2Q9 order (y axis = -row) */
    float *f5, *f6, *f7, *f8;
    float *border_f1, *border_f5, *border_f8;  /* x face outputs of get_border_d2q9 */
    float *border_f3, *border_f6, *border_f7;
    float *nb_border_f1, *nb_border_f5, *nb_border_f8;  /* neighbour faces for apply_border_d2q9 */
    float *nb_border_f3, *nb_border_f6, *nb_border_f7;
    int width, height;
    int deviceCount, dev;           /* slab decomposition along x: Zou-He only on the end slabs */
    float *plotBuffer;              /* per-device plot staging buffer (not used by the kernels) */
    float *valueCur;                /* 4 floats written by read_value_2d */
    cudaStream_t stream;
    float *psi;                     /* Shan-Chen pseudo-potential */
    float *ueq_x, *ueq_y;           /* equilibrium velocity handed to the Shan-Chen pass */
} DataD2Q9;

typedef struct {
    float *ux, *uy, *uz, *rho;
    bool *solid, *solid_bound;
    float *f0, *f1, *f2, *f3, *f4;  /* populations, D3Q19 order */
    float *f5, *f6, *f7, *f8, *f9;
    float *f10, *f11, *f12, *f13, *f14;
    float *f15, *f16, *f17, *f18;
    float *border_f1, *border_f7, *border_f8, *border_f9, *border_f10;
    float *border_f2, *border_f11, *border_f12, *border_f13, *border_f14;
    float *nb_border_f1, *nb_border_f7, *nb_border_f8, *nb_border_f9, *nb_border_f10;
    float *nb_border_f2, *nb_border_f11, *nb_border_f12, *nb_border_f13, *nb_border_f14;
    int width, height, depth;
    int deviceCount, dev;
    float *plotBuffer;
    float *valueCur;
    cudaStream_t stream;
} DataD3Q19;

#endif
