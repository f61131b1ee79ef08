/* stub: error checks of the CUDA samples helpers become no-ops on the host */
#pragma once
#define checkCudaErrors(x) (x)
#define getLastCudaError(m) ((void)0)
static inline int cudaDeviceSynchronize(void) { return 0; }
