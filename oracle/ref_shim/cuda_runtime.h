/* stub: the shim supplies the few CUDA runtime types the kernels name */
#pragma once
