/* gpu_cuda.h - the GB300 CUDA backend of ComputeQL's GPU layer (src/gpu/cuda/gpu_cuda.h in the
 * reference's tree).
 *
 * Part of the reference's unity build: included by src/gpu/gpu_inc.h when GPU_BACKEND_CUDA is set, after
 * gpu.h and gpu_backend.h, so GPU_Backend, String8, U32/U64/B32 and `internal` come from the base layer.
 * gpu_backend_register_all (src/gpu/gpu_dispatch.c:1-7) registers gpu_cuda_get_backend() under "cuda".
 */
#ifndef GPU_CUDA_H
#define GPU_CUDA_H

#include "cqlcuda.h"

internal GPU_Backend* gpu_cuda_get_backend(void);

#endif /* GPU_CUDA_H */
