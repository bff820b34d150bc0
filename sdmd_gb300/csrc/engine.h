// engine.h -- internal interface between the C ABI (api.cu) and the kernels.
#pragma once
#include <cstddef>
#include <cstdint>
#include <cuda_runtime.h>

namespace sdmd {
struct DSys;
struct DScal;

// exact FP64 path (loop_fp64.cu)
size_t fp64_smem_bytes(int nbcap);
__global__ void sweep_kernel_fp64(const DSys *systems, int full);
__global__ void loop_kernel_fp64(const DSys *systems, int64_t max_events, double t_end_override);
}  // namespace sdmd
