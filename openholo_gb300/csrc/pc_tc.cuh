// Tensor-core (tcgen05) Fresnel path: separable complex contraction
// H = Y * diag(a) * X^T over the points.
#pragma once

#include "ophpc.h"

#include <cuda_runtime.h>
#include <string>

namespace ophpc {

ophpc_status tc_generate_fresnel(cudaMemPool_t pool, const ophpc_config* cfg, const ophpc_vertex* d_vertices,
                                 uint64_t n_points, uint32_t mode, double* d_field, cudaStream_t stream,
                                 std::string* err);

}  // namespace ophpc
