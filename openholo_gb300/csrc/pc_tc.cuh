// Tensor-core (tcgen05) Fresnel path: separable complex contraction
// H = Y * diag(a) * X^T over the points.
#pragma once

#include "ophpc.h"
#include "pc_common.cuh"

#include <cuda_runtime.h>
#include <string>

namespace ophpc {

// Building blocks for callers that run a job as point-range steps (the
// serving engine): the factor tables of one chunk of up to `ld` points (a
// multiple of tc_fresnel_chunk_multiple()) and their tensor maps, the
// per-channel amplitude bound, one chunk (table + GEMM into the FP64 sums)
// and the finalisation of a channel's field (H = -i cmax S).
struct TcFresnelPlan {
    int pnX, pnY, ld;
    bool split;                      // split-BF16 (else FP16)
    void* ar[2];                     // table planes [hi, lo]
    void* ai[2];
    void* br[2];
    void* bi[2];
    alignas(64) unsigned char maps[12 * 128];   // encoded tensor maps
};
int tc_fresnel_chunk_multiple();
size_t tc_fresnel_table_bytes(int pnX, int pnY, int ld, bool split);
bool tc_fresnel_plan(TcFresnelPlan* plan, void* table_mem, int pnX, int pnY, int ld, bool split);
void launch_tc_fresnel_cmax(const PointRec* d_recs_ch, int64_t n_points, float* d_cmax, cudaStream_t stream);
cudaError_t launch_tc_fresnel_chunk(const TcFresnelPlan& plan, const PointRec* d_recs_ch, int64_t n_points,
                                    const ChannelGeom& g, int64_t k0, int kc, const float* d_cmax, double* sum_re,
                                    double* sum_im, bool accumulate, int* d_err, cudaStream_t stream);
void launch_tc_fresnel_finalize(const double* sum_re, const double* sum_im, const float* d_cmax, int64_t plane,
                                double2* d_field_ch, cudaStream_t stream);

// Tensor-core Fresnel generate. Synchronises `stream` at the end to read the
// kernels' error word, unless d_err_out is given: then that device word
// receives it (stream-ordered) and nothing waits (graph capture).
ophpc_status tc_generate_fresnel(cudaMemPool_t pool, const ophpc_config* cfg, const ophpc_vertex* d_vertices,
                                 uint64_t n_points, uint32_t mode, double* d_field, cudaStream_t stream,
                                 std::string* err, int* d_err_out = nullptr);

}  // namespace ophpc
