#include "pc_tc.cuh"

namespace ophpc {

ophpc_status tc_generate_fresnel(cudaMemPool_t, const ophpc_config*, const ophpc_vertex*, uint64_t, uint32_t,
                                 double*, cudaStream_t, std::string* err) {
    if (err) *err = "tensor-core Fresnel is not built yet";
    return OPHPC_ERROR_UNSUPPORTED;
}

}  // namespace ophpc
