/*
 * Reference-signature kernel launchers: the C ABI of the reference's
 * point-cloud kernels (ophgen/src/ophPointCloud_GPU.h:220-234), exported by
 * libophpc so that the reference's own host driver (genCghPointCloudGPU,
 * ophgen/src/ophPointCloud_GPU.cpp:179-413, minus cudaWrapper) links against
 * the GB300 kernels unchanged.
 *
 *   cudaPointCloud_RS       replaces ophgen/src/ophPCKernel.cu:893-912
 *   cudaPointCloud_Fresnel  replaces ophgen/src/ophPCKernel.cu:914-933
 *   sum_Kernel              replaces ophgen/src/ophPCKernel.cu:874-891
 *
 * Conventions kept from the reference: the config lives in device memory;
 * the field is accumulated into d_dst (+=), one channel per call, amplitude
 * color[iColor], wavelength lambda; vertices already scaled by nothing
 * (the config's scale and offset_depth are applied here) and already moved
 * by transVW when the viewing window is on, as the reference driver does
 * before upload; work is queued on the legacy default stream.
 *
 * Differences: nBlocks and nThreads are ignored (launch shapes are chosen
 * for sm_103a); the reference's `mode` bits (MODE_FLOAT, MODE_FASTMATH)
 * select nothing (one kernel per method, FP32 with an FP64 phase reduction
 * and FP64 output), while OPHPC_MODE_TENSOR_BF16X3 (0x200) in `mode`
 * selects the tensor-core tile kernels (split-BF16, relL2 ~1e-5 against
 * FP64), with which the call also waits for its kernels to read their
 * timeout word; k is taken as 2*pi/lambda.
 * The launch sizes and the scratch depend on the config, which lives in
 * device memory, so each call first reads the 120-byte config back with a
 * copy on the legacy stream: the call waits for the work queued on that
 * stream before it (in the reference driver's sequence, only the config
 * upload that its own blocking cudaMemcpy has just made,
 * ophgen/src/ophPointCloud_GPU.cpp:249-258) and returns while its own
 * kernels run. These functions return nothing, as the reference's do; a
 * failure is printed to stderr and reported by ophpc_refabi_last_status()
 * on the calling thread.
 */
#ifndef OPHPC_REFABI_H
#define OPHPC_REFABI_H

#include "ophpc.h"

#ifdef __cplusplus
extern "C" {
#endif

/* _CudaPointCloudConfig (ophgen/src/ophPointCloud_GPU.h:96-147), byte for
 * byte: 104 bytes. */
typedef struct ophpc_ref_pc_config {
    int32_t n_points;
    int32_t pad0;
    double scale_X, scale_Y, scale_Z;
    double offset_depth;
    int32_t pn_X, pn_Y;
    int32_t offset_X, offset_Y;
    double pp_X, pp_Y;
    double half_ss_X, half_ss_Y;
    double k;
    double lambda;
} ophpc_ref_pc_config;

/* _CudaPointCloudConfigRS (ophPointCloud_GPU.h:149-183): + det_tx, det_ty. */
typedef struct ophpc_ref_pc_config_rs {
    ophpc_ref_pc_config base;
    double det_tx, det_ty;
} ophpc_ref_pc_config_rs;

/* _CudaPointCloudConfigFresnel (ophPointCloud_GPU.h:185-215): + tx, ty. */
typedef struct ophpc_ref_pc_config_fresnel {
    ophpc_ref_pc_config base;
    double tx, ty;
} ophpc_ref_pc_config_fresnel;

/* The reference declares these with C++ references (const int&, ...),
 * which the ABI passes as pointers; C callers pass the pointers. d_dst is a
 * cuDoubleComplex array of pn_X * pn_Y (two doubles each). */
#ifdef __cplusplus
void sum_Kernel(const int& nBlocks, const int& nThreads, double* dst, double* src, int size);
void cudaPointCloud_RS(const int& nBlocks, const int& nThreads, ophpc_vertex* d_vertex, double* d_dst,
                       const ophpc_ref_pc_config_rs* d_config, const unsigned& iColor, const unsigned& mode);
void cudaPointCloud_Fresnel(const int& nBlocks, const int& nThreads, ophpc_vertex* d_vertex, double* d_dst,
                            const ophpc_ref_pc_config_fresnel* d_config, const unsigned& iColor,
                            const unsigned& mode);
#else
void sum_Kernel(const int* nBlocks, const int* nThreads, double* dst, double* src, int size);
void cudaPointCloud_RS(const int* nBlocks, const int* nThreads, ophpc_vertex* d_vertex, double* d_dst,
                       const ophpc_ref_pc_config_rs* d_config, const unsigned* iColor, const unsigned* mode);
void cudaPointCloud_Fresnel(const int* nBlocks, const int* nThreads, ophpc_vertex* d_vertex, double* d_dst,
                            const ophpc_ref_pc_config_fresnel* d_config, const unsigned* iColor,
                            const unsigned* mode);
#endif

/* Status of the calling thread's last launcher call above. */
ophpc_status ophpc_refabi_last_status(void);

#ifdef __cplusplus
}
#endif

#endif /* OPHPC_REFABI_H */
