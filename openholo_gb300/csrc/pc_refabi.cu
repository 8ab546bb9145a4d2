// Reference-signature launchers (include/ophpc_refabi.h): cudaPointCloud_RS,
// cudaPointCloud_Fresnel and sum_Kernel with the reference's C ABI
// (ophgen/src/ophPointCloud_GPU.h:220-234, ophgen/src/ophPCKernel.cu:874-933),
// running this library's kernels.
//
// Each call reads the device-resident config back (one 120-byte copy on the
// legacy stream, ordered after the caller's upload of it: the call waits for
// the work queued on that stream before it, and no longer), turns it into a
// one-channel ophpc_config and queues prep + RS/Fresnel on the legacy
// default stream with the amplitude taken from color[iColor] and the result
// added into d_dst; it returns while those kernels run. With
// OPHPC_MODE_TENSOR_BF16X3 set in `mode` (the reference's own mode bits
// select nothing) the tensor-core tile kernels run instead, and the call
// waits for them (it reads their timeout word back). One context per device
// is created on first use and kept for the life of the process.
#include "ophpc_refabi.h"
#include "pc_common.cuh"

#include <cuda_runtime.h>

#include <cstddef>
#include <cstdint>
#include <cstdio>
#include <mutex>

struct ophpc_context;

namespace ophpc {
ophpc_status generate_accumulate(ophpc_context* ctx, const ophpc_config* cfg, const ophpc_vertex* d_vertices,
                                 uint64_t n_points, uint32_t diff_flag, int color_offset, double* d_field,
                                 cudaStream_t s, uint32_t mode);
}

// The reference's config structs (ophPointCloud_GPU.h:89-217) as laid out by
// the x86-64 and aarch64 C++ ABIs: base members, then the derived pair.
static_assert(sizeof(ophpc_ref_pc_config) == 104, "CudaPointCloudConfig is 104 bytes");
static_assert(offsetof(ophpc_ref_pc_config, scale_X) == 8, "scale_X");
static_assert(offsetof(ophpc_ref_pc_config, offset_depth) == 32, "offset_depth");
static_assert(offsetof(ophpc_ref_pc_config, pn_X) == 40, "pn_X");
static_assert(offsetof(ophpc_ref_pc_config, offset_Y) == 52, "offset_Y");
static_assert(offsetof(ophpc_ref_pc_config, pp_X) == 56, "pp_X");
static_assert(offsetof(ophpc_ref_pc_config, lambda) == 96, "lambda");
static_assert(sizeof(ophpc_ref_pc_config_rs) == 120 && offsetof(ophpc_ref_pc_config_rs, det_tx) == 104, "RS config");
static_assert(sizeof(ophpc_ref_pc_config_fresnel) == 120 && offsetof(ophpc_ref_pc_config_fresnel, tx) == 104,
              "Fresnel config");

namespace {

thread_local ophpc_status t_last = OPHPC_SUCCESS;

constexpr int kMaxDevices = 64;
std::mutex g_mu;
ophpc_context* g_ctx[kMaxDevices] = {};

ophpc_context* context_for_current_device(ophpc_status* st) {
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= kMaxDevices) {
        cudaGetLastError();
        *st = OPHPC_ERROR_NO_DEVICE;
        return nullptr;
    }
    std::lock_guard<std::mutex> lk(g_mu);
    if (!g_ctx[dev]) {
        *st = ophpc_create(dev, &g_ctx[dev]);
        if (*st != OPHPC_SUCCESS) {
            g_ctx[dev] = nullptr;
            return nullptr;
        }
    }
    *st = OPHPC_SUCCESS;
    return g_ctx[dev];
}

void report(const char* fn, ophpc_status st, ophpc_context* ctx) {
    t_last = st;
    if (st != OPHPC_SUCCESS)
        std::fprintf(stderr, "%s: %s%s%s\n", fn, ophpc_status_string(st), ctx ? ": " : "",
                     ctx ? ophpc_last_error(ctx) : "");
}

void run(const char* fn, uint32_t diff_flag, const ophpc_vertex* d_vertex, double* d_dst, const void* d_config,
         unsigned i_color, unsigned mode) {
    ophpc_status st = OPHPC_SUCCESS;
    ophpc_context* ctx = context_for_current_device(&st);
    if (!ctx) return report(fn, st, nullptr);
    if (!d_config) return report(fn, OPHPC_ERROR_INVALID_ARGUMENT, nullptr);
    ophpc_ref_pc_config c;
    // legacy-stream copy: ordered after the caller's upload of the config
    cudaError_t e = cudaMemcpy(&c, d_config, sizeof(c), cudaMemcpyDeviceToHost);
    if (e != cudaSuccess) {
        cudaGetLastError();
        return report(fn, OPHPC_ERROR_CUDA, nullptr);
    }
    if (c.n_points < 0 || i_color >= OPHPC_MAX_CHANNELS) return report(fn, OPHPC_ERROR_INVALID_ARGUMENT, nullptr);
    ophpc_config cfg = {};
    cfg.pixel_number[0] = c.pn_X;
    cfg.pixel_number[1] = c.pn_Y;
    cfg.offset[0] = c.offset_X;
    cfg.offset[1] = c.offset_Y;
    cfg.pixel_pitch[0] = c.pp_X;
    cfg.pixel_pitch[1] = c.pp_Y;
    cfg.scale[0] = c.scale_X;
    cfg.scale[1] = c.scale_Y;
    cfg.scale[2] = c.scale_Z;
    cfg.distance = c.offset_depth;
    cfg.field_length = 0.0;
    cfg.viewing_window = 0;   // the reference driver applies transVW on the host
    cfg.n_channels = 1;
    cfg.wave_length[0] = c.lambda;
    st = ophpc::generate_accumulate(ctx, &cfg, d_vertex, (uint64_t)c.n_points, diff_flag, (int)i_color, d_dst,
                                    (cudaStream_t)0, mode);
    report(fn, st, ctx);
}

__global__ void sum_kernel(double2* __restrict__ dst, const double2* __restrict__ src, int size) {
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < size; i += gridDim.x * blockDim.x) {
        const double2 a = dst[i], b = src[i];
        dst[i] = make_double2(a.x + b.x, a.y + b.y);
    }
}

}  // namespace

extern "C" {

void sum_Kernel(const int&, const int&, double* dst, double* src, int size) {
    if (size <= 0) {
        t_last = OPHPC_SUCCESS;
        return;
    }
    if (!dst || !src || ((uintptr_t)dst & 15) != 0 || ((uintptr_t)src & 15) != 0)
        return report("sum_Kernel", OPHPC_ERROR_INVALID_ARGUMENT, nullptr);   // cuDoubleComplex is 16-byte aligned
    int dev = 0, sms = 152;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    const int threads = 256;
    const long long want = ((long long)size + threads - 1) / threads;
    const int blocks = (int)(want < (long long)sms * 8 ? want : (long long)sms * 8);
    ophpc::count_launches(1);
    sum_kernel<<<blocks, threads, 0, 0>>>(reinterpret_cast<double2*>(dst), reinterpret_cast<const double2*>(src),
                                          size);
    const cudaError_t e = cudaGetLastError();
    report("sum_Kernel", e == cudaSuccess ? OPHPC_SUCCESS : OPHPC_ERROR_CUDA, nullptr);
}

void cudaPointCloud_RS(const int&, const int&, ophpc_vertex* d_vertex, double* d_dst,
                       const ophpc_ref_pc_config_rs* d_config, const unsigned& iColor, const unsigned& mode) {
    run("cudaPointCloud_RS", OPHPC_DIFF_RS, d_vertex, d_dst, d_config, iColor, mode);
}

void cudaPointCloud_Fresnel(const int&, const int&, ophpc_vertex* d_vertex, double* d_dst,
                            const ophpc_ref_pc_config_fresnel* d_config, const unsigned& iColor,
                            const unsigned& mode) {
    run("cudaPointCloud_Fresnel", OPHPC_DIFF_FRESNEL, d_vertex, d_dst, d_config, iColor, mode);
}

ophpc_status ophpc_refabi_last_status(void) { return t_last; }

}  // extern "C"
