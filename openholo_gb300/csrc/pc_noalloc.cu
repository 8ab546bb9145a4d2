// Allocation-free variant of the RS / Fresnel generate call.
//
// ophpc_generate draws its scratch (the per-point records the kernels
// stream through shared memory, and partial sums for small fields) from a
// memory pool. Some callers cannot allocate device memory at all: a host
// application whose device memory is owned by its own allocator under a
// fixed budget, or a real-time loop that must never enter cudaMalloc /
// cudaFree (which can synchronise the whole device). For them this file
// keeps the scratch in one file-scope __device__ array, allocated once when
// the library's module is loaded on a device, and never allocates per call.
//
// The array is shared by every call on a device and keeps the last call's
// contents. The records of a call are written in full by its prep kernel
// before they are read, and the field is overwritten (the point range is
// never split, so there are no partial sums), so nothing has to start at
// zero. Two calls whose GPU work overlaps (different streams, or different
// host threads without ordering) race on the array.
//
// Nothing is cached between calls: every call looks up the array's device
// address and sets the kernels' shared-memory limits on the current device
// (neither allocates). A reset of the device (cudaDeviceReset, or a reset of
// the primary context) unloads the module, and with it the array and those
// attributes; the next call then loads the module again and finds the new
// address, so no stale address is ever handed to a kernel.
#include "ophpc.h"
#include "pc_common.cuh"

#include <cstdint>

#include <cmath>
#include <cstring>

namespace ophpc {
namespace {

constexpr size_t kStaticScratchBytes = (size_t)OPHPC_STATIC_SCRATCH_RECORDS * sizeof(PointRec);
static_assert(kStaticScratchBytes == 32ull * 1024 * 1024, "32 MiB of point records");

// The scratch itself. In host code `g_static_scratch` only names a host-side
// stand-in; kernels must be given the device address from
// cudaGetSymbolAddress (see scratch_on_current_device).
__device__ __align__(256) unsigned char g_static_scratch[kStaticScratchBytes];

// Per-call set-up with the calling thread's device current: the symbol's
// device address (a host-side stand-in must never reach a kernel) and the
// kernels' dynamic shared-memory limits. Both are looked up afresh on every
// call; neither allocates device memory.
cudaError_t scratch_on_current_device(void** out) {
    void* p = nullptr;
    cudaError_t e = cudaGetSymbolAddress(&p, g_static_scratch);
    if (e != cudaSuccess) return e;
    if ((e = rs_set_smem_limit()) != cudaSuccess) return e;
    if ((e = fresnel_set_smem_limit()) != cudaSuccess) return e;
    *out = p;
    return cudaSuccess;
}

bool positive_finite(double v) { return std::isfinite(v) && v > 0.0; }

bool config_ok(const ophpc_config* c) {
    if (!c || c->pixel_number[0] <= 0 || c->pixel_number[1] <= 0) return false;
    if ((int64_t)c->pixel_number[0] * c->pixel_number[1] > (int64_t)1 << 31) return false;
    if ((int64_t)c->pixel_number[1] > (int64_t)65535 * kTileH) return false;
    if (!positive_finite(c->pixel_pitch[0]) || !positive_finite(c->pixel_pitch[1])) return false;
    if (c->n_channels < 1 || c->n_channels > OPHPC_MAX_CHANNELS) return false;
    for (uint32_t i = 0; i < c->n_channels; ++i)
        if (!positive_finite(c->wave_length[i]) || c->wave_length[i] >= 2.0 * c->pixel_pitch[0] ||
            c->wave_length[i] >= 2.0 * c->pixel_pitch[1])
            return false;
    for (int i = 0; i < 3; ++i)
        if (!std::isfinite(c->scale[i])) return false;
    if (!std::isfinite(c->distance) || (c->viewing_window && !std::isfinite(c->field_length))) return false;
    return std::abs(c->offset[0]) <= (1 << 24) && std::abs(c->offset[1]) <= (1 << 24);
}

// Channel geometry with the reference's roundings (the same expressions as
// the pooled entry point: ophgen/src/ophGen.cpp:361-380).
JobGeom geometry(const ophpc_config* c, int64_t n_points) {
    JobGeom jg;
    std::memset(&jg, 0, sizeof(jg));
    jg.n_channels = (int32_t)c->n_channels;
    jg.n_points = n_points;
    for (uint32_t ch = 0; ch < c->n_channels; ++ch) {
        ChannelGeom& g = jg.ch[ch];
        g.pnX = c->pixel_number[0];
        g.pnY = c->pixel_number[1];
        g.offX = c->offset[0];
        g.offY = c->offset[1];
        g.ppX = c->pixel_pitch[0];
        g.ppY = c->pixel_pitch[1];
        const double ssX = g.pnX * g.ppX, ssY = g.pnY * g.ppY;
        g.x0 = -ssX / 2;
        g.y0 = -ssY / 2;
        const double lambda = c->wave_length[ch];
        g.lambda = lambda;
        g.inv_lambda = 1.0 / lambda;
        const double tx = lambda / (2 * g.ppX), ty = lambda / (2 * g.ppY);
        g.detx = tx / std::sqrt(1 - (tx * tx));
        g.dety = ty / std::sqrt(1 - (ty * ty));
    }
    jg.tiles_x = (c->pixel_number[0] + kTileW - 1) / kTileW;
    jg.tiles_y = (c->pixel_number[1] + kTileH - 1) / kTileH;
    jg.ksplit = 1;
    jg.points_per_split = std::max<int64_t>(kChunk, ((n_points + kChunk - 1) / kChunk) * kChunk);
    return jg;
}

// Device (or managed) memory of the current device only: a buffer on another
// GPU would be written through this device's kernels.
bool on_device(const void* p, int dev) {
    cudaPointerAttributes a;
    if (cudaPointerGetAttributes(&a, p) != cudaSuccess) {
        cudaGetLastError();   // our own query's error; nothing was pending on entry
        return false;
    }
    if (a.type == cudaMemoryTypeManaged) return true;
    return a.type == cudaMemoryTypeDevice && a.device == dev;
}

}  // namespace
}  // namespace ophpc

extern "C" ophpc_status ophpc_generate_static_scratch(const ophpc_config* cfg, const ophpc_vertex* d_vertices,
                                                      uint64_t n_points, uint32_t diff_flag, uint32_t mode,
                                                      double* d_field, void* stream) {
    using namespace ophpc;
    // an error already pending on this thread belongs to an earlier call:
    // report it without queueing work, and leave it pending for its owner
    if (cudaPeekAtLastError() != cudaSuccess) return OPHPC_ERROR_CUDA;
    if (!cfg) return OPHPC_ERROR_INVALID_ARGUMENT;
    if (!config_ok(cfg)) return OPHPC_ERROR_CONFIG;
    if (diff_flag != OPHPC_DIFF_RS && diff_flag != OPHPC_DIFF_FRESNEL) return OPHPC_ERROR_INVALID_ARGUMENT;
    if (mode & (OPHPC_MODE_TENSOR_FP16 | OPHPC_MODE_TENSOR_BF16X3)) return OPHPC_ERROR_UNSUPPORTED;
    // the size limit of the static scratch: one 64-byte record per (point, channel)
    if (n_points > (uint64_t)OPHPC_STATIC_SCRATCH_RECORDS / cfg->n_channels) return OPHPC_ERROR_INVALID_ARGUMENT;
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess) return OPHPC_ERROR_CUDA;
    if (!d_field || !on_device(d_field, dev)) return OPHPC_ERROR_INVALID_ARGUMENT;
    if (n_points > 0 && (!d_vertices || !on_device(d_vertices, dev))) return OPHPC_ERROR_INVALID_ARGUMENT;
    // the kernels move the field as 16-byte double2 words and read vertices as doubles
    if (((uintptr_t)d_field & 15) != 0 || ((uintptr_t)d_vertices & 7) != 0) return OPHPC_ERROR_INVALID_ARGUMENT;
    void* scratch = nullptr;
    if (scratch_on_current_device(&scratch) != cudaSuccess) return OPHPC_ERROR_CUDA;
    cudaStream_t s = (cudaStream_t)stream;
    const size_t field_bytes = sizeof(double2) * (size_t)cfg->pixel_number[0] * cfg->pixel_number[1] * cfg->n_channels;
    if (n_points == 0)
        return cudaMemsetAsync(d_field, 0, field_bytes, s) == cudaSuccess ? OPHPC_SUCCESS : OPHPC_ERROR_CUDA;
    const JobGeom jg = geometry(cfg, (int64_t)n_points);
    PointRec* recs = static_cast<PointRec*>(scratch);
    launch_prep(d_vertices, (int64_t)n_points, cfg->scale, cfg->distance, cfg->field_length, cfg->viewing_window,
                (int)diff_flag, jg, recs, s);
    if (diff_flag == OPHPC_DIFF_RS)
        launch_rs(recs, jg, reinterpret_cast<double2*>(d_field), nullptr, s);
    else
        launch_fresnel(recs, jg, reinterpret_cast<double2*>(d_field), nullptr, s);
    return cudaGetLastError() == cudaSuccess ? OPHPC_SUCCESS : OPHPC_ERROR_CUDA;
}
