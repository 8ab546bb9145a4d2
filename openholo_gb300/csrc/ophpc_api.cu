// C ABI of libophpc (declared in include/ophpc.h).
//
// Host driver for one GPU: validates the job, builds the per-channel geometry
// exactly as the reference forms it (ophgen/src/ophGen.cpp:361-380,447-462,
// with -ffp-contract=off on the host compiler), sizes the launch, allocates
// stream-ordered scratch from the context's memory pool and launches
// prep -> RS/Fresnel -> (partial sum). Replaces genCghPointCloudGPU
// (ophgen/src/ophPointCloud_GPU.cpp:179-413) and cudaWrapper
// (ophgen/src/cudaWrapper.cpp), which never return an error to the caller.
#include "ophpc.h"

#include "pc_common.cuh"
#include "pc_tc.cuh"
#include "pc_tcrs.cuh"
#include "ophpc_wrp.h"

#include <atomic>
#include <chrono>
#include <cmath>
#include <cstdio>
#include <cstdint>
#include <cstring>
#include <memory>
#include <mutex>
#include <string>

using namespace ophpc;

namespace ophpc {
static std::atomic<uint64_t> g_launches{0};
void count_launches(unsigned n) { g_launches.fetch_add(n, std::memory_order_relaxed); }
uint64_t launches_so_far() { return g_launches.load(std::memory_order_relaxed); }
}  // namespace ophpc

namespace ophpc {
bool wrp_sizes_supported(int pnx, int pny);
ophpc_status wrp_generate_device(cudaMemPool_t pool, const ophpc_wrp_config* cfg, const ophpc_vertex* d_vertices,
                                 uint64_t n_points, double* d_out, int plane_channel, cudaStream_t s,
                                 std::string* err);
ophpc_status fresnel_fft_device(cudaMemPool_t pool, int pnx, int pny, double ppx, double ppy, double lambda,
                                double distance, const double2* src, double2* dst, cudaStream_t s,
                                std::string* err);
bool ssb_sizes_supported(int pnx, int pny);
extern const uint32_t kSsbSidebandFlag;
ophpc_status ssb_encode_device(cudaMemPool_t pool, const double2* d_field, int n_channels, int pnx, int pny,
                               double ppx, double ppy, uint32_t encode_flag, uint32_t passband, double shift_x,
                               double shift_y, double* d_encoded, uint8_t* d_normalized, cudaStream_t s,
                               std::string* err);
}  // namespace ophpc

struct ophpc_context {
    int device = 0;
    int sm_count = 0;
    int rs_bps = 1, fr_bps = 1;
    cudaMemPool_t pool = nullptr;
    cudaStream_t host_stream = nullptr;
    std::mutex mu;
    std::string last_error;
};

namespace {

class DeviceGuard {
public:
    explicit DeviceGuard(int dev) {
        if (cudaGetDevice(&prev_) != cudaSuccess) prev_ = -1;
        if (prev_ != dev) cudaSetDevice(dev);
    }
    ~DeviceGuard() {
        if (prev_ >= 0) cudaSetDevice(prev_);
    }

private:
    int prev_ = -1;
};

ophpc_status fail(ophpc_context* ctx, ophpc_status st, const std::string& msg) {
    if (ctx) ctx->last_error = msg;
    return st;
}

ophpc_status cuda_fail(ophpc_context* ctx, cudaError_t e, const char* where) {
    std::string msg = std::string(where) + ": " + cudaGetErrorName(e) + " (" + cudaGetErrorString(e) + ")";
    if (ctx) ctx->last_error = msg;
    if (e == cudaErrorMemoryAllocation) return OPHPC_ERROR_OUT_OF_MEMORY;
    return OPHPC_ERROR_CUDA;
}

bool finite_pos(double v) { return std::isfinite(v) && v > 0.0; }

ophpc_status check_config(ophpc_context* ctx, const ophpc_config* cfg) {
    if (!cfg) return fail(ctx, OPHPC_ERROR_INVALID_ARGUMENT, "config is NULL");
    if (cfg->pixel_number[0] <= 0 || cfg->pixel_number[1] <= 0)
        return fail(ctx, OPHPC_ERROR_CONFIG, "pixel_number must be positive");
    if ((int64_t)cfg->pixel_number[0] * cfg->pixel_number[1] > (int64_t)1 << 31)
        return fail(ctx, OPHPC_ERROR_CONFIG, "more than 2^31 pixels per channel");
    if ((int64_t)cfg->pixel_number[1] > (int64_t)65535 * kTileH)
        return fail(ctx, OPHPC_ERROR_CONFIG, "pixel_number[1] above 65535 tiles of 32 rows");
    if (!finite_pos(cfg->pixel_pitch[0]) || !finite_pos(cfg->pixel_pitch[1]))
        return fail(ctx, OPHPC_ERROR_CONFIG, "pixel_pitch must be positive and finite");
    if (cfg->n_channels < 1 || cfg->n_channels > OPHPC_MAX_CHANNELS)
        return fail(ctx, OPHPC_ERROR_CONFIG, "n_channels must be 1..3 (Vertex carries 3 colours)");
    for (uint32_t c = 0; c < cfg->n_channels; ++c) {
        if (!finite_pos(cfg->wave_length[c]))
            return fail(ctx, OPHPC_ERROR_CONFIG, "wave_length must be positive and finite");
        // RS window slope tx/sqrt(1-tx^2) needs lambda < 2*pp
        if (cfg->wave_length[c] >= 2.0 * cfg->pixel_pitch[0] || cfg->wave_length[c] >= 2.0 * cfg->pixel_pitch[1])
            return fail(ctx, OPHPC_ERROR_CONFIG, "wave_length must be below twice the pixel pitch");
    }
    for (int i = 0; i < 3; ++i)
        if (!std::isfinite(cfg->scale[i])) return fail(ctx, OPHPC_ERROR_CONFIG, "scale must be finite");
    if (!std::isfinite(cfg->distance)) return fail(ctx, OPHPC_ERROR_CONFIG, "distance must be finite");
    if (cfg->viewing_window && !std::isfinite(cfg->field_length))
        return fail(ctx, OPHPC_ERROR_CONFIG, "field_length must be finite");
    if (std::abs(cfg->offset[0]) > (1 << 24) || std::abs(cfg->offset[1]) > (1 << 24))
        return fail(ctx, OPHPC_ERROR_CONFIG, "offset out of range");
    return OPHPC_SUCCESS;
}

// The WRP generator's configuration (ophgen/src/ophWRP.cpp:137-213 reads
// it; its splat and propagation need no more than finite values, and the
// padded transform sizes factor into 2, 3, 5, 7).
ophpc_status check_wrp_config(ophpc_context* ctx, const ophpc_wrp_config* cfg, bool propagates = true) {
    if (!cfg) return fail(ctx, OPHPC_ERROR_INVALID_ARGUMENT, "config is NULL");
    if (cfg->pixel_number[0] <= 0 || cfg->pixel_number[1] <= 0)
        return fail(ctx, OPHPC_ERROR_CONFIG, "pixel_number must be positive");
    // the padded transform of 2 pnX x 2 pnY: up to 32768 lines each way
    if (cfg->pixel_number[0] > 16384 || cfg->pixel_number[1] > 16384)
        return fail(ctx, OPHPC_ERROR_CONFIG, "pixel_number above 16384");
    if (!finite_pos(cfg->pixel_pitch[0]) || !finite_pos(cfg->pixel_pitch[1]))
        return fail(ctx, OPHPC_ERROR_CONFIG, "pixel_pitch must be positive and finite");
    if (cfg->n_channels < 1 || cfg->n_channels > OPHPC_MAX_CHANNELS)
        return fail(ctx, OPHPC_ERROR_CONFIG, "n_channels must be 1..3 (Vertex carries 3 colours)");
    for (uint32_t c = 0; c < cfg->n_channels; ++c)
        if (!finite_pos(cfg->wave_length[c]))
            return fail(ctx, OPHPC_ERROR_CONFIG, "wave_length must be positive and finite");
    for (int i = 0; i < 3; ++i)
        if (!std::isfinite(cfg->scale[i])) return fail(ctx, OPHPC_ERROR_CONFIG, "scale must be finite");
    if (!std::isfinite(cfg->wrp_location) || !std::isfinite(cfg->propagation_distance))
        return fail(ctx, OPHPC_ERROR_CONFIG, "wrp_location and propagation_distance must be finite");
    if (cfg->random_phase)
        return fail(ctx, OPHPC_ERROR_UNSUPPORTED, "random phase is not supported (the reference's is unseeded)");
    if (propagates && !wrp_sizes_supported(cfg->pixel_number[0], cfg->pixel_number[1]))
        return fail(ctx, OPHPC_ERROR_UNSUPPORTED, "2*pnX and 2*pnY must factor into 2, 3, 5 and 7");
    return OPHPC_SUCCESS;
}

// Per-channel geometry with the reference's roundings.
JobGeom make_geom(const ophpc_config* cfg, int64_t n_points) {
    JobGeom jg;
    std::memset(&jg, 0, sizeof(jg));
    jg.n_channels = (int32_t)cfg->n_channels;
    jg.n_points = n_points;
    for (uint32_t c = 0; c < cfg->n_channels; ++c) {
        ChannelGeom& g = jg.ch[c];
        g.pnX = cfg->pixel_number[0];
        g.pnY = cfg->pixel_number[1];
        g.offX = cfg->offset[0];
        g.offY = cfg->offset[1];
        g.ppX = cfg->pixel_pitch[0];
        g.ppY = cfg->pixel_pitch[1];
        const double ssX = g.pnX * g.ppX;
        const double ssY = g.pnY * g.ppY;
        g.x0 = -ssX / 2;
        g.y0 = -ssY / 2;
        const double lambda = cfg->wave_length[c];
        g.lambda = lambda;
        g.inv_lambda = 1.0 / lambda;
        const double tx = lambda / (2 * g.ppX);
        const double ty = lambda / (2 * g.ppY);
        const double sqrtX = std::sqrt(1 - (tx * tx));
        const double sqrtY = std::sqrt(1 - (ty * ty));
        g.detx = tx / sqrtX;
        g.dety = ty / sqrtY;
    }
    jg.tiles_x = (cfg->pixel_number[0] + kTileW - 1) / kTileW;
    jg.tiles_y = (cfg->pixel_number[1] + kTileH - 1) / kTileH;
    return jg;
}

// Splits the point range across CTAs when the tile count alone leaves the
// GPU's CTA slots badly quantised (small fields).
void choose_split(JobGeom& jg, int slots) {
    const int64_t tiles = (int64_t)jg.tiles_x * jg.tiles_y * jg.n_channels;
    const int64_t chunks = (jg.n_points + kChunk - 1) / kChunk;
    int best_k = 1;
    double best_eff = 0.0;
    const int kmax = (int)std::min<int64_t>(16, std::max<int64_t>(1, chunks));
    for (int k = 1; k <= kmax; ++k) {
        const double waves = (double)(tiles * k) / slots;
        const double eff = waves / std::ceil(waves);
        // each extra split adds one field-sized partial (small cost): demand 3% gain
        if (eff > best_eff + 0.03) {
            best_eff = eff;
            best_k = k;
        }
        if (tiles * k >= 8LL * slots) break;
    }
    jg.ksplit = best_k;
    const int64_t per = (jg.n_points + best_k - 1) / best_k;
    jg.points_per_split = std::max<int64_t>(kChunk, ((per + kChunk - 1) / kChunk) * kChunk);
}

// The kernels read and write the complex field as double2 (16-byte) words and
// the vertices / encoded values as doubles.
bool aligned(const void* p, uintptr_t bytes) { return ((uintptr_t)p & (bytes - 1)) == 0; }

bool is_device_ptr(const void* p) {
    cudaPointerAttributes a;
    if (cudaPointerGetAttributes(&a, p) != cudaSuccess) {
        cudaGetLastError();
        return false;
    }
    return a.type == cudaMemoryTypeDevice || a.type == cudaMemoryTypeManaged;
}

template <typename T>
cudaError_t pool_alloc(ophpc_context* ctx, T** p, size_t bytes, cudaStream_t s) {
    if (bytes == 0) {
        *p = nullptr;
        return cudaSuccess;
    }
    return cudaMallocFromPoolAsync((void**)p, bytes, ctx->pool, s);
}

// Device-side generate shared by the device and host entry points.
// accumulate: add into d_field instead of overwriting it (plain kernels only).
// d_err_out: the tensor-core paths copy their kernels' timeout word there
// instead of waiting for the stream (graph capture).
// Tensor-core generate added into d_field (the reference-signature
// launchers with OPHPC_MODE_TENSOR_BF16X3): point preparation, the
// amplitude bound (and, for RS, the window flag), then the tile kernel over
// the whole point range adding into the field, with the CUDA-core complement
// for RS. The kernels' timeout word is read back, so the call waits for its
// kernels.
ophpc_status tc_generate_accumulate(ophpc_context* ctx, const JobGeom& jg, const ophpc_config* cfg,
                                    const ophpc_vertex* d_vertices, uint64_t n_points, uint32_t diff_flag,
                                    int color_offset, double* d_field, cudaStream_t s) {
    const int64_t n = (int64_t)n_points;
    const int nch = (int)cfg->n_channels, pnx = cfg->pixel_number[0], pny = cfg->pixel_number[1];
    const bool rs = diff_flag == OPHPC_DIFF_RS;
    const size_t tiles = (size_t)nch * ((pnx + kRsTcTile - 1) / kRsTcTile) * ((pny + kRsTcTile - 1) / kRsTcTile);
    const int64_t mask_words = tc_rs_mask_words(n);
    auto al = [](size_t v) { return (v + 255) & ~(size_t)255; };
    const size_t rec_bytes = al(sizeof(PointRec) * (size_t)n * nch);
    const size_t left_bytes = rs ? al(sizeof(int32_t) * tiles) : 0;
    size_t mask_bytes = rs ? al(sizeof(uint32_t) * tiles * (size_t)mask_words) : 0;
    if (mask_bytes > ((size_t)4 << 30)) mask_bytes = 0;   // the complement re-tests eligibility instead
    unsigned char* mem = nullptr;
    cudaError_t e = pool_alloc(ctx, &mem, rec_bytes + left_bytes + mask_bytes + 256, s);
    if (e != cudaSuccess) return cuda_fail(ctx, e, "scratch allocation (tensor-core generate)");
    PointRec* recs = (PointRec*)mem;
    int32_t* left = rs ? (int32_t*)(mem + rec_bytes) : nullptr;
    uint32_t* mask = mask_bytes ? (uint32_t*)(mem + rec_bytes + left_bytes) : nullptr;
    float* amax = (float*)(mem + rec_bytes + left_bytes + mask_bytes);   // [4] words, then the error word
    int* errw = (int*)(amax + 4);
    e = cudaMemsetAsync(amax, 0, 32, s);
    if (e == cudaSuccess) {
        launch_prep(d_vertices, n, cfg->scale, cfg->distance, cfg->field_length, cfg->viewing_window,
                    (int)diff_flag, jg, recs, s, color_offset);
        if (rs) {
            launch_rs_amax(recs, n, nch, pnx, pny, amax, s);
            e = launch_tc_rs_range(jg, recs, 0, n, true, (double2*)d_field, amax, left, mask,
                                   mask ? mask_words : 0, errw, s);
        } else {
            launch_fresnel_amax(recs, n, nch, amax, s);
            e = launch_tc_fresnel_range(jg, recs, 0, n, true, (double2*)d_field, amax, errw, s);
        }
    }
    if (e == cudaSuccess) e = cudaGetLastError();
    int herr = 0;
    if (e == cudaSuccess) e = cudaMemcpyAsync(&herr, errw, sizeof(int), cudaMemcpyDeviceToHost, s);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    cudaFreeAsync(mem, s);
    if (e != cudaSuccess) return cuda_fail(ctx, e, "tensor-core generate");
    if (herr) return fail(ctx, OPHPC_ERROR_TIMEOUT, "tensor-core kernel wait timed out");
    return OPHPC_SUCCESS;
}

ophpc_status generate_device(ophpc_context* ctx, const ophpc_config* cfg, const ophpc_vertex* d_vertices,
                             uint64_t n_points, uint32_t diff_flag, uint32_t mode, double* d_field,
                             cudaStream_t s, int color_offset = 0, bool accumulate = false,
                             int* d_err_out = nullptr) {
    JobGeom jg = make_geom(cfg, (int64_t)n_points);
    jg.accumulate = accumulate ? 1 : 0;
    const int64_t plane = (int64_t)cfg->pixel_number[0] * cfg->pixel_number[1];
    const int64_t field_elems = plane * cfg->n_channels;
    const bool tensor = diff_flag == OPHPC_DIFF_FRESNEL && (mode & (OPHPC_MODE_TENSOR_FP16 | OPHPC_MODE_TENSOR_BF16X3));
    if (n_points == 0) {
        if (accumulate) return OPHPC_SUCCESS;
        cudaError_t e = cudaMemsetAsync(d_field, 0, sizeof(double2) * field_elems, s);
        return e == cudaSuccess ? OPHPC_SUCCESS : cuda_fail(ctx, e, "cudaMemsetAsync(field)");
    }
    if (accumulate && (mode & OPHPC_MODE_TENSOR_BF16X3))
        return tc_generate_accumulate(ctx, jg, cfg, d_vertices, n_points, diff_flag, color_offset, d_field, s);
    if (tensor && !accumulate) {
        // split-BF16: factors generated on chip per 128x128 tile; FP16:
        // factor tables in HBM and a tcgen05 GEMM over them
        if (mode & OPHPC_MODE_TENSOR_BF16X3)
            return tc_generate_fresnel_tiles(ctx->pool, jg, cfg, d_vertices, n_points, d_field, ctx->sm_count, s,
                                             &ctx->last_error, d_err_out);
        return tc_generate_fresnel(ctx->pool, cfg, d_vertices, n_points, mode, d_field, s, &ctx->last_error,
                                   d_err_out);
    }
    if (diff_flag == OPHPC_DIFF_RS && (mode & OPHPC_MODE_TENSOR_BF16X3) && !accumulate && color_offset == 0) {
        return tc_generate_rs(ctx->pool, jg, cfg, d_vertices, n_points, d_field, ctx->sm_count, s, &ctx->last_error,
                              d_err_out);
    }
    const int bps = diff_flag == OPHPC_DIFF_RS ? ctx->rs_bps : ctx->fr_bps;
    choose_split(jg, ctx->sm_count * bps);

    PointRec* d_recs = nullptr;
    double2* d_partials = nullptr;
    cudaError_t e = pool_alloc(ctx, &d_recs, sizeof(PointRec) * n_points * cfg->n_channels, s);
    if (e != cudaSuccess) return cuda_fail(ctx, e, "scratch allocation (point records)");
    e = pool_alloc(ctx, &d_partials, sizeof(double2) * field_elems * (jg.ksplit - 1), s);
    if (e != cudaSuccess) {
        cudaFreeAsync(d_recs, s);
        return cuda_fail(ctx, e, "scratch allocation (partials)");
    }
    launch_prep(d_vertices, (int64_t)n_points, cfg->scale, cfg->distance, cfg->field_length,
                cfg->viewing_window, (int)diff_flag, jg, d_recs, s, color_offset);
    if (diff_flag == OPHPC_DIFF_RS)
        launch_rs(d_recs, jg, (double2*)d_field, d_partials, s);
    else
        launch_fresnel(d_recs, jg, (double2*)d_field, d_partials, s);
    launch_sum_partials(jg, (double2*)d_field, d_partials, s);
    e = cudaGetLastError();
    cudaFreeAsync(d_recs, s);
    if (d_partials) cudaFreeAsync(d_partials, s);
    if (e != cudaSuccess) return cuda_fail(ctx, e, "kernel launch");
    return OPHPC_SUCCESS;
}

ophpc_status check_job(ophpc_context* ctx, const ophpc_config* cfg, uint64_t n_points, uint32_t diff_flag,
                       uint32_t mode) {
    if (!ctx) return OPHPC_ERROR_INVALID_ARGUMENT;
    ophpc_status st = check_config(ctx, cfg);
    if (st != OPHPC_SUCCESS) return st;
    if (diff_flag != OPHPC_DIFF_RS && diff_flag != OPHPC_DIFF_FRESNEL)
        return fail(ctx, OPHPC_ERROR_INVALID_ARGUMENT, "diff_flag must be PC_DIFF_RS (0) or PC_DIFF_FRESNEL (1)");
    if ((mode & OPHPC_MODE_TENSOR_FP16) && (mode & OPHPC_MODE_TENSOR_BF16X3))
        return fail(ctx, OPHPC_ERROR_INVALID_ARGUMENT, "choose one tensor mode");
    if (n_points > (uint64_t)INT32_MAX) return fail(ctx, OPHPC_ERROR_INVALID_ARGUMENT, "n_points above 2^31-1");
    return OPHPC_SUCCESS;
}

}  // namespace

namespace ophpc {

// For the reference-signature launchers (pc_refabi.cu): one channel, the
// amplitude from color[color_offset], added into d_field; the plain kernels,
// or with OPHPC_MODE_TENSOR_BF16X3 in `mode` the tensor-core tile kernels
// (other mode bits select nothing).
ophpc_status generate_accumulate(ophpc_context* ctx, const ophpc_config* cfg, const ophpc_vertex* d_vertices,
                                 uint64_t n_points, uint32_t diff_flag, int color_offset, double* d_field,
                                 cudaStream_t s, uint32_t mode) {
    if (!ctx) return OPHPC_ERROR_INVALID_ARGUMENT;
    std::lock_guard<std::mutex> lk(ctx->mu);
    ctx->last_error.clear();
    mode &= OPHPC_MODE_TENSOR_BF16X3;
    ophpc_status st = check_job(ctx, cfg, n_points, diff_flag, mode);
    if (st != OPHPC_SUCCESS) return st;
    if (color_offset < 0 || color_offset + (int)cfg->n_channels > OPHPC_MAX_CHANNELS)
        return fail(ctx, OPHPC_ERROR_INVALID_ARGUMENT, "colour index must be 0..2");
    DeviceGuard guard(ctx->device);
    if (!d_field || !is_device_ptr(d_field)) return fail(ctx, OPHPC_ERROR_INVALID_ARGUMENT, "d_dst must be device memory");
    if (n_points > 0 && (!d_vertices || !is_device_ptr(d_vertices)))
        return fail(ctx, OPHPC_ERROR_INVALID_ARGUMENT, "vertices must be device memory");
    if (!aligned(d_field, 16) || !aligned(d_vertices, 8))
        return fail(ctx, OPHPC_ERROR_INVALID_ARGUMENT, "d_dst must be 16-byte and vertices 8-byte aligned");
    return generate_device(ctx, cfg, d_vertices, n_points, diff_flag, mode, d_field, s, color_offset, true);
}

}  // namespace ophpc

namespace {

// ophpc_encode after validation (also captured into plans).
ophpc_status encode_device(ophpc_context* ctx, const double* d_field, uint32_t n_channels, uint64_t n_pixels,
                           uint32_t encode_flag, double* d_encoded, uint8_t* d_normalized, cudaStream_t s) {
    unsigned long long* d_mm = nullptr;
    cudaError_t e = pool_alloc(ctx, &d_mm, 8 * sizeof(unsigned long long), s);
    if (e != cudaSuccess) return cuda_fail(ctx, e, "scratch allocation (min/max)");
    double* d_tmp = nullptr;
    if (encode_flag >= OPHPC_ENCODE_SIMPLENI && !d_encoded) {
        const size_t bytes = sizeof(double) * (size_t)n_channels * (size_t)n_pixels;
        e = pool_alloc(ctx, &d_tmp, bytes, s);
        if (e == cudaSuccess) e = cudaMemsetAsync(d_tmp, 0, bytes, s);
        if (e != cudaSuccess) {
            if (d_tmp) cudaFreeAsync(d_tmp, s);
            cudaFreeAsync(d_mm, s);
            return cuda_fail(ctx, e, "scratch allocation (encoded)");
        }
    }
    launch_encode((const double2*)d_field, (int)n_channels, (int64_t)n_pixels, (int)encode_flag,
                  d_tmp ? d_tmp : d_encoded, d_normalized, d_mm, s);
    e = cudaGetLastError();
    if (d_tmp) cudaFreeAsync(d_tmp, s);
    cudaFreeAsync(d_mm, s);
    if (e != cudaSuccess) return cuda_fail(ctx, e, "encode launch");
    return OPHPC_SUCCESS;
}

}  // namespace

extern "C" {

int32_t ophpc_api_version(void) { return OPHPC_API_VERSION; }

uint64_t ophpc_kernel_launches(void) { return launches_so_far(); }

const char* ophpc_status_string(ophpc_status st) {
    switch (st) {
        case OPHPC_SUCCESS: return "success";
        case OPHPC_ERROR_INVALID_ARGUMENT: return "invalid argument";
        case OPHPC_ERROR_CUDA: return "CUDA error";
        case OPHPC_ERROR_OUT_OF_MEMORY: return "out of device memory";
        case OPHPC_ERROR_IO: return "I/O error";
        case OPHPC_ERROR_CONFIG: return "invalid configuration";
        case OPHPC_ERROR_UNSUPPORTED: return "unsupported";
        case OPHPC_ERROR_QUEUE_FULL: return "queue full";
        case OPHPC_ERROR_TIMEOUT: return "timeout";
        case OPHPC_ERROR_NOT_READY: return "not ready";
        case OPHPC_ERROR_NO_DEVICE: return "no CUDA device";
    }
    return "unknown status";
}

const char* ophpc_last_error(const ophpc_context* ctx) { return ctx ? ctx->last_error.c_str() : ""; }

ophpc_status ophpc_create(int32_t device, ophpc_context** out) {
    if (!out) return OPHPC_ERROR_INVALID_ARGUMENT;
    *out = nullptr;
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) {
        cudaGetLastError();
        return OPHPC_ERROR_NO_DEVICE;
    }
    if (device < 0 || device >= ndev) return OPHPC_ERROR_INVALID_ARGUMENT;
    auto* ctx = new (std::nothrow) ophpc_context();
    if (!ctx) return OPHPC_ERROR_OUT_OF_MEMORY;
    ctx->device = device;
    DeviceGuard guard(device);
    cudaDeviceProp prop;
    cudaError_t e = cudaGetDeviceProperties(&prop, device);
    if (e != cudaSuccess) {
        delete ctx;
        return OPHPC_ERROR_CUDA;
    }
    if (prop.major < 10) {
        delete ctx;
        return OPHPC_ERROR_UNSUPPORTED;   // kernels are built for sm_103a only
    }
    ctx->sm_count = prop.multiProcessorCount;
    ctx->rs_bps = rs_blocks_per_sm();
    ctx->fr_bps = fresnel_blocks_per_sm();
    cudaMemPoolProps pp;
    std::memset(&pp, 0, sizeof(pp));
    pp.allocType = cudaMemAllocationTypePinned;
    pp.handleTypes = cudaMemHandleTypeNone;
    pp.location.type = cudaMemLocationTypeDevice;
    pp.location.id = device;
    e = cudaMemPoolCreate(&ctx->pool, &pp);
    if (e == cudaSuccess) {
        uint64_t keep = UINT64_MAX;   // keep freed scratch cached between calls
        cudaMemPoolSetAttribute(ctx->pool, cudaMemPoolAttrReleaseThreshold, &keep);
        e = cudaStreamCreateWithFlags(&ctx->host_stream, cudaStreamNonBlocking);
    }
    if (e != cudaSuccess) {
        if (ctx->pool) cudaMemPoolDestroy(ctx->pool);
        delete ctx;
        return e == cudaErrorMemoryAllocation ? OPHPC_ERROR_OUT_OF_MEMORY : OPHPC_ERROR_CUDA;
    }
    *out = ctx;
    return OPHPC_SUCCESS;
}

ophpc_status ophpc_destroy(ophpc_context* ctx) {
    if (!ctx) return OPHPC_ERROR_INVALID_ARGUMENT;
    {
        std::lock_guard<std::mutex> lk(ctx->mu);
        DeviceGuard guard(ctx->device);
        if (ctx->host_stream) {
            cudaStreamSynchronize(ctx->host_stream);
            cudaStreamDestroy(ctx->host_stream);
        }
        if (ctx->pool) {
            cudaDeviceSynchronize();
            cudaMemPoolDestroy(ctx->pool);
        }
    }
    delete ctx;
    return OPHPC_SUCCESS;
}

ophpc_status ophpc_generate(ophpc_context* ctx, const ophpc_config* cfg, const ophpc_vertex* d_vertices,
                            uint64_t n_points, uint32_t diff_flag, uint32_t mode, double* d_field,
                            void* stream) {
    if (!ctx) return OPHPC_ERROR_INVALID_ARGUMENT;
    std::lock_guard<std::mutex> lk(ctx->mu);
    ctx->last_error.clear();
    ophpc_status st = check_job(ctx, cfg, n_points, diff_flag, mode);
    if (st != OPHPC_SUCCESS) return st;
    DeviceGuard guard(ctx->device);
    if (!d_field || !is_device_ptr(d_field))
        return fail(ctx, OPHPC_ERROR_INVALID_ARGUMENT, "d_field must be device memory");
    if (n_points > 0 && (!d_vertices || !is_device_ptr(d_vertices)))
        return fail(ctx, OPHPC_ERROR_INVALID_ARGUMENT, "d_vertices must be device memory");
    if (!aligned(d_field, 16) || !aligned(d_vertices, 8))
        return fail(ctx, OPHPC_ERROR_INVALID_ARGUMENT, "d_field must be 16-byte and d_vertices 8-byte aligned");
    return generate_device(ctx, cfg, d_vertices, n_points, diff_flag, mode, d_field, (cudaStream_t)stream);
}

ophpc_status ophpc_generate_host(ophpc_context* ctx, const ophpc_config* cfg, const ophpc_vertex* h_vertices,
                                 uint64_t n_points, uint32_t diff_flag, uint32_t mode,
                                 double* const* h_field_per_channel, double* seconds_out) {
    if (!ctx) return OPHPC_ERROR_INVALID_ARGUMENT;
    auto t0 = std::chrono::steady_clock::now();
    std::lock_guard<std::mutex> lk(ctx->mu);
    ctx->last_error.clear();
    ophpc_status st = check_job(ctx, cfg, n_points, diff_flag, mode);
    if (st != OPHPC_SUCCESS) return st;
    if (!h_field_per_channel) return fail(ctx, OPHPC_ERROR_INVALID_ARGUMENT, "field buffers are NULL");
    for (uint32_t c = 0; c < cfg->n_channels; ++c)
        if (!h_field_per_channel[c]) return fail(ctx, OPHPC_ERROR_INVALID_ARGUMENT, "field buffer is NULL");
    if (n_points > 0 && !h_vertices) return fail(ctx, OPHPC_ERROR_INVALID_ARGUMENT, "vertices are NULL");
    DeviceGuard guard(ctx->device);
    cudaStream_t s = ctx->host_stream;
    const int64_t plane = (int64_t)cfg->pixel_number[0] * cfg->pixel_number[1];
    ophpc_vertex* d_v = nullptr;
    double* d_f = nullptr;
    cudaError_t e = pool_alloc(ctx, &d_v, sizeof(ophpc_vertex) * n_points, s);
    if (e == cudaSuccess) e = pool_alloc(ctx, &d_f, sizeof(double2) * plane * cfg->n_channels, s);
    if (e != cudaSuccess) {
        if (d_v) cudaFreeAsync(d_v, s);
        cudaStreamSynchronize(s);
        return cuda_fail(ctx, e, "scratch allocation (host path)");
    }
    if (n_points) e = cudaMemcpyAsync(d_v, h_vertices, sizeof(ophpc_vertex) * n_points, cudaMemcpyHostToDevice, s);
    if (e == cudaSuccess) {
        st = generate_device(ctx, cfg, d_v, n_points, diff_flag, mode, d_f, s);
    } else {
        st = cuda_fail(ctx, e, "cudaMemcpyAsync(vertices)");
    }
    if (st == OPHPC_SUCCESS) {
        for (uint32_t c = 0; c < cfg->n_channels && e == cudaSuccess; ++c)
            e = cudaMemcpyAsync(h_field_per_channel[c], d_f + 2 * plane * c, sizeof(double2) * plane,
                                cudaMemcpyDeviceToHost, s);
        if (e != cudaSuccess) st = cuda_fail(ctx, e, "cudaMemcpyAsync(field)");
    }
    cudaFreeAsync(d_v, s);
    cudaFreeAsync(d_f, s);
    e = cudaStreamSynchronize(s);
    if (e != cudaSuccess && st == OPHPC_SUCCESS) st = cuda_fail(ctx, e, "generate (host path)");
    if (seconds_out)
        *seconds_out = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
    return st;
}

ophpc_status ophpc_wrp_generate(ophpc_context* ctx, const ophpc_wrp_config* cfg, const ophpc_vertex* d_vertices,
                                uint64_t n_points, double* d_field, void* stream) {
    if (!ctx) return OPHPC_ERROR_INVALID_ARGUMENT;
    std::lock_guard<std::mutex> lk(ctx->mu);
    ctx->last_error.clear();
    ophpc_status st = check_wrp_config(ctx, cfg);
    if (st != OPHPC_SUCCESS) return st;
    if (n_points > (uint64_t)INT32_MAX) return fail(ctx, OPHPC_ERROR_INVALID_ARGUMENT, "n_points above 2^31-1");
    DeviceGuard guard(ctx->device);
    if (!d_field || !is_device_ptr(d_field))
        return fail(ctx, OPHPC_ERROR_INVALID_ARGUMENT, "d_field must be device memory");
    if (n_points > 0 && (!d_vertices || !is_device_ptr(d_vertices)))
        return fail(ctx, OPHPC_ERROR_INVALID_ARGUMENT, "d_vertices must be device memory");
    if (!aligned(d_field, 16) || !aligned(d_vertices, 8))
        return fail(ctx, OPHPC_ERROR_INVALID_ARGUMENT, "d_field must be 16-byte and d_vertices 8-byte aligned");
    return wrp_generate_device(ctx->pool, cfg, d_vertices, n_points, d_field, -1, (cudaStream_t)stream,
                               &ctx->last_error);
}

ophpc_status ophpc_wrp_plane(ophpc_context* ctx, const ophpc_wrp_config* cfg, const ophpc_vertex* d_vertices,
                             uint64_t n_points, uint32_t channel, double* d_plane, void* stream) {
    if (!ctx) return OPHPC_ERROR_INVALID_ARGUMENT;
    std::lock_guard<std::mutex> lk(ctx->mu);
    ctx->last_error.clear();
    ophpc_status st = check_wrp_config(ctx, cfg, false);
    if (st != OPHPC_SUCCESS) return st;
    if (channel >= cfg->n_channels) return fail(ctx, OPHPC_ERROR_INVALID_ARGUMENT, "channel out of range");
    if (n_points > (uint64_t)INT32_MAX) return fail(ctx, OPHPC_ERROR_INVALID_ARGUMENT, "n_points above 2^31-1");
    DeviceGuard guard(ctx->device);
    if (!d_plane || !is_device_ptr(d_plane))
        return fail(ctx, OPHPC_ERROR_INVALID_ARGUMENT, "d_plane must be device memory");
    if (n_points > 0 && (!d_vertices || !is_device_ptr(d_vertices)))
        return fail(ctx, OPHPC_ERROR_INVALID_ARGUMENT, "d_vertices must be device memory");
    if (!aligned(d_plane, 16) || !aligned(d_vertices, 8))
        return fail(ctx, OPHPC_ERROR_INVALID_ARGUMENT, "d_plane must be 16-byte and d_vertices 8-byte aligned");
    return wrp_generate_device(ctx->pool, cfg, d_vertices, n_points, d_plane, (int)channel, (cudaStream_t)stream,
                               &ctx->last_error);
}

ophpc_status ophpc_wrp_generate_host(ophpc_context* ctx, const ophpc_wrp_config* cfg,
                                     const ophpc_vertex* h_vertices, uint64_t n_points,
                                     double* const* h_field_per_channel, double* seconds_out) {
    if (!ctx) return OPHPC_ERROR_INVALID_ARGUMENT;
    auto t0 = std::chrono::steady_clock::now();
    std::lock_guard<std::mutex> lk(ctx->mu);
    ctx->last_error.clear();
    ophpc_status st = check_wrp_config(ctx, cfg);
    if (st != OPHPC_SUCCESS) return st;
    if (n_points > (uint64_t)INT32_MAX) return fail(ctx, OPHPC_ERROR_INVALID_ARGUMENT, "n_points above 2^31-1");
    if (!h_field_per_channel) return fail(ctx, OPHPC_ERROR_INVALID_ARGUMENT, "field buffers are NULL");
    for (uint32_t c = 0; c < cfg->n_channels; ++c)
        if (!h_field_per_channel[c]) return fail(ctx, OPHPC_ERROR_INVALID_ARGUMENT, "field buffer is NULL");
    if (n_points > 0 && !h_vertices) return fail(ctx, OPHPC_ERROR_INVALID_ARGUMENT, "vertices are NULL");
    DeviceGuard guard(ctx->device);
    cudaStream_t s = ctx->host_stream;
    const int64_t plane = (int64_t)cfg->pixel_number[0] * cfg->pixel_number[1];
    ophpc_vertex* d_v = nullptr;
    double* d_f = nullptr;
    cudaError_t e = pool_alloc(ctx, &d_v, sizeof(ophpc_vertex) * n_points, s);
    if (e == cudaSuccess) e = pool_alloc(ctx, &d_f, sizeof(double2) * plane * cfg->n_channels, s);
    if (e != cudaSuccess) {
        if (d_v) cudaFreeAsync(d_v, s);
        cudaStreamSynchronize(s);
        return cuda_fail(ctx, e, "scratch allocation (WRP host path)");
    }
    if (n_points) e = cudaMemcpyAsync(d_v, h_vertices, sizeof(ophpc_vertex) * n_points, cudaMemcpyHostToDevice, s);
    if (e == cudaSuccess)
        st = wrp_generate_device(ctx->pool, cfg, d_v, n_points, d_f, -1, s, &ctx->last_error);
    else
        st = cuda_fail(ctx, e, "cudaMemcpyAsync(vertices)");
    if (st == OPHPC_SUCCESS) {
        for (uint32_t c = 0; c < cfg->n_channels && e == cudaSuccess; ++c)
            e = cudaMemcpyAsync(h_field_per_channel[c], d_f + 2 * plane * c, sizeof(double2) * plane,
                                cudaMemcpyDeviceToHost, s);
        if (e != cudaSuccess) st = cuda_fail(ctx, e, "cudaMemcpyAsync(field)");
    }
    cudaFreeAsync(d_v, s);
    cudaFreeAsync(d_f, s);
    e = cudaStreamSynchronize(s);
    if (e != cudaSuccess && st == OPHPC_SUCCESS) st = cuda_fail(ctx, e, "WRP generate (host path)");
    if (seconds_out) *seconds_out = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
    return st;
}

ophpc_status ophpc_fresnel_fft(ophpc_context* ctx, int32_t pnx, int32_t pny, double ppx, double ppy, double lambda,
                               double distance, const double* d_src, double* d_dst, void* stream) {
    if (!ctx) return OPHPC_ERROR_INVALID_ARGUMENT;
    std::lock_guard<std::mutex> lk(ctx->mu);
    ctx->last_error.clear();
    if (pnx <= 0 || pny <= 0 || pnx > 16384 || pny > 16384)
        return fail(ctx, OPHPC_ERROR_CONFIG, "pixel numbers must be 1..16384");
    if (!finite_pos(ppx) || !finite_pos(ppy) || !finite_pos(lambda) || !std::isfinite(distance))
        return fail(ctx, OPHPC_ERROR_CONFIG, "pitch, wavelength and distance must be finite (positive)");
    if (!wrp_sizes_supported(pnx, pny))
        return fail(ctx, OPHPC_ERROR_UNSUPPORTED, "2*pnX and 2*pnY must factor into 2, 3, 5 and 7");
    DeviceGuard guard(ctx->device);
    if (!d_src || !d_dst || !is_device_ptr(d_src) || !is_device_ptr(d_dst))
        return fail(ctx, OPHPC_ERROR_INVALID_ARGUMENT, "d_src and d_dst must be device memory");
    if (!aligned(d_src, 16) || !aligned(d_dst, 16))
        return fail(ctx, OPHPC_ERROR_INVALID_ARGUMENT, "d_src and d_dst must be 16-byte aligned");
    return fresnel_fft_device(ctx->pool, pnx, pny, ppx, ppy, lambda, distance, (const double2*)d_src, (double2*)d_dst,
                              (cudaStream_t)stream, &ctx->last_error);
}

ophpc_status ophpc_encode(ophpc_context* ctx, const double* d_field, uint32_t n_channels, uint64_t n_pixels,
                          uint32_t encode_flag, double* d_encoded, uint8_t* d_normalized, void* stream) {
    if (!ctx) return OPHPC_ERROR_INVALID_ARGUMENT;
    std::lock_guard<std::mutex> lk(ctx->mu);
    ctx->last_error.clear();
    if (encode_flag > OPHPC_ENCODE_TWOPHASE)
        return fail(ctx, OPHPC_ERROR_UNSUPPORTED,
                    "encode_flag: phase, amplitude, real, imaginary, SimpleNI, Burckhardt or TwoPhase only");
    if (n_channels < 1 || n_channels > OPHPC_MAX_CHANNELS)
        return fail(ctx, OPHPC_ERROR_INVALID_ARGUMENT, "n_channels must be 1..3");
    if (n_pixels == 0) return OPHPC_SUCCESS;
    DeviceGuard guard(ctx->device);
    if (!d_field || !is_device_ptr(d_field)) return fail(ctx, OPHPC_ERROR_INVALID_ARGUMENT, "d_field must be device memory");
    if (d_encoded && !is_device_ptr(d_encoded))
        return fail(ctx, OPHPC_ERROR_INVALID_ARGUMENT, "d_encoded must be device memory");
    if (d_normalized && !is_device_ptr(d_normalized))
        return fail(ctx, OPHPC_ERROR_INVALID_ARGUMENT, "d_normalized must be device memory");
    if (!aligned(d_field, 16) || !aligned(d_encoded, 8))
        return fail(ctx, OPHPC_ERROR_INVALID_ARGUMENT, "d_field must be 16-byte and d_encoded 8-byte aligned");
    return encode_device(ctx, d_field, n_channels, n_pixels, encode_flag, d_encoded, d_normalized,
                         (cudaStream_t)stream);
}

ophpc_status ophpc_encode_ssb(ophpc_context* ctx, const double* d_field, uint32_t n_channels, int32_t pnx,
                              int32_t pny, double ppx, double ppy, uint32_t encode_flag, uint32_t passband,
                              double shift_x, double shift_y, double* d_encoded, uint8_t* d_normalized,
                              void* stream) {
    if (!ctx) return OPHPC_ERROR_INVALID_ARGUMENT;
    std::lock_guard<std::mutex> lk(ctx->mu);
    ctx->last_error.clear();
    if (encode_flag != OPHPC_ENCODE_SSB && encode_flag != OPHPC_ENCODE_OFFSSB)
        return fail(ctx, OPHPC_ERROR_UNSUPPORTED, "encode_flag: OPHPC_ENCODE_SSB or OPHPC_ENCODE_OFFSSB");
    if (encode_flag == OPHPC_ENCODE_OFFSSB && passband > OPHPC_SSB_BOTTOM)
        return fail(ctx, OPHPC_ERROR_INVALID_ARGUMENT, "passband: OPHPC_SSB_LEFT, _RIGHT, _TOP or _BOTTOM");
    if (n_channels < 1 || n_channels > OPHPC_MAX_CHANNELS)
        return fail(ctx, OPHPC_ERROR_INVALID_ARGUMENT, "n_channels must be 1..3");
    if (pnx <= 0 || pny <= 0 || pnx > 16384 || pny > 16384)
        return fail(ctx, OPHPC_ERROR_CONFIG, "pixel numbers must be 1..16384");
    if (!finite_pos(ppx) || !finite_pos(ppy) || !std::isfinite(shift_x) || !std::isfinite(shift_y))
        return fail(ctx, OPHPC_ERROR_CONFIG, "pitches must be finite and positive, shifts finite");
    if (!ssb_sizes_supported(pnx, pny))
        return fail(ctx, OPHPC_ERROR_UNSUPPORTED, "pnX and pnY must factor into 2, 3, 5 and 7");
    DeviceGuard guard(ctx->device);
    if (!d_field || !is_device_ptr(d_field)) return fail(ctx, OPHPC_ERROR_INVALID_ARGUMENT, "d_field must be device memory");
    if (d_encoded && !is_device_ptr(d_encoded))
        return fail(ctx, OPHPC_ERROR_INVALID_ARGUMENT, "d_encoded must be device memory");
    if (d_normalized && !is_device_ptr(d_normalized))
        return fail(ctx, OPHPC_ERROR_INVALID_ARGUMENT, "d_normalized must be device memory");
    if (!aligned(d_field, 16) || !aligned(d_encoded, 8))
        return fail(ctx, OPHPC_ERROR_INVALID_ARGUMENT, "d_field must be 16-byte and d_encoded 8-byte aligned");
    return ssb_encode_device(ctx->pool, (const double2*)d_field, (int)n_channels, pnx, pny, ppx, ppy, encode_flag,
                             passband, shift_x, shift_y, d_encoded, d_normalized, (cudaStream_t)stream,
                             &ctx->last_error);
}

ophpc_status ophpc_encode_sideband(ophpc_context* ctx, const double* d_field, uint32_t n_channels, int32_t pnx,
                                   int32_t pny, double ppx, double ppy, uint32_t passband, double* d_encoded,
                                   uint8_t* d_normalized, void* stream) {
    if (!ctx) return OPHPC_ERROR_INVALID_ARGUMENT;
    std::lock_guard<std::mutex> lk(ctx->mu);
    ctx->last_error.clear();
    if (passband > OPHPC_SSB_BOTTOM)
        return fail(ctx, OPHPC_ERROR_INVALID_ARGUMENT, "passband: OPHPC_SSB_LEFT, _RIGHT, _TOP or _BOTTOM");
    if (n_channels < 1 || n_channels > OPHPC_MAX_CHANNELS)
        return fail(ctx, OPHPC_ERROR_INVALID_ARGUMENT, "n_channels must be 1..3");
    if (pnx <= 0 || pny <= 0 || pnx > 16384 || pny > 16384)
        return fail(ctx, OPHPC_ERROR_CONFIG, "pixel numbers must be 1..16384");
    if (!finite_pos(ppx) || !finite_pos(ppy)) return fail(ctx, OPHPC_ERROR_CONFIG, "pitches must be finite and positive");
    if (!ssb_sizes_supported(pnx, pny))
        return fail(ctx, OPHPC_ERROR_UNSUPPORTED, "pnX and pnY must factor into 2, 3, 5 and 7");
    DeviceGuard guard(ctx->device);
    if (!d_field || !is_device_ptr(d_field)) return fail(ctx, OPHPC_ERROR_INVALID_ARGUMENT, "d_field must be device memory");
    if (d_encoded && !is_device_ptr(d_encoded))
        return fail(ctx, OPHPC_ERROR_INVALID_ARGUMENT, "d_encoded must be device memory");
    if (d_normalized && !is_device_ptr(d_normalized))
        return fail(ctx, OPHPC_ERROR_INVALID_ARGUMENT, "d_normalized must be device memory");
    if (!aligned(d_field, 16) || !aligned(d_encoded, 8))
        return fail(ctx, OPHPC_ERROR_INVALID_ARGUMENT, "d_field must be 16-byte and d_encoded 8-byte aligned");
    return ssb_encode_device(ctx->pool, (const double2*)d_field, (int)n_channels, pnx, pny, ppx, ppy,
                             kSsbSidebandFlag, passband, 0.0, 0.0, d_encoded, d_normalized, (cudaStream_t)stream,
                             &ctx->last_error);
}

ophpc_status ophpc_normalize(ophpc_context* ctx, const double* d_encoded, uint32_t n_channels, uint64_t n_pixels,
                             uint8_t* d_normalized, void* stream) {
    if (!ctx) return OPHPC_ERROR_INVALID_ARGUMENT;
    std::lock_guard<std::mutex> lk(ctx->mu);
    ctx->last_error.clear();
    if (n_channels < 1 || n_channels > OPHPC_MAX_CHANNELS)
        return fail(ctx, OPHPC_ERROR_INVALID_ARGUMENT, "n_channels must be 1..3");
    if (n_pixels == 0) return OPHPC_SUCCESS;
    DeviceGuard guard(ctx->device);
    if (!d_encoded || !is_device_ptr(d_encoded))
        return fail(ctx, OPHPC_ERROR_INVALID_ARGUMENT, "d_encoded must be device memory");
    if (!d_normalized || !is_device_ptr(d_normalized))
        return fail(ctx, OPHPC_ERROR_INVALID_ARGUMENT, "d_normalized must be device memory");
    if (!aligned(d_encoded, 8)) return fail(ctx, OPHPC_ERROR_INVALID_ARGUMENT, "d_encoded must be 8-byte aligned");
    cudaStream_t s = (cudaStream_t)stream;
    unsigned long long* d_mm = nullptr;
    cudaError_t e = pool_alloc(ctx, &d_mm, 2 * sizeof(unsigned long long), s);
    if (e != cudaSuccess) return cuda_fail(ctx, e, "scratch allocation (min/max)");
    launch_normalize(d_encoded, (int)n_channels, (int64_t)n_pixels, d_normalized, d_mm, s);
    e = cudaGetLastError();
    cudaFreeAsync(d_mm, s);
    if (e != cudaSuccess) return cuda_fail(ctx, e, "normalize launch");
    return OPHPC_SUCCESS;
}

// ---- plans: one generate (+ encode) captured into a CUDA graph ---------------

struct ophpc_plan {
    ophpc_context* ctx = nullptr;
    int device = 0;
    cudaGraph_t graph = nullptr;
    cudaGraphExec_t exec = nullptr;
    int* d_err = nullptr;   // the tensor-core kernels' timeout word of the last replay
};

ophpc_status ophpc_plan_create(ophpc_context* ctx, const ophpc_config* cfg, const ophpc_vertex* d_vertices,
                               uint64_t n_points, uint32_t diff_flag, uint32_t mode, double* d_field,
                               uint32_t encode_flag, double* d_encoded, uint8_t* d_normalized, ophpc_plan** out) {
    if (!ctx || !out) return OPHPC_ERROR_INVALID_ARGUMENT;
    *out = nullptr;
    std::lock_guard<std::mutex> lk(ctx->mu);
    ctx->last_error.clear();
    ophpc_status st = check_job(ctx, cfg, n_points, diff_flag, mode);
    if (st != OPHPC_SUCCESS) return st;
    DeviceGuard guard(ctx->device);
    if (!d_field || !is_device_ptr(d_field))
        return fail(ctx, OPHPC_ERROR_INVALID_ARGUMENT, "d_field must be device memory");
    if (n_points > 0 && (!d_vertices || !is_device_ptr(d_vertices)))
        return fail(ctx, OPHPC_ERROR_INVALID_ARGUMENT, "d_vertices must be device memory");
    if (!aligned(d_field, 16) || !aligned(d_vertices, 8))
        return fail(ctx, OPHPC_ERROR_INVALID_ARGUMENT, "d_field must be 16-byte and d_vertices 8-byte aligned");
    const bool enc = encode_flag != OPHPC_PLAN_NO_ENCODE;
    const uint64_t n_pixels = (uint64_t)cfg->pixel_number[0] * cfg->pixel_number[1];
    if (enc) {
        if (encode_flag > OPHPC_ENCODE_TWOPHASE)
            return fail(ctx, OPHPC_ERROR_UNSUPPORTED,
                        "encode_flag: phase, amplitude, real, imaginary, SimpleNI, Burckhardt or TwoPhase only");
        if ((d_encoded && !is_device_ptr(d_encoded)) || (d_normalized && !is_device_ptr(d_normalized)))
            return fail(ctx, OPHPC_ERROR_INVALID_ARGUMENT, "d_encoded and d_normalized must be device memory");
        if (!aligned(d_encoded, 8)) return fail(ctx, OPHPC_ERROR_INVALID_ARGUMENT, "d_encoded must be 8-byte aligned");
    }
    std::unique_ptr<ophpc_plan> plan(new ophpc_plan());
    plan->ctx = ctx;
    plan->device = ctx->device;
    cudaError_t e = cudaMalloc((void**)&plan->d_err, sizeof(int));
    if (e != cudaSuccess) return cuda_fail(ctx, e, "cudaMalloc(plan error word)");
    auto release = [&]() {
        if (plan->exec) cudaGraphExecDestroy(plan->exec);
        if (plan->graph) cudaGraphDestroy(plan->graph);
        cudaFree(plan->d_err);
    };
    cudaStream_t cs = nullptr;
    e = cudaStreamCreateWithFlags(&cs, cudaStreamNonBlocking);
    if (e != cudaSuccess) {
        release();
        return cuda_fail(ctx, e, "cudaStreamCreate(capture)");
    }
    e = cudaStreamBeginCapture(cs, cudaStreamCaptureModeThreadLocal);
    if (e == cudaSuccess) {
        e = cudaMemsetAsync(plan->d_err, 0, sizeof(int), cs);
        if (e == cudaSuccess)
            st = generate_device(ctx, cfg, d_vertices, n_points, diff_flag, mode, d_field, cs, 0, false, plan->d_err);
        if (e == cudaSuccess && st == OPHPC_SUCCESS && enc && n_pixels > 0)
            st = encode_device(ctx, d_field, cfg->n_channels, n_pixels, encode_flag, d_encoded, d_normalized, cs);
        // end the capture whatever happened, so that the stream is usable
        const cudaError_t ee = cudaStreamEndCapture(cs, &plan->graph);
        if (e == cudaSuccess) e = ee;
    }
    cudaStreamDestroy(cs);
    if (st != OPHPC_SUCCESS) {
        release();
        return st;
    }
    if (e == cudaSuccess) e = cudaGraphInstantiate(&plan->exec, plan->graph, 0);
    if (e != cudaSuccess) {
        cudaGetLastError();
        release();
        return cuda_fail(ctx, e, "graph capture");
    }
    *out = plan.release();
    return OPHPC_SUCCESS;
}

ophpc_status ophpc_plan_launch(ophpc_plan* plan, void* stream) {
    if (!plan) return OPHPC_ERROR_INVALID_ARGUMENT;
    DeviceGuard guard(plan->device);
    const cudaError_t e = cudaGraphLaunch(plan->exec, (cudaStream_t)stream);
    if (e != cudaSuccess) {
        std::lock_guard<std::mutex> lk(plan->ctx->mu);
        return cuda_fail(plan->ctx, e, "cudaGraphLaunch");
    }
    return OPHPC_SUCCESS;
}

ophpc_status ophpc_plan_wait(ophpc_plan* plan, void* stream) {
    if (!plan) return OPHPC_ERROR_INVALID_ARGUMENT;
    DeviceGuard guard(plan->device);
    int herr = 0;
    cudaError_t e = cudaStreamSynchronize((cudaStream_t)stream);
    if (e == cudaSuccess) e = cudaMemcpy(&herr, plan->d_err, sizeof(int), cudaMemcpyDeviceToHost);
    std::lock_guard<std::mutex> lk(plan->ctx->mu);
    if (e != cudaSuccess) return cuda_fail(plan->ctx, e, "plan wait");
    if (herr) return fail(plan->ctx, OPHPC_ERROR_TIMEOUT, "tensor-core kernel wait timed out");
    return OPHPC_SUCCESS;
}

ophpc_status ophpc_plan_destroy(ophpc_plan* plan) {
    if (!plan) return OPHPC_ERROR_INVALID_ARGUMENT;
    DeviceGuard guard(plan->device);
    cudaGraphExecDestroy(plan->exec);
    cudaGraphDestroy(plan->graph);
    cudaFree(plan->d_err);
    delete plan;
    return OPHPC_SUCCESS;
}

}  // extern "C"



