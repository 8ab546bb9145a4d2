/*
 * ophpc — GB300-native point-cloud hologram generation (C ABI).
 *
 * Drop-in for Openholo's point-cloud path:
 *   ophPointCloud::generateHologram(PC_DIFF_RS | PC_DIFF_FRESNEL)
 *     (ophgen/src/ophPointCloud.cpp:151-191 -> genCghPointCloudGPU,
 *      ophgen/src/ophPointCloud_GPU.cpp:179-413)
 *   ophGen::encoding(ENCODE_PHASE | ENCODE_AMPLITUDE) + ophGen::normalize()
 *     (ophgen/src/ophGen.cpp:816-849, 654-687)
 *
 * Conventions (all entry points):
 *   - every call returns an ophpc_status and never exits the process
 *     (the reference's HANDLE_ERROR calls exit(): ophPointCloud_GPU.h:71-81);
 *   - plain pointers and sizes only; `stream` is a cudaStream_t passed as
 *     void* (NULL = the legacy default stream);
 *   - device-pointer entry points are asynchronous on `stream`; host-pointer
 *     entry points are synchronous;
 *   - a context may be used from several host threads; calls on one context
 *     are serialised by its lock. Device work of calls on different streams
 *     may overlap: each call allocates its own stream-ordered scratch.
 *   - one GPU per context, chosen at creation.
 */
#ifndef OPHPC_H
#define OPHPC_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define OPHPC_API_VERSION 1
#define OPHPC_MAX_CHANNELS 3

typedef enum ophpc_status {
    OPHPC_SUCCESS = 0,
    OPHPC_ERROR_INVALID_ARGUMENT = 1,
    OPHPC_ERROR_CUDA = 2,
    OPHPC_ERROR_OUT_OF_MEMORY = 3,
    OPHPC_ERROR_IO = 4,
    OPHPC_ERROR_CONFIG = 5,
    OPHPC_ERROR_UNSUPPORTED = 6,
    OPHPC_ERROR_QUEUE_FULL = 7,
    OPHPC_ERROR_TIMEOUT = 8,
    OPHPC_ERROR_NOT_READY = 9,
    OPHPC_ERROR_NO_DEVICE = 10
} ophpc_status;

/* PC_DIFF_FLAG values (ophgen/src/ophPointCloud.h:550-553). */
#define OPHPC_DIFF_RS 0u
#define OPHPC_DIFF_FRESNEL 1u

/* Mode bits, bit-compatible with Openholo/src/define.h:155-159. */
#define OPHPC_MODE_CPU 0u
#define OPHPC_MODE_GPU 1u
#define OPHPC_MODE_DOUBLE 0u
#define OPHPC_MODE_FLOAT 2u
#define OPHPC_MODE_FASTMATH 4u
/* GB300 additions (no reference counterpart): Fresnel as a separable complex
 * contraction on the tcgen05 tensor cores, FP16 operands or split-BF16
 * (hi/lo, three products), FP32 accumulation. With PC_DIFF_RS,
 * OPHPC_MODE_TENSOR_BF16X3 runs RS on the tensor cores too: per 128x128
 * pixel tile a row-factor x column-factor expansion plus a first-order
 * cross pair, split-BF16 (cross pair FP16), with the pairs the expansion
 * does not hold for added by the FP32-core RS kernel; OPHPC_MODE_TENSOR_FP16
 * is ignored for RS. */
#define OPHPC_MODE_TENSOR_FP16 0x100u
#define OPHPC_MODE_TENSOR_BF16X3 0x200u

/* ophGen::ENCODE_FLAG values (ophgen/src/ophGen.h:84-95) handled on device. */
#define OPHPC_ENCODE_PHASE 0u
#define OPHPC_ENCODE_AMPLITUDE 1u
#define OPHPC_ENCODE_REAL 2u
#define OPHPC_ENCODE_IMAGINARY 3u
#define OPHPC_ENCODE_SIMPLENI 4u
#define OPHPC_ENCODE_BURCKHARDT 5u
#define OPHPC_ENCODE_TWOPHASE 6u
#define OPHPC_ENCODE_SSB 7u
#define OPHPC_ENCODE_OFFSSB 8u

/* ophGen::SSB_PASSBAND (ophgen/src/ophGen.h:295): the half of the spectrum
 * ENCODE_OFFSSB keeps. */
#define OPHPC_SSB_LEFT 0u
#define OPHPC_SSB_RIGHT 1u
#define OPHPC_SSB_TOP 2u
#define OPHPC_SSB_BOTTOM 3u

/* Vertex (Openholo/src/struct.h:86-106): packed pos[3], color[3], phase —
 * 56 bytes, colour channels in [0, 1]; color[ch] is channel ch's amplitude. */
typedef struct ophpc_vertex {
    double pos[3];
    double color[3];
    double phase;
} ophpc_vertex;

/* The OphConfig (Openholo/src/Openholo.h:96-120) and OphPointCloudConfig
 * (ophgen/src/ophGen.h:546-567) fields the path reads. */
typedef struct ophpc_config {
    int32_t pixel_number[2];   /* SLM_PixelNumX/Y */
    int32_t offset[2];         /* context_.offset (setOffset) */
    double pixel_pitch[2];     /* SLM_PixelPitchX/Y, metres */
    double scale[3];           /* ScaleX/Y/Z */
    double distance;           /* Distance, metres, added to scaled z */
    double field_length;       /* FieldLength, used when viewing_window != 0 */
    int32_t viewing_window;    /* setViewingWindow(true): transVW before scaling */
    uint32_t n_channels;       /* SLM_WaveNum, 1..OPHPC_MAX_CHANNELS */
    double wave_length[OPHPC_MAX_CHANNELS]; /* SLM_WaveLength_i, metres */
} ophpc_config;

typedef struct ophpc_context ophpc_context;

/* Version of this header's ABI. */
int32_t ophpc_api_version(void);

/* Number of CUDA kernels this library has launched since it was loaded
 * (instrumentation; no reference counterpart). */
uint64_t ophpc_kernel_launches(void);

/* Human-readable text of a status code (static storage). */
const char* ophpc_status_string(ophpc_status status);

/* Detail of the last failure on this context (valid until the next call). */
const char* ophpc_last_error(const ophpc_context* ctx);

/* Creates a context on CUDA device `device`. Replaces cudaWrapper's
 * singleton device query (ophgen/src/cudaWrapper.cpp:50-177), which divides
 * by zero on sm_10x. */
ophpc_status ophpc_create(int32_t device, ophpc_context** out);
ophpc_status ophpc_destroy(ophpc_context* ctx);

/* Device buffers passed to this library: complex fields (d_field,
 * [re, im] pairs) must be 16-byte aligned and vertex and encoded buffers
 * 8-byte aligned, as cudaMalloc and PyTorch allocations are; a buffer that
 * is not is rejected with OPHPC_ERROR_INVALID_ARGUMENT before any work is
 * queued. */

/* Device path of generateHologram: d_vertices holds n_points ophpc_vertex
 * records in device memory; d_field receives the complex field of every
 * channel as interleaved doubles [n_channels][pnY][pnX][re, im] (the
 * layout of complex_H, Openholo/src/Openholo.h:490), overwritten. mode takes
 * the OPHPC_MODE_* bits; the kernels always run on the GPU. Asynchronous on
 * `stream`. Replaces genCghPointCloudGPU's single-GPU branch
 * (ophgen/src/ophPointCloud_GPU.cpp:218-286) and the launchers
 * cudaPointCloud_RS / cudaPointCloud_Fresnel (ophgen/src/ophPCKernel.cu:893-933). */
ophpc_status ophpc_generate(ophpc_context* ctx, const ophpc_config* cfg,
                            const ophpc_vertex* d_vertices, uint64_t n_points,
                            uint32_t diff_flag, uint32_t mode, double* d_field, void* stream);

/* Host path, what genCghPointCloudGPU does end to end: host vertices in,
 * one host buffer of pnX*pnY Complex<double> per channel out (complex_H[ch]).
 * Synchronous. seconds_out (optional) receives the elapsed wall time, as
 * generateHologram returns it (ophgen/src/ophPointCloud.cpp:187-190). */
ophpc_status ophpc_generate_host(ophpc_context* ctx, const ophpc_config* cfg,
                                 const ophpc_vertex* h_vertices, uint64_t n_points,
                                 uint32_t diff_flag, uint32_t mode,
                                 double* const* h_field_per_channel, double* seconds_out);

/* Device encoding + normalisation (ophGen::encoding + ophGen::normalize):
 * d_field: [n_channels][n_pixels][re, im] doubles. d_encoded (optional,
 * NULL to skip): [n_channels][n_pixels] doubles = m_lpEncoded.
 * d_normalized (optional): [n_channels][n_pixels] bytes = m_lpNormalized,
 * using the min/max over all channels. encode_flag: PHASE, AMPLITUDE, REAL,
 * IMAGINARY, SIMPLENI, BURCKHARDT or TWOPHASE (ophGen.cpp:1821-1974);
 * the last three work per channel on the field divided by its largest
 * sampled magnitude. BURCKHARDT writes two of every three entries and
 * TWOPHASE the first 2*(n_pixels/2): the others keep what d_encoded held
 * (as m_lpEncoded keeps an earlier encoding in the reference), or count as
 * 0 when d_encoded is NULL. SSB and off-axis SSB need the 2-D size:
 * ophpc_encode_ssb; the binary encoders are OPHPC_ERROR_UNSUPPORTED.
 * Precision: FP64 throughout; the phase value takes a table-driven atan2
 * (within 4 eps of the reference's (atan2 + pi) / (2 pi) on a correctly
 * rounded atan2) and the codes follow the reference's rounding bit for bit
 * given the values. Asynchronous on `stream`. */
ophpc_status ophpc_encode(ophpc_context* ctx, const double* d_field, uint32_t n_channels,
                          uint64_t n_pixels, uint32_t encode_flag, double* d_encoded,
                          uint8_t* d_normalized, void* stream);

/* ophPointCloud::encoding(ENCODE_SSB | ENCODE_OFFSSB, passband)
 * (ophgen/src/ophPointCloud.cpp:247-251) on device, FP64, on the field
 * d_field [n_channels][pny][pnx][re, im]:
 *   OPHPC_ENCODE_SSB: ophPointCloud::encodeHologram
 *     (ophPointCloud.cpp:191-240) per channel: the field through the
 *     reference's shifted forward and backward FFTs (unnormalised), its real
 *     part times cos(pi x shift_x / ppx + pi y shift_y / ppy) at the pixel
 *     coordinates the reference uses; shift_x, shift_y are its
 *     spectrum_shift (default 0.0, 0.5); passband is not used (nor is it
 *     there);
 *   OPHPC_ENCODE_OFFSSB: ophGen::encoding(ENCODE_OFFSSB, passband)
 *     (ophgen/src/ophGen.cpp:882-921): freqShift(0, 100) then
 *     singleSideBand(passband) of channel 0's field, normalised to [0, 1],
 *     written to every channel (the reference reads complex_H[0] for each).
 * d_encoded (optional) receives m_lpEncoded, d_normalized (optional) the
 * 8-bit codes of ophGen::normalize over all channels. pnx, pny up to 16384,
 * each factoring into 2, 3, 5 and 7 (OPHPC_ERROR_UNSUPPORTED otherwise).
 * This is what the reference's code describes; its own runs alias the FFT
 * input with the array being shifted and are not reproducible. Allocates
 * scratch from the context's pool; asynchronous on `stream`. */
ophpc_status ophpc_encode_ssb(ophpc_context* ctx, const double* d_field, uint32_t n_channels, int32_t pnx,
                              int32_t pny, double ppx, double ppy, uint32_t encode_flag, uint32_t passband,
                              double shift_x, double shift_y, double* d_encoded, uint8_t* d_normalized,
                              void* stream);

/* ophGen::encodeSideBand(passband) (ophgen/src/ophGen.cpp:1607-1695, with
 * getShiftPhaseValue :1741-1781) on device, FP64: per channel the field
 * cropped to the central half along the passband's axis, the reference's
 * shifted inverse FFT normalised by pnX pnY, times the passband's carrier,
 * real part, into d_encoded (m_lpEncoded; optional), and ophGen::normalize's
 * codes into d_normalized (optional). passband: OPHPC_SSB_*. The reference
 * keeps this method protected (ophDepthMap and ophIFTA call it); it is
 * exposed here for callers of the device buffers. Same size limits as
 * ophpc_encode_ssb; asynchronous on `stream`. */
ophpc_status ophpc_encode_sideband(ophpc_context* ctx, const double* d_field, uint32_t n_channels, int32_t pnx,
                                   int32_t pny, double ppx, double ppy, uint32_t passband, double* d_encoded,
                                   uint8_t* d_normalized, void* stream);

/* Largest n_points * n_channels that ophpc_generate_static_scratch accepts:
 * its scratch is a fixed 32 MiB device array of 64-byte point records. */
#define OPHPC_STATIC_SCRATCH_RECORDS 524288u

/* Allocation-free generate; this entry point has no counterpart in the
 * reference. For callers that cannot allocate device memory — a host
 * application that owns all device memory through its own allocator under a
 * fixed budget, or a real-time loop that must never enter cudaMalloc /
 * cudaFree, which can synchronise the whole device. Same arguments and
 * result as ophpc_generate (plain RS and Fresnel kernels; tensor modes return
 * OPHPC_ERROR_UNSUPPORTED; a NULL cfg is OPHPC_ERROR_INVALID_ARGUMENT), but no
 * context: it runs on the calling thread's current device, and its scratch is
 * one file-scope 32 MiB device array that every GPU loading the library holds
 * until the process exits. It allocates nothing. Every call looks up the
 * array's device address on the current device and sets the kernels'
 * shared-memory limits there (neither allocates), so a device reset between
 * calls is harmless; the first call on a device also loads the library's
 * device code there, so make that first call before any stream capture.
 * n_points * n_channels above OPHPC_STATIC_SCRATCH_RECORDS is rejected with
 * OPHPC_ERROR_INVALID_ARGUMENT before any work is queued, and so are field
 * and vertex buffers in another device's memory. A CUDA error already
 * pending on the calling thread is reported as OPHPC_ERROR_CUDA before any
 * work is queued and is left pending. All calls on a device share the array
 * and it keeps the last call's contents; nothing in it needs to start at
 * zero, but calls whose GPU work overlaps (other streams, unsynchronised
 * threads) race on it. Small fields run slower than through ophpc_generate:
 * with no room for partial sums, the point range is never split across CTAs,
 * so a field of few 64x32 tiles leaves most SMs idle. Asynchronous on
 * `stream`. */
ophpc_status ophpc_generate_static_scratch(const ophpc_config* cfg, const ophpc_vertex* d_vertices,
                                           uint64_t n_points, uint32_t diff_flag, uint32_t mode,
                                           double* d_field, void* stream);

/* ophGen::normalize alone on device: min/max over all channels of
 * d_encoded ([n_channels][n_pixels] doubles) and the 8-bit codes into
 * d_normalized. Asynchronous on `stream`. */
ophpc_status ophpc_normalize(ophpc_context* ctx, const double* d_encoded, uint32_t n_channels,
                             uint64_t n_pixels, uint8_t* d_normalized, void* stream);

/* Plans: one ophpc_generate (and, unless encode_flag is
 * OPHPC_PLAN_NO_ENCODE, one ophpc_encode of its field) captured once into a
 * CUDA graph and replayed by ophpc_plan_launch. This entry point has no
 * counterpart in the reference. It is for callers that generate the same
 * shapes over and over (successive frames of a moving point cloud, many
 * small jobs): one graph launch replaces the host work and kernel launches
 * of every call. The buffers are fixed at creation and must stay valid;
 * each replay reads the vertices currently in d_vertices, so the caller
 * writes the next frame's points there (on the replay's stream, or before
 * it) and launches again. Scratch is allocated and freed inside the graph.
 * Replays of one plan must not overlap in time (wait for one before the
 * next on another stream); ophpc_plan_wait synchronises `stream` and
 * reports the tensor-core kernels' timeout word of the last replay
 * (OPHPC_ERROR_TIMEOUT), which ophpc_generate reports itself. Results are
 * bit-identical to the direct calls. ophpc_kernel_launches counts a plan's
 * kernels once, at creation. */
#define OPHPC_PLAN_NO_ENCODE 0xffffffffu
typedef struct ophpc_plan ophpc_plan;
ophpc_status ophpc_plan_create(ophpc_context* ctx, const ophpc_config* cfg, const ophpc_vertex* d_vertices,
                               uint64_t n_points, uint32_t diff_flag, uint32_t mode, double* d_field,
                               uint32_t encode_flag, double* d_encoded, uint8_t* d_normalized,
                               ophpc_plan** out);
ophpc_status ophpc_plan_launch(ophpc_plan* plan, void* stream);
ophpc_status ophpc_plan_wait(ophpc_plan* plan, void* stream);
ophpc_status ophpc_plan_destroy(ophpc_plan* plan);

#ifdef __cplusplus
}
#endif

#endif /* OPHPC_H */
