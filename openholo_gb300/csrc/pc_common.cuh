// Shared definitions of the point-cloud hologram kernels (sm_103a).
//
// Data layout in HBM for one generate call:
//   vertices  : caller's ophpc_vertex[n] (56 B packed AoS, read once by prep)
//   PointRec  : [n_channels][n_points] 64-byte records written by prep_points
//               (FP64 scaled position, amplitude coefficient, window rectangle)
//   field     : [n_channels][pnY][pnX] double2 (re, im), the complex_H layout
//   partials  : [ksplit-1][n_channels][pnY][pnX] double2, only when the point
//               range is split across CTAs to fill the GPU on small fields
#pragma once

#include <cstdint>
#include <cuda_runtime.h>

namespace ophpc {

// Pixel tile of one CTA and the per-thread pixel block.
constexpr int kTileW = 64;          // pixels along x per CTA
constexpr int kTileH = 32;          // pixels along y per CTA
constexpr int kThreads = 128;       // 16 x 8 threads
constexpr int kPixW = 4;            // columns per thread (adjacent)
constexpr int kPixH = 4;            // rows per thread (adjacent)
constexpr int kThreadsX = kTileW / kPixW;   // 16
constexpr int kChunk = 256;         // points staged per shared-memory round

static_assert(kThreadsX * (kTileH / kPixH) == kThreads, "tile / thread layout mismatch");

// Per (channel, point) record produced by prep_points.
struct __align__(16) PointRec {
    double x, y, z;     // scaled (and viewing-window transformed) position; z includes Distance
    double coef;        // RS: amp*z/lambda   Fresnel: amp/(lambda*z)
    int32_t x_lo, x_hi; // window rectangle, pixel columns [x_lo, x_hi), clipped to [0, pnX]
    int32_t y_lo, y_hi; // pixel rows [y_lo, y_hi), clipped to [0, pnY]
    double aux;         // Fresnel: 1/(2*z*lambda); RS: z*z
    double pad;
};
static_assert(sizeof(PointRec) == 64, "PointRec must stay 64 bytes");

// Geometry of one channel, passed by value.
struct ChannelGeom {
    int32_t pnX, pnY, offX, offY;
    double ppX, ppY;
    double x0, y0;          // -ssX/2, -ssY/2 with ss = pn*pp (ophGen.cpp:368-379)
    double lambda, inv_lambda;
    double detx, dety;      // RS window slopes tx/sqrt(1-tx^2), tx = lambda/(2pp)
};

struct JobGeom {
    ChannelGeom ch[3];
    int32_t n_channels;
    int32_t tiles_x, tiles_y;
    int32_t ksplit;         // point-range splits per tile
    int64_t n_points;
    int64_t points_per_split;
    // Point range of this launch, [p0, p1); p1 == 0 means all n_points.
    // With accumulate != 0 the kernels add into the field instead of
    // overwriting it (a job computed as several point-range launches).
    int64_t p0, p1;
    int32_t accumulate;
    // RS only, set for the CUDA-core complement of the tensor-core RS
    // kernel: skip the (point, tile) pairs that kernel evaluated
    // (rs_tc_eligible on the enclosing 128x128 tile). tc_left[ch][ty][tx]
    // counts, per 128x128 tile, the pairs left to the CUDA cores; tiles with
    // none are skipped whole.
    int32_t tc_skip;
    const int32_t* tc_left;
    int32_t tc_tiles_x, tc_tiles_y;
    // When set: per 128x128 tile, one bit per point of the launch's range
    // (bit i of word i / 32, i relative to p0; tc_mask_words words a tile,
    // [ch][ty][tx][word]) for the pairs that kernel left; the complement
    // reads these instead of re-testing eligibility, and skips the rest
    // without loading them.
    const uint32_t* tc_mask;
    int64_t tc_mask_words;
};

// Pixel-centre coordinates, exactly as the reference forms them
// (ophGen.cpp:413,422; ophPCKernel.cu:97-98): explicit roundings, no FMA.
__device__ __forceinline__ double pixel_x(const ChannelGeom& g, int xi) {
    return __dadd_rn(g.x0, __dmul_rn((double)(xi - 1 + g.offX), g.ppX));
}
__device__ __forceinline__ double pixel_y(const ChannelGeom& g, int yi) {
    return __dadd_rn(g.y0, __dmul_rn((double)(g.pnY - yi + g.offY), g.ppY));
}

// Reduce a phase in turns to [-0.5, 0.5]: t - rint(t) with the 1.5*2^23
// round-to-nearest constant, kept on the FP32 add pipe.
__device__ __forceinline__ float reduce_turns(float t) {
    const float kMagic = 12582912.0f;
    float r = __fsub_rn(__fadd_rn(t, kMagic), kMagic);
    return __fsub_rn(t, r);
}

// sin(2 pi t) and cos(2 pi t) for t in [-0.5, 0.5]: sin = t S(t^2) (degree 5
// in t^2), cos = C(t^2) (degree 6), least-squares fits on Chebyshev nodes of
// [0, 0.5] made for this library; evaluated with FMA in FP32 the error is
// below 4e-7 (sin) and 6e-7 (cos) absolute, as good as the MUFU's.
__device__ __forceinline__ void sincos_turns_poly(float t, float* s, float* c) {
    const float u = t * t;
    float ps = -1.230215740e+01f;
    ps = fmaf(ps, u, 4.122758102e+01f);
    ps = fmaf(ps, u, -7.658597565e+01f);
    ps = fmaf(ps, u, 8.159687805e+01f);
    ps = fmaf(ps, u, -4.134145737e+01f);
    ps = fmaf(ps, u, 6.283183575e+00f);
    float pc = 6.547553062e+00f;
    pc = fmaf(pc, u, -2.598241234e+01f);
    pc = fmaf(pc, u, 6.017204666e+01f);
    pc = fmaf(pc, u, -8.545075989e+01f);
    pc = fmaf(pc, u, 6.493915558e+01f);
    pc = fmaf(pc, u, -1.973920631e+01f);
    pc = fmaf(pc, u, 1.0f);
    *s = ps * t;
    *c = pc;
}

// Packed FP32 pairs (sm_100+ .f32x2 arithmetic): one instruction issues two
// FP32 operations, halving issue slots in the per-pixel loops. A pair lives
// in a 64-bit register (low half = first element).
namespace f2 {
typedef unsigned long long v2;
__device__ __forceinline__ v2 pack(float lo, float hi) {
    v2 r;
    asm("mov.b64 %0, {%1, %2};" : "=l"(r) : "f"(lo), "f"(hi));
    return r;
}
__device__ __forceinline__ v2 splat(float x) { return pack(x, x); }
__device__ __forceinline__ void unpack(v2 v, float& lo, float& hi) {
    asm("mov.b64 {%0, %1}, %2;" : "=f"(lo), "=f"(hi) : "l"(v));
}
__device__ __forceinline__ v2 add(v2 a, v2 b) {
    v2 d;
    asm("add.rn.f32x2 %0, %1, %2;" : "=l"(d) : "l"(a), "l"(b));
    return d;
}
__device__ __forceinline__ v2 sub(v2 a, v2 b) {
    v2 d;
    asm("sub.rn.f32x2 %0, %1, %2;" : "=l"(d) : "l"(a), "l"(b));
    return d;
}
__device__ __forceinline__ v2 mul(v2 a, v2 b) {
    v2 d;
    asm("mul.rn.f32x2 %0, %1, %2;" : "=l"(d) : "l"(a), "l"(b));
    return d;
}
__device__ __forceinline__ v2 fma(v2 a, v2 b, v2 c) {
    v2 d;
    asm("fma.rn.f32x2 %0, %1, %2, %3;" : "=l"(d) : "l"(a), "l"(b), "l"(c));
    return d;
}
// t - rint(t) on both halves (1.5*2^23 round-to-nearest constant)
__device__ __forceinline__ v2 reduce_turns(v2 t) {
    const v2 m = splat(12582912.0f);
    return sub(t, sub(add(t, m), m));
}
}  // namespace f2

// Count of kernels this library has launched (all contexts, all threads);
// read through ophpc_kernel_launches().
void count_launches(unsigned n);
uint64_t launches_so_far();

// Launchers (defined in the .cu files).
// color_offset: channel c takes its amplitude from color[c + color_offset].
void launch_prep(const void* d_vertices, int64_t n_points, const double* scale, double distance,
                 double field_length, int viewing_window, int diff_flag, const JobGeom& jg,
                 PointRec* d_recs, cudaStream_t stream, int color_offset = 0);
void launch_rs(const PointRec* d_recs, const JobGeom& jg, double2* d_field, double2* d_partials,
               cudaStream_t stream);
void launch_fresnel(const PointRec* d_recs, const JobGeom& jg, double2* d_field, double2* d_partials,
                    cudaStream_t stream);
void launch_sum_partials(const JobGeom& jg, double2* d_field, const double2* d_partials,
                         cudaStream_t stream);
// d_minmax: 5 words of device scratch (global min/max + per-channel |H|
// maxima). For SIMPLENI, BURCKHARDT and TWOPHASE d_encoded is required and
// in/out (entries the encoder skips keep their value).
void launch_encode(const double2* d_field, int n_channels, int64_t n_pixels, int encode_flag,
                   double* d_encoded, uint8_t* d_normalized, unsigned long long* d_minmax,
                   cudaStream_t stream);
void launch_normalize(const double* d_encoded, int n_channels, int64_t n_pixels, uint8_t* d_normalized,
                      unsigned long long* d_minmax, cudaStream_t stream);
int rs_blocks_per_sm();
int fresnel_blocks_per_sm();
// Raise the kernels' dynamic shared-memory limit on the current device (a
// per-module attribute: it is lost when the context is reset).
cudaError_t rs_set_smem_limit();
cudaError_t fresnel_set_smem_limit();

}  // namespace ophpc
