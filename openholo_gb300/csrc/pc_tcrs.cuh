// Tensor-core Rayleigh-Sommerfeld: which (point, tile) pairs it evaluates.
//
// The tensor-core RS kernel (pc_tcrs.cu) covers the field in 128x128 pixel
// tiles and expands each point's phase around the tile centre; the CUDA-core
// RS kernel (pc_rs.cu) then adds every pair the expansion does not hold for.
// Both kernels call rs_tc_eligible on the same (point, 128x128 tile) and
// must reach the same decision, so every operation in it is explicitly
// rounded or a pinned hardware instruction (no FMA contraction is left to the
// compiler).
#pragma once

#include "pc_common.cuh"
#include "ophpc.h"

#include <string>

namespace ophpc {

constexpr int kRsTcTile = 128;   // pixels per side of a tensor-core RS tile
constexpr int kRsTcHalf = kRsTcTile / 2;

// Expansion limits (see pc_tcrs.cu): |w_x| + |w_y| bound, the dropped
// cross-term error, and the phase terms left out of the factors (turns).
constexpr float kRsTcMaxW = 1e-3f;
constexpr float kRsTcMaxCross = 8e-3f;       // radians, first-order e^{i theta}: error theta^2/2 <= 3.2e-5
constexpr float kRsTcMaxDropped = 2e-7f;     // turns

// Constants of one 128x128 tile (origin X0, Y0) that the eligibility test
// uses; both kernels form them with rs_tc_tile.
struct RsTcTile {
    int32_t X0, Y0, vx1, vy1;     // origin and end of the valid pixels
    int32_t xc, yc;               // centre pixel indices (X0 + 64, Y0 + 64)
    double Xc, Yc;                // centre pixel coordinates
    double ppx, ppy;              // pixel pitches
    float umin, umax, vmin, vmax; // offsets of the valid pixels from the centre (u with the column, v against the row)
    float uext, vext;             // 64 pitches
    float detx, dety, inv_lambda;
};

__device__ __forceinline__ RsTcTile rs_tc_tile(const ChannelGeom& g, int X0, int Y0) {
    RsTcTile t;
    t.X0 = X0;
    t.Y0 = Y0;
    t.vx1 = min(X0 + kRsTcTile, g.pnX);
    t.vy1 = min(Y0 + kRsTcTile, g.pnY);
    const int xc = X0 + kRsTcHalf, yc = Y0 + kRsTcHalf;
    t.xc = xc;
    t.yc = yc;
    t.ppx = g.ppX;
    t.ppy = g.ppY;
    t.Xc = pixel_x(g, xc);
    t.Yc = pixel_y(g, yc);
    t.umin = __double2float_rn(__dmul_rn((double)(X0 - xc), g.ppX));
    t.umax = __double2float_rn(__dmul_rn((double)(t.vx1 - 1 - xc), g.ppX));
    t.vmax = __double2float_rn(__dmul_rn((double)(yc - Y0), g.ppY));
    t.vmin = __double2float_rn(__dmul_rn((double)(yc - (t.vy1 - 1)), g.ppY));
    t.uext = __double2float_rn(__dmul_rn((double)kRsTcHalf, g.ppX));
    t.vext = __double2float_rn(__dmul_rn((double)kRsTcHalf, g.ppY));
    t.detx = __double2float_rn(g.detx);
    t.dety = __double2float_rn(g.dety);
    t.inv_lambda = __double2float_rn(g.inv_lambda);
    return t;
}

// Hardware reciprocal square root and reciprocal (MUFU), pinned through
// inline PTX so that both kernels execute the same instruction: their ~1e-7
// relative error sits far inside the test's margins, and they are far cheaper
// than the IEEE-rounded sqrt and division.
__device__ __forceinline__ float rsqrt_hw(float x) {
    float r;
    asm("rsqrt.approx.ftz.f32 %0, %1;" : "=f"(r) : "f"(x));
    return r;
}
__device__ __forceinline__ float rcp_hw(float x) {
    float r;
    asm("rcp.approx.ftz.f32 %0, %1;" : "=f"(r) : "f"(x));
    return r;
}

// Decides whether the tensor-core RS kernel evaluates point p on tile t.
// True only when
//  - the point's window rectangle meets the tile (the pixels outside the
//    rectangle get zero factors: the rectangle is separable),
//  - every valid pixel of the tile inside the rectangle passes the
//    reference's cone test (ophgen/src/ophGen.cpp:415-428) with a relative
//    margin of 1e-5 (near a window edge this fails only on the rectangle's
//    first column, where the reference's pixel grid puts |X - x| at or
//    beyond the half-width),
//  - |w| = |r_p^2 - r_c^2| / r_c^2 <= kRsTcMaxW over the tile, the phase
//    terms the factors drop stay under kRsTcMaxDropped turns and the cross
//    phase under kRsTcMaxCross radians.
// wxm / wym receive the bounds of |w_x|, |w_y| over the tile. A pair whose
// rectangle holds the tile is decided on the tile's own bounds.
__device__ __forceinline__ bool rs_tc_eligible(const PointRec& p, const RsTcTile& t, float* wxm_out,
                                               float* wym_out) {
    const int ix0 = max(t.X0, p.x_lo), ix1 = min(t.vx1, p.x_hi);
    const int iy0 = max(t.Y0, p.y_lo), iy1 = min(t.vy1, p.y_hi);
    if (!(ix0 < ix1 && iy0 < iy1)) return false;
    float umin = t.umin, umax = t.umax, vmin = t.vmin, vmax = t.vmax;
    if (!(ix0 == t.X0 && ix1 == t.vx1 && iy0 == t.Y0 && iy1 == t.vy1)) {
        umin = __double2float_rn(__dmul_rn((double)(ix0 - t.xc), t.ppx));
        umax = __double2float_rn(__dmul_rn((double)(ix1 - 1 - t.xc), t.ppx));
        vmax = __double2float_rn(__dmul_rn((double)(t.yc - iy0), t.ppy));
        vmin = __double2float_rn(__dmul_rn((double)(t.yc - (iy1 - 1)), t.ppy));
    }
    const float dxf = __double2float_rn(__dsub_rn(t.Xc, p.x));
    const float dyf = __double2float_rn(__dsub_rn(t.Yc, p.y));
    const float zzf = __double2float_rn(p.aux);
    // cone test over the tile's pixels inside the rectangle, conservative
    const float xa = __fadd_rn(dxf, umin), xb = __fadd_rn(dxf, umax);
    const float ya = __fadd_rn(dyf, vmin), yb = __fadd_rn(dyf, vmax);
    const float slack = __fmul_rn(1e-6f, __fadd_rn(__fadd_rn(fabsf(dxf), fabsf(dyf)), __fadd_rn(t.uext, t.vext)));
    const float maxdx = __fadd_rn(fmaxf(fabsf(xa), fabsf(xb)), slack);
    const float maxdy = __fadd_rn(fmaxf(fabsf(ya), fabsf(yb)), slack);
    const float mindx = fmaxf(__fsub_rn((xa <= 0.f && xb >= 0.f) ? 0.f : fminf(fabsf(xa), fabsf(xb)), slack), 0.f);
    const float mindy = fmaxf(__fsub_rn((ya <= 0.f && yb >= 0.f) ? 0.f : fminf(fabsf(ya), fabsf(yb)), slack), 0.f);
    const float keep = 1.f - 1e-5f;
    // sqrt(q) as q * rsqrt(q) (q >= z^2 > 0)
    const float qx = __fadd_rn(__fmul_rn(mindy, mindy), zzf), qy = __fadd_rn(__fmul_rn(mindx, mindx), zzf);
    const float rx = __fmul_rn(__fmul_rn(t.detx, __fmul_rn(qx, rsqrt_hw(qx))), keep);
    const float ry = __fmul_rn(__fmul_rn(t.dety, __fmul_rn(qy, rsqrt_hw(qy))), keep);
    if (!(maxdx < rx && maxdy < ry)) return false;
    // expansion bounds
    const float rc2 = __fadd_rn(__fadd_rn(__fmul_rn(dxf, dxf), __fmul_rn(dyf, dyf)), zzf);
    const float hf = rcp_hw(rc2);
    const float grow = 1.0f + 1e-4f;
    const float nxm = __fadd_rn(__fmul_rn(__fmul_rn(2.f, fabsf(dxf)), t.uext), __fmul_rn(t.uext, t.uext));
    const float nym = __fadd_rn(__fmul_rn(__fmul_rn(2.f, fabsf(dyf)), t.vext), __fmul_rn(t.vext, t.vext));
    const float wxm = __fmul_rn(__fmul_rn(nxm, hf), grow);
    const float wym = __fmul_rn(__fmul_rn(nym, hf), grow);
    const float tau = __fmul_rn(__fmul_rn(__fmul_rn(rc2, rsqrt_hw(rc2)), t.inv_lambda), grow);
    const float s = __fadd_rn(wxm, wym);
    const float pxy = __fmul_rn(wxm, wym);
    const float cross = __fmul_rn(__fmul_rn(1.5707964f, tau), pxy);
    const float third = __fmul_rn(__fmul_rn(0.1875f, tau), __fmul_rn(pxy, s));
    const float s2 = __fmul_rn(s, s);
    const float fourth = __fmul_rn(__fmul_rn(0.0390625f, tau), __fmul_rn(s2, s2));
    *wxm_out = wxm;
    *wym_out = wym;
    return s <= kRsTcMaxW && cross <= kRsTcMaxCross && third <= kRsTcMaxDropped && fourth <= kRsTcMaxDropped;
}

// Host entry (pc_tcrs.cu): RS generate on the tensor cores plus the
// CUDA-core complement. jg comes from the plain path's geometry; sm_count
// sizes the point-range split. The call synchronises `stream` at the end to
// read the kernels' error word, unless d_err_out is given: then that device
// word receives it (stream-ordered) and nothing waits, so that the call can
// be captured into a CUDA graph.
ophpc_status tc_generate_rs(cudaMemPool_t pool, const JobGeom& jg, const ophpc_config* cfg,
                            const ophpc_vertex* d_vertices, uint64_t n_points, double* d_field, int sm_count,
                            cudaStream_t stream, std::string* err, int* d_err_out = nullptr);

// Building blocks for callers that run a job as point-range steps (the
// serving engine). launch_rs_amax: per channel the largest coef / z^2 of the
// RS records into d_amax[0..n_channels), and into word 3 a flag set when
// some point's window rectangle leaves part of the pnX x pnY field out
// (d_amax holds 4 words, zeroed by the caller).
// launch_tc_rs_range: points [p0, p1) of the records on the tensor cores,
// overwriting the field (accumulate false) or adding into it, then the
// CUDA-core complement for the same range; d_left holds n_channels x tiles
// ints (128x128 tiles) of scratch; d_mask (optional) n_channels x tiles x
// mask_words words, mask_words >= tc_rs_mask_words(p1 - p0), through which
// the complement finds the pairs left to it; *d_err is set on a kernel
// timeout.
void launch_rs_amax(const PointRec* d_recs, int64_t n_points, int n_channels, int pnX, int pnY, float* d_amax,
                    cudaStream_t stream);
inline int64_t tc_rs_mask_words(int64_t n_points) { return (n_points + 255) / 256 * 8; }
cudaError_t launch_tc_rs_range(const JobGeom& jg, const PointRec* d_recs, int64_t p0, int64_t p1, bool accumulate,
                               double2* d_field, const float* d_amax, int32_t* d_left, uint32_t* d_mask,
                               int64_t mask_words, int* d_err, cudaStream_t stream);

// Fresnel on the tensor cores with the factors generated on chip
// (tc_fresnel_kernel, split-BF16, FP32 accumulation, FP64 field): the same
// 128x128 tile pipeline as the RS kernel; the phase splits exactly and the
// window is a rectangle, so every pair runs on the tensor cores. Whole call
// (same conventions as tc_generate_rs), and the point-range building blocks
// for the serving engine: launch_fresnel_amax (per channel the largest coef
// into d_amax, zeroed by the caller) and launch_tc_fresnel_range.
ophpc_status tc_generate_fresnel_tiles(cudaMemPool_t pool, const JobGeom& jg, const ophpc_config* cfg,
                                       const ophpc_vertex* d_vertices, uint64_t n_points, double* d_field,
                                       int sm_count, cudaStream_t stream, std::string* err, int* d_err_out = nullptr);
void launch_fresnel_amax(const PointRec* d_recs, int64_t n_points, int n_channels, float* d_amax, cudaStream_t stream);
cudaError_t launch_tc_fresnel_range(const JobGeom& jg, const PointRec* d_recs, int64_t p0, int64_t p1,
                                    bool accumulate, double2* d_field, const float* d_amax, int* d_err,
                                    cudaStream_t stream);

}  // namespace ophpc
