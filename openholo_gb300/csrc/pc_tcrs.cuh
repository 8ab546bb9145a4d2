// Tensor-core Rayleigh-Sommerfeld: which (point, tile) pairs it evaluates.
//
// The tensor-core RS kernel (pc_tcrs.cu) covers the field in 128x128 pixel
// tiles and expands each point's phase around the tile centre; the CUDA-core
// RS kernel (pc_rs.cu) then adds every pair the expansion does not hold for.
// Both kernels call rs_tc_eligible on the same (point, 128x128 tile) and
// must reach the same decision, so every operation in it is explicitly
// rounded (no FMA contraction is left to the compiler).
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
constexpr float kRsTcMaxCross = 4e-3f;       // radians, first-order e^{i theta}: error theta^2/2
constexpr float kRsTcMaxDropped = 2e-7f;     // turns

// Decides whether the tensor-core RS kernel evaluates point p on the
// 128x128 tile with origin (X0, Y0) of channel g. True only when
//  - the point's window rectangle holds every valid pixel of the tile,
//  - every valid pixel of the tile passes the reference's cone test
//    (ophgen/src/ophGen.cpp:415-428) with a relative margin of 1e-5,
//  - |w| = |r_p^2 - r_c^2| / r_c^2 <= kRsTcMaxW over the tile, the phase
//    terms the factors drop stay under kRsTcMaxDropped turns and the cross
//    phase under kRsTcMaxCross radians.
// wxm / wym receive the bounds of |w_x|, |w_y| over the tile.
__device__ __forceinline__ bool rs_tc_eligible(const PointRec& p, const ChannelGeom& g, int X0, int Y0,
                                               float* wxm_out, float* wym_out) {
    const int vx1 = min(X0 + kRsTcTile, g.pnX), vy1 = min(Y0 + kRsTcTile, g.pnY);
    if (!(p.x_lo <= X0 && p.x_hi >= vx1 && p.y_lo <= Y0 && p.y_hi >= vy1)) return false;
    const int xc = X0 + kRsTcHalf, yc = Y0 + kRsTcHalf;
    const float dxf = __double2float_rn(__dsub_rn(pixel_x(g, xc), p.x));
    const float dyf = __double2float_rn(__dsub_rn(pixel_y(g, yc), p.y));
    const float zzf = __double2float_rn(p.aux);
    // offsets of the valid pixels from the centre: u grows with the column,
    // v falls with the row
    const float umin = __double2float_rn(__dmul_rn((double)(X0 - xc), g.ppX));
    const float umax = __double2float_rn(__dmul_rn((double)(vx1 - 1 - xc), g.ppX));
    const float vmax = __double2float_rn(__dmul_rn((double)(yc - Y0), g.ppY));
    const float vmin = __double2float_rn(__dmul_rn((double)(yc - (vy1 - 1)), g.ppY));
    const float uext = __double2float_rn(__dmul_rn((double)kRsTcHalf, g.ppX));
    const float vext = __double2float_rn(__dmul_rn((double)kRsTcHalf, g.ppY));
    // cone test over the tile, conservative
    const float xa = __fadd_rn(dxf, umin), xb = __fadd_rn(dxf, umax);
    const float ya = __fadd_rn(dyf, vmin), yb = __fadd_rn(dyf, vmax);
    const float slack = __fmul_rn(1e-6f, __fadd_rn(__fadd_rn(fabsf(dxf), fabsf(dyf)), __fadd_rn(uext, vext)));
    const float maxdx = __fadd_rn(fmaxf(fabsf(xa), fabsf(xb)), slack);
    const float maxdy = __fadd_rn(fmaxf(fabsf(ya), fabsf(yb)), slack);
    const float mindx = fmaxf(__fsub_rn((xa <= 0.f && xb >= 0.f) ? 0.f : fminf(fabsf(xa), fabsf(xb)), slack), 0.f);
    const float mindy = fmaxf(__fsub_rn((ya <= 0.f && yb >= 0.f) ? 0.f : fminf(fabsf(ya), fabsf(yb)), slack), 0.f);
    const float detx = __double2float_rn(g.detx), dety = __double2float_rn(g.dety);
    const float keep = 1.f - 1e-5f;
    const float rx = __fmul_rn(__fmul_rn(detx, __fsqrt_rn(__fadd_rn(__fmul_rn(mindy, mindy), zzf))), keep);
    const float ry = __fmul_rn(__fmul_rn(dety, __fsqrt_rn(__fadd_rn(__fmul_rn(mindx, mindx), zzf))), keep);
    if (!(maxdx < rx && maxdy < ry)) return false;
    // expansion bounds
    const float rc2 = __fadd_rn(__fadd_rn(__fmul_rn(dxf, dxf), __fmul_rn(dyf, dyf)), zzf);
    const float hf = __fdiv_rn(1.0f, rc2);
    const float grow = 1.0f + 1e-4f;
    const float nxm = __fadd_rn(__fmul_rn(__fmul_rn(2.f, fabsf(dxf)), uext), __fmul_rn(uext, uext));
    const float nym = __fadd_rn(__fmul_rn(__fmul_rn(2.f, fabsf(dyf)), vext), __fmul_rn(vext, vext));
    const float wxm = __fmul_rn(__fmul_rn(nxm, hf), grow);
    const float wym = __fmul_rn(__fmul_rn(nym, hf), grow);
    const float tau = __fmul_rn(__fmul_rn(__fsqrt_rn(rc2), __double2float_rn(g.inv_lambda)), grow);
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
// CUDA-core complement. jg comes from the plain path's geometry; the call
// synchronises `stream` at the end to read the kernels' error word.
ophpc_status tc_generate_rs(cudaMemPool_t pool, const JobGeom& jg, const ophpc_config* cfg,
                            const ophpc_vertex* d_vertices, uint64_t n_points, double* d_field,
                            cudaStream_t stream, std::string* err);

}  // namespace ophpc
