// Rayleigh-Sommerfeld point-cloud kernel (sm_103a, FP32 core with FP64 phase
// reduction).
//
// Computes, for every pixel p of every channel, the reference's sum
//   H(p) = sum_j  a_j z_j / (lambda r_pj^2) * (sin(k r_pj), -cos(k r_pj))
// over the points whose anti-aliasing window contains p
// (ophgen/src/ophGen.cpp:361-445; GPU counterpart ophgen/src/ophPCKernel.cu:66-176).
//
// Work decomposition: one CTA owns a 64x32 pixel tile (4x4 adjacent pixels
// per thread) of one channel and streams the point list through shared
// memory in chunks of 256. Per (point, tile) the CTA evaluates in FP64 the
// distance r_c from the point to the tile centre and keeps only
// frac(r_c/lambda) — the only FP64 step; k*r reaches ~6e6 rad. Per pixel the
// remaining phase is carried in FP32 through the compensated form
//   r_p - r_c = r_c (sqrt(1+w) - 1),  w = (r_p^2 - r_c^2) / r_c^2,
// where r_p^2 - r_c^2 = 2 dx_c u + u^2 + 2 dy_c v + v^2 is formed from small
// tile-local offsets (u, v) and splits into a per-column plus a per-row part.
// In the FAST class (tile inside the window, |w| small) the series
// w/2 - w^2/8 replaces sqrt and division, and the phase is carried in
// radians: 2 pi frac(r_c/lambda) plus tile-local offsets that the class
// keeps within +-16 turns, so the MUFU sin/cos (whose own argument scaling
// stays accurate to ~1e-5 rad there) needs no per-pixel reduction. A pixel
// costs 7 FP32 issue slots and two MUFU (sin, cos); two pixels of each 4x4
// block instead take the phase in turns, reduce it, and evaluate sin/cos as
// polynomials on the FMA pipe, which relieves the MUFU (the kernel's bound).
// Points whose tile-local phase offsets exceed +-16 turns (off-axis points
// close to the SLM) stay in the FAST class with the phase carried in turns
// and reduced to [-0.5, 0.5] per pixel before the MUFU: three more FP32
// slots, the same two MUFU. Tiles the window cuts, or with large |w|, go to the
// EXACT class: integer rectangle test, the reference's cone test (FP32 with
// a margin, FP64 replica of ophGen.cpp:415-428 when inside the margin;
// skipped when the window and the cone test hold for the whole tile) and
// the exact r_p. Sums run in FP32 per chunk and are folded into FP64
// shared-memory sums after every chunk; every pixel is stored once.
#include "pc_common.cuh"
#include "pc_tcrs.cuh"

namespace ophpc {

namespace {

struct __align__(16) RsSRec {
    float P, Q, h, g;        // FAST: 2dxc/rc2, 2dyc/rc2, 1/rc2, pi rc/lambda. EXACT: 2dxc, 2dyc, rc2, rc
    float fc, ac, dxc, dyc;  // FAST: 2 pi frac(rc/lambda), coef/rc2, -pi rc/(4 lambda), -
                             // EXACT: frac(rc/lambda) in [-.5,.5], coef, dxc, dyc
    float zz, mabs;          // FAST: rc/(2 lambda), -rc/(8 lambda) (turns). EXACT: z^2, margin of the FP32 cone test
    int32_t idx;             // EXACT: point index (FP64 fallback)
    int32_t xl, xh, yl, yh;  // EXACT: window rectangle relative to the tile origin
    int32_t whole;           // EXACT: 1 when the window and the cone test hold for the whole tile; 2: FAST, reduced phase
};
static_assert(sizeof(RsSRec) == 64, "RsSRec size");

constexpr float kTwoPi = 6.283185307179586f;
// FAST requires (rc/lambda) * |w|^3 / 16 below this many turns (series error,
// below the FP32 rounding of the phase itself: ~1.5e-6 turns at the 25
// turns the tile-local offsets reach) and |w| below kMaxW (the dropped
// amplitude term is w^2).
constexpr float kSeriesTol = 1e-7f;
constexpr float kMaxW = 1e-3f;
// FAST also requires the tile-local phase offset (tc/2)|w| + (tc/8)w^2 below
// this many turns: the FP32 phase in radians then stays under ~103 rad.
constexpr float kMaxTurns = 16.f;
constexpr float kPi = 3.14159265358979f;

// Pixels of a thread's 4x4 block (bit r*4 + c) whose sin/cos run as
// polynomials on the FMA pipe instead of the MUFU, to balance the two pipes:
// two corner pixels of 16. Measured at sphere_fhd on GB300: 0 pixels
// 2.28e12 interactions/s, 1 2.37e12, 2 2.36-2.43e12 (by placement), 3
// 2.26e12, 4 2.15e12; the block issue rate, not the MUFU, binds beyond two.
constexpr unsigned kPolyMask = 0x8001u;


// One FAST point's terms for the thread's 4x4 pixels. REDUCE: the phase in
// turns, reduced to [-0.5, 0.5], then the MUFU sin/cos of 2 pi t; else the
// phase in radians straight into the MUFU (tile-local offsets within +-16
// turns). The pixels of kPolyMask always take the reduced phase and the
// FMA-pipe polynomials.
template <bool REDUCE>
__device__ __forceinline__ void fast_point(const RsSRec& rec, const float (&u)[kPixW], const float (&uu)[kPixW],
                                           const float (&v)[kPixH], const float (&vv)[kPixH],
                                           float (&sr)[kPixH * kPixW], float (&si)[kPixH * kPixW]) {
    const float4 a = *reinterpret_cast<const float4*>(&rec.P);    // P, Q, h, pi tc
    const float4 b = *reinterpret_cast<const float4*>(&rec.fc);   // 2 pi fc, ac, -pi tc/4, fc
    const float2 tq = *reinterpret_cast<const float2*>(&rec.zz);   // tc/2, -tc/8 (turns)
    float A[kPixW], B[kPixH];
#pragma unroll
    for (int c = 0; c < kPixW; ++c) A[c] = fmaf(a.x, u[c], a.z * uu[c]);
#pragma unroll
    for (int r = 0; r < kPixH; ++r) B[r] = fmaf(a.y, v[r], a.z * vv[r]);
#pragma unroll
    for (int r = 0; r < kPixH; ++r) {
#pragma unroll
        for (int c = 0; c < kPixW; ++c) {
            const float w = A[c] + B[r];
            const int k = r * kPixW + c;
            float s, co;
            if ((kPolyMask >> k) & 1u) {
                const float tt = reduce_turns(fmaf(w, fmaf(w, tq.y, tq.x), b.w));
                sincos_turns_poly(tt, &s, &co);
            } else if (REDUCE) {
                const float tt = reduce_turns(fmaf(w, fmaf(w, tq.y, tq.x), b.w));
                __sincosf(tt * kTwoPi, &s, &co);
            } else {
                const float ph = fmaf(w, fmaf(w, b.z, a.w), b.x);   // radians, |ph| < ~103
                __sincosf(ph, &s, &co);
            }
            const float amp = fmaf(-b.y, w, b.y);
            sr[k] = fmaf(amp, s, sr[k]);
            si[k] = fmaf(amp, co, si[k]);
        }
    }
}

// The thread's offsets u = X - Xc, v = Y - Yc of its 4x4 pixels from the
// tile centre, and their squares.
__device__ __forceinline__ void pixel_offsets(const ChannelGeom& g, float (&u)[kPixW], float (&uu)[kPixW],
                                              float (&v)[kPixH], float (&vv)[kPixH]) {
    const int tx = threadIdx.x % kThreadsX, ty = threadIdx.x / kThreadsX;
#pragma unroll
    for (int c = 0; c < kPixW; ++c) {
        u[c] = (float)((double)(tx * kPixW + c - kTileW / 2) * g.ppX);
        uu[c] = u[c] * u[c];
    }
#pragma unroll
    for (int r = 0; r < kPixH; ++r) {
        v[r] = (float)((double)(kTileH / 2 - (ty * kPixH + r)) * g.ppY);
        vv[r] = v[r] * v[r];
    }
}

// The paths below are out of line, so that the FAST loop keeps the
// registers it has without them; a CTA calls them only for chunks that have
// such records. Both add into acc (re [0, 16), im [16, 32)).

// FAST records whose tile-local phase offsets exceed +-16 turns (whole ==
// 2 among the n records stored from the back of the chunk): the phase in
// turns, reduced per pixel.
__device__ __noinline__ void reduced_records(const RsSRec* recs, int n, const ChannelGeom g, float* acc) {
    float u[kPixW], uu[kPixW], v[kPixH], vv[kPixH];
    pixel_offsets(g, u, uu, v, vv);
    float sr[kPixH * kPixW], si[kPixH * kPixW];
#pragma unroll
    for (int k = 0; k < kPixH * kPixW; ++k) {
        sr[k] = acc[k];
        si[k] = acc[kPixH * kPixW + k];
    }
#pragma unroll 1
    for (int j = 0; j < n; ++j) {
        const RsSRec& e = recs[kChunk - 1 - j];
        if (e.whole == 2) fast_point<true>(e, u, uu, v, vv, sr, si);   // uniform over the CTA
    }
#pragma unroll
    for (int k = 0; k < kPixH * kPixW; ++k) {
        acc[k] = sr[k];
        acc[kPixH * kPixW + k] = si[k];
    }
}

// EXACT records (window cuts the tile, or |w| too large for the series:
// whole < 2 among the n records stored from the back of the chunk).
__device__ __noinline__ void exact_records(const RsSRec* recs, int n, const ChannelGeom g, const PointRec* chrec,
                                           int X0, int Y0, float* acc) {
    const int tx = threadIdx.x % kThreadsX, ty = threadIdx.x / kThreadsX;
    float u[kPixW], uu[kPixW], v[kPixH], vv[kPixH];
    pixel_offsets(g, u, uu, v, vv);
    const float inv_lambda_f = (float)g.inv_lambda;
    const float detx_f = (float)g.detx, dety_f = (float)g.dety;
    float sr[kPixH * kPixW], si[kPixH * kPixW];
#pragma unroll
    for (int k = 0; k < kPixH * kPixW; ++k) {
        sr[k] = acc[k];
        si[k] = acc[kPixH * kPixW + k];
    }
#pragma unroll 1
    for (int j = 0; j < n; ++j) {
        const RsSRec& e = recs[kChunk - 1 - j];
        if (e.whole == 2) continue;   // uniform over the CTA
        bool inx[kPixW], iny[kPixH];
        float dx[kPixW], dy[kPixH], nx[kPixW], ny[kPixH];
#pragma unroll
        for (int c = 0; c < kPixW; ++c) {
            const int cl = tx * kPixW + c;
            inx[c] = cl >= e.xl && cl < e.xh;
            dx[c] = e.dxc + u[c];
            nx[c] = u[c] * (e.P + u[c]);
        }
#pragma unroll
        for (int r = 0; r < kPixH; ++r) {
            const int rl = ty * kPixH + r;
            iny[r] = rl >= e.yl && rl < e.yh;
            dy[r] = e.dyc + v[r];
            ny[r] = v[r] * (e.Q + v[r]);
        }
#pragma unroll
        for (int r = 0; r < kPixH; ++r) {
#pragma unroll
            for (int c = 0; c < kPixW; ++c) {
                if (!(inx[c] && iny[r])) continue;
                // cone test (ophGen.cpp:415-428): |X-x| < detx*sqrt((Y-y)^2+z^2)
                // and |Y-y| < dety*sqrt((X-x)^2+z^2), unless it holds for the whole tile
                bool inside = true;
                if (!e.whole) {
                    const float lx = fabsf(dx[c]), rx = detx_f * sqrtf(fmaf(dy[r], dy[r], e.zz));
                    const float ly = fabsf(dy[r]), ry = dety_f * sqrtf(fmaf(dx[c], dx[c], e.zz));
                    const float mx = 1e-5f * (lx + rx) + e.mabs, my = 1e-5f * (ly + ry) + e.mabs;
                    const bool xpass = rx - lx > mx, xfail = lx - rx > mx;
                    const bool ypass = ry - ly > my, yfail = ly - ry > my;
                    if (xfail || yfail) {
                        inside = false;
                    } else if (xpass && ypass) {
                        inside = true;
                    } else {
                        // FP64 replica of the reference decision
                        const PointRec p = chrec[e.idx];
                        const double xxx = pixel_x(g, X0 + tx * kPixW + c);
                        const double yyy = pixel_y(g, Y0 + ty * kPixH + r);
                        const double ddy = __dsub_rn(yyy, p.y), ddx = __dsub_rn(xxx, p.x);
                        const double hx = fabs(__dmul_rn(g.detx, sqrt(__dadd_rn(__dmul_rn(ddy, ddy), p.aux))));
                        const double hy = fabs(__dmul_rn(g.dety, sqrt(__dadd_rn(__dmul_rn(ddx, ddx), p.aux))));
                        inside = (xxx < __dadd_rn(p.x, hx)) && (xxx > __dsub_rn(p.x, hx)) &&
                                 (yyy < __dadd_rn(p.y, hy)) && (yyy > __dsub_rn(p.y, hy));
                    }
                }
                if (!inside) continue;
                const float nn = nx[c] + ny[r];
                const float rp2 = e.h + nn;
                const float ri = rsqrtf(rp2);
                const float rp = rp2 * ri;
                const float dt = __fdividef(nn * inv_lambda_f, rp + e.g);
                const float t = reduce_turns(e.fc + dt);
                float s, co;
                __sincosf(t * kTwoPi, &s, &co);
                const float amp = e.ac * ri * ri;
                const int k = r * kPixW + c;
                sr[k] = fmaf(amp, s, sr[k]);
                si[k] = fmaf(amp, co, si[k]);
            }
        }
    }
#pragma unroll
    for (int k = 0; k < kPixH * kPixW; ++k) {
        acc[k] = sr[k];
        acc[kPixH * kPixW + k] = si[k];
    }
}

__device__ __forceinline__ int warp_prefix(unsigned ballot) {
    return __popc(ballot & ((1u << (threadIdx.x & 31)) - 1u));
}

__global__ void __launch_bounds__(kThreads, 4)
rs_kernel(const PointRec* __restrict__ recs, const JobGeom jg, double2* __restrict__ field,
          double2* __restrict__ partials) {
    extern __shared__ __align__(16) unsigned char s_raw[];
    RsSRec* s_rec = reinterpret_cast<RsSRec*>(s_raw);
    // FP64 running sums, [pixel][thread]: consecutive threads hit consecutive 16-byte words
    double2* s_acc = reinterpret_cast<double2*>(s_raw + sizeof(RsSRec) * kChunk);
    __shared__ int s_cnt[2][2][kThreads / 32];   // [fast|back][q][warp]

    const int ch = blockIdx.z / jg.ksplit;
    const int part = blockIdx.z % jg.ksplit;
    const ChannelGeom& g = jg.ch[ch];
    const int X0 = blockIdx.x * kTileW, Y0 = blockIdx.y * kTileH;
    // complement of the tensor-core RS kernel: the enclosing 128x128 tile,
    // skipped whole when that kernel left none of its pairs
    const int tcX0 = X0 / kRsTcTile * kRsTcTile, tcY0 = Y0 / kRsTcTile * kRsTcTile;
    if (jg.tc_skip &&
        jg.tc_left[((int64_t)ch * jg.tc_tiles_y + tcY0 / kRsTcTile) * jg.tc_tiles_x + tcX0 / kRsTcTile] == 0)
        return;
    RsTcTile tct;
    if (jg.tc_skip) tct = rs_tc_tile(g, tcX0, tcY0);
    // the tensor-core kernel's bits for the pairs it left (relative to p0)
    const uint32_t* left_mask =
        jg.tc_skip && jg.tc_mask
            ? jg.tc_mask + (((int64_t)ch * jg.tc_tiles_y + tcY0 / kRsTcTile) * jg.tc_tiles_x + tcX0 / kRsTcTile) *
                               jg.tc_mask_words
            : nullptr;
    const int vx1 = min(X0 + kTileW, g.pnX), vy1 = min(Y0 + kTileH, g.pnY);
    const int xc = X0 + kTileW / 2, yc = Y0 + kTileH / 2;
    const double Xc = pixel_x(g, xc), Yc = pixel_y(g, yc);
    // offsets of the tile's valid pixels from its centre pixel: u = X - Xc
    // (grows with the column), v = Y - Yc (falls with the row)
    const float umin_f = (float)((double)(X0 - xc) * g.ppX), umax_f = (float)((double)(vx1 - 1 - xc) * g.ppX);
    const float vmax_f = (float)((double)(yc - Y0) * g.ppY), vmin_f = (float)((double)(yc - (vy1 - 1)) * g.ppY);
    const float uext_f = (float)((kTileW / 2) * g.ppX), vext_f = (float)((kTileH / 2) * g.ppY);

    const int tx = threadIdx.x % kThreadsX, ty = threadIdx.x / kThreadsX;
    const int warp = threadIdx.x >> 5;
    float u[kPixW], uu[kPixW], v[kPixH], vv[kPixH];
#pragma unroll
    for (int c = 0; c < kPixW; ++c) {
        u[c] = (float)((double)(tx * kPixW + c - kTileW / 2) * g.ppX);
        uu[c] = u[c] * u[c];
    }
#pragma unroll
    for (int r = 0; r < kPixH; ++r) {
        v[r] = (float)((double)(kTileH / 2 - (ty * kPixH + r)) * g.ppY);
        vv[r] = v[r] * v[r];
    }
    const float detx_f = (float)g.detx, dety_f = (float)g.dety;

#pragma unroll
    for (int k = 0; k < kPixH * kPixW; ++k) s_acc[k * kThreads + threadIdx.x] = make_double2(0.0, 0.0);

    const int64_t n = jg.n_points;
    const int64_t range_end = jg.p1 > 0 ? min(jg.p1, n) : n;
    const int64_t p_beg = jg.p0 + (int64_t)part * jg.points_per_split;
    const int64_t p_end = min(range_end, p_beg + jg.points_per_split);
    const PointRec* chrec = recs + (int64_t)ch * n;

    for (int64_t cb = p_beg; cb < p_end; cb += kChunk) {
        // ---- classify the chunk's points against this tile (FP64) --------
        int cls[2];
        RsSRec tmp[2];
#pragma unroll
        for (int q = 0; q < 2; ++q) {
            cls[q] = 0;  // 0 skip, 1 fast, 2 exact, 3 fast with the reduced phase
            const int64_t idx = cb + threadIdx.x + q * kThreads;
            const int64_t rel = idx - jg.p0;
            if (idx < p_end && (!left_mask || ((left_mask[rel >> 5] >> (rel & 31)) & 1u))) {
                const PointRec p = chrec[idx];
                const int ix0 = max(X0, p.x_lo), ix1 = min(vx1, p.x_hi);
                const int iy0 = max(Y0, p.y_lo), iy1 = min(vy1, p.y_hi);
                float wxm_t, wym_t;
                if (ix0 < ix1 && iy0 < iy1 && (left_mask || !(jg.tc_skip && rs_tc_eligible(p, tct, &wxm_t, &wym_t)))) {
                    // FP64: only frac(r_c / lambda). sqrt from an FP32 seed
                    // refined by two Newton steps (relative error < 1e-20).
                    const double dxc = Xc - p.x, dyc = Yc - p.y;
                    const double rc2 = fma(dxc, dxc, fma(dyc, dyc, p.aux));
                    const double y0 = (double)rsqrtf((float)rc2);
                    const double hy = 0.5 * y0;
                    double rc = rc2 * y0;
                    rc = fma(hy, fma(-rc, rc, rc2), rc);
                    rc = fma(hy, fma(-rc, rc, rc2), rc);
                    const double tc = rc * g.inv_lambda;
                    const float fc = (float)(tc - rint(tc));
                    // FP32: classification (conservative margins) and the record
                    const float dxf = (float)dxc, dyf = (float)dyc, zzf = (float)p.aux;
                    const float rc2f = (float)rc2, rcf = (float)rc, tcf = (float)tc;
                    const float hf = 1.0f / rc2f;
                    const bool rect_full = p.x_lo <= X0 && p.x_hi >= vx1 && p.y_lo <= Y0 && p.y_hi >= vy1;
                    const float xa = dxf + umin_f, xb = dxf + umax_f;   // X - x over the tile
                    const float ya = dyf + vmin_f, yb = dyf + vmax_f;   // Y - y over the tile
                    const float slack = 1e-6f * (fabsf(dxf) + fabsf(dyf) + uext_f + vext_f);
                    const float maxdx = fmaxf(fabsf(xa), fabsf(xb)) + slack;
                    const float maxdy = fmaxf(fabsf(ya), fabsf(yb)) + slack;
                    const float mindx = fmaxf(((xa <= 0.f && xb >= 0.f) ? 0.f : fminf(fabsf(xa), fabsf(xb))) - slack, 0.f);
                    const float mindy = fmaxf(((ya <= 0.f && yb >= 0.f) ? 0.f : fminf(fabsf(ya), fabsf(yb))) - slack, 0.f);
                    const bool cone_full = maxdx < detx_f * sqrtf(fmaf(mindy, mindy, zzf)) * (1.f - 1e-5f) &&
                                           maxdy < dety_f * sqrtf(fmaf(mindx, mindx, zzf)) * (1.f - 1e-5f);
                    const float nmax = fmaf(2.f * fabsf(dxf), uext_f, uext_f * uext_f) +
                                       fmaf(2.f * fabsf(dyf), vext_f, vext_f * vext_f);
                    const float wmax = nmax * hf;
                    const bool series_ok = wmax < kMaxW && tcf * wmax * wmax * wmax * (1.f / 16.f) < kSeriesTol;
                    const bool turns_ok = tcf * wmax * fmaf(0.125f, wmax, 0.5f) < kMaxTurns;
                    RsSRec& t = tmp[q];
                    t.fc = fc;
                    if (rect_full && cone_full && series_ok) {
                        cls[q] = turns_ok ? 1 : 3;
                        t.whole = 2;   // tells the cls 3 records apart at the back of the chunk
                        t.P = 2.f * dxf * hf;
                        t.Q = 2.f * dyf * hf;
                        t.h = hf;
                        // phase (rad) = 2 pi (fc + (tc/2) w - (tc/8) w^2);
                        // the same in turns for the polynomial pixels
                        t.fc = kTwoPi * fc;
                        t.g = kPi * tcf;
                        t.dxc = -0.25f * kPi * tcf;
                        t.dyc = fc;
                        t.zz = 0.5f * tcf;
                        t.mabs = -0.125f * tcf;
                        t.ac = (float)p.coef * hf;
                    } else {
                        cls[q] = 2;
                        t.P = 2.f * dxf;
                        t.Q = 2.f * dyf;
                        t.h = rc2f;
                        t.g = rcf;
                        t.ac = (float)p.coef;
                        t.dxc = dxf;
                        t.dyc = dyf;
                        t.zz = zzf;
                        t.mabs = 1e-6f * (fabsf(dxf) + fabsf(dyf) + uext_f + vext_f + sqrtf(zzf)) *
                                 (1.f + detx_f + dety_f);
                        t.idx = (int32_t)idx;
                        t.xl = p.x_lo - X0;
                        t.xh = p.x_hi - X0;
                        t.yl = p.y_lo - Y0;
                        t.yh = p.y_hi - Y0;
                        t.whole = rect_full && cone_full ? 1 : 0;
                    }
                }
            }
        }
        // ---- deterministic compaction: FAST from the front, the rest (EXACT,
        // and FAST with the reduced phase) from the back
        unsigned bf[2], be[2];
#pragma unroll
        for (int q = 0; q < 2; ++q) {
            bf[q] = __ballot_sync(0xffffffffu, cls[q] == 1);
            be[q] = __ballot_sync(0xffffffffu, cls[q] >= 2);
            if ((threadIdx.x & 31) == 0) {
                s_cnt[0][q][warp] = __popc(bf[q]);
                s_cnt[1][q][warp] = __popc(be[q]);
            }
        }
        __syncthreads();
        int n_fast = 0, n_back = 0;
        int off_f[2], off_b[2];
#pragma unroll
        for (int q = 0; q < 2; ++q) {
#pragma unroll
            for (int w = 0; w < kThreads / 32; ++w) {
                if (w == warp) {
                    off_f[q] = n_fast;
                    off_b[q] = n_back;
                }
                n_fast += s_cnt[0][q][w];
                n_back += s_cnt[1][q][w];
            }
        }
#pragma unroll
        for (int q = 0; q < 2; ++q) {
            if (cls[q] == 1) s_rec[off_f[q] + warp_prefix(bf[q])] = tmp[q];
            else if (cls[q] >= 2) s_rec[kChunk - 1 - (off_b[q] + warp_prefix(be[q]))] = tmp[q];
        }
        __syncthreads();

        // ---- FAST: whole tile inside the window, series phase --------------
        float sr[kPixH * kPixW], si[kPixH * kPixW];
#pragma unroll
        for (int k = 0; k < kPixH * kPixW; ++k) sr[k] = si[k] = 0.f;
#pragma unroll 1
        for (int j = 0; j < n_fast; ++j) fast_point<false>(s_rec[j], u, uu, v, vv, sr, si);
        // ---- the records at the back (FAST with the reduced phase, EXACT):
        // out of line, uniform over the CTA
        if (n_back > 0) {
            float acc[2 * kPixH * kPixW];
#pragma unroll
            for (int k = 0; k < kPixH * kPixW; ++k) {
                acc[k] = sr[k];
                acc[kPixH * kPixW + k] = si[k];
            }
            reduced_records(s_rec, n_back, g, acc);
            exact_records(s_rec, n_back, g, chrec, X0, Y0, acc);
#pragma unroll
            for (int k = 0; k < kPixH * kPixW; ++k) {
                sr[k] = acc[k];
                si[k] = acc[kPixH * kPixW + k];
            }
        }
#pragma unroll
        for (int k = 0; k < kPixH * kPixW; ++k) {
            double2 a = s_acc[k * kThreads + threadIdx.x];
            a.x += (double)sr[k];
            a.y += (double)si[k];
            s_acc[k * kThreads + threadIdx.x] = a;
        }
        __syncthreads();   // s_rec is rewritten by the next chunk
    }

    // ---- store: (sum a sin, -sum a cos), the reference's (sin, -cos) terms
    double2* dst = (part == 0) ? field
                               : partials + (int64_t)(part - 1) * jg.n_channels * g.pnX * (int64_t)g.pnY;
    dst += (int64_t)ch * g.pnX * (int64_t)g.pnY;
#pragma unroll
    for (int r = 0; r < kPixH; ++r) {
        const int row = Y0 + ty * kPixH + r;
        if (row >= g.pnY) continue;
#pragma unroll
        for (int c = 0; c < kPixW; ++c) {
            const int col = X0 + tx * kPixW + c;
            if (col >= g.pnX) continue;
            const double2 a = s_acc[(r * kPixW + c) * kThreads + threadIdx.x];
            double2* o = dst + (int64_t)row * g.pnX + col;
            if (jg.accumulate && part == 0) {
                const double2 prev = *o;
                *o = make_double2(prev.x + a.x, prev.y - a.y);
            } else {
                *o = make_double2(a.x, -a.y);
            }
        }
    }
}

}  // namespace

constexpr size_t kRsSmem = sizeof(RsSRec) * kChunk + sizeof(double2) * kPixH * kPixW * kThreads;

cudaError_t rs_set_smem_limit() {
    return cudaFuncSetAttribute(rs_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kRsSmem);
}

int rs_blocks_per_sm() {
    rs_set_smem_limit();
    int nb = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, rs_kernel, kThreads, kRsSmem) != cudaSuccess) nb = 1;
    return nb > 0 ? nb : 1;
}

void launch_rs(const PointRec* d_recs, const JobGeom& jg, double2* d_field, double2* d_partials,
               cudaStream_t stream) {
    dim3 grid((unsigned)jg.tiles_x, (unsigned)jg.tiles_y, (unsigned)(jg.n_channels * jg.ksplit));
    count_launches(1);
    rs_kernel<<<grid, kThreads, kRsSmem, stream>>>(d_recs, jg, d_field, d_partials);
}

}  // namespace ophpc
