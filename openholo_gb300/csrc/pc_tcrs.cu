// Tensor-core Rayleigh-Sommerfeld (tcgen05, sm_103a).
//
// The reference's RS sum (ophgen/src/ophGen.cpp:361-445)
//   H(p) = sum_j coef_j / r_pj^2 * (sin(k r_pj), -cos(k r_pj)),  coef = a z / lambda,
// is not separable over the whole SLM, but it is over one 128x128 pixel
// tile. With the tile centre (Xc, Yc), dx = Xc - x_j, dy = Yc - y_j,
// r_c^2 = dx^2 + dy^2 + z^2 and pixel offsets u = X - Xc, v = Y - Yc:
//   r_p^2 = r_c^2 (1 + w_x + w_y),  w_x = (2 dx u + u^2) / r_c^2,  w_y = (2 dy v + v^2) / r_c^2
//   r_p / lambda = tau + tau S(w_x) + tau S(w_y) - tau w_x w_y / 4 + O(tau w^3 cross, tau w^4)
//   S(w) = w/2 - w^2/8 + w^3/16,  tau = r_c / lambda
//   1 / r_p^2 = (1 / r_c^2)(1 - w_x + w_x^2)(1 - w_y + w_y^2) (1 + O(w_x w_y))
// so that, with theta = -(pi/2) tau w_x w_y and e^{i theta} ~ 1 + i theta,
//   coef / r_p^2 e^{i 2 pi r_p / lambda} ~ R_j(v) C_j(u) + [i k_j w_y R_j(v)] [w_x C_j(u) / wxm_j]
//   R_j(v) = (coef / r_c^2) (1 - w_y + w_y^2) e^{i 2 pi (frac(tau) + tau S(w_y))}
//   C_j(u) = (1 - w_x + w_x^2) e^{i 2 pi tau S(w_x)},    k_j = -(pi/2) tau wxm_j
// a complex rank-2 update per point. The tile's field is then the complex
// contraction D = sum_j A_j B_j^T over the points, run on the tensor cores:
//
//   warps 9-11  per (point, tile) records of the next chunk of 256 points
//               (FP64 for frac(tau) only; k r reaches ~6e6 rad) into a
//               double-buffered record ring, off the stage pipeline's
//               critical path;
//   warps 0-7   producers: per stage of 16
//               points threads 0-127 write the row factors A (two rows x 8
//               points each) and threads 128-255 the column factors B
//               into shared memory in the UMMA K-major 32-byte-swizzle
//               layout: split-BF16 (hi + lo) for R and C, FP16 for the cross
//               pair;
//   warp 8      allocates 512 TMEM columns; its lane 0 only issues per stage
//               twelve tcgen05.mma kind::f16, M=128, K=16, three per complex
//               product: Ar x [Br; Bi] (N=256: D_re and D_im at once), then
//               D_re -= Ai Bi (N=128, the instruction's negate-A bit) and
//               D_im += Ai Br (N=128), so that no negated plane is stored;
//               products (hi,hi), (hi,lo), (lo,hi) in BF16 and the cross
//               pair in FP16;
//   warps 0-7   also drain the TMEM accumulator D: every 64 stages (1024
//               points; the tensor core's FP32 accumulation loses ~1e-8 of
//               the sum per point) into a running sum S in the other 256
//               TMEM columns, and every 16 drains into the FP64 field.
//
// A pair whose window rectangle cuts the tile keeps the tile-centre
// expansion and gets 0/1 factor masks from the rectangle (the window is
// separable); the stages holding such a pair run a masked instance of the
// producer loop. Pairs for which the expansion does not hold (the cone test
// is not passed by the tile's pixels inside the rectangle, |w| or the cross
// phase too large: rs_tc_eligible) get zero factors here and are added afterwards by the
// CUDA-core rs_kernel. The record warps mark them in a per-tile bitmask
// (one ballot word per 32 points, each word written by one warp of one
// CTA), which that kernel reads: it evaluates exactly the pairs left here
// and loads no other point.
//
// Every mbarrier wait is bounded (%globaltimer); on a timeout the CTA raises
// an error word, waits (bounded) for its issued MMAs, frees TMEM and returns.
#include "pc_tcrs.cuh"

#include "pc_tcgen05.cuh"

#include <cuda_bf16.h>
#include <cuda_fp16.h>

#include <algorithm>
#include <cmath>
#include <cstring>
#include <type_traits>

namespace ophpc {
namespace {

using namespace tc5;

constexpr int kProdWarps = 8;                            // factor producers (and drains)
constexpr int kProducers = 32 * kProdWarps;              // 256: rows 0-127, then columns 0-127
constexpr int kMmaWarp = kProdWarps;                     // warp 8: TMEM allocation, MMA issue
constexpr int kRecWarps = 3;                             // warps 9-11: point records
constexpr int kRecThreads = 32 * kRecWarps;
constexpr int kThreadsTc = kProducers + 32 + kRecThreads;   // 384: 12 warps, 168 registers each
constexpr int kStagePts = 16;                            // points per stage: one K=16 MMA step
constexpr int kPlane = kRsTcTile * kStagePts * 2;        // 4096 B: 128 rows x 32 B
// Planes of one stage ([Br; Bi] of each B part contiguous: one N=256
// operand). RS (FR false): split-BF16 hi/lo of A and B plus the FP16 cross
// pair A2/B2, 12 planes, 3 stages. Fresnel (FR true): no cross pair, 8
// planes, and the shared memory this frees goes to a fourth stage.
template <bool FR>
struct Lay {
    enum : int {
        Ahr = 0, Ahi = 1, Alr = 2, Ali = 3,
        A2r = FR ? -1 : 4, A2i = FR ? -1 : 5,
        Bhr = FR ? 4 : 6, Bhi = FR ? 5 : 7, Blr = FR ? 6 : 8, Bli = FR ? 7 : 9,
        B2r = FR ? -1 : 10, B2i = FR ? -1 : 11,
        Planes = FR ? 8 : 12,
        Stages = FR ? 4 : 3
    };
    static constexpr int kStageBytes = Planes * kPlane;   // RS 49,152; Fresnel 32,768
};
constexpr int kChunkTc = kProducers;                     // points per record round (one per producer)
constexpr int kStagesPerChunk = kChunkTc / kStagePts;    // 16
constexpr int kPeriod = 64;                              // stages per TMEM accumulation run (1024 points)
constexpr int kFlushPeriods = 16;                        // runs summed in TMEM before an FP64 flush
constexpr int kDCols = 2 * kRsTcTile;                    // accumulator D: re [0,128), im [128,256)
constexpr int kTmemColsTc = 2 * kDCols;                  // D, then the running sum S
constexpr uint64_t kWaitNs = 10ull * 1000 * 1000 * 1000; // 10 s per wait
constexpr float kCrossScale = 64.f;                      // moves the cross pair into FP16's normal range
constexpr float kTwoPiF = 6.283185307179586f;

// Per (point, tile) values, stored for two consecutive points side by side
// so that the factor arithmetic runs on packed FP32 pairs. The column side
// reads the first four pairs only.
struct __align__(16) TcRsPair {
    float2 h, tau, P, bx;   // 1 / rc^2, rc / lambda, 2 dx / rc^2, 1 / (64 wxm)
    float2 Q, fc, ac, k2;   // 2 dy / rc^2, frac(rc / lambda), coef / (rc^2 amax) (0: pair not taken), 64 k
};
static_assert(sizeof(TcRsPair) == 64, "TcRsPair size");

// stages, the record ring, 512 bytes of barriers and flags, and the window
// words of the two record buffers (RS: one uint32 per point)
template <bool FR>
constexpr size_t smem_tc() {
    return 1024 + (size_t)Lay<FR>::Stages * Lay<FR>::kStageBytes + sizeof(TcRsPair) * kChunkTc + 512 +
           sizeof(uint32_t) * 2 * kChunkTc;
}
constexpr size_t kSmemTc = smem_tc<false>();
constexpr size_t kSmemTcFr = smem_tc<true>();
static_assert(kSmemTc <= 232448 && kSmemTcFr <= 232448, "shared memory per CTA");

// Word of the per-job amplitude buffer (after the OPHPC_MAX_CHANNELS
// per-channel bounds) that holds the RS window flag.
constexpr int kWindowWord = 3;
static_assert(OPHPC_MAX_CHANNELS <= kWindowWord, "window flag after the channel bounds");

struct TcRsArgs {
    JobGeom jg;
    const PointRec* recs;   // [n_channels][n_points]
    double2* field;         // [n_channels][pnY][pnX], overwritten
    const float* amax;      // [n_channels]: max coef / z^2; word kWindowWord (RS): window flag (rs_amax_kernel)
    int32_t* left;          // [n_channels][tiles_y][tiles_x]: pairs left to the CUDA cores
    int* error;
    int32_t tiles_x, tiles_y;
    // Points [p_base, p_base + p_count) of the records. The range of every
    // tile is split into ksplit parts of pps points (blockIdx.x = tile
    // column * ksplit + part: the parts of a tile are launched side by side
    // and run at the same time) so that the CTA count fills whole waves;
    // part 0 writes (or, with jg.accumulate, adds into) the field, part k > 0
    // writes partials[k - 1] (same layout). The last part of a tile to finish
    // (tickets[tile], zeroed by the caller) adds the partial tiles into the
    // field in part order and discards their lines from L2, so that the
    // partials, read while still in L2, are never written back to DRAM.
    int64_t p_base, p_count;
    int32_t ksplit;
    int64_t pps;            // a multiple of kChunkTc
    double2* partials;
    int32_t* tickets;       // [n_channels][tiles_y][tiles_x], when ksplit > 1
    // per tile, one bit per point of [p_base, p_base + p_count) for the
    // pairs left to the CUDA cores (word (i - p_base) / 32); mask_words words a tile
    uint32_t* mask;
    int64_t mask_words;
};

__device__ __forceinline__ void fence_async_smem() { asm volatile("fence.proxy.async.shared::cta;" ::: "memory"); }
__device__ __forceinline__ void st_v4(uint32_t addr, uint32_t w0, uint32_t w1, uint32_t w2, uint32_t w3) {
    asm volatile("st.shared.v4.b32 [%0], {%1, %2, %3, %4};" ::"r"(addr), "r"(w0), "r"(w1), "r"(w2), "r"(w3)
                 : "memory");
}
__device__ __forceinline__ uint32_t bf2(float lo, float hi) {
    const __nv_bfloat162 v = __floats2bfloat162_rn(lo, hi);
    return *reinterpret_cast<const uint32_t*>(&v);
}
__device__ __forceinline__ uint32_t h2(float lo, float hi) {
    const __half2 v = __floats2half2_rn(lo, hi);
    return *reinterpret_cast<const uint32_t*>(&v);
}

// bf16 pair (low half = first) -> packed FP32 pair
__device__ __forceinline__ f2::v2 bf2_to_v2(uint32_t w) {
    return f2::pack(__uint_as_float(w << 16), __uint_as_float(w & 0xffff0000u));
}
__device__ __forceinline__ uint32_t bf2v(f2::v2 v) {
    float a, b;
    f2::unpack(v, a, b);
    return bf2(a, b);
}
__device__ __forceinline__ uint32_t h2v(f2::v2 v) {
    float a, b;
    f2::unpack(v, a, b);
    return h2(a, b);
}

// 1.0 where tile-relative index i lies in [lo, hi) held in bytes `sh` (lo)
// and `sh + 8` (hi) of a window word (xlo, xhi, ylo, yhi), else 0.
__device__ __forceinline__ float in_window_u(uint32_t w, int sh, int i) {
    const int lo = (int)((w >> sh) & 0xffu), hi = (int)((w >> (sh + 8)) & 0xffu);
    return (i >= lo && i < hi) ? 1.f : 0.f;
}

// Factors of 8 points of a stage (4 record pairs: one 16-byte chunk of a
// row of every plane) for two rows (SIDE_A) or columns of this thread, at
// offsets offa and offb, written at ro0 and ro1. A lane pair covers the two
// chunks of a row, so that one st.shared.v4 of a warp fills 16 whole rows.
// Two points at a time in packed FP32 pairs. CUT: the 8 points' window words
// (wins) turn into 0/1 masks of the thread's rows (columns) ia and ib.
template <bool SIDE_A, bool CUT>
__device__ __forceinline__ void produce_stage(const TcRsPair* prs, float offa, float offb, uint32_t ro0, uint32_t ro1,
                                              const uint32_t* wins, int ia, int ib) {
    using f2::v2;
    const v2 offpa = f2::splat(offa), off2pa = f2::splat(offa * offa);
    const v2 offpb = f2::splat(offb), off2pb = f2::splat(offb * offb);
    const v2 c16 = f2::splat(0.0625f), c8 = f2::splat(-0.125f), c2 = f2::splat(0.5f), one = f2::splat(1.f);
    const v2 two_pi = f2::splat(kTwoPiF);
    uint32_t w_hr[8], w_hi[8], w_lr[8], w_li[8], w_xr[8], w_xi[8];
#pragma unroll
    for (int qq = 0; qq < 8; ++qq) {
        const int q = (qq & 1) * 4 + (qq >> 1);   // output slot: row (qq & 1), pair qq >> 1
        const v2 offp = (qq & 1) ? offpb : offpa, off2p = (qq & 1) ? off2pb : off2pa;
        const ulonglong2* R = reinterpret_cast<const ulonglong2*>(&prs[qq >> 1]);
        const ulonglong2 r0 = R[0];   // h, tau
        const ulonglong2 r1 = R[1];   // P, bx
        v2 w, ph;
        ulonglong2 r2, r3;
        if (SIDE_A) {
            r2 = R[2];   // Q, fc
            r3 = R[3];   // ac, k2
            w = f2::fma(r2.x, offp, f2::mul(r0.x, off2p));
        } else {
            w = f2::fma(r1.x, offp, f2::mul(r0.x, off2p));
        }
        const v2 s3 = f2::fma(w, f2::fma(w, c16, c8), c2);   // S(w) / w
        if (SIDE_A) ph = f2::fma(f2::mul(r0.y, w), s3, r2.y);   // turns
        else ph = f2::mul(f2::mul(r0.y, w), s3);
        // radians straight into the MUFU sin/cos (|ph| <= ~25 turns here):
        // its own range reduction keeps the error at the FP32 rounding of
        // the phase in turns; reducing first measured no better (relL2 vs
        // FP64 1.03e-5 with, 1.04e-5 without, sphere_fhd)
        ph = f2::mul(ph, two_pi);
        float p0, p1, s0, c0, s1, c1;
        f2::unpack(ph, p0, p1);
        __sincosf(p0, &s0, &c0);
        __sincosf(p1, &s1, &c1);
        v2 amp = f2::fma(w, w, f2::sub(one, w));
        if (SIDE_A) amp = f2::mul(amp, r3.x);
        if (CUT) {
            // zero outside the window rectangle: rows by (ylo, yhi), columns by (xlo, xhi)
            const int idx = (qq & 1) ? ib : ia, sh = SIDE_A ? 16 : 0;
            const uint2 wp = reinterpret_cast<const uint2*>(wins)[qq >> 1];   // the pair's two window words
            amp = f2::mul(amp, f2::pack(in_window_u(wp.x, sh, idx), in_window_u(wp.y, sh, idx)));
        }
        const v2 vr = f2::mul(amp, f2::pack(c0, c1)), vi = f2::mul(amp, f2::pack(s0, s1));
        w_hr[q] = bf2v(vr);
        w_hi[q] = bf2v(vi);
        w_lr[q] = bf2v(f2::sub(vr, bf2_to_v2(w_hr[q])));
        w_li[q] = bf2v(f2::sub(vi, bf2_to_v2(w_hi[q])));
        if (SIDE_A) {
            const v2 kw = f2::mul(r3.y, w);   // i k w_y R = (-kw vi, kw vr)
            w_xr[q] = h2v(f2::mul(kw, vi)) ^ 0x80008000u;
            w_xi[q] = h2v(f2::mul(kw, vr));
        } else {
            const v2 sc = f2::mul(w, r1.y);   // w_x C / (64 wxm)
            w_xr[q] = h2v(f2::mul(sc, vr));
            w_xi[q] = h2v(f2::mul(sc, vi));
        }
    }
#pragma unroll
    for (int h = 0; h < 2; ++h) {
        const uint32_t ro = h ? ro1 : ro0;
        const int o = 4 * h;
#define ST(plane, w) st_v4(ro + (plane) * kPlane, w[o], w[o + 1], w[o + 2], w[o + 3])
        using L = Lay<false>;
        if (SIDE_A) {
            ST(L::Ahr, w_hr);
            ST(L::Ahi, w_hi);
            ST(L::Alr, w_lr);
            ST(L::Ali, w_li);
            ST(L::A2r, w_xr);
            ST(L::A2i, w_xi);
        } else {
            ST(L::Bhr, w_hr);
            ST(L::Bhi, w_hi);
            ST(L::Blr, w_lr);
            ST(L::Bli, w_li);
            ST(L::B2r, w_xr);
            ST(L::B2i, w_xi);
        }
#undef ST
    }
}

// 1.0 where tile-relative index i lies in the window [lo, hi) held in
// bytes `sh` (lo) and `sh + 8` (hi) of the packed window word, else 0.
__device__ __forceinline__ float in_window(float packed, int sh, int i) {
    return in_window_u(__float_as_uint(packed), sh, i);
}

// Fresnel factors of 8 points of a stage for two rows (SIDE_A) or columns,
// the Fresnel counterpart of produce_stage: the phase splits exactly into
// a row part and a column part, so there is no series and no cross pair.
// CUT: some point of the stage has a window that cuts the tile; then the
// window rectangle becomes 0/1 factor masks (ia, ib: tile-relative indices
// of the thread's two rows/columns) and each point's expansion centre
// (u0, v0: offset from the tile centre) lies inside its window, so that the
// factor phases stay within the window's chirp (<= 64 turns) however far the
// point lies from the tile centre. Otherwise u0 = v0 = 0 and every mask is 1.
template <bool SIDE_A, bool CUT>
__device__ __forceinline__ void produce_stage_fr(const TcRsPair* prs, float offa, float offb, int ia, int ib,
                                                 uint32_t ro0, uint32_t ro1) {
    using f2::v2;
    const v2 offpa = f2::splat(offa), off2pa = f2::splat(offa * offa);
    const v2 offpb = f2::splat(offb), off2pb = f2::splat(offb * offb);
    const v2 two_pi = f2::splat(kTwoPiF);
    uint32_t w_hr[8], w_hi[8], w_lr[8], w_li[8];
#pragma unroll
    for (int qq = 0; qq < 8; ++qq) {
        const int q = (qq & 1) * 4 + (qq >> 1);   // output slot: row (qq & 1), pair qq >> 1
        const v2 offp = (qq & 1) ? offpb : offpa;
        const ulonglong2* R = reinterpret_cast<const ulonglong2*>(&prs[qq >> 1]);
        const ulonglong2 r0 = R[0];   // h, P
        v2 d, d2;
        ulonglong2 r1;
        if (CUT) {
            r1 = R[1];   // u0, window
        }
        if (SIDE_A) {
            const ulonglong2 r2 = R[2];   // Q, v0
            const ulonglong2 r3 = R[3];   // fc, ac
            if (CUT) {
                d = f2::sub(offp, r2.y);
                d2 = f2::mul(d, d);
            } else {
                d = offp;
                d2 = (qq & 1) ? off2pb : off2pa;
            }
            v2 ph = f2::fma(r2.x, d, f2::fma(r0.x, d2, r3.x));   // turns
            v2 amp = r3.y;
            if (CUT) {
                float wa, wb;
                f2::unpack(r1.y, wa, wb);
                const int idx = (qq & 1) ? ib : ia;
                amp = f2::mul(amp, f2::pack(in_window(wa, 16, idx), in_window(wb, 16, idx)));
            }
            ph = f2::mul(ph, two_pi);
            float p0, p1, s0, c0, s1, c1;
            f2::unpack(ph, p0, p1);
            __sincosf(p0, &s0, &c0);
            __sincosf(p1, &s1, &c1);
            const v2 vr = f2::mul(amp, f2::pack(c0, c1)), vi = f2::mul(amp, f2::pack(s0, s1));
            w_hr[q] = bf2v(vr);
            w_hi[q] = bf2v(vi);
            w_lr[q] = bf2v(f2::sub(vr, bf2_to_v2(w_hr[q])));
            w_li[q] = bf2v(f2::sub(vi, bf2_to_v2(w_hi[q])));
        } else {
            if (CUT) {
                d = f2::sub(offp, r1.x);
                d2 = f2::mul(d, d);
            } else {
                d = offp;
                d2 = (qq & 1) ? off2pb : off2pa;
            }
            v2 ph = f2::fma(r0.y, d, f2::mul(r0.x, d2));
            ph = f2::mul(ph, two_pi);
            float p0, p1, s0, c0, s1, c1;
            f2::unpack(ph, p0, p1);
            __sincosf(p0, &s0, &c0);
            __sincosf(p1, &s1, &c1);
            v2 vr = f2::pack(c0, c1), vi = f2::pack(s0, s1);
            if (CUT) {
                float wa, wb;
                f2::unpack(r1.y, wa, wb);
                const int idx = (qq & 1) ? ib : ia;
                const v2 m = f2::pack(in_window(wa, 0, idx), in_window(wb, 0, idx));
                vr = f2::mul(vr, m);
                vi = f2::mul(vi, m);
            }
            w_hr[q] = bf2v(vr);
            w_hi[q] = bf2v(vi);
            w_lr[q] = bf2v(f2::sub(vr, bf2_to_v2(w_hr[q])));
            w_li[q] = bf2v(f2::sub(vi, bf2_to_v2(w_hi[q])));
        }
    }
#pragma unroll
    for (int h = 0; h < 2; ++h) {
        const uint32_t ro = h ? ro1 : ro0;
        const int o = 4 * h;
        using L = Lay<true>;
#define ST(plane, w) st_v4(ro + (plane) * kPlane, w[o], w[o + 1], w[o + 2], w[o + 3])
        if (SIDE_A) {
            ST(L::Ahr, w_hr);
            ST(L::Ahi, w_hi);
            ST(L::Alr, w_lr);
            ST(L::Ali, w_li);
        } else {
            ST(L::Bhr, w_hr);
            ST(L::Bhi, w_hi);
            ST(L::Blr, w_lr);
            ST(L::Bli, w_li);
        }
#undef ST
    }
}

// Issues the twelve MMAs of stage k (the MMA warp's lane 0): waits until the
// producers filled the stage and, when k opens an accumulation run, until
// every producer warp drained the previous run out of D. Issuing blocks
// while the tensor core's queue is full (about as long as a stage's MMAs
// take), which is why a warp of its own does it. False on abort.
template <bool FR>
__device__ __forceinline__ bool issue_stage(int k, int total, unsigned char* base, uint64_t* full, uint64_t* empty,
                                            uint64_t* acc_full, uint64_t* acc_empty, volatile int* abort,
                                            uint32_t tmem) {
    using L = Lay<FR>;
    constexpr uint32_t id_bf256 = idesc_f16(1u, false, kRsTcTile, 2 * kRsTcTile);   // BF16, N=256
    constexpr uint32_t id_bf = idesc_f16(1u, false, kRsTcTile, kRsTcTile);          // BF16, N=128
    constexpr uint32_t id_bfn = idesc_f16(1u, true, kRsTcTile, kRsTcTile);          // BF16, N=128, -A
    constexpr uint32_t id_h256 = idesc_f16(0u, false, kRsTcTile, 2 * kRsTcTile);    // FP16, ...
    constexpr uint32_t id_h = idesc_f16(0u, false, kRsTcTile, kRsTcTile);
    constexpr uint32_t id_hn = idesc_f16(0u, true, kRsTcTile, kRsTcTile);
    const int p = k / kPeriod;
    const bool opens = (k % kPeriod) == 0;
    if (opens && p >= 1 && !mbar_wait_for(acc_empty, (uint32_t)(p - 1) & 1u, abort, kWaitNs)) return false;
    const int s = k % L::Stages;
    if (!mbar_wait_for(&full[s], (uint32_t)(k / L::Stages) & 1u, abort, kWaitNs)) return false;
    tc_fence_after();
    const uint32_t d = tmem;
    const uint32_t st = smem_u32(base + s * L::kStageBytes);
#define PL(x) sw32_desc(st + (uint32_t)((x) * kPlane))
    const uint32_t dre = d, dim = d + kRsTcTile, acc = opens ? 0u : 1u;
    umma(d, PL(L::Ahr), PL(L::Bhr), id_bf256, acc);   // re += Ar Br, im += Ar Bi
    umma(dre, PL(L::Ahi), PL(L::Bhi), id_bfn, 1u);    // re -= Ai Bi
    umma(dim, PL(L::Ahi), PL(L::Bhr), id_bf, 1u);     // im += Ai Br
    umma(d, PL(L::Ahr), PL(L::Blr), id_bf256, 1u);
    umma(dre, PL(L::Ahi), PL(L::Bli), id_bfn, 1u);
    umma(dim, PL(L::Ahi), PL(L::Blr), id_bf, 1u);
    umma(d, PL(L::Alr), PL(L::Bhr), id_bf256, 1u);
    umma(dre, PL(L::Ali), PL(L::Bhi), id_bfn, 1u);
    umma(dim, PL(L::Ali), PL(L::Bhr), id_bf, 1u);
    if constexpr (!FR) {
        umma(d, PL(L::A2r), PL(L::B2r), id_h256, 1u);
        umma(dre, PL(L::A2i), PL(L::B2i), id_hn, 1u);
        umma(dim, PL(L::A2i), PL(L::B2r), id_h, 1u);
    }
#undef PL
    umma_commit(&empty[s]);   // frees the stage once these MMAs have read it
    if ((k % kPeriod) == kPeriod - 1 || k == total - 1) umma_commit(acc_full);
    return true;
}

// Drains run p out of D (warp-collective, every producer warp): this warp's
// 32 TMEM lanes x (64 columns of D_re + the 64 of D_im) are added into the running
// sum S (or replace it when S was just flushed); on a flush run the sum goes
// into the FP64 field instead. False when the CTA is aborting.
__device__ __forceinline__ bool drain_run(int p, int periods, uint64_t* acc_full, uint64_t* acc_empty,
                                          volatile int* abort, uint32_t tmem, int warp, int lane,
                                          const TcRsArgs& a, int ch, double2* out, int X0, int Y0, float amax,
                                          bool& wrote) {
    bool ok = true;
    if (lane == 0) ok = mbar_wait_for(acc_full, (uint32_t)p & 1u, abort, kWaitNs) && !*abort;
    ok = __shfl_sync(0xffffffffu, ok, 0);
    tc_fence_after();
    if (!ok) return false;
    const bool fresh = (p % kFlushPeriods) == 0;                      // S holds nothing yet
    const bool flush = (p % kFlushPeriods) == kFlushPeriods - 1 || p == periods - 1;
    const int grp = warp & 3, half = warp >> 2;
    const uint32_t lanes = (uint32_t)(grp * 32) << 16;
    const ChannelGeom& g = a.jg.ch[ch];
    const int row = Y0 + grp * 32 + lane;
#pragma unroll 1
    for (int k = 0; k < 4; ++k) {
        const uint32_t cre = (uint32_t)(half * 64 + k * 16), cim = cre + kRsTcTile;
        uint32_t dr[16], di[16], sr[16], si[16];
        tmem_ld16(tmem + lanes + cre, dr);
        tmem_ld16(tmem + lanes + cim, di);
        if (!fresh) {
            tmem_ld16(tmem + lanes + kDCols + cre, sr);
            tmem_ld16(tmem + lanes + kDCols + cim, si);
        }
        tmem_wait_ld();
        float vr[16], vi[16];
#pragma unroll
        for (int i = 0; i < 16; ++i) {
            vr[i] = __uint_as_float(dr[i]) + (fresh ? 0.f : __uint_as_float(sr[i]));
            vi[i] = __uint_as_float(di[i]) + (fresh ? 0.f : __uint_as_float(si[i]));
        }
        if (flush) {
            // field (+)= amax * (-i) (vr + i vi)
            if (row < g.pnY) {
                double2* dst = out + ((int64_t)ch * g.pnY + row) * g.pnX;
#pragma unroll
                for (int i = 0; i < 16; ++i) {
                    const int col = X0 + (int)cre + i;
                    if (col < g.pnX) {
                        const double re = (double)vi[i] * (double)amax, im = -(double)vr[i] * (double)amax;
                        if (wrote) {
                            const double2 o = dst[col];
                            dst[col] = make_double2(o.x + re, o.y + im);
                        } else {
                            dst[col] = make_double2(re, im);
                        }
                    }
                }
            }
        } else {
#pragma unroll
            for (int i = 0; i < 16; ++i) {
                sr[i] = __float_as_uint(vr[i]);
                si[i] = __float_as_uint(vi[i]);
            }
            tmem_st16(tmem + lanes + kDCols + cre, sr);
            tmem_st16(tmem + lanes + kDCols + cim, si);
        }
    }
    if (flush) wrote = true;
    tmem_wait_st();
    tc_fence_before();
    __syncwarp();
    if (lane == 0) mbar_arrive(acc_empty);
    return true;
}

// Per (point, tile) values of point idx into record pair slot t of buf
// (zeros when the pair is not taken). True (and counted in left) for a pair
// left to the CUDA cores: the window overlaps the tile, the expansion does
// not hold. For a pair taken while its window rectangle cuts the tile, cut
// is set and win holds the rectangle relative to the tile (bytes xlo, xhi,
// ylo, yhi; the whole tile otherwise).
__device__ __forceinline__ bool make_record(TcRsPair* buf, int t, bool valid, const PointRec& p,
                                            const RsTcTile& tile, double inv_lambda, float inv_amax, int X0, int Y0,
                                            int& left, bool& cut, uint32_t& win) {
    bool is_left = false;
    cut = false;
    win = (uint32_t)kRsTcTile << 8 | (uint32_t)kRsTcTile << 24;
    float h = 0.f, tau = 0.f, P = 0.f, bx = 0.f, Q = 0.f, fc = 0.f, ac = 0.f, k2 = 0.f;
    if (valid) {
        const int ix0 = max(X0, p.x_lo), ix1 = min(tile.vx1, p.x_hi);
        const int iy0 = max(Y0, p.y_lo), iy1 = min(tile.vy1, p.y_hi);
        float wxm, wym;
        if (ix0 < ix1 && iy0 < iy1) {
            if (rs_tc_eligible(p, tile, &wxm, &wym)) {
                // FP64: frac(r_c / lambda) only. sqrt from an FP32 seed
                // refined by one Newton step (relative error ~1e-14: 1e-8
                // turns at tau ~1e6).
                const double dxc = tile.Xc - p.x, dyc = tile.Yc - p.y;
                const double rc2 = fma(dxc, dxc, fma(dyc, dyc, p.aux));
                const double y0 = (double)rsqrtf((float)rc2);
                const double hy = 0.5 * y0;
                double rcd = rc2 * y0;
                rcd = fma(hy, fma(-rcd, rcd, rc2), rcd);
                const double tc = rcd * inv_lambda;
                const float hf = 1.0f / (float)rc2;
                h = hf;
                tau = (float)tc;
                P = 2.f * (float)dxc * hf;
                bx = 1.f / (wxm * kCrossScale);
                Q = 2.f * (float)dyc * hf;
                fc = (float)(tc - rint(tc));
                ac = (float)p.coef * hf * inv_amax;
                k2 = -1.5707963267948966f * tau * wxm * kCrossScale;
                cut = !(ix0 == X0 && ix1 == tile.vx1 && iy0 == Y0 && iy1 == tile.vy1);
                win = (uint32_t)(ix0 - X0) | ((uint32_t)(ix1 - X0) << 8) | ((uint32_t)(iy0 - Y0) << 16) |
                      ((uint32_t)(iy1 - Y0) << 24);
            } else {
                ++left;
                is_left = true;
            }
        }
    }
    float* f = reinterpret_cast<float*>(&buf[t >> 1]) + (t & 1);
    f[0] = h;
    f[2] = tau;
    f[4] = P;
    f[6] = bx;
    f[8] = Q;
    f[10] = fc;
    f[12] = ac;
    f[14] = k2;
    return is_left;
}

// Fresnel values of point idx on the tile into record pair slot t of buf
// (ophgen/src/ophGen.cpp:447-514): with s = 1/(2 z lambda) and an expansion
// centre (Xe, Ye) = tile centre + (u0, v0), dx0 = Xe - x, dy0 = Ye - y,
//   phase (turns) = frac(s (dx0^2 + dy0^2) + z / lambda)      [FP64, ~1e6 turns]
//                 + s (2 dy0 e + e^2) + s (2 dx0 d + d^2),     e = v - v0, d = u - u0
// exactly. h = s, P = 2 dx0 s, Q = 2 dy0 s and the amplitude coef / amax
// (0 when the window misses the tile). The window rectangle, relative to the
// tile's first column and row, is packed in bytes (xlo, xhi, ylo, yhi). When
// the window holds the whole tile the centre is the tile centre (u0 = v0 =
// 0); otherwise it is the tile centre clamped into the window. Returns true
// for a point whose window cuts the tile (masks needed).
__device__ __forceinline__ bool make_record_fr(TcRsPair* buf, int t, bool valid, const PointRec& p,
                                               const RsTcTile& tile, double inv_lambda, float inv_amax,
                                               const ChannelGeom& g, int X0, int Y0) {
    float h = 0.f, P = 0.f, u0 = 0.f, win = 0.f, Q = 0.f, v0 = 0.f, fc = 0.f, ac = 0.f;
    bool cut = false;
    if (valid) {
        const int ix0 = max(X0, p.x_lo), ix1 = min(tile.vx1, p.x_hi);
        const int iy0 = max(Y0, p.y_lo), iy1 = min(tile.vy1, p.y_hi);
        if (ix0 < ix1 && iy0 < iy1) {
            const int xlo = ix0 - X0, xhi = ix1 - X0, ylo = iy0 - Y0, yhi = iy1 - Y0;
            const bool cut_x = !(ix0 == X0 && ix1 == tile.vx1), cut_y = !(iy0 == Y0 && iy1 == tile.vy1);
            cut = cut_x || cut_y;
            const int c0 = cut_x ? min(max(kRsTcHalf, xlo), xhi - 1) : kRsTcHalf;
            const int r0 = cut_y ? min(max(kRsTcHalf, ylo), yhi - 1) : kRsTcHalf;
            const double du0 = (double)(c0 - kRsTcHalf) * g.ppX, dv0 = (double)(kRsTcHalf - r0) * g.ppY;
            const double dxc = (tile.Xc - p.x) + du0, dyc = (tile.Yc - p.y) + dv0;
            const double sq = p.aux;   // 1 / (2 z lambda)
            const double tc = sq * (dxc * dxc + dyc * dyc) + p.z * inv_lambda;
            h = (float)sq;
            P = (float)(2.0 * dxc * sq);
            Q = (float)(2.0 * dyc * sq);
            u0 = (float)du0;
            v0 = (float)dv0;
            fc = (float)(tc - rint(tc));
            ac = (float)p.coef * inv_amax;
            win = __uint_as_float((uint32_t)xlo | ((uint32_t)xhi << 8) | ((uint32_t)ylo << 16) |
                                  ((uint32_t)yhi << 24));
        }
    }
    float* f = reinterpret_cast<float*>(&buf[t >> 1]) + (t & 1);
    f[0] = h;
    f[2] = P;
    f[4] = u0;
    f[6] = win;
    f[8] = Q;
    f[10] = v0;
    f[12] = fc;
    f[14] = ac;
    return cut;
}

// One CTA per 128x128 tile of one channel. Warps 0-7 produce the factors
// (threads 0-127 the rows, 128-255 the columns: two rows or columns and 8
// points of a stage each) and drain the accumulator; warp 8 allocates TMEM and its lane 0
// issues the MMAs; warps 9-11 form the point records of the chunks, one
// chunk ahead of the producers (double-buffered, an mbarrier pair per buffer).
// Called by every part of a tile once its own writes are done: the last
// part to arrive adds the partial tiles into the field (field + partials[0]
// + ... in that order, whoever arrives last, so the result is
// deterministic) and discards the partials' 128-byte lines that lie wholly
// inside the tile from L2 (nothing reads them again). s_flag: one word of
// shared memory.
__device__ __noinline__ void sum_parts(const TcRsArgs& a, int ch, int tx, int X0, int Y0, int* s_flag) {
    const ChannelGeom& g = a.jg.ch[0];
    const int64_t plane = (int64_t)g.pnX * g.pnY;
    const int64_t field_elems = plane * a.jg.n_channels;
    __syncthreads();   // every thread of this part has written its share
    if (threadIdx.x == 0) {
        __threadfence();   // release this part's writes before taking a ticket
        const int t = atomicAdd(&a.tickets[((int64_t)ch * a.tiles_y + blockIdx.y) * a.tiles_x + tx], 1);
        *s_flag = (t == a.ksplit - 1);
        if (*s_flag) __threadfence();   // acquire the other parts' writes
    }
    __syncthreads();
    if (!*s_flag) return;
    const int cols = min(kRsTcTile, g.pnX - X0), rows = min(kRsTcTile, g.pnY - Y0);
    double2* field = a.field + (int64_t)ch * plane;
    for (int i = threadIdx.x; i < rows * cols; i += blockDim.x) {
        const int r = i / cols, c = i - r * cols;
        const int64_t o = (int64_t)(Y0 + r) * g.pnX + X0 + c;
        double2 v = __ldcg(&field[o]);   // written by part 0, possibly on another SM
        for (int k = 1; k < a.ksplit; ++k) {
            const double2 p = __ldcg(&a.partials[(int64_t)(k - 1) * field_elems + (int64_t)ch * plane + o]);
            v.x += p.x;
            v.y += p.y;
        }
        field[o] = v;
    }
    __syncthreads();
    // 128-byte lines of the partial rows that lie wholly inside the tile
    const int lines_per_row = kRsTcTile * (int)sizeof(double2) / 128 + 1;
    for (int k = 1; k < a.ksplit; ++k) {
        const char* base =
            reinterpret_cast<const char*>(a.partials + (int64_t)(k - 1) * field_elems + (int64_t)ch * plane);
        for (int i = threadIdx.x; i < rows * lines_per_row; i += blockDim.x) {
            const int r = i / lines_per_row, l = i - r * lines_per_row;
            const uintptr_t b0 = (uintptr_t)(base + ((int64_t)(Y0 + r) * g.pnX + X0) * (int64_t)sizeof(double2));
            const uintptr_t b1 = b0 + (uintptr_t)cols * sizeof(double2);
            const uintptr_t line = ((b0 + 127) & ~(uintptr_t)127) + (uintptr_t)l * 128;
            if (line + 128 <= b1) asm volatile("discard.global.L2 [%0], 128;" ::"l"(line) : "memory");
        }
    }
}

// FR: Fresnel, else RS. MASKS (RS): some point's window rectangle may cut a
// tile, so the producers run the masked loop instance for the chunks that
// hold such a pair; without it the kernel carries no mask code at all.
template <bool FR, bool MASKS>
__device__ __forceinline__ void tile_body(const TcRsArgs& a) {
    using L = Lay<FR>;
    extern __shared__ __align__(1024) unsigned char smem_raw[];
    unsigned char* base = (unsigned char*)(((uintptr_t)smem_raw + 1023) & ~(uintptr_t)1023);
    TcRsPair* s_rec = reinterpret_cast<TcRsPair*>(base + L::Stages * L::kStageBytes);   // [2][kChunkTc / 2]
    uint64_t* full = reinterpret_cast<uint64_t*>(s_rec + kChunkTc);
    uint64_t* empty = full + L::Stages;
    uint64_t* acc_full = empty + L::Stages;   // MMA -> drains: D holds a finished run
    uint64_t* acc_empty = acc_full + 1;       // drains -> MMA: D was read
    uint64_t* drain_bar = acc_empty + 1;      // abort path: issued MMAs complete
    uint64_t* rec_full = drain_bar + 1;       // [2] record warps -> producers: a chunk's records are formed
    uint64_t* rec_empty = rec_full + 2;       // [2] producers -> record warps: a chunk's records were read
    uint32_t* tmem_slot = reinterpret_cast<uint32_t*>(rec_empty + 2);
    volatile int* abort = reinterpret_cast<volatile int*>(tmem_slot + 1);
    int* s_left = reinterpret_cast<int*>(tmem_slot + 2);
    // per record buffer, one word per stage: nonzero when a point of the
    // stage has a window that cuts the tile (factor masks needed), at byte
    // 256 of the 512-byte tail (16-byte aligned for uint4 reads; the
    // barriers and words above end before byte 136)
    uint32_t* s_cut = reinterpret_cast<uint32_t*>(reinterpret_cast<unsigned char*>(full) + 256);   // [2][16]
    // RS: the window words of the points of the two record buffers
    uint32_t* s_win = reinterpret_cast<uint32_t*>(reinterpret_cast<unsigned char*>(full) + 512);   // [2][kChunkTc]

    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int ch = blockIdx.z, part = blockIdx.x % a.ksplit, tx = blockIdx.x / a.ksplit;
    const ChannelGeom& g = a.jg.ch[ch];
    const int X0 = tx * kRsTcTile, Y0 = blockIdx.y * kRsTcTile;
    const int64_t p_beg = a.p_base + (int64_t)part * a.pps;
    const int64_t n = min(a.p_base + a.p_count, p_beg + a.pps) - p_beg;   // this CTA's points: [p_beg, p_beg + n)
    double2* out = part == 0 ? a.field
                             : a.partials + (int64_t)(part - 1) * a.jg.n_channels * a.jg.ch[0].pnX * a.jg.ch[0].pnY;
    const int total = (int)((n + kStagePts - 1) / kStagePts);
    const int nchunks = (int)((n + kChunkTc - 1) / kChunkTc);
    const int periods = (total + kPeriod - 1) / kPeriod;

    if (threadIdx.x == 0) {
        for (int s = 0; s < L::Stages; ++s) {
            mbar_init(&full[s], kProdWarps);
            mbar_init(&empty[s], 1);
        }
        mbar_init(acc_full, 1);
        mbar_init(acc_empty, kProdWarps);
        mbar_init(drain_bar, 1);
        for (int b = 0; b < 2; ++b) {
            mbar_init(&rec_full[b], kRecWarps);
            mbar_init(&rec_empty[b], kProdWarps);
        }
        *abort = 0;
        *s_left = 0;
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    if (warp == kMmaWarp) tmem_alloc(tmem_slot, kTmemColsTc);

    const int t = threadIdx.x;
    const bool side_a = t < kRsTcTile;         // rows (A) or columns (B)
    // rows (columns) rc and rc + 64 of the tile, points 8 kc .. 8 kc + 7 of every stage
    const int rc = (t & (kRsTcTile - 1)) >> 1, kc = t & 1;
    const float off = side_a ? (float)((double)(kRsTcHalf - rc) * g.ppY) : (float)((double)(rc - kRsTcHalf) * g.ppX);
    const float offb = side_a ? (float)((double)(kRsTcHalf - rc - 64) * g.ppY)
                              : (float)((double)(rc + 64 - kRsTcHalf) * g.ppX);
    // 32-byte swizzle: rows 4-7 of every 8 swap their two 16-byte halves
    // (rows rc and rc + 64 alike)
    const uint32_t swz = (uint32_t)((rc >> 2) & 1);
    const uint32_t row_off0 = (uint32_t)rc * 32u + (((uint32_t)kc ^ swz) << 4), row_off1 = row_off0 + 64u * 32u;
    const RsTcTile tile = rs_tc_tile(g, X0, Y0);
    const float amax = a.amax[ch];
    const float inv_amax = amax > 0.f ? 1.f / amax : 0.f;
    const PointRec* chrec = a.recs + (int64_t)ch * a.jg.n_points + p_beg;
    bool dead = false;
    bool wrote = part == 0 && a.jg.accumulate != 0;
    int left = 0, drained = 0, issued = 0;

    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    const uint32_t tmem = *tmem_slot;

    if (warp == kMmaWarp) {
        if (lane == 0) {
            for (; issued < total; ++issued)
                if (!issue_stage<FR>(issued, total, base, full, empty, acc_full, acc_empty, abort, tmem)) break;
            if (issued < total && issued > 0) {
                // aborted: wait (bounded) for the MMAs already issued before TMEM is released
                umma_commit(drain_bar);
                const uint64_t dl = global_ns() + 1000ull * 1000 * 1000;
                while (!mbar_try_wait(drain_bar, 0) && global_ns() < dl) {
                }
            }
        }
    } else if (warp > kMmaWarp) {
        // records of chunk c into buffer c & 1, once the producers released
        // the chunk that used it before (c - 2)
        const int rt = t - (kProducers + 32);
        const int64_t mask_base = (((int64_t)ch * a.tiles_y + blockIdx.y) * a.tiles_x + tx) * a.mask_words;
        for (int c = 0; c < nchunks && !dead; ++c) {
            const int b = c & 1;
            if (c >= 2) {
                const bool ok = mbar_wait_for(&rec_empty[b], (uint32_t)((c >> 1) - 1) & 1u, abort, kWaitNs);
                dead = !__all_sync(0xffffffffu, ok);
                if (dead) break;
            }
            TcRsPair* buf = s_rec + b * (kChunkTc / 2);
            for (int j = rt; j < kChunkTc; j += kRecThreads) {
                const int64_t idx = (int64_t)c * kChunkTc + j;
                const bool valid = idx < n;
                if constexpr (FR) {
                    const bool cut = make_record_fr(buf, j, valid, chrec[valid ? idx : 0], tile, g.inv_lambda,
                                                    inv_amax, g, X0, Y0);
                    // the warp's 32 consecutive points are two whole stages
                    const uint32_t bits = __ballot_sync(0xffffffffu, cut);
                    if (lane == 0) {
                        s_cut[b * kStagesPerChunk + (j >> 4)] = bits & 0xffffu;
                        s_cut[b * kStagesPerChunk + (j >> 4) + 1] = bits >> 16;
                    }
                } else {
                    bool cut;
                    uint32_t win;
                    const bool l = make_record(buf, j, valid, chrec[valid ? idx : 0], tile, g.inv_lambda, inv_amax,
                                               X0, Y0, left, cut, win);
                    if (MASKS) s_win[b * kChunkTc + j] = win;
                    // the warp's 32 consecutive points -> one word of the left-pair
                    // mask (this CTA alone writes it: pps is a multiple of kChunkTc)
                    // and the cut flags of two whole stages
                    const uint32_t bits = __ballot_sync(0xffffffffu, l);
                    const uint32_t cbits = MASKS ? __ballot_sync(0xffffffffu, cut) : 0u;
                    if (lane == 0) {
                        if (a.mask) a.mask[mask_base + (((int64_t)part * a.pps + idx) >> 5)] = bits;
                        if (MASKS) {
                            s_cut[b * kStagesPerChunk + (j >> 4)] = cbits & 0xffffu;
                            s_cut[b * kStagesPerChunk + (j >> 4) + 1] = cbits >> 16;
                        }
                    }
                }
            }
            __syncwarp();
            if (lane == 0) mbar_arrive(&rec_full[b]);
        }
        const int wl = __reduce_add_sync(0xffffffffu, left);
        if (lane == 0 && wl) atomicAdd(s_left, wl);
    } else {
        for (int c = 0; c < nchunks && !dead; ++c) {
            const int b = c & 1;
            // every lane waits: each one acquires the record warps' stores
            const bool rok = mbar_wait_for(&rec_full[b], (uint32_t)(c >> 1) & 1u, abort, kWaitNs);
            dead = !__all_sync(0xffffffffu, rok);
            if (dead) break;
            const TcRsPair* rb = s_rec + b * (kChunkTc / 2);
            const int it0 = c * kStagesPerChunk, it1 = min(total, it0 + kStagesPerChunk);
            // the chunk's per-stage cut flags, read once: bit k for stage it0 + k
            uint32_t cutmask = 0;
#pragma unroll
            for (int q = 0; q < (FR || MASKS ? kStagesPerChunk / 4 : 0); ++q) {
                const uint4 f = reinterpret_cast<const uint4*>(s_cut + b * kStagesPerChunk)[q];
                cutmask |= (uint32_t)(f.x != 0) << (4 * q) | (uint32_t)(f.y != 0) << (4 * q + 1) |
                           (uint32_t)(f.z != 0) << (4 * q + 2) | (uint32_t)(f.w != 0) << (4 * q + 3);
            }
            // The chunk's stages. RS runs a separate instance of the loop
            // (masks true) for a chunk that holds a window-cut pair.
            auto stages = [&](auto masks) {
                constexpr bool kMasks = decltype(masks)::value;
                for (int it = it0; it < it1; ++it) {
                    const int s = it % L::Stages;
                    bool ok = true;
                    if (lane == 0)
                        ok = mbar_wait_for(&empty[s], ((uint32_t)(it / L::Stages) & 1u) ^ 1u, abort, kWaitNs);
                    dead = !__shfl_sync(0xffffffffu, ok, 0);
                    if (dead) break;
                    const uint32_t sb = smem_u32(base + s * L::kStageBytes);
                    const TcRsPair* recs8 = rb + ((it - it0) * kStagePts) / 2 + 4 * kc;
                    const bool cut = (cutmask >> (it - it0)) & 1u;   // warp-uniform
                    if constexpr (FR) {
                        if (cut) {
                            if (side_a) produce_stage_fr<true, true>(recs8, off, offb, rc, rc + 64, sb + row_off0,
                                                                     sb + row_off1);
                            else produce_stage_fr<false, true>(recs8, off, offb, rc, rc + 64, sb + row_off0,
                                                               sb + row_off1);
                        } else {
                            if (side_a) produce_stage_fr<true, false>(recs8, off, offb, rc, rc + 64, sb + row_off0,
                                                                      sb + row_off1);
                            else produce_stage_fr<false, false>(recs8, off, offb, rc, rc + 64, sb + row_off0,
                                                                sb + row_off1);
                        }
                    } else {
                        const uint32_t* wins = s_win + b * kChunkTc + (it - it0) * kStagePts + 8 * kc;
                        if (kMasks && cut) {
                            if (side_a) produce_stage<true, kMasks>(recs8, off, offb, sb + row_off0, sb + row_off1,
                                                                    wins, rc, rc + 64);
                            else produce_stage<false, kMasks>(recs8, off, offb, sb + row_off0, sb + row_off1, wins,
                                                              rc, rc + 64);
                        } else {
                            if (side_a) produce_stage<true, false>(recs8, off, offb, sb + row_off0, sb + row_off1,
                                                                   wins, rc, rc + 64);
                            else produce_stage<false, false>(recs8, off, offb, sb + row_off0, sb + row_off1, wins,
                                                             rc, rc + 64);
                        }
                    }
                    fence_async_smem();   // generic-proxy writes -> visible to the tensor core
                    __syncwarp();
                    if (lane == 0) mbar_arrive(&full[s]);
                    // the previous run is drained (by every producer warp) once
                    // the first stage of the next one is filled: the MMA warp
                    // needs D free only to issue that stage
                    if ((it % kPeriod) == 0 && it > 0) {
                        dead = !drain_run(drained, periods, acc_full, acc_empty, abort, tmem, warp, lane, a, ch, out,
                                          X0, Y0, amax, wrote);
                        ++drained;
                        if (dead) break;
                    }
                }
            };
            if constexpr (!FR && MASKS) {
                if (cutmask != 0) stages(std::true_type{});
                else stages(std::false_type{});
            } else {
                stages(std::false_type{});
            }
            __syncwarp();
            if (lane == 0) mbar_arrive(&rec_empty[b]);   // this chunk's records are no longer read
        }
        // the runs not drained yet (the last one flushes into the field)
        for (int p = drained; p < periods && !dead; ++p)
            dead = !drain_run(p, periods, acc_full, acc_empty, abort, tmem, warp, lane, a, ch, out, X0, Y0, amax,
                              wrote);
    }
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    if (warp == kMmaWarp) tmem_dealloc(tmem, kTmemColsTc);
    if (threadIdx.x == 0) {
        if (*s_left) atomicAdd(&a.left[((int64_t)ch * a.tiles_y + blockIdx.y) * a.tiles_x + tx], *s_left);
        if (*abort) atomicExch(a.error, 1);
    }
    if (a.ksplit > 1) sum_parts(a, ch, tx, X0, Y0, s_left);
}

// The RS tile with factor masks, out of line: its register allocation
// stays apart from that of the full-window tile body in tc_rs_kernel.
__device__ __noinline__ void tile_body_rs_masked(const TcRsArgs& a) { tile_body<false, true>(a); }

// RS: the masked tile body when some point's window rectangle leaves part of
// the field out (the flag word written by rs_amax_kernel), else the
// full-window one: no pair can then cut a tile.
__global__ void __launch_bounds__(kThreadsTc, 1) tc_rs_kernel(const __grid_constant__ TcRsArgs a) {
    if (reinterpret_cast<const int*>(a.amax)[kWindowWord] != 0) tile_body_rs_masked(a);
    else tile_body<false, false>(a);
}

// Fresnel on the tensor cores, factors generated on chip: the same tile
// pipeline with no cross pair and no CUDA-core complement.
__global__ void __launch_bounds__(kThreadsTc, 1) tc_fresnel_kernel(const __grid_constant__ TcRsArgs a) {
    tile_body<true, false>(a);
}

// Largest coef / z^2 of a channel: bounds every coef / r_c^2, so the
// factors stay within [-1, 1] (FP16 range for the cross pair).
// (RS: coef / z^2; Fresnel, with per_z2 false: coef, the factor amplitude
// before any window.) With window_flag (RS), also sets *window_flag to 1
// when a point's non-empty window rectangle does not cover the whole
// pnX x pnY field (its window can then cut a tile).
__global__ void rs_amax_kernel(const PointRec* __restrict__ recs, int64_t n, float* out, bool per_z2 = true,
                               int* window_flag = nullptr, int pnX = 0, int pnY = 0) {
    float m = 0.f;
    bool part = false;
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        const PointRec& p = recs[i];
        m = fmaxf(m, fabsf((float)(per_z2 ? p.coef / p.aux : p.coef)));
        part |= p.x_lo < p.x_hi && p.y_lo < p.y_hi && !(p.x_lo <= 0 && p.x_hi >= pnX && p.y_lo <= 0 && p.y_hi >= pnY);
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) m = fmaxf(m, __shfl_xor_sync(0xffffffffu, m, o));
    if ((threadIdx.x & 31) == 0) atomicMax(reinterpret_cast<int*>(out), __float_as_int(m));   // m >= 0
    if (window_flag && __any_sync(0xffffffffu, part) && (threadIdx.x & 31) == 0) atomicExch(window_flag, 1);
}

size_t align_up(size_t v, size_t al) { return (v + al - 1) / al * al; }

// One CTA per SM: split every tile's points into k parts so that the CTA
// count fills whole waves (each extra part costs a field-sized partial and a
// summing pass: demand a 3% gain, at least 1,024 points a part, at most
// 2 GiB of partials). Parts are whole chunks of kChunkTc points (the
// left-pair mask words of a part are its own), and none is empty.
void choose_tile_split(int64_t tiles, int64_t n_points, size_t field_bytes, int sm_count, int* ksplit_out,
                       int64_t* pps_out) {
    const int slots = sm_count > 0 ? sm_count : 1;
    auto part_points = [&](int k) {
        const int64_t p = (n_points + k - 1) / k;
        return (p + kChunkTc - 1) / kChunkTc * kChunkTc;
    };
    int ksplit = 1;
    double best = 0.0;
    for (int k = 1; k <= 8; ++k) {
        if (k > 1 && (n_points / k < 1024 || (size_t)(k - 1) * field_bytes > ((size_t)2 << 30) ||
                      n_points - (k - 1) * part_points(k) < 1))
            break;
        const double waves = (double)(tiles * k) / slots;
        const double eff = waves / std::ceil(waves);
        if (eff > best + 0.03) {
            best = eff;
            ksplit = k;
        }
    }
    *ksplit_out = ksplit;
    *pps_out = part_points(ksplit);
}

}  // namespace

ophpc_status tc_generate_rs(cudaMemPool_t pool, const JobGeom& jg, const ophpc_config* cfg,
                            const ophpc_vertex* d_vertices, uint64_t n_points, double* d_field, int sm_count,
                            cudaStream_t s, std::string* err, int* d_err_out) {
    auto fail = [&](ophpc_status st, const char* msg) {
        if (err) *err = msg;
        return st;
    };
    // per call: the attribute belongs to the current device
    if (cudaFuncSetAttribute(tc_rs_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kSmemTc) != cudaSuccess)
        return fail(OPHPC_ERROR_CUDA, "cudaFuncSetAttribute(tc_rs_kernel) failed");
    const int nch = jg.n_channels;
    const int pnX = cfg->pixel_number[0], pnY = cfg->pixel_number[1];
    const int tiles_x = (pnX + kRsTcTile - 1) / kRsTcTile, tiles_y = (pnY + kRsTcTile - 1) / kRsTcTile;
    const size_t rec_bytes = align_up(sizeof(PointRec) * n_points * nch, 256);
    const size_t left_bytes = align_up(sizeof(int32_t) * (size_t)nch * tiles_x * tiles_y, 256);
    const int64_t tiles = (int64_t)tiles_x * tiles_y * nch;
    const size_t field_bytes = sizeof(double2) * (size_t)nch * pnX * pnY;
    int ksplit = 1;
    int64_t pps = 0;
    choose_tile_split(tiles, (int64_t)n_points, field_bytes, sm_count, &ksplit, &pps);
    const size_t part_bytes = align_up(field_bytes * (size_t)(ksplit - 1), 256);
    const size_t ticket_bytes = align_up(sizeof(int32_t) * (size_t)tiles, 256);
    // left-pair mask: one bit per (tile, point); without room for it the
    // complement re-tests eligibility instead
    static_assert(kChunkTc == 256, "tc_rs_mask_words assumes chunks of 256 points");
    const int64_t mask_words = tc_rs_mask_words((int64_t)n_points);
    size_t mask_bytes = align_up(sizeof(uint32_t) * (size_t)tiles * (size_t)mask_words, 256);
    if (mask_bytes > ((size_t)4 << 30)) mask_bytes = 0;
    unsigned char* buf = nullptr;
    if (cudaMallocFromPoolAsync((void**)&buf, rec_bytes + left_bytes + ticket_bytes + part_bytes + mask_bytes + 256,
                                pool, s) != cudaSuccess)
        return fail(OPHPC_ERROR_OUT_OF_MEMORY, "tensor-core RS scratch allocation failed");
    PointRec* recs = (PointRec*)buf;
    int32_t* left = (int32_t*)(buf + rec_bytes);
    int32_t* tickets = (int32_t*)(buf + rec_bytes + left_bytes);
    double2* partials = ksplit > 1 ? (double2*)(buf + rec_bytes + left_bytes + ticket_bytes) : nullptr;
    uint32_t* mask = mask_bytes ? (uint32_t*)(buf + rec_bytes + left_bytes + ticket_bytes + part_bytes) : nullptr;
    float* amax = (float*)(buf + rec_bytes + left_bytes + ticket_bytes + part_bytes + mask_bytes);   // [3]
    int* errw = (int*)(amax + 4);
    cudaMemsetAsync(amax, 0, 32, s);   // amax[0..3] and the error word
    cudaMemsetAsync(left, 0, left_bytes + ticket_bytes, s);

    launch_prep(d_vertices, (int64_t)n_points, cfg->scale, cfg->distance, cfg->field_length, cfg->viewing_window,
                (int)OPHPC_DIFF_RS, jg, recs, s);
    for (int c = 0; c < nch; ++c) {
        count_launches(1);
        rs_amax_kernel<<<256, 256, 0, s>>>(recs + (int64_t)c * n_points, (int64_t)n_points, amax + c, true,
                                           reinterpret_cast<int*>(amax) + kWindowWord, pnX, pnY);
    }
    TcRsArgs ta;
    std::memset(&ta, 0, sizeof(ta));
    ta.jg = jg;
    ta.jg.accumulate = 0;
    ta.recs = recs;
    ta.field = (double2*)d_field;
    ta.amax = amax;
    ta.left = left;
    ta.error = errw;
    ta.tiles_x = tiles_x;
    ta.tiles_y = tiles_y;
    ta.p_base = 0;
    ta.p_count = (int64_t)n_points;
    ta.ksplit = ksplit;
    ta.pps = pps;
    ta.partials = partials;
    ta.tickets = tickets;
    ta.mask = mask;
    ta.mask_words = mask_words;
    count_launches(1);
    tc_rs_kernel<<<dim3((unsigned)(tiles_x * ksplit), (unsigned)tiles_y, (unsigned)nch), kThreadsTc, kSmemTc, s>>>(ta);

    // the CUDA-core complement: the pairs the tensor-core kernel left
    JobGeom jc = jg;
    jc.ksplit = 1;
    jc.points_per_split = (int64_t)n_points;
    jc.p0 = 0;
    jc.p1 = 0;
    jc.accumulate = 1;
    jc.tc_skip = 1;
    jc.tc_left = left;
    jc.tc_tiles_x = tiles_x;
    jc.tc_tiles_y = tiles_y;
    jc.tc_mask = mask;
    jc.tc_mask_words = mask_words;
    launch_rs(recs, jc, (double2*)d_field, nullptr, s);

    cudaError_t e = cudaGetLastError();
    int herr = 0;
    if (d_err_out) {
        // the caller reads the timeout word later (graph capture: nothing
        // here may wait for the stream)
        if (e == cudaSuccess) e = cudaMemcpyAsync(d_err_out, errw, sizeof(int), cudaMemcpyDeviceToDevice, s);
    } else {
        if (e == cudaSuccess) e = cudaMemcpyAsync(&herr, errw, sizeof(int), cudaMemcpyDeviceToHost, s);
        if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    }
    cudaFreeAsync(buf, s);
    if (e != cudaSuccess) return fail(OPHPC_ERROR_CUDA, cudaGetErrorString(e));
    if (herr) return fail(OPHPC_ERROR_TIMEOUT, "tensor-core RS kernel wait timed out");
    return OPHPC_SUCCESS;
}

void launch_rs_amax(const PointRec* d_recs, int64_t n_points, int n_channels, int pnX, int pnY, float* d_amax,
                    cudaStream_t s) {
    for (int c = 0; c < n_channels; ++c) {
        count_launches(1);
        rs_amax_kernel<<<256, 256, 0, s>>>(d_recs + (int64_t)c * n_points, n_points, d_amax + c, true,
                                           reinterpret_cast<int*>(d_amax) + kWindowWord, pnX, pnY);
    }
}

cudaError_t launch_tc_rs_range(const JobGeom& jg, const PointRec* d_recs, int64_t p0, int64_t p1, bool accumulate,
                               double2* d_field, const float* d_amax, int32_t* d_left, uint32_t* d_mask,
                               int64_t mask_words, int* d_err, cudaStream_t s) {
    cudaError_t e = cudaFuncSetAttribute(tc_rs_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kSmemTc);
    if (e != cudaSuccess || p1 <= p0) return e;
    if (d_mask && tc_rs_mask_words(p1 - p0) > mask_words) return cudaErrorInvalidValue;
    const int nch = jg.n_channels;
    const int pnX = jg.ch[0].pnX, pnY = jg.ch[0].pnY;
    const int tiles_x = (pnX + kRsTcTile - 1) / kRsTcTile, tiles_y = (pnY + kRsTcTile - 1) / kRsTcTile;
    e = cudaMemsetAsync(d_left, 0, sizeof(int32_t) * (size_t)nch * tiles_x * tiles_y, s);
    if (e != cudaSuccess) return e;
    TcRsArgs ta;
    std::memset(&ta, 0, sizeof(ta));
    ta.jg = jg;
    ta.jg.accumulate = accumulate ? 1 : 0;
    ta.recs = d_recs;
    ta.field = d_field;
    ta.amax = d_amax;
    ta.left = d_left;
    ta.error = d_err;
    ta.tiles_x = tiles_x;
    ta.tiles_y = tiles_y;
    ta.p_base = p0;
    ta.p_count = p1 - p0;
    ta.ksplit = 1;
    ta.pps = p1 - p0;
    ta.mask = d_mask;
    ta.mask_words = mask_words;
    count_launches(1);
    tc_rs_kernel<<<dim3((unsigned)tiles_x, (unsigned)tiles_y, (unsigned)nch), kThreadsTc, kSmemTc, s>>>(ta);
    JobGeom jc = jg;
    jc.ksplit = 1;
    jc.points_per_split = p1 - p0;
    jc.p0 = p0;
    jc.p1 = p1;
    jc.accumulate = 1;
    jc.tc_skip = 1;
    jc.tc_left = d_left;
    jc.tc_tiles_x = tiles_x;
    jc.tc_tiles_y = tiles_y;
    jc.tc_mask = d_mask;
    jc.tc_mask_words = mask_words;
    launch_rs(d_recs, jc, d_field, nullptr, s);
    return cudaGetLastError();
}

ophpc_status tc_generate_fresnel_tiles(cudaMemPool_t pool, const JobGeom& jg, const ophpc_config* cfg,
                                       const ophpc_vertex* d_vertices, uint64_t n_points, double* d_field,
                                       int sm_count, cudaStream_t s, std::string* err, int* d_err_out) {
    auto fail = [&](ophpc_status st, const char* msg) {
        if (err) *err = msg;
        return st;
    };
    if (cudaFuncSetAttribute(tc_fresnel_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kSmemTcFr) !=
        cudaSuccess)
        return fail(OPHPC_ERROR_CUDA, "cudaFuncSetAttribute(tc_fresnel_kernel) failed");
    const int nch = jg.n_channels;
    const int pnX = cfg->pixel_number[0], pnY = cfg->pixel_number[1];
    const int tiles_x = (pnX + kRsTcTile - 1) / kRsTcTile, tiles_y = (pnY + kRsTcTile - 1) / kRsTcTile;
    const int64_t tiles = (int64_t)tiles_x * tiles_y * nch;
    const size_t field_bytes = sizeof(double2) * (size_t)nch * pnX * pnY;
    int ksplit = 1;
    int64_t pps = 0;
    choose_tile_split(tiles, (int64_t)n_points, field_bytes, sm_count, &ksplit, &pps);
    const size_t rec_bytes = align_up(sizeof(PointRec) * n_points * nch, 256);
    const size_t part_bytes = align_up(field_bytes * (size_t)(ksplit - 1), 256);
    const size_t ticket_bytes = align_up(sizeof(int32_t) * (size_t)tiles, 256);
    unsigned char* buf = nullptr;
    if (cudaMallocFromPoolAsync((void**)&buf, rec_bytes + ticket_bytes + part_bytes + 256, pool, s) != cudaSuccess)
        return fail(OPHPC_ERROR_OUT_OF_MEMORY, "tensor-core Fresnel scratch allocation failed");
    PointRec* recs = (PointRec*)buf;
    int32_t* tickets = (int32_t*)(buf + rec_bytes);
    double2* partials = ksplit > 1 ? (double2*)(buf + rec_bytes + ticket_bytes) : nullptr;
    float* amax = (float*)(buf + rec_bytes + ticket_bytes + part_bytes);   // [3]
    int* errw = (int*)(amax + 4);
    cudaMemsetAsync(amax, 0, 32, s);   // amax[0..3] and the error word
    cudaMemsetAsync(tickets, 0, ticket_bytes, s);
    launch_prep(d_vertices, (int64_t)n_points, cfg->scale, cfg->distance, cfg->field_length, cfg->viewing_window,
                (int)OPHPC_DIFF_FRESNEL, jg, recs, s);
    for (int c = 0; c < nch; ++c) {
        count_launches(1);
        rs_amax_kernel<<<256, 256, 0, s>>>(recs + (int64_t)c * n_points, (int64_t)n_points, amax + c, false);
    }
    TcRsArgs ta;
    std::memset(&ta, 0, sizeof(ta));
    ta.jg = jg;
    ta.jg.accumulate = 0;
    ta.recs = recs;
    ta.field = (double2*)d_field;
    ta.amax = amax;
    ta.error = errw;
    ta.tiles_x = tiles_x;
    ta.tiles_y = tiles_y;
    ta.p_base = 0;
    ta.p_count = (int64_t)n_points;
    ta.ksplit = ksplit;
    ta.pps = pps;
    ta.partials = partials;
    ta.tickets = tickets;
    count_launches(1);
    tc_fresnel_kernel<<<dim3((unsigned)(tiles_x * ksplit), (unsigned)tiles_y, (unsigned)nch), kThreadsTc, kSmemTcFr,
                        s>>>(ta);
    cudaError_t e = cudaGetLastError();
    int herr = 0;
    if (d_err_out) {
        if (e == cudaSuccess) e = cudaMemcpyAsync(d_err_out, errw, sizeof(int), cudaMemcpyDeviceToDevice, s);
    } else {
        if (e == cudaSuccess) e = cudaMemcpyAsync(&herr, errw, sizeof(int), cudaMemcpyDeviceToHost, s);
        if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    }
    cudaFreeAsync(buf, s);
    if (e != cudaSuccess) return fail(OPHPC_ERROR_CUDA, cudaGetErrorString(e));
    if (herr) return fail(OPHPC_ERROR_TIMEOUT, "tensor-core Fresnel kernel wait timed out");
    return OPHPC_SUCCESS;
}

void launch_fresnel_amax(const PointRec* d_recs, int64_t n_points, int n_channels, float* d_amax, cudaStream_t s) {
    for (int c = 0; c < n_channels; ++c) {
        count_launches(1);
        rs_amax_kernel<<<256, 256, 0, s>>>(d_recs + (int64_t)c * n_points, n_points, d_amax + c, false);
    }
}

cudaError_t launch_tc_fresnel_range(const JobGeom& jg, const PointRec* d_recs, int64_t p0, int64_t p1,
                                    bool accumulate, double2* d_field, const float* d_amax, int* d_err,
                                    cudaStream_t s) {
    cudaError_t e = cudaFuncSetAttribute(tc_fresnel_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         (int)kSmemTcFr);
    if (e != cudaSuccess || p1 <= p0) return e;
    const int nch = jg.n_channels;
    const int pnX = jg.ch[0].pnX, pnY = jg.ch[0].pnY;
    const int tiles_x = (pnX + kRsTcTile - 1) / kRsTcTile, tiles_y = (pnY + kRsTcTile - 1) / kRsTcTile;
    TcRsArgs ta;
    std::memset(&ta, 0, sizeof(ta));
    ta.jg = jg;
    ta.jg.accumulate = accumulate ? 1 : 0;
    ta.recs = d_recs;
    ta.field = d_field;
    ta.amax = d_amax;
    ta.error = d_err;
    ta.tiles_x = tiles_x;
    ta.tiles_y = tiles_y;
    ta.p_base = p0;
    ta.p_count = p1 - p0;
    ta.ksplit = 1;
    ta.pps = p1 - p0;
    count_launches(1);
    tc_fresnel_kernel<<<dim3((unsigned)tiles_x, (unsigned)tiles_y, (unsigned)nch), kThreadsTc, kSmemTcFr, s>>>(ta);
    return cudaGetLastError();
}

}  // namespace ophpc
