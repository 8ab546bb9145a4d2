// Device encoding and 8-bit normalisation.
//
// ophGen::encoding (ophgen/src/ophGen.cpp:816-849) maps every complex pixel
// to a real value; ophGen::normalize (ophgen/src/ophGen.cpp:654-687) then
// takes the min and max over ALL channels (minOfArr/maxOfArr,
// Openholo/src/function.h:79-99: min starts at MAX_DOUBLE, max at
// MIN_DOUBLE = 2.2250738585072014e-308, strict comparisons, so NaNs never
// win) and writes (uchar)(((v - min) / gap) * 255 + 0.5).
//
// Two launches, both grid-stride over [n_channels * n_pixels]:
//   encode_minmax : value per pixel (FP64, optional store) + block min/max,
//                   folded into two 64-bit words with atomicMin/atomicMax on
//                   an order-preserving integer image of the doubles;
//   normalize     : re-derives (or re-reads) the value and writes the byte.
// The encoded value is recomputed in the second pass when it is not stored,
// so the field is read twice but no FP64 intermediate is written.
// All FP64 arithmetic uses explicit _rn operations (no FMA) to round exactly
// as the x86-64 reference does.
#include "pc_common.cuh"
#include "ophpc.h"

#include <cfloat>

namespace ophpc {

namespace {

constexpr double kPi = 3.14159265358979323846;
constexpr double kMaxDouble = 1.7976931348623158e+308;
constexpr double kMinDouble = 2.2250738585072014e-308;

// FP32 image of a double from its high word: sign, exponent, the top 20
// mantissa bits (truncated: relative error < 2^-20). ok turns false where
// the image cannot stand in: subnormal, or outside 2^-62 .. 2^62 (squares
// stay normal floats), infinite or NaN.
__device__ __forceinline__ float hi_float(double d, bool& ok) {
    const unsigned long long b = (unsigned long long)__double_as_longlong(d);
    const unsigned hi = (unsigned)(b >> 32);
    const int ex = (int)((hi >> 20) & 0x7ffu);
    const unsigned sign = hi & 0x80000000u;
    if (ex == 0) {
        if ((hi & 0xfffffu) | (unsigned)b) ok = false;   // subnormal
        return __int_as_float((int)sign);                  // signed zero, as atan2 sees it
    }
    if (ex < 1023 - 62 || ex > 1023 + 62) {
        ok = false;
        return 0.f;
    }
    return __int_as_float((int)(sign | ((unsigned)(ex - 1023 + 127) << 23) | ((hi & 0xfffffu) << 3)));
}

// ---- the phase encoder's value -----------------------------------------------
// (atan2(y, x) + pi) / (2 pi) with a table-driven atan2 (argument reduction
// by a tabulated angle, then the Maclaurin series of atan): about 19 FP64
// operations, where CUDA's atan2 and a divide take several times that on
// GB300's narrow FP64 pipe. An FP32 estimate (atan2f of the high words)
// picks the nearest tabulated angle theta_k = fl(k pi / 128),
// k = -128..128. Rotating (x, y) by -theta_k with the table's FP64 cos and
// sin leaves a = |z| cos(delta) > 0 and b = |z| sin(delta),
// |delta| <= pi / 256 plus the estimate's error, so |t| = |b / a| < 0.0123
// and delta = atan(t) = t - t^3/3 + t^5/5 - t^7/7, the first omitted term
// below 1e-18. theta = theta_k + delta lies within a few 1e-16 rad of the
// correctly rounded atan2, and then goes through the reference's
// (theta + pi) / (2 pi), the division as a product with the reciprocal and
// one FMA residual step (Markstein's correction for a quotient). Zeros on
// both axes, subnormal, huge and non-finite inputs take CUDA's atan2.
struct AtanTable {
    double c[257], s[257], th[257];   // cos, sin and theta_k of entry k + 128
};

// sin and cos of |r| <= pi / 4 by their Maclaurin series: 20 terms each, a
// term below 1e-200 ending its series (so that none underflows), summed
// from the smallest
constexpr double abs_c(double v) { return v < 0.0 ? -v : v; }
constexpr void series_sincos(double r, double& s, double& c) {
    const double r2 = r * r;
    double ts[20] = {}, tc[20] = {};
    ts[0] = r;
    tc[0] = 1.0;
    for (int m = 0; m + 1 < 20; ++m) {
        ts[m + 1] = abs_c(ts[m]) < 1e-200 ? 0.0 : ts[m] * (-r2 / ((2.0 * m + 2.0) * (2.0 * m + 3.0)));
        tc[m + 1] = abs_c(tc[m]) < 1e-200 ? 0.0 : tc[m] * (-r2 / ((2.0 * m + 1.0) * (2.0 * m + 2.0)));
    }
    s = 0.0;
    c = 0.0;
    for (int m = 19; m >= 0; --m) {
        s += ts[m];
        c += tc[m];
    }
}

// Entry k + 128: theta_k = fl(k pi / 128) and its cos and sin, from the
// series at theta_k less the nearest multiple q pi / 2 (fl(pi) / 2 taken
// off exactly, then the rest of pi / 2), turned by the q quarter turns.
constexpr AtanTable make_atan_table() {
    AtanTable t{};
    constexpr double kPiLo = 1.2246467991473532e-16;   // pi - fl(pi)
    for (int k = 0; k <= 128; ++k) {
        const double th = (double)k * (kPi / 128.0);
        const int q = (k + 32) / 64;
        const double r = (th - q * (kPi / 2.0)) - q * (kPiLo / 2.0);
        double sr = 0.0, cr = 0.0;
        series_sincos(r, sr, cr);
        const double c = q == 0 ? cr : q == 1 ? -sr : -cr;
        const double sn = q == 0 ? sr : q == 1 ? cr : -sr;
        t.c[128 + k] = c;
        t.s[128 + k] = sn;
        t.th[128 + k] = th;
        if (k > 0) {
            t.c[128 - k] = c;
            t.s[128 - k] = -sn;
            t.th[128 - k] = -th;
        }
    }
    return t;
}

__device__ constexpr AtanTable kAtanTab = make_atan_table();

constexpr double kTwoPi = 2.0 * kPi;
constexpr double kInvTwoPi = 0.15915494309189535;   // fl(1 / (2 pi))

__device__ __forceinline__ double phase_value(double y, double x) {
    bool ok = true;
    const float xf = hi_float(x, ok), yf = hi_float(y, ok);
    double theta;
    if (!ok || (xf == 0.f && yf == 0.f)) {
        theta = atan2(y, x);
    } else {
        int k = __float2int_rn(atan2f(yf, xf) * 40.74366543152521f);   // 128 / pi
        k = min(128, max(-128, k)) + 128;
        const double c = __ldg(&kAtanTab.c[k]), s = __ldg(&kAtanTab.s[k]);
        const double a = __fma_rn(x, c, __dmul_rn(y, s));
        const double b = __fma_rn(y, c, -__dmul_rn(x, s));
        // t = b / a: an FP32 reciprocal, then one residual step
        const double r0 = (double)__frcp_rn((float)a);
        const double t0 = __dmul_rn(b, r0);
        const double t = __fma_rn(__fma_rn(-a, t0, b), r0, t0);
        const double u = __dmul_rn(t, t);
        const double p = __fma_rn(__fma_rn(u, -1.0 / 7.0, 1.0 / 5.0), u, -1.0 / 3.0);
        theta = __dadd_rn(__ldg(&kAtanTab.th[k]), __fma_rn(__dmul_rn(t, u), p, t));
    }
    const double sum = __dadd_rn(theta, kPi);
    const double q = __dmul_rn(sum, kInvTwoPi);
    return __fma_rn(__fma_rn(-q, kTwoPi, sum), kInvTwoPi, q);
}

__device__ __forceinline__ double encode_value(double2 h, int flag) {
    switch (flag) {
        case 0:    // Phase: (atan2(im, re) + pi) / (2 pi)   (ophGen.cpp:1843-1853)
            return phase_value(h.y, h.x);
        case 1:    // Amplitude: sqrt(re^2 + im^2)            (ophGen.cpp:1855-1864)
            return sqrt(__dadd_rn(__dmul_rn(h.x, h.x), __dmul_rn(h.y, h.y)));
        case 2:    // RealPart                                 (ophGen.cpp:1821-1830)
            return h.x;
        default:   // ImaginaryPart                            (ophGen.cpp:1832-1841)
            return h.y;
    }
}

// Order-preserving map double -> uint64 (for non-NaN values).
__device__ __forceinline__ unsigned long long ordered_bits(double d) {
    unsigned long long b = (unsigned long long)__double_as_longlong(d);
    return (b & 0x8000000000000000ull) ? ~b : (b | 0x8000000000000000ull);
}

__device__ __forceinline__ uint64_t global_ns_enc() {
    uint64_t t;
    asm volatile("mov.u64 %0, %globaltimer;" : "=l"(t));
    return t;
}

// min and max on the order-preserving integer images of the values (ALU
// work, not the FP64 pipe's); NaN never wins, as with the reference's strict
// comparisons
__device__ __forceinline__ void fold_value(double e, unsigned long long& omn, unsigned long long& omx) {
    const unsigned long long b = (unsigned long long)__double_as_longlong(e);
    if ((b & 0x7fffffffffffffffull) > 0x7ff0000000000000ull) return;   // NaN
    const unsigned long long o = (b & 0x8000000000000000ull) ? ~b : (b | 0x8000000000000000ull);
    omn = o < omn ? o : omn;
    omx = o > omx ? o : omx;
}

// the block's min and max into minmax[0] / minmax[1] (256 threads)
__device__ __forceinline__ void block_fold(unsigned long long omn, unsigned long long omx,
                                           unsigned long long* __restrict__ minmax) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        const unsigned long long a = __shfl_xor_sync(0xffffffffu, omn, o);
        const unsigned long long b = __shfl_xor_sync(0xffffffffu, omx, o);
        omn = a < omn ? a : omn;
        omx = b > omx ? b : omx;
    }
    __shared__ unsigned long long s_mn[8], s_mx[8];
    const int w = threadIdx.x >> 5;
    if ((threadIdx.x & 31) == 0) {
        s_mn[w] = omn;
        s_mx[w] = omx;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        for (int k = 1; k < (int)(blockDim.x >> 5); ++k) {
            omn = s_mn[k] < omn ? s_mn[k] : omn;
            omx = s_mx[k] > omx ? s_mx[k] : omx;
        }
        atomicMin(&minmax[0], omn);
        atomicMax(&minmax[1], omx);
    }
}

__global__ void __launch_bounds__(256) encode_minmax_kernel(const double2* __restrict__ field, int64_t n,
                                                            int flag, double* __restrict__ encoded,
                                                            unsigned long long* __restrict__ minmax) {
    unsigned long long omn = ordered_bits(kMaxDouble), omx = ordered_bits(kMinDouble);
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n;
         i += (int64_t)gridDim.x * blockDim.x) {
        const double e = encode_value(field[i], flag);
        if (encoded) encoded[i] = e;
        fold_value(e, omn, omx);
    }
    block_fold(omn, omx, minmax);
}

// min/max of an already encoded buffer (normalize() on its own)
__global__ void __launch_bounds__(256) minmax_kernel(const double* __restrict__ encoded, int64_t n,
                                                     unsigned long long* __restrict__ minmax) {
    unsigned long long omn = ordered_bits(kMaxDouble), omx = ordered_bits(kMinDouble);
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n;
         i += (int64_t)gridDim.x * blockDim.x)
        fold_value(encoded[i], omn, omx);
    block_fold(omn, omx, minmax);
}

__device__ __forceinline__ double from_ordered(unsigned long long b) {
    b = (b & 0x8000000000000000ull) ? (b & 0x7fffffffffffffffull) : ~b;
    return __longlong_as_double((long long)b);
}

// The byte (uchar)(((e - mn) / gap) * 255 + 0.5) with the reference's
// roundings. In FP32 from d = e - mn it lands within 5e-5 of the reference's
// value (d and 255 / gap rounded to FP32: 6e-8 relative each of at most
// 255.5, the FMA's rounding 1.5e-5), so where it lies more than 1e-4 from a
// code boundary its floor is the code; elsewhere (and for NaN, a gap of 0
// or a scale FP32 cannot hold) the FP64 division decides. Double -> uchar
// truncation: NaN and out-of-range values map to 0.
__device__ __forceinline__ uint8_t code_of(double e, double mn, double gap, float scale) {
    const double d = __dsub_rn(e, mn);
    const float v = __fmaf_rn((float)d, scale, 0.5f);
    const float f = floorf(v);
    if (v - f > 1e-4f && f + 1.f - v > 1e-4f && f >= 0.f && f <= 255.f) return (uint8_t)(int)f;
    const double val = __dadd_rn(__dmul_rn(__ddiv_rn(d, gap), 255.0), 0.5);
    return (val >= 0.0 && val < 256.0) ? (uint8_t)(int)val : (uint8_t)0;
}

__global__ void __launch_bounds__(256) normalize_kernel(const double2* __restrict__ field,
                                                        const double* __restrict__ encoded, int64_t n,
                                                        int flag, const unsigned long long* __restrict__ minmax,
                                                        uint8_t* __restrict__ out) {
    const double mn = from_ordered(minmax[0]);
    const double mx = from_ordered(minmax[1]);
    const double gap = __dsub_rn(mx, mn);
    const float scale = (gap > 0.0 && gap <= DBL_MAX) ? (float)__ddiv_rn(255.0, gap) : __int_as_float(0x7fc00000);
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n;
         i += (int64_t)gridDim.x * blockDim.x) {
        const double e = encoded ? encoded[i] : encode_value(field[i], flag);
        out[i] = code_of(e, mn, gap, scale);
    }
}

// n_words 2: the global min/max; 5: also the per-channel |H| maxima of the
// normalising encoders (words 2..4)
__global__ void init_minmax_kernel(unsigned long long* minmax, int n_words) {
    // initial values MAX_DOUBLE / MIN_DOUBLE of minOfArr / maxOfArr
    minmax[0] = ordered_bits(kMaxDouble);
    for (int k = 1; k < n_words; ++k) minmax[k] = ordered_bits(kMinDouble);
}

// ---------------------------------------------------------------------------
// Encoders that normalise the field by its largest magnitude first, one
// channel at a time as ophGen::encoding calls them (ophGen.cpp:845-847):
//   SimpleNI   (ophGen.cpp:1955-1974): m = max |H|; e = |H + m|^2 for every
//              pixel (the sqrt is squared again, as the reference does);
//   Burckhardt (ophGen.cpp:1897-1953): every third pixel H[3i], i < n/3,
//              divided by max |H[3i]|; its phase code p = (arg + pi)/(2 pi)
//              (in [0, 1]) and magnitude a pick one of three 120-degree
//              sectors compared in radians, so only the first is reached;
//              two of the three entries 3i..3i+2 are written;
//   TwoPhase   (ophGen.cpp:1866-1895): H[2i], i < n/2, divided by
//              max |H[2i]|; e[2i] = (p + pi) + acos(a), e[2i+1] = (p + pi) - acos(a).
// Entries an encoder does not write keep what the encoded buffer held.
// Launches: absmax over the sampled pixels (grid.y = channel, atomicMax on
// the ordered image of non-negative doubles), then the encoder; the 8-bit
// codes come from the generic minmax + normalize pair over the buffer.

__device__ __forceinline__ double mag_rn(double re, double im) {
    return __dsqrt_rn(__dadd_rn(__dmul_rn(re, re), __dmul_rn(im, im)));
}

__device__ __forceinline__ int64_t sample_count(int64_t n, int flag) {
    return flag == OPHPC_ENCODE_BURCKHARDT ? n / 3 : (flag == OPHPC_ENCODE_TWOPHASE ? n >> 1 : n);
}

__global__ void __launch_bounds__(256) chan_absmax_kernel(const double2* __restrict__ field, int64_t n_pixels,
                                                          int flag, unsigned long long* __restrict__ absmax) {
    const int c = blockIdx.y;
    const int64_t count = sample_count(n_pixels, flag);
    const int64_t stride = flag == OPHPC_ENCODE_BURCKHARDT ? 3 : (flag == OPHPC_ENCODE_TWOPHASE ? 2 : 1);
    const double2* f = field + (int64_t)c * n_pixels;
    double mx = kMinDouble;
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < count;
         i += (int64_t)gridDim.x * blockDim.x) {
        const double2 h = f[i * stride];
        const double a = mag_rn(h.x, h.y);
        if (a > mx) mx = a;
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) mx = fmax(mx, __shfl_xor_sync(0xffffffffu, mx, o));
    __shared__ double s_mx[8];
    if ((threadIdx.x & 31) == 0) s_mx[threadIdx.x >> 5] = mx;
    __syncthreads();
    if (threadIdx.x == 0) {
        for (int k = 1; k < (int)(blockDim.x >> 5); ++k) mx = fmax(mx, s_mx[k]);
        atomicMax(&absmax[c], ordered_bits(mx));
    }
}

__global__ void __launch_bounds__(256) encode_normalised_kernel(const double2* __restrict__ field, int64_t n_pixels,
                                                                int flag,
                                                                const unsigned long long* __restrict__ absmax,
                                                                double* __restrict__ encoded) {
    const int c = blockIdx.y;
    const double m = from_ordered(absmax[c]);
    const double2* f = field + (int64_t)c * n_pixels;
    double* e = encoded + (int64_t)c * n_pixels;
    const int64_t count = sample_count(n_pixels, flag);
    const double pi2 = kPi * 2, sqrt3 = __dsqrt_rn(3.0);
    const double third = __ddiv_rn(pi2, 3.0), two_thirds = __ddiv_rn(kPi * 4, 3.0);
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < count;
         i += (int64_t)gridDim.x * blockDim.x) {
        if (flag == OPHPC_ENCODE_SIMPLENI) {
            const double2 h = f[i];
            const double t = mag_rn(__dadd_rn(h.x, m), h.y);
            e[i] = __dmul_rn(t, t);
            continue;
        }
        const double2 h = f[flag == OPHPC_ENCODE_BURCKHARDT ? 3 * i : 2 * i];
        const double re = __ddiv_rn(h.x, m), im = __ddiv_rn(h.y, m);
        const double p = __ddiv_rn(__dadd_rn(atan2(im, re), kPi), pi2);
        const double a = mag_rn(re, im);
        if (flag == OPHPC_ENCODE_TWOPHASE) {
            const double d = acos(a), base = __dadd_rn(p, kPi);
            e[2 * i] = __dadd_rn(base, d);
            e[2 * i + 1] = __dsub_rn(base, d);
            continue;
        }
        // Burckhardt: a * (cos q + sin q / sqrt3) and 2 sin q / sqrt3 for the
        // sector's q, into the sector's two entries
        double q;
        int lo, hi;
        if (p >= 0 && p < third) {
            q = p, lo = 0, hi = 1;
        } else if (p >= third && p < two_thirds) {
            q = __dsub_rn(p, third), lo = 1, hi = 2;
        } else if (p >= two_thirds && p < pi2) {
            q = __dsub_rn(p, two_thirds), lo = 2, hi = 0;
        } else {
            continue;
        }
        const double sq = sin(q), cq = cos(q);
        e[3 * i + lo] = __dmul_rn(a, __dadd_rn(cq, __ddiv_rn(sq, sqrt3)));
        e[3 * i + hi] = __ddiv_rn(__dmul_rn(2.0, sq), sqrt3);
    }
}


// ---- phase / amplitude codes without the FP64 values -----------------------
// With no m_lpEncoded wanted, the codes come from FP32 estimates of the
// encoded values; FP64 (the functions above) only where an estimate cannot
// decide. The codes are the FP64 path's, bit for bit:
//   - the exact min/max: pixels whose estimate lies within twice its error
//     bound of the estimated min/max (the pixel that holds the exact one is
//     always among them) and pixels without a usable estimate, in FP64;
//   - a code: from the estimate unless it lies within its error bound of a
//     code boundary, else in FP64.
// Error bounds, in units of the encoded value: phase 1e-6 (inputs truncated
// to 20 mantissa bits: <= 9.5e-7 rad; atan2f: <= 3 ulp of pi; the FP32
// offset and scale: <= 3.3e-7 rad; / 2 pi = 3.2e-7, bound taken 3x),
// amplitude 4e-6 relative (<= 9.5e-7 from the inputs + 4 ulp, bound 3x).
constexpr float kPhaseErr = 1e-6f;
constexpr float kAmpErrRel = 4e-6f;

template <int FLAG>
__device__ __forceinline__ float estimate(double2 h, bool& ok) {
    ok = true;
    const float x = hi_float(h.x, ok), y = hi_float(h.y, ok);
    if (FLAG == 0) return (atan2f(y, x) + 3.14159265f) * 0.159154943f;
    return sqrtf(x * x + y * y);
}

__device__ __forceinline__ unsigned ordered32(float f) {
    const unsigned b = (unsigned)__float_as_int(f);
    return (b & 0x80000000u) ? ~b : (b | 0x80000000u);
}
__device__ __forceinline__ float from_ordered32(unsigned b) {
    return __int_as_float((int)((b & 0x80000000u) ? (b & 0x7fffffffu) : ~b));
}

// exact min/max words [0], [1]; estimated min/max (ordered 32-bit) in the
// two halves of word [2]
__global__ void init_est_minmax_kernel(unsigned long long* minmax) {
    minmax[0] = ordered_bits(kMaxDouble);
    minmax[1] = ordered_bits(kMinDouble);
    unsigned* w = reinterpret_cast<unsigned*>(minmax + 2);
    w[0] = ordered32(__int_as_float(0x7f800000));    // +inf
    w[1] = ordered32(__int_as_float((int)0xff800000u));   // -inf
    minmax[3] = 0;   // single-pass codes: grid barrier count
    minmax[4] = 0;   //                    barrier timeout
}

// block reduction of a min and a max pair of doubles into the exact words
__device__ __forceinline__ void fold_exact(double mn, double mx, unsigned long long* minmax) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        mn = fmin(mn, __shfl_xor_sync(0xffffffffu, mn, o));
        mx = fmax(mx, __shfl_xor_sync(0xffffffffu, mx, o));
    }
    __shared__ double s_mn[8], s_mx[8];
    const int w = threadIdx.x >> 5;
    if ((threadIdx.x & 31) == 0) {
        s_mn[w] = mn;
        s_mx[w] = mx;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        for (int k = 1; k < (int)(blockDim.x >> 5); ++k) {
            mn = fmin(mn, s_mn[k]);
            mx = fmax(mx, s_mx[k]);
        }
        if (mn != kMaxDouble) atomicMin(&minmax[0], ordered_bits(mn));
        if (mx != kMinDouble) atomicMax(&minmax[1], ordered_bits(mx));
    }
}

// pass 1: estimated min/max; pixels without an estimate go to the exact words
template <int FLAG>
__global__ void __launch_bounds__(256) est_minmax_kernel(const double2* __restrict__ field, int64_t n,
                                                         unsigned long long* __restrict__ minmax) {
    float mn = __int_as_float(0x7f800000), mx = -mn;
    double emn = kMaxDouble, emx = kMinDouble;
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        const double2 h = field[i];
        bool ok;
        const float e = estimate<FLAG>(h, ok);
        if (ok) {
            mn = fminf(mn, e);
            mx = fmaxf(mx, e);
        } else {
            const double x = encode_value(h, FLAG);
            if (x < emn) emn = x;
            if (x > emx) emx = x;
        }
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        mn = fminf(mn, __shfl_xor_sync(0xffffffffu, mn, o));
        mx = fmaxf(mx, __shfl_xor_sync(0xffffffffu, mx, o));
    }
    unsigned* w = reinterpret_cast<unsigned*>(minmax + 2);
    if ((threadIdx.x & 31) == 0) {
        atomicMin(&w[0], ordered32(mn));
        atomicMax(&w[1], ordered32(mx));
    }
    fold_exact(emn, emx, minmax);
}

template <int FLAG>
__device__ __forceinline__ float est_band(float mx_est) {
    return FLAG == 0 ? 2.f * kPhaseErr : 2.f * kAmpErrRel * fabsf(mx_est);
}

// The code of one pixel from its cached estimate e (NaN: none) when the
// estimate decides it: false where it lies within its error margin of a
// code boundary (or there is none), and code_exact then computes it in
// FP64. This is est_codes_kernel's rule, so the codes are the same bit for
// bit.
__device__ __forceinline__ bool code_fast(float e, bool usable, float mn_f, float sc_f, float margin,
                                          uint32_t& code) {
    const float v = (e - mn_f) * sc_f + 0.5f;
    const float fl = floorf(v);
    code = (uint32_t)(int)fl;
    return usable && e == e && v - fl > margin && fl + 1.f - v > margin && fl >= 0.f && fl <= 255.f;
}
template <int FLAG>
__device__ __forceinline__ uint32_t code_exact(const double2* __restrict__ px, double gmn, double gap) {
    const double x = encode_value(*px, FLAG);
    const double val = __dadd_rn(__dmul_rn(__ddiv_rn(__dsub_rn(x, gmn), gap), 255.0), 0.5);
    return (val >= 0.0 && val < 256.0) ? (uint32_t)(int)val : 0u;
}

// Pixels of a CTA that need FP64 (band pixels before the barrier, boundary
// pixels after it) are listed in shared memory and computed together, one
// per thread, instead of where a thread meets them: the FP64 pipe then runs
// a few full warps rather than many warps with one lane each. A list that
// fills up leaves the rest to be computed where they are met.
constexpr int kFp64List = 512;

// pass 2: the exact value of every pixel whose estimate is within the band
// of the estimated min or max
template <int FLAG>
__global__ void __launch_bounds__(256) refine_minmax_kernel(const double2* __restrict__ field, int64_t n,
                                                            unsigned long long* __restrict__ minmax) {
    __shared__ int64_t s_list[kFp64List];
    __shared__ int s_nlist;
    if (threadIdx.x == 0) s_nlist = 0;
    __syncthreads();
    const unsigned* w = reinterpret_cast<const unsigned*>(minmax + 2);
    const float mn_e = from_ordered32(w[0]), mx_e = from_ordered32(w[1]);
    const float band = est_band<FLAG>(mx_e);
    double emn = kMaxDouble, emx = kMinDouble;
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        const double2 h = field[i];
        bool ok;
        const float e = estimate<FLAG>(h, ok);
        if (ok && (e <= mn_e + band || e >= mx_e - band)) {
            const int slot = atomicAdd(&s_nlist, 1);
            if (slot < kFp64List) {
                s_list[slot] = i;
            } else {
                const double x = encode_value(h, FLAG);
                if (x < emn) emn = x;
                if (x > emx) emx = x;
            }
        }
    }
    __syncthreads();
    for (int k = threadIdx.x; k < min(s_nlist, kFp64List); k += blockDim.x) {
        const double x = encode_value(field[s_list[k]], FLAG);
        if (x < emn) emn = x;
        if (x > emx) emx = x;
    }
    fold_exact(emn, emx, minmax);
}

// pass 3: the codes
template <int FLAG>
__global__ void __launch_bounds__(256) est_codes_kernel(const double2* __restrict__ field, int64_t n,
                                                        const unsigned long long* __restrict__ minmax,
                                                        uint8_t* __restrict__ out) {
    const double mn = from_ordered(minmax[0]);
    const double mx = from_ordered(minmax[1]);
    const double gap = __dsub_rn(mx, mn);
    const bool usable = gap > 0.0 && gap < 1e30 && mn > -1e30 && mn < 1e30;
    const float mn_f = (float)mn, sc_f = usable ? (float)(255.0 / gap) : 0.f;
    const float err = FLAG == 0 ? kPhaseErr : kAmpErrRel * (float)fmax(fabs(mx), fabs(mn));
    // estimate error in code units, the FP32 rounding of the code itself on top
    const float margin = 2.f * err * sc_f + 1e-4f;
    __shared__ int64_t s_list[kFp64List];
    __shared__ int s_nlist;
    if (threadIdx.x == 0) s_nlist = 0;
    __syncthreads();
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        bool ok;
        const float e = estimate<FLAG>(field[i], ok);
        uint32_t code;
        if (!code_fast(ok ? e : __int_as_float(0x7fc00000), usable, mn_f, sc_f, margin, code)) {
            const int slot = atomicAdd(&s_nlist, 1);
            if (slot < kFp64List) {
                s_list[slot] = i;
                code = 0u;   // written below
            } else {
                code = code_exact<FLAG>(field + i, mn, gap);
            }
        }
        out[i] = (uint8_t)code;
    }
    __syncthreads();   // orders the stores above before those below
    for (int k = threadIdx.x; k < min(s_nlist, kFp64List); k += blockDim.x)
        out[s_list[k]] = (uint8_t)code_exact<FLAG>(field + s_list[k], mn, gap);
}

// Single pass of the codes, for fields whose FP32 estimates fit in the
// shared memory of the CTAs the GPU holds at once (cooperative launch):
// every CTA owns `per` consecutive pixels (a multiple of 32) and every
// thread four consecutive ones at a time (four 16-byte loads in flight, one
// 4-byte store of codes):
//   1. reads them once, keeps their estimates in shared memory (NaN where
//      there is none) and reduces its estimated min/max;
//   2. computes in FP64 the pixels within the band of its own estimated
//      extremes (the pixel holding the CTA's exact extreme is among them, so
//      the grid's exact extremes are found) and those without an estimate,
//      and folds them into the exact words;
//   3. waits at a grid barrier (all CTAs are resident; the wait is bounded by
//      %globaltimer and records a timeout in word [4], after which the CTA
//      writes zero codes);
//   4. writes every code its cached estimate decides (code_fast), then the
//      others in FP64 (code_exact).
// The field is read once (plus the few FP64 pixels); words [3] and [4]
// (barrier count, timeout) are zeroed by init_est_minmax_kernel. `out` is
// 4-byte aligned.
template <int FLAG>
__global__ void __launch_bounds__(256) fused_codes_kernel(const double2* __restrict__ field, int64_t n, int64_t per,
                                                          unsigned long long* __restrict__ minmax,
                                                          uint8_t* __restrict__ out) {
    extern __shared__ float4 s_est4[];
    __shared__ float s_red[2][8];
    __shared__ int s_list[kFp64List];
    __shared__ int s_nlist;
    if (threadIdx.x == 0) s_nlist = 0;
    const int64_t base = (int64_t)blockIdx.x * per;
    const int cnt = base < n ? (int)min(per, n - base) : 0;
    const double2* fb = field + base;
    const float qnan = __int_as_float(0x7fc00000);
    float mn = __int_as_float(0x7f800000), mx = -mn;
    double emn = kMaxDouble, emx = kMinDouble;
    for (int j = 4 * threadIdx.x; j < cnt; j += 4 * blockDim.x) {
        double2 h[4];
#pragma unroll
        for (int k = 0; k < 4; ++k) h[k] = (j + k < cnt) ? fb[j + k] : make_double2(0.0, 0.0);
        float e[4];
#pragma unroll
        for (int k = 0; k < 4; ++k) {
            bool ok;
            e[k] = estimate<FLAG>(h[k], ok);
            if (j + k >= cnt) {
                e[k] = qnan;
            } else if (ok) {
                mn = fminf(mn, e[k]);
                mx = fmaxf(mx, e[k]);
            } else {
                e[k] = qnan;
                const double x = encode_value(h[k], FLAG);
                if (x < emn) emn = x;
                if (x > emx) emx = x;
            }
        }
        s_est4[j >> 2] = make_float4(e[0], e[1], e[2], e[3]);
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        mn = fminf(mn, __shfl_xor_sync(0xffffffffu, mn, o));
        mx = fmaxf(mx, __shfl_xor_sync(0xffffffffu, mx, o));
    }
    if ((threadIdx.x & 31) == 0) {
        s_red[0][threadIdx.x >> 5] = mn;
        s_red[1][threadIdx.x >> 5] = mx;
    }
    __syncthreads();
    for (int k = 0; k < (int)(blockDim.x >> 5); ++k) {
        mn = fminf(mn, s_red[0][k]);
        mx = fmaxf(mx, s_red[1][k]);
    }
    const float band = est_band<FLAG>(mx);
    for (int j = 4 * threadIdx.x; j < cnt; j += 4 * blockDim.x) {
        const float4 e4 = s_est4[j >> 2];
        const float e[4] = {e4.x, e4.y, e4.z, e4.w};
#pragma unroll
        for (int k = 0; k < 4; ++k) {
            if (e[k] == e[k] && (e[k] <= mn + band || e[k] >= mx - band)) {
                const int slot = atomicAdd(&s_nlist, 1);
                if (slot < kFp64List) {
                    s_list[slot] = j + k;
                } else {
                    const double x = encode_value(fb[j + k], FLAG);
                    if (x < emn) emn = x;
                    if (x > emx) emx = x;
                }
            }
        }
    }
    __syncthreads();
    for (int i = threadIdx.x; i < min(s_nlist, kFp64List); i += blockDim.x) {
        const double x = encode_value(fb[s_list[i]], FLAG);
        if (x < emn) emn = x;
        if (x > emx) emx = x;
    }
    fold_exact(emn, emx, minmax);
    // grid barrier
    __shared__ int s_ok;
    __syncthreads();
    if (threadIdx.x == 0) {
        s_nlist = 0;   // the list again, for the boundary pixels
        __threadfence();
        atomicAdd(&minmax[3], 1ull);
        const uint64_t t0 = global_ns_enc();
        bool ok = true;
        while (*(volatile unsigned long long*)&minmax[3] < (unsigned long long)gridDim.x) {
            if (global_ns_enc() - t0 > 2000000000ull) {
                ok = false;
                atomicExch(&minmax[4], 1ull);
                break;
            }
            __nanosleep(128);
        }
        __threadfence();
        s_ok = ok;
    }
    __syncthreads();
    const double gmn = from_ordered(__ldcg(&minmax[0]));
    const double gmx = from_ordered(__ldcg(&minmax[1]));
    const double gap = __dsub_rn(gmx, gmn);
    const bool usable = gap > 0.0 && gap < 1e30 && gmn > -1e30 && gmn < 1e30;
    const float mn_f = (float)gmn, sc_f = usable ? (float)(255.0 / gap) : 0.f;
    const float err = FLAG == 0 ? kPhaseErr : kAmpErrRel * (float)fmax(fabs(gmx), fabs(gmn));
    const float margin = 2.f * err * sc_f + 1e-4f;
    uint8_t* ob = out + base;
    for (int j = 4 * threadIdx.x; j < cnt; j += 4 * blockDim.x) {
        const float4 e4 = s_est4[j >> 2];
        const float e[4] = {e4.x, e4.y, e4.z, e4.w};
        uint32_t c[4] = {0u, 0u, 0u, 0u};
        if (s_ok) {
#pragma unroll
            for (int k = 0; k < 4; ++k) {
                if (j + k < cnt && !code_fast(e[k], usable, mn_f, sc_f, margin, c[k])) {
                    const int slot = atomicAdd(&s_nlist, 1);
                    if (slot < kFp64List) {
                        s_list[slot] = j + k;
                        c[k] = 0u;   // written below
                    } else {
                        c[k] = code_exact<FLAG>(fb + j + k, gmn, gap);
                    }
                }
            }
        }
        if (j + 4 <= cnt) {
            *reinterpret_cast<uint32_t*>(ob + j) = c[0] | c[1] << 8 | c[2] << 16 | c[3] << 24;
        } else {
            for (int k = 0; j + k < cnt; ++k) ob[j + k] = (uint8_t)c[k];
        }
    }
    __syncthreads();   // orders the 4-byte stores above before the byte stores below
    for (int i = threadIdx.x; i < min(s_nlist, kFp64List); i += blockDim.x) {
        const int j = s_list[i];
        ob[j] = (uint8_t)code_exact<FLAG>(fb + j, gmn, gap);
    }
}

}  // namespace

namespace {
int grid_for(int64_t n, int threads) {
    int dev = 0, sms = 152;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    const int64_t want = (n + threads - 1) / threads;
    return (int)(want < (int64_t)sms * 8 ? want : (int64_t)sms * 8);
}
// Cooperative single-pass codes when the grid of resident CTAs can cache
// every estimate (4 bytes a pixel) and the codes buffer is 4-byte aligned.
// False otherwise (the three-pass kernels run instead).
bool launch_fused_codes(const double2* d_field, int64_t n, int flag, unsigned long long* d_minmax,
                        uint8_t* d_codes, cudaStream_t stream) {
    // not inside a stream capture (a plan): there the three-pass kernels run
    cudaStreamCaptureStatus cap = cudaStreamCaptureStatusNone;
    if (cudaStreamIsCapturing(stream, &cap) != cudaSuccess || cap != cudaStreamCaptureStatusNone) {
        cudaGetLastError();
        return false;
    }
    if (((uintptr_t)d_codes & 3u) != 0) return false;   // the kernel stores four codes at a time
    int dev = 0, sms = 0, coop = 0;
    if (cudaGetDevice(&dev) != cudaSuccess) return false;
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    cudaDeviceGetAttribute(&coop, cudaDevAttrCooperativeLaunch, dev);
    if (!coop || sms <= 0) return false;
    const void* fn = flag == 0 ? (const void*)fused_codes_kernel<0> : (const void*)fused_codes_kernel<1>;
    for (int bps = 8; bps >= 1; bps >>= 1) {
        const int64_t grid = (int64_t)sms * bps;
        const int64_t per = ((n + grid - 1) / grid + 31) / 32 * 32;
        const size_t smem = (size_t)per * sizeof(float);
        if (smem > 200 * 1024) continue;
        if (cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem) != cudaSuccess) {
            cudaGetLastError();
            return false;
        }
        int fit = 0;
        if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&fit, fn, 256, smem) != cudaSuccess || fit < bps) continue;
        count_launches(2);
        init_est_minmax_kernel<<<1, 1, 0, stream>>>(d_minmax);
        void* args[] = {(void*)&d_field, (void*)&n, (void*)&per, (void*)&d_minmax, (void*)&d_codes};
        const cudaError_t e = cudaLaunchCooperativeKernel(fn, dim3((unsigned)grid), dim3(256), args, smem, stream);
        if (e != cudaSuccess) {
            cudaGetLastError();
            return false;   // the three-pass kernels run instead (init is repeated there)
        }
        return true;
    }
    return false;
}

}  // namespace

void launch_normalize(const double* d_encoded, int n_channels, int64_t n_pixels, uint8_t* d_normalized,
                      unsigned long long* d_minmax, cudaStream_t stream) {
    const int64_t n = (int64_t)n_channels * n_pixels;
    if (n <= 0) return;
    const int threads = 256, blocks = grid_for(n, threads);
    count_launches(3);
    init_minmax_kernel<<<1, 1, 0, stream>>>(d_minmax, 2);
    minmax_kernel<<<blocks, threads, 0, stream>>>(d_encoded, n, d_minmax);
    normalize_kernel<<<blocks, threads, 0, stream>>>(nullptr, d_encoded, n, 0, d_minmax, d_normalized);
}

void launch_encode(const double2* d_field, int n_channels, int64_t n_pixels, int encode_flag,
                   double* d_encoded, uint8_t* d_normalized, unsigned long long* d_minmax,
                   cudaStream_t stream) {
    const int64_t n = (int64_t)n_channels * n_pixels;
    if (n <= 0) return;
    const int threads = 256, blocks = grid_for(n, threads);
    if (encode_flag >= (int)OPHPC_ENCODE_SIMPLENI) {
        // d_encoded is required (the caller provides scratch) and in/out
        const int per = grid_for(n_pixels, threads);
        const dim3 grid((unsigned)per, (unsigned)n_channels);
        count_launches(d_normalized ? 5 : 3);
        init_minmax_kernel<<<1, 1, 0, stream>>>(d_minmax, 5);
        chan_absmax_kernel<<<grid, threads, 0, stream>>>(d_field, n_pixels, encode_flag, d_minmax + 2);
        encode_normalised_kernel<<<grid, threads, 0, stream>>>(d_field, n_pixels, encode_flag, d_minmax + 2,
                                                              d_encoded);
        if (d_normalized) {
            minmax_kernel<<<blocks, threads, 0, stream>>>(d_encoded, n, d_minmax);
            normalize_kernel<<<blocks, threads, 0, stream>>>(nullptr, d_encoded, n, 0, d_minmax, d_normalized);
        }
        return;
    }
    if (!d_encoded && d_normalized && (encode_flag == 0 || encode_flag == 1)) {
        // codes only: FP32 estimates, FP64 where they cannot decide; one
        // pass when the estimates fit in the resident CTAs' shared memory
        if (launch_fused_codes(d_field, n, encode_flag, d_minmax, d_normalized, stream)) return;
        count_launches(4);
        init_est_minmax_kernel<<<1, 1, 0, stream>>>(d_minmax);
        if (encode_flag == 0) {
            est_minmax_kernel<0><<<blocks, threads, 0, stream>>>(d_field, n, d_minmax);
            refine_minmax_kernel<0><<<blocks, threads, 0, stream>>>(d_field, n, d_minmax);
            est_codes_kernel<0><<<blocks, threads, 0, stream>>>(d_field, n, d_minmax, d_normalized);
        } else {
            est_minmax_kernel<1><<<blocks, threads, 0, stream>>>(d_field, n, d_minmax);
            refine_minmax_kernel<1><<<blocks, threads, 0, stream>>>(d_field, n, d_minmax);
            est_codes_kernel<1><<<blocks, threads, 0, stream>>>(d_field, n, d_minmax, d_normalized);
        }
        return;
    }
    count_launches(d_normalized ? 3 : 2);
    init_minmax_kernel<<<1, 1, 0, stream>>>(d_minmax, 2);
    encode_minmax_kernel<<<blocks, threads, 0, stream>>>(d_field, n, encode_flag, d_encoded, d_minmax);
    if (d_normalized)
        normalize_kernel<<<blocks, threads, 0, stream>>>(d_field, d_encoded, n, encode_flag, d_minmax,
                                                         d_normalized);
}

}  // namespace ophpc
