// Batched FP64 Stockham FFT passes (declared in pc_fft.cuh).
//
// Pass p of radix R, with Ns the product of the earlier radices: for every
// j in [0, n/R), k = j mod Ns,
//   v[r] = in[j + r n/R] * w^(k r),  w = e^(-+2 pi i / (Ns R)),  r = 0..R-1
//   v = DFT_R(v)
//   out[(j / Ns) Ns R + k + r Ns] = v[r]
// After the last pass the output is the DFT in natural order (the Stockham
// auto-sort formulation; no bit reversal).
#include "pc_fft.cuh"
#include "pc_common.cuh"

#include <cmath>

namespace ophpc {
namespace {

__device__ __forceinline__ double2 cmul(double2 a, double2 b) {
    return make_double2(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x);
}
__device__ __forceinline__ double2 cadd(double2 a, double2 b) { return make_double2(a.x + b.x, a.y + b.y); }
__device__ __forceinline__ double2 csub(double2 a, double2 b) { return make_double2(a.x - b.x, a.y - b.y); }
// a * (-i) for the forward transform, a * (+i) for the inverse
__device__ __forceinline__ double2 rot_q(double2 a, bool inv) {
    return inv ? make_double2(-a.y, a.x) : make_double2(a.y, -a.x);
}

template <int R>
__device__ __forceinline__ void dft(double2* v, bool inv);

template <>
__device__ __forceinline__ void dft<2>(double2* v, bool) {
    const double2 a = v[0], b = v[1];
    v[0] = cadd(a, b);
    v[1] = csub(a, b);
}

template <>
__device__ __forceinline__ void dft<4>(double2* v, bool inv) {
    const double2 s02 = cadd(v[0], v[2]), d02 = csub(v[0], v[2]);
    const double2 s13 = cadd(v[1], v[3]), d13 = rot_q(csub(v[1], v[3]), inv);
    v[0] = cadd(s02, s13);
    v[2] = csub(s02, s13);
    v[1] = cadd(d02, d13);
    v[3] = csub(d02, d13);
}

template <>
__device__ __forceinline__ void dft<8>(double2* v, bool inv) {
    // two radix-4 DFTs over the even and odd entries, then radix-2 with
    // the eighth roots of unity
    double2 e[4] = {v[0], v[2], v[4], v[6]}, o[4] = {v[1], v[3], v[5], v[7]};
    dft<4>(e, inv);
    dft<4>(o, inv);
    const double h = 0.70710678118654752440;
    const double sg = inv ? 1.0 : -1.0;
    // o[q] *= e^(sg i 2 pi q / 8)
    o[1] = make_double2(h * (o[1].x - sg * o[1].y), h * (o[1].y + sg * o[1].x));
    o[2] = rot_q(o[2], inv);
    o[3] = make_double2(h * (-o[3].x - sg * o[3].y), h * (-o[3].y + sg * o[3].x));
#pragma unroll
    for (int q = 0; q < 4; ++q) {
        v[q] = cadd(e[q], o[q]);
        v[q + 4] = csub(e[q], o[q]);
    }
}

// Radix 7: the direct sum with the 7th roots of unity, cos(2 pi m / 7) and
// sin(2 pi m / 7) as literal constants.
template <int R>
__device__ __forceinline__ double2 root(int m, double sg);

template <>
__device__ __forceinline__ double2 root<7>(int m, double sg) {
    constexpr double c[7] = {1.00000000000000000000, 0.62348980185873359439, -0.22252093395631433737, -0.90096886790241903498, -0.90096886790241914600, -0.22252093395631458717, 0.62348980185873337234};
    constexpr double s[7] = {0.00000000000000000000, 0.78183148246802980363, 0.97492791218182361934, 0.43388373911755823142, -0.43388373911755800938, -0.97492791218182361934, -0.78183148246802991466};
    return make_double2(c[m], sg * s[m]);
}

template <int R>
__device__ __forceinline__ void dft_direct(double2* v, bool inv) {
    double2 out[R];
    const double sg = inv ? 1.0 : -1.0;
#pragma unroll
    for (int q = 0; q < R; ++q) {
        double2 acc = v[0];
#pragma unroll
        for (int r = 1; r < R; ++r) {
            const int m = (q * r) % R;
            acc = cadd(acc, cmul(v[r], root<R>(m, sg)));
        }
        out[q] = acc;
    }
#pragma unroll
    for (int q = 0; q < R; ++q) v[q] = out[q];
}
// Radix 3 and 5 from the sums and differences of the entries paired by
// symmetry (the textbook small DFTs: X_k and X_(R-k) share the real-cosine
// part and differ in the sign of the sine part), 4.7 and 7.2 FP64
// operations an element against 12 and 24 for the direct sum; GB300's FP64
// pipe is narrow, so a pass costs its operation count. Constants are the
// correctly rounded cos and sin of 2 pi / 3, 2 pi / 5 and 4 pi / 5.
template <>
__device__ __forceinline__ void dft<3>(double2* v, bool inv) {
    constexpr double s = 0.866025403784438646763723170753;   // sin(2 pi / 3)
    const double2 t1 = cadd(v[1], v[2]), t2 = csub(v[1], v[2]);
    const double2 a = make_double2(__fma_rn(-0.5, t1.x, v[0].x), __fma_rn(-0.5, t1.y, v[0].y));
    const double2 b = rot_q(make_double2(s * t2.x, s * t2.y), inv);
    v[0] = cadd(v[0], t1);
    v[1] = cadd(a, b);
    v[2] = csub(a, b);
}
template <>
__device__ __forceinline__ void dft<5>(double2* v, bool inv) {
    constexpr double c1 = 0.309016994374947424102293417183;    // cos(2 pi / 5)
    constexpr double c2 = -0.809016994374947424102293417183;   // cos(4 pi / 5)
    constexpr double s1 = 0.951056516295153572116439333379;    // sin(2 pi / 5)
    constexpr double s2 = 0.587785252292473129168705954639;    // sin(4 pi / 5)
    const double2 t1 = cadd(v[1], v[4]), t2 = cadd(v[2], v[3]);
    const double2 t3 = csub(v[1], v[4]), t4 = csub(v[2], v[3]);
    const double2 a1 = make_double2(__fma_rn(c2, t2.x, __fma_rn(c1, t1.x, v[0].x)),
                                    __fma_rn(c2, t2.y, __fma_rn(c1, t1.y, v[0].y)));
    const double2 a2 = make_double2(__fma_rn(c1, t2.x, __fma_rn(c2, t1.x, v[0].x)),
                                    __fma_rn(c1, t2.y, __fma_rn(c2, t1.y, v[0].y)));
    const double2 b1 = rot_q(make_double2(__fma_rn(s2, t4.x, s1 * t3.x), __fma_rn(s2, t4.y, s1 * t3.y)), inv);
    const double2 b2 = rot_q(make_double2(__fma_rn(-s1, t4.x, s2 * t3.x), __fma_rn(-s1, t4.y, s2 * t3.y)), inv);
    v[0] = cadd(v[0], cadd(t1, t2));
    v[1] = cadd(a1, b1);
    v[4] = csub(a1, b1);
    v[2] = cadd(a2, b2);
    v[3] = csub(a2, b2);
}
template <>
__device__ __forceinline__ void dft<7>(double2* v, bool inv) { dft_direct<7>(v, inv); }

// One pass over `lines` lines. Thread x runs along the contiguous
// direction: the butterfly index j for rows, the line for columns.
template <int R>
__global__ void __launch_bounds__(256) fft_pass_kernel(const double2* __restrict__ in, double2* __restrict__ out,
                                                       int n, int ns, const double2* __restrict__ tw, int64_t lines,
                                                       int64_t elem_stride, int64_t line_stride, int inv,
                                                       int rows) {
    const int m = n / R;
    int64_t j, l;
    if (rows) {
        j = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
        l = (int64_t)blockIdx.y * blockDim.y + threadIdx.y;
    } else {
        l = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
        j = (int64_t)blockIdx.y * blockDim.y + threadIdx.y;
    }
    if (j >= m || l >= lines) return;
    const int k = (int)(j % ns);
    const double2* src = in + l * line_stride;
    double2 v[R];
#pragma unroll
    for (int r = 0; r < R; ++r) v[r] = src[(j + (int64_t)r * m) * elem_stride];
    if (ns > 1) {
        const double2* t = tw + (int64_t)k * (R - 1);
#pragma unroll
        for (int r = 1; r < R; ++r) {
            double2 w = t[r - 1];
            if (inv) w.y = -w.y;
            v[r] = cmul(v[r], w);
        }
    }
    dft<R>(v, inv != 0);
    const int64_t base = (j / ns) * (int64_t)ns * R + k;
    double2* dst = out + l * line_stride;
#pragma unroll
    for (int r = 0; r < R; ++r) dst[(base + (int64_t)r * ns) * elem_stride] = v[r];
}

// Twiddles of one pass: t[k (R-1) + r - 1] = e^(-2 pi i k r / (Ns R)).
__global__ void twiddle_kernel(double2* t, int ns, int R) {
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= (int64_t)ns * (R - 1)) return;
    const int64_t k = i / (R - 1), r = i % (R - 1) + 1;
    const int64_t nr = (int64_t)ns * R;
    const int64_t e = (k * r) % nr;
    double s, c;
    sincospi(-2.0 * (double)e / (double)nr, &s, &c);
    t[i] = make_double2(c, s);
}

int factor(int n, int* radix) {
    int count = 0;
    const int order[] = {8, 4, 2, 3, 5, 7};
    for (int r : order) {
        while (n % r == 0 && count < kFftMaxPasses) {
            radix[count++] = r;
            n /= r;
        }
    }
    return n == 1 ? count : -1;
}

template <int R>
void launch_pass(const double2* in, double2* out, const FftPlan& p, int pass, int64_t lines, int64_t elem_stride,
                 int64_t line_stride, bool inv, cudaStream_t s) {
    const int64_t m = p.n / R;
    const bool rows = elem_stride == 1;
    dim3 block, grid;
    if (rows) {
        block = dim3(m >= 128 ? 128 : 32, m >= 128 ? 2 : 8);
        grid = dim3((unsigned)((m + block.x - 1) / block.x), (unsigned)((lines + block.y - 1) / block.y));
    } else {
        block = dim3(32, 8);
        grid = dim3((unsigned)((lines + 31) / 32), (unsigned)((m + 7) / 8));
    }
    count_launches(1);
    fft_pass_kernel<R><<<grid, block, 0, s>>>(in, out, p.n, p.ns[pass], p.twiddles + p.tw_offset[pass], lines,
                                              elem_stride, line_stride, inv ? 1 : 0, rows ? 1 : 0);
}

}  // namespace

bool fft_supported(int n) {
    int r[kFftMaxPasses];
    return n > 0 && factor(n, r) >= 0;
}

int64_t fft_twiddle_count(int n) {
    int r[kFftMaxPasses];
    const int c = factor(n, r);
    if (c < 0) return 0;
    int64_t total = 0, ns = 1;
    for (int i = 0; i < c; ++i) {
        total += ns * (r[i] - 1);
        ns *= r[i];
    }
    return total > 0 ? total : 1;
}

bool fft_plan_init(FftPlan* p, int n, double2* tw, cudaStream_t s) {
    const int c = factor(n, p->radix);
    if (c < 0) return false;
    p->n = n;
    p->passes = c;
    p->twiddles = tw;
    int64_t off = 0, ns = 1;
    for (int i = 0; i < c; ++i) {
        p->ns[i] = (int)ns;
        p->tw_offset[i] = off;
        const int64_t cnt = ns * (p->radix[i] - 1);
        if (cnt > 0) {
            count_launches(1);
            twiddle_kernel<<<(unsigned)((cnt + 255) / 256), 256, 0, s>>>(tw + off, (int)ns, p->radix[i]);
        }
        off += cnt;
        ns *= p->radix[i];
    }
    return true;
}

int fft_run(const FftPlan& p, double2* const buf[2], int64_t lines, int64_t elem_stride, int64_t line_stride,
            bool inverse, cudaStream_t s) {
    int cur = 0;
    for (int i = 0; i < p.passes; ++i) {
        const double2* in = buf[cur];
        double2* out = buf[cur ^ 1];
        switch (p.radix[i]) {
            case 8: launch_pass<8>(in, out, p, i, lines, elem_stride, line_stride, inverse, s); break;
            case 4: launch_pass<4>(in, out, p, i, lines, elem_stride, line_stride, inverse, s); break;
            case 2: launch_pass<2>(in, out, p, i, lines, elem_stride, line_stride, inverse, s); break;
            case 3: launch_pass<3>(in, out, p, i, lines, elem_stride, line_stride, inverse, s); break;
            case 5: launch_pass<5>(in, out, p, i, lines, elem_stride, line_stride, inverse, s); break;
            default: launch_pass<7>(in, out, p, i, lines, elem_stride, line_stride, inverse, s); break;
        }
        cur ^= 1;
    }
    return cur;
}

}  // namespace ophpc
