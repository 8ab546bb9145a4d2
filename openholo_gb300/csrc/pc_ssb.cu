// Single-sideband encodings of the point-cloud hologram, FP64 on the
// library's own FFT passes (pc_fft.cuh).
//
// ENCODE_SSB — ophPointCloud::encoding(ENCODE_SSB, passband) runs
// ophPointCloud::encodeHologram (ophgen/src/ophPointCloud.cpp:191-240) per
// channel: T = B(F(H)) with F = S FFT S and B = S IFFT S (Openholo::fft2
// with its default shift, Openholo/src/Openholo.cpp:698-745; S is
// Openholo::fftShift, :749-767; FFTW's unnormalised forward and backward
// transforms), then
//   m_lpEncoded[i] = Re(T[i]) * (cos X cos Y - sin X sin Y),
//   X = pi x shift_x / ppX, x = -ssX/2 + ppX w + ppX/2,
//   Y = pi y shift_y / ppY, y = (ssY - ppY) - ppY h     (w, h: column, row).
// The passband and the band limit are not used there, and are not here.
//
// ENCODE_OFFSSB — ophGen::encoding(flag, passband) (ophgen/src/ophGen.cpp:
// 882-921) encodes the field of channel 0 into every channel: ophGen::
// freqShift(H, 0, 100) (:1079-1098: F, circShift by 100 along the second
// index of Openholo's x-major [x][y] view, function.h:273-283, B), then
// ophGen::singleSideBand (:1023-1077: F, one half of the spectrum zeroed —
// SSB_LEFT the columns from nX/2 on in every row, SSB_RIGHT the first nX/2
// columns, SSB_TOP the elements from N/2 on, SSB_BOTTOM the first N/2 — B,
// the real part, and oph::normalize to [0, 1] with minOfArr / maxOfArr,
// function.h:79-99, 188-196).
//
// SIDEBAND — ophGen::encodeSideBand(passband) (ophgen/src/ophGen.cpp:
// 1607-1653, encodeSideBand_CPU :1655-1695, getShiftPhaseValue :1741-1781)
// per channel: the field cropped to the central half along one axis (all
// columns and rows [c1, c2] for SSB_TOP / SSB_BOTTOM, all rows and columns
// [c1, c2] for SSB_LEFT / SSB_RIGHT; h = floor(n/2), c1 = h - floor(h/2) - 1,
// c2 = c1 + h - 1), B normalised by N, times the carrier e^{i theta} and the
// real part; theta = +-2 pi yy / (4 ppY), yy = ssY/2 - ppY r - ppY (TOP +,
// BOTTOM -), or theta = -+2 pi xx / (4 ppX), xx = -ssX/2 - ppX c - ppX (LEFT
// -, RIGHT +). That path's FFTW plan reads FFTW's own buffer, so the
// reference's output is well defined and pins this one
// (tests/golden/sideband.npz).
//
// The reference runs these transforms through FFTW plans whose input buffer
// aliases the array being shifted, so its own outputs are not reproducible;
// what is computed here is what the code describes, restated in FP64 numpy
// by the oracle (oracle.ssb_encode). FP64 arithmetic, explicitly rounded
// where the reference's order of operations matters.
#include "pc_common.cuh"
#include "pc_fft.cuh"
#include "ophpc.h"

#include <cstring>
#include <string>

namespace ophpc {
namespace {

constexpr double kPiSsb = 3.14159265358979323846;
// ssb_encode_device's flag for ophGen::encodeSideBand (not an ENCODE_FLAG)
constexpr uint32_t kEncodeSideband = 0x10000u;
constexpr double kMaxDoubleSsb = 1.7976931348623158e+308;
constexpr double kMinDoubleSsb = 2.2250738585072014e-308;

// out[(i - nx/2) mod nx + ((j - ny/2) mod ny) nx] = in[i + j nx]
__global__ void ssb_shift_kernel(const double2* __restrict__ in, double2* __restrict__ out, int nx, int ny) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x, j = blockIdx.y;
    if (i >= nx) return;
    int ti = i - (nx >> 1), tj = j - (ny >> 1);
    if (ti < 0) ti += nx;
    if (tj < 0) tj += ny;
    out[ti + (int64_t)tj * nx] = in[i + (int64_t)j * nx];
}

// Openholo's circShift(src, dst, 0, shift_y, xdim, ydim) over the flat
// array: element i * ydim + j moves to i * ydim + (j + shift_y) mod ydim.
__global__ void ssb_circshift_kernel(const double2* __restrict__ in, double2* __restrict__ out, int64_t n, int ydim,
                                     int shift_y) {
    for (int64_t f = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; f < n; f += (int64_t)gridDim.x * blockDim.x) {
        const int64_t i = f / ydim;
        const int j = (int)(f - i * ydim);
        int tj = (j + shift_y) % ydim;
        if (tj < 0) tj += ydim;
        out[i * ydim + tj] = in[f];
    }
}

// Zeroes one half of the (shifted) spectrum, as singleSideBand's memsets do.
__global__ void ssb_passband_kernel(double2* __restrict__ as, int nx, int ny, int passband) {
    const int64_t n = (int64_t)nx * ny, half_n = n >> 1;
    const int half_nx = nx >> 1;
    for (int64_t f = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; f < n; f += (int64_t)gridDim.x * blockDim.x) {
        const int c = (int)(f % nx);
        bool zero;
        switch (passband) {
            case OPHPC_SSB_LEFT: zero = c >= half_nx && c < 2 * half_nx; break;
            case OPHPC_SSB_RIGHT: zero = c < half_nx; break;
            case OPHPC_SSB_TOP: zero = f >= half_n && f < 2 * half_n; break;
            default: zero = f < half_n; break;   // OPHPC_SSB_BOTTOM
        }
        if (zero) as[f] = make_double2(0.0, 0.0);
    }
}

// The field inside the crop rectangle [x1, x2] x [y1, y2] (inclusive), zero
// elsewhere.
__global__ void ssb_crop_kernel(const double2* __restrict__ in, double2* __restrict__ out, int nx, int ny, int x1,
                                int x2, int y1, int y2) {
    const int x = blockIdx.x * blockDim.x + threadIdx.x, y = blockIdx.y;
    if (x >= nx) return;
    const int64_t i = (int64_t)y * nx + x;
    out[i] = (x >= x1 && x <= x2 && y >= y1 && y <= y2) ? in[i] : make_double2(0.0, 0.0);
}

// encodeSideBand_CPU's carrier angle theta of one row (SSB_TOP / _BOTTOM)
// or column (SSB_LEFT / _RIGHT), k < the axis length: cs[k] = (cos, sin),
// evaluated once per row or column instead of at every pixel (the same
// values; FP64 sin and cos are costly on GB300's narrow FP64 pipe).
__global__ void ssb_carrier_kernel(double2* __restrict__ cs, int pnx, int pny, double ppx, double ppy, int passband) {
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    const bool rows = passband == OPHPC_SSB_TOP || passband == OPHPC_SSB_BOTTOM;
    if (k >= (rows ? pny : pnx)) return;
    const double two_pi = 2 * kPiSsb;
    double theta;
    if (rows) {
        const double ssy = __dmul_rn((double)pny, ppy);
        const double yy = __dsub_rn(__dsub_rn(ssy / 2.0, __dmul_rn(ppy, (double)k)), ppy);
        theta = __dmul_rn(two_pi, __ddiv_rn(passband == OPHPC_SSB_TOP ? yy : -yy, __dmul_rn(4.0, ppy)));
    } else {
        const double ssx = __dmul_rn((double)pnx, ppx);
        const double xx = __dsub_rn(__dsub_rn(-ssx / 2.0, __dmul_rn(ppx, (double)k)), ppx);
        theta = __dmul_rn(two_pi, __ddiv_rn(passband == OPHPC_SSB_LEFT ? -xx : xx, __dmul_rn(4.0, ppx)));
    }
    cs[k] = make_double2(cos(theta), sin(theta));
}

// encodeSideBand_CPU's carrier and real part (one channel); t is the
// unnormalised inverse transform, divided by n here as fft2's bNormalized
// does; cs from ssb_carrier_kernel.
__global__ void ssb_fringe_kernel(const double2* __restrict__ t, double* __restrict__ enc, int pnx, int pny,
                                  const double2* __restrict__ cs, int passband) {
    const int c = blockIdx.x * blockDim.x + threadIdx.x, r = blockIdx.y;
    if (c >= pnx) return;
    const double n = (double)((int64_t)pnx * pny);
    const double2 ct = cs[(passband == OPHPC_SSB_TOP || passband == OPHPC_SSB_BOTTOM) ? r : c];
    const int64_t i = (int64_t)r * pnx + c;
    const double2 v = t[i];
    const double re = __ddiv_rn(v.x, n), im = __ddiv_rn(v.y, n);
    enc[i] = __dsub_rn(__dmul_rn(re, ct.x), __dmul_rn(im, ct.y));
}

// cos and sin of encodeHologram's X for every column (cs[0, pnx)) and Y for
// every row (cs[pnx, pnx + pny)), once each instead of at every pixel (the
// same values).
__global__ void ssb_axis_kernel(double2* __restrict__ cs, int pnx, int pny, double ppx, double ppy, double shift_x,
                                double shift_y) {
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= pnx + pny) return;
    double a;
    if (k < pnx) {
        const double ssx = __dmul_rn((double)pnx, ppx);
        const double x = __dadd_rn(__dadd_rn(-(ssx / 2), __dmul_rn(ppx, (double)k)), ppx / 2);
        a = __ddiv_rn(__dmul_rn(__dmul_rn(kPiSsb, x), shift_x), ppx);
    } else {
        const double ssy = __dmul_rn((double)pny, ppy);
        const double y = __dsub_rn(__dsub_rn(ssy, ppy), __dmul_rn(ppy, (double)(k - pnx)));
        a = __ddiv_rn(__dmul_rn(__dmul_rn(kPiSsb, y), shift_y), ppy);
    }
    cs[k] = make_double2(cos(a), sin(a));
}

// encodeHologram's shifted real part into enc (one channel): with X of the
// column and Y of the row (cs from ssb_axis_kernel),
// Re(T) (cos X cos Y - sin X sin Y).
__global__ void ssb_point_cloud_kernel(const double2* __restrict__ t, double* __restrict__ enc, int pnx, int pny,
                                       const double2* __restrict__ cs) {
    const int w = blockIdx.x * blockDim.x + threadIdx.x, h = blockIdx.y;
    if (w >= pnx) return;
    const double2 cx = cs[w], cy = cs[pnx + h];
    const double c = __dsub_rn(__dmul_rn(cx.x, cy.x), __dmul_rn(cx.y, cy.y));
    const int64_t i = (int64_t)h * pnx + w;
    const double2 v = t[i];
    // (T * (c, 0)).real()
    enc[i] = __dsub_rn(__dmul_rn(v.x, c), __dmul_rn(v.y, 0.0));
}

__device__ __forceinline__ unsigned long long ordered_ssb(double d) {
    const unsigned long long b = (unsigned long long)__double_as_longlong(d);
    return (b & 0x8000000000000000ull) ? ~b : (b | 0x8000000000000000ull);
}
__device__ __forceinline__ double unordered_ssb(unsigned long long b) {
    b = (b & 0x8000000000000000ull) ? (b & 0x7fffffffffffffffull) : ~b;
    return __longlong_as_double((long long)b);
}

__global__ void ssb_minmax_init_kernel(unsigned long long* mm) {
    mm[0] = ordered_ssb(kMaxDoubleSsb);
    mm[1] = ordered_ssb(kMinDoubleSsb);
}

// Real part into re, and minOfArr / maxOfArr of it (strict comparisons from
// MAX_DOUBLE / MIN_DOUBLE: NaNs never win) into mm.
__global__ void __launch_bounds__(256) ssb_real_minmax_kernel(const double2* __restrict__ f, int64_t n,
                                                              double* __restrict__ re, unsigned long long* mm) {
    double mn = kMaxDoubleSsb, mx = kMinDoubleSsb;
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        const double v = f[i].x;
        re[i] = v;
        if (v < mn) mn = v;
        if (v > mx) mx = v;
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        mn = fmin(mn, __shfl_xor_sync(0xffffffffu, mn, o));
        mx = fmax(mx, __shfl_xor_sync(0xffffffffu, mx, o));
    }
    if ((threadIdx.x & 31) == 0) {
        atomicMin(&mm[0], ordered_ssb(mn));
        atomicMax(&mm[1], ordered_ssb(mx));
    }
}

// oph::normalize(src, dst, N): (x - min) / (max - min) into every channel.
__global__ void ssb_unit_normalize_kernel(const double* __restrict__ re, int64_t n, int n_channels,
                                          const unsigned long long* __restrict__ mm, double* __restrict__ enc) {
    const double mn = unordered_ssb(mm[0]), mx = unordered_ssb(mm[1]);
    const double gap = __dsub_rn(mx, mn);
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        const double v = __ddiv_rn(__dsub_rn(re[i], mn), gap);
        for (int c = 0; c < n_channels; ++c) enc[(int64_t)c * n + i] = v;
    }
}

int grid_ssb(int64_t n) {
    const int64_t b = (n + 255) / 256;
    return (int)(b < 4096 ? b : 4096);
}

size_t align_ssb(size_t v) { return (v + 255) & ~(size_t)255; }

// Openholo::fft2(src, dst, nx, ny, type) with its shift: dst = S FFT S src
// (inverse: S IFFT S), unnormalised. dst may equal src; buf[0] and buf[1]
// are the transform's own.
cudaError_t shifted_fft2(const double2* src, double2* dst, double2* const buf[2], const FftPlan& px, const FftPlan& py,
                         int nx, int ny, bool inverse, cudaStream_t s) {
    const dim3 g((unsigned)((nx + 255) / 256), (unsigned)ny);
    count_launches(1);
    ssb_shift_kernel<<<g, 256, 0, s>>>(src, buf[0], nx, ny);
    const int r = fft_run(px, buf, ny, 1, nx, inverse, s);
    double2* cols[2] = {buf[r], buf[r ^ 1]};
    const int c = fft_run(py, cols, nx, nx, 1, inverse, s);
    count_launches(1);
    ssb_shift_kernel<<<g, 256, 0, s>>>(cols[c], dst, nx, ny);
    return cudaGetLastError();
}

}  // namespace

bool ssb_sizes_supported(int pnx, int pny) { return fft_supported(pnx) && fft_supported(pny); }
extern const uint32_t kSsbSidebandFlag = kEncodeSideband;

ophpc_status ssb_encode_device(cudaMemPool_t pool, const double2* d_field, int n_channels, int pnx, int pny,
                               double ppx, double ppy, uint32_t encode_flag, uint32_t passband, double shift_x,
                               double shift_y, double* d_encoded, uint8_t* d_normalized, cudaStream_t s,
                               std::string* err) {
    const int64_t n = (int64_t)pnx * pny;
    const size_t plane = align_ssb(sizeof(double2) * (size_t)n);
    const size_t tw_bytes = align_ssb(sizeof(double2) * (size_t)(fft_twiddle_count(pnx) + fft_twiddle_count(pny)));
    const size_t enc_bytes = d_encoded ? 0 : align_ssb(sizeof(double) * (size_t)n * n_channels);
    const size_t re_bytes = align_ssb(sizeof(double) * (size_t)n);
    const size_t cs_bytes = align_ssb(sizeof(double2) * (size_t)(pnx + pny));
    unsigned char* mem = nullptr;
    if (cudaMallocFromPoolAsync((void**)&mem, 4 * plane + tw_bytes + enc_bytes + re_bytes + cs_bytes + 256, pool,
                                s) != cudaSuccess) {
        if (err) *err = "SSB scratch allocation failed";
        return OPHPC_ERROR_OUT_OF_MEMORY;
    }
    double2* buf[2] = {(double2*)mem, (double2*)(mem + plane)};
    double2* w2 = (double2*)(mem + 2 * plane);
    double2* w3 = (double2*)(mem + 3 * plane);
    double2* tw = (double2*)(mem + 4 * plane);
    double* enc = d_encoded ? d_encoded : (double*)(mem + 4 * plane + tw_bytes);
    double* re = (double*)(mem + 4 * plane + tw_bytes + enc_bytes);
    double2* cs = (double2*)(mem + 4 * plane + tw_bytes + enc_bytes + re_bytes);
    unsigned long long* mm = (unsigned long long*)(mem + 4 * plane + tw_bytes + enc_bytes + re_bytes + cs_bytes);
    FftPlan plan_x, plan_y;
    fft_plan_init(&plan_x, pnx, tw, s);
    fft_plan_init(&plan_y, pny, tw + fft_twiddle_count(pnx), s);
    cudaError_t e = cudaSuccess;
    const dim3 g2((unsigned)((pnx + 255) / 256), (unsigned)pny);
    if (encode_flag == kEncodeSideband) {
        int x1 = 0, x2 = pnx - 1, y1 = 0, y2 = pny - 1;
        if (passband == OPHPC_SSB_TOP || passband == OPHPC_SSB_BOTTOM) {
            const int h = pny / 2;
            y1 = h - h / 2 - 1;
            y2 = y1 + h - 1;
        } else {
            const int h = pnx / 2;
            x1 = h - h / 2 - 1;
            x2 = x1 + h - 1;
        }
        const int axis = (passband == OPHPC_SSB_TOP || passband == OPHPC_SSB_BOTTOM) ? pny : pnx;
        count_launches(1);
        ssb_carrier_kernel<<<(unsigned)((axis + 255) / 256), 256, 0, s>>>(cs, pnx, pny, ppx, ppy, (int)passband);
        for (int c = 0; c < n_channels && e == cudaSuccess; ++c) {
            count_launches(1);
            ssb_crop_kernel<<<g2, 256, 0, s>>>(d_field + (int64_t)c * n, w2, pnx, pny, x1, x2, y1, y2);
            e = shifted_fft2(w2, w2, buf, plan_x, plan_y, pnx, pny, true, s);
            if (e == cudaSuccess) {
                count_launches(1);
                ssb_fringe_kernel<<<g2, 256, 0, s>>>(w2, enc + (int64_t)c * n, pnx, pny, cs, (int)passband);
                e = cudaGetLastError();
            }
        }
    } else if (encode_flag == OPHPC_ENCODE_SSB) {
        count_launches(1);
        ssb_axis_kernel<<<(unsigned)((pnx + pny + 255) / 256), 256, 0, s>>>(cs, pnx, pny, ppx, ppy, shift_x, shift_y);
        for (int c = 0; c < n_channels && e == cudaSuccess; ++c) {
            e = shifted_fft2(d_field + (int64_t)c * n, w2, buf, plan_x, plan_y, pnx, pny, false, s);
            if (e == cudaSuccess) e = shifted_fft2(w2, w2, buf, plan_x, plan_y, pnx, pny, true, s);
            if (e == cudaSuccess) {
                count_launches(1);
                ssb_point_cloud_kernel<<<dim3((unsigned)((pnx + 255) / 256), (unsigned)pny), 256, 0, s>>>(
                    w2, enc + (int64_t)c * n, pnx, pny, cs);
                e = cudaGetLastError();
            }
        }
    } else {
        // freqShift(H0, 0, 100), then singleSideBand
        e = shifted_fft2(d_field, w2, buf, plan_x, plan_y, pnx, pny, false, s);
        if (e == cudaSuccess) {
            count_launches(1);
            ssb_circshift_kernel<<<grid_ssb(n), 256, 0, s>>>(w2, w3, n, pny, 100);
            e = shifted_fft2(w3, w3, buf, plan_x, plan_y, pnx, pny, true, s);
        }
        if (e == cudaSuccess) e = shifted_fft2(w3, w2, buf, plan_x, plan_y, pnx, pny, false, s);
        if (e == cudaSuccess) {
            count_launches(1);
            ssb_passband_kernel<<<grid_ssb(n), 256, 0, s>>>(w2, pnx, pny, (int)passband);
            e = shifted_fft2(w2, w2, buf, plan_x, plan_y, pnx, pny, true, s);
        }
        if (e == cudaSuccess) {
            count_launches(3);
            ssb_minmax_init_kernel<<<1, 1, 0, s>>>(mm);
            ssb_real_minmax_kernel<<<grid_ssb(n), 256, 0, s>>>(w2, n, re, mm);
            ssb_unit_normalize_kernel<<<grid_ssb(n), 256, 0, s>>>(re, n, n_channels, mm, enc);
            e = cudaGetLastError();
        }
    }
    if (e == cudaSuccess && d_normalized) {
        launch_normalize(enc, n_channels, n, d_normalized, mm, s);   // ophGen::normalize over every channel
        e = cudaGetLastError();
    }
    cudaFreeAsync(mem, s);
    if (e != cudaSuccess) {
        if (err) *err = cudaGetErrorString(e);
        return OPHPC_ERROR_CUDA;
    }
    return OPHPC_SUCCESS;
}

}  // namespace ophpc
