// WRP (wavefront recording plane) hologram generation on GB300
// (include/ophpc_wrp.h).
//
// The reference (ophWRP::calculateWRPCPU, ophgen/src/ophWRP.cpp:321-433)
// adds, for every point, amp * (cos(k r) cos(2 pi), -sin(k r) sin(2 pi)) / r
// over a (2w) x (2w) pixel square anchored at ((int)(x / ppX) + pnX/2,
// (int)(y / ppY) + pnY/2), with one depth difference dz = wrp_location - zmax
// for all points (ophWRP.cpp:345), r = sign(dz) sqrt(dx^2 + dy^2 + dz^2) and
// w = (int)(|lambda dz / (2 ppX^2)| * 2). The square's values depend on the
// pixel offset only, so the plane is the correlation of an amplitude image
// (every point's amplitude added at its anchor) with one (2w) x (2w) kernel
// table per channel:
//
//   wrp_stats_kernel   zmax of the scaled depths (from MIN_DOUBLE, as
//                      autoScaling starts it) and the largest |amplitude|;
//                      read back once to size the splat
//   wrp_bin_kernel     amplitudes into per-channel anchor grids of 64-bit
//                      fixed point (integer atomics: the same sums in any
//                      order, so the result is deterministic)
//   wrp_amp_kernel     the fixed-point sums turned into FP64 amplitudes in
//                      place, once per anchor
//   wrp_kernel_table   the (2w)^2 kernel values in FP64
//   wrp_conv_kernel    per plane pixel the FP64 sum over the square, written
//                      into the centre of the zero-padded FFT buffer
//
// and the plane is propagated (ophGen::Fresnel_FFT, ophgen/src/ophGen.cpp:
// 516-580) as out = crop(IFFT2(T . FFT2(pad(plane)))), unnormalised, with
// T = exp(i 2 pi d sqrt(1/lambda^2 - fx^2 - fy^2)) in natural frequency
// order: the reference's fftShift pairs around both transforms cancel for
// the even padded sizes. The FFTs are this library's Stockham passes
// (pc_fft.cu); rows that are all zero are not transformed.
#include "ophpc_wrp.h"

#include "pc_common.cuh"
#include "pc_fft.cuh"

#include <algorithm>
#include <cmath>
#include <cstring>
#include <string>

namespace ophpc {
namespace {

constexpr double kMinDouble = 2.2250738585072014e-308;   // MIN_DOUBLE, Openholo/src/define.h:148

// Order-preserving map of doubles onto unsigned 64-bit keys.
__host__ __device__ inline unsigned long long order_key(double v) {
    unsigned long long u;
    memcpy(&u, &v, 8);
    return (u >> 63) ? ~u : (u | 0x8000000000000000ull);
}
inline double from_key(unsigned long long k) {
    const unsigned long long u = (k >> 63) ? (k & 0x7fffffffffffffffull) : ~k;
    double v;
    memcpy(&v, &u, 8);
    return v;
}

struct WrpStats {
    unsigned long long zmax_key;   // order_key of the largest scaled z
    unsigned long long amax_bits;  // bits of the largest |amplitude| (non-negative: ordered as integers)
};

__global__ void wrp_stats_kernel(const double* __restrict__ verts, int64_t n, double scale_z, int nch,
                                 WrpStats* __restrict__ st) {
    unsigned long long zk = order_key(kMinDouble), ab = 0;
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        const double* v = verts + i * 7;
        const unsigned long long k = order_key(v[2] * scale_z);
        zk = k > zk ? k : zk;
        for (int c = 0; c < nch; ++c) {
            const unsigned long long b = (unsigned long long)__double_as_longlong(fabs(v[3 + c]));
            ab = b > ab ? b : ab;
        }
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        const unsigned long long zo = __shfl_xor_sync(0xffffffffu, zk, o), ao = __shfl_xor_sync(0xffffffffu, ab, o);
        zk = zo > zk ? zo : zk;
        ab = ao > ab ? ao : ab;
    }
    if ((threadIdx.x & 31) == 0) {
        atomicMax(&st->zmax_key, zk);
        atomicMax(&st->amax_bits, ab);
    }
}

struct BinArgs {
    double scale_x, scale_y, ppx, ppy, fixed_scale;
    int hpnx, hpny, w, gx, gy, nch;
};

// Anchor grids [nch][gy][gx], anchor (tx, ty) at (tx + w, ty + w): anchors in
// [-w, pnX + w) x [-w, pnY + w) can reach the plane.
__global__ void wrp_bin_kernel(const double* __restrict__ verts, int64_t n, BinArgs a,
                               unsigned long long* __restrict__ grid) {
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const double* v = verts + i * 7;
    const double qx = (v[0] * a.scale_x) / a.ppx, qy = (v[1] * a.scale_y) / a.ppy;
    if (!(fabs(qx) < 1e9 && fabs(qy) < 1e9)) return;   // cannot reach the plane (or not a number)
    const int ax = __double2int_rz(qx) + a.hpnx + a.w, ay = __double2int_rz(qy) + a.hpny + a.w;
    if (ax < 0 || ax >= a.gx || ay < 0 || ay >= a.gy) return;
    const int64_t plane = (int64_t)a.gx * a.gy;
    for (int c = 0; c < a.nch; ++c) {
        const long long q = __double2ll_rn(v[3 + c] * a.fixed_scale);
        atomicAdd(&grid[c * plane + (int64_t)ay * a.gx + ax], (unsigned long long)q);
    }
}

// The anchor grids' fixed-point sums as FP64 amplitudes, in place (the
// conversion the splat would otherwise repeat for every pixel an anchor
// reaches; GB300's FP64 pipe is narrow).
__global__ void wrp_amp_kernel(unsigned long long* __restrict__ grid, int64_t n, double inv_fixed) {
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        const long long q = (long long)grid[i];
        if (q != 0) grid[i] = (unsigned long long)__double_as_longlong((double)q * inv_fixed);
    }
}

// Kernel values K[wy + w][wx + w] of one channel (ophWRP.cpp:396-408, with
// the amplitude factored out).
__global__ void wrp_kernel_table(double2* __restrict__ K, int w, double ppx, double ppy, double dzz, int sign_pos,
                                 double k, double crand, double srand) {
    const int side = 2 * w;
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= side * side) return;
    const int wy = i / side - w, wx = i % side - w;
    const double dy = wy * ppy, dyy = dy * dy;
    const double dx = wx * ppx;
    const double rr = sqrt(dx * dx + dyy + dzz);
    const double r = sign_pos ? rr : -rr;
    const double kr = k * r;
    double s, c;
    sincos(kr, &s, &c);
    K[i] = make_double2((c * crand) / r, (-s * srand) / r);
}

struct ConvArgs {
    int pnx, pny, w, gx, gy;
    int64_t out_stride;         // elements per output row
};

// Plane pixel (px, py): sum over the square of anchor amplitude x kernel,
// wy outer, wx inner (a fixed order). Anchors without points hold zero bits
// (+0.0, the only zero wrp_amp_kernel writes), and an FMA with them leaves
// the sum as it is (the kernel values are finite, the sum never -0.0), so a
// warp skips a row of the square where none of its 32 pixels meets a point:
// an integer OR over the row's anchors, a vote, and the row's FMAs only
// when some lane needs them. On GB300's narrow FP64 pipe the FMAs are the
// cost; a per-anchor test is turned into predicated FMAs that still take
// the pipe. Every lane of a warp reaches the vote (lanes past the plane's
// edge read nothing and store nothing). The kernel table sits in shared
// memory when it fits.
__global__ void __launch_bounds__(256, 4) wrp_conv_kernel(const unsigned long long* __restrict__ grid,
                                                       const double2* __restrict__ K, ConvArgs a,
                                                       double2* __restrict__ out, int k_in_smem) {
    extern __shared__ double2 sK[];
    const int side = 2 * a.w;
    if (k_in_smem) {
        for (int i = threadIdx.y * blockDim.x + threadIdx.x; i < side * side; i += blockDim.x * blockDim.y)
            sK[i] = K[i];
        __syncthreads();
    }
    const double2* Kt = k_in_smem ? sK : K;
    const int px = blockIdx.x * blockDim.x + threadIdx.x, py = blockIdx.y * blockDim.y + threadIdx.y;
    const bool inside = px < a.pnx && py < a.pny;
    const int qx = inside ? px : 0, qy = inside ? py : 0;
    double re = 0.0, im = 0.0;
    for (int wy = -a.w; wy < a.w; ++wy) {
        const unsigned long long* row = grid + (int64_t)(qy - wy + a.w) * a.gx + (qx + a.w);
        unsigned long long any = 0;
        if (inside)
            for (int wx = -a.w; wx < a.w; ++wx) any |= __ldg(row - wx);
        if (!__any_sync(0xffffffffu, any != 0)) continue;
        const double2* krow = Kt + (wy + a.w) * side + a.w;
        for (int wx = -a.w; wx < a.w; ++wx) {
            const double amp = inside ? __longlong_as_double((long long)__ldg(row - wx)) : 0.0;
            const double2 kv = krow[wx];
            re = fma(amp, kv.x, re);
            im = fma(amp, kv.y, im);
        }
    }
    if (inside) out[(int64_t)py * a.out_stride + px] = make_double2(re, im);
}

// buf *= exp(i 2 pi d sqrt(1/lambda^2 - fx^2 - fy^2)), natural frequency
// order (signed index / (2 ss), as Fresnel_FFT's LUT_fx after its shift).
// T depends on fx^2 and fy^2 only, and (-k) / (2 ss) is exactly -(k / (2 ss)),
// so one thread computes T for |kx| = j, |ky| = i (j <= nx/2, i <= ny/2)
// and applies it to the up to four entries with those magnitudes: a quarter
// of the FP64 sqrt and sincos, bit for bit the values of one per entry.
__global__ void wrp_transfer_kernel(double2* __restrict__ buf, int nx, int ny, double ssx2, double ssy2,
                                    double inv_lambda_sq, double two_pi_d) {
    const int j = blockIdx.x * blockDim.x + threadIdx.x, i = blockIdx.y;
    const int hx = nx / 2, hy = ny / 2;
    if (j > hx || i > hy) return;
    // index j < nx/2 holds kx = j; index nx/2 holds kx = -nx/2 (no mirror)
    const int kx = j < hx ? j : -hx, ky = i < hy ? i : -hy;
    const double fx = (double)kx / ssx2, fy = (double)ky / ssy2;
    const double sq = sqrt(inv_lambda_sq - fx * fx - fy * fy);
    double s, c;
    sincos(two_pi_d * sq, &s, &c);
    const int cols[2] = {j, (j > 0 && j < hx) ? nx - j : -1};
    const int rows[2] = {i, (i > 0 && i < hy) ? ny - i : -1};
#pragma unroll
    for (int a = 0; a < 2; ++a) {
#pragma unroll
        for (int b = 0; b < 2; ++b) {
            if (rows[a] < 0 || cols[b] < 0) continue;
            const int64_t o = (int64_t)rows[a] * nx + cols[b];
            const double2 v = buf[o];
            buf[o] = make_double2(v.x * c - v.y * s, v.x * s + v.y * c);
        }
    }
}

// dst[py][px] = src[(hy + py) * nx + hx + px]
__global__ void wrp_crop_kernel(const double2* __restrict__ src, int nx, int hx, int hy, int pnx, int pny,
                                double2* __restrict__ dst) {
    const int px = blockIdx.x * blockDim.x + threadIdx.x, py = blockIdx.y;
    if (px >= pnx || py >= pny) return;
    dst[(int64_t)py * pnx + px] = src[(int64_t)(hy + py) * nx + hx + px];
}

// src [pny][pnx] into the centre (hy, hx) of a zeroed [ny][nx] buffer
__global__ void wrp_embed_kernel(const double2* __restrict__ src, int pnx, int pny, int nx, int hx, int hy,
                                 double2* __restrict__ dst) {
    const int px = blockIdx.x * blockDim.x + threadIdx.x, py = blockIdx.y;
    if (px >= pnx || py >= pny) return;
    dst[(int64_t)(hy + py) * nx + hx + px] = src[(int64_t)py * pnx + px];
}

size_t align256(size_t v) { return (v + 255) & ~(size_t)255; }

// The propagation of a plane already embedded at (pny/2, pnx/2) of buf[0]
// (buf[1] zeroed): FFT rows (only the plane's rows), FFT columns, transfer,
// inverse columns, inverse rows (the plane's rows), crop into dst.
cudaError_t propagate(double2* const buf[2], const FftPlan& px_plan, const FftPlan& py_plan, int pnx, int pny,
                      double ppx, double ppy, double lambda, double distance, double2* dst, cudaStream_t s) {
    const int nx = 2 * pnx, ny = 2 * pny, hx = pnx >> 1, hy = pny >> 1;
    double2* rows[2] = {buf[0] + (int64_t)hy * nx, buf[1] + (int64_t)hy * nx};
    const int r1 = fft_run(px_plan, rows, pny, 1, nx, false, s);
    double2* cols[2] = {buf[r1], buf[r1 ^ 1]};
    const int c1 = fft_run(py_plan, cols, nx, nx, 1, false, s);
    double2* spec = cols[c1];
    const double ssx2 = (pnx * ppx) * 2, ssy2 = (pny * ppy) * 2;
    count_launches(1);
    wrp_transfer_kernel<<<dim3((unsigned)((nx / 2 + 1 + 255) / 256), (unsigned)(ny / 2 + 1)), 256, 0, s>>>(
        spec, nx, ny, ssx2, ssy2, 1.0 / (lambda * lambda), 2 * M_PI * distance);
    double2* icol[2] = {spec, cols[c1 ^ 1]};
    const int c2 = fft_run(py_plan, icol, nx, nx, 1, true, s);
    double2* back = icol[c2];
    double2* other = icol[c2 ^ 1];
    double2* irow[2] = {back + (int64_t)hy * nx, other + (int64_t)hy * nx};
    const int r2 = fft_run(px_plan, irow, pny, 1, nx, true, s);
    count_launches(1);
    wrp_crop_kernel<<<dim3((unsigned)((pnx + 255) / 256), (unsigned)pny), 256, 0, s>>>(r2 ? other : back, nx, hx, hy,
                                                                                        pnx, pny, dst);
    return cudaGetLastError();
}

}  // namespace

bool wrp_sizes_supported(int pnx, int pny) { return fft_supported(2 * pnx) && fft_supported(2 * pny); }

ophpc_status wrp_generate_device(cudaMemPool_t pool, const ophpc_wrp_config* cfg, const ophpc_vertex* d_vertices,
                                 uint64_t n_points, double* d_out, int plane_channel, cudaStream_t s,
                                 std::string* err) {
    auto fail = [&](ophpc_status st, const std::string& msg) {
        if (err) *err = msg;
        return st;
    };
    const int pnx = cfg->pixel_number[0], pny = cfg->pixel_number[1];
    const int nch = (int)cfg->n_channels;
    const double ppx = cfg->pixel_pitch[0], ppy = cfg->pixel_pitch[1];
    const int nx = 2 * pnx, ny = 2 * pny;
    const bool full = plane_channel < 0;
    // depth range and amplitude bound, read back once
    WrpStats* d_st = nullptr;
    if (cudaMallocFromPoolAsync((void**)&d_st, sizeof(WrpStats), pool, s) != cudaSuccess)
        return fail(OPHPC_ERROR_OUT_OF_MEMORY, "WRP scratch allocation failed");
    WrpStats h_st;
    h_st.zmax_key = order_key(kMinDouble);
    h_st.amax_bits = 0;
    cudaError_t e = cudaMemcpyAsync(d_st, &h_st, sizeof(h_st), cudaMemcpyHostToDevice, s);
    if (n_points > 0 && e == cudaSuccess) {
        count_launches(1);
        wrp_stats_kernel<<<256, 256, 0, s>>>(reinterpret_cast<const double*>(d_vertices), (int64_t)n_points,
                                             cfg->scale[2], nch, d_st);
        e = cudaGetLastError();
    }
    if (e == cudaSuccess) e = cudaMemcpyAsync(&h_st, d_st, sizeof(h_st), cudaMemcpyDeviceToHost, s);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    cudaFreeAsync(d_st, s);
    if (e != cudaSuccess) return fail(OPHPC_ERROR_CUDA, cudaGetErrorString(e));
    const double zmax = from_key(h_st.zmax_key);
    double amax;
    memcpy(&amax, &h_st.amax_bits, 8);
    // ophWRP.cpp:338-347, 376-381 (one dz for every point)
    const double ppXX = ppx * ppx * 2;
    const double pi2 = 2 * M_PI;
    const double dz = cfg->wrp_location - zmax;
    const double dzz = dz * dz;
    int wmax = 0;
    int w[OPHPC_MAX_CHANNELS];
    for (int c = 0; c < nch; ++c) {
        const double tw = std::fabs(cfg->wave_length[c] * dz / ppXX) * 2;
        if (!(tw < 8192.0)) return fail(OPHPC_ERROR_UNSUPPORTED, "WRP splat wider than 16384 pixels");
        w[c] = (int)tw;
        wmax = w[c] > wmax ? w[c] : wmax;
    }
    // fixed point for the anchor sums: |sum| <= amax * n < 2^61
    double fixed = 1.0;
    if (amax > 0.0 && n_points > 0) {
        const int e2 = (int)std::ceil(std::log2(amax * (double)n_points));
        fixed = std::ldexp(1.0, 61 - e2);
    }
    const int gx = pnx + 2 * wmax, gy = pny + 2 * wmax;
    const size_t grid_bytes = align256(sizeof(unsigned long long) * (size_t)gx * gy * nch);
    const size_t k_bytes = align256(sizeof(double2) * (size_t)(2 * wmax) * (2 * wmax) + 16);
    const size_t buf_bytes = full ? align256(sizeof(double2) * (size_t)nx * ny) : 0;
    const size_t tw_bytes = full ? align256(sizeof(double2) * (size_t)(fft_twiddle_count(nx) + fft_twiddle_count(ny)))
                                 : 0;
    unsigned char* mem = nullptr;
    if (cudaMallocFromPoolAsync((void**)&mem, grid_bytes + k_bytes + 2 * buf_bytes + tw_bytes, pool, s) != cudaSuccess)
        return fail(OPHPC_ERROR_OUT_OF_MEMORY, "WRP scratch allocation failed");
    unsigned long long* grid = (unsigned long long*)mem;
    double2* K = (double2*)(mem + grid_bytes);
    double2* buf[2] = {full ? (double2*)(mem + grid_bytes + k_bytes) : nullptr,
                       full ? (double2*)(mem + grid_bytes + k_bytes + buf_bytes) : nullptr};
    double2* tw = full ? (double2*)(mem + grid_bytes + k_bytes + 2 * buf_bytes) : nullptr;
    FftPlan plan_x, plan_y;
    if (full) {
        fft_plan_init(&plan_x, nx, tw, s);
        fft_plan_init(&plan_y, ny, tw + fft_twiddle_count(nx), s);
    }
    e = cudaMemsetAsync(grid, 0, grid_bytes, s);
    if (n_points > 0 && e == cudaSuccess) {
        BinArgs ba;
        ba.scale_x = cfg->scale[0];
        ba.scale_y = cfg->scale[1];
        ba.ppx = ppx;
        ba.ppy = ppy;
        ba.fixed_scale = fixed;
        ba.hpnx = pnx >> 1;
        ba.hpny = pny >> 1;
        ba.w = wmax;
        ba.gx = gx;
        ba.gy = gy;
        ba.nch = nch;
        const int64_t cells = (int64_t)gx * gy * nch;
        count_launches(2);
        wrp_bin_kernel<<<(unsigned)((n_points + 255) / 256), 256, 0, s>>>(reinterpret_cast<const double*>(d_vertices),
                                                                         (int64_t)n_points, ba, grid);
        wrp_amp_kernel<<<(unsigned)std::min<int64_t>((cells + 255) / 256, 4096), 256, 0, s>>>(grid, cells,
                                                                                            1.0 / fixed);
    }
    // the reference's random-phase factor with RandomPhase off: 2 pi * 1.0
    const double crand = std::cos(pi2 * 1.0), srand_ = std::sin(pi2 * 1.0);
    const int c0 = full ? 0 : plane_channel, c1 = full ? nch : plane_channel + 1;
    for (int c = c0; c < c1 && e == cudaSuccess; ++c) {
        const int wc = w[c], side = 2 * wc;
        if (side > 0) {
            count_launches(1);
            wrp_kernel_table<<<(unsigned)((side * side + 255) / 256), 256, 0, s>>>(
                K, wc, ppx, ppy, dzz, dz > 0.0 ? 1 : 0, pi2 / cfg->wave_length[c], crand, srand_);
        }
        // the splat of this channel: its anchors are offset by wmax in the grid
        ConvArgs ca;
        ca.pnx = pnx;
        ca.pny = pny;
        ca.w = wc;
        ca.gx = gx;
        ca.gy = gy;
        const unsigned long long* gch = grid + (size_t)c * gx * gy + (size_t)(wmax - wc) * gx + (wmax - wc);
        double2* dst;
        if (full) {
            e = cudaMemsetAsync(buf[0], 0, buf_bytes, s);
            if (e == cudaSuccess) e = cudaMemsetAsync(buf[1], 0, buf_bytes, s);
            dst = buf[0] + (int64_t)(pny >> 1) * nx + (pnx >> 1);
            ca.out_stride = nx;
        } else {
            dst = reinterpret_cast<double2*>(d_out);
            ca.out_stride = pnx;
        }
        const size_t ks = sizeof(double2) * (size_t)side * side;
        const int in_smem = ks <= 96 * 1024;
        if (in_smem && ks > 48 * 1024)
            cudaFuncSetAttribute(wrp_conv_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)ks);
        count_launches(1);
        wrp_conv_kernel<<<dim3((unsigned)((pnx + 31) / 32), (unsigned)((pny + 7) / 8)), dim3(32, 8),
                          in_smem ? ks : 0, s>>>(gch, K, ca, dst, in_smem);
        if (e == cudaSuccess) e = cudaGetLastError();
        if (full && e == cudaSuccess)
            e = propagate(buf, plan_x, plan_y, pnx, pny, ppx, ppy, cfg->wave_length[c], cfg->propagation_distance,
                          reinterpret_cast<double2*>(d_out) + (int64_t)c * pnx * pny, s);
    }
    cudaFreeAsync(mem, s);
    if (e != cudaSuccess) return fail(OPHPC_ERROR_CUDA, cudaGetErrorString(e));
    return OPHPC_SUCCESS;
}

ophpc_status fresnel_fft_device(cudaMemPool_t pool, int pnx, int pny, double ppx, double ppy, double lambda,
                                double distance, const double2* src, double2* dst, cudaStream_t s,
                                std::string* err) {
    const int nx = 2 * pnx, ny = 2 * pny;
    const size_t buf_bytes = align256(sizeof(double2) * (size_t)nx * ny);
    const size_t tw_bytes = align256(sizeof(double2) * (size_t)(fft_twiddle_count(nx) + fft_twiddle_count(ny)));
    unsigned char* mem = nullptr;
    if (cudaMallocFromPoolAsync((void**)&mem, 2 * buf_bytes + tw_bytes, pool, s) != cudaSuccess) {
        if (err) *err = "Fresnel FFT scratch allocation failed";
        return OPHPC_ERROR_OUT_OF_MEMORY;
    }
    double2* buf[2] = {(double2*)mem, (double2*)(mem + buf_bytes)};
    double2* tw = (double2*)(mem + 2 * buf_bytes);
    FftPlan plan_x, plan_y;
    fft_plan_init(&plan_x, nx, tw, s);
    fft_plan_init(&plan_y, ny, tw + fft_twiddle_count(nx), s);
    cudaError_t e = cudaMemsetAsync(mem, 0, 2 * buf_bytes, s);
    if (e == cudaSuccess) {
        count_launches(1);
        wrp_embed_kernel<<<dim3((unsigned)((pnx + 255) / 256), (unsigned)pny), 256, 0, s>>>(src, pnx, pny, nx, pnx >> 1,
                                                                                           pny >> 1, buf[0]);
        e = propagate(buf, plan_x, plan_y, pnx, pny, ppx, ppy, lambda, distance, dst, s);
    }
    cudaFreeAsync(mem, s);
    if (e != cudaSuccess) {
        if (err) *err = cudaGetErrorString(e);
        return OPHPC_ERROR_CUDA;
    }
    return OPHPC_SUCCESS;
}

}  // namespace ophpc
