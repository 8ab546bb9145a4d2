// Per-point preparation: one thread per (channel, point).
//
// Restates, in FP64 with the reference's roundings (explicit _rn intrinsics,
// no FMA contraction, so the window rectangles match the x86 reference bit
// for bit):
//   transVW                      ophgen/src/ophGen.cpp:1976-1985
//   pos *= scale                 ophgen/src/ophPointCloud.cpp:304-306
//   z = pos.z + distance         ophgen/src/ophGen.cpp:381 / 464
//   amplitude = color[ch]        ophgen/src/ophPointCloud.cpp:302
//   RS window rectangle          ophgen/src/ophGen.cpp:385-409
//   Fresnel window rectangle     ophgen/src/ophGen.cpp:470-492
#include "pc_common.cuh"

namespace ophpc {

namespace {

struct PrepArgs {
    double scale[3];
    double distance;
    double field_length;
    int viewing_window;
    int diff_flag;
    int color_offset;
};

__device__ __forceinline__ double trans_vw(double p, double f) {
    // -f * p / (p - f)
    return __ddiv_rn(__dmul_rn(-f, p), __dsub_rn(p, f));
}

// floor((b - x0) / pp) + 1, and pn - floor((b - y0) / pp).
__device__ __forceinline__ void window_rect(const ChannelGeom& g, double px, double py, double hwx,
                                            double hwy, PointRec& r) {
    double xb0 = __dadd_rn(px, hwx), xb1 = __dsub_rn(px, hwx);
    double yb0 = __dadd_rn(py, hwy), yb1 = __dsub_rn(py, hwy);
    double Xb0 = floor(__ddiv_rn(__dsub_rn(xb0, g.x0), g.ppX)) + 1.0;
    double Xb1 = floor(__ddiv_rn(__dsub_rn(xb1, g.x0), g.ppX)) + 1.0;
    double Yb0 = (double)g.pnY - floor(__ddiv_rn(__dsub_rn(yb1, g.y0), g.ppY));
    double Yb1 = (double)g.pnY - floor(__ddiv_rn(__dsub_rn(yb0, g.y0), g.ppY));
    if (Xb0 > g.pnX) Xb0 = g.pnX;
    if (Xb1 < 0) Xb1 = 0;
    if (Yb0 > g.pnY) Yb0 = g.pnY;
    if (Yb1 < 0) Yb1 = 0;
    // Both ends are integral; clamp to a safe int range before converting.
    auto to_i = [](double v) -> int32_t {
        if (!(v == v)) return 0;
        v = fmax(-1.0, fmin(v, 2147483000.0));
        return (int32_t)v;
    };
    r.x_lo = to_i(Xb1);
    r.x_hi = to_i(Xb0);
    r.y_lo = to_i(Yb1);
    r.y_hi = to_i(Yb0);
    if (r.x_hi < r.x_lo) r.x_hi = r.x_lo;
    if (r.y_hi < r.y_lo) r.y_hi = r.y_lo;
}

__global__ void __launch_bounds__(256) prep_points_kernel(const double* __restrict__ verts,
                                                          int64_t n_points, PrepArgs a, JobGeom jg,
                                                          PointRec* __restrict__ out) {
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    const int ch = blockIdx.y;
    if (i >= n_points) return;
    const ChannelGeom& g = jg.ch[ch];
    const double* v = verts + i * 7;   // packed 56-byte Vertex
    double x = v[0], y = v[1], zs = v[2];
    if (a.viewing_window) {
        x = trans_vw(x, a.field_length);
        y = trans_vw(y, a.field_length);
        zs = trans_vw(zs, a.field_length);
    }
    x = __dmul_rn(x, a.scale[0]);
    y = __dmul_rn(y, a.scale[1]);
    zs = __dmul_rn(zs, a.scale[2]);
    const double z = __dadd_rn(zs, a.distance);
    const double amp = v[3 + ch + a.color_offset];
    PointRec r;
    r.x = x;
    r.y = y;
    r.z = z;
    r.pad = 0.0;
    if (a.diff_flag == 0) {
        // abs(tx / sqrtX * z): detx already holds tx / sqrtX.
        const double hwx = fabs(__dmul_rn(g.detx, z));
        const double hwy = fabs(__dmul_rn(g.dety, z));
        window_rect(g, x, y, hwx, hwy, r);
        r.coef = __dmul_rn(amp, z) * g.inv_lambda;      // amp*z/lambda (amplitude only)
        r.aux = __dmul_rn(z, z);                         // zz, as the reference forms it
    } else {
        // abs(operand / (2 * pp)), operand = lambda * z
        const double operand = __dmul_rn(g.lambda, z);
        const double hwx = fabs(__ddiv_rn(operand, 2.0 * g.ppX));
        const double hwy = fabs(__ddiv_rn(operand, 2.0 * g.ppY));
        window_rect(g, x, y, hwx, hwy, r);
        r.coef = amp / operand;                          // amp/(lambda*z)
        r.aux = 1.0 / (2.0 * z * g.lambda);              // turns per m^2 of (dx^2+dy^2)
    }
    out[(int64_t)ch * n_points + i] = r;
}

}  // namespace

void launch_prep(const void* d_vertices, int64_t n_points, const double* scale, double distance,
                 double field_length, int viewing_window, int diff_flag, const JobGeom& jg,
                 PointRec* d_recs, cudaStream_t stream, int color_offset) {
    if (n_points <= 0) return;
    PrepArgs a;
    a.color_offset = color_offset;
    for (int i = 0; i < 3; ++i) a.scale[i] = scale[i];
    a.distance = distance;
    a.field_length = field_length;
    a.viewing_window = viewing_window;
    a.diff_flag = diff_flag;
    dim3 grid((unsigned)((n_points + 255) / 256), (unsigned)jg.n_channels);
    count_launches(1);
    prep_points_kernel<<<grid, 256, 0, stream>>>((const double*)d_vertices, n_points, a, jg, d_recs);
}

}  // namespace ophpc
