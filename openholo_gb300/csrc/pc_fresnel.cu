// Fresnel point-cloud kernel on the FP32 cores (sm_103a).
//
// Computes the reference's sum (ophgen/src/ophGen.cpp:447-514; GPU
// counterpart ophgen/src/ophPCKernel.cu:516-601)
//   H(p) = sum_j  a_j / (lambda z_j) * (sin phi, -cos phi),
//   phi/2pi = ((X-x)^2 + (Y-y)^2 + 2 z^2) / (2 z lambda),
// over the points whose window rectangle contains p. The Fresnel window is a
// rectangle (no per-pixel cone test), so the term factorises over columns and
// rows: with the tile centre (Xc, Yc), dx = dxc + u, dy = dyc + v,
//   phi/2pi = tau_c + s(2 dxc u + u^2) + s(2 dyc v + v^2),  s = 1/(2 z lambda).
// tau_c is evaluated in FP64 per (point, tile) and reduced mod 1 (the one FP64
// step); each thread then forms one complex factor per column and per row of
// its 4x4 pixel block (8 sin/cos pairs) and accumulates their products: a
// complex rank-1 update per point, four FMAs per pixel. Points whose window
// holds the whole tile and whose column / row phases span under 16 turns
// (FAST, the common case) carry the phases in radians straight into the
// MUFU sin/cos, with no reduction and no masks; for the others (CUT) the
// phases are reduced mod 1 and the rectangle is applied as 0/1 masks on the
// factors. Sums run in FP32 per chunk of 256
// points and fold into FP64 shared-memory sums; every pixel is stored once.
#include "pc_common.cuh"

#include <cstddef>

namespace ophpc {

namespace {

// Values duplicated into pairs for the packed FP32 arithmetic.
// The CUT loop reads xl..yh as one int4, so they sit at a 16-byte offset.
struct __align__(16) FrSRec {
    float2 P, Q;             // 2 dxc s, 2 dyc s
    float2 s, fc;            // s, frac(tau_c)
    int32_t xl, xh;          // window columns relative to the tile origin
    int32_t yl, yh;          // window rows relative to the tile origin
    float ac;                // amp / (lambda z)
    int32_t pad[3];
};
static_assert(sizeof(FrSRec) == 64, "FrSRec size");
static_assert(offsetof(FrSRec, xl) % 16 == 0, "xl..yh are read as one int4");

constexpr float kTwoPi = 6.283185307179586f;
// FAST class: column and row phases stay within this many turns over the
// tile, so the FP32 phase in radians stays under ~101 rad and MUFU sin/cos
// take it without a reduction.
constexpr float kMaxTurns = 16.f;

__device__ __forceinline__ int warp_prefix(unsigned ballot) {
    return __popc(ballot & ((1u << (threadIdx.x & 31)) - 1u));
}

__global__ void __launch_bounds__(kThreads, 4)
fresnel_kernel(const PointRec* __restrict__ recs, const JobGeom jg, double2* __restrict__ field,
               double2* __restrict__ partials) {
    extern __shared__ __align__(16) unsigned char s_raw[];
    FrSRec* s_rec = reinterpret_cast<FrSRec*>(s_raw);
    // FP64 running sums, [pixel][thread]: consecutive threads hit consecutive 16-byte words
    double2* s_acc = reinterpret_cast<double2*>(s_raw + sizeof(FrSRec) * kChunk);
    __shared__ int s_cnt[2][2][kThreads / 32];   // [fast|cut][q][warp]

    const int ch = blockIdx.z / jg.ksplit;
    const int part = blockIdx.z % jg.ksplit;
    const ChannelGeom& g = jg.ch[ch];
    const int X0 = blockIdx.x * kTileW, Y0 = blockIdx.y * kTileH;
    const int vx1 = min(X0 + kTileW, g.pnX), vy1 = min(Y0 + kTileH, g.pnY);
    const double Xc = pixel_x(g, X0 + kTileW / 2), Yc = pixel_y(g, Y0 + kTileH / 2);

    const int tx = threadIdx.x % kThreadsX, ty = threadIdx.x / kThreadsX;
    const int warp = threadIdx.x >> 5;
    // largest |u|, |v| of a tile pixel from the tile centre (one column /
    // row of slack)
    const float uext_f = (float)((kTileW / 2 + 1) * g.ppX), vext_f = (float)((kTileH / 2 + 1) * g.ppY);
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

    f2::v2 up[kPixW / 2], uup[kPixW / 2], vp[kPixH / 2], vvp[kPixH / 2];
#pragma unroll
    for (int p = 0; p < kPixW / 2; ++p) {
        up[p] = f2::pack(u[2 * p], u[2 * p + 1]);
        uup[p] = f2::pack(uu[2 * p], uu[2 * p + 1]);
    }
#pragma unroll
    for (int p = 0; p < kPixH / 2; ++p) {
        vp[p] = f2::pack(v[2 * p], v[2 * p + 1]);
        vvp[p] = f2::pack(vv[2 * p], vv[2 * p + 1]);
    }

#pragma unroll
    for (int k = 0; k < kPixH * kPixW; ++k) s_acc[k * kThreads + threadIdx.x] = make_double2(0.0, 0.0);

    const int64_t n = jg.n_points;
    const int64_t range_end = jg.p1 > 0 ? min(jg.p1, n) : n;
    const int64_t p_beg = jg.p0 + (int64_t)part * jg.points_per_split;
    const int64_t p_end = min(range_end, p_beg + jg.points_per_split);
    const PointRec* chrec = recs + (int64_t)ch * n;

    for (int64_t cb = p_beg; cb < p_end; cb += kChunk) {
        int cls[2];   // 0 skip, 1 FAST (window holds the tile, small phase spans), 2 CUT
        FrSRec tmp[2];
#pragma unroll
        for (int q = 0; q < 2; ++q) {
            cls[q] = 0;
            const int64_t idx = cb + threadIdx.x + q * kThreads;
            if (idx < p_end) {
                const PointRec p = chrec[idx];
                const int ix0 = max(X0, p.x_lo), ix1 = min(vx1, p.x_hi);
                const int iy0 = max(Y0, p.y_lo), iy1 = min(vy1, p.y_hi);
                if (ix0 < ix1 && iy0 < iy1) {
                    const double dxc = Xc - p.x, dyc = Yc - p.y;
                    const double s = p.aux;   // 1 / (2 z lambda)
                    const double tc = (dxc * dxc + dyc * dyc + 2.0 * p.z * p.z) * s;
                    FrSRec& t = tmp[q];
                    const float P = (float)(2.0 * dxc * s), Q = (float)(2.0 * dyc * s), sf = (float)s;
                    const float fc = (float)(tc - rint(tc));
                    const bool full = p.x_lo <= X0 && p.x_hi >= vx1 && p.y_lo <= Y0 && p.y_hi >= vy1;
                    // column phase fc + P u + s u^2 and row phase Q v + s v^2 (turns) over the tile
                    const float colspan = 0.5f + fabsf(P) * uext_f + sf * uext_f * uext_f;
                    const float rowspan = fabsf(Q) * vext_f + sf * vext_f * vext_f;
                    if (full && colspan < kMaxTurns && rowspan < kMaxTurns) {
                        cls[q] = 1;   // phases in radians, no masks, no reduction
                        t.P = make_float2(kTwoPi * P, kTwoPi * P);
                        t.Q = make_float2(kTwoPi * Q, kTwoPi * Q);
                        t.s = make_float2(kTwoPi * sf, kTwoPi * sf);
                        t.fc = make_float2(kTwoPi * fc, kTwoPi * fc);
                    } else {
                        cls[q] = 2;
                        t.P = make_float2(P, P);
                        t.Q = make_float2(Q, Q);
                        t.s = make_float2(sf, sf);
                        t.fc = make_float2(fc, fc);
                    }
                    t.ac = (float)p.coef;
                    t.xl = p.x_lo - X0;
                    t.xh = p.x_hi - X0;
                    t.yl = p.y_lo - Y0;
                    t.yh = p.y_hi - Y0;
                }
            }
        }
        // deterministic compaction: FAST from the front, CUT from the back
        unsigned bf[2], bc[2];
#pragma unroll
        for (int q = 0; q < 2; ++q) {
            bf[q] = __ballot_sync(0xffffffffu, cls[q] == 1);
            bc[q] = __ballot_sync(0xffffffffu, cls[q] == 2);
            if ((threadIdx.x & 31) == 0) {
                s_cnt[0][q][warp] = __popc(bf[q]);
                s_cnt[1][q][warp] = __popc(bc[q]);
            }
        }
        __syncthreads();
        int n_fast = 0, n_cut = 0, off_f[2], off_c[2];
#pragma unroll
        for (int q = 0; q < 2; ++q) {
#pragma unroll
            for (int w = 0; w < kThreads / 32; ++w) {
                if (w == warp) {
                    off_f[q] = n_fast;
                    off_c[q] = n_cut;
                }
                n_fast += s_cnt[0][q][w];
                n_cut += s_cnt[1][q][w];
            }
        }
#pragma unroll
        for (int q = 0; q < 2; ++q) {
            if (cls[q] == 1) s_rec[off_f[q] + warp_prefix(bf[q])] = tmp[q];
            else if (cls[q] == 2) s_rec[kChunk - 1 - (off_c[q] + warp_prefix(bc[q]))] = tmp[q];
        }
        __syncthreads();

        // accumulators: one packed (re, im) pair per pixel
        f2::v2 acc[kPixH * kPixW];
#pragma unroll
        for (int k = 0; k < kPixH * kPixW; ++k) acc[k] = 0ull;
        const f2::v2 two_pi = f2::splat(kTwoPi);
        // ---- FAST: radians, no window masks, no reduction -----------------
#pragma unroll 1
        for (int j = 0; j < n_fast; ++j) {
            const ulonglong2* R = reinterpret_cast<const ulonglong2*>(&s_rec[j]);
            const ulonglong2 r0 = R[0], r1 = R[1];
            const f2::v2 P = r0.x, Q = r0.y, sp = r1.x, fc = r1.y;
            const float ac = s_rec[j].ac;
            f2::v2 ca[kPixW], cb[kPixW];
#pragma unroll
            for (int p = 0; p < kPixW / 2; ++p) {
                const f2::v2 t = f2::fma(P, up[p], f2::fma(sp, uup[p], fc));
                float x[2];
                f2::unpack(t, x[0], x[1]);
#pragma unroll
                for (int k = 0; k < 2; ++k) {
                    float sn, cs;
                    __sincosf(x[k], &sn, &cs);
                    ca[2 * p + k] = f2::splat(ac * cs);
                    cb[2 * p + k] = f2::splat(ac * sn);
                }
            }
            f2::v2 r1p[kPixH], r2p[kPixH];
#pragma unroll
            for (int p = 0; p < kPixH / 2; ++p) {
                const f2::v2 t = f2::fma(Q, vp[p], f2::mul(sp, vvp[p]));
                float x[2];
                f2::unpack(t, x[0], x[1]);
#pragma unroll
                for (int k = 0; k < 2; ++k) {
                    float sn, cs;
                    __sincosf(x[k], &sn, &cs);
                    r1p[2 * p + k] = f2::pack(cs, sn);
                    r2p[2 * p + k] = f2::pack(-sn, cs);
                }
            }
#pragma unroll
            for (int r = 0; r < kPixH; ++r) {
#pragma unroll
                for (int c = 0; c < kPixW; ++c) {
                    const int k = r * kPixW + c;
                    acc[k] = f2::fma(ca[c], r1p[r], f2::fma(cb[c], r2p[r], acc[k]));
                }
            }
        }
        // ---- CUT: the window cuts the tile or a phase span is large --------
#pragma unroll 1
        for (int jj = 0; jj < n_cut; ++jj) {
            const int j = kChunk - 1 - jj;
            const ulonglong2* R = reinterpret_cast<const ulonglong2*>(&s_rec[j]);
            const ulonglong2 r0 = R[0], r1 = R[1];
            const f2::v2 P = r0.x, Q = r0.y, sp = r1.x, fc = r1.y;
            const float ac = s_rec[j].ac;
            const int4 wb = *reinterpret_cast<const int4*>(&s_rec[j].xl);
            // column factors ac*e^{i 2pi alpha_c}, broadcast into pairs
            f2::v2 ca[kPixW], cb[kPixW];
#pragma unroll
            for (int p = 0; p < kPixW / 2; ++p) {
                f2::v2 t = f2::fma(P, up[p], f2::fma(sp, uup[p], fc));
                t = f2::mul(f2::reduce_turns(t), two_pi);
                float x[2];
                f2::unpack(t, x[0], x[1]);
#pragma unroll
                for (int k = 0; k < 2; ++k) {
                    const int c = 2 * p + k;
                    const int cl = tx * kPixW + c;
                    float sn, cs;
                    __sincosf(x[k], &sn, &cs);
                    const float m = (cl >= wb.x && cl < wb.y) ? ac : 0.f;
                    ca[c] = f2::splat(m * cs);
                    cb[c] = f2::splat(m * sn);
                }
            }
            // row factors e^{i 2pi beta_r} as (c, d) and (-d, c)
            f2::v2 r1p[kPixH], r2p[kPixH];
#pragma unroll
            for (int p = 0; p < kPixH / 2; ++p) {
                f2::v2 t = f2::fma(Q, vp[p], f2::mul(sp, vvp[p]));
                t = f2::mul(f2::reduce_turns(t), two_pi);
                float x[2];
                f2::unpack(t, x[0], x[1]);
#pragma unroll
                for (int k = 0; k < 2; ++k) {
                    const int r = 2 * p + k;
                    const int rl = ty * kPixH + r;
                    float sn, cs;
                    __sincosf(x[k], &sn, &cs);
                    const float m = (rl >= wb.z && rl < wb.w) ? 1.f : 0.f;
                    r1p[r] = f2::pack(m * cs, m * sn);
                    r2p[r] = f2::pack(-m * sn, m * cs);
                }
            }
#pragma unroll
            for (int r = 0; r < kPixH; ++r) {
#pragma unroll
                for (int c = 0; c < kPixW; ++c) {
                    const int k = r * kPixW + c;
                    acc[k] = f2::fma(ca[c], r1p[r], f2::fma(cb[c], r2p[r], acc[k]));
                }
            }
        }
        float sr[kPixH * kPixW], si[kPixH * kPixW];
#pragma unroll
        for (int k = 0; k < kPixH * kPixW; ++k) f2::unpack(acc[k], sr[k], si[k]);
#pragma unroll
        for (int k = 0; k < kPixH * kPixW; ++k) {
            double2 a = s_acc[k * kThreads + threadIdx.x];
            a.x += (double)sr[k];
            a.y += (double)si[k];
            s_acc[k * kThreads + threadIdx.x] = a;
        }
        __syncthreads();
    }

    // H = -i * S: the reference's (sin phi, -cos phi) = (Im e^{i phi}, -Re e^{i phi})
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
                *o = make_double2(prev.x + a.y, prev.y - a.x);
            } else {
                *o = make_double2(a.y, -a.x);
            }
        }
    }
}

__global__ void sum_partials_kernel(double2* __restrict__ field, const double2* __restrict__ partials,
                                    int64_t n, int nparts) {
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    double2 a = field[i];
    for (int p = 0; p < nparts; ++p) {
        const double2 b = partials[(int64_t)p * n + i];
        a.x += b.x;
        a.y += b.y;
    }
    field[i] = a;
}

}  // namespace

constexpr size_t kFresnelSmem = sizeof(FrSRec) * kChunk + sizeof(double2) * kPixH * kPixW * kThreads;

cudaError_t fresnel_set_smem_limit() {
    return cudaFuncSetAttribute(fresnel_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kFresnelSmem);
}

int fresnel_blocks_per_sm() {
    fresnel_set_smem_limit();
    int nb = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, fresnel_kernel, kThreads, kFresnelSmem) != cudaSuccess) nb = 1;
    return nb > 0 ? nb : 1;
}

void launch_fresnel(const PointRec* d_recs, const JobGeom& jg, double2* d_field, double2* d_partials,
                    cudaStream_t stream) {
    dim3 grid((unsigned)jg.tiles_x, (unsigned)jg.tiles_y, (unsigned)(jg.n_channels * jg.ksplit));
    count_launches(1);
    fresnel_kernel<<<grid, kThreads, kFresnelSmem, stream>>>(d_recs, jg, d_field, d_partials);
}

void launch_sum_partials(const JobGeom& jg, double2* d_field, const double2* d_partials,
                         cudaStream_t stream) {
    if (jg.ksplit <= 1) return;
    const int64_t n = (int64_t)jg.n_channels * jg.ch[0].pnX * (int64_t)jg.ch[0].pnY;
    const int threads = 256;
    count_launches(1);
    sum_partials_kernel<<<(unsigned)((n + threads - 1) / threads), threads, 0, stream>>>(
        d_field, d_partials, n, jg.ksplit - 1);
}

}  // namespace ophpc
