// Tensor-core Fresnel (tcgen05, sm_103a): the Fresnel sum as a separable
// complex contraction over the points,
//
//   S(y, x) = sum_j A_j(y) B_j(x),   H = -i * cmax * S
//   A_j(y) = (a_j / cmax) e^{i 2 pi (z_j/lambda + (Y_y - y_j)^2 s_j)} [y in window]
//   B_j(x) = e^{i 2 pi (X_x - x_j)^2 s_j} [x in window],   s_j = 1 / (2 z_j lambda)
//
// which is exactly the reference's Fresnel term (ophgen/src/ophGen.cpp:447-514):
// phi/2pi = ((X-x)^2 + (Y-y)^2 + 2 z^2) s and the window rectangle factorises.
//
// Two kernels per chunk of points:
//   tc_table_kernel  A (pnY x K) and B (pnX x K) factor tables, re and im
//                    planes, 16-bit (FP16, or BF16 hi + lo), K-major rows.
//                    The phase is reduced mod 1 in FP64 once per (point,
//                    32-pixel segment) and carried in FP32 inside a segment.
//   tc_gemm_kernel   one CTA per 128x128 output tile: TMA (128B swizzle) ->
//                    shared memory (3-stage ring, mbarriers) -> tcgen05.mma
//                    kind::f16 issued by one thread into FP32 accumulators
//                    D_re, D_im in TMEM. The tensor core's accumulation
//                    loses ~1e-8 of the sum per point accumulated, so the
//                    accumulators are double-buffered (512 columns) and
//                    every 1024 points 8 epilogue warps drain one buffer
//                    (tcgen05.ld) into FP32 registers while the MMAs fill the
//                    other; at the end they add into FP64 sums in global
//                    memory.
//   Per k-block four real products: D_re += Ar Br - Ai Bi (the second with
//   the A-negate bit), D_im += Ar Bi + Ai Br. Split-BF16 runs three passes
//   over K: (hi, hi), (hi, lo), (lo, hi).
// A final kernel writes the FP64 field (H = -i cmax S).
//
// Every mbarrier wait is bounded (%globaltimer); on a timeout the CTA sets
// an error word, drains its own TMA copies and MMAs, frees TMEM and returns.
#include "pc_tc.cuh"

#include "pc_common.cuh"
#include "pc_tcgen05.cuh"

#include <cuda.h>
#include <cuda_bf16.h>
#include <cuda_fp16.h>

#include <algorithm>
#include <cmath>
#include <cstring>
#include <mutex>

namespace ophpc {
namespace {

using namespace tc5;

constexpr int kBM = 128;            // SLM rows per tile = TMEM lanes
constexpr int kBN = 128;            // SLM columns per tile
constexpr int kBK = 64;             // points per k-block: one 128-byte swizzle row of 16-bit values
constexpr int kStages = 3;
constexpr int kTileBytes = kBM * kBK * 2;           // 16 KB (A and B tiles alike)
constexpr int kStageBytes = 4 * kTileBytes;         // Ar, Ai, Br, Bi
constexpr int kAccCols = 2 * kBN;                   // one accumulator buffer: D_re [0,128), D_im [128,256)
constexpr int kTmemCols = 2 * kAccCols;             // two buffers (all 512 TMEM columns)
constexpr int kEpiWarps = 8;                        // 2 per TMEM lane group, each half of the columns
constexpr int kEpiCols = kBN / (kEpiWarps / 4);     // 64 columns of D_re and of D_im per epilogue thread
constexpr int kGemmThreads = 64 + 32 * kEpiWarps;   // warp 0 TMA, warp 1 MMA + TMEM, warps 2-9 epilogue
static_assert(kEpiCols % 16 == 0, "16-column TMEM loads");
static_assert(2 * kBM * (kBN + 1) * 4 <= kStages * kStageBytes, "epilogue staging fits in the stage ring");
// k-blocks accumulated in TMEM before the epilogue drains them into FP32
// registers: the tensor-core accumulator loses ~1e-8 of the sum per point,
// so runs are kept to 16 k-blocks (1024 points).
constexpr int kDrainKb = 16;
constexpr int kSeg = 32;                            // table rows per FP64 phase reduction
constexpr int kTablePoints = 128;                   // points per table-kernel block
constexpr uint64_t kWaitLimitNs = 10ull * 1000 * 1000 * 1000;   // 10 s per wait
constexpr size_t kGemmSmem = (size_t)kStages * kStageBytes + 1024 + 256;


// Instruction descriptor of this kernel's MMAs: M = 128, N = kBN.
__host__ __device__ constexpr uint32_t make_idesc(uint32_t ab_format, bool negate_a) {
    return idesc_f16(ab_format, negate_a, kBM, kBN);
}

// ------------------------------------------------------------------ tables

struct TableArgs {
    int64_t n_points;        // points of this channel
    int64_t k0;              // first point of the chunk
    int32_t kc;              // points in the chunk
    int32_t ld;              // row length of every table (kc rounded up to kBK)
    int32_t rows_a, rows_b;  // pnY, pnX
    int32_t split;           // 1: BF16 hi + lo, 0: FP16
    int32_t pad;
    ChannelGeom g;
    const float* cmax;       // device: max amplitude coefficient
    void* ar[2];             // [hi, lo] planes (lo only when split)
    void* ai[2];
    void* br[2];
    void* bi[2];
};

template <typename T>
__device__ __forceinline__ T to16(float x);
template <>
__device__ __forceinline__ __half to16<__half>(float x) { return __float2half_rn(x); }
template <>
__device__ __forceinline__ __nv_bfloat16 to16<__nv_bfloat16>(float x) { return __float2bfloat16_rn(x); }
template <typename T>
__device__ __forceinline__ float from16(T x);
template <>
__device__ __forceinline__ float from16<__half>(__half x) { return __half2float(x); }
template <>
__device__ __forceinline__ float from16<__nv_bfloat16>(__nv_bfloat16 x) { return __bfloat162float(x); }

template <typename T>
__device__ __forceinline__ void put(void* const* plane, int split, size_t off, float v) {
    const T hi = to16<T>(v);
    static_cast<T*>(plane[0])[off] = hi;
    if (split) static_cast<T*>(plane[1])[off] = to16<T>(v - from16<T>(hi));
}

// Grid: x = point blocks of the chunk, y = 32-row segments of A then of B.
template <typename T>
__global__ void __launch_bounds__(kTablePoints) tc_table_kernel(const PointRec* __restrict__ recs, TableArgs a) {
    const int local = blockIdx.x * kTablePoints + threadIdx.x;   // column of the tables
    if (local >= a.ld) return;
    const int segs_a = (a.rows_a + kSeg - 1) / kSeg;
    const bool is_a = (int)blockIdx.y < segs_a;
    const int seg = is_a ? (int)blockIdx.y : (int)blockIdx.y - segs_a;
    const int rows = is_a ? a.rows_a : a.rows_b;
    const int r0 = seg * kSeg, r1 = min(r0 + kSeg, rows);
    const int64_t j = a.k0 + local;
    void* const* re = is_a ? a.ar : a.br;
    void* const* im = is_a ? a.ai : a.bi;
    if (local >= a.kc || j >= a.n_points) {
        for (int r = r0; r < r1; ++r) {
            put<T>(re, a.split, (size_t)r * a.ld + local, 0.f);
            put<T>(im, a.split, (size_t)r * a.ld + local, 0.f);
        }
        return;
    }
    const PointRec p = recs[j];
    const ChannelGeom& g = a.g;
    const double s = p.aux;                        // 1 / (2 z lambda)
    const int rc = r0 + kSeg / 2;                  // segment centre pixel
    double tc, dc;
    float pitch;
    int lo, hi;
    if (is_a) {
        // rows: phi_A / 2pi = (dy^2 + 2 z^2) s ; Y falls with the row index
        dc = pixel_y(g, rc) - p.y;
        tc = (dc * dc + 2.0 * p.z * p.z) * s;
        pitch = -(float)g.ppY;
        lo = p.y_lo;
        hi = p.y_hi;
    } else {
        dc = pixel_x(g, rc) - p.x;
        tc = dc * dc * s;
        pitch = (float)g.ppX;
        lo = p.x_lo;
        hi = p.x_hi;
    }
    const float fc = (float)(tc - rint(tc));
    const float P = (float)(2.0 * dc * s), sf = (float)s;
    const float cm = *a.cmax;
    const float amp = is_a ? (cm > 0.f ? (float)p.coef / cm : 0.f) : 1.f;
    for (int r = r0; r < r1; ++r) {
        const float d = (float)(r - rc) * pitch;   // offset from the segment centre
        float t = fmaf(d, fmaf(sf, d, P), fc);
        t = reduce_turns(t);
        float sn, cs;
        __sincosf(t * 6.283185307179586f, &sn, &cs);
        const float m = (r >= lo && r < hi) ? amp : 0.f;
        put<T>(re, a.split, (size_t)r * a.ld + local, m * cs);
        put<T>(im, a.split, (size_t)r * a.ld + local, m * sn);
    }
}

__global__ void cmax_kernel(const PointRec* __restrict__ recs, int64_t n, float* out) {
    float m = 0.f;
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
        m = fmaxf(m, fabsf((float)recs[i].coef));
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) m = fmaxf(m, __shfl_xor_sync(0xffffffffu, m, o));
    if ((threadIdx.x & 31) == 0) atomicMax(reinterpret_cast<int*>(out), __float_as_int(m));   // m >= 0
}

// ------------------------------------------------------------------ GEMM

struct GemmMaps {
    CUtensorMap ar[3], ai[3], br[3], bi[3];   // per pass
};

struct GemmArgs {
    int32_t num_kb;          // k-blocks per pass
    int32_t passes;          // 1 (FP16) or 3 (split-BF16)
    int32_t pnX, pnY;
    int32_t accumulate;      // add into the FP64 sums (0: overwrite)
    uint32_t idesc, idesc_neg;
    double* sum_re;          // [pnY][pnX]
    double* sum_im;
    int* error;
};

__global__ void __launch_bounds__(kGemmThreads, 1)
tc_gemm_kernel(const __grid_constant__ GemmMaps maps, const GemmArgs args) {
    extern __shared__ __align__(1024) unsigned char smem_raw[];
    // stage buffers on a 1024-byte boundary (128-byte swizzle atoms)
    unsigned char* base = (unsigned char*)(((uintptr_t)smem_raw + 1023) & ~(uintptr_t)1023);
    uint64_t* full = reinterpret_cast<uint64_t*>(base + kStages * kStageBytes);
    uint64_t* empty = full + kStages;
    uint64_t* acc_full = empty + kStages;    // [2]: MMA -> epilogue, buffer ready
    uint64_t* acc_empty = acc_full + 2;      // [2]: epilogue -> MMA, buffer drained
    uint64_t* drain = acc_empty + 2;         // abort path: issued MMAs complete
    uint32_t* tmem_slot = reinterpret_cast<uint32_t*>(drain + 1);
    volatile int* abort = reinterpret_cast<volatile int*>(tmem_slot + 1);

    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int n0 = blockIdx.x * kBN, m0 = blockIdx.y * kBM;
    const int total = args.num_kb * args.passes;
    const int periods = (total + kDrainKb - 1) / kDrainKb;
    const uint64_t t0 = global_ns();

    if (threadIdx.x == 0) {
        for (int s = 0; s < kStages; ++s) {
            mbar_init(&full[s], 1);
            mbar_init(&empty[s], 1);
        }
        for (int b = 0; b < 2; ++b) {
            mbar_init(&acc_full[b], 1);
            mbar_init(&acc_empty[b], kEpiWarps);
        }
        mbar_init(drain, 1);
        *abort = 0;
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    if (warp == 1) tmem_alloc(tmem_slot, kTmemCols);
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    const uint32_t tmem = *tmem_slot;
    int issued = 0;   // producer: k-iterations whose TMA was issued

    if (warp == 0 && lane == 0) {
        // ---------------- TMA producer
        for (int it = 0; it < total; ++it) {
            const int s = it % kStages;
            const uint32_t ph = (uint32_t)(it / kStages) & 1u;
            if (!mbar_wait(&empty[s], ph ^ 1u, abort, t0 + kWaitLimitNs)) break;
            const int pass = it / args.num_kb, kb = it % args.num_kb;
            unsigned char* st = base + s * kStageBytes;
            mbar_expect_tx(&full[s], kStageBytes);
            const int kx = kb * kBK;
            tma_load_2d(st + 0 * kTileBytes, &maps.ar[pass], &full[s], kx, m0);
            tma_load_2d(st + 1 * kTileBytes, &maps.ai[pass], &full[s], kx, m0);
            tma_load_2d(st + 2 * kTileBytes, &maps.br[pass], &full[s], kx, n0);
            tma_load_2d(st + 3 * kTileBytes, &maps.bi[pass], &full[s], kx, n0);
            ++issued;
        }
    } else if (warp == 1 && lane == 0) {
        // ---------------- MMA issuer
        int it = 0;
        for (; it < total; ++it) {
            const int p = it / kDrainKb, b = p & 1;
            const bool opens = (it % kDrainKb) == 0;
            // buffer b last held period p-2: wait until the epilogue drained it
            if (opens && p >= 2 &&
                !mbar_wait(&acc_empty[b], (uint32_t)((p / 2) - 1) & 1u, abort, t0 + kWaitLimitNs))
                break;
            const int s = it % kStages;
            const uint32_t ph = (uint32_t)(it / kStages) & 1u;
            if (!mbar_wait(&full[s], ph, abort, t0 + kWaitLimitNs)) break;
            tc_fence_after();
            const uint32_t d_re = tmem + (uint32_t)(b * kAccCols), d_im = d_re + kBN;
            const uint32_t st = smem_u32(base + s * kStageBytes);
            const uint64_t dar = sw128_desc(st), dai = sw128_desc(st + kTileBytes);
            const uint64_t dbr = sw128_desc(st + 2 * kTileBytes), dbi = sw128_desc(st + 3 * kTileBytes);
#pragma unroll
            for (int kk = 0; kk < kBK / 16; ++kk) {
                const uint64_t o = (uint64_t)(kk * 32) >> 4;   // 16 values = 32 bytes along K
                const uint32_t first = (opens && kk == 0) ? 0u : 1u;
                umma(d_re, dar + o, dbr + o, args.idesc, first);
                umma(d_re, dai + o, dbi + o, args.idesc_neg, 1u);
                umma(d_im, dar + o, dbi + o, args.idesc, first);
                umma(d_im, dai + o, dbr + o, args.idesc, 1u);
            }
            umma_commit(&empty[s]);   // frees the stage once these MMAs have read it
            if ((it % kDrainKb) == kDrainKb - 1 || it == total - 1) umma_commit(&acc_full[b]);
        }
        if (it != total) {
            // aborted: track the MMAs already issued and wait (bounded) for
            // them before TMEM is released
            umma_commit(drain);
            const uint64_t dl = global_ns() + 1000ull * 1000 * 1000;
            while (!mbar_try_wait(drain, 0) && global_ns() < dl) {
            }
        }
    } else if (warp >= 2) {
        // ---------------- epilogue: TMEM -> FP32 registers, per period
        const int grp = warp & 3;                      // TMEM lanes 32*grp .. +31
        const int quarter = (warp - 2) >> 2;           // column block [kEpiCols*quarter, +kEpiCols)
        const uint32_t lane_addr = (uint32_t)(grp * 32) << 16;
        // one row (TMEM lane), kEpiCols columns of D_re and D_im, in FP32 registers
        float acc_re[kEpiCols], acc_im[kEpiCols];
#pragma unroll
        for (int i = 0; i < kEpiCols; ++i) acc_re[i] = acc_im[i] = 0.f;
        bool ok = true;
        for (int p = 0; p < periods && ok; ++p) {
            const int b = p & 1;
            ok = mbar_wait(&acc_full[b], (uint32_t)(p / 2) & 1u, abort, t0 + kWaitLimitNs);
            tc_fence_after();
            ok = __all_sync(0xffffffffu, ok && !*abort);   // tcgen05.ld is warp-collective
            if (!ok) break;
            const uint32_t col = tmem + lane_addr + (uint32_t)(b * kAccCols + quarter * kEpiCols);
#pragma unroll
            for (int c = 0; c < kEpiCols; c += 16) {
                tmem_ld16_add(col + (uint32_t)c, acc_re + c);
                tmem_ld16_add(col + (uint32_t)(kBN + c), acc_im + c);
            }
            tc_fence_before();
            __syncwarp();
            if (lane == 0) mbar_arrive(&acc_empty[b]);
        }
        // Stage the tile through shared memory (the stage ring is idle once
        // the last period has drained: every TMA load has been consumed), so
        // that the FP64 read-modify-write of the sums is row-contiguous.
        constexpr int kLd = kBN + 1;   // padded row: conflict-free column writes
        float* tre = reinterpret_cast<float*>(base);
        float* tim = tre + kBM * kLd;
        if (ok) {
            const int r = grp * 32 + lane;
#pragma unroll
            for (int i = 0; i < kEpiCols; ++i) {
                tre[r * kLd + quarter * kEpiCols + i] = acc_re[i];
                tim[r * kLd + quarter * kEpiCols + i] = acc_im[i];
            }
        }
        asm volatile("bar.sync 1, %0;" ::"n"(32 * kEpiWarps) : "memory");   // epilogue warps only
        if (!*abort) {
            const int t = threadIdx.x - 64;
            for (int idx = t; idx < kBM * kBN; idx += 32 * kEpiWarps) {
                const int r = idx / kBN, c = idx % kBN;
                const int row = m0 + r, colx = n0 + c;
                if (row < args.pnY && colx < args.pnX) {
                    const size_t o = (size_t)row * args.pnX + colx;
                    const double vr = (double)tre[r * kLd + c], vi = (double)tim[r * kLd + c];
                    args.sum_re[o] = args.accumulate ? args.sum_re[o] + vr : vr;
                    args.sum_im[o] = args.accumulate ? args.sum_im[o] + vi : vi;
                }
            }
        }
    }
    // on abort the producer waits (bounded) for its copies still in flight:
    // the most recent use of each stage
    if (warp == 0 && lane == 0 && *abort) {
        const uint64_t dl = global_ns() + 1000ull * 1000 * 1000;
        for (int it = max(0, issued - kStages); it < issued; ++it) {
            const int s = it % kStages;
            const uint32_t ph = (uint32_t)(it / kStages) & 1u;
            while (!mbar_try_wait(&full[s], ph) && global_ns() < dl) {
            }
        }
    }
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    if (warp == 1) tmem_dealloc(tmem, kTmemCols);
    if (threadIdx.x == 0 && *abort) atomicExch(args.error, 1);
}

__global__ void tc_finalize_kernel(const double* __restrict__ sre, const double* __restrict__ sim,
                                   const float* __restrict__ cmax, int64_t n, double2* __restrict__ field) {
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const double c = (double)*cmax;
    // H = -i * cmax * S: the reference's (sin phi, -cos phi) terms
    field[i] = make_double2(sim[i] * c, -sre[i] * c);
}

// ------------------------------------------------------------------ host

typedef CUresult (*EncodeTiledFn)(CUtensorMap*, CUtensorMapDataType, cuuint32_t, void*, const cuuint64_t*,
                                  const cuuint64_t*, const cuuint32_t*, const cuuint32_t*, CUtensorMapInterleave,
                                  CUtensorMapSwizzle, CUtensorMapL2promotion, CUtensorMapFloatOOBfill);

EncodeTiledFn encode_fn() {
    static EncodeTiledFn fn = nullptr;
    static std::once_flag once;
    std::call_once(once, [] {
        void* p = nullptr;
        cudaDriverEntryPointQueryResult q;
        if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) ==
                cudaSuccess &&
            q == cudaDriverEntryPointSuccess)
            fn = reinterpret_cast<EncodeTiledFn>(p);
    });
    return fn;
}

bool make_map(CUtensorMap* m, void* base, int rows, int ld, bool bf16) {
    EncodeTiledFn fn = encode_fn();
    if (!fn) return false;
    const cuuint64_t dims[2] = {(cuuint64_t)ld, (cuuint64_t)rows};
    const cuuint64_t strides[1] = {(cuuint64_t)ld * 2};
    const cuuint32_t box[2] = {(cuuint32_t)kBK, (cuuint32_t)kBM};
    const cuuint32_t estr[2] = {1, 1};
    return fn(m, bf16 ? CU_TENSOR_MAP_DATA_TYPE_BFLOAT16 : CU_TENSOR_MAP_DATA_TYPE_FLOAT16, 2, base, dims, strides,
              box, estr, CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_128B,
              CU_TENSOR_MAP_L2_PROMOTION_L2_256B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) == CUDA_SUCCESS;
}

size_t align_up(size_t v, size_t a) { return (v + a - 1) / a * a; }

}  // namespace

static_assert(sizeof(GemmMaps) <= sizeof(((TcFresnelPlan*)nullptr)->maps), "tensor maps fit the plan");

size_t tc_fresnel_table_bytes(int pnX, int pnY, int ld, bool split) {
    const size_t plane_a = align_up((size_t)pnY * ld * 2, 1024), plane_b = align_up((size_t)pnX * ld * 2, 1024);
    return (2 * plane_a + 2 * plane_b) * (split ? 2 : 1);
}

int tc_fresnel_chunk_multiple() { return kBK; }

bool tc_fresnel_plan(TcFresnelPlan* plan, void* table_mem, int pnX, int pnY, int ld, bool split) {
    if (!encode_fn() || ld <= 0 || ld % kBK != 0) return false;
    std::memset(plan, 0, sizeof(*plan));
    plan->pnX = pnX;
    plan->pnY = pnY;
    plan->ld = ld;
    plan->split = split;
    const size_t plane_a = align_up((size_t)pnY * ld * 2, 1024), plane_b = align_up((size_t)pnX * ld * 2, 1024);
    unsigned char* q = static_cast<unsigned char*>(table_mem);
    for (int p = 0; p < (split ? 2 : 1); ++p) {
        plan->ar[p] = q; q += plane_a;
        plan->ai[p] = q; q += plane_a;
        plan->br[p] = q; q += plane_b;
        plan->bi[p] = q; q += plane_b;
    }
    GemmMaps* maps = reinterpret_cast<GemmMaps*>(plan->maps);
    // pass p: (A plane, B plane) = (hi, hi), (hi, lo), (lo, hi)
    const int pa[3] = {0, 0, 1}, pb[3] = {0, 1, 0};
    bool ok = true;
    for (int p = 0; p < (split ? 3 : 1); ++p) {
        ok = ok && make_map(&maps->ar[p], plan->ar[pa[p]], pnY, ld, split) &&
             make_map(&maps->ai[p], plan->ai[pa[p]], pnY, ld, split) &&
             make_map(&maps->br[p], plan->br[pb[p]], pnX, ld, split) &&
             make_map(&maps->bi[p], plan->bi[pb[p]], pnX, ld, split);
    }
    return ok;
}

void launch_tc_fresnel_cmax(const PointRec* d_recs_ch, int64_t n_points, float* d_cmax, cudaStream_t s) {
    count_launches(1);
    cmax_kernel<<<256, 256, 0, s>>>(d_recs_ch, n_points, d_cmax);
}

cudaError_t launch_tc_fresnel_chunk(const TcFresnelPlan& plan, const PointRec* d_recs_ch, int64_t n_points,
                                    const ChannelGeom& g, int64_t k0, int kc, const float* d_cmax, double* sum_re,
                                    double* sum_im, bool accumulate, int* d_err, cudaStream_t s) {
    // per call: the attribute belongs to the current device
    cudaError_t e = cudaFuncSetAttribute(tc_gemm_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kGemmSmem);
    if (e != cudaSuccess) return e;
    TableArgs ta;
    std::memset(&ta, 0, sizeof(ta));
    ta.n_points = n_points;
    ta.k0 = k0;
    ta.kc = std::min(kc, plan.ld);
    ta.ld = plan.ld;
    ta.rows_a = plan.pnY;
    ta.rows_b = plan.pnX;
    ta.split = plan.split ? 1 : 0;
    ta.g = g;
    ta.cmax = d_cmax;
    for (int p = 0; p < 2; ++p) {
        ta.ar[p] = plan.ar[p];
        ta.ai[p] = plan.ai[p];
        ta.br[p] = plan.br[p];
        ta.bi[p] = plan.bi[p];
    }
    const int segs = (plan.pnY + kSeg - 1) / kSeg + (plan.pnX + kSeg - 1) / kSeg;
    const dim3 tgrid((unsigned)((plan.ld + kTablePoints - 1) / kTablePoints), (unsigned)segs);
    count_launches(2);
    if (plan.split)
        tc_table_kernel<__nv_bfloat16><<<tgrid, kTablePoints, 0, s>>>(d_recs_ch, ta);
    else
        tc_table_kernel<__half><<<tgrid, kTablePoints, 0, s>>>(d_recs_ch, ta);
    GemmArgs ga;
    ga.num_kb = plan.ld / kBK;
    ga.passes = plan.split ? 3 : 1;
    ga.pnX = plan.pnX;
    ga.pnY = plan.pnY;
    ga.accumulate = accumulate ? 1 : 0;
    ga.idesc = make_idesc(plan.split ? 1u : 0u, false);
    ga.idesc_neg = make_idesc(plan.split ? 1u : 0u, true);
    ga.sum_re = sum_re;
    ga.sum_im = sum_im;
    ga.error = d_err;
    const dim3 ggrid((unsigned)((plan.pnX + kBN - 1) / kBN), (unsigned)((plan.pnY + kBM - 1) / kBM));
    tc_gemm_kernel<<<ggrid, kGemmThreads, kGemmSmem, s>>>(*reinterpret_cast<const GemmMaps*>(plan.maps), ga);
    return cudaGetLastError();
}

void launch_tc_fresnel_finalize(const double* sum_re, const double* sum_im, const float* d_cmax, int64_t plane,
                                double2* d_field_ch, cudaStream_t s) {
    count_launches(1);
    tc_finalize_kernel<<<(unsigned)((plane + 255) / 256), 256, 0, s>>>(sum_re, sum_im, d_cmax, plane, d_field_ch);
}

ophpc_status tc_generate_fresnel(cudaMemPool_t pool, const ophpc_config* cfg, const ophpc_vertex* d_vertices,
                                 uint64_t n_points, uint32_t mode, double* d_field, cudaStream_t s,
                                 std::string* err, int* d_err_out) {
    auto fail = [&](ophpc_status st, const char* msg) {
        if (err) *err = msg;
        return st;
    };
    const bool split = (mode & OPHPC_MODE_TENSOR_BF16X3) != 0;
    if (!encode_fn()) return fail(OPHPC_ERROR_UNSUPPORTED, "cuTensorMapEncodeTiled unavailable");
    const int pnX = cfg->pixel_number[0], pnY = cfg->pixel_number[1];
    const int64_t plane = (int64_t)pnX * pnY;
    const int nch = (int)cfg->n_channels;

    // geometry and point records, as the plain path forms them
    JobGeom jg;
    std::memset(&jg, 0, sizeof(jg));
    jg.n_channels = nch;
    jg.n_points = (int64_t)n_points;
    for (int c = 0; c < nch; ++c) {
        ChannelGeom& g = jg.ch[c];
        g.pnX = pnX;
        g.pnY = pnY;
        g.offX = cfg->offset[0];
        g.offY = cfg->offset[1];
        g.ppX = cfg->pixel_pitch[0];
        g.ppY = cfg->pixel_pitch[1];
        const double ssX = g.pnX * g.ppX, ssY = g.pnY * g.ppY;
        g.x0 = -ssX / 2;
        g.y0 = -ssY / 2;
        g.lambda = cfg->wave_length[c];
        g.inv_lambda = 1.0 / g.lambda;
        const double tx = g.lambda / (2 * g.ppX), ty = g.lambda / (2 * g.ppY);
        g.detx = tx / std::sqrt(1 - (tx * tx));
        g.dety = ty / std::sqrt(1 - (ty * ty));
    }

    // chunk of points per table build: tables of at most ~2 GiB
    const size_t per_point = (size_t)(pnX + pnY) * 2 * 2 * (split ? 2 : 1);
    int64_t kc = (int64_t)((size_t)2 << 30) / (int64_t)per_point;
    kc = std::max<int64_t>(kBK, std::min<int64_t>(kc, 65536));
    kc = kc / kBK * kBK;
    kc = std::min<int64_t>(kc, (int64_t)align_up(n_points, kBK));
    const int ld = (int)kc;
    const size_t table_bytes = tc_fresnel_table_bytes(pnX, pnY, ld, split);
    const size_t rec_bytes = sizeof(PointRec) * n_points * nch;
    const size_t sum_bytes = sizeof(double) * plane * 2;

    unsigned char* buf = nullptr;
    const size_t total = align_up(rec_bytes, 1024) + table_bytes + align_up(sum_bytes, 1024) + 1024;
    if (cudaMallocFromPoolAsync((void**)&buf, total, pool, s) != cudaSuccess)
        return fail(OPHPC_ERROR_OUT_OF_MEMORY, "tensor-core scratch allocation failed");
    unsigned char* q = buf;
    PointRec* recs = (PointRec*)q;
    q += align_up(rec_bytes, 1024);
    TcFresnelPlan plan;
    const bool planned = tc_fresnel_plan(&plan, q, pnX, pnY, ld, split);
    q += table_bytes;
    double* sre = (double*)q;
    double* sim = sre + plane;
    q += align_up(sum_bytes, 1024);
    float* cmax = (float*)q;
    int* errw = (int*)(q + 16);
    if (!planned) {
        cudaFreeAsync(buf, s);
        return fail(OPHPC_ERROR_CUDA, "tensor map encoding failed");
    }
    cudaMemsetAsync(errw, 0, sizeof(int), s);
    launch_prep(d_vertices, (int64_t)n_points, cfg->scale, cfg->distance, cfg->field_length, cfg->viewing_window, 1,
                jg, recs, s);
    cudaError_t e = cudaSuccess;
    for (int c = 0; c < nch && e == cudaSuccess; ++c) {
        const PointRec* crec = recs + (int64_t)c * n_points;
        cudaMemsetAsync(cmax, 0, sizeof(float), s);
        launch_tc_fresnel_cmax(crec, (int64_t)n_points, cmax, s);
        for (int64_t k0 = 0; k0 < (int64_t)n_points && e == cudaSuccess; k0 += kc)
            e = launch_tc_fresnel_chunk(plan, crec, (int64_t)n_points, jg.ch[c], k0,
                                        (int)std::min<int64_t>(kc, (int64_t)n_points - k0), cmax, sre, sim, k0 > 0, errw,
                                        s);
        launch_tc_fresnel_finalize(sre, sim, cmax, plane, (double2*)d_field + (int64_t)c * plane, s);
    }
    if (e == cudaSuccess) e = cudaGetLastError();
    int herr = 0;
    if (d_err_out) {   // read later by the caller (graph capture: nothing here may wait)
        if (e == cudaSuccess) e = cudaMemcpyAsync(d_err_out, errw, sizeof(int), cudaMemcpyDeviceToDevice, s);
    } else {
        if (e == cudaSuccess) e = cudaMemcpyAsync(&herr, errw, sizeof(int), cudaMemcpyDeviceToHost, s);
        if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    }
    cudaFreeAsync(buf, s);
    if (e != cudaSuccess) return fail(OPHPC_ERROR_CUDA, cudaGetErrorString(e));
    if (herr) return fail(OPHPC_ERROR_TIMEOUT, "tensor-core kernel wait timed out");
    return OPHPC_SUCCESS;
}

}  // namespace ophpc
