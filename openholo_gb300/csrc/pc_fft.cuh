// Batched FP64 complex FFTs along one axis of a row-major 2-D array, for the
// angular-spectrum propagation of the WRP generator (pc_wrp.cu).
//
// A transform of length n = r1 r2 ... rk (radices 8, 4, 2, 3, 5, 7) runs as k
// Stockham auto-sort passes; each pass reads the whole array and writes it
// to the other of two buffers, radix-r butterflies with the twiddles of that
// pass read from a table built once per plan. Rows (elements contiguous) or
// columns (elements a row apart) of any number of lines are transformed at
// once, the threads of a warp always on contiguous addresses. Forward is
// e^{-2 pi i j k / n}, inverse e^{+2 pi i j k / n}, neither normalised
// (FFTW's FFTW_FORWARD / FFTW_BACKWARD convention, which the reference
// uses).
#pragma once

#include <cstdint>
#include <cuda_runtime.h>

namespace ophpc {

constexpr int kFftMaxPasses = 40;

struct FftPlan {
    int n = 0;
    int passes = 0;
    int radix[kFftMaxPasses] = {};
    int ns[kFftMaxPasses] = {};              // product of the radices before the pass
    int64_t tw_offset[kFftMaxPasses] = {};   // into the twiddle table
    double2* twiddles = nullptr;             // device, fft_twiddle_count(n) entries
};

// True when n > 0 factors completely into the supported radices.
bool fft_supported(int n);
// Twiddle-table entries a plan of length n needs.
int64_t fft_twiddle_count(int n);
// Factorises n and fills `tw` (device memory of fft_twiddle_count(n)
// entries) on `stream`. False when n is not supported.
bool fft_plan_init(FftPlan* plan, int n, double2* tw, cudaStream_t stream);

// Transforms `lines` lines of length plan.n. Element e of line l sits at
// l * line_stride + e * elem_stride (elem_stride 1: rows; line_stride 1:
// columns). The data starts in buf[0] and the result is left in
// buf[result] (returned), the other buffer being overwritten on the way.
int fft_run(const FftPlan& plan, double2* const buf[2], int64_t lines, int64_t elem_stride, int64_t line_stride,
            bool inverse, cudaStream_t stream);

}  // namespace ophpc
