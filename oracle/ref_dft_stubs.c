/*
 * FFTW stand-ins that compute the transform, for the reference's side-band
 * build (oracle/_ref/libophref_sideband.so).
 *
 * TEST INFRASTRUCTURE ONLY. FFTW is not installed here; these definitions
 * implement the few FFTW calls the reference's ophGen::encodeSideBand_CPU
 * makes (a 2-D plan, fftw_execute_dft, fftw_malloc / fftw_free) with a
 * direct separable DFT in FP64: rows, then columns, each output element a
 * sum over the line with twiddles e^{sign 2 pi i j k / n} taken from a table
 * of cos / sin of 2 pi m / n (m = j k mod n). Unnormalised, FFTW's sign
 * convention (-1 forward, +1 backward). O(n^2) per line: for the small
 * fixture sizes only. The CUDA symbols of the reference's GPU encoders
 * abort if reached.
 */
#include <math.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

typedef struct {
    int nx, ny, sign;
    double* in;
    double* out;
} dft_plan;

static void unreachable(const char* name)
{
    fprintf(stderr, "oracle/_ref (side-band build): stubbed symbol %s was called\n", name);
    abort();
}

static void dft_lines(double* data, int n, int lines, long long elem_stride, long long line_stride, int sign)
{
    double* tw = (double*)malloc(sizeof(double) * 2 * (size_t)n);
    double* tmp = (double*)malloc(sizeof(double) * 2 * (size_t)n);
    for (int m = 0; m < n; ++m) {
        const double a = 2.0 * M_PI * (double)m / (double)n;
        tw[2 * m] = cos(a);
        tw[2 * m + 1] = sign * sin(a);
    }
    for (int l = 0; l < lines; ++l) {
        double* base = data + 2 * (size_t)(l * line_stride);
        for (int k = 0; k < n; ++k) {
            double re = 0.0, im = 0.0;
            for (int j = 0; j < n; ++j) {
                const int m = (int)(((long long)j * k) % n);
                const double* v = base + 2 * (size_t)(j * elem_stride);
                re += v[0] * tw[2 * m] - v[1] * tw[2 * m + 1];
                im += v[0] * tw[2 * m + 1] + v[1] * tw[2 * m];
            }
            tmp[2 * k] = re;
            tmp[2 * k + 1] = im;
        }
        for (int k = 0; k < n; ++k) {
            double* v = base + 2 * (size_t)(k * elem_stride);
            v[0] = tmp[2 * k];
            v[1] = tmp[2 * k + 1];
        }
    }
    free(tw);
    free(tmp);
}

static void run(const dft_plan* p, const double* in, double* out)
{
    const size_t n = (size_t)p->nx * (size_t)p->ny;
    double* work = (double*)malloc(sizeof(double) * 2 * n);
    memcpy(work, in, sizeof(double) * 2 * n);
    dft_lines(work, p->nx, p->ny, 1, p->nx, p->sign);   /* rows */
    dft_lines(work, p->ny, p->nx, p->nx, 1, p->sign);   /* columns */
    memcpy(out, work, sizeof(double) * 2 * n);
    free(work);
}

int fftw_init_threads(void) { return 1; }
void fftw_plan_with_nthreads(int n) { (void)n; }
void fftw_cleanup_threads(void) {}
void* fftw_malloc(size_t n) { return calloc(1, n ? n : 1); }
void fftw_free(void* p) { free(p); }

void* fftw_plan_dft_2d(int ny, int nx, void* in, void* out, int sign, unsigned flags)
{
    (void)flags;
    dft_plan* p = (dft_plan*)malloc(sizeof(dft_plan));
    p->nx = nx;
    p->ny = ny;
    p->sign = sign < 0 ? -1 : 1;
    p->in = (double*)in;
    p->out = (double*)out;
    return p;
}
void fftw_execute(void* plan)
{
    const dft_plan* p = (const dft_plan*)plan;
    run(p, p->in, p->out);
}
void fftw_execute_dft(void* plan, void* in, void* out)
{
    run((const dft_plan*)plan, (const double*)in, (double*)out);
}
void fftw_destroy_plan(void* p) { free(p); }
void* fftw_plan_dft_1d(void) { unreachable("fftw_plan_dft_1d"); return NULL; }
void* fftw_plan_dft_3d(void) { unreachable("fftw_plan_dft_3d"); return NULL; }

int cudaMalloc(void) { unreachable("cudaMalloc"); return 1; }
int cudaFree(void) { unreachable("cudaFree"); return 1; }
int cudaMemcpy(void) { unreachable("cudaMemcpy"); return 1; }
int cudaMemcpyAsync(void) { unreachable("cudaMemcpyAsync"); return 1; }
int cudaMemsetAsync(void) { unreachable("cudaMemsetAsync"); return 1; }
int cudaStreamCreate(void) { unreachable("cudaStreamCreate"); return 1; }
int cudaStreamDestroy(void) { unreachable("cudaStreamDestroy"); return 1; }
void cudaFFT(void) { unreachable("cudaFFT"); }
void cudaCropFringe(void) { unreachable("cudaCropFringe"); }
void cudaGetFringe(void) { unreachable("cudaGetFringe"); }
