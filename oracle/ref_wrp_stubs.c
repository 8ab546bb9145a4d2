/*
 * FFTW stand-ins for the reference WRP build (oracle/_ref/libophref_wrp.so).
 *
 * TEST INFRASTRUCTURE ONLY. The reference's Fresnel_FFT plans a forward 2-D
 * FFT on the zero-padded WRP plane; this stand-in copies that input out
 * (oracle/ref_wrp_driver.cpp reads it) and otherwise computes nothing:
 * execute is a no-op, memory comes zeroed and is never freed (the reference
 * hands buffers it allocated with new[] to fftw_free). No FFT result of this
 * build is used. The CUDA symbols that only the GPU encoders reach abort.
 */
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

static double* g_buf;
static long long g_nx, g_ny;
static int g_max, g_count;

void ophref_wrp_capture_begin(double* buf, long long nx, long long ny, int max_captures)
{
    g_buf = buf;
    g_nx = nx;
    g_ny = ny;
    g_max = max_captures;
    g_count = 0;
}

int ophref_wrp_capture_count(void) { return g_count; }

static void unreachable(const char* name)
{
    fprintf(stderr, "oracle/_ref (WRP build): stubbed symbol %s was called\n", name);
    abort();
}

int fftw_init_threads(void) { return 1; }
void fftw_plan_with_nthreads(int n) { (void)n; }
void fftw_cleanup_threads(void) {}
void* fftw_malloc(size_t n) { return calloc(1, n ? n : 1); }
void fftw_free(void* p) { (void)p; }

/* FFTW_FORWARD is -1 */
void* fftw_plan_dft_2d(int ny, int nx, void* in, void* out, int sign, unsigned flags)
{
    (void)out;
    (void)flags;
    if (sign == -1 && g_buf && g_count < g_max && (long long)nx == g_nx && (long long)ny == g_ny) {
        memcpy(g_buf + (size_t)g_count * 2 * (size_t)nx * (size_t)ny, in, sizeof(double) * 2 * (size_t)nx * (size_t)ny);
        ++g_count;
    }
    return (void*)1;
}
void* fftw_plan_dft_1d(void) { unreachable("fftw_plan_dft_1d"); return NULL; }
void* fftw_plan_dft_3d(void) { unreachable("fftw_plan_dft_3d"); return NULL; }
void fftw_execute(void* p) { (void)p; }
void fftw_execute_dft(void* p, void* in, void* out) { (void)p; (void)in; (void)out; }
void fftw_destroy_plan(void* p) { (void)p; }

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
