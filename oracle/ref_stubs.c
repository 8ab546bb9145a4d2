/*
 * Link-only stubs for the reference CPU build (oracle/_ref).
 *
 * TEST INFRASTRUCTURE ONLY. The reference's core classes link against FFTW
 * and a few cuFFT helper wrappers that the point-cloud generate / encode /
 * normalise path never calls (FFTW is used by Fresnel_FFT, ASM and the SSB
 * encoders; the cuFFT wrappers by the GPU SSB encoder). Neither library is
 * installed here, so these definitions satisfy the linker. The thread-setup
 * calls made by the Openholo constructor/destructor
 * (Openholo/src/Openholo.cpp:67-68,83) are harmless no-ops; every other
 * stub aborts loudly if it is ever reached, so a stubbed code path can never
 * silently feed a golden vector.
 *
 * Only C linkage names matter to the linker; the signatures below are
 * deliberately generic and this file includes no reference header.
 */
#include <stdio.h>
#include <stdlib.h>

static void ophref_unreachable(const char* name)
{
    fprintf(stderr, "oracle/_ref: stubbed symbol %s was called; the point-cloud path must not use it\n", name);
    abort();
}

int fftw_init_threads(void) { return 1; }
void fftw_plan_with_nthreads(int n) { (void)n; }
void fftw_cleanup_threads(void) {}

void* fftw_malloc(size_t n) { (void)n; ophref_unreachable("fftw_malloc"); return NULL; }
void fftw_free(void* p) { (void)p; ophref_unreachable("fftw_free"); }
void* fftw_plan_dft_1d(void) { ophref_unreachable("fftw_plan_dft_1d"); return NULL; }
void* fftw_plan_dft_2d(void) { ophref_unreachable("fftw_plan_dft_2d"); return NULL; }
void* fftw_plan_dft_3d(void) { ophref_unreachable("fftw_plan_dft_3d"); return NULL; }
void fftw_execute(void* p) { (void)p; ophref_unreachable("fftw_execute"); }
void fftw_execute_dft(void) { ophref_unreachable("fftw_execute_dft"); }
void fftw_destroy_plan(void* p) { (void)p; ophref_unreachable("fftw_destroy_plan"); }

/* CUDA runtime calls made only by ophGen's GPU SSB/off-axis encoders. */
int cudaMalloc(void) { ophref_unreachable("cudaMalloc"); return 1; }
int cudaFree(void) { ophref_unreachable("cudaFree"); return 1; }
int cudaMemcpy(void) { ophref_unreachable("cudaMemcpy"); return 1; }
int cudaMemcpyAsync(void) { ophref_unreachable("cudaMemcpyAsync"); return 1; }
int cudaMemsetAsync(void) { ophref_unreachable("cudaMemsetAsync"); return 1; }
int cudaStreamCreate(void) { ophref_unreachable("cudaStreamCreate"); return 1; }
int cudaStreamDestroy(void) { ophref_unreachable("cudaStreamDestroy"); return 1; }

void cudaFFT(void) { ophref_unreachable("cudaFFT"); }
void cudaCropFringe(void) { ophref_unreachable("cudaCropFringe"); }
void cudaGetFringe(void) { ophref_unreachable("cudaGetFringe"); }
