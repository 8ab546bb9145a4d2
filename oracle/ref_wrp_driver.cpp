// C entry point over the reference's own WRP splat (oracle/_ref/libophref_wrp.so).
//
// TEST INFRASTRUCTURE ONLY: compiled together with the reference sources
// (read in place, never copied) by oracle/Makefile; tests/golden/make_golden.py
// uses it to write the WRP-plane fixtures that pin oracle/ophpc_oracle_wrp.c.
// Nothing in the product links or loads it.
//
// ophWRP::calculateWRPCPU (ophgen/src/ophWRP.cpp:321-433) splats every point
// into p_wrp_ and hands the plane to Fresnel_FFT (ophgen/src/ophGen.cpp:516-580),
// which copies it into the centre of a zero-padded (2 pnX) x (2 pnY) buffer
// and plans its first forward FFT on that buffer. In this build FFTW is
// replaced by oracle/ref_wrp_stubs.c, whose forward plan copies that buffer
// out (one capture per channel); everything the reference computes after it
// is discarded. Call sequence as Example/examWRP/examWRP.cpp: readConfig,
// point cloud, generateHologram (MODE_CPU).
#include "ophWRP.h"

#include <cstring>
#include <vector>

// The GPU splat (ophgen/src/ophWRP_GPU.cpp) is not part of this CPU build.
void ophWRP::calculateWRPGPU(void) {}

extern "C" void ophref_wrp_capture_begin(double* buf, long long nx, long long ny, int max_captures);
extern "C" int ophref_wrp_capture_count(void);

namespace {
// The point cloud goes into the protected members loadPointCloud fills.
struct WrpProbe : public ophWRP {
    void set_points(const Vertex* v, unsigned long long n) {
        obj_.vertices = new Vertex[n ? n : 1];
        if (n) std::memcpy(obj_.vertices, v, sizeof(Vertex) * n);
        obj_.n_points = n;
        obj_.n_colors = 3;
        n_points = (int)n;
    }
};
}  // namespace

extern "C" {

// One WRP plane per channel into planes_out [n_channels][pnY][pnX][re, im].
// Returns the channel count, or a negative value on failure.
int ophref_wrp_planes(const char* xml_path, const void* vertices, unsigned long long n_points, double* planes_out,
                      int max_channels)
{
    WrpProbe* p = new WrpProbe();
    if (!p->readConfig(xml_path)) {
        p->release();
        return -1;
    }
    OphConfig& ctx = p->getContext();
    const long long pnX = ctx.pixel_number[_X], pnY = ctx.pixel_number[_Y];
    const int nch = (int)ctx.waveNum;
    if (nch < 1 || nch > max_channels) {
        p->release();
        return -2;
    }
    p->set_points(static_cast<const Vertex*>(vertices), n_points);
    p->SetMode(MODE_CPU);
    std::vector<double> cap((size_t)nch * 2 * (size_t)(2 * pnX) * (size_t)(2 * pnY));
    ophref_wrp_capture_begin(cap.data(), 2 * pnX, 2 * pnY, nch);
    p->generateHologram();
    const int got = ophref_wrp_capture_count();
    ophref_wrp_capture_begin(nullptr, 0, 0, 0);
    p->release();
    if (got != nch) return -3;
    // the plane sits at (pnY / 2, pnX / 2) of the padded buffer (Fresnel_FFT's half_pnY, half_pnX)
    const long long hx = pnX >> 1, hy = pnY >> 1, W = 2 * pnX;
    for (int c = 0; c < nch; ++c) {
        const double* src = cap.data() + (size_t)c * 2 * (size_t)W * (size_t)(2 * pnY);
        double* dst = planes_out + (size_t)c * 2 * (size_t)pnX * (size_t)pnY;
        for (long long y = 0; y < pnY; ++y)
            std::memcpy(dst + 2 * y * pnX, src + 2 * ((y + hy) * W + hx), sizeof(double) * 2 * (size_t)pnX);
    }
    return nch;
}

}  // extern "C"
