// C entry point over the reference's own ophGen::encodeSideBand
// (oracle/_ref/libophref_sideband.so).
//
// TEST INFRASTRUCTURE ONLY: compiled together with the reference sources
// (read in place, never copied) by oracle/Makefile, with FFTW replaced by
// the FP64 DFT of oracle/ref_dft_stubs.c; tests/golden/make_golden.py uses it
// to write the side-band fixtures that pin oracle.sideband_encode. Nothing in
// the product links or loads it.
//
// ophGen::encodeSideBand (ophgen/src/ophGen.cpp:1607-1653) is protected; a
// probe subclass of ophPointCloud calls it. Its CPU body
// (encodeSideBand_CPU, :1655-1695) runs when MODE_GPU is set (the
// reference's test of the mode bit is inverted), and its transform goes
// through a plan whose input is FFTW's own buffer, so it is well defined.
#include "ophPointCloud.h"

#include <cstring>

// The GPU generate (ophgen/src/ophPointCloud_GPU.cpp) is not part of this CPU build.
void ophPointCloud::genCghPointCloudGPU(uint) {}

namespace {
struct SidebandProbe : public ophPointCloud {
    void run(unsigned passband) { encodeSideBand(passband); }
};
}  // namespace

extern "C" {

// field_in [n_channels][pnY][pnX][re, im] into complex_H, then
// encodeSideBand(passband); m_lpEncoded into enc_out [n_channels][pnY][pnX].
// Returns the channel count, or a negative value on failure.
int ophref_sideband(const char* xml_path, const double* field_in, unsigned passband, double* enc_out,
                    int max_channels)
{
    SidebandProbe* p = new SidebandProbe();
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
    Complex<Real>** H = p->getComplexField();
    for (int c = 0; c < nch; ++c)
        std::memcpy(H[c], field_in + (size_t)c * 2 * pnX * pnY, sizeof(double) * 2 * (size_t)(pnX * pnY));
    p->SetMode(MODE_GPU);   // selects encodeSideBand_CPU (ophGen.cpp:1647-1652)
    p->run(passband);
    Real** enc = p->getEncodedBuffer();
    for (int c = 0; c < nch; ++c)
        std::memcpy(enc_out + (size_t)c * pnX * pnY, enc[c], sizeof(double) * (size_t)(pnX * pnY));
    p->release();
    return nch;
}

}  // extern "C"
