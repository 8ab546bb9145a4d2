// C entry points over the reference's own ophPointCloud CPU path (oracle/_ref).
//
// TEST INFRASTRUCTURE ONLY: this file is compiled together with the
// reference sources (read in place, never copied) by oracle/Makefile, and the
// resulting library is used by tests/golden/make_golden.py to generate golden
// vectors and to pin the C restatement in oracle/ophpc_oracle.c. It is also
// the timed "reference" CPU arm where it exists. Nothing in the product links
// or loads it.
//
// Call sequence mirrors Example/examPointCloud/examPointCloud.cpp:54-132:
// readConfig -> loadPointCloud | setNumberOfPoints+setPointCloudModel ->
// SetMode(MODE_CPU) -> generateHologram -> encoding -> normalize.
#include "ophPointCloud.h"

#include <chrono>
#include <cstring>

// The GPU driver (ophgen/src/ophPointCloud_GPU.cpp) is not part of the CPU
// oracle: it needs cudaWrapper, which divides by zero on sm_10x
// (ophgen/src/cudaWrapper.cpp:125-152,174). MODE_CPU never reaches it.
void ophPointCloud::genCghPointCloudGPU(uint) {}

namespace {
struct Holder {
    ophPointCloud* pc = nullptr;
    ~Holder() { if (pc) pc->release(); }
};
}  // namespace

extern "C" {

// Reads only the config and reports its shape. Returns 0 on success.
int ophref_query(const char* xml_path, int* pnx, int* pny, int* n_channels)
{
    Holder h;
    h.pc = new ophPointCloud();
    if (!h.pc->readConfig(xml_path)) return -1;
    OphConfig& ctx = h.pc->getContext();
    *pnx = ctx.pixel_number[_X];
    *pny = ctx.pixel_number[_Y];
    *n_channels = (int)ctx.waveNum;
    return 0;
}

// Loads a PLY through PLYparser (Openholo/src/PLYparser.cpp:142-449) and
// copies up to `cap` 56-byte Vertex records out. Returns the point count,
// or -1 on failure.
long long ophref_load_ply(const char* ply_path, void* vertices_out, unsigned long long cap)
{
    Holder h;
    h.pc = new ophPointCloud();
    int n = h.pc->loadPointCloud(ply_path);
    if (n < 0) return -1;
    unsigned long long nn = h.pc->getNumberOfPoints();
    if (vertices_out && nn) {
        unsigned long long c = nn < cap ? nn : cap;
        std::memcpy(vertices_out, h.pc->getPointCloudModel(), c * sizeof(Vertex));
    }
    return (long long)nn;
}

// Full reference run. `vertices` (n_points packed 56-byte Vertex records) is
// used when ply_path is NULL. encode_flag: 0 = ENCODE_PHASE, 1 =
// ENCODE_AMPLITUDE, 2 = both (phase first), anything else = none.
// field_out: [n_channels][pnY*pnX][re,im] doubles; encoded_out:
// [n_channels][pnY*pnX] doubles; normalized_out: [n_channels][pnY*pnX] bytes.
// Any output pointer may be NULL. Returns 0 on success.
int ophref_run(const char* xml_path, const char* ply_path, const void* vertices,
               unsigned long long n_points, int viewing_window, unsigned diff_flag,
               unsigned encode_flag, double* field_out, double* encoded_out,
               unsigned char* normalized_out, double* seconds_out)
{
    Holder h;
    h.pc = new ophPointCloud();
    if (!h.pc->readConfig(xml_path)) return -1;
    if (ply_path) {
        if (h.pc->loadPointCloud(ply_path) < 0) return -2;
    } else {
        h.pc->setNumberOfPoints(n_points);
        h.pc->setPointCloudModel((Vertex*)vertices);
    }
    h.pc->setViewingWindow(viewing_window != 0);
    h.pc->SetMode(MODE_CPU);
    Real secs = h.pc->generateHologram(diff_flag);
    if (seconds_out) *seconds_out = secs;

    OphConfig& ctx = h.pc->getContext();
    const long long pnXY = (long long)ctx.pixel_number[_X] * ctx.pixel_number[_Y];
    const unsigned nch = ctx.waveNum;
    Complex<Real>** H = h.pc->getComplexField();
    if (field_out) {
        for (unsigned c = 0; c < nch; ++c)
            for (long long i = 0; i < pnXY; ++i) {
                field_out[(c * pnXY + i) * 2 + 0] = H[c][i].real();
                field_out[(c * pnXY + i) * 2 + 1] = H[c][i].imag();
            }
    }
    // encode_flag 0 / 1: that encoding; 2: phase then amplitude of the same
    // field, stored one after the other in encoded_out / normalized_out.
    const unsigned flags[2] = {encode_flag == 1 ? 1u : 0u, 1u};
    const int n_enc = encode_flag == 2 ? 2 : (encode_flag <= 1 ? 1 : 0);
    for (int k = 0; k < n_enc; ++k) {
        h.pc->encoding(flags[k] == 0 ? ophGen::ENCODE_PHASE : ophGen::ENCODE_AMPLITUDE);
        h.pc->normalize();
        Real** E = h.pc->getEncodedBuffer();
        uchar** U = h.pc->getNormalizedBuffer();
        for (unsigned c = 0; c < nch; ++c) {
            if (encoded_out) std::memcpy(encoded_out + (k * nch + c) * pnXY, E[c], sizeof(Real) * pnXY);
            if (normalized_out) std::memcpy(normalized_out + (k * nch + c) * pnXY, U[c], (size_t)pnXY);
        }
    }
    return 0;
}

// Runs the reference path (as ophref_run, phase encoding) and saves the
// hologram through ophGen::save (ophgen/src/ophGen.cpp:689-769) with
// `bits_per_pixel`. Returns 0 on success.
int ophref_run_save(const char* xml_path, const void* vertices, unsigned long long n_points,
                    unsigned diff_flag, unsigned encode_flag, const char* bmp_path, int bits_per_pixel)
{
    Holder h;
    h.pc = new ophPointCloud();
    if (!h.pc->readConfig(xml_path)) return -1;
    h.pc->setNumberOfPoints(n_points);
    h.pc->setPointCloudModel((Vertex*)vertices);
    h.pc->SetMode(MODE_CPU);
    h.pc->generateHologram(diff_flag);
    h.pc->encoding(encode_flag == 1 ? ophGen::ENCODE_AMPLITUDE : ophGen::ENCODE_PHASE);
    h.pc->normalize();
    return h.pc->save(bmp_path, (uint8_t)bits_per_pixel) ? 0 : -3;
}

// Runs the reference generate and writes the complex field with
// Openholo::saveAsOhc (Openholo/src/Openholo.cpp:252-279). Returns 0 on success.
int ophref_run_save_ohc(const char* xml_path, const void* vertices, unsigned long long n_points,
                        unsigned diff_flag, const char* ohc_path)
{
    Holder h;
    h.pc = new ophPointCloud();
    if (!h.pc->readConfig(xml_path)) return -1;
    h.pc->setNumberOfPoints(n_points);
    h.pc->setPointCloudModel((Vertex*)vertices);
    h.pc->SetMode(MODE_CPU);
    h.pc->generateHologram(diff_flag);
    return h.pc->saveAsOhc(ohc_path) ? 0 : -3;
}

// Encodes a given field with the reference's ophGen::encoding +
// ophGen::normalize (ophgen/src/ophGen.cpp:816-849,654-687). The config
// (xml_path) sets the shape; field_in: [n_channels][pnY*pnX][re,im]. When
// pre_flag >= 0 that encoding (and normalize) runs first on the same object,
// so the encoders that write only some entries (Burckhardt, TwoPhase) leave
// its values in the others. Outputs as in ophref_run. Returns 0 on success.
int ophref_encode_field(const char* xml_path, const double* field_in, int pre_flag, unsigned flag,
                        double* encoded_out, unsigned char* normalized_out)
{
    Holder h;
    h.pc = new ophPointCloud();
    if (!h.pc->readConfig(xml_path)) return -1;
    OphConfig& ctx = h.pc->getContext();
    const long long pnXY = (long long)ctx.pixel_number[_X] * ctx.pixel_number[_Y];
    const unsigned nch = ctx.waveNum;
    Complex<Real>** H = h.pc->getComplexField();
    for (unsigned c = 0; c < nch; ++c)
        for (long long i = 0; i < pnXY; ++i)
            H[c][i] = Complex<Real>(field_in[(c * pnXY + i) * 2], field_in[(c * pnXY + i) * 2 + 1]);
    if (pre_flag >= 0) {
        h.pc->encoding((unsigned)pre_flag);
        h.pc->normalize();
    }
    h.pc->encoding(flag);
    h.pc->normalize();
    Real** E = h.pc->getEncodedBuffer();
    uchar** U = h.pc->getNormalizedBuffer();
    for (unsigned c = 0; c < nch; ++c) {
        if (encoded_out) std::memcpy(encoded_out + c * pnXY, E[c], sizeof(Real) * pnXY);
        if (normalized_out) std::memcpy(normalized_out + c * pnXY, U[c], (size_t)pnXY);
    }
    return 0;
}

// Loads a .ohc with Openholo::loadAsOhc (Openholo/src/Openholo.cpp:280-319)
// and copies out the shape (shape[0..2] = pnX, pnY, channels), pitch[2],
// wavelengths[3] and, when field is non-NULL and cap_doubles suffices,
// complex_H as [channel][re, im per pixel]. Returns 0 on success.
int ophref_load_ohc(const char* ohc_path, int* shape, double* pitch, double* wavelengths, double* field,
                    unsigned long long cap_doubles)
{
    Holder h;
    h.pc = new ophPointCloud();
    if (!h.pc->loadAsOhc(ohc_path)) return -1;
    OphConfig& c = h.pc->getContext();
    shape[0] = c.pixel_number[_X];
    shape[1] = c.pixel_number[_Y];
    shape[2] = (int)c.waveNum;
    pitch[0] = c.pixel_pitch[_X];
    pitch[1] = c.pixel_pitch[_Y];
    for (unsigned i = 0; i < c.waveNum && i < 3; ++i) wavelengths[i] = c.wave_length[i];
    const unsigned long long pnXY = (unsigned long long)shape[0] * shape[1];
    if (field && cap_doubles >= 2 * pnXY * c.waveNum) {
        Complex<Real>** H = h.pc->getComplexField();
        for (unsigned ch = 0; ch < c.waveNum; ++ch)
            std::memcpy(field + 2 * pnXY * ch, H[ch], sizeof(double) * 2 * pnXY);
    }
    return 0;
}

}  // extern "C"
