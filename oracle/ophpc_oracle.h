/*
 * ophpc_oracle — CPU restatement of Openholo's point-cloud hologram path.
 *
 * TEST INFRASTRUCTURE ONLY. This is the checker: tests/, the smoke check and
 * the CPU arm of bench.py may call it; the product (libophpc) never does.
 *
 * Everything is plain IEEE double arithmetic in the reference's own operation
 * order (built with -ffp-contract=off), restating:
 *   genCghPointCloudCPU      ophgen/src/ophPointCloud.cpp:253-329
 *   ophGen::RS_Diffraction   ophgen/src/ophGen.cpp:361-445
 *   ophGen::Fresnel_Diffraction ophgen/src/ophGen.cpp:447-514
 *   ophGen::transVW          ophgen/src/ophGen.cpp:1976-1985
 *   ophGen::Phase/Amplitude/RealPart/ImaginaryPart ophgen/src/ophGen.cpp:1821-1864
 *   ophGen::TwoPhase/Burckhardt/SimpleNI ophgen/src/ophGen.cpp:1866-1974
 *   ophGen::normalize        ophgen/src/ophGen.cpp:654-687 (+ function.h:79-99)
 * Parity of this restatement is pinned against the reference itself
 * (oracle/_ref, built from the reference sources) by tests/test_oracle.py
 * through the committed fixtures in tests/golden/.
 */
#ifndef OPHPC_ORACLE_H
#define OPHPC_ORACLE_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* OphConfig (Openholo/src/Openholo.h:96-120) + OphPointCloudConfig fields
 * the path reads. */
typedef struct oracle_config {
    int32_t pixel_number[2];
    int32_t offset[2];
    double pixel_pitch[2];
    double scale[3];
    double distance;
    double field_length;
    int32_t viewing_window;
    int32_t n_channels;
    double wave_length[3];
} oracle_config;

/* Vertex (Openholo/src/struct.h:86-106): 7 packed doubles per point:
 * pos[3], color[3], phase. */

/* Full field, point-major scatter with OpenMP atomics exactly like the
 * reference CPU path. field_out: [n_channels][pnY][pnX][re, im]; it is
 * zeroed first (resetBuffer). Returns 0, or -1 on bad arguments. */
int oracle_generate(const oracle_config* cfg, const double* vertices, int64_t n_points,
                    int32_t diff_flag, double* field_out);

/* Field of one channel at selected pixels (flat index y*pnX + x), pixel-major
 * gather over points in index order with the same per-(point, pixel) window
 * decision and term as oracle_generate. out: [n_pix][re, im]. */
int oracle_field_at(const oracle_config* cfg, const double* vertices, int64_t n_points,
                    int32_t diff_flag, int32_t channel, const int64_t* pixel_index,
                    int64_t n_pix, double* out);

/* One channel of n pixels, as ophGen::encoding calls its encoder per
 * channel: ENCODE_PHASE 0, AMPLITUDE 1, REAL 2, IMAGINARY 3, SIMPLENI 4,
 * BURCKHARDT 5, TWOPHASE 6. field: [n][re, im]. Burckhardt and TwoPhase
 * leave the entries they do not write as they were (encoded is in/out). */
int oracle_encode(const double* field, int64_t n, int32_t encode_flag, double* encoded);

/* Global min/max over all channels, then (uchar)(((v-min)/gap)*255 + 0.5). */
void oracle_normalize(const double* encoded, int32_t n_channels, int64_t n_per_channel,
                      uint8_t* out, double* min_out, double* max_out);

/* WRP generator (ophgen/src/ophWRP.cpp, ophWRPConfig ophgen/src/ophGen.h:643-660):
 * the geometry and the two WRP depths the splat reads. */
typedef struct oracle_wrp_config {
    int32_t pixel_number[2];
    double pixel_pitch[2];
    double scale[3];
    double wrp_location;          /* LocationOfWRP */
    double propagation_distance;  /* Distance */
    int32_t n_channels;
    double wave_length[3];
} oracle_wrp_config;

/* autoScaling's zmax: the largest scaled z, starting from MIN_DOUBLE. */
double oracle_wrp_zmax(const oracle_wrp_config* cfg, const double* vertices, int64_t n_points);

/* One channel's WRP plane (calculateWRPCPU's splat, RandomPhase off):
 * plane_out [pnY][pnX][re, im], zeroed first. Returns 0, or -1 on bad
 * arguments. (oracle/ophpc_oracle_wrp.c) */
int oracle_wrp_plane(const oracle_wrp_config* cfg, const double* vertices, int64_t n_points, int32_t channel,
                     double* plane_out);

#ifdef __cplusplus
}
#endif

#endif
