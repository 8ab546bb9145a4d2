/*
 * ophpc WRP — wavefront-recording-plane hologram generation on GB300 (C ABI).
 *
 * Drop-in for Openholo's WRP generator (ophgen/src/ophWRP.h, ophWRP.cpp):
 *   ophWRP::generateHologram   ophgen/src/ophWRP.cpp:435-461
 *     autoScaling              ophgen/src/ophWRP.cpp:71-129
 *     calculateWRPCPU          ophgen/src/ophWRP.cpp:321-433
 *     ophGen::Fresnel_FFT      ophgen/src/ophGen.cpp:516-580
 * Every point of the cloud is splatted onto a plane near the object (the
 * WRP) over a small square whose size follows from the depth difference,
 * and the plane is propagated to the SLM by the angular-spectrum method
 * (2x zero padding, FFT, transfer function, inverse FFT, centre crop).
 *
 * Same conventions as ophpc.h: status codes, explicit streams, device
 * buffers aligned as cudaMalloc returns them; the same context serves both
 * generators. The device entry points read the vertices' depth range back
 * to the host once (one synchronisation of `stream`) to size the splat.
 */
#ifndef OPHPC_WRP_H
#define OPHPC_WRP_H

#include "ophpc.h"

#ifdef __cplusplus
extern "C" {
#endif

/* OphWRPConfig (ophgen/src/ophGen.h:643-660) and the OphConfig fields the
 * WRP generator reads. */
typedef struct ophpc_wrp_config {
    int32_t pixel_number[2];                /* SLM_PixelNumX/Y */
    double pixel_pitch[2];                  /* SLM_PixelPitchX/Y, metres; also the WRP pitch */
    double scale[3];                        /* ScaleX/Y/Z */
    double wrp_location;                    /* LocationOfWRP, metres */
    double propagation_distance;            /* Distance: WRP -> SLM, metres */
    uint32_t n_channels;                    /* SLM_WaveNum, 1..OPHPC_MAX_CHANNELS */
    double wave_length[OPHPC_MAX_CHANNELS]; /* SLM_WaveLength_i, metres */
    int32_t random_phase;                   /* RandomPhase: must be 0 (see below) */
} ophpc_wrp_config;

/* Device path of ophWRP::generateHologram: d_vertices holds n_points
 * ophpc_vertex records; d_field receives [n_channels][pnY][pnX][re, im]
 * doubles (complex_H), overwritten. Channel c takes its amplitude from
 * color[c]. The splat and the propagation are computed in FP64 and
 * unnormalised, as the reference's backward FFT leaves them (the field is
 * 4 pnX pnY times the physical propagation). Pixel numbers up to 16384;
 * 2 pnX and 2 pnY must factor into 2, 3, 5 and 7 (OPHPC_ERROR_UNSUPPORTED
 * otherwise); random_phase
 * != 0 is OPHPC_ERROR_UNSUPPORTED (the reference draws an unseeded random
 * number per point and pixel). */
ophpc_status ophpc_wrp_generate(ophpc_context* ctx, const ophpc_wrp_config* cfg, const ophpc_vertex* d_vertices,
                                uint64_t n_points, double* d_field, void* stream);

/* Host path: host vertices in, one host buffer of pnX*pnY Complex<double>
 * per channel out. Synchronous; seconds_out (optional) receives the elapsed
 * wall time. */
ophpc_status ophpc_wrp_generate_host(ophpc_context* ctx, const ophpc_wrp_config* cfg,
                                     const ophpc_vertex* h_vertices, uint64_t n_points,
                                     double* const* h_field_per_channel, double* seconds_out);

/* The WRP plane of one channel before propagation (p_wrp_ of
 * calculateWRPCPU, ophgen/src/ophWRP.cpp:355-416; ophWRP::getWRPBuff):
 * d_plane receives [pnY][pnX][re, im] doubles. Any pixel numbers (no
 * transform is involved). */
ophpc_status ophpc_wrp_plane(ophpc_context* ctx, const ophpc_wrp_config* cfg, const ophpc_vertex* d_vertices,
                             uint64_t n_points, uint32_t channel, double* d_plane, void* stream);

/* ophGen::Fresnel_FFT (ophgen/src/ophGen.cpp:516-580) on a given complex
 * plane: d_src [pnY][pnX][re, im] propagated by `distance` at wavelength
 * `lambda` into d_dst (same layout; d_dst may equal d_src). Unnormalised. */
ophpc_status ophpc_fresnel_fft(ophpc_context* ctx, int32_t pnx, int32_t pny, double ppx, double ppy,
                               double lambda, double distance, const double* d_src, double* d_dst, void* stream);

#ifdef __cplusplus
}
#endif

#endif /* OPHPC_WRP_H */
