/*
 * CPU restatement of Openholo's WRP (wavefront recording plane) splat.
 *
 * TEST INFRASTRUCTURE ONLY: a checker for tests/ and the accuracy legs of
 * bench.py; the product never links it.
 *
 * Restates, in the reference's operation order (built with
 * -ffp-contract=off):
 *   ophWRP::autoScaling       ophgen/src/ophWRP.cpp:71-129 (the active branch:
 *                             pos *= scale, zmax from MIN_DOUBLE up)
 *   ophWRP::calculateWRPCPU   ophgen/src/ophWRP.cpp:321-420, the per-channel
 *                             splat into p_wrp_ before Fresnel_FFT, with
 *                             RandomPhase off (randVal = 1.0)
 * Every point is splatted with the same depth difference dz = wrp_location -
 * zmax (ophWRP.cpp:345), over a (2w) x (2w) square anchored at
 * ((int)(x / ppX) + pnX/2, (int)(y / ppY) + pnY/2), w = (int)(|lambda dz /
 * (2 ppX^2)| * 2). Points are added one after the other in index order; the
 * reference adds them in OpenMP atomic order, which changes only the last
 * bits of each sum.
 */
#include "ophpc_oracle.h"

#include <float.h>
#include <math.h>
#include <string.h>

#ifndef M_PI
#define M_PI 3.14159265358979323846
#endif

/* MIN_DOUBLE of Openholo/src/define.h:148 */
#define ORA_MIN_DOUBLE ((double)2.2250738585072014e-308)

double oracle_wrp_zmax(const oracle_wrp_config* c, const double* vertices, int64_t n_points)
{
    double zmax = ORA_MIN_DOUBLE;
    for (int64_t i = 0; i < n_points; ++i) {
        const double z = vertices[i * 7 + 2] * c->scale[2];
        if (zmax < z) zmax = z;
    }
    return zmax;
}

int oracle_wrp_plane(const oracle_wrp_config* c, const double* vertices, int64_t n_points, int32_t channel,
                     double* plane_out)
{
    if (!c || !plane_out || (n_points > 0 && !vertices)) return -1;
    if (c->pixel_number[0] <= 0 || c->pixel_number[1] <= 0 || channel < 0 || channel >= c->n_channels ||
        c->n_channels > 3)
        return -1;
    const int pnX = c->pixel_number[0], pnY = c->pixel_number[1];
    const double ppX = c->pixel_pitch[0], ppY = c->pixel_pitch[1];
    const int hpnX = pnX >> 1, hpnY = pnY >> 1;
    memset(plane_out, 0, sizeof(double) * 2 * (size_t)pnX * (size_t)pnY);
    const double zmax = oracle_wrp_zmax(c, vertices, n_points);
    const double ppXX = ppX * ppX * 2;
    const double pi2 = 2 * M_PI;
    const double dz = c->wrp_location - zmax;
    const double dzz = dz * dz;
    const double lambda = c->wave_length[channel];
    const double k = pi2 / lambda;
    const double randpi2 = pi2 * 1.0;
    const double crand = cos(randpi2), srand_ = sin(randpi2);
    for (int64_t i = 0; i < n_points; ++i) {
        const double* v = vertices + i * 7;
        const double x = v[0] * c->scale[0];
        const double y = v[1] * c->scale[1];
        const double amplitude = v[3 + channel];
        const int sign = dz > 0.0;
        const double tw = fabs(lambda * dz / ppXX) * 2;
        const int w = (int)tw;
        const int tx = (int)(x / ppX) + hpnX;
        const int ty = (int)(y / ppY) + hpnY;
        for (int wy = -w; wy < w; ++wy) {
            const double dy = wy * ppY;
            const double dyy = dy * dy;
            const int tmpY = wy + ty;
            for (int wx = -w; wx < w; ++wx) {
                const int tmpX = wx + tx;
                if (tmpX >= 0 && tmpX < pnX && tmpY >= 0 && tmpY < pnY) {
                    const int64_t adr = (int64_t)tmpX + (int64_t)tmpY * pnX;
                    const double dx = wx * ppX;
                    const double r = sign ? sqrt(dx * dx + dyy + dzz) : -sqrt(dx * dx + dyy + dzz);
                    const double kr = k * r;
                    const double re = (amplitude * cos(kr) * crand) / r;
                    const double im = (-amplitude * sin(kr) * srand_) / r;
                    plane_out[2 * adr] += re;
                    plane_out[2 * adr + 1] += im;
                }
            }
        }
    }
    return 0;
}
