/*
 * ophpc_oracle — CPU restatement of Openholo's point-cloud hologram path.
 * TEST INFRASTRUCTURE ONLY (see ophpc_oracle.h): never linked by the product.
 *
 * Each helper names the reference lines it restates. Operation order follows
 * the reference so that, compiled with -ffp-contract=off, every double
 * rounding is the one the reference performs.
 */
#define _GNU_SOURCE
#include "ophpc_oracle.h"

#include <float.h>
#include <math.h>
#include <stdlib.h>
#include <string.h>

#ifndef M_PI
#define M_PI 3.14159265358979323846
#endif

/* MIN_DOUBLE / MAX_DOUBLE: Openholo/src/define.h:140-150. */
#define ORA_MAX_DOUBLE ((double)1.7976931348623158e+308)
#define ORA_MIN_DOUBLE ((double)2.2250738585072014e-308)

typedef struct {
    /* per-point state after transVW, scaling and the distance offset */
    double px, py, z, amp;
    /* window rectangle: pixels [x_lo, x_hi) x [y_lo, y_hi) */
    int64_t x_lo, x_hi, y_lo, y_hi;
} ora_point;

typedef struct {
    int pnX, pnY, offX, offY;
    double ppX, ppY, ssX, ssY, x0, y0, lambda, k;
    /* RS only: tx / sqrt(1 - tx^2) evaluated as the reference does */
    double tx, ty, sqrtX, sqrtY;
} ora_geom;

static void ora_geom_init(const oracle_config* c, double lambda, ora_geom* g)
{
    g->pnX = c->pixel_number[0];
    g->pnY = c->pixel_number[1];
    g->offX = c->offset[0];
    g->offY = c->offset[1];
    g->ppX = c->pixel_pitch[0];
    g->ppY = c->pixel_pitch[1];
    g->ssX = g->pnX * g->ppX;              /* ophGen.cpp:368-369 */
    g->ssY = g->pnY * g->ppY;
    g->x0 = -g->ssX / 2;                   /* ophGen.cpp:378-379 */
    g->y0 = -g->ssY / 2;
    g->lambda = lambda;
    g->k = (2 * M_PI) / lambda;            /* ophGen.cpp:380 */
    g->tx = lambda / (2 * g->ppX);         /* ophGen.cpp:374-377 */
    g->ty = lambda / (2 * g->ppY);
    g->sqrtX = sqrt(1 - (g->tx * g->tx));
    g->sqrtY = sqrt(1 - (g->ty * g->ty));
}

/* Window rectangle, ophGen.cpp:385-409 (RS) and 470-492 (Fresnel): the
 * half-widths differ, the floor/+1 rules and the clipping are shared. */
static void ora_bounds(const ora_geom* g, double px, double py, double hwx, double hwy,
                       ora_point* p)
{
    double xb0 = px + hwx, xb1 = px - hwx;
    double yb0 = py + hwy, yb1 = py - hwy;
    double Xb0 = floor((xb0 - g->x0) / g->ppX) + 1;
    double Xb1 = floor((xb1 - g->x0) / g->ppX) + 1;
    double Yb0 = g->pnY - floor((yb1 - g->y0) / g->ppY);
    double Yb1 = g->pnY - floor((yb0 - g->y0) / g->ppY);
    if (Xb0 > g->pnX) Xb0 = g->pnX;
    if (Xb1 < 0) Xb1 = 0;
    if (Yb0 > g->pnY) Yb0 = g->pnY;
    if (Yb1 < 0) Yb1 = 0;
    /* the loops run `for (int i = lo; i < hi; ++i)`; lo is integral here */
    p->x_lo = (int64_t)Xb1;
    p->x_hi = (int64_t)ceil(Xb0);
    p->y_lo = (int64_t)Yb1;
    p->y_hi = (int64_t)ceil(Yb0);
}

/* Per point setup: transVW (ophGen.cpp:1976-1985) when enabled, then
 * `pc.pos *= scale` (ophPointCloud.cpp:304-306), z += distance and the window
 * rectangle. */
static void ora_point_init(const oracle_config* c, const ora_geom* g, const double* v,
                           int channel, int32_t diff_flag, ora_point* p)
{
    double x = v[0], y = v[1], zs = v[2];
    if (c->viewing_window) {
        double f = c->field_length;
        x = -f * x / (x - f);
        y = -f * y / (y - f);
        zs = -f * zs / (zs - f);
    }
    x *= c->scale[0];
    y *= c->scale[1];
    zs *= c->scale[2];
    p->px = x;
    p->py = y;
    p->z = zs + c->distance;               /* ophGen.cpp:381 / 464 */
    p->amp = v[3 + channel];               /* ophPointCloud.cpp:302 */
    if (diff_flag == 0) {
        double hwx = fabs(g->tx / g->sqrtX * p->z);
        double hwy = fabs(g->ty / g->sqrtY * p->z);
        ora_bounds(g, x, y, hwx, hwy, p);
    } else {
        double operand = g->lambda * p->z;
        double hwx = fabs(operand / (2 * g->ppX));
        double hwy = fabs(operand / (2 * g->ppY));
        ora_bounds(g, x, y, hwx, hwy, p);
    }
}

/* RS window test + term for one (point, pixel): ophGen.cpp:411-432.
 * Returns 1 and the term when the pixel lies inside the window. */
static int ora_rs_term(const ora_geom* g, const ora_point* p, int64_t xxtr, int64_t yytr,
                       double* re, double* im)
{
    double zz = p->z * p->z;
    double ampZ = p->amp * p->z;
    double yyy = g->y0 + ((g->pnY - (int)yytr + g->offY) * g->ppY);
    double rx0 = p->px + fabs(g->tx / g->sqrtX * sqrt((yyy - p->py) * (yyy - p->py) + zz));
    double rx1 = p->px - fabs(g->tx / g->sqrtX * sqrt((yyy - p->py) * (yyy - p->py) + zz));
    double xxx = g->x0 + (((int)xxtr - 1 + g->offX) * g->ppX);
    double r = sqrt((xxx - p->px) * (xxx - p->px) + (yyy - p->py) * (yyy - p->py) + zz);
    double ry0 = p->py + fabs(g->ty / g->sqrtY * sqrt((xxx - p->px) * (xxx - p->px) + zz));
    double ry1 = p->py - fabs(g->ty / g->sqrtY * sqrt((xxx - p->px) * (xxx - p->px) + zz));
    if (((xxx < rx0) && (xxx > rx1)) && ((yyy < ry0) && (yyy > ry1))) {
        double kr = g->k * r;
        double operand = g->lambda * r * r;
        *re = (ampZ * sin(kr)) / operand;
        *im = (-ampZ * cos(kr)) / operand;
        return 1;
    }
    return 0;
}

/* Fresnel term for one (point, pixel): ophGen.cpp:493-506. */
static void ora_fresnel_term(const ora_geom* g, const ora_point* p, int64_t xxtr, int64_t yytr,
                             double* re, double* im)
{
    double zz = p->z * p->z;
    double operand = g->lambda * p->z;
    double yyy = (g->y0 + (g->pnY - (int)yytr + g->offY) * g->ppY) - p->py;
    double xxx = (g->x0 + ((int)xxtr - 1 + g->offX) * g->ppX) - p->px;
    double ph = g->k * (xxx * xxx + yyy * yyy + 2 * zz) / (2 * p->z);
    *re = p->amp * sin(ph) / operand;
    *im = p->amp * (-cos(ph)) / operand;
}

static int ora_check(const oracle_config* c, int32_t diff_flag)
{
    if (!c) return -1;
    if (c->pixel_number[0] <= 0 || c->pixel_number[1] <= 0) return -1;
    if (c->n_channels < 1 || c->n_channels > 3) return -1;
    if (diff_flag != 0 && diff_flag != 1) return -1;
    return 0;
}

int oracle_generate(const oracle_config* c, const double* vertices, int64_t n_points,
                    int32_t diff_flag, double* field_out)
{
    if (ora_check(c, diff_flag) || (n_points > 0 && !vertices) || !field_out) return -1;
    const int64_t pnXY = (int64_t)c->pixel_number[0] * c->pixel_number[1];
    memset(field_out, 0, sizeof(double) * 2 * pnXY * c->n_channels);
    for (int ch = 0; ch < c->n_channels; ++ch) {
        ora_geom g;
        ora_geom_init(c, c->wave_length[ch], &g);
        double* dst = field_out + (int64_t)ch * pnXY * 2;
#pragma omp parallel for schedule(dynamic, 16)
        for (int64_t i = 0; i < n_points; ++i) {
            ora_point p;
            ora_point_init(c, &g, vertices + i * 7, ch, diff_flag, &p);
            for (int64_t yytr = p.y_lo; yytr < p.y_hi; ++yytr) {
                int64_t row = yytr * g.pnX;
                for (int64_t xxtr = p.x_lo; xxtr < p.x_hi; ++xxtr) {
                    double re, im;
                    if (diff_flag == 0) {
                        if (!ora_rs_term(&g, &p, xxtr, yytr, &re, &im)) continue;
                    } else {
                        ora_fresnel_term(&g, &p, xxtr, yytr, &re, &im);
                    }
#pragma omp atomic
                    dst[(row + xxtr) * 2 + 0] += re;
#pragma omp atomic
                    dst[(row + xxtr) * 2 + 1] += im;
                }
            }
        }
    }
    return 0;
}

int oracle_field_at(const oracle_config* c, const double* vertices, int64_t n_points,
                    int32_t diff_flag, int32_t channel, const int64_t* pixel_index,
                    int64_t n_pix, double* out)
{
    if (ora_check(c, diff_flag) || channel < 0 || channel >= c->n_channels) return -1;
    if ((n_points > 0 && !vertices) || (n_pix > 0 && (!pixel_index || !out))) return -1;
    const int64_t pnX = c->pixel_number[0];
    const int64_t pnXY = pnX * c->pixel_number[1];
    for (int64_t q = 0; q < n_pix; ++q)
        if (pixel_index[q] < 0 || pixel_index[q] >= pnXY) return -1;
    ora_geom g;
    ora_geom_init(c, c->wave_length[channel], &g);
    ora_point* pts = (ora_point*)malloc(sizeof(ora_point) * (size_t)(n_points > 0 ? n_points : 1));
    if (!pts) return -1;
#pragma omp parallel for schedule(static)
    for (int64_t i = 0; i < n_points; ++i)
        ora_point_init(c, &g, vertices + i * 7, channel, diff_flag, &pts[i]);
#pragma omp parallel for schedule(dynamic, 4)
    for (int64_t q = 0; q < n_pix; ++q) {
        int64_t xxtr = pixel_index[q] % pnX, yytr = pixel_index[q] / pnX;
        double sre = 0.0, sim = 0.0;
        for (int64_t i = 0; i < n_points; ++i) {
            const ora_point* p = &pts[i];
            if (xxtr < p->x_lo || xxtr >= p->x_hi || yytr < p->y_lo || yytr >= p->y_hi) continue;
            double re, im;
            if (diff_flag == 0) {
                if (!ora_rs_term(&g, p, xxtr, yytr, &re, &im)) continue;
            } else {
                ora_fresnel_term(&g, p, xxtr, yytr, &re, &im);
            }
            sre += re;
            sim += im;
        }
        out[q * 2 + 0] = sre;
        out[q * 2 + 1] = sim;
    }
    free(pts);
    return 0;
}

/* |z| as Complex<T>::mag / oph::absCplx: sqrt(re*re + im*im). */
static double ora_mag(double re, double im) { return sqrt(re * re + im * im); }

/* oph::maxOfArr over |field[i * stride]|, i < count (function.h:93-99,
 * 176-186): starts at MIN_DOUBLE, strict '>'. */
static double ora_absmax(const double* field, int64_t count, int64_t stride)
{
    double mx = ORA_MIN_DOUBLE;
    for (int64_t i = 0; i < count; ++i) {
        const double a = ora_mag(field[2 * i * stride], field[2 * i * stride + 1]);
        if (a > mx) mx = a;
    }
    return mx;
}

int oracle_encode(const double* field, int64_t n, int32_t encode_flag, double* encoded)
{
    if (n > 0 && (!field || !encoded)) return -1;
    const double pi2 = M_PI * 2;           /* ophGen.cpp:1846 */
    switch (encode_flag) {
    case 0:                                /* Phase, ophGen.cpp:1843-1853 */
#pragma omp parallel for
        for (int64_t i = 0; i < n; ++i)
            encoded[i] = (atan2(field[2 * i + 1], field[2 * i]) + M_PI) / pi2;
        break;
    case 1:                                /* Amplitude, ophGen.cpp:1855-1864 */
#pragma omp parallel for
        for (int64_t i = 0; i < n; ++i) encoded[i] = ora_mag(field[2 * i], field[2 * i + 1]);
        break;
    case 2:                                /* RealPart, ophGen.cpp:1821-1830 */
        for (int64_t i = 0; i < n; ++i) encoded[i] = field[2 * i];
        break;
    case 3:                                /* ImaginaryPart, ophGen.cpp:1832-1841 */
        for (int64_t i = 0; i < n; ++i) encoded[i] = field[2 * i + 1];
        break;
    case 4: {                              /* SimpleNI, ophGen.cpp:1955-1974 */
        const double mx = ora_absmax(field, n, 1);
        for (int64_t i = 0; i < n; ++i) {
            const double t = ora_mag(field[2 * i] + mx, field[2 * i + 1]);
            encoded[i] = t * t;
        }
        break;
    }
    case 5: {                              /* Burckhardt, ophGen.cpp:1897-1953 */
        const int64_t m = n / 3;
        const double mx = ora_absmax(field, m, 3);
        const double sqrt3 = sqrt(3), p2 = 2 * M_PI, p4 = 4 * M_PI;
        for (int64_t i = 0; i < m; ++i) {
            const double re = field[6 * i] / mx, im = field[6 * i + 1] / mx;
            const double ph = (atan2(im, re) + M_PI) / pi2;
            const double am = ora_mag(re, im);
            if (ph >= 0 && ph < (p2 / 3)) {
                encoded[3 * i] = am * (cos(ph) + sin(ph) / sqrt3);
                encoded[3 * i + 1] = 2 * sin(ph) / sqrt3;
            } else if (ph >= (p2 / 3) && ph < (p4 / 3)) {
                encoded[3 * i + 1] = am * (cos(ph - (p2 / 3)) + sin(ph - (p2 / 3)) / sqrt3);
                encoded[3 * i + 2] = 2 * sin(ph - (p2 / 3)) / sqrt3;
            } else if (ph >= (p4 / 3) && ph < (p2)) {
                encoded[3 * i + 2] = am * (cos(ph - (p4 / 3)) + sin(ph - (p4 / 3)) / sqrt3);
                encoded[3 * i] = 2 * sin(ph - (p4 / 3)) / sqrt3;
            }
        }
        break;
    }
    case 6: {                              /* TwoPhase, ophGen.cpp:1866-1895 */
        const int64_t m = n >> 1;
        const double mx = ora_absmax(field, m, 2);
        for (int64_t i = 0; i < m; ++i) {
            const double re = field[4 * i] / mx, im = field[4 * i + 1] / mx;
            const double ph = (atan2(im, re) + M_PI) / pi2;
            const double d = acos(ora_mag(re, im));
            encoded[2 * i] = (ph + M_PI) + d;
            encoded[2 * i + 1] = (ph + M_PI) - d;
        }
        break;
    }
    default:
        return -1;
    }
    return 0;
}

void oracle_normalize(const double* encoded, int32_t n_channels, int64_t n_per_channel,
                      uint8_t* out, double* min_out, double* max_out)
{
    double mn = ORA_MAX_DOUBLE, mx = ORA_MIN_DOUBLE;
    for (int32_t ch = 0; ch < n_channels; ++ch) {
        const double* e = encoded + (int64_t)ch * n_per_channel;
        double lmn = ORA_MAX_DOUBLE, lmx = ORA_MIN_DOUBLE;
        for (int64_t i = 0; i < n_per_channel; ++i) {
            if (e[i] < lmn) lmn = e[i];
            if (e[i] > lmx) lmx = e[i];
        }
        if (mn > lmn) mn = lmn;
        if (mx < lmx) mx = lmx;
    }
    double gap = mx - mn;
    if (min_out) *min_out = mn;
    if (max_out) *max_out = mx;
    const int64_t total = (int64_t)n_channels * n_per_channel;
#pragma omp parallel for
    for (int64_t i = 0; i < total; ++i) {
        double v = ((encoded[i] - mn) / gap) * 255 + 0.5;
        /* double -> uchar truncates; the value is in [0.5, 255.5] unless gap
         * is 0 (NaN), which both x86-64 and aarch64 conversions map to 0. */
        out[i] = (v >= 0.0 && v < 256.0) ? (uint8_t)(int)v : (uint8_t)0;
    }
}
