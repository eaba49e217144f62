/*
 * gerstner_f64.c — FP64 truth for the Gerstner water-surface path.
 * Test infrastructure only (see wt_oracle.h); never used by the product.
 *
 * Follows assets/shaders/water-grid.vert:
 *   :87-91, :123-125  grid position = mix(mix(BL,BR,u), mix(TL,TR,u), v),
 *                     u = col/(L-1), v = row/(L-1); the corners' y is dropped
 *                     because the Gerstner start point is vec3(x, 0, z) (:75)
 *   :74-85            theta = w*dot(D, xz) + phi*t;
 *                     P += A*(D.x*Q*cos, sin, D.z*Q*cos)
 *   :93-111, :141-144 heightmap sampled at the displaced (x', -z') scaled by
 *                     heightmapSampleScale, y += scale*2*(r - 0.5)
 *   :147              y += verticalBounceWaveDisplacement
 * with the sampler state of src/texture.cpp:63-66 (GL_LINEAR, REPEAT or
 * MIRRORED_REPEAT texel wrap) and the wave mapping of include/wt.h
 * (w = k = 2*pi/lambda, phi = speed*k, plus a constant phase).
 * The normal is the exact one of the displaced surface, dP/dz x dP/dx,
 * including the heightmap gradient; the reference's central differences
 * (water-grid.vert:164-187) are restated in reference_mode.c instead.
 */
#include <math.h>
#include <string.h>
#include "wt_oracle.h"

#define TWO_PI 6.283185307179586476925286766559

static double wave_k(const wt_wave* w) {
    double lam = (double)w->wavelength;
    if (isinf(lam)) return 0.0;
    return TWO_PI / lam;
}

void wto_grid_xz_f64(const wt_patch* p, uint32_t row, uint32_t col, double* x, double* z) {
    double u = (double)col / (double)(p->cols - 1);
    double v = (double)row / (double)(p->rows - 1);
    /* mix(a, b, t) = a*(1-t) + b*t (GLSL definition) */
    double bx = (double)p->bl[0] * (1.0 - u) + (double)p->br[0] * u;
    double bz = (double)p->bl[1] * (1.0 - u) + (double)p->br[1] * u;
    double tx = (double)p->tl[0] * (1.0 - u) + (double)p->tr[0] * u;
    double tz = (double)p->tl[1] * (1.0 - u) + (double)p->tr[1] * u;
    *x = bx * (1.0 - v) + tx * v;
    *z = bz * (1.0 - v) + tz * v;
}

/* Texel index wrap of the GL spec (texture wrap modes table):
 * REPEAT: i mod n;  MIRRORED_REPEAT: (n-1) - mirror((i mod 2n) - n),
 * mirror(a) = a >= 0 ? a : -(1 + a). */
static int64_t wrap_index(int64_t i, int64_t n, uint32_t mode) {
    if (mode == WT_WRAP_MIRRORED_REPEAT) {
        int64_t m = i % (2 * n);
        if (m < 0) m += 2 * n;
        int64_t a = m - n;
        int64_t mir = a >= 0 ? a : -(1 + a);
        return n - 1 - mir;
    }
    int64_t m = i % n;
    if (m < 0) m += n;
    return m;
}

typedef struct hm_sample {
    double h;     /* height contribution disp*2*(r-0.5) */
    double hx;    /* dh/dX' */
    double hz;    /* dh/dZ' */
    double hxz;   /* d2h/dX'dZ' (the bilinear cross term; d2/dX'2 = d2/dZ'2 = 0) */
    double edge;  /* distance to the nearest cell boundary, texels */
} hm_sample;

static hm_sample sample_hm(const wto_heightmap* hm, double X, double Z) {
    hm_sample r;
    double W = (double)hm->width, H = (double)hm->height;
    double su = (double)hm->sample_scale * X * W - 0.5;
    double sv = (double)hm->sample_scale * (-Z) * H - 0.5;
    double fi = floor(su), fj = floor(sv);
    double a = su - fi, b = sv - fj;
    int64_t i0 = (int64_t)fi, j0 = (int64_t)fj;
    int64_t ia = wrap_index(i0, hm->width, hm->wrap), ib = wrap_index(i0 + 1, hm->width, hm->wrap);
    int64_t ja = wrap_index(j0, hm->height, hm->wrap), jb = wrap_index(j0 + 1, hm->height, hm->wrap);
    double t00 = hm->texels[ja * hm->width + ia], t10 = hm->texels[ja * hm->width + ib];
    double t01 = hm->texels[jb * hm->width + ia], t11 = hm->texels[jb * hm->width + ib];
    double rr = (1.0 - b) * ((1.0 - a) * t00 + a * t10) + b * ((1.0 - a) * t01 + a * t11);
    double dru = (1.0 - b) * (t10 - t00) + b * (t11 - t01);
    double drv = (1.0 - a) * (t01 - t00) + a * (t11 - t10);
    double k2 = 2.0 * (double)hm->disp_scale;
    double du_dX = (double)hm->sample_scale * W, dv_dZ = -(double)hm->sample_scale * H;
    r.h = k2 * (rr - 0.5);
    r.hx = k2 * dru * du_dX;
    r.hz = k2 * drv * dv_dZ;
    r.hxz = k2 * (t00 - t10 - t01 + t11) * du_dX * dv_dZ;
    double e = a < 1.0 - a ? a : 1.0 - a;
    double eb = b < 1.0 - b ? b : 1.0 - b;
    r.edge = e < eb ? e : eb;
    return r;
}

/* Sums of one vertex over the waves of a patch. */
typedef struct wsum {
    double dx, dy, dz;       /* displacement */
    double jx, jz;           /* d(y)/dx, d(y)/dz */
    double sxx, sxz, szz;    /* sum Q A k D_a D_b sin(theta) */
} wsum;

static void wave_sums(const wt_patch* p, const wt_wave* waves, double x, double z, wsum* s) {
    memset(s, 0, sizeof(*s));
    double t = p->time_s;
    for (uint32_t i = 0; i < p->wave_count; ++i) {
        const wt_wave* w = &waves[p->wave_offset + i];
        double k = wave_k(w);
        double A = w->amplitude, Q = w->steepness_q, Dx = w->dir_x, Dz = w->dir_z;
        double th = k * (Dx * x + Dz * z) + (double)w->speed * k * t + (double)w->phase;
        double c = cos(th), sn = sin(th);
        s->dx += Q * A * Dx * c;
        s->dy += A * sn;
        s->dz += Q * A * Dz * c;
        s->jx += A * k * Dx * c;
        s->jz += A * k * Dz * c;
        s->sxx += Q * A * k * Dx * Dx * sn;
        s->sxz += Q * A * k * Dx * Dz * sn;
        s->szz += Q * A * k * Dz * Dz * sn;
    }
}

/* One vertex: displaced position, displacement, unit normal, texel-edge
 * distance (any output may be NULL). */
static void vertex_f64(const wt_patch* p, const wt_wave* waves, const wto_heightmap* hm, uint32_t row,
                       uint32_t col, double* pos, double* disp, double* nrm, double* edge) {
    double x, z;
    wto_grid_xz_f64(p, row, col, &x, &z);
    wsum s;
    wave_sums(p, waves, x, z, &s);
    /* dP/dx and dP/dz of the Gerstner surface */
    double px[3] = {1.0 - s.sxx, s.jx, -s.sxz};
    double pz[3] = {-s.sxz, s.jz, 1.0 - s.szz};
    double dy = s.dy;
    double e = INFINITY;
    if (hm && hm->texels) {
        hm_sample h = sample_hm(hm, x + s.dx, z + s.dz);
        dy += h.h;
        px[1] += h.hx * px[0] + h.hz * px[2];
        pz[1] += h.hx * pz[0] + h.hz * pz[2];
        e = h.edge;
    }
    dy += (double)p->y_offset;
    if (pos) { pos[0] = x + s.dx; pos[1] = dy; pos[2] = z + s.dz; }
    if (disp) { disp[0] = s.dx; disp[1] = dy; disp[2] = s.dz; }
    if (nrm) {
        double n0 = pz[1] * px[2] - pz[2] * px[1];
        double n1 = pz[2] * px[0] - pz[0] * px[2];
        double n2 = pz[0] * px[1] - pz[1] * px[0];
        double inv = 1.0 / sqrt(n0 * n0 + n1 * n1 + n2 * n2);
        nrm[0] = n0 * inv; nrm[1] = n1 * inv; nrm[2] = n2 * inv;
    }
    if (edge) *edge = e;
}

void wto_displace_f64(const wt_patch* p, const wt_wave* waves, const wto_heightmap* hm,
                      uint32_t row0, uint32_t row1,
                      double* pos, double* disp, double* nrm, double* edge) {
    for (uint32_t row = row0; row < row1 && row < p->rows; ++row)
        for (uint32_t col = 0; col < p->cols; ++col) {
            size_t v = (size_t)row * p->cols + col;
            vertex_f64(p, waves, hm, row, col, pos ? pos + 3 * v : NULL, disp ? disp + 3 * v : NULL,
                       nrm ? nrm + 3 * v : NULL, edge ? edge + v : NULL);
        }
}

void wto_displace_f64_rows(const wt_patch* p, const wt_wave* waves, const wto_heightmap* hm,
                           const uint32_t* rows, uint32_t n_rows, double* pos, double* disp, double* nrm,
                           double* edge) {
    for (uint32_t k = 0; k < n_rows; ++k)
        for (uint32_t col = 0; col < p->cols; ++col) {
            size_t v = (size_t)k * p->cols + col;
            vertex_f64(p, waves, hm, rows[k], col, pos ? pos + 3 * v : NULL, disp ? disp + 3 * v : NULL,
                       nrm ? nrm + 3 * v : NULL, edge ? edge + v : NULL);
        }
}

/* Reverse mode by hand.  Per vertex the loss touches the wave sums through
 * pos = (x + dx, dy + H(x+dx, z+dz) + y_offset, z + dz) and through the unit
 * normal of N = Pz x Px; the adjoints of the eight sums are formed first, then
 * every wave's contribution to each sum is differentiated with respect to its
 * parameters. */
void wto_adjoint_f64(const wt_patch* p, const wt_wave* waves, const wto_heightmap* hm,
                     const float* gpos, const float* gnrm, double* grad) {
    double t = p->time_s;
    for (uint32_t row = 0; row < p->rows; ++row) {
        for (uint32_t col = 0; col < p->cols; ++col) {
            size_t v = (size_t)p->out_offset + (size_t)row * p->cols + col;
            double x, z;
            wto_grid_xz_f64(p, row, col, &x, &z);
            wsum s;
            wave_sums(p, waves, x, z, &s);
            double a1 = 1.0 - s.sxx, a3 = -s.sxz, b1 = -s.sxz, b3 = 1.0 - s.szz;
            hm_sample h = {0, 0, 0, 0, INFINITY};
            if (hm && hm->texels) h = sample_hm(hm, x + s.dx, z + s.dz);
            double px[3] = {a1, s.jx + h.hx * a1 + h.hz * a3, a3};
            double pz[3] = {b1, s.jz + h.hx * b1 + h.hz * b3, b3};
            double gpx[3] = {0, 0, 0}, gpz[3] = {0, 0, 0};
            if (gnrm) {
                double N[3] = {pz[1] * px[2] - pz[2] * px[1], pz[2] * px[0] - pz[0] * px[2],
                               pz[0] * px[1] - pz[1] * px[0]};
                double len = sqrt(N[0] * N[0] + N[1] * N[1] + N[2] * N[2]);
                double n[3] = {N[0] / len, N[1] / len, N[2] / len};
                double gn[3] = {gnrm[4 * v], gnrm[4 * v + 1], gnrm[4 * v + 2]};
                double d = n[0] * gn[0] + n[1] * gn[1] + n[2] * gn[2];
                double gN[3] = {(gn[0] - n[0] * d) / len, (gn[1] - n[1] * d) / len,
                                (gn[2] - n[2] * d) / len};
                /* N = Pz x Px: g_Pz = Px x gN, g_Px = gN x Pz */
                gpz[0] = px[1] * gN[2] - px[2] * gN[1];
                gpz[1] = px[2] * gN[0] - px[0] * gN[2];
                gpz[2] = px[0] * gN[1] - px[1] * gN[0];
                gpx[0] = gN[1] * pz[2] - gN[2] * pz[1];
                gpx[1] = gN[2] * pz[0] - gN[0] * pz[2];
                gpx[2] = gN[0] * pz[1] - gN[1] * pz[0];
            }
            double g_jx = gpx[1], g_jz = gpz[1];
            double g_a1 = gpx[0] + gpx[1] * h.hx, g_a3 = gpx[2] + gpx[1] * h.hz;
            double g_b1 = gpz[0] + gpz[1] * h.hx, g_b3 = gpz[2] + gpz[1] * h.hz;
            double g_hx = gpx[1] * a1 + gpz[1] * b1, g_hz = gpx[1] * a3 + gpz[1] * b3;
            double g_h = gpos[4 * v + 1];
            double g_X = g_h * h.hx + g_hz * h.hxz;
            double g_Z = g_h * h.hz + g_hx * h.hxz;
            double g_dx = gpos[4 * v] + g_X, g_dz = gpos[4 * v + 2] + g_Z, g_dy = gpos[4 * v + 1];
            double g_sxx = -g_a1, g_sxz = -g_a3 - g_b1, g_szz = -g_b3;
            for (uint32_t i = 0; i < p->wave_count; ++i) {
                const wt_wave* w = &waves[p->wave_offset + i];
                double* g = &grad[8 * (size_t)(p->wave_offset + i)];
                double k = wave_k(w);
                double A = w->amplitude, Q = w->steepness_q, Dx = w->dir_x, Dz = w->dir_z;
                double sp = w->speed;
                double th = k * (Dx * x + Dz * z) + sp * k * t + (double)w->phase;
                double c = cos(th), sn = sin(th);
                /* coefficient of cos (dx, dz, jx, jz) and of sin (dy, sxx, sxz, szz) */
                double Ec = g_dx * Q * A * Dx + g_dz * Q * A * Dz + g_jx * A * k * Dx + g_jz * A * k * Dz;
                double Es = g_dy * A + (g_sxx * Dx * Dx + g_sxz * Dx * Dz + g_szz * Dz * Dz) * Q * A * k;
                double gth = -Ec * sn + Es * c;
                double gA = (A != 0.0) ? (Ec * c + Es * sn) / A
                                       : ((g_dx * Q * Dx + g_dz * Q * Dz + g_jx * k * Dx + g_jz * k * Dz) * c +
                                          (g_dy + (g_sxx * Dx * Dx + g_sxz * Dx * Dz + g_szz * Dz * Dz) * Q * k) * sn);
                double gQ = A * ((g_dx * Dx + g_dz * Dz) * c +
                                 (g_sxx * Dx * Dx + g_sxz * Dx * Dz + g_szz * Dz * Dz) * k * sn);
                double gk_exp = A * ((g_jx * Dx + g_jz * Dz) * c +
                                     (g_sxx * Dx * Dx + g_sxz * Dx * Dz + g_szz * Dz * Dz) * Q * sn);
                double gk = gk_exp + gth * (Dx * x + Dz * z + sp * t);
                double gDx = g_dx * Q * A * c + g_jx * A * k * c + Q * A * k * (2.0 * Dx * g_sxx + Dz * g_sxz) * sn + gth * k * x;
                double gDz = g_dz * Q * A * c + g_jz * A * k * c + Q * A * k * (2.0 * Dz * g_szz + Dx * g_sxz) * sn + gth * k * z;
                double lam = w->wavelength;
                g[0] += gA;
                g[1] += isinf(lam) ? 0.0 : -gk * k / lam;
                g[2] += -Dz * gDx + Dx * gDz;
                g[3] += gQ;
                g[4] += gth;
                g[5] += gth * k * t;
                g[6] += gDx;
                g[7] += gDz;
            }
        }
    }
}
