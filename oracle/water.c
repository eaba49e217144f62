/*
 * water.c — oracle of the water fragment stage.  TEST INFRASTRUCTURE ONLY:
 * loaded by tests/ as the checker of wt_water_raster and wt_water_shade;
 * never linked into the library.
 *
 *  - wto_water_fragment: assets/shaders/water-grid.frag:65-151 restated in
 *    FP32, statement by statement, with the GLSL built-ins and sampler state
 *    of oracle/glsl_frag_shim.hpp; pinned bit for bit against the shader
 *    source itself compiled as C++ (oracle/_ref).
 *  - wto_water_raster / wto_water_shade: the rasterisation rules that stand in
 *    for the GL driver's (there is no GL here): clip-space clipping of
 *    triangles that reach behind the near plane or beyond a guard band of 64
 *    viewports, window coordinates snapped to 1/256 pixel, exact integer edge
 *    functions at pixel centres with a left/top fill rule, window depth
 *    interpolated linearly in screen space and tested GL_LESS against the
 *    scene depth, nearest fragment per pixel (ties to the lower triangle
 *    index); varyings interpolated perspective-correctly from the three
 *    clip-space vertices (2D homogeneous barycentrics).
 * Compiled with -ffp-contract=off: every FP32 operation rounds once, in
 * source order, like the CUDA kernels built with -fmad=false.
 */
#include <math.h>
#include <stdint.h>
#include <string.h>

#include "wt_oracle.h"

/* ---- samplers (as oracle/glsl_frag_shim.hpp) ------------------------------ */

static uint32_t clampi(int64_t i, uint32_t n) { return (uint32_t)(i < 0 ? 0 : (i >= (int64_t)n ? n - 1 : i)); }

static void bilinear_rgba8(const uint8_t* px, uint32_t w, uint32_t h, float s, float t, float o[4]) {
    float u = s * (float)w - 0.5f;
    float v = t * (float)h - 0.5f;
    float fi = floorf(u), fj = floorf(v);
    float a = u - fi, b = v - fj;
    uint32_t i0 = clampi((int64_t)fi, w), i1 = clampi((int64_t)fi + 1, w);
    uint32_t j0 = clampi((int64_t)fj, h), j1 = clampi((int64_t)fj + 1, h);
    for (int c = 0; c < 4; ++c) {
        float t00 = (float)px[4 * ((size_t)j0 * w + i0) + c] / 255.0f;
        float t10 = (float)px[4 * ((size_t)j0 * w + i1) + c] / 255.0f;
        float t01 = (float)px[4 * ((size_t)j1 * w + i0) + c] / 255.0f;
        float t11 = (float)px[4 * ((size_t)j1 * w + i1) + c] / 255.0f;
        o[c] = (1.0f - b) * ((1.0f - a) * t00 + a * t10) + b * ((1.0f - a) * t01 + a * t11);
    }
}

static void sample_2d(const uint8_t* px, uint32_t w, uint32_t h, float s, float t, float o[4]) {
    if (!px) {
        o[0] = o[1] = o[2] = o[3] = 0.0f;
        return;
    }
    bilinear_rgba8(px, w, h, s, t, o);
}

static float sample_depth(const float* d, uint32_t w, uint32_t h, float s, float t) {
    if (!d) return 1.0f;
    uint32_t i = clampi((int64_t)floorf(s * (float)w), w);
    uint32_t j = clampi((int64_t)floorf(t * (float)h), h);
    return d[(size_t)j * w + i];
}

/* OpenGL 4.1 table 3.19: face by the major axis, then (s, t) on that face */
static void sample_cube(const uint8_t* faces, uint32_t size, const float r[3], float o[4]) {
    float ax = fabsf(r[0]), ay = fabsf(r[1]), az = fabsf(r[2]);
    int face;
    float sc, tc, ma;
    if (ax >= ay && ax >= az) {
        face = r[0] >= 0.0f ? 0 : 1;
        sc = r[0] >= 0.0f ? -r[2] : r[2];
        tc = -r[1];
        ma = ax;
    } else if (ay >= az) {
        face = r[1] >= 0.0f ? 2 : 3;
        sc = r[0];
        tc = r[1] >= 0.0f ? r[2] : -r[2];
        ma = ay;
    } else {
        face = r[2] >= 0.0f ? 4 : 5;
        sc = r[2] >= 0.0f ? r[0] : -r[0];
        tc = -r[1];
        ma = az;
    }
    float s = (sc / ma + 1.0f) / 2.0f;
    float t = (tc / ma + 1.0f) / 2.0f;
    bilinear_rgba8(faces + (size_t)face * size * size * 4, size, size, s, t, o);
}

static float clampf(float x, float lo, float hi) { return fminf(fmaxf(x, lo), hi); }
static float mixf(float x, float y, float a) { return x * (1.0f - a) + y * a; }
static float dot3(const float a[3], const float b[3]) { return a[0] * b[0] + a[1] * b[1] + a[2] * b[2]; }

/* ---- water-grid.frag:65-151 ----------------------------------------------- */

static float linearize_depth(const wto_frag_uniforms* u, float depth) {
    return (u->s.z_near * depth) / (u->s.z_far - depth * (u->s.z_far - u->s.z_near));
}

static void fragment(const wto_frag_uniforms* u, const wto_frag_in* f, float out[4]) {
    const wt_water_shading* s = &u->s;
    float view_len = sqrtf(dot3(f->view, f->view));
    float view_depth = clampf(view_len / s->z_far, 0.0f, 1.0f);
    float vv[3] = {f->view[0] / view_len, f->view[1] / view_len, f->view[2] / view_len};
    float uv[2] = {f->frag_coord[0] / (float)u->width, f->frag_coord[1] / (float)u->height};
    float uv0[2] = {(f->ndc0[0] + 1.0f) / 2.0f, (f->ndc0[1] + 1.0f) / 2.0f};
    float back = linearize_depth(u, sample_depth(u->tex.scene_depth, u->width, u->height, uv[0], uv[1]));
    float sky_behind = back > 0.999f ? 0.0f : 1.0f;
    float here = linearize_depth(u, f->frag_coord[2]);
    float delta = clampf(back - here, 0.0f, 1.0f);
    /* R = reflect(-viewVec, normal) = I - 2 dot(N, I) N */
    float I[3] = {-vv[0], -vv[1], -vv[2]};
    float k = 2.0f * dot3(f->normal, I);
    float R[3] = {I[0] - k * f->normal[0], I[1] - k * f->normal[1], I[2] - k * f->normal[2]};
    float sky[4];
    sample_cube(u->tex.skybox, u->tex.skybox_size, R, sky);
    float sun_s = s->sun_strength * 1.0f;
    float sun_p = powf(clampf(dot3(R, s->sun_position), 0.0f, 1.0f), s->sun_shininess);
    float sun = sun_s * sun_p;
    float cos_t = dot3(f->normal, vv);
    float fres = 0.02f + (1.0f - 0.02f) * powf(1.0f - cos_t, 5.0f);
    float refl_s = 0.1f * (1.0f - view_depth);
    float refr_s = 0.1f * (1.0f - view_depth);
    float uvl[2], uvr[2];
    uvl[0] = clampf(mixf(uv[0], uv0[0], refl_s) + refl_s * f->normal_yaw[0], 0.0f, 1.0f);
    uvl[1] = clampf(mixf(uv[1], uv0[1], refl_s) + refl_s * -f->normal_yaw[2], 0.0f, 1.0f);
    uvr[0] = clampf(mixf(uv[0], uv0[0], refr_s) + refr_s * -f->normal_yaw[0], 0.0f, 1.0f);
    uvr[1] = clampf(mixf(uv[1], uv0[1], refr_s) + refr_s * f->normal_yaw[2], 0.0f, 1.0f);
    float lrefl[4], lrefr[4];
    sample_2d(u->tex.local_reflections, u->width, u->height, uvl[0], uvl[1], lrefl);
    sample_2d(u->tex.local_refractions, u->width, u->height, uvr[0], uvr[1], lrefr);
    static const float deep[3] = {0.0f, 0.341f, 0.482f}, shallow[3] = {0.3f, 0.941f, 0.903f};
    float tint_f = 0.0f == s->tint_threshold
                       ? 0.0f
                       : sky_behind * (1.0f - clampf(delta / s->tint_threshold, 0.0f, 1.0f));
    float day = clampf(s->sun_position[1], 0.0f, 1.0f);
    float clarity = s->water_clarity * lrefr[3] * (1.0f - delta);
    for (int c = 0; c < 3; ++c) {
        float tint = day * mixf(deep[c], shallow[c], tint_f);
        float trans = mixf(tint, lrefr[c], clarity);
        float refl = mixf(sky[c] + sun, lrefl[c], lrefl[3]);
        out[c] = mixf(trans, refl, fres);
    }
    out[3] = 0.0f == s->soft_edges_threshold
                 ? 1.0f
                 : 1.0f - (sky_behind * (1.0f - clampf(delta / s->soft_edges_threshold, 0.0f, 1.0f)));
    float fog_a = view_depth >= s->fog_radius_far
                      ? s->fog_colour[3]
                      : view_depth <= s->fog_radius_near
                            ? 0.0f
                            : s->fog_colour[3] * ((view_depth - s->fog_radius_near) /
                                                  (s->fog_radius_far - s->fog_radius_near));
    for (int c = 0; c < 3; ++c) out[c] = mixf(out[c], s->fog_colour[c], fog_a);
}

void wto_water_fragment(const wto_frag_uniforms* u, const wto_frag_in* f, uint64_t n, float* colour4) {
    for (uint64_t i = 0; i < n; ++i) fragment(u, f + i, colour4 + 4 * i);
}

/* ---- rasterisation -------------------------------------------------------- */

#define WTO_SUB 256.0f
#define WTO_GUARD 64.0f

typedef struct { float x, y, z, w; } cv4;

static float f_bits_as(uint32_t b) { float f; memcpy(&f, &b, 4); return f; }
static uint32_t f_as_bits(float f) { uint32_t b; memcpy(&b, &f, 4); return b; }

static void raster_window_tri(const int32_t X[3], const int32_t Y[3], const float Z[3], uint32_t tri,
                              uint32_t W, uint32_t H, uint64_t* frag) {
    int64_t area = (int64_t)(X[1] - X[0]) * (Y[2] - Y[0]) - (int64_t)(Y[1] - Y[0]) * (X[2] - X[0]);
    if (area == 0) return;
    int32_t x[3] = {X[0], X[1], X[2]}, y[3] = {Y[0], Y[1], Y[2]};
    float z[3] = {Z[0], Z[1], Z[2]};
    if (area < 0) {
        x[1] = X[2]; y[1] = Y[2]; z[1] = Z[2];
        x[2] = X[1]; y[2] = Y[1]; z[2] = Z[1];
        area = -area;
    }
    int32_t xmin = x[0], xmax = x[0], ymin = y[0], ymax = y[0];
    for (int k = 1; k < 3; ++k) {
        xmin = x[k] < xmin ? x[k] : xmin; xmax = x[k] > xmax ? x[k] : xmax;
        ymin = y[k] < ymin ? y[k] : ymin; ymax = y[k] > ymax ? y[k] : ymax;
    }
    int64_t px0 = -((128 - (int64_t)xmin) >> 8), px1 = ((int64_t)xmax - 128) >> 8;
    int64_t py0 = -((128 - (int64_t)ymin) >> 8), py1 = ((int64_t)ymax - 128) >> 8;
    if (px0 < 0) px0 = 0;
    if (py0 < 0) py0 = 0;
    if (px1 > (int64_t)W - 1) px1 = (int64_t)W - 1;
    if (py1 > (int64_t)H - 1) py1 = (int64_t)H - 1;
    /* edge k runs from vertex k+1 to vertex k+2, opposite vertex k */
    int incl[3];
    for (int k = 0; k < 3; ++k) {
        int a = (k + 1) % 3, b = (k + 2) % 3;
        int32_t dx = x[b] - x[a], dy = y[b] - y[a];
        incl[k] = dy < 0 || (dy == 0 && dx < 0);
    }
    const float fa = (float)area;
    for (int64_t py = py0; py <= py1; ++py)
        for (int64_t px = px0; px <= px1; ++px) {
            int64_t cx = px * 256 + 128, cy = py * 256 + 128;
            int64_t e[3];
            int in = 1;
            for (int k = 0; k < 3; ++k) {
                int a = (k + 1) % 3, b = (k + 2) % 3;
                e[k] = (int64_t)(x[b] - x[a]) * (cy - y[a]) - (int64_t)(y[b] - y[a]) * (cx - x[a]);
                if (!(e[k] > 0 || (e[k] == 0 && incl[k]))) in = 0;
            }
            if (!in) continue;
            float d = ((float)e[0] * z[0] + (float)e[1] * z[1] + (float)e[2] * z[2]) / fa;
            if (!(d >= 0.0f && d <= 1.0f)) continue;
            d = d + 0.0f;
            uint64_t key = ((uint64_t)f_as_bits(d) << 32) | (uint64_t)(tri + 1);
            uint64_t* slot = frag + (size_t)py * W + px;
            if (key < *slot) *slot = key;
        }
}

static void to_window(cv4 c, uint32_t W, uint32_t H, int32_t* X, int32_t* Y, float* Z) {
    float xw = (c.x / c.w + 1.0f) * ((float)W * 0.5f);
    float yw = (c.y / c.w + 1.0f) * ((float)H * 0.5f);
    *X = (int32_t)rintf(xw * WTO_SUB);
    *Y = (int32_t)rintf(yw * WTO_SUB);
    *Z = (c.z / c.w) * 0.5f + 0.5f;
}

static float plane_dist(int p, cv4 c) {
    switch (p) {
        case 0: return c.z + c.w;
        case 1: return WTO_GUARD * c.w - c.x;
        case 2: return WTO_GUARD * c.w + c.x;
        case 3: return WTO_GUARD * c.w - c.y;
        default: return WTO_GUARD * c.w + c.y;
    }
}

/* Sutherland-Hodgman against the near plane and the guard band (<= 8 vertices) */
static int clip_polygon(cv4* poly, int n) {
    cv4 tmp[10];
    for (int p = 0; p < 5 && n > 0; ++p) {
        int m = 0;
        for (int i = 0; i < n; ++i) {
            cv4 a = poly[i], b = poly[(i + 1) % n];
            float da = plane_dist(p, a), db = plane_dist(p, b);
            if (da >= 0.0f) tmp[m++] = a;
            if ((da >= 0.0f) != (db >= 0.0f)) {
                float t = da / (da - db);
                cv4 q = {a.x + t * (b.x - a.x), a.y + t * (b.y - a.y), a.z + t * (b.z - a.z), a.w + t * (b.w - a.w)};
                tmp[m++] = q;
            }
        }
        for (int i = 0; i < m; ++i) poly[i] = tmp[i];
        n = m;
    }
    return n;
}

static int fast_path(const cv4 v[3]) {
    for (int k = 0; k < 3; ++k)
        if (!(v[k].w > 0.0f && fabsf(v[k].x) <= WTO_GUARD * v[k].w && fabsf(v[k].y) <= WTO_GUARD * v[k].w)) return 0;
    return 1;
}

void wto_water_raster(const float* clip4, uint64_t n_vertices, const uint32_t* idx, uint64_t n_triangles,
                      uint32_t width, uint32_t height, const float* scene_depth, uint64_t* fragments) {
    for (uint64_t p = 0; p < (uint64_t)width * height; ++p) {
        float d = scene_depth ? scene_depth[p] : 1.0f;
        fragments[p] = (uint64_t)f_as_bits(d) << 32;
    }
    for (uint64_t t = 0; t < n_triangles; ++t) {
        cv4 v[3];
        int ok = 1;
        for (int k = 0; k < 3; ++k) {
            uint32_t i = idx[3 * t + k];
            if (i >= n_vertices) { ok = 0; break; }
            v[k].x = clip4[4 * (size_t)i]; v[k].y = clip4[4 * (size_t)i + 1];
            v[k].z = clip4[4 * (size_t)i + 2]; v[k].w = clip4[4 * (size_t)i + 3];
        }
        if (!ok) continue;
        int32_t X[3], Y[3];
        float Z[3];
        if (fast_path(v)) {
            for (int k = 0; k < 3; ++k) to_window(v[k], width, height, &X[k], &Y[k], &Z[k]);
            raster_window_tri(X, Y, Z, (uint32_t)t, width, height, fragments);
            continue;
        }
        cv4 poly[10] = {v[0], v[1], v[2]};
        int n = clip_polygon(poly, 3);
        if (n < 3) continue;
        int bad = 0;
        for (int k = 0; k < n; ++k) bad |= !(poly[k].w > 0.0f);
        if (bad) continue;
        for (int k = 1; k + 1 < n; ++k) {
            cv4 s[3] = {poly[0], poly[k], poly[k + 1]};
            for (int j = 0; j < 3; ++j) to_window(s[j], width, height, &X[j], &Y[j], &Z[j]);
            raster_window_tri(X, Y, Z, (uint32_t)t, width, height, fragments);
        }
    }
}

/* ---- shading -------------------------------------------------------------- */

void wto_water_shade(const uint64_t* fragments, const float* clip4, const uint32_t* idx, const float* facing4,
                     const float* nyaw4, const float* view4, const float* ndc0, const wto_frag_uniforms* u,
                     float* colour_out, float* composite) {
    const uint32_t W = u->width, H = u->height;
    for (uint32_t py = 0; py < H; ++py)
        for (uint32_t px = 0; px < W; ++px) {
            size_t p = (size_t)py * W + px;
            uint64_t key = fragments[p];
            uint32_t tri1 = (uint32_t)(key & 0xffffffffu);
            float col[4] = {0.0f, 0.0f, 0.0f, 0.0f};
            if (tri1 != 0) {
                uint32_t t = tri1 - 1;
                uint32_t vi[3] = {idx[3 * (size_t)t], idx[3 * (size_t)t + 1], idx[3 * (size_t)t + 2]};
                float nx = (2.0f * ((float)px + 0.5f)) / (float)W - 1.0f;
                float ny = (2.0f * ((float)py + 0.5f)) / (float)H - 1.0f;
                float v[3][3];
                for (int k = 0; k < 3; ++k) {
                    v[k][0] = clip4[4 * (size_t)vi[k]];
                    v[k][1] = clip4[4 * (size_t)vi[k] + 1];
                    v[k][2] = clip4[4 * (size_t)vi[k] + 3];
                }
                float c[3];
                for (int k = 0; k < 3; ++k) {
                    const float* a = v[(k + 1) % 3];
                    const float* b = v[(k + 2) % 3];
                    float cx = a[1] * b[2] - a[2] * b[1];
                    float cy = a[2] * b[0] - a[0] * b[2];
                    float cz = a[0] * b[1] - a[1] * b[0];
                    c[k] = cx * nx + cy * ny + cz;
                }
                float sum = c[0] + c[1] + c[2];
                float l[3] = {c[0] / sum, c[1] / sum, c[2] / sum};
                wto_frag_in f;
                f.frag_coord[0] = (float)px + 0.5f;
                f.frag_coord[1] = (float)py + 0.5f;
                f.frag_coord[2] = f_bits_as((uint32_t)(key >> 32));
                f.frag_coord[3] = 1.0f;
                for (int j = 0; j < 3; ++j) {
                    f.normal[j] = l[0] * facing4[4 * (size_t)vi[0] + j] + l[1] * facing4[4 * (size_t)vi[1] + j] +
                                  l[2] * facing4[4 * (size_t)vi[2] + j];
                    f.normal_yaw[j] = l[0] * nyaw4[4 * (size_t)vi[0] + j] + l[1] * nyaw4[4 * (size_t)vi[1] + j] +
                                      l[2] * nyaw4[4 * (size_t)vi[2] + j];
                    f.view[j] = l[0] * view4[4 * (size_t)vi[0] + j] + l[1] * view4[4 * (size_t)vi[1] + j] +
                                l[2] * view4[4 * (size_t)vi[2] + j];
                }
                for (int j = 0; j < 2; ++j)
                    f.ndc0[j] = l[0] * ndc0[2 * (size_t)vi[0] + j] + l[1] * ndc0[2 * (size_t)vi[1] + j] +
                                l[2] * ndc0[2 * (size_t)vi[2] + j];
                fragment(u, &f, col);
            }
            if (colour_out)
                for (int j = 0; j < 4; ++j) colour_out[4 * p + j] = col[j];
            if (composite && tri1 != 0) {
                float a = col[3];
                for (int j = 0; j < 4; ++j)
                    composite[4 * p + j] = col[j] * a + composite[4 * p + j] * (1.0f - a);
            }
        }
}
