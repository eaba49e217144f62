/*
 * reference_mode.c — FP32 restatement of assets/shaders/water-grid.vert.
 * Test infrastructure only (see wt_oracle.h); never used by the product.
 *
 * Every operation keeps the shader's order so that, compiled with
 * -ffp-contract=off, it reproduces bit for bit the shader source compiled as
 * C++ over the GLSL built-ins of oracle/glsl_shim.hpp (oracle/_ref).  The
 * built-ins follow the GLSL 4.10 definitions:
 *   mix(x, y, a) = x*(1-a) + y*a            mod(x, y) = x - y*floor(x/y)
 *   cross, dot, normalize = v / length(v)   sin/cos = C sinf/cosf
 *   texture(): GL_LINEAR at texel centres, GL_REPEAT / GL_MIRRORED_REPEAT
 *   texel wrap (src/texture.cpp:63-66), grey texels returned as (r, r, r, 1)
 *   (RGBA expansion of the 8-bit grey PNG, src/render-engine.cpp:1311).
 */
#include <math.h>
#include <pthread.h>
#include <stdatomic.h>
#include <stdlib.h>
#include <string.h>
#include "wt_oracle.h"

typedef struct { float x, y; } v2;
typedef struct { float x, y, z; } v3;
typedef struct { float x, y, z, w; } v4;

static float glsl_mix(float x, float y, float a) { return x * (1.0f - a) + y * a; }
static v4 mix4(v4 x, v4 y, float a) {
    v4 r = {glsl_mix(x.x, y.x, a), glsl_mix(x.y, y.y, a), glsl_mix(x.z, y.z, a), glsl_mix(x.w, y.w, a)};
    return r;
}
static float glsl_mod(float x, float y) { return x - y * floorf(x / y); }
static float dot2(v2 a, v2 b) { return a.x * b.x + a.y * b.y; }
static float dot3(v3 a, v3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
static v3 cross3(v3 a, v3 b) {
    v3 r = {a.y * b.z - b.y * a.z, a.z * b.x - b.z * a.x, a.x * b.y - b.x * a.y};
    return r;
}
static v3 normalize3(v3 a) {
    float l = sqrtf(dot3(a, a));
    v3 r = {a.x / l, a.y / l, a.z / l};
    return r;
}
/* column-major mat4 * vec4, summed in column order */
static v4 mat4_mul(const float* m, v4 v) {
    v4 r;
    r.x = m[0] * v.x + m[4] * v.y + m[8] * v.z + m[12] * v.w;
    r.y = m[1] * v.x + m[5] * v.y + m[9] * v.z + m[13] * v.w;
    r.z = m[2] * v.x + m[6] * v.y + m[10] * v.z + m[14] * v.w;
    r.w = m[3] * v.x + m[7] * v.y + m[11] * v.z + m[15] * v.w;
    return r;
}

static int64_t wrap_i(int64_t i, int64_t n, uint32_t mode) {
    if (mode == WT_WRAP_MIRRORED_REPEAT) {
        int64_t m = i % (2 * n);
        if (m < 0) m += 2 * n;
        int64_t a = m - n;
        return n - 1 - (a >= 0 ? a : -(1 + a));
    }
    int64_t m = i % n;
    return m < 0 ? m + n : m;
}

/* texture(sampler2D, vec2) with GL_LINEAR on the base level. */
static v4 texture2d(const wto_heightmap* hm, v2 st) {
    v4 r = {0.0f, 0.0f, 0.0f, 0.0f};
    if (!hm->texels) return r;
    float u = st.x * (float)hm->width - 0.5f;
    float v = st.y * (float)hm->height - 0.5f;
    float fi = floorf(u), fj = floorf(v);
    float a = u - fi, b = v - fj;
    int64_t i0 = (int64_t)fi, j0 = (int64_t)fj;
    int64_t ia = wrap_i(i0, hm->width, hm->wrap), ib = wrap_i(i0 + 1, hm->width, hm->wrap);
    int64_t ja = wrap_i(j0, hm->height, hm->wrap), jb = wrap_i(j0 + 1, hm->height, hm->wrap);
    float t00 = hm->texels[ja * hm->width + ia], t10 = hm->texels[ja * hm->width + ib];
    float t01 = hm->texels[jb * hm->width + ia], t11 = hm->texels[jb * hm->width + ib];
    float g = (1.0f - b) * ((1.0f - a) * t00 + a * t10) + b * ((1.0f - a) * t01 + a * t11);
    r.x = g; r.y = g; r.z = g; r.w = 1.0f;
    return r;
}

static v4 u4(const float* a) { v4 r = {a[0], a[1], a[2], a[3]}; return r; }

/* water-grid.vert:87-91 */
static v4 grid_position(const wto_ref_uniforms* U, v2 uv) {
    v4 m1 = mix4(u4(U->bottom_left), u4(U->bottom_right), uv.x);
    v4 m2 = mix4(u4(U->top_left), u4(U->top_right), uv.x);
    return mix4(m1, m2, uv.y);
}

/* water-grid.vert:74-85 (+ optional constant phase per wave) */
static v3 gerstner(const wto_ref_uniforms* U, v2 xz, float t) {
    v3 P = {xz.x, 0.0f, xz.y};
    for (uint32_t i = 0; i < U->wave_count; ++i) {
        const wto_ref_wave* w = &U->waves[i];
        v2 D = {w->dir_x, w->dir_z};
        float c1 = w->frequency_w * dot2(D, xz) + w->phaseConstant_phi * t;
        if (U->phase_offset) c1 = c1 + U->phase_offset[i];
        float q = w->steepness_Q_i * cosf(c1);
        v3 g = {w->amplitude_A * (D.x * q), w->amplitude_A * sinf(c1), w->amplitude_A * (D.y * q)};
        P.x = P.x + g.x; P.y = P.y + g.y; P.z = P.z + g.z;
    }
    return P;
}

/* water-grid.vert:93-111 */
static v4 sample_heightmap(const wto_ref_uniforms* U, v4 p) {
    v2 st = {U->hm.sample_scale * p.x, U->hm.sample_scale * -p.z};
    return texture2d(&U->hm, st);
}
static float hm_displacement(const wto_ref_uniforms* U, v4 s) {
    float i01 = s.x;
    float i11 = 2.0f * (i01 - 0.5f);
    return U->hm.disp_scale * i11;
}

/* one displaced surface point: grid -> Gerstner -> heightmap -> bounce */
static v4 surface(const wto_ref_uniforms* U, v2 uv, v4* colour) {
    v4 g = grid_position(U, uv);
    v2 xz = {g.x, g.z};
    v3 P = gerstner(U, xz, U->time_s);
    v4 p = {P.x, P.y, P.z, 1.0f};
    v4 c = sample_heightmap(U, p);
    if (colour) *colour = c;
    p.y += hm_displacement(U, c);
    p.y += U->vertical_bounce;
    return p;
}

void wto_reference_vertex(const wto_ref_uniforms* U, uint32_t id0, uint32_t id1,
                          const wto_ref_outputs* out) {
    const uint32_t L = U->grid_length;
    for (uint32_t id = id0; id < id1; ++id) {
        int vid = (int)id; /* gl_VertexID */
        float du = 1.0f / (float)(L - 1);
        float dv = 1.0f / (float)(L - 1);
        v2 uv = {glsl_mod((float)vid, (float)L) * du, (float)((unsigned)vid / L) * dv};
        v4 colour;
        v4 position = surface(U, uv, &colour);
        v4 clip = mat4_mul(U->view_projection, position);
        v4 h0 = {position.x, 0.0f, position.z, 1.0f};
        v4 c0 = mat4_mul(U->view_projection, h0);
        v3 view = {U->camera_position[0] - position.x, U->camera_position[1] - position.y,
                   U->camera_position[2] - position.z};
        v2 uvmu = {uv.x - du, uv.y - 0.0f}, uvpu = {uv.x + du, uv.y + 0.0f};
        v2 uvmv = {uv.x - 0.0f, uv.y - dv}, uvpv = {uv.x + 0.0f, uv.y + dv};
        v4 pmu = surface(U, uvmu, NULL), ppu = surface(U, uvpu, NULL);
        v4 pmv = surface(U, uvmv, NULL), ppv = surface(U, uvpv, NULL);
        v3 e1 = {ppu.x - pmu.x, ppu.y - pmu.y, ppu.z - pmu.z};
        v3 e2 = {ppv.x - pmv.x, ppv.y - pmv.y, ppv.z - pmv.z};
        v3 n = normalize3(cross3(e1, e2));
        if (dot3(n, normalize3(view)) < 0.0f) { n.x *= -1.0f; n.y *= -1.0f; n.z *= -1.0f; }
        v4 n4 = {n.x, n.y, n.z, 0.0f};
        v4 ny4 = mat4_mul(U->view_only_yaw, n4);
        v3 ny3 = {ny4.x, ny4.y, ny4.z};
        v3 nyaw = normalize3(ny3);
        size_t o = id - id0;
        if (out->position) memcpy(out->position + 4 * o, &position, 16);
        if (out->clip) memcpy(out->clip + 4 * o, &clip, 16);
        if (out->ndc0) { out->ndc0[2 * o] = c0.x / c0.w; out->ndc0[2 * o + 1] = c0.y / c0.w; }
        if (out->view) memcpy(out->view + 3 * o, &view, 12);
        if (out->normal) memcpy(out->normal + 3 * o, &n, 12);
        if (out->normal_yaw) memcpy(out->normal_yaw + 3 * o, &nyaw, 12);
        if (out->colour) memcpy(out->colour + 4 * o, &colour, 16);
    }
}

void wto_wave_to_reference(const wt_wave* w, wto_ref_wave* out) {
    double lam = (double)w->wavelength;
    float k = isinf(lam) ? 0.0f : (float)(6.283185307179586476925286766559 / lam);
    out->amplitude_A = w->amplitude;
    out->frequency_w = k;
    out->phaseConstant_phi = w->speed * k;
    out->steepness_Q_i = w->steepness_q;
    out->dir_x = w->dir_x;
    out->dir_z = w->dir_z;
}

/* ---- multi-threaded CPU baseline ---------------------------------------- */

typedef struct job {
    const wt_patch* patches;
    uint32_t n_patches;
    const wt_wave* waves;
    const wto_heightmap* hm;
    uint32_t row_limit;
    uint32_t row_stride, row_phase;  /* rows r = row_phase + k * row_stride, r < row_limit */
    float* pos4;
    float* nrm4;
    int analytic;
    uint64_t* row_start;   /* prefix of rows-to-run per patch */
    uint64_t total_rows;
    atomic_ullong next;
    atomic_ullong verts;
} job;

static const float IDENT[16] = {1, 0, 0, 0, 0, 1, 0, 0, 0, 0, 1, 0, 0, 0, 0, 1};

static void run_row_reference(job* J, uint32_t pi, uint32_t row, wto_ref_wave* rw, float* phase) {
    const wt_patch* p = &J->patches[pi];
    wto_ref_uniforms U;
    memset(&U, 0, sizeof(U));
    float c[4][2] = {{p->bl[0], p->bl[1]}, {p->br[0], p->br[1]}, {p->tl[0], p->tl[1]}, {p->tr[0], p->tr[1]}};
    float* dst[4] = {U.bottom_left, U.bottom_right, U.top_left, U.top_right};
    for (int i = 0; i < 4; ++i) { dst[i][0] = c[i][0]; dst[i][1] = 0.0f; dst[i][2] = c[i][1]; dst[i][3] = 1.0f; }
    U.camera_position[0] = 0.0f; U.camera_position[1] = 1.0e4f; U.camera_position[2] = 0.0f;
    U.grid_length = p->cols;
    U.wave_count = p->wave_count;
    for (uint32_t i = 0; i < p->wave_count; ++i) {
        wto_wave_to_reference(&J->waves[p->wave_offset + i], &rw[i]);
        phase[i] = J->waves[p->wave_offset + i].phase;
    }
    U.waves = rw;
    U.phase_offset = phase;
    if (J->hm) U.hm = *J->hm;
    U.vertical_bounce = p->y_offset;
    U.time_s = (float)p->time_s;
    memcpy(U.view_only_yaw, IDENT, sizeof(IDENT));
    memcpy(U.view_projection, IDENT, sizeof(IDENT));
    uint32_t id0 = row * p->cols, id1 = id0 + p->cols;
    float n3[3 * 4096];
    float* pos = J->pos4 + 4 * (size_t)p->out_offset;
    wto_ref_outputs o;
    memset(&o, 0, sizeof(o));
    for (uint32_t a = id0; a < id1; a += 4096) {
        uint32_t b = a + 4096 < id1 ? a + 4096 : id1;
        o.position = pos + 4 * (size_t)a;
        o.normal = n3;
        wto_reference_vertex(&U, a, b, &o);
        if (J->nrm4)
            for (uint32_t id = a; id < b; ++id) {
                float* d = J->nrm4 + 4 * ((size_t)p->out_offset + id);
                d[0] = n3[3 * (id - a)]; d[1] = n3[3 * (id - a) + 1]; d[2] = n3[3 * (id - a) + 2]; d[3] = 0.0f;
            }
    }
}

/* One FP32 surface evaluation per vertex with the exact normal. */
static void run_row_analytic(job* J, uint32_t pi, uint32_t row, wto_ref_wave* rw, float* phase) {
    const wt_patch* p = &J->patches[pi];
    for (uint32_t i = 0; i < p->wave_count; ++i) {
        wto_wave_to_reference(&J->waves[p->wave_offset + i], &rw[i]);
        phase[i] = J->waves[p->wave_offset + i].phase;
    }
    float t = (float)p->time_s;
    float v = (float)row / (float)(p->rows - 1);
    for (uint32_t col = 0; col < p->cols; ++col) {
        float u = (float)col / (float)(p->cols - 1);
        float x = glsl_mix(glsl_mix(p->bl[0], p->br[0], u), glsl_mix(p->tl[0], p->tr[0], u), v);
        float z = glsl_mix(glsl_mix(p->bl[1], p->br[1], u), glsl_mix(p->tl[1], p->tr[1], u), v);
        float dx = 0, dy = 0, dz = 0, jx = 0, jz = 0, sxx = 0, sxz = 0, szz = 0;
        for (uint32_t i = 0; i < p->wave_count; ++i) {
            const wto_ref_wave* w = &rw[i];
            float th = w->frequency_w * (w->dir_x * x + w->dir_z * z) + w->phaseConstant_phi * t + phase[i];
            float c = cosf(th), s = sinf(th);
            float A = w->amplitude_A, Q = w->steepness_Q_i, k = w->frequency_w;
            dx += Q * A * w->dir_x * c; dy += A * s; dz += Q * A * w->dir_z * c;
            jx += A * k * w->dir_x * c; jz += A * k * w->dir_z * c;
            sxx += Q * A * k * w->dir_x * w->dir_x * s;
            sxz += Q * A * k * w->dir_x * w->dir_z * s;
            szz += Q * A * k * w->dir_z * w->dir_z * s;
        }
        float px[3] = {1.0f - sxx, jx, -sxz}, pz[3] = {-sxz, jz, 1.0f - szz};
        if (J->hm && J->hm->texels) {
            const wto_heightmap* hm = J->hm;
            float su = hm->sample_scale * (x + dx) * (float)hm->width - 0.5f;
            float sv = hm->sample_scale * -(z + dz) * (float)hm->height - 0.5f;
            float fi = floorf(su), fj = floorf(sv), a = su - fi, b = sv - fj;
            int64_t ia = wrap_i((int64_t)fi, hm->width, hm->wrap), ib = wrap_i((int64_t)fi + 1, hm->width, hm->wrap);
            int64_t ja = wrap_i((int64_t)fj, hm->height, hm->wrap), jb = wrap_i((int64_t)fj + 1, hm->height, hm->wrap);
            float t00 = hm->texels[ja * hm->width + ia], t10 = hm->texels[ja * hm->width + ib];
            float t01 = hm->texels[jb * hm->width + ia], t11 = hm->texels[jb * hm->width + ib];
            float r = (1 - b) * ((1 - a) * t00 + a * t10) + b * ((1 - a) * t01 + a * t11);
            float k2 = 2.0f * hm->disp_scale;
            float hx = k2 * ((1 - b) * (t10 - t00) + b * (t11 - t01)) * hm->sample_scale * hm->width;
            float hz = -k2 * ((1 - a) * (t01 - t00) + a * (t11 - t10)) * hm->sample_scale * hm->height;
            dy += k2 * (r - 0.5f);
            px[1] += hx * px[0] + hz * px[2];
            pz[1] += hx * pz[0] + hz * pz[2];
        }
        dy += p->y_offset;
        float n0 = pz[1] * px[2] - pz[2] * px[1], n1 = pz[2] * px[0] - pz[0] * px[2], n2 = pz[0] * px[1] - pz[1] * px[0];
        float inv = 1.0f / sqrtf(n0 * n0 + n1 * n1 + n2 * n2);
        size_t o = (size_t)p->out_offset + (size_t)row * p->cols + col;
        float* P = J->pos4 + 4 * o;
        P[0] = x + dx; P[1] = dy; P[2] = z + dz; P[3] = 1.0f;
        if (J->nrm4) { float* N = J->nrm4 + 4 * o; N[0] = n0 * inv; N[1] = n1 * inv; N[2] = n2 * inv; N[3] = 0.0f; }
    }
}

static void* worker(void* arg) {
    job* J = (job*)arg;
    uint32_t maxw = 0;
    for (uint32_t i = 0; i < J->n_patches; ++i)
        if (J->patches[i].wave_count > maxw) maxw = J->patches[i].wave_count;
    wto_ref_wave* rw = (wto_ref_wave*)malloc(sizeof(wto_ref_wave) * (maxw + 1));
    float* phase = (float*)malloc(sizeof(float) * (maxw + 1));
    for (;;) {
        uint64_t r = atomic_fetch_add(&J->next, 1);
        if (r >= J->total_rows) break;
        /* find patch: row_start is a prefix over patches */
        uint32_t lo = 0, hi = J->n_patches;
        while (hi - lo > 1) {
            uint32_t mid = (lo + hi) / 2;
            if (J->row_start[mid] <= r) lo = mid; else hi = mid;
        }
        uint32_t row = J->row_phase + (uint32_t)(r - J->row_start[lo]) * J->row_stride;
        if (J->analytic) run_row_analytic(J, lo, row, rw, phase);
        else run_row_reference(J, lo, row, rw, phase);
        atomic_fetch_add(&J->verts, J->patches[lo].cols);
    }
    free(rw);
    free(phase);
    return NULL;
}

static uint64_t run_jobs(const wt_patch* patches, uint32_t n_patches, const wt_wave* waves,
                         const wto_heightmap* hm, uint32_t row_limit, uint32_t row_stride, uint32_t row_phase,
                         int threads, float* pos4, float* nrm4, int analytic) {
    if (n_patches == 0 || row_stride == 0) return 0;
    job J;
    memset(&J, 0, sizeof(J));
    J.patches = patches; J.n_patches = n_patches; J.waves = waves; J.hm = hm;
    J.row_limit = row_limit; J.pos4 = pos4; J.nrm4 = nrm4; J.analytic = analytic;
    J.row_stride = row_stride; J.row_phase = row_phase;
    J.row_start = (uint64_t*)malloc(sizeof(uint64_t) * (n_patches + 1));
    uint64_t acc = 0;
    for (uint32_t i = 0; i < n_patches; ++i) {
        J.row_start[i] = acc;
        uint32_t lim = patches[i].rows < row_limit ? patches[i].rows : row_limit;
        acc += lim > row_phase ? (lim - row_phase + row_stride - 1) / row_stride : 0;
    }
    J.row_start[n_patches] = acc;
    J.total_rows = acc;
    atomic_init(&J.next, 0);
    atomic_init(&J.verts, 0);
    if (threads < 1) threads = 1;
    pthread_t* th = (pthread_t*)malloc(sizeof(pthread_t) * threads);
    for (int i = 0; i < threads; ++i) pthread_create(&th[i], NULL, worker, &J);
    for (int i = 0; i < threads; ++i) pthread_join(th[i], NULL);
    free(th);
    free(J.row_start);
    return atomic_load(&J.verts);
}

uint64_t wto_cpu_reference(const wt_patch* patches, uint32_t n_patches, const wt_wave* waves,
                           const wto_heightmap* hm, uint32_t row_limit, int threads,
                           float* pos4, float* nrm4) {
    return run_jobs(patches, n_patches, waves, hm, row_limit, 1, 0, threads, pos4, nrm4, 0);
}

uint64_t wto_cpu_analytic(const wt_patch* patches, uint32_t n_patches, const wt_wave* waves,
                          const wto_heightmap* hm, uint32_t row_limit, int threads,
                          float* pos4, float* nrm4) {
    return run_jobs(patches, n_patches, waves, hm, row_limit, 1, 0, threads, pos4, nrm4, 1);
}

uint64_t wto_cpu_reference_rows(const wt_patch* patches, uint32_t n_patches, const wt_wave* waves,
                                const wto_heightmap* hm, uint32_t row_stride, uint32_t row_phase, int threads,
                                float* pos4, float* nrm4, int analytic) {
    return run_jobs(patches, n_patches, waves, hm, 0xffffffffu, row_stride, row_phase, threads, pos4, nrm4,
                    analytic != 0);
}
