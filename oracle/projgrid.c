/*
 * projgrid.c — oracle of the per-frame set-up and of the vertex-stage
 * outputs that follow the displacement.  TEST INFRASTRUCTURE ONLY: loaded by
 * tests/ as the checker of wt_projected_grid, wt_projected_grid_async and
 * wt_vertex_stage; never linked into the library.
 *
 *  - wto_projected_grid_f32: src/render-engine.cpp:797-1042 in FP32, the
 *    reference's precision (reference mode);
 *  - wto_projected_grid_f64: the same statements in FP64 (truth);
 *  - wto_vertex_stage_f64: water-grid.vert:150-158, 190-193 in FP64 on given
 *    positions and normals.
 */
#include <math.h>
#include <stdint.h>
#include <string.h>

#include "wt_oracle.h"

#define REAL float
#define SFX(n) n##_f32
#define R_SIN sinf
#define R_COS cosf
#define R_TAN tanf
#define R_SQRT sqrtf
#define R_ACOS acosf
#define R_FLOOR floorf
#include "projgrid_body.inc"
#undef REAL
#undef SFX
#undef R_SIN
#undef R_COS
#undef R_TAN
#undef R_SQRT
#undef R_ACOS
#undef R_FLOOR

#define REAL double
#define SFX(n) n##_f64
#define R_SIN sin
#define R_COS cos
#define R_TAN tan
#define R_SQRT sqrt
#define R_ACOS acos
#define R_FLOOR floor
#include "projgrid_body.inc"

void wto_vertex_stage_f64(const wt_view* v, const float* pos4, const float* nrm4, uint64_t n, double* clip4,
                          double* ndc2, double* view3, double* facing3, double* nyaw3) {
    const float* M = v->view_projection;
    const float* Y = v->view_only_yaw;
    for (uint64_t i = 0; i < n; ++i) {
        const double p[3] = {pos4[4 * i], pos4[4 * i + 1], pos4[4 * i + 2]};
        /* gl_Position = viewProjection * position (:150) */
        for (int r = 0; r < 4 && clip4; ++r)
            clip4[4 * i + r] = (double)M[r] * p[0] + (double)M[4 + r] * p[1] + (double)M[8 + r] * p[2] + (double)M[12 + r];
        /* :153-154 */
        if (ndc2) {
            double c[4];
            for (int r = 0; r < 4; ++r) c[r] = (double)M[r] * p[0] + (double)M[8 + r] * p[2] + (double)M[12 + r];
            ndc2[2 * i] = c[0] / c[3];
            ndc2[2 * i + 1] = c[1] / c[3];
        }
        /* :158 */
        const double w[3] = {v->camera_position[0] - p[0], v->camera_position[1] - p[1], v->camera_position[2] - p[2]};
        if (view3)
            for (int k = 0; k < 3; ++k) view3[3 * i + k] = w[k];
        if (!facing3 && !nyaw3) continue;
        /* :190 */
        double nv[3] = {nrm4[4 * i], nrm4[4 * i + 1], nrm4[4 * i + 2]};
        const double wl = sqrt(w[0] * w[0] + w[1] * w[1] + w[2] * w[2]);
        if ((nv[0] * w[0] + nv[1] * w[1] + nv[2] * w[2]) / wl < 0.0)
            for (int k = 0; k < 3; ++k) nv[k] = -nv[k];
        if (facing3)
            for (int k = 0; k < 3; ++k) facing3[3 * i + k] = nv[k];
        /* :193 */
        if (nyaw3) {
            double q[3];
            for (int r = 0; r < 3; ++r) q[r] = (double)Y[r] * nv[0] + (double)Y[4 + r] * nv[1] + (double)Y[8 + r] * nv[2];
            const double l = sqrt(q[0] * q[0] + q[1] * q[1] + q[2] * q[2]);
            for (int k = 0; k < 3; ++k) nyaw3[3 * i + k] = q[k] / l;
        }
    }
}
