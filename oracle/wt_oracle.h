/*
 * wt_oracle.h — CPU oracle of the Gerstner water-surface path.
 *
 * TEST INFRASTRUCTURE ONLY.  This is the checker that the CUDA path is
 * compared against; it is never linked into, called by, or used as a fallback
 * for the library under wave-tool_gb300/.  Only tests/, the smoke check and
 * the CPU-baseline leg of bench.py load it.
 *
 * Two restatements of assets/shaders/water-grid.vert (the reference runs this
 * path only as a GLSL vertex shader; it has no CPU implementation):
 *
 *  1. FP64 truth (gerstner_f64.c): the same wave sum in double precision, the
 *     exact normal of the displaced surface, FP64 bilinear sampling of the
 *     stored texels.  The CUDA kernels are held to it.
 *  2. FP32 reference mode (reference_mode.c): a line-by-line FP32 restatement
 *     of water-grid.vert:74-194 (five surface evaluations per vertex,
 *     central-difference normals, camera-facing flip), pinned bit-exactly
 *     against the reference shader source itself compiled as C++ (oracle/_ref,
 *     built by oracle/build_ref.py) and against tests/golden fixtures.
 *
 * Plus the index buffer (src/program.cpp:686-717), the noise heightmap and a
 * hand-derived FP64 adjoint.
 */
#ifndef WT_ORACLE_H
#define WT_ORACLE_H

#include <stdint.h>
#include "../include/wt.h"

#ifdef __cplusplus
extern "C" {
#endif

/* Heightmap as the oracle sees it: host texels, R channel in [0, 1]. */
typedef struct wto_heightmap {
    const float* texels;
    uint32_t width, height;
    float sample_scale, disp_scale;
    uint32_t wrap;
    uint32_t _pad;
} wto_heightmap;

/* ---- FP64 truth ---------------------------------------------------------- */

/* Rows [row0, row1) of one patch.  Any output pointer may be NULL.  Arrays are
 * indexed by the vertex's position inside the patch (row*cols + col):
 *   pos  : 3 doubles, displaced world position (incl. heightmap + y_offset)
 *   disp : 3 doubles, pos - undisplaced grid position (summed directly)
 *   nrm  : 3 doubles, unit normal normalize(dP/dz x dP/dx)
 *   edge : 1 double, distance (in texels) of the heightmap sample point from
 *          the nearest texel-cell boundary (+inf without a heightmap); the
 *          bilinear gradient jumps across those boundaries. */
void wto_displace_f64(const wt_patch* p, const wt_wave* waves, const wto_heightmap* hm,
                      uint32_t row0, uint32_t row1,
                      double* pos, double* disp, double* nrm, double* edge);

/* The same for an explicit list of rows, written compactly (row k of the
 * list at k*cols); any output may be NULL. */
void wto_displace_f64_rows(const wt_patch* p, const wt_wave* waves, const wto_heightmap* hm,
                           const uint32_t* rows, uint32_t n_rows, double* pos, double* disp, double* nrm,
                           double* edge);

/* Undisplaced grid position (x, z) of vertex (row, col), water-grid.vert:87-91
 * and :123-125 in FP64. */
void wto_grid_xz_f64(const wt_patch* p, uint32_t row, uint32_t col, double* x, double* z);

/* ---- FP64 adjoint -------------------------------------------------------- */

/* Gradient of  L = sum_v <gpos_v, pos_v> + <gnrm_v, nrm_v>  with respect to the
 * waves of one patch, accumulated (+=) into grad (8 doubles per wave, the
 * wt_wave_grad field order) for waves [p->wave_offset, +wave_count).
 * gpos: 4 floats per vertex (w ignored); gnrm: 4 floats per vertex or NULL.
 * Indexed like the outputs (p->out_offset + row*cols + col). */
void wto_adjoint_f64(const wt_patch* p, const wt_wave* waves, const wto_heightmap* hm,
                     const float* gpos, const float* gnrm, double* grad);

/* ---- FP32 reference mode ------------------------------------------------- */

/* The shader's own uniform set (water-grid.vert:37-64). */
typedef struct wto_ref_wave {
    float amplitude_A, frequency_w, phaseConstant_phi, steepness_Q_i, dir_x, dir_z;
} wto_ref_wave;

typedef struct wto_ref_uniforms {
    float bottom_left[4], bottom_right[4], top_left[4], top_right[4];
    float camera_position[3];
    uint32_t grid_length;
    uint32_t wave_count;          /* <= number of entries in `waves` */
    const wto_ref_wave* waves;
    const float* phase_offset;    /* NULL, or one constant phase per wave (an
                                     extension; NULL reproduces the shader) */
    wto_heightmap hm;             /* hm.texels NULL: texture reads return 0 */
    float vertical_bounce;
    float time_s;
    float view_only_yaw[16];      /* column-major, as glUniformMatrix4fv(GL_FALSE) */
    float view_projection[16];
} wto_ref_uniforms;

/* Per-vertex outputs of water-grid.vert, any may be NULL:
 *   position (4): world position after displacement (the `position` local)
 *   clip (4): gl_Position;  ndc0 (2): xyPositionNDCSpaceHeight0
 *   view (3): viewVecRaw;   normal (3): `normal` after the camera flip
 *   normal_yaw (3): normalVecInViewSpaceOnlyYaw;  colour (4): heightmap_colour */
typedef struct wto_ref_outputs {
    float* position;
    float* clip;
    float* ndc0;
    float* view;
    float* normal;
    float* normal_yaw;
    float* colour;
} wto_ref_outputs;

/* Runs the vertex stage for gl_VertexID in [id0, id1); outputs of vertex id
 * are written at index id - id0. */
void wto_reference_vertex(const wto_ref_uniforms* u, uint32_t id0, uint32_t id1,
                          const wto_ref_outputs* out);

/* ---- CPU baseline (timed, multi-threaded) -------------------------------- */

/* Runs the FP32 reference-mode vertex stage (5 surface evaluations per vertex,
 * finite-difference normals) over rows [0, row_limit) of every patch, with
 * `threads` POSIX threads, writing float4 positions and normals at the
 * patches' out_offset.  Returns the number of vertices processed. */
uint64_t wto_cpu_reference(const wt_patch* patches, uint32_t n_patches, const wt_wave* waves,
                           const wto_heightmap* hm, uint32_t row_limit, int threads,
                           float* pos4, float* nrm4);

/* Same vertices, one FP32 surface evaluation per vertex with analytic normals. */
uint64_t wto_cpu_analytic(const wt_patch* patches, uint32_t n_patches, const wt_wave* waves,
                          const wto_heightmap* hm, uint32_t row_limit, int threads,
                          float* pos4, float* nrm4);

/* Either form over the rows r = row_phase + k * row_stride of every patch (a
 * sample spread evenly over each patch; the row_stride phases together cover
 * the whole table). */
uint64_t wto_cpu_reference_rows(const wt_patch* patches, uint32_t n_patches, const wt_wave* waves,
                                const wto_heightmap* hm, uint32_t row_stride, uint32_t row_phase, int threads,
                                float* pos4, float* nrm4, int analytic);

/* Maps one wt_wave of a patch to the shader's uniforms: frequency_w =
 * 2*pi/lambda, phaseConstant_phi = speed * frequency_w (FP32). */
void wto_wave_to_reference(const wt_wave* w, wto_ref_wave* out);

/* ---- index buffer, noise ------------------------------------------------- */

/* src/program.cpp:686-717 generalised to cols x rows and a base vertex. */
void wto_grid_indices(uint32_t cols, uint32_t rows, uint32_t base_vertex, uint32_t* out);

/* FP64 noise heightmap normalised to [0, 1]; the _at form with per-term phase
 * rates (radians per second, NULL = none) at time_s. */
void wto_noise_f64_at(const wt_noise_term* terms, uint32_t n_terms, const float* rates, double time_s,
                      uint32_t width, uint32_t height, double* out);
void wto_noise_f64(const wt_noise_term* terms, uint32_t n_terms, uint32_t width,
                   uint32_t height, double* out);


/* ---- per-frame set-up and the rest of the vertex stage (projgrid.c) ------ */

/* src/render-engine.cpp:797-1042 for one camera: corners (x, z) in the order
 * BL, BR, TL, TR; the camera's view-projection and yaw-only view matrices
 * (column-major); the number of frustum points inside the slab.  Returns 1
 * (visible), 0 (the frustum misses the slab) or -1 (a corner ray parallel to
 * the base plane). */
int wto_projected_grid_f32(const wt_camera* cam, float corners[4][2], float vp[16], float view_yaw[16],
                           uint32_t* n_points);
int wto_projected_grid_f64(const wt_camera* cam, double corners[4][2], double vp[16], double view_yaw[16],
                           uint32_t* n_points);

/* water-grid.vert:150-158, 190-193 in FP64 on float4 positions and normals;
 * outputs may be NULL: clip (4), ndc0 (2), view (3), facing normal (3),
 * yaw-only view-space normal (3) doubles per vertex. */
void wto_vertex_stage_f64(const wt_view* v, const float* pos4, const float* nrm4, uint64_t n, double* clip4,
                          double* ndc2, double* view3, double* facing3, double* nyaw3);


/* ---- the water fragment stage (water.c) ---------------------------------- */

/* Inputs of one fragment of water-grid.frag: gl_FragCoord and the varyings. */
typedef struct wto_frag_in {
    float frag_coord[4];  /* window x, y (pixel centre), depth z, 1/w (unused) */
    float normal[3];
    float normal_yaw[3];
    float view[3];
    float ndc0[2];
} wto_frag_in;

/* Its uniforms: the shading parameters, the textures (host memory here) and
 * the viewport size. */
typedef struct wto_frag_uniforms {
    wt_water_shading s;
    wt_water_textures tex;
    uint32_t width, height;
} wto_frag_uniforms;

/* water-grid.frag:65-151 for n fragments -> RGBA colour (FP32 restatement). */
void wto_water_fragment(const wto_frag_uniforms* u, const wto_frag_in* f, uint64_t n, float* colour4);

/* The rasteriser of wt_water_raster, restated: fragments[width*height]. */
void wto_water_raster(const float* clip4, uint64_t n_vertices, const uint32_t* idx, uint64_t n_triangles,
                      uint32_t width, uint32_t height, const float* scene_depth, uint64_t* fragments);

/* wt_water_shade restated: perspective-correct varyings of each pixel's
 * fragment, then wto_water_fragment; colour_out / composite as there (either
 * may be NULL).  Vertex arrays are float4 (ndc0: float2). */
void wto_water_shade(const uint64_t* fragments, const float* clip4, const uint32_t* idx, const float* facing4,
                     const float* nyaw4, const float* view4, const float* ndc0, const wto_frag_uniforms* u,
                     float* colour_out, float* composite);

#ifdef __cplusplus
}
#endif

#endif
