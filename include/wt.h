/*
 * wt.h — C ABI of the GB300-native Gerstner water-surface path.
 *
 * This header replaces the water-grid hot path of wave-tool: the host side in
 * src/render-engine.cpp:1045-1115 (uniform upload + glDrawElements) and the
 * per-vertex work in assets/shaders/water-grid.vert:74-194 (Gerstner sum,
 * heightmap displacement, vertical bounce, normals), plus the projected-grid
 * index buffer built in src/program.cpp:686-717.
 *
 * Conventions
 *  - Plain C: no C++ types, no exceptions, no CUDA headers needed.
 *    `wt_stream` is ABI-identical to cudaStream_t (pass one directly; NULL is
 *    the legacy default stream).
 *  - Every entry point returns a wt_status; wt_last_error() gives a message
 *    for the last failure on the calling thread.
 *  - The caller owns all device memory. Entry points that need scratch take a
 *    caller-provided device `workspace` sized by the matching *_workspace_size
 *    query; nothing allocates inside a launch call, so launch calls can be
 *    captured into a CUDA graph.
 *  - Launch calls are asynchronous on `stream`. Host-side validation errors are
 *    returned immediately; device-side validation of the patch table (which
 *    lives in device memory) is recorded in the workspace and read back with
 *    wt_workspace_status().
 */
#ifndef WT_H
#define WT_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef struct CUstream_st* wt_stream; /* same type as cudaStream_t */

typedef enum wt_status {
    WT_OK = 0,
    WT_ERR_INVALID_ARG = 1,  /* bad pointer, size, alignment or parameter */
    WT_ERR_CUDA = 2,         /* a CUDA runtime call failed (see wt_last_error) */
    WT_ERR_TIMEOUT = 3,      /* reserved: no kernel of this library spins on a flag or on
                                another kernel, so no call returns it */
    WT_ERR_NOMEM = 4,        /* workspace smaller than the size query asked for */
    WT_ERR_UNSUPPORTED = 5   /* a parameter combination this build does not handle */
} wt_status;

/* One Gerstner wave.  Replaces `struct GerstnerWave`
 * (src/render-engine.h:130-167) and the per-wave uniforms
 * (assets/shaders/water-grid.vert:45-51, src/render-engine.cpp:1067-1081).
 *
 *   theta = k * dot(D, xz) + speed * k * t + phase,   k = 2*pi / wavelength
 *   P    += A * (D.x * Q * cos(theta), sin(theta), D.z * Q * cos(theta))
 *
 * `steepness_q` is the per-wave Q_i the shader consumes (the reference divides
 * its user steepness by k*A*count on the host, render-engine.cpp:1073; use
 * wt_wave_from_reference to apply that).  `speed * k` is the reference's
 * phaseConstant_phi; `phase` is an extra constant offset (0 reproduces the
 * reference).  wavelength = +inf means k = 0.  32 bytes, two float4 loads. */
typedef struct wt_wave {
    float amplitude;   /* A >= 0, metres */
    float wavelength;  /* lambda > 0 (or +inf), metres */
    float dir_x;       /* D, a unit xz direction */
    float dir_z;
    float steepness_q; /* Q_i */
    float speed;       /* crest speed, m/s (omega = speed * k) */
    float phase;       /* constant phase offset, radians */
    float _pad;        /* must be 0 */
} wt_wave;

/* One projected-grid patch: a cols x rows vertex grid bilinearly spanning four
 * world-space corners on the y = 0 plane (water-grid.vert:37-38,59-60,87-91).
 * Vertex (row, col) has u = col/(cols-1), v = row/(rows-1); row 0 is the
 * BL-BR edge, matching gl_VertexID = row*cols + col (water-grid.vert:115-125).
 * Its outputs live at vertex index out_offset + row*cols + col. 72 bytes. */
typedef struct wt_patch {
    float bl[2];          /* world (x, z) of the bottom-left corner  (u=0, v=0) */
    float br[2];          /* bottom-right (u=1, v=0) */
    float tl[2];          /* top-left     (u=0, v=1) */
    float tr[2];          /* top-right    (u=1, v=1) */
    uint32_t cols;        /* vertices along u, >= 2 (the reference's gridLength) */
    uint32_t rows;        /* vertices along v, >= 2 */
    uint32_t wave_offset; /* first wave of this patch in the wave array */
    uint32_t wave_count;  /* number of waves (0 allowed) */
    double time_s;        /* wave animation time, seconds (waveAnimationTimeInSeconds) */
    float y_offset;       /* vertical bounce displacement added to y (render-engine.cpp:299-300) */
    uint32_t flags;       /* reserved, must be 0 */
    uint64_t out_offset;  /* first output vertex of this patch */
} wt_patch;

enum { WT_WRAP_REPEAT = 0, WT_WRAP_MIRRORED_REPEAT = 1 };

/* The heightmap-noise layer (water-grid.vert:93-111; sampler state
 * src/texture.cpp:54-71).  Sampled at the Gerstner-displaced position with
 * GL_LINEAR semantics (texel centres at i + 0.5) at texture coordinates
 * sample_scale * (x', -z'); adds disp_scale * 2 * (r - 0.5) to y.
 * `texels` is device memory, R32F, width*height values, texel (i, j) at
 * texels[j*width + i], j = 0 is the t = 0 row.  The struct itself is a host
 * struct passed by pointer. */
typedef struct wt_heightmap {
    const float* texels;
    uint32_t width;
    uint32_t height;
    float sample_scale;   /* heightmapSampleScale */
    float disp_scale;     /* heightmapDisplacementScale */
    uint32_t wrap;        /* WT_WRAP_* */
    uint32_t _pad;
} wt_heightmap;

/* Flags of wt_gerstner_displace / wt_gerstner_adjoint. */
enum {
    WT_OUT_WORLD = 0,           /* pos_out = displaced world position, w = 1 */
    WT_OUT_DISPLACEMENT = 1,    /* pos_out = displaced - undisplaced grid position, w = 0 */
    WT_LAYOUT_FLOAT4 = 0,       /* 16-byte stride per vertex (x, y, z, w) */
    WT_LAYOUT_VEC3 = 2,         /* 12-byte tightly packed vec3 (the reference VAO layout,
                                   render-engine.cpp:1175-1191) */
    WT_PHASE_FP64 = 0,          /* per-wave phase reduced mod 2*pi in FP64 (default) */
    WT_PHASE_FP32_NAIVE = 4     /* the reference's FP32 phase w*dot(D,xz) + phi*t, for
                                   precision studies (water-grid.vert:78) */
};

/* Per-wave gradient of a loss.  d_direction is with respect to the angle of D
 * (D = (cos a, sin a)); d_dir_x / d_dir_z are the raw component gradients. */
typedef struct wt_wave_grad {
    float d_amplitude;
    float d_wavelength;
    float d_direction;
    float d_steepness_q;
    float d_phase;
    float d_speed;
    float d_dir_x;
    float d_dir_z;
} wt_wave_grad;

/* One term of the tileable noise heightmap:
 *   h(i, j) += amplitude * sin(2*pi*(kx*i + ky*j)/size + phase). */
typedef struct wt_noise_term {
    int32_t kx;
    int32_t ky;
    float amplitude;
    float phase;
} wt_noise_term;

/* ---- queries ------------------------------------------------------------ */

const char* wt_version(void);
/* Message for the last failing call on this thread ("" if none). */
const char* wt_last_error(void);

/* Workspace for wt_gerstner_displace over `n_patches` patches whose
 * wave_count values sum to `total_wave_slots`. */
wt_status wt_displace_workspace_size(uint32_t n_patches, uint64_t total_wave_slots,
                                     size_t* bytes);

/* Workspace for wt_gerstner_adjoint.  Takes a HOST copy of the patch table
 * (the per-tile gradient partials depend on every patch's size). */
wt_status wt_adjoint_workspace_size(const wt_patch* host_patches, uint32_t n_patches,
                                    size_t* bytes);

/* Reads back (synchronising `stream`) the device-side validation word that the
 * last launch with this workspace wrote: WT_OK, or WT_ERR_INVALID_ARG with
 * the first offending patch index in *bad_patch (may be NULL). */
wt_status wt_workspace_status(const void* workspace, wt_stream stream, uint32_t* bad_patch);

/* ---- the hot path ------------------------------------------------------- */

/* Gerstner displacement + analytic normals (+ heightmap noise, + bounce) for
 * every vertex of every patch, in one persistent launch.
 * Replaces water-grid.vert:114-194 driven by render-engine.cpp:1045-1115.
 *   patches, waves : device arrays
 *   hm             : host struct (NULL = no heightmap layer)
 *   pos_out        : device, out_capacity vertices, layout per flags
 *   nrm_out        : device or NULL; unit normal oriented +y (w = 0)
 * Normals are the exact normal of the displaced surface,
 * normalize(dP/dz x dP/dx), not the reference's central differences. */
wt_status wt_gerstner_displace(const wt_patch* patches, uint32_t n_patches,
                               const wt_wave* waves, uint32_t n_waves,
                               const wt_heightmap* hm,
                               float* pos_out, float* nrm_out, uint64_t out_capacity,
                               uint32_t flags, void* workspace, size_t workspace_bytes,
                               wt_stream stream);

/* Limits of wt_gerstner_displace_noalloc. */
#define WT_NOALLOC_MAX_PATCHES 1024u
#define WT_NOALLOC_MAX_WAVE_SLOTS 16384u

/* wt_gerstner_displace for callers that cannot allocate device memory: a
 * renderer or engine plugin that runs inside a host application's frame,
 * where the host owns every device buffer and a cudaMalloc (which may
 * synchronise the whole device) would stall the frame, or a caller that only
 * receives ready-made input and output buffers and has no allocator of its
 * own.  The scratch that wt_gerstner_displace takes as `workspace` lives here
 * in a fixed array inside the library (about 1.1 MiB, held on every GPU that
 * loads the library until the process exits); nothing is allocated by this
 * call.  It has no counterpart in the reference.
 *   - n_patches <= WT_NOALLOC_MAX_PATCHES and total_wave_slots (the sum of the
 *     patches' wave_count) <= WT_NOALLOC_MAX_WAVE_SLOTS, else
 *     WT_ERR_INVALID_ARG;
 *   - the first call on a device looks up the array's device address and
 *     keeps it for the life of the process; make that first call before any
 *     stream capture.  A cudaDeviceReset (or anything else that destroys the
 *     device's primary context) reloads the library's device code and may
 *     move the array: do not call this entry point on a device after
 *     resetting it;
 *   - every call on a device shares the one array, so calls that overlap on
 *     the GPU (e.g. on two streams at once) race: order them on one stream;
 *   - the first kernel of each call resets the array's queue and status words,
 *     so no clearing is needed between calls;
 *   - total_wave_slots is checked on the host; when the patches' real sum of
 *     wave_count is larger than the array holds (about 17,000 slots), or a
 *     patch fails the device-side validation, the call still returns WT_OK
 *     and leaves the outputs of the whole table (or of the failing patch)
 *     unwritten; wt_noalloc_status reads that device-side result back. */
wt_status wt_gerstner_displace_noalloc(const wt_patch* patches, uint32_t n_patches,
                                       uint64_t total_wave_slots,
                                       const wt_wave* waves, uint32_t n_waves,
                                       const wt_heightmap* hm,
                                       float* pos_out, float* nrm_out, uint64_t out_capacity,
                                       uint32_t flags, wt_stream stream);

/* wt_workspace_status for the no-alloc entry point: reads back (synchronising
 * `stream`) the validation word that the last wt_gerstner_displace_noalloc
 * call on the current device wrote into the library's array: WT_OK,
 * WT_ERR_NOMEM when the patches' wave slots did not fit it (nothing written),
 * or WT_ERR_INVALID_ARG with the first offending patch in *bad_patch (may be
 * NULL).  Allocates nothing; WT_OK before any call on the device. */
wt_status wt_noalloc_status(wt_stream stream, uint32_t* bad_patch);

/* The same work issued as one launch pair per patch (no batching).  Exists to
 * measure the batched launch against; results are identical. */
wt_status wt_gerstner_displace_unbatched(const wt_patch* host_patches,
                                         const wt_patch* patches, uint32_t n_patches,
                                         const wt_wave* waves, uint32_t n_waves,
                                         const wt_heightmap* hm,
                                         float* pos_out, float* nrm_out,
                                         uint64_t out_capacity, uint32_t flags,
                                         void* workspace, size_t workspace_bytes,
                                         wt_stream stream);

/* Vector-Jacobian product of wt_gerstner_displace: given dL/dpos (per
 * vertex, the layout flag selects float4 or packed vec3; w ignored) and
 * dL/dnrm (same layout, or NULL), writes dL/dwave for every wave (device
 * array grad_out of n_waves; waves no patch uses get zeros; patches that share
 * a wave add up).  The gradient is the same for world and displacement
 * outputs.  `host_patches` is a host copy of the device patch table (the
 * per-tile partial sums are laid out from it; wt_adjoint_workspace_size gives
 * the workspace).  Deterministic: the FP32 partial sums of each run of one or
 * two tiles are summed with Kahan compensation in a fixed order, and the
 * per-wave gradients are formed and added in FP64 in a fixed order.  No
 * reference counterpart (the reference has no derivatives); the forward it
 * differentiates is water-grid.vert:74-111. */
wt_status wt_gerstner_adjoint(const wt_patch* host_patches, const wt_patch* patches, uint32_t n_patches,
                              const wt_wave* waves, uint32_t n_waves,
                              const wt_heightmap* hm,
                              const float* d_pos, const float* d_nrm, uint64_t out_capacity,
                              uint32_t flags, wt_wave_grad* grad_out,
                              void* workspace, size_t workspace_bytes, wt_stream stream);

/* wt_gerstner_displace that also writes each output vertex's eight wave sums
 * (the displacement and surface-Jacobian sums the normal is built from) to
 * sums_out: device, 16-byte aligned, 8 floats per output vertex (32 *
 * out_capacity bytes), vertex v at sums_out[8v .. 8v+7].  With them,
 * wt_gerstner_adjoint_saved skips recomputing the forward, the way an
 * autograd function saves its activations.  No reference counterpart. */
wt_status wt_gerstner_displace_saving(const wt_patch* patches, uint32_t n_patches,
                                      const wt_wave* waves, uint32_t n_waves,
                                      const wt_heightmap* hm,
                                      float* pos_out, float* nrm_out, uint64_t out_capacity,
                                      uint32_t flags, float* sums_out, void* workspace,
                                      size_t workspace_bytes, wt_stream stream);

/* wt_gerstner_adjoint from the sums a wt_gerstner_displace_saving call wrote
 * for the same patches and waves (same arguments otherwise, same gradients up
 * to FP32 rounding: the saved sums come from the forward's own tiling). */
wt_status wt_gerstner_adjoint_saved(const wt_patch* host_patches, const wt_patch* patches, uint32_t n_patches,
                                    const wt_wave* waves, uint32_t n_waves,
                                    const wt_heightmap* hm,
                                    const float* d_pos, const float* d_nrm, uint64_t out_capacity,
                                    uint32_t flags, const float* sums, wt_wave_grad* grad_out,
                                    void* workspace, size_t workspace_bytes, wt_stream stream);

/* The projected-grid triangle list: for each cell (row, col) the triangles
 * (r,c),(r+1,c+1),(r+1,c) and (r,c),(r,c+1),(r+1,c+1), vertex (r,c) =
 * base_vertex + r*cols + c.  6*(cols-1)*(rows-1) uint32 into idx_out (device).
 * Bit-exact with src/program.cpp:686-717 (there cols = rows = 513, base 0). */
wt_status wt_grid_indices(uint32_t cols, uint32_t rows, uint32_t base_vertex,
                          uint32_t* idx_out, wt_stream stream);

/* Tileable noise heightmap: sum of integer-wavenumber sinusoids over a
 * width x height texel grid, then normalised to [0, 1] (min -> 0, max -> 1)
 * so the reference's 2*(r - 0.5) mapping (water-grid.vert:106-111) holds:
 *   h(i, j) = sum_m a_m sin(2 pi (kx_m i / width + ky_m j / height) + phase_m).
 * terms: device array.  workspace: wt_noise_workspace_size bytes (the
 * separable factor tables, 8 bytes per term and texel row / column, and the
 * min / max).  No reference counterpart: the reference loads a fixed PNG
 * (render-engine.cpp:1308-1322). */
wt_status wt_noise_workspace_size(uint32_t n_terms, uint32_t width, uint32_t height, size_t* bytes);
wt_status wt_noise_synth(const wt_noise_term* terms, uint32_t n_terms,
                         uint32_t width, uint32_t height, float* texels_out,
                         void* workspace, size_t workspace_bytes, wt_stream stream);

/* The same heightmap animated in time: term m's phase advances by rates[m]
 * radians per second, phase_m + rates[m] * time_s (FP64, reduced mod 2 pi
 * before the sine), so that calling it every frame with the frame time
 * animates the noise layer (the "animate the heightmap displacement values
 * over time" TODO at water-grid.vert:113).  rates: device array or NULL
 * (static).  Same workspace as wt_noise_synth. */
wt_status wt_noise_synth_animated(const wt_noise_term* terms, uint32_t n_terms, const float* rates,
                                  double time_s, uint32_t width, uint32_t height, float* texels_out,
                                  void* workspace, size_t workspace_bytes, wt_stream stream);

/* ---- frame set-up and the rest of the vertex stage ----------------------- */

/* The reference's fly camera (src/camera.cpp:47-146, src/camera.h) as the
 * projected grid needs it.  forward = (cos yaw cos pitch, sin pitch,
 * sin yaw cos pitch), world up +y, right-handed look-at view, OpenGL
 * perspective with depth in [-1, 1].  The reference's camera starts at
 * yaw -90 (looking along -z), fov 72, near 0.1, far 100, position (0, 4, 70)
 * (src/render-engine.cpp:52, src/render-engine.h:213-215).  80 bytes. */
typedef struct wt_camera {
    double position[3];
    double yaw_deg;        /* taken mod 360 (Camera::setRotation) */
    double pitch_deg;      /* clamped to [-89, 89] (Camera::rotate / setRotation) */
    double fov_deg;        /* vertical field of view, in (0, 180) */
    double aspect;         /* width / height, > 0 */
    double z_near;         /* 0 < z_near < z_far */
    double z_far;
    /* half height of the displaceable slab |y| <= this: the sum of the wave
     * amplitudes + the heightmap displacement scale + the bounce amplitude
     * (DISPLACEABLE_AMPLITUDE, src/render-engine.cpp:803), >= 0 */
    double displaceable_amplitude;
} wt_camera;

enum {
    WT_VIEW_EMPTY = 0,          /* the frustum misses the slab: the reference draws no water */
    WT_VIEW_VISIBLE = 1,
    WT_VIEW_INVALID_CAMERA = 2  /* wt_projected_grid_async only: the device camera failed validation */
};

/* Per-frame uniforms of the vertex stage (water-grid.vert:24-33 and the values
 * src/render-engine.cpp:277-286 derives from the camera).  Matrices are
 * column-major (element (row r, column c) at [4*c + r], OpenGL order).
 * 144 bytes. */
typedef struct wt_view {
    float view_projection[16]; /* clip = M * (x, y, z, 1) */
    float view_only_yaw[16];   /* view matrix of the camera with its pitch set to 0 */
    float camera_position[3];
    uint32_t status;           /* WT_VIEW_* */
} wt_view;

/* The projected grid (src/render-engine.cpp:797-1042, after the projective
 * grid of Johanson 2004): intersects the camera frustum (x and y widened by
 * 1.2) with the slab |y| <= displaceable_amplitude, aims a projector placed
 * at least displaceable_amplitude + 1 above the base plane at a point blended
 * between the camera's bird's-eye and horizon aim points, bounds the
 * intersection points in the projector's NDC, and casts the four corners of
 * that range onto y = 0.  Host only, FP64 throughout (the reference computes
 * in FP32 with GLM).
 *   patch : host; bl, br, tl, tr are written (the rest is left as it is); left
 *           untouched when the view is empty
 *   view  : host or NULL; the camera's view-projection, yaw-only view matrix
 *           and position, rounded to FP32, and the status
 *   status: host or NULL; WT_VIEW_VISIBLE or WT_VIEW_EMPTY
 * The reference's result is undefined where the projector looks straight
 * down (it normalises a zero vector); here the projector pitch is then -89
 * degrees, the clamp the reference applies to every pitch. */
wt_status wt_projected_grid(const wt_camera* camera, wt_patch* patch, wt_view* view, uint32_t* status);

/* The same computation as one single-thread kernel on `stream`, reading the
 * camera from device memory and writing the corners of the device patch and
 * the device wt_view, so a camera -> vertices frame (this, then
 * wt_gerstner_displace, then wt_vertex_stage) can be captured and replayed as
 * one CUDA graph.  An invalid camera gives status WT_VIEW_INVALID_CAMERA and
 * leaves the patch untouched. */
wt_status wt_projected_grid_async(const wt_camera* camera, wt_patch* patch, wt_view* view,
                                  wt_stream stream);

/* The vertex-stage outputs other than position and normal
 * (water-grid.vert:150-158, 190-193), from the displaced world positions and
 * normals wt_gerstner_displace wrote with WT_OUT_WORLD:
 *   clip_out      float4  view_projection * (p, 1)              (gl_Position)
 *   ndc0_out      float2  xy / w of view_projection * (p.x, 0, p.z, 1)
 *                         (xyPositionNDCSpaceHeight0)
 *   view_out      layout  camera_position - p                   (viewVecRaw)
 *   facing_out    layout  the normal, negated where it faces away from the
 *                         camera (dot(n, view) < 0); may be nrm itself
 *   nrm_yaw_out   layout  normalize(view_only_yaw * (n_facing, 0))
 *                         (normalVecInViewSpaceOnlyYaw)
 * Every output may be NULL; nrm may be NULL when facing_out and nrm_yaw_out
 * are.  `layout` (flags: WT_LAYOUT_FLOAT4 or WT_LAYOUT_VEC3) applies to pos,
 * nrm, view_out, facing_out and nrm_yaw_out; float4 outputs get w = 0.
 * view: device (e.g. written by wt_projected_grid_async). */
wt_status wt_vertex_stage(const wt_view* view, const float* pos, const float* nrm, uint64_t n_vertices,
                          uint32_t flags, float* clip_out, float* ndc0_out, float* view_out,
                          float* facing_out, float* nrm_yaw_out, wt_stream stream);

/* Vertex-stage output buffers (device, any may be NULL), as wt_vertex_stage
 * writes them: clip float4, ndc0 float2, view / facing / nrm_yaw float4. */
typedef struct wt_stage_outputs {
    float* clip;
    float* ndc0;
    float* view;
    float* facing;
    float* nrm_yaw;
} wt_stage_outputs;

/* wt_gerstner_displace with wt_vertex_stage fused into its epilogue: each
 * vertex's clip position, NDC at height 0, view vector, camera-facing normal
 * and yaw-only normal (water-grid.vert:150-158, :190-193) are computed from
 * the world position and normal in registers and written straight to
 * `outputs` (float4 / float2 layouts), bit-identical to wt_vertex_stage on
 * the positions and normals wt_gerstner_displace writes.  pos_out and nrm_out
 * may each be NULL (that output is then not written); flags: 0 or
 * WT_LAYOUT_VEC3 (the layout of pos_out / nrm_out only); WT_OUT_DISPLACEMENT and WT_PHASE_FP32_NAIVE are
 * refused.  view: device wt_view (e.g. from wt_projected_grid_async on the
 * same stream). */
wt_status wt_gerstner_displace_stage(const wt_patch* patches, uint32_t n_patches,
                                     const wt_wave* waves, uint32_t n_waves,
                                     const wt_heightmap* hm, const wt_view* view,
                                     float* pos_out, float* nrm_out, uint64_t out_capacity,
                                     uint32_t flags, const wt_stage_outputs* outputs,
                                     void* workspace, size_t workspace_bytes, wt_stream stream);

/* ---- water shading (the fragment stage) ---------------------------------- */

/* Uniforms of the water fragment shader (assets/shaders/water-grid.frag:34-53),
 * with the reference's defaults (src/render-engine.h:221-235,
 * src/render-engine.cpp:288-296, 1061-1111).  72 bytes. */
typedef struct wt_water_shading {
    float sun_position[3];      /* sunPosition: world-space direction towards the sun, (cos a, sin a, 0) */
    float sun_shininess;        /* 50 */
    float sun_strength;         /* 1 */
    float water_clarity;        /* 0.3 */
    float soft_edges_threshold; /* softEdgesDeltaDepthThreshold, 0.05 */
    float tint_threshold;       /* tintDeltaDepthThreshold, 0.1 */
    float fog_colour[4];        /* fogColourFarAtCurrentTime: rgb, a = density at the far radius */
    float fog_radius_near;      /* fogDepthRadiusNear, 0 */
    float fog_radius_far;       /* fogDepthRadiusFar, 1 */
    float z_near;               /* 0.1 */
    float z_far;                /* 100 */
} wt_water_shading;

/* The render targets the water pass samples, at the viewport's size (device
 * memory; row 0 is the bottom row, as GL stores them).  40 bytes. */
typedef struct wt_water_textures {
    const float* scene_depth;          /* depthTexture2D: width*height window depths in [0, 1] of what
                                          was drawn before the water; NULL = cleared (1.0) */
    const uint8_t* local_reflections;  /* localReflectionsTexture2D, width*height RGBA8; NULL = (0,0,0,0) */
    const uint8_t* local_refractions;  /* localRefractionsTexture2D, width*height RGBA8; NULL = (0,0,0,0) */
    const uint8_t* skybox;             /* the sky cube map: 6 faces (+X, -X, +Y, -Y, +Z, -Z) of
                                          skybox_size^2 RGBA8, face row 0 at t = 0 */
    uint32_t skybox_size;
    uint32_t _pad;
} wt_water_textures;

/* Rasterises the grid's triangles (the glDrawElements of
 * src/render-engine.cpp:1120, triangle list from wt_grid_indices) into a
 * visibility buffer: fragments[y*width + x] = (window depth bits << 32) |
 * (triangle + 1) of the nearest water fragment at pixel centre (x+0.5, y+0.5)
 * that passes GL_LESS against scene_depth, or (scene depth bits << 32) | 0
 * where none does.  Vertices are the clip positions wt_vertex_stage wrote
 * (float4).  Window coordinates are snapped to 1/256 pixel and covered
 * with exact integer edge functions (pixel centres on an edge belong to the
 * triangle whose edge is a left or top edge); triangles reaching behind the
 * near plane or far outside the viewport are clipped in clip space first.
 * Ties in depth go to the lower triangle index (the first one drawn, as
 * GL_LESS keeps it).  Independent of launch order: bitwise reproducible.
 * fragments: device, width*height uint64; workspace: device, 16-byte aligned,
 * wt_water_raster_workspace_size bytes. */
wt_status wt_water_raster(const float* clip, uint64_t n_vertices, const uint32_t* indices, uint64_t n_triangles,
                          uint32_t width, uint32_t height, const float* scene_depth, uint64_t* fragments,
                          void* workspace, size_t workspace_bytes, wt_stream stream);

/* Workspace of wt_water_raster: 16 bytes per vertex (each vertex's snapped
 * window coordinates, computed once for the triangles that share it), 16
 * bytes, and 16 bytes per triangle (the queue of triangles with more than 128
 * pixels in their box, or that need clipping, which a second pass rasterises
 * with whole warps).  At most 2^40 vertices and 2^32 - 2 triangles. */
wt_status wt_water_raster_workspace_size(uint64_t n_vertices, uint64_t n_triangles, size_t* bytes);

/* Shades every water pixel of a visibility buffer with the arithmetic of
 * water-grid.frag:65-151: perspective-correct varyings (facing normal, yaw-only
 * normal, view vector, NDC at height 0 from wt_vertex_stage, float4 / float2
 * layouts), sky-box reflection plus sun highlight, Schlick Fresnel, distorted
 * local reflection / refraction look-ups, depth tint, soft edges and fog.
 *   colour_out : device RGBA float per pixel or NULL: the water fragment's
 *                colour (alpha = edge hardness), (0, 0, 0, 0) where no water
 *   composite  : device RGBA float per pixel or NULL: blended over in place with
 *                glBlendFunc(GL_SRC_ALPHA, GL_ONE_MINUS_SRC_ALPHA)
 *                (src/render-engine.cpp:302-303)
 * Pixels whose triangle or vertices lie outside n_triangles / n_vertices are
 * treated as showing no water.
 * shading, textures: host structs (texture pointers are device memory). */
wt_status wt_water_shade(const uint64_t* fragments, const float* clip, uint64_t n_vertices,
                         const uint32_t* indices, uint64_t n_triangles,
                         const float* facing, const float* nrm_yaw, const float* view, const float* ndc0,
                         uint32_t width, uint32_t height, const wt_water_shading* shading,
                         const wt_water_textures* textures, float* colour_out, float* composite,
                         wt_stream stream);

/* Heightmap texels from an 8-bit image already decoded into device memory,
 * as the reference loads its heightmap (src/render-engine.cpp:1308-1322):
 * stbi_load with vertical flip on load, forced to RGBA8, then sampled as a
 * UNORM8 texture whose red channel is used (water-grid.vert:106).
 *   texel (i, j) = pixels[src_row * row_stride_bytes + i * channels] / 255
 * with src_row = height - 1 - j when flip_vertically (the reference's
 * setting), else j: channel 0 is the red of RGB/RGBA pixels and the grey
 * of grey / grey-alpha pixels, which stb's RGBA conversion copies to red.
 * pixels: device, channels in [1, 4]; texels_out: device, width*height floats,
 * ready for wt_heightmap.texels. */
wt_status wt_heightmap_from_unorm8(const uint8_t* pixels, uint32_t width, uint32_t height, uint32_t channels,
                                   uint64_t row_stride_bytes, uint32_t flip_vertically, float* texels_out,
                                   wt_stream stream);

/* ---- reference parameter conversion (host only) ------------------------- */

/* Converts one reference GerstnerWave (render-engine.h:137-141) into a
 * wt_wave, applying the steepness normalisation of render-engine.cpp:1073
 * (Q_i = Q / (w*A*count), 0 when w*A == 0) in the reference's FP32 order.
 * wavelength = 2*pi/w, speed = phi/w, phase = 0.  A reference wave with w = 0
 * and A*phi != 0 (a spatially uniform bob) has no wt_wave form and gives
 * WT_ERR_UNSUPPORTED. */
wt_status wt_wave_from_reference(float amplitude_A, float frequency_w,
                                 float phase_constant_phi, float steepness_Q,
                                 float dir_x, float dir_z, uint32_t wave_count,
                                 wt_wave* out);

/* ---- launch tuning ------------------------------------------------------- */

/* Launch shape of the persistent forward kernel (supported: 8 vertices per
 * lane with 8 or 16 warps and either epilogue, or 20 warps and the register
 * epilogue (the saving and vertex-stage forwards run it as 16); 4 vertices per
 * lane with 8 warps and the register epilogue).  Process-wide; applies to
 * launches issued after it is set.  No reference counterpart (the reference
 * has one fixed draw call). */
typedef struct wt_tuning {
    uint32_t warps_per_block; /* 8, 16 or 20 (0 = 16) */
    uint32_t blocks_per_sm;   /* 0 = as many as fit */
    uint32_t wave_chunk;      /* waves staged per warp at a time: 8, 16 or 32 (0 = 32) */
    uint32_t max_vertices_per_lane; /* widest tile = 32 * this; 4 or 8 (0 = 8).  4 halves
                                       the accumulator registers for more resident warps */
    uint32_t epilogue_in_shared;    /* 1: per-vertex epilogue as one rolled loop over sums
                                       parked in shared memory; 0: unrolled from registers.
                                       The saving and vertex-stage forwards always use 0. */
} wt_tuning;

/* The default shape (used where the autotuner has not run); setting it also
 * drops the autotuned shapes.  NULL restores the built-in default. */
wt_status wt_set_tuning(const wt_tuning* tuning);
wt_status wt_get_tuning(wt_tuning* tuning);

/* Times every candidate launch shape on the given (device-resident) workload
 * (CUDA events on `stream`, synchronising it; after 4 * reps warm-up
 * launches, each candidate's best of three batches of `reps` launches, over
 * two passes; each timed launch follows a clear of pos_out and nrm_out, which
 * evicts the previous launch's lines from L2 when the outputs outsize it,
 * so the shapes are ranked as a launch with cold inputs finds them) and
 * caches the fastest for the workload's shape bucket (the bit lengths of
 * n_patches and n_waves): later wt_gerstner_displace calls in that bucket use
 * it.  Returns it in *best (may be NULL).  Arguments as wt_gerstner_displace;
 * the outputs are overwritten. */
wt_status wt_autotune_displace(const wt_patch* patches, uint32_t n_patches,
                               const wt_wave* waves, uint32_t n_waves,
                               const wt_heightmap* hm,
                               float* pos_out, float* nrm_out, uint64_t out_capacity,
                               uint32_t flags, void* workspace, size_t workspace_bytes,
                               uint32_t reps, wt_tuning* best, wt_stream stream);

/* The same for wt_gerstner_displace_stage (the vertex stage in the
 * displacement's epilogue favours other shapes: on a 1024^2 frame grid 4
 * vertices per lane ran 47 us against 52.5 us for the plain forward's 8).
 * The winner is kept for later wt_gerstner_displace_stage calls in the bucket
 * (which otherwise use the plain forward's shape); wt_set_tuning drops it.
 * Arguments as wt_gerstner_displace_stage; the outputs are overwritten. */
wt_status wt_autotune_displace_stage(const wt_patch* patches, uint32_t n_patches,
                                     const wt_wave* waves, uint32_t n_waves,
                                     const wt_heightmap* hm, const wt_view* view,
                                     float* pos_out, float* nrm_out, uint64_t out_capacity,
                                     uint32_t flags, const wt_stage_outputs* outputs,
                                     void* workspace, size_t workspace_bytes,
                                     uint32_t reps, wt_tuning* best, wt_stream stream);

/* ---- measurement helpers ------------------------------------------------ */

/* Measures this GPU's FP32 FMA rate (FMA/s) and MUFU sine rate (sin/s) with
 * dependent-chain microkernels on `stream`.  scratch: device, >= 4 MiB.
 * Synchronises the stream.  Used for the roofline denominator. */
wt_status wt_measure_peaks(void* scratch, size_t scratch_bytes, double* fma_per_s,
                           double* sin_per_s, wt_stream stream);

#ifdef __cplusplus
}
#endif

#endif /* WT_H */
