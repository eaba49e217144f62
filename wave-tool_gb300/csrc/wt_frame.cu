// wt_frame.cu — per-frame set-up of the projected grid, and the vertex-stage
// outputs that follow the displacement.
//
// The projected grid restates src/render-engine.cpp:797-1042 in FP64 as a
// set of __host__ __device__ steps: wt_projected_grid runs them one after
// another on the host, wt_projected_grid_async spreads them over one warp of
// a kernel that reads the camera from device memory, so that camera ->
// corners -> displaced vertices is one stream of kernels a CUDA graph can
// replay with a new camera every frame.
//
// k_vertex_stage computes the rest of water-grid.vert's outputs
// (:150-158, :190-193) from the displaced positions and exact normals: a
// streaming, HBM-bound kernel (reads 2 x 16 B, writes up to 72 B per vertex).
#include <cuda_runtime.h>

#include <atomic>
#include <cmath>
#include <cstdio>
#include <cstring>

#include "wt_nvtx.h"
#include "wt_internal.h"
#include "wt_stage.cuh"

namespace {

using wt::StageOut;

#define WT_HD __host__ __device__ inline


// Constants of the reference's projected grid (src/render-engine.cpp).
constexpr double kFrustumPad = 1.2;          // SAFETY_PADDING_SCALAR, :826
constexpr double kProjectorElevation = 1.0;  // PROJECTOR_ELEVATION_FROM_CAMERA, :915
constexpr double kHorizonEpsilon = 0.001;    // SAFE_EPSILON, :925
constexpr double kPitchLimit = 89.0;         // Camera::setRotation clamp, src/camera.cpp:100

struct D3 {
    double x, y, z;
};
WT_HD D3 operator+(D3 a, D3 b) { return {a.x + b.x, a.y + b.y, a.z + b.z}; }
WT_HD D3 operator-(D3 a, D3 b) { return {a.x - b.x, a.y - b.y, a.z - b.z}; }
WT_HD D3 operator*(double s, D3 a) { return {s * a.x, s * a.y, s * a.z}; }
WT_HD double dot(D3 a, D3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
WT_HD D3 cross(D3 a, D3 b) { return {a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x}; }
WT_HD D3 unit(D3 a) { return (1.0 / sqrt(dot(a, a))) * a; }

// 4x4 matrix in OpenGL (column-major) order: m[c][r] is row r of column c.
struct M4 {
    double m[4][4];
};

WT_HD M4 identity() {
    M4 r;
    for (int c = 0; c < 4; ++c)
        for (int k = 0; k < 4; ++k) r.m[c][k] = (c == k) ? 1.0 : 0.0;
    return r;
}

WT_HD M4 mul(const M4& a, const M4& b) {
    M4 r;
    for (int c = 0; c < 4; ++c)
        for (int k = 0; k < 4; ++k) {
            double s = 0.0;
            for (int j = 0; j < 4; ++j) s += a.m[j][k] * b.m[c][j];
            r.m[c][k] = s;
        }
    return r;
}

// The camera's basis (Camera::updateBasisVectors, src/camera.cpp:130-137)
// for a yaw given by its cosine and sine: pitch clamped, world up +y.  The
// right vector normalize(cross(forward, +y)) is (-sin yaw, 0, cos yaw) for
// every pitch.
struct Basis {
    D3 pos, fwd, right, up;
};

// sin and cos of pi * x (exact argument reduction on the device).
WT_HD void sincos_pi(double x, double* s, double* c) {
#ifdef __CUDA_ARCH__
    sincospi(x, s, c);
#else
    sincos(x * 3.14159265358979323846, s, c);
#endif
}

// cos(89 degrees), the smallest cosine of a clamped pitch
WT_HD double cos89() { return 0.017452406437283512819; }

WT_HD Basis camera_basis(D3 pos, double cy, double sy, double sp, double cp) {
    Basis b;
    b.pos = pos;
    b.fwd = unit(D3{cy * cp, sp, sy * cp});
    b.right = D3{-sy, 0.0, cy};
    b.up = unit(cross(b.right, b.fwd));
    return b;
}

// Right-handed look-at along the basis' forward vector (glm::lookAt, whose
// side vector normalize(cross(forward, up)) is the basis' right vector).
WT_HD M4 view_matrix(const Basis& b) {
    const D3 s = b.right, u = b.up;
    M4 v = identity();
    v.m[0][0] = s.x; v.m[1][0] = s.y; v.m[2][0] = s.z; v.m[3][0] = -dot(s, b.pos);
    v.m[0][1] = u.x; v.m[1][1] = u.y; v.m[2][1] = u.z; v.m[3][1] = -dot(u, b.pos);
    v.m[0][2] = -b.fwd.x; v.m[1][2] = -b.fwd.y; v.m[2][2] = -b.fwd.z; v.m[3][2] = dot(b.fwd, b.pos);
    return v;
}

// OpenGL perspective, depth mapped to [-1, 1] (glm::perspective).
WT_HD M4 perspective(double tan_half_fov, double aspect, double zn, double zf) {
    const double f = 1.0 / tan_half_fov;
    M4 p;
    for (int c = 0; c < 4; ++c)
        for (int k = 0; k < 4; ++k) p.m[c][k] = 0.0;
    p.m[0][0] = f / aspect;
    p.m[1][1] = f;
    p.m[2][2] = -(zf + zn) / (zf - zn);
    p.m[2][3] = -1.0;
    p.m[3][2] = -2.0 * zf * zn / (zf - zn);
    return p;
}

WT_HD bool camera_ok(const wt_camera& c) {
    const double v[10] = {c.position[0], c.position[1], c.position[2], c.yaw_deg, c.pitch_deg,
                          c.fov_deg, c.aspect, c.z_near, c.z_far, c.displaceable_amplitude};
    for (double x : v)
        if (!isfinite(x)) return false;
    return c.fov_deg > 0.0 && c.fov_deg < 180.0 && c.aspect > 0.0 && c.z_near > 0.0 && c.z_far > c.z_near &&
           c.displaceable_amplitude >= 0.0;
}

struct Grid {
    double corner[4][2];  // world (x, z) of BL, BR, TL, TR
    M4 view_projection, view_only_yaw;
    bool visible;
};

// What the per-item steps of the projected grid need: the camera and
// projector bases and the frustum's tangents.
struct Frame {
    double amp, tx, ty, itx, ity, z_near, z_far;
    Basis cam, pj;
};

// src/render-engine.cpp:897-984 from the sines and cosines of the yaw, the
// clamped pitch and half the field of view.  NDC (X, Y) at view depth d is
// pos + d * (X*tx*right + Y*ty*up + fwd), tx = tan(fov/2) * aspect,
// ty = tan(fov/2): the view-projection inverses the reference forms with
// glm::inverse are used in this closed form.
WT_HD void frame_setup(const wt_camera& c, double sy, double cy, double sp, double cp, double sf, double cf,
                       Frame* f) {
    f->amp = c.displaceable_amplitude;
    f->z_near = c.z_near;
    f->z_far = c.z_far;
    const D3 eye{c.position[0], c.position[1], c.position[2]};
    f->cam = camera_basis(eye, cy, sy, sp, cp);
    f->ty = sf / cf;
    f->tx = f->ty * c.aspect;
    f->itx = 1.0 / f->tx;
    f->ity = 1.0 / f->ty;
    // the projector: the camera raised out of the slab and pitched down at
    // an aim point blended between the bird's-eye and horizon aims
    const bool underwater = eye.y < 0.0;
    const double min_height = f->amp + kProjectorElevation;
    D3 ppos = eye;
    if (eye.y < min_height) ppos.y = underwater ? min_height - eye.y : min_height;
    D3 fs = f->cam.fwd;
    if (fabs(fs.y) < kHorizonEpsilon) fs.y = (fs.y >= 0.0) ? kHorizonEpsilon : -kHorizonEpsilon;
    const bool looking_down = fs.y < 0.0;
    const D3 ray = (looking_down != underwater) ? fs : D3{fs.x, -fs.y, fs.z};
    const D3 aim1 = eye + (-eye.y / ray.y) * ray;
    D3 aim2 = eye + f->cam.fwd;
    aim2.y = 0.0;
    const double a = fabs(fs.y);
    const D3 aim = (1.0 - a) * aim2 + a * aim1;
    const D3 d = aim - ppos;
    // pitched down by the angle of d below the horizon (the reference's
    // -acos(normalize(d) . normalize(d.x, 0, d.z))), clamped at 89 degrees:
    // its sine and cosine come straight from d
    const double hz = sqrt(d.x * d.x + d.z * d.z), r = sqrt(hz * hz + d.y * d.y);
    double psp = -fabs(d.y) / r, pcp = hz / r;
    if (!(pcp >= cos89())) sincos_pi(-kPitchLimit / 180.0, &psp, &pcp);
    f->pj = camera_basis(ppos, cy, sy, psp, pcp);
}

// Frustum corner i with NDC x and y widened (:815-838); bit 2 = right,
// bit 1 = top, bit 0 = far.
WT_HD D3 frustum_corner(const Frame& f, int i) {
    const double depth = (i & 1) ? f.z_far : f.z_near;
    const double X = ((i & 4) ? kFrustumPad : -kFrustumPad) * f.tx * depth;
    const double Y = ((i & 2) ? kFrustumPad : -kFrustumPad) * f.ty * depth;
    return f.cam.pos + X * f.cam.right + Y * f.cam.up + depth * f.cam.fwd;
}

// The 12 frustum edges (corner pairs differing in one bit).
WT_HD int edge_end(int e, int which) {
    const int a = e < 3 ? 0 : e < 5 ? 1 : e < 7 ? 2 : e < 8 ? 3 : e < 10 ? 4 : e < 11 ? 5 : 6;
    const int bit[12] = {1, 2, 4, 2, 4, 1, 4, 4, 1, 2, 2, 1};
    return which ? (a | bit[e]) : a;
}

// Where edge (e0, e1) crosses the planes y = +-amp (:857-883): 0 to 2 points.
WT_HD int edge_points(const Frame& f, D3 e0, D3 e1, double px[2], double pz[2]) {
    if (e0.y == e1.y) return 0;  // parallel to the planes: no single crossing
    const double lo = fmin(e0.y, e1.y), hi = fmax(e0.y, e1.y);
    int n = 0;
    for (int sgn = 0; sgn < 2; ++sgn) {
        const double h = sgn ? -f.amp : f.amp;
        if (lo <= h && h <= hi) {
            const double t = (h - e0.y) / (e1.y - e0.y);
            px[n] = e0.x + t * (e1.x - e0.x);
            pz[n] = e0.z + t * (e1.z - e0.z);
            ++n;
        }
    }
    return n;
}

// NDC of the base-plane point (px, 0, pz) in the projector (:993-1005).
WT_HD void projector_ndc(const Frame& f, double px, double pz, double* X, double* Y) {
    const D3 q = D3{px, 0.0, pz} - f.pj.pos;
    const double iw = 1.0 / dot(f.pj.fwd, q);
    *X = dot(f.pj.right, q) * f.itx * iw;
    *Y = dot(f.pj.up, q) * f.ity * iw;
}

// The projector's ray through NDC (X, Y) cast onto y = 0 (:1007-1036).
WT_HD bool corner_ray(const Frame& f, double X, double Y, double* cx, double* cz) {
    const D3 dir = (X * f.tx) * f.pj.right + (Y * f.ty) * f.pj.up + f.pj.fwd;
    if (dir.y == 0.0) return false;
    const double t = -f.pj.pos.y / dir.y;
    *cx = f.pj.pos.x + t * dir.x;
    *cz = f.pj.pos.z + t * dir.z;
    return isfinite(*cx) && isfinite(*cz);
}

WT_HD void view_matrices(const wt_camera& c, const Frame& f, double sy, double cy, M4* vp, M4* yaw) {
    *vp = mul(perspective(f.ty, c.aspect, c.z_near, c.z_far), view_matrix(f.cam));
    *yaw = view_matrix(Basis{f.cam.pos, D3{cy, 0.0, sy}, D3{-sy, 0.0, cy}, D3{0.0, 1.0, 0.0}});
}

WT_HD void camera_trig(const wt_camera& c, int which, double* s, double* co) {
    if (which == 0) sincos_pi((c.yaw_deg - 360.0 * floor(c.yaw_deg / 360.0)) / 180.0, s, co);
    else if (which == 1) sincos_pi(fmin(fmax(c.pitch_deg, -kPitchLimit), kPitchLimit) / 180.0, s, co);
    else sincos_pi(c.fov_deg / 360.0, s, co);
}

// src/render-engine.cpp:797-1042, one step after another (host).  The slab
// points only enter through their x and z (they are flattened onto y = 0
// before projection, :989-991) and only through the bounds of their
// projector NDC, so they are bounded as they are found.
inline void projected_grid(const wt_camera& c, Grid* g) {
    double t[6];
    for (int k = 0; k < 3; ++k) camera_trig(c, k, &t[2 * k], &t[2 * k + 1]);
    Frame f;
    frame_setup(c, t[0], t[1], t[2], t[3], t[4], t[5], &f);
    view_matrices(c, f, t[0], t[1], &g->view_projection, &g->view_only_yaw);
    g->visible = false;
    D3 fc[8];
    for (int i = 0; i < 8; ++i) fc[i] = frustum_corner(f, i);
    double x0 = 0.0, x1 = 0.0, y0 = 0.0, y1 = 0.0;
    bool any = false;
    auto add = [&](double px, double pz) {
        double X, Y;
        projector_ndc(f, px, pz, &X, &Y);
        x0 = any ? fmin(x0, X) : X;
        x1 = any ? fmax(x1, X) : X;
        y0 = any ? fmin(y0, Y) : Y;
        y1 = any ? fmax(y1, Y) : Y;
        any = true;
    };
    for (int e = 0; e < 12; ++e) {
        double px[2], pz[2];
        const int n = edge_points(f, fc[edge_end(e, 0)], fc[edge_end(e, 1)], px, pz);
        for (int k = 0; k < n; ++k) add(px[k], pz[k]);
    }
    for (int i = 0; i < 8; ++i)
        if (-f.amp <= fc[i].y && fc[i].y <= f.amp) add(fc[i].x, fc[i].z);
    if (!any) return;
    for (int k = 0; k < 4; ++k)
        if (!corner_ray(f, (k & 1) ? x1 : x0, (k & 2) ? y1 : y0, &g->corner[k][0], &g->corner[k][1])) return;
    g->visible = true;
}

WT_HD void store_result(const wt_camera& c, const Grid& g, wt_patch* patch, wt_view* view) {
    if (view) {
        for (int col = 0; col < 4; ++col)
            for (int r = 0; r < 4; ++r) {
                view->view_projection[4 * col + r] = (float)g.view_projection.m[col][r];
                view->view_only_yaw[4 * col + r] = (float)g.view_only_yaw.m[col][r];
            }
        for (int k = 0; k < 3; ++k) view->camera_position[k] = (float)c.position[k];
        view->status = g.visible ? WT_VIEW_VISIBLE : WT_VIEW_EMPTY;
    }
    if (patch && g.visible) {
        float* dst[4] = {patch->bl, patch->br, patch->tl, patch->tr};
        for (int k = 0; k < 4; ++k) {
            dst[k][0] = (float)g.corner[k][0];
            dst[k][1] = (float)g.corner[k][1];
        }
    }
}

__device__ __forceinline__ D3 shfl_d3(D3 v, int src) {
    return D3{__shfl_sync(0xffffffffu, v.x, src), __shfl_sync(0xffffffffu, v.y, src),
              __shfl_sync(0xffffffffu, v.z, src)};
}

// The same steps spread over one warp: three lanes take the trigonometry,
// eight the frustum corners, twelve the edges and eight the corners inside
// the slab, the NDC bounds are reduced across lanes, four lanes cast the grid
// corners and sixteen write the matrices.  A single thread on GB300's FP64
// pipe spends most of its time in dependent-instruction latency.
__global__ void __launch_bounds__(32) k_projected_grid(const wt_camera* __restrict__ camera, wt_patch* patch,
                                                       wt_view* view) {
    const int lane = threadIdx.x;
    const wt_camera c = *camera;
    if (!camera_ok(c)) {
        if (lane == 0) view->status = WT_VIEW_INVALID_CAMERA;
        return;
    }
    // lanes 0-2: camera_trig(c, lane) with one shared instruction stream (a
    // warp-wide FP64 operation costs ~64 cycles and a division ~550 on
    // GB300; three divergent branches ran three sines and cosines one after
    // another): each lane selects its own numerator and denominator
    double ts = 0.0, tc = 1.0;
    if (lane < 3) {
        const double yaw = c.yaw_deg - 360.0 * floor(c.yaw_deg / 360.0);
        const double pitch = fmin(fmax(c.pitch_deg, -kPitchLimit), kPitchLimit);
        const double num = lane == 0 ? yaw : (lane == 1 ? pitch : c.fov_deg);
        sincos_pi(num / (lane == 2 ? 360.0 : 180.0), &ts, &tc);
    }
    const double sy = __shfl_sync(0xffffffffu, ts, 0), cy = __shfl_sync(0xffffffffu, tc, 0);
    const double sp = __shfl_sync(0xffffffffu, ts, 1), cp = __shfl_sync(0xffffffffu, tc, 1);
    const double sf = __shfl_sync(0xffffffffu, ts, 2), cf = __shfl_sync(0xffffffffu, tc, 2);
    Frame f;
    frame_setup(c, sy, cy, sp, cp, sf, cf, &f);

    const D3 mine = frustum_corner(f, lane & 7);
    const int e = lane < 12 ? lane : 0;
    const D3 ea = shfl_d3(mine, edge_end(e, 0)), eb = shfl_d3(mine, edge_end(e, 1));
    const D3 corner = shfl_d3(mine, (lane >= 12 && lane < 20) ? lane - 12 : 0);
    double px[2], pz[2];
    int n = 0;
    if (lane < 12) {
        n = edge_points(f, ea, eb, px, pz);
    } else if (lane < 20 && -f.amp <= corner.y && corner.y <= f.amp) {
        px[0] = corner.x;
        pz[0] = corner.z;
        n = 1;
    }
    double x0 = INFINITY, x1 = -INFINITY, y0 = INFINITY, y1 = -INFINITY;
    for (int k = 0; k < n; ++k) {
        double X, Y;
        projector_ndc(f, px[k], pz[k], &X, &Y);
        x0 = fmin(x0, X);
        x1 = fmax(x1, X);
        y0 = fmin(y0, Y);
        y1 = fmax(y1, Y);
    }
    const bool any = __ballot_sync(0xffffffffu, n > 0) != 0;
    for (int o = 16; o > 0; o >>= 1) {
        x0 = fmin(x0, __shfl_xor_sync(0xffffffffu, x0, o));
        x1 = fmax(x1, __shfl_xor_sync(0xffffffffu, x1, o));
        y0 = fmin(y0, __shfl_xor_sync(0xffffffffu, y0, o));
        y1 = fmax(y1, __shfl_xor_sync(0xffffffffu, y1, o));
    }
    double gx = 0.0, gz = 0.0;
    const bool ok = lane < 4 && any && corner_ray(f, (lane & 1) ? x1 : x0, (lane & 2) ? y1 : y0, &gx, &gz);
    const bool visible = (__ballot_sync(0xffffffffu, ok) & 0xfu) == 0xfu;
    if (lane < 16) {
        // view_matrices, one element per lane: the two factors of the
        // view-projection in full (cheap), then this lane's element of
        // their product in mul's order
        const M4 P = perspective(f.ty, c.aspect, c.z_near, c.z_far), V = view_matrix(f.cam);
        const M4 yaw = view_matrix(Basis{f.cam.pos, D3{cy, 0.0, sy}, D3{-sy, 0.0, cy}, D3{0.0, 1.0, 0.0}});
        const int col = lane >> 2, row = lane & 3;
        double e = 0.0;
        for (int j = 0; j < 4; ++j) e += P.m[j][row] * V.m[col][j];
        view->view_projection[lane] = (float)e;
        view->view_only_yaw[lane] = (float)yaw.m[col][row];
    }
    if (lane < 3) view->camera_position[lane] = (float)c.position[lane];
    if (lane == 0) view->status = visible ? WT_VIEW_VISIBLE : WT_VIEW_EMPTY;
    if (visible && lane < 4) {
        float* dst = lane == 0 ? patch->bl : lane == 1 ? patch->br : lane == 2 ? patch->tl : patch->tr;
        dst[0] = (float)gx;
        dst[1] = (float)gz;
    }
}

// ---- vertex-stage outputs ---------------------------------------------------

constexpr int kStageThreads = 256;

// One vertex per thread per iteration of a grid-stride loop.  The 36 floats
// of wt_view are staged once per block in shared memory.
template <bool VEC3>
__global__ void __launch_bounds__(kStageThreads) k_vertex_stage(const wt_view* __restrict__ view, const float* pos,
                                                                 const float* nrm, uint64_t n, StageOut o) {
    __shared__ float u[36];
    if (threadIdx.x < 36) u[threadIdx.x] = reinterpret_cast<const float*>(view)[threadIdx.x];
    __syncthreads();
    const uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
    const bool need_n = o.facing || o.nyaw;
    for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += stride) {
        const float3 p = wt::dev::load3<VEC3>(pos, i);
        const float3 nv = need_n ? wt::dev::load3<VEC3>(nrm, i) : make_float3(0.0f, 0.0f, 0.0f);
        wt::dev::stage_vertex<VEC3>(u, p, nv, i, o);
    }
}

wt_status fail(wt_status s, const char* msg) {
    wt::set_last_error(msg);
    return s;
}

wt_status cuda_fail(cudaError_t e, const char* what) {
    char buf[256];
    snprintf(buf, sizeof(buf), "%s: %s (%s)", what, cudaGetErrorName(e), cudaGetErrorString(e));
    wt::set_last_error(buf);
    return WT_ERR_CUDA;
}

bool aligned(const void* p, size_t a) { return (reinterpret_cast<uintptr_t>(p) % a) == 0; }

std::atomic<int> g_stage_blocks[64];  // blocks per launch of the vertex stage, per device

}  // namespace

extern "C" wt_status wt_projected_grid(const wt_camera* camera, wt_patch* patch, wt_view* view, uint32_t* status) {
    if (!camera) return fail(WT_ERR_INVALID_ARG, "wt_projected_grid: camera is NULL");
    if (!camera_ok(*camera))
        return fail(WT_ERR_INVALID_ARG,
                    "wt_projected_grid: camera needs finite values, 0 < fov < 180, aspect > 0, "
                    "0 < z_near < z_far, displaceable_amplitude >= 0");
    Grid g;
    projected_grid(*camera, &g);
    store_result(*camera, g, patch, view);
    if (status) *status = g.visible ? WT_VIEW_VISIBLE : WT_VIEW_EMPTY;
    return WT_OK;
}

extern "C" wt_status wt_projected_grid_async(const wt_camera* camera, wt_patch* patch, wt_view* view,
                                             wt_stream stream) {
    WT_NVTX_RANGE("wt_projected_grid_async");
    if (!camera || !aligned(camera, 8)) return fail(WT_ERR_INVALID_ARG, "wt_projected_grid_async: camera NULL or misaligned");
    if (!patch || !aligned(patch, 8)) return fail(WT_ERR_INVALID_ARG, "wt_projected_grid_async: patch NULL or misaligned");
    if (!view || !aligned(view, 4)) return fail(WT_ERR_INVALID_ARG, "wt_projected_grid_async: view NULL or misaligned");
    k_projected_grid<<<1, 32, 0, (cudaStream_t)stream>>>(camera, patch, view);
    const cudaError_t e = cudaGetLastError();
    return e == cudaSuccess ? WT_OK : cuda_fail(e, "wt_projected_grid_async launch");
}

extern "C" wt_status wt_vertex_stage(const wt_view* view, const float* pos, const float* nrm, uint64_t n_vertices,
                                     uint32_t flags, float* clip_out, float* ndc0_out, float* view_out,
                                     float* facing_out, float* nrm_yaw_out, wt_stream stream) {
    WT_NVTX_RANGE("wt_vertex_stage");
    if (flags & ~(uint32_t)WT_LAYOUT_VEC3) return fail(WT_ERR_INVALID_ARG, "wt_vertex_stage: flags other than WT_LAYOUT_VEC3");
    const bool vec3 = (flags & WT_LAYOUT_VEC3) != 0;
    const size_t la = vec3 ? 4 : 16;
    if (!view || !aligned(view, 4)) return fail(WT_ERR_INVALID_ARG, "wt_vertex_stage: view NULL or misaligned");
    if (!pos || !aligned(pos, la)) return fail(WT_ERR_INVALID_ARG, "wt_vertex_stage: pos NULL or misaligned");
    const bool need_nrm = facing_out || nrm_yaw_out;
    if (need_nrm && (!nrm || !aligned(nrm, la)))
        return fail(WT_ERR_INVALID_ARG, "wt_vertex_stage: nrm NULL or misaligned while normal outputs are asked for");
    if (clip_out && !aligned(clip_out, 16)) return fail(WT_ERR_INVALID_ARG, "wt_vertex_stage: clip_out not 16-byte aligned");
    if (ndc0_out && !aligned(ndc0_out, 8)) return fail(WT_ERR_INVALID_ARG, "wt_vertex_stage: ndc0_out not 8-byte aligned");
    float* lay[3] = {view_out, facing_out, nrm_yaw_out};
    for (float* p : lay)
        if (p && !aligned(p, la)) return fail(WT_ERR_INVALID_ARG, "wt_vertex_stage: output misaligned for its layout");
    if (n_vertices == 0) return WT_OK;
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return cuda_fail(e, "cudaGetDevice");
    if (dev < 0 || dev >= 64) return fail(WT_ERR_UNSUPPORTED, "device ordinal beyond 63");
    int cap = g_stage_blocks[dev].load(std::memory_order_relaxed);
    if (cap == 0) {
        int occ = 0;
        const int sms = wt::sm_count();
        if (sms <= 0) return fail(WT_ERR_CUDA, "cannot read the device's SM count");
        e = vec3 ? cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, k_vertex_stage<true>, kStageThreads, 0)
                 : cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, k_vertex_stage<false>, kStageThreads, 0);
        if (e != cudaSuccess) return cuda_fail(e, "occupancy query");
        cap = sms * (occ > 0 ? occ : 1);
        g_stage_blocks[dev].store(cap, std::memory_order_relaxed);
    }
    const uint64_t need = (n_vertices + kStageThreads - 1) / kStageThreads;
    const unsigned blocks = (unsigned)(need < (uint64_t)cap ? need : (uint64_t)cap);
    const StageOut o{clip_out, ndc0_out, view_out, facing_out, nrm_yaw_out};
    cudaStream_t s = (cudaStream_t)stream;
    if (vec3)
        k_vertex_stage<true><<<blocks, kStageThreads, 0, s>>>(view, pos, nrm, n_vertices, o);
    else
        k_vertex_stage<false><<<blocks, kStageThreads, 0, s>>>(view, pos, nrm, n_vertices, o);
    e = cudaGetLastError();
    return e == cudaSuccess ? WT_OK : cuda_fail(e, "wt_vertex_stage launch");
}
