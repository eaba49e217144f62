// wt_water.cu — the water fragment stage: rasterisation of the grid's
// triangles into a visibility buffer, then per-pixel shading with the
// arithmetic of assets/shaders/water-grid.frag:65-151.
//
// This file is compiled with -fmad=false: every FP32 operation rounds once,
// in source order, so coverage, depth and all but the transcendental-bearing
// colour terms reproduce a scalar CPU restatement bit for bit.
//
// Rasterisation (k_water_raster): one lane per triangle.  Window coordinates
// are snapped to 1/256 pixel and covered with exact 64-bit integer edge
// functions at pixel centres (left/top fill rule); the window depth is
// interpolated linearly in screen space and folded with the triangle index
// into one 64-bit key, (depth bits << 32) | (triangle + 1), kept per pixel by
// a 64-bit atomic minimum (no return value, so no round trip per fragment):
// nearest fragment wins, ties go to the lower index, and the
// result does not depend on launch order.  Triangles with more than
// kOwnPixels pixels in their box, and triangles that reach behind the near
// plane or past a guard band of 64 viewports (clipped in clip space first),
// go to a queue; a second pass (k_water_raster_deferred) spreads the queue
// over every warp of a resident grid, each triangle rasterised by a whole
// warp, lanes striding over the pixels.
//
// Shading (k_water_shade): one thread per pixel; perspective-correct
// barycentrics from the triangle's three clip-space vertices (2D homogeneous
// form), varyings, then the fragment shader's terms.
#include <cuda_runtime.h>

#include <atomic>
#include <cmath>
#include <cstdio>

#include "wt_nvtx.h"
#include "wt_internal.h"

namespace {

constexpr float kSub = 256.0f;   // sub-pixel steps per pixel
constexpr float kGuard = 64.0f;  // guard band, in NDC units
// Triangles with at most kOwnPixels pixels in their box are rasterised by
// their own thread in the first pass; 6 blocks of 256 threads a multiprocessor
// (40 registers) hide its gather latency.  1080p frame of a 1024^2 grid:
// 16 / 64 / 128 / 256 pixels -> 94 / 62 / 57 / 64 us for the whole call.
#ifndef WT_OWN_PIXELS
#define WT_OWN_PIXELS 128
#endif
constexpr int kOwnPixels = WT_OWN_PIXELS;
#ifndef WT_RASTER_MINB
#define WT_RASTER_MINB 6
#endif
constexpr int64_t kSmallExtent = 1 << 13;  // sub-pixel steps (32 pixels)
constexpr unsigned kFull = 0xffffffffu;

struct CV4 {
    float x, y, z, w;
};

struct WinTri {
    int32_t X[3], Y[3];
    float Z[3];
};

__device__ __forceinline__ void to_window(const CV4& c, float hw, float hh, int32_t& X, int32_t& Y, float& Z) {
    const float xw = (c.x / c.w + 1.0f) * hw;
    const float yw = (c.y / c.w + 1.0f) * hh;
    X = __float2int_rn(xw * kSub);
    Y = __float2int_rn(yw * kSub);
    Z = (c.z / c.w) * 0.5f + 0.5f;
}

__device__ __forceinline__ bool inside_guard(const CV4& c) {
    return c.w > 0.0f && fabsf(c.x) <= kGuard * c.w && fabsf(c.y) <= kGuard * c.w;
}

__device__ __forceinline__ float plane_dist(int p, const CV4& c) {
    switch (p) {
        case 0: return c.z + c.w;              // near: z >= -w
        case 1: return kGuard * c.w - c.x;
        case 2: return kGuard * c.w + c.x;
        case 3: return kGuard * c.w - c.y;
        default: return kGuard * c.w + c.y;
    }
}

// Sutherland-Hodgman against the near plane and the guard band; <= 8 vertices.
__device__ int clip_polygon(CV4* poly, int n) {
    CV4 tmp[8];
    for (int p = 0; p < 5 && n > 0; ++p) {
        int m = 0;
        for (int i = 0; i < n; ++i) {
            const CV4 a = poly[i], b = poly[i + 1 < n ? i + 1 : 0];
            const float da = plane_dist(p, a), db = plane_dist(p, b);
            if (da >= 0.0f && m < 8) tmp[m++] = a;
            if ((da >= 0.0f) != (db >= 0.0f) && m < 8) {
                const float t = da / (da - db);
                tmp[m++] = CV4{a.x + t * (b.x - a.x), a.y + t * (b.y - a.y), a.z + t * (b.z - a.z),
                               a.w + t * (b.w - a.w)};
            }
        }
        for (int i = 0; i < m; ++i) poly[i] = tmp[i];
        n = m;
    }
    return n;
}

// Oriented triangle with its pixel box and fill-rule flags.
struct Setup {
    int32_t x[3], y[3];
    float z[3];
    float area_f;
    int32_t px0, px1, py0, py1;
    int incl;   // bit k: edge k (vertex k+1 -> k+2) owns pixel centres exactly on it
    bool small; // extent below kSmallExtent in x and y (exact 32-bit edge functions)
};

__device__ __forceinline__ bool setup_tri(const WinTri& w, uint32_t W, uint32_t H, Setup& s) {
    const int32_t xmn = min(w.X[0], min(w.X[1], w.X[2])), xmx = max(w.X[0], max(w.X[1], w.X[2]));
    const int32_t ymn = min(w.Y[0], min(w.Y[1], w.Y[2])), ymx = max(w.Y[0], max(w.Y[1], w.Y[2]));
    // pixel centres (p * 256 + 128) inside the box, clamped to the viewport;
    // most far-field triangles of a projected grid hold none and stop here.
    // Window coordinates stay below 2^28 in magnitude (guard band of 64
    // viewports, viewport <= 16384, 1/256 pixel), so 32 bits hold these.
    int32_t px0 = -((128 - xmn) >> 8), px1 = (xmx - 128) >> 8;
    int32_t py0 = -((128 - ymn) >> 8), py1 = (ymx - 128) >> 8;
    px0 = max(px0, 0);
    py0 = max(py0, 0);
    px1 = min(px1, (int32_t)W - 1);
    py1 = min(py1, (int32_t)H - 1);
    if (px0 > px1 || py0 > py1) return false;
    const bool small = xmx - xmn < (int32_t)kSmallExtent && ymx - ymn < (int32_t)kSmallExtent;
    bool ccw;
    if (small) {  // |products| < 2^26: exact in 32 bits
        int32_t area = (w.X[1] - w.X[0]) * (w.Y[2] - w.Y[0]) - (w.Y[1] - w.Y[0]) * (w.X[2] - w.X[0]);
        if (area == 0) return false;
        ccw = area > 0;
        s.area_f = (float)(ccw ? area : -area);
    } else {
        int64_t area = (int64_t)(w.X[1] - w.X[0]) * (w.Y[2] - w.Y[0]) - (int64_t)(w.Y[1] - w.Y[0]) * (w.X[2] - w.X[0]);
        if (area == 0) return false;
        ccw = area > 0;
        s.area_f = (float)(ccw ? area : -area);
    }
    const int a = ccw ? 1 : 2, b = ccw ? 2 : 1;  // counter-clockwise order
    s.x[0] = w.X[0]; s.y[0] = w.Y[0]; s.z[0] = w.Z[0];
    s.x[1] = w.X[a]; s.y[1] = w.Y[a]; s.z[1] = w.Z[a];
    s.x[2] = w.X[b]; s.y[2] = w.Y[b]; s.z[2] = w.Z[b];
    s.px0 = px0; s.px1 = px1; s.py0 = py0; s.py1 = py1;
    s.small = small;
    s.incl = 0;
    for (int k = 0; k < 3; ++k) {
        const int i = k == 2 ? 0 : k + 1, j = k == 0 ? 2 : (k == 1 ? 0 : 1);
        const int32_t dx = s.x[j] - s.x[i], dy = s.y[j] - s.y[i];
        if (dy < 0 || (dy == 0 && dx < 0)) s.incl |= 1 << k;
    }
    return true;
}

__device__ __forceinline__ void raster_pixel(const Setup& s, int32_t px, int32_t py, uint32_t tri, uint32_t W,
                                             unsigned long long* frag) {
    const int64_t cx = (int64_t)px * 256 + 128, cy = (int64_t)py * 256 + 128;
    int64_t e[3];
#pragma unroll
    for (int k = 0; k < 3; ++k) {
        const int i = k == 2 ? 0 : k + 1, j = k == 0 ? 2 : (k == 1 ? 0 : 1);
        e[k] = (int64_t)(s.x[j] - s.x[i]) * (cy - s.y[i]) - (int64_t)(s.y[j] - s.y[i]) * (cx - s.x[i]);
        if (!(e[k] > 0 || (e[k] == 0 && ((s.incl >> k) & 1)))) return;
    }
    float d = ((float)e[0] * s.z[0] + (float)e[1] * s.z[1] + (float)e[2] * s.z[2]) / s.area_f;
    if (!(d >= 0.0f && d <= 1.0f)) return;
    d = d + 0.0f;  // -0 -> +0
    const unsigned long long key = ((unsigned long long)__float_as_uint(d) << 32) | (unsigned long long)(tri + 1u);
    atomicMin(frag + (size_t)py * W + px, key);
}

// Triangles less than kSmallExtent sub-pixel steps wide and high: the edge
// functions, taken relative to vertex 0, stay below 2^28 in magnitude, so they
// are evaluated exactly in 32-bit integers, stepping from pixel to pixel (the
// same values the 64-bit form gives).
__device__ __forceinline__ void raster_small(const Setup& s, uint32_t tri, uint32_t W, unsigned long long* frag) {
    int32_t e0[3], dx[3], dy[3];
    const int32_t cx0 = s.px0 * 256 + 128 - s.x[0], cy0 = s.py0 * 256 + 128 - s.y[0];
#pragma unroll
    for (int k = 0; k < 3; ++k) {
        const int i = k == 2 ? 0 : k + 1, j = k == 0 ? 2 : (k == 1 ? 0 : 1);
        const int32_t ex = s.x[j] - s.x[i], ey = s.y[j] - s.y[i];
        e0[k] = ex * (cy0 - (s.y[i] - s.y[0])) - ey * (cx0 - (s.x[i] - s.x[0]));
        dx[k] = -ey * 256;
        dy[k] = ex * 256;
    }
    // inside edge k: e_k > 0, or e_k == 0 where the edge owns its centres,
    // i.e. e_k - 1 + incl_k >= 0: all three at once by the sign of an OR
    int32_t b[3];
#pragma unroll
    for (int k = 0; k < 3; ++k) {
        b[k] = ((s.incl >> k) & 1) - 1;
        e0[k] += b[k];
    }
    for (int32_t py = s.py0; py <= s.py1; ++py) {
        int32_t e[3] = {e0[0], e0[1], e0[2]};
        for (int32_t px = s.px0; px <= s.px1; ++px) {
            if ((e[0] | e[1] | e[2]) >= 0) {
                float d = ((float)(e[0] - b[0]) * s.z[0] + (float)(e[1] - b[1]) * s.z[1] +
                           (float)(e[2] - b[2]) * s.z[2]) / s.area_f;
                if (d >= 0.0f && d <= 1.0f) {
                    d = d + 0.0f;  // -0 -> +0
                    const unsigned long long key =
                        ((unsigned long long)__float_as_uint(d) << 32) | (unsigned long long)(tri + 1u);
                    atomicMin(frag + (size_t)py * W + px, key);
                }
            }
#pragma unroll
            for (int k = 0; k < 3; ++k) e[k] += dx[k];
        }
#pragma unroll
        for (int k = 0; k < 3; ++k) e0[k] += dy[k];
    }
}

__device__ __forceinline__ void raster_own(const Setup& s, uint32_t tri, uint32_t W, unsigned long long* frag) {
    for (int32_t py = s.py0; py <= s.py1; ++py)
        for (int32_t px = s.px0; px <= s.px1; ++px) raster_pixel(s, px, py, tri, W, frag);
}

// raster_pixel for a small-extent triangle: the same edge values in 32 bits.
__device__ __forceinline__ void raster_pixel32(const Setup& s, int32_t px, int32_t py, uint32_t tri, uint32_t W,
                                               unsigned long long* frag) {
    const int32_t cx = px * 256 + 128, cy = py * 256 + 128;
    int32_t e[3], out = 0;
#pragma unroll
    for (int k = 0; k < 3; ++k) {
        const int i = k == 2 ? 0 : k + 1, j = k == 0 ? 2 : (k == 1 ? 0 : 1);
        e[k] = (s.x[j] - s.x[i]) * (cy - s.y[i]) - (s.y[j] - s.y[i]) * (cx - s.x[i]);
        out |= e[k] + ((s.incl >> k) & 1) - 1;  // negative: outside edge k (as in raster_small)
    }
    if (out < 0) return;
    float d = ((float)e[0] * s.z[0] + (float)e[1] * s.z[1] + (float)e[2] * s.z[2]) / s.area_f;
    if (!(d >= 0.0f && d <= 1.0f)) return;
    d = d + 0.0f;  // -0 -> +0
    atomicMin(frag + (size_t)py * W + px,
              ((unsigned long long)__float_as_uint(d) << 32) | (unsigned long long)(tri + 1u));
}

__device__ __forceinline__ void raster_warp(const Setup& s, uint32_t tri, uint32_t W, unsigned long long* frag,
                                            int lane) {
    // box <= 16384^2 pixels: 32-bit indices
    const uint32_t bw = (uint32_t)(s.px1 - s.px0 + 1);
    const uint32_t n = bw * (uint32_t)(s.py1 - s.py0 + 1);
    if (s.small) {
        // pixel p = r * bw + c walked in steps of 32 = qs * bw + rs (one
        // division per triangle, none per pixel)
        const uint32_t qs = 32u / bw, rs = 32u - qs * bw;
        uint32_t r = (uint32_t)lane / bw, c = (uint32_t)lane - r * bw;
        for (uint32_t p = (uint32_t)lane; p < n; p += 32) {
            raster_pixel32(s, s.px0 + (int32_t)c, s.py0 + (int32_t)r, tri, W, frag);
            c += rs;
            r += qs;
            if (c >= bw) { c -= bw; ++r; }
        }
        return;
    }
    for (uint32_t p = (uint32_t)lane; p < n; p += 32) {
        const uint32_t r = p / bw;
        raster_pixel(s, s.px0 + (int32_t)(p - r * bw), s.py0 + (int32_t)r, tri, W, frag);
    }
}

// One pass before the triangles: the visibility buffer cleared to the scene
// depth (or 1, the far plane) with no triangle, the queue emptied, and the
// per-vertex window coordinates, computed once for the ~6 triangles sharing a
// vertex: (X, Y, depth bits, 1) for vertices inside the guard band, w = 0
// otherwise (their triangles take the clipping path).
__global__ void __launch_bounds__(256) k_water_prepare(const float* __restrict__ scene_depth, uint64_t npx,
                                                       unsigned long long* __restrict__ frag,
                                                       const float4* __restrict__ clip, uint64_t nv, uint32_t W,
                                                       uint32_t H, int4* __restrict__ win,
                                                       uint32_t* __restrict__ queue_count) {
    // the first raster pass may be scheduled now; it waits for this grid's
    // results before it reads them
    cudaTriggerProgrammaticLaunchCompletion();
    const float hw = (float)W * 0.5f, hh = (float)H * 0.5f;
    if (queue_count && blockIdx.x == 0 && threadIdx.x == 0) *queue_count = 0;
    const uint64_t n = npx > nv ? npx : nv;
    for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < n; i += (uint64_t)gridDim.x * blockDim.x) {
        if (i < nv) {
            const float4 c4 = clip[i];
            const CV4 c{c4.x, c4.y, c4.z, c4.w};
            int4 o = make_int4(0, 0, 0, 0);
            if (inside_guard(c)) {
                float z;
                to_window(c, hw, hh, o.x, o.y, z);
                o.z = __float_as_int(z);
                o.w = 1;
            }
            win[i] = o;
        }
        if (i < npx) {
            const float d = scene_depth ? scene_depth[i] : 1.0f;
            frag[i] = (unsigned long long)__float_as_uint(d) << 32;
        }
    }
}

__device__ __forceinline__ Setup shfl_setup(const Setup& s, int src) {
    Setup o;
#pragma unroll
    for (int k = 0; k < 3; ++k) {
        o.x[k] = __shfl_sync(kFull, s.x[k], src);
        o.y[k] = __shfl_sync(kFull, s.y[k], src);
        o.z[k] = __shfl_sync(kFull, s.z[k], src);
    }
    o.area_f = __shfl_sync(kFull, s.area_f, src);
    o.px0 = __shfl_sync(kFull, s.px0, src);
    o.px1 = __shfl_sync(kFull, s.px1, src);
    o.py0 = __shfl_sync(kFull, s.py0, src);
    o.py1 = __shfl_sync(kFull, s.py1, src);
    const int flags = __shfl_sync(kFull, s.incl | (s.small ? 8 : 0), src);
    o.incl = flags & 7;
    o.small = (flags & 8) != 0;
    return o;
}

// First pass: one thread per triangle (the grid covers them all).  Triangles
// whose pixel box holds at most kOwnPixels pixels are rasterised by their
// own thread; the others (larger boxes, and triangles that need clipping) are
// appended to a queue for the second pass (the triangle and its three vertex
// indices), with one atomic per warp.  Launched dependent on the preparing
// pass: the index loads are issued before it waits for that pass's results.
__global__ void __launch_bounds__(256, WT_RASTER_MINB) k_water_raster(const int4* __restrict__ win,
                                                         uint64_t n_vertices, const uint32_t* __restrict__ idx,
                                                         uint64_t n_tri, uint32_t W, uint32_t H,
                                                         unsigned long long* frag, uint32_t* __restrict__ queue_count,
                                                         uint4* __restrict__ queue) {
    const int lane = threadIdx.x & 31;
    const uint64_t t = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x;
    bool defer = false, own = false;
    Setup s;
    uint32_t v0 = 0, v1 = 0, v2 = 0;
    if (t < n_tri) {
        v0 = idx[3 * t];
        v1 = idx[3 * t + 1];
        v2 = idx[3 * t + 2];
    }
    cudaGridDependencySynchronize();                // window coordinates, cleared buffer, empty queue
    cudaTriggerProgrammaticLaunchCompletion();      // the second pass may be scheduled
    if (t < n_tri) {
        if (v0 < n_vertices && v1 < n_vertices && v2 < n_vertices) {
            const int4 a = win[v0], b = win[v1], c = win[v2];
            if (a.w & b.w & c.w) {
                WinTri w;
                w.X[0] = a.x; w.Y[0] = a.y; w.Z[0] = __int_as_float(a.z);
                w.X[1] = b.x; w.Y[1] = b.y; w.Z[1] = __int_as_float(b.z);
                w.X[2] = c.x; w.Y[2] = c.y; w.Z[2] = __int_as_float(c.z);
                if (setup_tri(w, W, H, s)) {
                    // box <= 16384^2 pixels: 32 bits hold its size
                    const int32_t npix = (s.px1 - s.px0 + 1) * (s.py1 - s.py0 + 1);
                    own = npix <= kOwnPixels;
                    defer = !own;
                }
            } else {
                defer = true;
            }
        }
    }
    const unsigned m = __ballot_sync(kFull, defer);
    if (m) {
        const int leader = __ffs(m) - 1;
        uint32_t q0 = 0;
        if (lane == leader) q0 = atomicAdd(queue_count, (uint32_t)__popc(m));
        q0 = __shfl_sync(kFull, q0, leader);
        // at most n_tri <= 2^32 - 2 entries: the queue holds them all
        if (defer) queue[q0 + (uint32_t)__popc(m & ((1u << lane) - 1u))] = make_uint4((uint32_t)t, v0, v1, v2);
    }
    if (own) {
        if (s.small) raster_small(s, (uint32_t)t, W, frag);
        else raster_own(s, (uint32_t)t, W, frag);
    }
}

// Second pass over the queue (launched dependent on the first, whose
// completion it waits for): every warp of a resident grid takes `per`
// consecutive entries a round (loads and triangle set-up in parallel, one
// lane each), then rasterises them one after another with all 32 lanes
// striding over the pixels; clipped triangles are cut into a fan first.
// Spreading the queue over every warp keeps the near-camera rows, whose
// triangles are the large ones and lie next to one another in the index
// buffer, off a few warps.
__global__ void __launch_bounds__(256) k_water_raster_deferred(const float4* __restrict__ clip,
                                                               const int4* __restrict__ win,
                                                               uint32_t W, uint32_t H, unsigned long long* frag,
                                                               const uint32_t* __restrict__ queue_count,
                                                               const uint4* __restrict__ queue) {
    cudaGridDependencySynchronize();  // the first pass is complete: the queue and its count
    const uint64_t n = *queue_count;
    const int lane = threadIdx.x & 31;
    const uint64_t warps = (uint64_t)gridDim.x * (blockDim.x >> 5);
    const uint64_t warp = blockIdx.x * (uint64_t)(blockDim.x >> 5) + (threadIdx.x >> 5);
    const uint64_t want = (n + warps - 1) / warps;
    const uint32_t per = want < 1 ? 1u : (want > 32 ? 32u : (uint32_t)want);
    const float hw = (float)W * 0.5f, hh = (float)H * 0.5f;
    for (uint64_t e0 = warp * per; e0 < n; e0 += warps * per) {
        const uint64_t e = e0 + lane;
        int kind = 0;  // 0 nothing, 2 window triangle set up, 3 clip first
        uint32_t t = 0;
        uint32_t vi[3] = {0u, 0u, 0u};
        Setup s;
        if ((uint32_t)lane < per && e < n) {
            // the first pass queued only triangles whose three indices are in range
            const uint4 q = queue[e];
            t = q.x;
            vi[0] = q.y;
            vi[1] = q.z;
            vi[2] = q.w;
            const int4 a = win[vi[0]], b = win[vi[1]], c = win[vi[2]];
            if (a.w & b.w & c.w) {
                WinTri w;
                w.X[0] = a.x; w.Y[0] = a.y; w.Z[0] = __int_as_float(a.z);
                w.X[1] = b.x; w.Y[1] = b.y; w.Z[1] = __int_as_float(b.z);
                w.X[2] = c.x; w.Y[2] = c.y; w.Z[2] = __int_as_float(c.z);
                if (setup_tri(w, W, H, s)) kind = 2;
            } else {
                kind = 3;
            }
        }
        unsigned todo = __ballot_sync(kFull, kind != 0);
        while (todo) {
            const int src = __ffs(todo) - 1;
            todo &= todo - 1;
            const int k = __shfl_sync(kFull, kind, src);
            const uint32_t tri = __shfl_sync(kFull, t, src);
            if (k == 2) {
                raster_warp(shfl_setup(s, src), tri, W, frag, lane);
                continue;
            }
            CV4 poly[8];
#pragma unroll
            for (int j = 0; j < 3; ++j) {
                const float4 c = clip[__shfl_sync(kFull, vi[j], src)];
                poly[j] = CV4{c.x, c.y, c.z, c.w};
            }
            const int nv = clip_polygon(poly, 3);
            bool bad = nv < 3;
            for (int j = 0; j < nv; ++j) bad |= !(poly[j].w > 0.0f);
            if (bad) continue;
            for (int j = 1; j + 1 < nv; ++j) {
                WinTri sw;
                to_window(poly[0], hw, hh, sw.X[0], sw.Y[0], sw.Z[0]);
                to_window(poly[j], hw, hh, sw.X[1], sw.Y[1], sw.Z[1]);
                to_window(poly[j + 1], hw, hh, sw.X[2], sw.Y[2], sw.Z[2]);
                Setup cs;
                if (setup_tri(sw, W, H, cs)) raster_warp(cs, tri, W, frag, lane);
            }
        }
    }
}

// ---- shading ---------------------------------------------------------------

struct ShadeTex {
    const float* depth;
    const uint8_t* refl;
    const uint8_t* refr;
    const uint8_t* sky;
    uint32_t sky_size;
};

// Texel index clamped to [0, n): the coordinates come from texture
// coordinates in [0, 1] (or NaN, which converts to 0), so 32 bits hold them.
__device__ __forceinline__ uint32_t clampi(int32_t i, uint32_t n) {
    return (uint32_t)(i < 0 ? 0 : (i >= (int32_t)n ? (int32_t)n - 1 : i));
}

// UNORM8 -> float (c / 255, correctly rounded), one table per block.
__shared__ float s_unorm8[256];

// GL_LINEAR, CLAMP_TO_EDGE over RGBA8 texels converted to c / 255.
__device__ float4 bilinear_rgba8(const uint8_t* px, uint32_t w, uint32_t h, float s, float t) {
    const float u = s * (float)w - 0.5f, v = t * (float)h - 0.5f;
    const float fi = floorf(u), fj = floorf(v);
    const float a = u - fi, b = v - fj;
    const int32_t ii = (int32_t)fi, jj = (int32_t)fj;
    const uint32_t i0 = clampi(ii, w), i1 = clampi(ii + 1, w);
    const uint32_t j0 = clampi(jj, h), j1 = clampi(jj + 1, h);
    const uchar4 q00 = *reinterpret_cast<const uchar4*>(px + 4 * ((size_t)j0 * w + i0));
    const uchar4 q10 = *reinterpret_cast<const uchar4*>(px + 4 * ((size_t)j0 * w + i1));
    const uchar4 q01 = *reinterpret_cast<const uchar4*>(px + 4 * ((size_t)j1 * w + i0));
    const uchar4 q11 = *reinterpret_cast<const uchar4*>(px + 4 * ((size_t)j1 * w + i1));
    auto f = [&](unsigned char c00, unsigned char c10, unsigned char c01, unsigned char c11) {
        const float t00 = s_unorm8[c00], t10 = s_unorm8[c10];
        const float t01 = s_unorm8[c01], t11 = s_unorm8[c11];
        return (1.0f - b) * ((1.0f - a) * t00 + a * t10) + b * ((1.0f - a) * t01 + a * t11);
    };
    return make_float4(f(q00.x, q10.x, q01.x, q11.x), f(q00.y, q10.y, q01.y, q11.y), f(q00.z, q10.z, q01.z, q11.z),
                       f(q00.w, q10.w, q01.w, q11.w));
}

// Cube-map face by the major axis (OpenGL 4.1 table 3.19), then bilinear.
__device__ float4 sample_cube(const uint8_t* faces, uint32_t size, float rx, float ry, float rz) {
    const float ax = fabsf(rx), ay = fabsf(ry), az = fabsf(rz);
    int face;
    float sc, tc, ma;
    if (ax >= ay && ax >= az) {
        face = rx >= 0.0f ? 0 : 1;
        sc = rx >= 0.0f ? -rz : rz;
        tc = -ry;
        ma = ax;
    } else if (ay >= az) {
        face = ry >= 0.0f ? 2 : 3;
        sc = rx;
        tc = ry >= 0.0f ? rz : -rz;
        ma = ay;
    } else {
        face = rz >= 0.0f ? 4 : 5;
        sc = rz >= 0.0f ? rx : -rx;
        tc = -ry;
        ma = az;
    }
    const float s = (sc / ma + 1.0f) / 2.0f, t = (tc / ma + 1.0f) / 2.0f;
    return bilinear_rgba8(faces + (size_t)face * size * size * 4, size, size, s, t);
}

__device__ __forceinline__ float clampf(float x, float lo, float hi) { return fminf(fmaxf(x, lo), hi); }
__device__ __forceinline__ float mixf(float x, float y, float a) { return x * (1.0f - a) + y * a; }

__global__ void __launch_bounds__(256) k_water_shade(const unsigned long long* __restrict__ frag,
                                                     const float4* __restrict__ clip, uint64_t n_vertices,
                                                     const uint32_t* __restrict__ idx, uint64_t n_tri,
                                                     const float4* __restrict__ facing,
                                                     const float4* __restrict__ nyaw, const float4* __restrict__ view,
                                                     const float2* __restrict__ ndc0, uint32_t W, uint32_t H,
                                                     wt_water_shading sh, ShadeTex tex, float4* colour_out,
                                                     float4* composite) {
    for (uint32_t c = threadIdx.x; c < 256; c += blockDim.x) s_unorm8[c] = (float)c / 255.0f;
    __syncthreads();
    const uint64_t n = (uint64_t)W * H;
    for (uint64_t p = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; p < n; p += (uint64_t)gridDim.x * blockDim.x) {
        const unsigned long long key = frag[p];
        const uint32_t tri1 = (uint32_t)(key & 0xffffffffull);
        const size_t t = tri1 - 1;
        uint32_t vi[3] = {0u, 0u, 0u};
        bool water = tri1 != 0 && t < n_tri;
        if (water) {
            vi[0] = idx[3 * t];
            vi[1] = idx[3 * t + 1];
            vi[2] = idx[3 * t + 2];
            water = vi[0] < n_vertices && vi[1] < n_vertices && vi[2] < n_vertices;
        }
        if (!water) {
            if (colour_out) colour_out[p] = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
            continue;
        }
        const uint32_t py = (uint32_t)(p / W), px = (uint32_t)(p - (uint64_t)py * W);
        // perspective-correct weights: lambda_k ~ (v_{k+1} x v_{k+2}) . (ndc x, ndc y, 1)
        const float nx = (2.0f * ((float)px + 0.5f)) / (float)W - 1.0f;
        const float ny = (2.0f * ((float)py + 0.5f)) / (float)H - 1.0f;
        float cv[3][3];
#pragma unroll
        for (int k = 0; k < 3; ++k) {
            const float4 c = clip[vi[k]];
            cv[k][0] = c.x;
            cv[k][1] = c.y;
            cv[k][2] = c.w;
        }
        float c[3];
#pragma unroll
        for (int k = 0; k < 3; ++k) {
            const float* a = cv[k == 2 ? 0 : k + 1];
            const float* b = cv[k == 0 ? 2 : (k == 1 ? 0 : 1)];
            const float cx = a[1] * b[2] - a[2] * b[1];
            const float cy = a[2] * b[0] - a[0] * b[2];
            const float cz = a[0] * b[1] - a[1] * b[0];
            c[k] = cx * nx + cy * ny + cz;
        }
        const float sum = c[0] + c[1] + c[2];
        const float l0 = c[0] / sum, l1 = c[1] / sum, l2 = c[2] / sum;
        const float4 n0 = facing[vi[0]], n1 = facing[vi[1]], n2 = facing[vi[2]];
        const float4 y0 = nyaw[vi[0]], y1 = nyaw[vi[1]], y2 = nyaw[vi[2]];
        const float4 w0 = view[vi[0]], w1 = view[vi[1]], w2 = view[vi[2]];
        const float2 d0 = ndc0[vi[0]], d1 = ndc0[vi[1]], d2 = ndc0[vi[2]];
        const float N[3] = {l0 * n0.x + l1 * n1.x + l2 * n2.x, l0 * n0.y + l1 * n1.y + l2 * n2.y,
                            l0 * n0.z + l1 * n1.z + l2 * n2.z};
        const float NY[3] = {l0 * y0.x + l1 * y1.x + l2 * y2.x, l0 * y0.y + l1 * y1.y + l2 * y2.y,
                             l0 * y0.z + l1 * y1.z + l2 * y2.z};
        const float V[3] = {l0 * w0.x + l1 * w1.x + l2 * w2.x, l0 * w0.y + l1 * w1.y + l2 * w2.y,
                            l0 * w0.z + l1 * w1.z + l2 * w2.z};
        const float D0[2] = {l0 * d0.x + l1 * d1.x + l2 * d2.x, l0 * d0.y + l1 * d1.y + l2 * d2.y};
        const float fz = __uint_as_float((uint32_t)(key >> 32));

        // water-grid.frag:65-151
        const float view_len = sqrtf(V[0] * V[0] + V[1] * V[1] + V[2] * V[2]);
        const float view_depth = clampf(view_len / sh.z_far, 0.0f, 1.0f);
        const float vv[3] = {V[0] / view_len, V[1] / view_len, V[2] / view_len};
        const float u0 = ((float)px + 0.5f) / (float)W, u1 = ((float)py + 0.5f) / (float)H;
        const float h0 = (D0[0] + 1.0f) / 2.0f, h1 = (D0[1] + 1.0f) / 2.0f;
        float back_raw = 1.0f;
        if (tex.depth)
            back_raw = tex.depth[(size_t)clampi((int32_t)floorf(u1 * (float)H), H) * W +
                                 clampi((int32_t)floorf(u0 * (float)W), W)];
        const float back = (sh.z_near * back_raw) / (sh.z_far - back_raw * (sh.z_far - sh.z_near));
        const float sky_behind = back > 0.999f ? 0.0f : 1.0f;
        const float here = (sh.z_near * fz) / (sh.z_far - fz * (sh.z_far - sh.z_near));
        const float delta = clampf(back - here, 0.0f, 1.0f);
        const float I[3] = {-vv[0], -vv[1], -vv[2]};
        const float kr = 2.0f * (N[0] * I[0] + N[1] * I[1] + N[2] * I[2]);
        const float R[3] = {I[0] - kr * N[0], I[1] - kr * N[1], I[2] - kr * N[2]};
        const float4 sky = sample_cube(tex.sky, tex.sky_size, R[0], R[1], R[2]);
        const float sun_p = powf(
            clampf(R[0] * sh.sun_position[0] + R[1] * sh.sun_position[1] + R[2] * sh.sun_position[2], 0.0f, 1.0f),
            sh.sun_shininess);
        const float sun = (sh.sun_strength * 1.0f) * sun_p;
        const float cos_t = N[0] * vv[0] + N[1] * vv[1] + N[2] * vv[2];
        // pow(1 - cos, 5) as products, as shader compilers expand a constant
        // integer exponent (within a few ulp of powf)
        const float om = 1.0f - cos_t, om2 = om * om;
        const float fres = 0.02f + (1.0f - 0.02f) * (om2 * om2 * om);
        const float ds = 0.1f * (1.0f - view_depth);  // both distortion strengths are 0.1
        const float ul0 = clampf(mixf(u0, h0, ds) + ds * NY[0], 0.0f, 1.0f);
        const float ul1 = clampf(mixf(u1, h1, ds) + ds * -NY[2], 0.0f, 1.0f);
        const float ur0 = clampf(mixf(u0, h0, ds) + ds * -NY[0], 0.0f, 1.0f);
        const float ur1 = clampf(mixf(u1, h1, ds) + ds * NY[2], 0.0f, 1.0f);
        const float4 lrefl = tex.refl ? bilinear_rgba8(tex.refl, W, H, ul0, ul1) : make_float4(0.f, 0.f, 0.f, 0.f);
        const float4 lrefr = tex.refr ? bilinear_rgba8(tex.refr, W, H, ur0, ur1) : make_float4(0.f, 0.f, 0.f, 0.f);
        const float tint_f = 0.0f == sh.tint_threshold
                                 ? 0.0f
                                 : sky_behind * (1.0f - clampf(delta / sh.tint_threshold, 0.0f, 1.0f));
        const float day = clampf(sh.sun_position[1], 0.0f, 1.0f);
        const float clarity = sh.water_clarity * lrefr.w * (1.0f - delta);
        const float deep[3] = {0.0f, 0.341f, 0.482f}, shallow[3] = {0.3f, 0.941f, 0.903f};
        const float skyc[3] = {sky.x, sky.y, sky.z}, lrc[3] = {lrefl.x, lrefl.y, lrefl.z};
        const float ltc[3] = {lrefr.x, lrefr.y, lrefr.z};
        float out[4];
#pragma unroll
        for (int k = 0; k < 3; ++k) {
            const float tint = day * mixf(deep[k], shallow[k], tint_f);
            const float trans = mixf(tint, ltc[k], clarity);
            const float refl = mixf(skyc[k] + sun, lrc[k], lrefl.w);
            out[k] = mixf(trans, refl, fres);
        }
        out[3] = 0.0f == sh.soft_edges_threshold
                     ? 1.0f
                     : 1.0f - (sky_behind * (1.0f - clampf(delta / sh.soft_edges_threshold, 0.0f, 1.0f)));
        const float fog_a = view_depth >= sh.fog_radius_far
                                ? sh.fog_colour[3]
                                : view_depth <= sh.fog_radius_near
                                      ? 0.0f
                                      : sh.fog_colour[3] * ((view_depth - sh.fog_radius_near) /
                                                            (sh.fog_radius_far - sh.fog_radius_near));
#pragma unroll
        for (int k = 0; k < 3; ++k) out[k] = mixf(out[k], sh.fog_colour[k], fog_a);
        const float4 col = make_float4(out[0], out[1], out[2], out[3]);
        if (colour_out) colour_out[p] = col;
        if (composite) {
            const float4 d = composite[p];
            const float a = col.w;
            composite[p] = make_float4(col.x * a + d.x * (1.0f - a), col.y * a + d.y * (1.0f - a),
                                       col.z * a + d.z * (1.0f - a), col.w * a + d.w * (1.0f - a));
        }
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

// Grid of a grid-stride kernel: as many 256-thread blocks as are resident at
// once (SMs x blocks per SM, the latter read once per device), so that every
// block runs from the start instead of a partial last wave of blocks.
template <typename K>
unsigned resident_grid(K kernel, std::atomic<int> (&cache)[64], int sms, uint64_t items) {
    int dev = 0, occ = 1;
    if (cudaGetDevice(&dev) == cudaSuccess && dev >= 0 && dev < 64) {
        occ = cache[dev].load(std::memory_order_relaxed);
        if (occ == 0) {
            int o = 0;
            if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&o, kernel, 256, 0) != cudaSuccess || o < 1) o = 1;
            cache[dev].store(o, std::memory_order_relaxed);
            occ = o;
        }
    }
    const uint64_t need = (items + 255) / 256, cap = (uint64_t)sms * (uint64_t)occ;
    return (unsigned)(need < cap ? need : cap);
}

std::atomic<int> g_occ_prepare[64], g_occ_deferred[64], g_occ_shade[64];

// 256-thread launch that may begin before the previous kernel on the stream
// has finished (programmatic dependent launch); the kernel waits for that
// kernel's results (cudaGridDependencySynchronize) before it reads them.
template <typename K, typename... Args>
cudaError_t launch_dependent(K kernel, dim3 grid, cudaStream_t s, Args... args) {
    cudaLaunchConfig_t lc = {};
    lc.gridDim = grid;
    lc.blockDim = dim3(256);
    lc.stream = s;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
    attr[0].val.programmaticStreamSerializationAllowed = 1;
    lc.attrs = attr;
    lc.numAttrs = 1;
    return cudaLaunchKernelEx(&lc, kernel, args...);
}

wt_status sms_of_device(int* sms) {
    *sms = wt::sm_count();
    if (*sms <= 0) return fail(WT_ERR_CUDA, "cannot read the device's SM count");
    return WT_OK;
}

bool viewport_ok(uint32_t w, uint32_t h) { return w >= 1 && h >= 1 && w <= 16384 && h <= 16384; }

}  // namespace

// Workspace: the vertices' window coordinates (int4 each), the queue's
// entry count (16 bytes, for alignment), then the queue (uint4 per triangle:
// the triangle and its vertex indices).
namespace {
constexpr uint64_t kMaxRasterVertices = 1ull << 40;
size_t raster_queue_offset(uint64_t n_vertices) { return 16 * (size_t)n_vertices; }
size_t raster_workspace_bytes(uint64_t n_vertices, uint64_t n_triangles) {
    return raster_queue_offset(n_vertices) + 16 + 16 * (size_t)n_triangles;
}
}  // namespace

extern "C" wt_status wt_water_raster_workspace_size(uint64_t n_vertices, uint64_t n_triangles, size_t* bytes) {
    if (!bytes) return fail(WT_ERR_INVALID_ARG, "wt_water_raster_workspace_size: bytes is NULL");
    if (n_vertices > kMaxRasterVertices || n_triangles > (1ull << 32) - 2)
        return fail(WT_ERR_INVALID_ARG, "wt_water_raster_workspace_size: more than 2^40 vertices or 2^32 - 2 triangles");
    *bytes = raster_workspace_bytes(n_vertices, n_triangles);
    return WT_OK;
}

extern "C" wt_status wt_water_raster(const float* clip, uint64_t n_vertices, const uint32_t* indices,
                                     uint64_t n_triangles, uint32_t width, uint32_t height, const float* scene_depth,
                                     uint64_t* fragments, void* workspace, size_t workspace_bytes,
                                     wt_stream stream) {
    WT_NVTX_RANGE("wt_water_raster");
    if (!viewport_ok(width, height)) return fail(WT_ERR_INVALID_ARG, "wt_water_raster: viewport outside [1, 16384]^2");
    if (!fragments || !aligned(fragments, 8)) return fail(WT_ERR_INVALID_ARG, "wt_water_raster: fragments NULL or misaligned");
    if (scene_depth && !aligned(scene_depth, 4)) return fail(WT_ERR_INVALID_ARG, "wt_water_raster: scene_depth misaligned");
    if (n_triangles > 0) {
        if (!clip || !aligned(clip, 16)) return fail(WT_ERR_INVALID_ARG, "wt_water_raster: clip NULL or not 16-byte aligned");
        if (!indices || !aligned(indices, 4)) return fail(WT_ERR_INVALID_ARG, "wt_water_raster: indices NULL or misaligned");
        if (n_triangles > (1ull << 32) - 2) return fail(WT_ERR_INVALID_ARG, "wt_water_raster: more than 2^32 - 2 triangles");
        if (!workspace || !aligned(workspace, 16)) return fail(WT_ERR_INVALID_ARG, "wt_water_raster: workspace NULL or not 16-byte aligned");
        if (n_vertices > kMaxRasterVertices) return fail(WT_ERR_INVALID_ARG, "wt_water_raster: more than 2^40 vertices");
        if (workspace_bytes < raster_workspace_bytes(n_vertices, n_triangles))
            return fail(WT_ERR_NOMEM, "wt_water_raster: workspace below wt_water_raster_workspace_size");
    }
    int sms = 0;
    wt_status st = sms_of_device(&sms);
    if (st != WT_OK) return st;
    cudaStream_t s = (cudaStream_t)stream;
    const uint64_t npx = (uint64_t)width * height;
    const bool tris = n_triangles > 0 && n_vertices > 0;
    const uint64_t nv = tris ? n_vertices : 0;
    int4* win = static_cast<int4*>(workspace);
    uint32_t* queue_count =
        tris ? reinterpret_cast<uint32_t*>(static_cast<char*>(workspace) + raster_queue_offset(n_vertices)) : nullptr;
    uint4* queue = tris ? reinterpret_cast<uint4*>(queue_count + 4) : nullptr;
    unsigned long long* frag = reinterpret_cast<unsigned long long*>(fragments);
    k_water_prepare<<<resident_grid(k_water_prepare, g_occ_prepare, sms, npx > nv ? npx : nv), 256, 0, s>>>(
        scene_depth, npx, frag, reinterpret_cast<const float4*>(clip), nv, width, height, win, queue_count);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return cuda_fail(e, "wt_water_raster prepare launch");
    if (!tris) return WT_OK;
    // one thread per triangle (at most 2^24 blocks): most cost almost nothing
    const uint64_t rb = (n_triangles + 255) / 256;
    e = launch_dependent(k_water_raster, dim3((unsigned)rb), s, static_cast<const int4*>(win), n_vertices, indices,
                         n_triangles, width, height, frag, queue_count, queue);
    if (e != cudaSuccess) return cuda_fail(e, "wt_water_raster launch");
    // the queue: a resident grid, at most one warp per triangle
    e = launch_dependent(k_water_raster_deferred,
                         dim3(resident_grid(k_water_raster_deferred, g_occ_deferred, sms, 32 * n_triangles)), s,
                         reinterpret_cast<const float4*>(clip), static_cast<const int4*>(win), width, height, frag,
                         static_cast<const uint32_t*>(queue_count), static_cast<const uint4*>(queue));
    return e == cudaSuccess ? WT_OK : cuda_fail(e, "wt_water_raster deferred launch");
}

extern "C" wt_status wt_water_shade(const uint64_t* fragments, const float* clip, uint64_t n_vertices,
                                    const uint32_t* indices, uint64_t n_triangles, const float* facing, const float* nrm_yaw, const float* view, const float* ndc0,
                                    uint32_t width, uint32_t height, const wt_water_shading* shading,
                                    const wt_water_textures* textures, float* colour_out, float* composite,
                                    wt_stream stream) {
    WT_NVTX_RANGE("wt_water_shade");
    if (!viewport_ok(width, height)) return fail(WT_ERR_INVALID_ARG, "wt_water_shade: viewport outside [1, 16384]^2");
    if (!fragments || !aligned(fragments, 8)) return fail(WT_ERR_INVALID_ARG, "wt_water_shade: fragments NULL or misaligned");
    const float* v16[4] = {clip, facing, nrm_yaw, view};
    for (const float* q : v16)
        if (!q || !aligned(q, 16)) return fail(WT_ERR_INVALID_ARG, "wt_water_shade: vertex array NULL or not 16-byte aligned");
    if (!ndc0 || !aligned(ndc0, 8)) return fail(WT_ERR_INVALID_ARG, "wt_water_shade: ndc0 NULL or misaligned");
    if (!indices || !aligned(indices, 4)) return fail(WT_ERR_INVALID_ARG, "wt_water_shade: indices NULL or misaligned");
    if (!shading || !textures) return fail(WT_ERR_INVALID_ARG, "wt_water_shade: shading or textures NULL");
    if (!textures->skybox || textures->skybox_size == 0 || textures->skybox_size > 16384 || !aligned(textures->skybox, 4))
        return fail(WT_ERR_INVALID_ARG, "wt_water_shade: a sky box (6 RGBA8 faces, 4-byte aligned) is required");
    if ((textures->local_reflections && !aligned(textures->local_reflections, 4)) ||
        (textures->local_refractions && !aligned(textures->local_refractions, 4)) ||
        (textures->scene_depth && !aligned(textures->scene_depth, 4)))
        return fail(WT_ERR_INVALID_ARG, "wt_water_shade: texture misaligned");
    const float* vals = &shading->sun_position[0];
    for (size_t i = 0; i < sizeof(wt_water_shading) / sizeof(float); ++i)
        if (!std::isfinite(vals[i])) return fail(WT_ERR_INVALID_ARG, "wt_water_shade: non-finite shading parameter");
    if (!(shading->z_near > 0.0f && shading->z_far > shading->z_near))
        return fail(WT_ERR_INVALID_ARG, "wt_water_shade: need 0 < z_near < z_far");
    if (!colour_out && !composite) return WT_OK;
    if ((colour_out && !aligned(colour_out, 16)) || (composite && !aligned(composite, 16)))
        return fail(WT_ERR_INVALID_ARG, "wt_water_shade: colour outputs must be 16-byte aligned");
    int sms = 0;
    wt_status st = sms_of_device(&sms);
    if (st != WT_OK) return st;
    const uint64_t npx = (uint64_t)width * height;
    const ShadeTex tx{textures->scene_depth, textures->local_reflections, textures->local_refractions,
                      textures->skybox, textures->skybox_size};
    k_water_shade<<<resident_grid(k_water_shade, g_occ_shade, sms, npx), 256, 0, (cudaStream_t)stream>>>(
        reinterpret_cast<const unsigned long long*>(fragments), reinterpret_cast<const float4*>(clip), n_vertices,
        indices, n_triangles,
        reinterpret_cast<const float4*>(facing), reinterpret_cast<const float4*>(nrm_yaw),
        reinterpret_cast<const float4*>(view), reinterpret_cast<const float2*>(ndc0), width, height, *shading, tx,
        reinterpret_cast<float4*>(colour_out), reinterpret_cast<float4*>(composite));
    const cudaError_t e = cudaGetLastError();
    return e == cudaSuccess ? WT_OK : cuda_fail(e, "wt_water_shade launch");
}
