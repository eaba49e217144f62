// wt_stage.cuh — the per-vertex arithmetic of the remaining vertex-shader
// outputs (water-grid.vert:150-158, :190-193), shared by the stand-alone
// vertex stage (wt_frame.cu:k_vertex_stage) and the forward kernel's fused
// epilogue (wt_displace.cu:k_forward), so that both write the same bits.
#pragma once
#include <cuda_runtime.h>
#include <cstdint>

#include "wt_internal.h"

namespace wt {
namespace dev {

template <bool VEC3>
__device__ __forceinline__ float3 load3(const float* p, uint64_t i) {
    if (VEC3) return make_float3(p[3 * i], p[3 * i + 1], p[3 * i + 2]);
    const float4 v = reinterpret_cast<const float4*>(p)[i];
    return make_float3(v.x, v.y, v.z);
}

template <bool VEC3>
__device__ __forceinline__ void store3(float* p, uint64_t i, float3 v) {
    if (VEC3) {
        p[3 * i] = v.x;
        p[3 * i + 1] = v.y;
        p[3 * i + 2] = v.z;
    } else {
        reinterpret_cast<float4*>(p)[i] = make_float4(v.x, v.y, v.z, 0.0f);
    }
}

// One vertex: world position p, unit normal n (read only when a normal
// output is asked for), u = the 36 floats of wt_view (view_projection
// column-major, view_only_yaw, camera position).
//   clip   = M (p, 1)                              (:150)
//   ndc0   = (M (p.x, 0, p.z, 1)).xy / w            (:153-154, height 0)
//   view   = camera - p                            (:158)
//   facing = n, negated when dot(n, view) < 0      (:190)
//   yaw    = normalize(mat3(view_only_yaw) facing)  (:193)
template <bool VEC3>
__device__ __forceinline__ void stage_vertex(const float* __restrict__ u, float3 p, float3 n, uint64_t i,
                                             const StageOut& o) {
    const float* M = u;       // view_projection, column-major
    const float* Y = u + 16;  // view_only_yaw
    if (o.clip) {
        float4 c;
        c.x = fmaf(M[0], p.x, fmaf(M[4], p.y, fmaf(M[8], p.z, M[12])));
        c.y = fmaf(M[1], p.x, fmaf(M[5], p.y, fmaf(M[9], p.z, M[13])));
        c.z = fmaf(M[2], p.x, fmaf(M[6], p.y, fmaf(M[10], p.z, M[14])));
        c.w = fmaf(M[3], p.x, fmaf(M[7], p.y, fmaf(M[11], p.z, M[15])));
        reinterpret_cast<float4*>(o.clip)[i] = c;
    }
    if (o.ndc0) {
        const float x = fmaf(M[0], p.x, fmaf(M[8], p.z, M[12]));
        const float y = fmaf(M[1], p.x, fmaf(M[9], p.z, M[13]));
        const float w = fmaf(M[3], p.x, fmaf(M[11], p.z, M[15]));
        reinterpret_cast<float2*>(o.ndc0)[i] = make_float2(x / w, y / w);
    }
    const float3 v = make_float3(u[32] - p.x, u[33] - p.y, u[34] - p.z);
    if (o.view) store3<VEC3>(o.view, i, v);
    if (o.facing || o.nyaw) {
        float3 nv = n;
        // the sign of dot(n, normalize(v)) is the sign of dot(n, v)
        if (fmaf(nv.x, v.x, fmaf(nv.y, v.y, nv.z * v.z)) < 0.0f) nv = make_float3(-nv.x, -nv.y, -nv.z);
        if (o.facing) store3<VEC3>(o.facing, i, nv);
        if (o.nyaw) {
            float3 q;
            q.x = fmaf(Y[0], nv.x, fmaf(Y[4], nv.y, Y[8] * nv.z));
            q.y = fmaf(Y[1], nv.x, fmaf(Y[5], nv.y, Y[9] * nv.z));
            q.z = fmaf(Y[2], nv.x, fmaf(Y[6], nv.y, Y[10] * nv.z));
            const float s = 1.0f / sqrtf(fmaf(q.x, q.x, fmaf(q.y, q.y, q.z * q.z)));
            store3<VEC3>(o.nyaw, i, make_float3(q.x * s, q.y * s, q.z * s));
        }
    }
}

}  // namespace dev
}  // namespace wt
