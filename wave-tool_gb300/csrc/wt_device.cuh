// wt_device.cuh — device code shared by the forward (wt_displace.cu) and
// adjoint (wt_adjoint.cu) kernels: row tiling, the per-wave staging and
// Chebyshev wave loop, heightmap footprints, block scans.
#pragma once
#include <cuda_runtime.h>
#include <cstdint>

#include "wt_internal.h"
#include "wt_stage.cuh"

namespace wt {
namespace dev {

constexpr double kTwoPi = 6.283185307179586476925286766559;
constexpr float kTurnToRad = 1.4629180792671596e-09f;  // 2*pi / 2^32

// Block-wide exclusive scan of a u32 array in global memory, in place, in
// chunks of blockDim.x.  Returns the total.  All threads must call.
static __device__ uint32_t block_exclusive_scan(uint32_t* a, uint32_t n) {
    __shared__ uint32_t warp_sums[32];
    __shared__ uint32_t carry;
    if (threadIdx.x == 0) carry = 0;
    __syncthreads();
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nwarps = blockDim.x >> 5;
    for (uint32_t base = 0; base < n; base += blockDim.x) {
        uint32_t i = base + threadIdx.x;
        uint32_t v = i < n ? a[i] : 0u;
        uint32_t x = v;
        for (int o = 1; o < 32; o <<= 1) {
            uint32_t y = __shfl_up_sync(0xffffffffu, x, o);
            if (lane >= o) x += y;
        }
        if (lane == 31) warp_sums[warp] = x;
        __syncthreads();
        if (warp == 0) {
            uint32_t w = lane < nwarps ? warp_sums[lane] : 0u;
            for (int o = 1; o < 32; o <<= 1) {
                uint32_t y = __shfl_up_sync(0xffffffffu, w, o);
                if (lane >= o) w += y;
            }
            warp_sums[lane] = w;  // inclusive
        }
        __syncthreads();
        uint32_t excl = carry + (warp > 0 ? warp_sums[warp - 1] : 0u) + x - v;
        if (i < n) a[i] = excl;
        __syncthreads();
        if (threadIdx.x == 0) carry += warp_sums[nwarps - 1];
        __syncthreads();
    }
    return carry;
}

// The adjoint's queue set-up, by one block after the prep's scans (needs
// sorted, tile_pre and pair_off, and the header's total_tiles): each patch's
// sorted rank, its chunks of tiles (chunk_max tiles per chunk when there are
// at least min_tiles tiles, else single tiles) and the exclusive prefixes of
// chunks and of records (chunks x waves) over the sorted order.
__device__ inline void adj_scan_body(char* ws, const AdjLayout& L, uint32_t n, uint32_t chunk_max,
                                     uint32_t min_tiles) {
    WsHeader* hdr = reinterpret_cast<WsHeader*>(ws);
    const uint32_t* sorted = reinterpret_cast<const uint32_t*>(ws + L.f.sorted);
    const uint32_t* tile_pre = reinterpret_cast<const uint32_t*>(ws + L.f.tile_pre);
    const uint32_t* pair_off = reinterpret_cast<const uint32_t*>(ws + L.f.pair_off);
    uint32_t* rank = reinterpret_cast<uint32_t*>(ws + L.rank);
    uint32_t* part_off = reinterpret_cast<uint32_t*>(ws + L.part_off);
    uint32_t* chunk_pre = reinterpret_cast<uint32_t*>(ws + L.chunk_pre);
    const uint32_t chunk = hdr->total_tiles >= min_tiles ? chunk_max : 1u;
    for (uint32_t q = threadIdx.x; q < n; q += blockDim.x) {
        const uint32_t p = sorted[q];
        rank[p] = q;
        const uint32_t chunks = (tile_pre[q + 1] - tile_pre[q] + chunk - 1) / chunk;
        chunk_pre[q] = chunks;
        const uint64_t rec = (uint64_t)chunks * (pair_off[p + 1] - pair_off[p]);
        part_off[q] = rec > 0xffffffffull ? 0xffffffffu : (uint32_t)rec;
    }
    __syncthreads();
    const uint32_t total = block_exclusive_scan(part_off, n);
    __syncthreads();  // every thread has read the first scan's total
    const uint32_t chunks = block_exclusive_scan(chunk_pre, n);
    if (threadIdx.x == 0) {
        part_off[n] = total;
        chunk_pre[n] = chunks;
        hdr->total_chunks = chunks;
        hdr->adj_chunk = chunk;
        if ((uint64_t)total > L.cap_records || total == 0xffffffffu || hdr->total_tiles == 0) {
            // the device patches need more records than the host copy said
            // (or the prep refused them)
            if (hdr->total_tiles != 0) atomicCAS(&hdr->status, 0u, (uint32_t)WT_ERR_NOMEM);
            hdr->total_chunks = 0;
        }
    }
}

// Tiling of a patch row (forward and adjoint): tiles of 32*smax columns, the
// row's last tile only as many 32-column blocks as the row still needs (so a
// row is padded to a multiple of 32 columns, not of 32*smax).
__host__ __device__ __forceinline__ uint32_t tiles_per_row(uint32_t cols, uint32_t smax) {
    return (cols + 32 * smax - 1) / (32 * smax);
}

// ---- shared epilogue -------------------------------------------------------

// Texel coordinate -> the two texel indices of the GL_LINEAR footprint and
// the weight, with the GL wrap of integer texel indices (REPEAT: i mod n;
// MIRRORED_REPEAT: (n-1) - mirror((i mod 2n) - n)).  The coordinate is first
// reduced by the wrap period (exact for |x| < 2^24); indices are clamped into
// range whatever the input (huge or NaN coordinates give garbage, never an
// out-of-bounds read).
struct Footprint {
    int i0, i1;
    float w;
};

__device__ __forceinline__ int mirror_index(int m, int n) {
    int a = m - n;
    return n - 1 - (a >= 0 ? a : -(1 + a));
}

// FAST: REPEAT with a power-of-two size, known at compile time (the wrap is
// one mask, no mirror selects).
template <bool FAST = false>
__device__ __forceinline__ Footprint footprint(float x, int n, uint32_t mode, bool pow2) {
    if (FAST) {
        Footprint f;
        f.w = x - floorf(x);
        f.i0 = __float2int_rd(x) & (n - 1);
        f.i1 = (f.i0 + 1) & (n - 1);
        return f;
    }
    const bool mir = mode == WT_WRAP_MIRRORED_REPEAT;
    const int P = mir ? 2 * n : n;
    Footprint f;
    int i0;
    if (pow2) {
        // power-of-two sizes: the wrap is a mask; the saturating conversion
        // keeps any input (NaN -> 0) in range
        f.w = x - floorf(x);
        i0 = __float2int_rd(x) & (P - 1);
    } else {
        const float Pf = (float)P;
        const float r = x - Pf * floorf(x * (1.0f / Pf));
        f.w = r - floorf(r);
        i0 = __float2int_rd(r);
        i0 += i0 < 0 ? P : 0;
        i0 -= i0 >= P ? P : 0;
        i0 = min(max(i0, 0), P - 1);
    }
    const int i1 = i0 + 1 == P ? 0 : i0 + 1;
    f.i0 = mir ? mirror_index(i0, n) : i0;
    f.i1 = mir ? mirror_index(i1, n) : i1;
    return f;
}

// Heightmap layer at the displaced local point (xl + dx, zl + dz) of a
// patch: h = disp*2*(r - 0.5) and its derivatives with respect to world x'
// and z' (the bilinear cross term hxz is what the adjoint of the normal needs;
// d2h/dx'2 = d2h/dz'2 = 0 inside a texel cell).
struct HmSample {
    float h, hx, hz, hxz;
};

// The four texels of a sample's footprint and its weights (the loads), and
// the layer value and derivatives formed from them (hm_combine).
struct HmTexels {
    float t00, t10, t01, t11, al, be;
};

template <bool FAST = false>
__device__ __forceinline__ HmTexels hm_fetch(const HmDev& hm, const PatchAux& a, float xd, float zd, bool pow2) {
    const float ut = fmaf(a.su, xd, a.hu0);
    const float vt = fmaf(a.sv, zd, a.hv0);
    const int W = (int)hm.width, H = (int)hm.height;
    const Footprint fu = footprint<FAST>(ut, W, hm.wrap, pow2), fv = footprint<FAST>(vt, H, hm.wrap, pow2);
    HmTexels T;
    T.al = fu.w;
    T.be = fv.w;
    T.t00 = __ldg(hm.texels + fv.i0 * W + fu.i0);
    T.t10 = __ldg(hm.texels + fv.i0 * W + fu.i1);
    T.t01 = __ldg(hm.texels + fv.i1 * W + fu.i0);
    T.t11 = __ldg(hm.texels + fv.i1 * W + fu.i1);
    return T;
}

__device__ __forceinline__ HmSample hm_combine(const HmDev& hm, const PatchAux& a, const HmTexels& T) {
    const float al = T.al, be = T.be, t00 = T.t00, t10 = T.t10, t01 = T.t01, t11 = T.t11;
    const float r0 = fmaf(al, t10 - t00, t00), r1 = fmaf(al, t11 - t01, t01);
    const float r = fmaf(be, r1 - r0, r0);
    const float dru = fmaf(be, (t11 - t01) - (t10 - t00), t10 - t00);
    const float drv = r1 - r0;
    const float k2 = 2.0f * hm.disp_scale;
    HmSample o;
    o.h = k2 * (r - 0.5f);
    o.hx = k2 * dru * a.su;
    o.hz = k2 * drv * a.sv;
    o.hxz = k2 * ((t11 - t01) - (t10 - t00)) * a.su * a.sv;
    return o;
}

template <bool FAST = false>
__device__ __forceinline__ HmSample hm_sample(const HmDev& hm, const PatchAux& a, float xd, float zd, bool pow2) {
    return hm_combine(hm, a, hm_fetch<FAST>(hm, a, xd, zd, pow2));
}

struct VertexSums {
    float dx, dy, dz, jx, jz, sxx, sxz, szz;
};

// What the forward's epilogue writes besides position and normal.
enum FwdMode : int {
    kModePlain = 0,  // positions and normals
    kModeSave = 1,   // also the vertex's eight wave sums (two float4 at 2*vidx) for a later adjoint
    kModeStage = 2,  // also the vertex-stage outputs (pos and nrm optional; world positions)
};

// Bounce, normal, stores for one vertex, its heightmap texels fetched
// already (T; used when hm.present).  su: the 36 floats of wt_view in shared
// memory (kModeStage only).
template <int MODE>
__device__ __forceinline__ void finish_vertex_t(const VertexSums& s, float xl, float zl, const PatchAux& a,
                                                const HmDev& hm, const HmTexels& T, uint64_t vidx,
                                                float* __restrict__ pos, float* __restrict__ nrm,
                                                uint32_t flags, float4* __restrict__ sums,
                                                const float* __restrict__ su, const StageOut& so) {
    if (MODE == kModeSave) {
        __stcs(sums + 2 * vidx, make_float4(s.dx, s.dy, s.dz, s.jx));
        __stcs(sums + 2 * vidx + 1, make_float4(s.jz, s.sxx, s.sxz, s.szz));
    }
    float px0 = 1.0f - s.sxx, px1 = s.jx, px2 = -s.sxz;
    float pz0 = -s.sxz, pz1 = s.jz, pz2 = 1.0f - s.szz;
    float dy = s.dy;
    if (hm.present) {
        const HmSample g = hm_combine(hm, a, T);
        dy += g.h;
        px1 = fmaf(g.hx, px0, fmaf(g.hz, px2, px1));
        pz1 = fmaf(g.hx, pz0, fmaf(g.hz, pz2, pz1));
    }
    dy += a.y_offset;
    // N = dP/dz x dP/dx
    float n0 = pz1 * px2 - pz2 * px1;
    float n1 = pz2 * px0 - pz0 * px2;
    float n2 = pz0 * px1 - pz1 * px0;
    float inv = rsqrtf(fmaf(n0, n0, fmaf(n1, n1, n2 * n2)));
    float ox, oz, ow;
    if (flags & WT_OUT_DISPLACEMENT) { ox = s.dx; oz = s.dz; ow = 0.0f; }
    else { ox = a.blx + (xl + s.dx); oz = a.blz + (zl + s.dz); ow = 1.0f; }
    if (MODE != kModeStage || pos) {
        if (flags & WT_LAYOUT_VEC3) {
            float* P = pos + 3 * vidx;
            __stcs(P, ox); __stcs(P + 1, dy); __stcs(P + 2, oz);
            if (nrm) {
                float* N = nrm + 3 * vidx;
                __stcs(N, n0 * inv); __stcs(N + 1, n1 * inv); __stcs(N + 2, n2 * inv);
            }
        } else {
            __stcs(reinterpret_cast<float4*>(pos) + vidx, make_float4(ox, dy, oz, ow));
            if (nrm) __stcs(reinterpret_cast<float4*>(nrm) + vidx, make_float4(n0 * inv, n1 * inv, n2 * inv, 0.0f));
        }
    } else if (nrm) {
        if (flags & WT_LAYOUT_VEC3) {
            float* N = nrm + 3 * vidx;
            __stcs(N, n0 * inv); __stcs(N + 1, n1 * inv); __stcs(N + 2, n2 * inv);
        } else {
            __stcs(reinterpret_cast<float4*>(nrm) + vidx, make_float4(n0 * inv, n1 * inv, n2 * inv, 0.0f));
        }
    }
    if (MODE == kModeStage)
        stage_vertex<false>(su, make_float3(ox, dy, oz), make_float3(n0 * inv, n1 * inv, n2 * inv), vidx, so);
}

// Heightmap, bounce, normal, stores for one vertex.  FAST: the heightmap
// wraps by REPEAT and has power-of-two sides.
template <int MODE, bool FAST = false>
__device__ __forceinline__ void finish_vertex(const VertexSums& s, float xl, float zl, const PatchAux& a,
                                              const HmDev& hm, bool pow2, uint64_t vidx,
                                              float* __restrict__ pos, float* __restrict__ nrm,
                                              uint32_t flags, float4* __restrict__ sums,
                                              const float* __restrict__ su, const StageOut& so) {
    HmTexels T{};
    if (hm.present) T = hm_fetch<FAST>(hm, a, xl + s.dx, zl + s.dz, pow2);
    finish_vertex_t<MODE>(s, xl, zl, a, hm, T, vidx, pos, nrm, flags, sums, su, so);
}

__device__ __forceinline__ uint32_t hi32_round(unsigned long long x) {
    return (uint32_t)((x + 0x80000000ull) >> 32);
}

// Per-wave staging in shared memory (3 float4 per wave, up to 32 waves per warp):
//   [0] t32, a32 (fixed-point turns), cos d, sin d      d = one 32-column step
//   [1] Q*A*Dx, A,  Q*A*Dz, Q*A*k*Dx^2
//   [2] A*k*Dx, Q*A*k*Dx*Dz,  A*k*Dz, Q*A*k*Dz^2
// i.e. four (cos coefficient, sin coefficient) pairs, one per pair of sums
// (dx, dy), (dz, sxx), (jx, sxz), (jz, szz): each pair of sums takes one paired
// FP32 FMA (__ffma2_rn, sm_100+) of its coefficients with (cos, sin) of the
// vertex, two correctly rounded FMAs in one instruction.
// Lane l's vertices j = 0..S-1 sit at columns c0 + l + 32 j.  Vertex 0 takes
// a MUFU sincos of its exact start phase, vertex 1 an exact rotation by d, and
// vertices j >= 2 the Chebyshev recurrence x[j] = 2 cos(d) x[j-1] - x[j-2]
// (one FMA per value, cos and sin paired; its error grows at most linearly
// in j).
constexpr int kStage = 3;

// The eight sums of one vertex as the wave loop accumulates them:
//   p[0] = (dx, dy)  p[1] = (dz, sxx)  p[2] = (jx, sxz)  p[3] = (jz, szz)
__device__ __forceinline__ VertexSums sums_of(const float2 (&p)[4]) {
    return VertexSums{p[0].x, p[0].y, p[1].x, p[2].x, p[3].x, p[1].y, p[2].y, p[3].y};
}

// One lane's share of the staging: wave constants for the tile at (c0, row).
__device__ __forceinline__ void stage_wave(const PairCoef& c, uint32_t c0, uint32_t row, float4* __restrict__ d) {
    // phase of this wave at (c0, row) and its per-column step on this row
    const unsigned long long t64 = c.t00 + (unsigned long long)c0 * c.ta + (unsigned long long)row * c.tb +
                                   (unsigned long long)c0 * row * c.tg;
    const unsigned long long a64 = c.ta + (unsigned long long)row * c.tg;
    const uint32_t t32 = hi32_round(t64), a32 = hi32_round(a64), d32 = hi32_round(a64 * 32ull);
    // rotation by the 32-column step: sincospi of the high part (exact in
    // FP32), then a first-order turn by the low 8 bits
    const uint32_t dhi = d32 & 0xffffff00u;
    float sd, cd;
    sincospif((float)(int)dhi * 4.656612873077393e-10f, &sd, &cd);  // sin(2*pi*turns)
    const float eps = (float)(d32 - dhi) * kTurnToRad;
    const float cdn = fmaf(-sd, eps, cd);
    sd = fmaf(cd, eps, sd);
    cd = cdn;
    d[0] = make_float4(__uint_as_float(t32), __uint_as_float(a32), cd, sd);
    d[1] = make_float4(c.qadx, c.a, c.qadz, c.qakxx);
    d[2] = make_float4(c.akdx, c.qakxz, c.akdz, c.qakzz);
}

// The wave loop of one tile for a compile-time S: sums of nw staged waves
// into acc[0..S-1] (pairs as in sums_of).
// Two waves per iteration with 4 vertices per lane, one with 8 (two would
// spill at the 8-vertex shapes' 128 registers).
template <int S, int SMAX>
__device__ __forceinline__ void wave_loop(float2 (&acc)[SMAX][4], const float4* __restrict__ wst, uint32_t nw,
                                          uint32_t lane) {
    constexpr int kUnroll = SMAX <= 4 ? 2 : 1;
#pragma unroll kUnroll
    for (uint32_t i = 0; i < nw; ++i) {
        const float4 w0v = wst[kStage * i];
        const float4 w1 = wst[kStage * i + 1];
        const float4 w2 = wst[kStage * i + 2];
        const uint32_t tl = __float_as_uint(w0v.x) + lane * __float_as_uint(w0v.y);
        const float ang = (float)(int)tl * kTurnToRad;
        const float cd = w0v.z, sd = w0v.w, tc = 2.0f * cd;
        const float2 k0 = make_float2(w1.x, w1.y), k1 = make_float2(w1.z, w1.w);
        const float2 k2 = make_float2(w2.x, w2.y), k3 = make_float2(w2.z, w2.w);
        const float2 tc2 = make_float2(tc, tc);
        float2 x, xp = make_float2(0.0f, 0.0f);  // (cos, sin) at vertex j and j - 1
        __sincosf(ang, &x.y, &x.x);
#pragma unroll
        for (int j = 0; j < S; ++j) {
            if (j == 1) {
                const float2 xn = make_float2(fmaf(x.x, cd, -x.y * sd), fmaf(x.y, cd, x.x * sd));
                xp = x;
                x = xn;
            } else if (j >= 2) {
                const float2 xn = __ffma2_rn(tc2, x, make_float2(-xp.x, -xp.y));
                xp = x;
                x = xn;
            }
            acc[j][0] = __ffma2_rn(k0, x, acc[j][0]);
            acc[j][1] = __ffma2_rn(k1, x, acc[j][1]);
            acc[j][2] = __ffma2_rn(k2, x, acc[j][2]);
            acc[j][3] = __ffma2_rn(k3, x, acc[j][3]);
        }
    }
}

}  // namespace dev
}  // namespace wt

namespace wt {
namespace dev {

// The wave loop for the tile's S (warp-uniform), compile-time in each branch.
template <int SMAX>
__device__ __forceinline__ void wave_loop_dispatch(uint32_t S, float2 (&acc)[SMAX][4], const float4* __restrict__ wst,
                                                   uint32_t nw, uint32_t lane) {
    if (SMAX == 4) {
        switch (S) {
            case 1: wave_loop<1, SMAX>(acc, wst, nw, lane); break;
            case 2: wave_loop<2, SMAX>(acc, wst, nw, lane); break;
            case 3: wave_loop<3, SMAX>(acc, wst, nw, lane); break;
            default: wave_loop<(SMAX >= 4 ? 4 : SMAX), SMAX>(acc, wst, nw, lane); break;
        }
    } else {
        switch (S) {
            case 1: wave_loop<1, SMAX>(acc, wst, nw, lane); break;
            case 2: wave_loop<2, SMAX>(acc, wst, nw, lane); break;
            case 3: wave_loop<3, SMAX>(acc, wst, nw, lane); break;
            case 4: wave_loop<4, SMAX>(acc, wst, nw, lane); break;
            case 5: wave_loop<(SMAX >= 5 ? 5 : SMAX), SMAX>(acc, wst, nw, lane); break;
            case 6: wave_loop<(SMAX >= 6 ? 6 : SMAX), SMAX>(acc, wst, nw, lane); break;
            case 7: wave_loop<(SMAX >= 7 ? 7 : SMAX), SMAX>(acc, wst, nw, lane); break;
            default: wave_loop<SMAX, SMAX>(acc, wst, nw, lane); break;
        }
    }
}

}  // namespace dev
}  // namespace wt
