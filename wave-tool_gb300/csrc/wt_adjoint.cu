// wt_adjoint.cu — vector-Jacobian product of the forward path with respect
// to every wave's parameters (no reference counterpart; the forward it
// differentiates is water-grid.vert:74-111, see wt_displace.cu).
//
// After the shared prep stages (validation, LPT order, FP64 phase constants;
// the scan kernel also ranks the patches and lays out the chunk queue and the
// records, wt_device.cuh:adj_scan_body):
//   k_adjoint    (persistent) per chunk of 1 or 2 tiles, per tile:
//       phase 1, one vertex per lane (as the forward, in two 4-vertex
//       halves): recompute the eight wave sums (or read the forward's saved
//       ones), the heightmap sample and the normal, and turn dL/dpos and
//       dL/dnrm into the adjoints of the eight sums, parked in shared memory;
//       phase 2, one wave per lane: walk the tile's vertices (broadcast from
//       shared memory), regenerate the wave's sin/cos there (MUFU start +
//       Chebyshev steps) and accumulate 11 per-wave moments; add them into
//       the chunk's record for that wave (no cross-lane reduction).
//   k_adj_cols   column sums of each patch's records over its chunks (FP32
//                Kahan, fixed order)
//   k_adj_pairs  closed-form FP64 gradient per (patch, wave) pair, one per thread
//   k_adj_waves  one warp per wave: the pair gradients of the patches that
//                use the wave, added in a fixed order.
// Every sum has a fixed order, so the result is bitwise reproducible.
//
// With g_q the adjoint of sum q per vertex and (c, s) the wave's cos/sin
// there, the records hold M_q = sum g_q c (q = dx, dz, jx, jz) or
// sum g_q s (q = dy, sxx, sxz, szz), T0 = sum g_theta, Tx = sum g_theta x,
// Tz = sum g_theta z, where g_theta = u_s c - u_c s is the adjoint of the
// phase.  All parameter gradients follow from these eleven sums.
#include <cuda_runtime.h>
#include <cstdint>

#include <atomic>

#include "wt_device.cuh"
#include "wt_internal.h"

namespace wt {
namespace {

using namespace wt::dev;

constexpr int kAdjWarps = 4;                 // warps per block
// Tiles per queue item ("chunk"): a warp takes this many consecutive tiles of
// one patch and adds their per-wave sums into one record, so the records (and
// the column sums that read them back) shrink by this factor, against a
// coarser queue.  Measured on 64 uneven patches: 2 tiles per chunk make the
// recomputing adjoint 1.6 % faster than 1, while the saved-sums adjoint (less
// work per tile) is 1.5 % slower at 2; 4 and 8 are slower for both.  With
// fewer than kAdjChunkMinTilesPerWarp tiles per resident warp the queue would
// run dry, so chunks stay single tiles (one 512^2 patch: 1024 tiles for 2432
// warps).  The workspace holds records for chunks of 1.
constexpr uint32_t kAdjChunkRecompute = 2;
constexpr uint32_t kAdjChunkSaved = 1;
constexpr uint32_t kAdjChunkMinTilesPerWarp = 8;
constexpr int kGbufVerts = 256;              // vertices per tile (32 lanes x S <= 8)
constexpr int kGbufF4 = 2;                   // float4 per parked vertex

// Adjoints of the eight sums at one vertex.  Order: dx, dy, dz, jx, jz, sxx,
// sxz, szz.  See oracle/gerstner_f64.c:wto_adjoint_f64 for the same algebra.
__device__ __forceinline__ void vertex_adjoint(const VertexSums& s, float xl, float zl, const PatchAux& a,
                                               const HmDev& hm, bool pow2, const float* __restrict__ gpos,
                                               const float* __restrict__ gnrm, uint64_t vidx, bool vec3,
                                               float g[8]) {
    const float a1 = 1.0f - s.sxx, a3 = -s.sxz, b1 = -s.sxz, b3 = 1.0f - s.szz;
    HmSample h = {0.0f, 0.0f, 0.0f, 0.0f};
    if (hm.present) h = hm_sample(hm, a, xl + s.dx, zl + s.dz, pow2);
    const float px0 = a1, px1 = fmaf(h.hx, a1, fmaf(h.hz, a3, s.jx)), px2 = a3;
    const float pz0 = b1, pz1 = fmaf(h.hx, b1, fmaf(h.hz, b3, s.jz)), pz2 = b3;
    const float* gp = gpos + (vec3 ? 3 : 4) * vidx;
    const float gpx_ = gp[0], gpy_ = gp[1], gpz_ = gp[2];
    float gPx0 = 0.0f, gPx1 = 0.0f, gPx2 = 0.0f, gPz0 = 0.0f, gPz1 = 0.0f, gPz2 = 0.0f;
    if (gnrm) {
        const float* gn = gnrm + (vec3 ? 3 : 4) * vidx;
        const float N0 = pz1 * px2 - pz2 * px1, N1 = pz2 * px0 - pz0 * px2, N2 = pz0 * px1 - pz1 * px0;
        const float inv = rsqrtf(fmaf(N0, N0, fmaf(N1, N1, N2 * N2)));
        const float n0 = N0 * inv, n1 = N1 * inv, n2 = N2 * inv;
        const float d = fmaf(n0, gn[0], fmaf(n1, gn[1], n2 * gn[2]));
        const float gN0 = (gn[0] - n0 * d) * inv, gN1 = (gn[1] - n1 * d) * inv, gN2 = (gn[2] - n2 * d) * inv;
        // N = Pz x Px:  g_Pz = Px x gN,  g_Px = gN x Pz
        gPz0 = px1 * gN2 - px2 * gN1;
        gPz1 = px2 * gN0 - px0 * gN2;
        gPz2 = px0 * gN1 - px1 * gN0;
        gPx0 = gN1 * pz2 - gN2 * pz1;
        gPx1 = gN2 * pz0 - gN0 * pz2;
        gPx2 = gN0 * pz1 - gN1 * pz0;
    }
    const float g_a1 = fmaf(gPx1, h.hx, gPx0), g_a3 = fmaf(gPx1, h.hz, gPx2);
    const float g_b1 = fmaf(gPz1, h.hx, gPz0), g_b3 = fmaf(gPz1, h.hz, gPz2);
    const float g_hx = fmaf(gPx1, a1, gPz1 * b1), g_hz = fmaf(gPx1, a3, gPz1 * b3);
    const float g_X = fmaf(gpy_, h.hx, g_hz * h.hxz), g_Z = fmaf(gpy_, h.hz, g_hx * h.hxz);
    g[0] = gpx_ + g_X;        // dx
    g[1] = gpy_;              // dy
    g[2] = gpz_ + g_Z;        // dz
    g[3] = gPx1;              // jx
    g[4] = gPz1;              // jz
    g[5] = -g_a1;             // sxx
    g[6] = -g_a3 - g_b1;      // sxz
    g[7] = -g_b3;             // szz
}

// Phase 2: lane = one wave; vertices l + 32 j of the tile (gbuf holds the
// eight vertex adjoints as two float4 of (cos-sum, sin-sum) pairs, (dx, dy)
// (dz, sxx) | (jx, sxz) (jz, szz)).  The eight moments are four paired FP32
// FMAs of a pair with the vertex's (cos, sin) and the recurrence one (0.907 ->
// 0.897 ms on 64 uneven patches, same bits; pairing the phase projections
// (uc, us) too ran 7 % slower: a paired FMA holds the FMA pipe two cycles).
// The position-weighted phase sums use x(l, j) = xb + l*gx + 32 j*gx: per
// vertex only sum(g_theta) and sum(j*g_theta) are kept, and folded into Tx,
// Tz once per l.
template <int SC>  // SC > 0: compile-time S; 0: runtime S
__device__ __forceinline__ void wave_moments(const float4* __restrict__ gbuf, uint32_t S_rt, uint32_t l0,
                                             uint32_t lstep, uint32_t nvalid, uint32_t t32, uint32_t a32, float cd,
                                             float sd, const PairCoef& k, float xb, float zb, float gx, float gz,
                                             float m[11]) {
    const uint32_t S = SC > 0 ? (uint32_t)SC : S_rt;
    const float tc = 2.0f * cd;
    const float2 tc2 = make_float2(tc, tc);
    float2 P0 = make_float2(m[0], m[1]), P1 = make_float2(m[2], m[5]);
    float2 P2 = make_float2(m[3], m[6]), P3 = make_float2(m[4], m[7]);
    for (uint32_t l = l0; l < nvalid; l += lstep) {
        const uint32_t tl = t32 + l * a32;
        float2 x, xp = make_float2(0.0f, 0.0f);
        __sincosf((float)(int)tl * kTurnToRad, &x.y, &x.x);
        float G0 = 0.0f, G1 = 0.0f;
#pragma unroll
        for (int j = 0; j < (SC > 0 ? SC : 8); ++j) {
            if (SC == 0 && (uint32_t)j >= S) break;
            if (j == 1) {
                const float2 xn = make_float2(fmaf(x.x, cd, -x.y * sd), fmaf(x.y, cd, x.x * sd));
                xp = x;
                x = xn;
            } else if (j >= 2) {
                const float2 xn = __ffma2_rn(tc2, x, make_float2(-xp.x, -xp.y));
                xp = x;
                x = xn;
            }
            const float4* v = gbuf + 2 * (l + 32 * j);
            const float4 g0 = v[0], g1 = v[1];
            const float2 q0 = make_float2(g0.x, g0.y), q1 = make_float2(g0.z, g0.w);
            const float2 q2 = make_float2(g1.x, g1.y), q3 = make_float2(g1.z, g1.w);
            P0 = __ffma2_rn(q0, x, P0);
            P1 = __ffma2_rn(q1, x, P1);
            P2 = __ffma2_rn(q2, x, P2);
            P3 = __ffma2_rn(q3, x, P3);
            const float uc = fmaf(k.qadx, q0.x, fmaf(k.qadz, q1.x, fmaf(k.akdx, q2.x, k.akdz * q3.x)));
            const float us = fmaf(k.a, q0.y, fmaf(k.qakxx, q1.y, fmaf(k.qakxz, q2.y, k.qakzz * q3.y)));
            const float gth = fmaf(us, x.x, -uc * x.y);
            G0 += gth;
            G1 = fmaf((float)j, gth, G1);
        }
        const float xl = fmaf((float)l, gx, xb), zl = fmaf((float)l, gz, zb);
        m[8] += G0;
        m[9] = fmaf(xl, G0, fmaf(32.0f * gx, G1, m[9]));
        m[10] = fmaf(zl, G0, fmaf(32.0f * gz, G1, m[10]));
    }
    m[0] = P0.x; m[1] = P0.y; m[2] = P1.x; m[5] = P1.y;
    m[3] = P2.x; m[6] = P2.y; m[4] = P3.x; m[7] = P3.y;
}

// Waves of the next phase-2 chunk, out of rem still to do: 32 while at least
// 32 remain; else the rest when it fills its power-of-two lane group to
// within an eighth (or is at most 3); else the largest power of two below it.
// A chunk's lanes idle where its waves fall short of the power of two, so a
// remainder of 20 waves runs as 16 + 4 (20 lanes' work) instead of as one
// 32-lane group.
__device__ __forceinline__ uint32_t adj_chunk_waves(uint32_t rem) {
    if (rem >= 32u) return 32u;
    if (rem <= 3u) return rem;
    const uint32_t P = 1u << (32 - __clz(rem - 1u));  // smallest power of two >= rem
    return 8u * (P - rem) <= P ? rem : P >> 1;
}

// SAVED: phase 1 reads the forward's saved sums instead of recomputing them
// (a compile-time switch, so that the recomputing kernel carries no test);
// both forms fit 96 registers and run 5 blocks (20 warps) per SM.
template <bool SAVED>
__global__ void __launch_bounds__(32 * kAdjWarps, 5)
k_adjoint(const wt_patch* __restrict__ patches, HmDev hm, const float* __restrict__ gpos,
          const float* __restrict__ gnrm, uint32_t flags, char* __restrict__ ws, AdjLayout L,
          const float4* __restrict__ sums) {
#if __CUDA_ARCH__ >= 900
    cudaGridDependencySynchronize();
#endif
    extern __shared__ float4 smem[];
    const int warp = threadIdx.x >> 5;
    const uint32_t lane = threadIdx.x & 31;
    float4* wst = smem + warp * (32 * kStage + kGbufVerts * kGbufF4);
    float4* gbuf = wst + 32 * kStage;
    WsHeader* hdr = reinterpret_cast<WsHeader*>(ws);
    const uint32_t* sorted = reinterpret_cast<const uint32_t*>(ws + L.f.sorted);
    const uint32_t* tile_pre = reinterpret_cast<const uint32_t*>(ws + L.f.tile_pre);
    const PatchAux* aux = reinterpret_cast<const PatchAux*>(ws + L.f.aux);
    const PairCoef* coef = reinterpret_cast<const PairCoef*>(ws + L.f.coef);
    const uint32_t* part_off = reinterpret_cast<const uint32_t*>(ws + L.part_off);
    const uint32_t* chunk_pre = reinterpret_cast<const uint32_t*>(ws + L.chunk_pre);
    float* partials = reinterpret_cast<float*>(ws + L.partials);
    const uint32_t n = hdr->n_patches;
    const uint32_t total = hdr->total_chunks;
    const uint32_t chunk = hdr->adj_chunk;
    const bool pow2 = hm.present && (hm.width & (hm.width - 1)) == 0 && (hm.height & (hm.height - 1)) == 0;
    const bool vec3 = (flags & WT_LAYOUT_VEC3) != 0;

    uint32_t t_next = 0;
    if (lane == 0) t_next = atomicAdd(&hdr->tile_counter, 1u);
    uint32_t t = __shfl_sync(0xffffffffu, t_next, 0);
    uint32_t q = 0;
    while (t < total) {
        if (lane == 0) t_next = atomicAdd(&hdr->tile_counter, 1u);
        if (chunk_pre[q + 1] <= t) {
            uint32_t step = 1, lo = q + 1, hi = q + 2;
            while (hi <= n && chunk_pre[hi] <= t) { lo = hi; step <<= 1; hi = lo + step; }
            hi = min(hi, n + 1);
            while (hi - lo > 1) {
                const uint32_t mid = (lo + hi) >> 1;
                if (chunk_pre[mid] <= t) lo = mid; else hi = mid;
            }
            q = lo;
        }
        const uint32_t p = sorted[q];
        const uint32_t lc = t - chunk_pre[q];
        const uint32_t lt0 = lc * chunk;
        const uint32_t lt1 = min(lt0 + chunk, tile_pre[q + 1] - tile_pre[q]);
        for (uint32_t lt = lt0; lt < lt1; ++lt) {
            const uint32_t cols = patches[p].cols;
            const uint32_t nwaves = patches[p].wave_count;
            const uint64_t out0 = patches[p].out_offset;
            const PatchAux a = aux[p];
            // the forward's tiling: 256-column tiles, each row's last tile narrower
            const uint32_t tpr = tiles_per_row(cols, 8);
            const uint32_t row = lt / tpr;
            const uint32_t c0 = (lt - row * tpr) * 256u;
            const uint32_t S = min(8u, (cols - c0 + 31u) / 32u);
            if (nwaves > 0) {
                const uint64_t rowbase = out0 + (uint64_t)row * cols;
                if (SAVED) {
                    // ---- phase 1 from the forward's saved sums: park them
                    for (uint32_t j = 0; j < S; ++j) {
                        const uint32_t col = c0 + lane + 32 * j;
                        float4* d = gbuf + kGbufF4 * (lane + 32 * j);
                        if (col < cols) {
                            d[0] = __ldcs(sums + 2 * (rowbase + col));
                            d[1] = __ldcs(sums + 2 * (rowbase + col) + 1);
                        }
                    }
                } else {
                    // ---- phase 1: forward sums recomputed, vertex per lane, in
                    // two 128-column halves of 4 vertices per lane (the forward's
                    // 4-vertex tiles; half the accumulator registers, so the
                    // kernel fits 5 blocks per SM)
                    for (uint32_t h = 0; h < 2; ++h) {
                        const uint32_t Sh = h == 0 ? min(S, 4u) : (S > 4u ? S - 4u : 0u);
                        if (Sh == 0) break;
                        const uint32_t ch = c0 + 128u * h;
                        float2 acc[4][4];
#pragma unroll
                        for (int j = 0; j < 4; ++j)
#pragma unroll
                            for (int mm = 0; mm < 4; ++mm) acc[j][mm] = make_float2(0.0f, 0.0f);
                        for (uint32_t w0 = 0; w0 < nwaves; w0 += 32) {
                            const uint32_t nw = min(32u, nwaves - w0);
                            __syncwarp();
                            if (lane < nw) stage_wave(coef[a.pair_offset + w0 + lane], ch, row, wst + kStage * lane);
                            __syncwarp();
                            wave_loop_dispatch<4>(Sh, acc, wst, nw, lane);
                        }
                        // park the eight sums of each vertex
#pragma unroll
                        for (int j = 0; j < 4; ++j) {
                            if ((uint32_t)j < Sh) {
                                float4* d = gbuf + kGbufF4 * (lane + 32 * (4 * h + j));
                                const VertexSums v = sums_of(acc[j]);
                                d[0] = make_float4(v.dx, v.dy, v.dz, v.jx);
                                d[1] = make_float4(v.jz, v.sxx, v.sxz, v.szz);
                            }
                        }
                    }
                }
                // then turn them into the vertex adjoints in a rolled loop (one
                // copy of that code)
                const float v = (float)row * a.inv_rm1;
                const float gx = (a.e1x + v * a.e3x) * a.inv_cm1, gz = (a.e1z + v * a.e3z) * a.inv_cm1;
                const float xb0 = fmaf((float)c0, gx, v * a.e2x), zb0 = fmaf((float)c0, gz, v * a.e2z);
                for (uint32_t j = 0; j < S; ++j) {
                    const uint32_t vi = lane + 32 * j;
                    const uint32_t col = c0 + vi;
                    float4* d = gbuf + kGbufF4 * vi;
                    float g[8] = {0, 0, 0, 0, 0, 0, 0, 0};
                    if (col < cols) {
                        const float4 s0 = d[0], s1 = d[1];
                        const float xl = fmaf((float)vi, gx, xb0), zl = fmaf((float)vi, gz, zb0);
                        VertexSums sm{s0.x, s0.y, s0.z, s0.w, s1.x, s1.y, s1.z, s1.w};
                        vertex_adjoint(sm, xl, zl, a, hm, pow2, gpos, gnrm, rowbase + col, vec3, g);
                    }
                    // (cos-sum, sin-sum) pairs: (dx, dy) (dz, sxx) | (jx, sxz) (jz, szz)
                    d[0] = make_float4(g[0], g[1], g[2], g[5]);
                    d[1] = make_float4(g[3], g[6], g[4], g[7]);
                }
                __syncwarp();
                // ---- phase 2: wave per lane, records of this tile
                const uint32_t nvalid0 = min(32u, cols - c0);  // valid lanes at j = 0
                const uint32_t rec0 = part_off[q] + lc * nwaves;
                for (uint32_t w0 = 0, nwc = 0; w0 < nwaves; w0 += nwc) {
                    // a chunk of nwc <= 32 waves: lanes form 32 / P groups of P
                    // lanes (P = nwc rounded up to a power of two); group g walks
                    // the vertex lanes l = g, g + G, ... and the groups' moments
                    // are combined by a fixed shuffle tree
                    nwc = adj_chunk_waves(nwaves - w0);
                    uint32_t P = 1;
                    while (P < nwc) P <<= 1;
                    const uint32_t G = 32u / P;
                    const uint32_t wl = lane & (P - 1), grp = lane / P;
                    const uint32_t wi = w0 + wl;
                    const bool active = wl < nwc;
                    const PairCoef k = coef[a.pair_offset + (active ? wi : w0)];
                    float4 st[3];
                    stage_wave(k, c0, row, st);
                    float m[11];
#pragma unroll
                    for (int i = 0; i < 11; ++i) m[i] = 0.0f;
                    const uint32_t t32 = __float_as_uint(st[0].x), a32 = __float_as_uint(st[0].y);
                    if (S == 8)
                        wave_moments<8>(gbuf, 8, grp, G, nvalid0, t32, a32, st[0].z, st[0].w, k, xb0, zb0, gx, gz, m);
                    else
                        wave_moments<0>(gbuf, S, grp, G, nvalid0, t32, a32, st[0].z, st[0].w, k, xb0, zb0, gx, gz, m);
                    for (uint32_t o = P; o < 32; o <<= 1) {
#pragma unroll
                        for (int i = 0; i < 11; ++i) m[i] += __shfl_down_sync(0xffffffffu, m[i], o);
                    }
                    if (active && grp == 0) {
                        // the chunk's tiles add into one record, in tile order
                        // (the same lane writes it for every tile of the chunk)
                        float* r = partials + (size_t)kAdjRecord * (rec0 + wi);
                        if (lt == lt0) {
#pragma unroll
                            for (int i = 0; i < 11; ++i) r[i] = m[i];
                        } else {
#pragma unroll
                            for (int i = 0; i < 11; ++i) r[i] += m[i];
                        }
                    }
                }
                __syncwarp();
            }
        }  // tiles of the chunk
        t = __shfl_sync(0xffffffffu, t_next, 0);
    }
}

// Column sums of the records.  A patch's records form a [tiles][waves * 11]
// matrix; block (x, y) sums columns 32x .. 32x+31 of patch y over its tiles:
// 32 tile-lanes per column, each summing every 32nd tile in order with Kahan
// compensation (FP32: this part's FP64 rate is low), combined in a fixed
// order.  Output: colsum[pair][11] (FP32).
constexpr int kColLanes = 32;

__global__ void __launch_bounds__(32 * kColLanes) k_adj_cols(uint32_t n, const char* __restrict__ ws, AdjLayout L) {
#if __CUDA_ARCH__ >= 900
    cudaGridDependencySynchronize();
#endif
    __shared__ float red[kColLanes][32];
    const uint32_t* pair_off = reinterpret_cast<const uint32_t*>(ws + L.f.pair_off);
    const uint32_t* chunk_pre = reinterpret_cast<const uint32_t*>(ws + L.chunk_pre);
    const uint32_t* rank = reinterpret_cast<const uint32_t*>(ws + L.rank);
    const uint32_t* part_off = reinterpret_cast<const uint32_t*>(ws + L.part_off);
    const float* partials = reinterpret_cast<const float*>(ws + L.partials);
    const WsHeader* hdr = reinterpret_cast<const WsHeader*>(ws);
    float* colsum = reinterpret_cast<float*>(const_cast<char*>(ws) + L.colsum);
    const bool ran = hdr->total_chunks > 0;
    const uint32_t cl = threadIdx.x & 31, tl = threadIdx.x >> 5;
    for (uint32_t p = blockIdx.y; p < n; p += gridDim.y) {
        const uint32_t nw = pair_off[p + 1] - pair_off[p];
        const uint32_t width = nw * kAdjRecord;
        const uint32_t col = blockIdx.x * 32 + cl;
        if (blockIdx.x * 32 >= width) continue;  // block-uniform
        const uint32_t qs = rank[p];
        const uint32_t ntiles = chunk_pre[qs + 1] - chunk_pre[qs];  // records per column
        const float* base = partials + (size_t)kAdjRecord * part_off[qs];
        float sum = 0.0f, comp = 0.0f;
        if (ran && col < width) {
#pragma unroll 8
            for (uint32_t t = tl; t < ntiles; t += kColLanes) {
                const float y = base[(size_t)t * width + col] - comp;
                const float tt = sum + y;
                comp = (tt - sum) - y;
                sum = tt;
            }
        }
        __syncthreads();
        red[tl][cl] = sum;
        __syncthreads();
        if (tl == 0 && col < width) {
            float total = 0.0f;
#pragma unroll 8
            for (int i = 0; i < kColLanes; ++i) total += red[i][cl];
            colsum[(size_t)kAdjRecord * pair_off[p] + col] = total;
        }
    }
}

// Closed-form FP64 gradient of every (patch, wave) pair from its eleven
// column sums, one pair per thread (GB300's FP64 rate is low: a warp per
// wave with one busy lane spent 16 us here on 64 patches).
__global__ void __launch_bounds__(256) k_adj_pairs(const wt_patch* __restrict__ patches, uint32_t n,
                                                   const wt_wave* __restrict__ waves, const char* __restrict__ ws,
                                                   AdjLayout L) {
#if __CUDA_ARCH__ >= 900
    cudaGridDependencySynchronize();
#endif
    const uint32_t* pair_off_g = reinterpret_cast<const uint32_t*>(ws + L.f.pair_off);
    const float* colsum = reinterpret_cast<const float*>(ws + L.colsum);
    double* g64 = reinterpret_cast<double*>(const_cast<char*>(ws) + L.pair_g64);
    constexpr uint32_t kSmemOffsets = 4096;
    __shared__ uint32_t off_s[kSmemOffsets];
    const bool in_smem = n + 1 <= kSmemOffsets;
    if (in_smem)
        for (uint32_t i = threadIdx.x; i <= n; i += blockDim.x) off_s[i] = pair_off_g[i];
    __syncthreads();
    const uint32_t* pair_off = in_smem ? off_s : pair_off_g;
    const uint32_t total = pair_off[n];
    for (uint32_t P = blockIdx.x * blockDim.x + threadIdx.x; P < total; P += gridDim.x * blockDim.x) {
        uint32_t lo = 0, hi = n + 1;
        while (lo < hi) {
            const uint32_t mid = (lo + hi) >> 1;
            if (pair_off[mid] <= P) lo = mid + 1; else hi = mid;
        }
        const uint32_t p = lo - 1;
        const wt_wave w = waves[patches[p].wave_offset + (P - pair_off[p])];
        const double lam = w.wavelength;
        const double k = isinf(lam) ? 0.0 : kTwoPi / lam;
        const double A = w.amplitude, Q = w.steepness_q, Dx = w.dir_x, Dz = w.dir_z, sp = w.speed;
        const float* m = colsum + (size_t)kAdjRecord * P;
        const double t = patches[p].time_s;
        const double Mdx = m[0], Mdy = m[1], Mdz = m[2], Mjx = m[3], Mjz = m[4];
        const double Mxx = m[5], Mxz = m[6], Mzz = m[7], T0 = m[8];
        const double Xw = (double)m[9] + (double)patches[p].bl[0] * T0;
        const double Zw = (double)m[10] + (double)patches[p].bl[1] * T0;
        const double P3 = Dx * Dx * Mxx + Dx * Dz * Mxz + Dz * Dz * Mzz;
        const double gk = A * (Dx * Mjx + Dz * Mjz + Q * P3) + Dx * Xw + Dz * Zw + sp * t * T0;
        const double gDx = Q * A * Mdx + A * k * Mjx + Q * A * k * (2.0 * Dx * Mxx + Dz * Mxz) + k * Xw;
        const double gDz = Q * A * Mdz + A * k * Mjz + Q * A * k * (2.0 * Dz * Mzz + Dx * Mxz) + k * Zw;
        double* g = g64 + 8 * (size_t)P;
        g[0] = Q * (Dx * Mdx + Dz * Mdz) + k * (Dx * Mjx + Dz * Mjz) + Mdy + Q * k * P3;
        g[1] = isinf(lam) ? 0.0 : -gk * k / lam;
        g[2] = -Dz * gDx + Dx * gDz;
        g[3] = A * (Dx * Mdx + Dz * Mdz + k * P3);
        g[4] = T0;
        g[5] = k * t * T0;
        g[6] = gDx;
        g[7] = gDz;
    }
}

// One warp per wave: lane l takes patches l, l+32, ... that use the wave and
// adds their pair gradients; the lanes are then combined by a fixed shuffle
// tree, or, when one lane alone holds a contribution (a wave used by one
// patch), taken from it.
__global__ void __launch_bounds__(256) k_adj_waves(const wt_patch* __restrict__ patches, uint32_t n,
                                                   uint32_t n_waves, const char* __restrict__ ws, AdjLayout L,
                                                   wt_wave_grad* __restrict__ grad) {
#if __CUDA_ARCH__ >= 900
    cudaGridDependencySynchronize();
#endif
    const uint32_t* pair_off = reinterpret_cast<const uint32_t*>(ws + L.f.pair_off);
    const double* g64 = reinterpret_cast<const double*>(ws + L.pair_g64);
    const uint32_t lane = threadIdx.x & 31;
    const uint32_t warps = (gridDim.x * blockDim.x) >> 5;
    for (uint32_t wi = (blockIdx.x * blockDim.x + threadIdx.x) >> 5; wi < n_waves; wi += warps) {
        double g[8] = {0, 0, 0, 0, 0, 0, 0, 0};
        bool has = false;
        for (uint32_t p = lane; p < n; p += 32) {
            const uint32_t nw = pair_off[p + 1] - pair_off[p];  // 0 for invalid patches
            const uint32_t off = patches[p].wave_offset;
            if (nw == 0 || wi < off || wi - off >= nw) continue;
            has = true;
            const double* q = g64 + 8 * (size_t)(pair_off[p] + (wi - off));
#pragma unroll
            for (int i = 0; i < 8; ++i) g[i] += q[i];
        }
        const unsigned holders = __ballot_sync(0xffffffffu, has);
        if (holders != 0 && (holders & (holders - 1)) == 0) {
            const int src = __ffs(holders) - 1;
#pragma unroll
            for (int i = 0; i < 8; ++i) g[i] = __shfl_sync(0xffffffffu, g[i], src);
        } else if (holders != 0) {
#pragma unroll
            for (int i = 0; i < 8; ++i)
                for (int o = 16; o > 0; o >>= 1) g[i] += __shfl_xor_sync(0xffffffffu, g[i], o);
        }
        if (lane == 0) {
            wt_wave_grad o;
            o.d_amplitude = (float)g[0];
            o.d_wavelength = (float)g[1];
            o.d_direction = (float)g[2];
            o.d_steepness_q = (float)g[3];
            o.d_phase = (float)g[4];
            o.d_speed = (float)g[5];
            o.d_dir_x = (float)g[6];
            o.d_dir_z = (float)g[7];
            grad[wi] = o;
        }
    }
}

int device_sms() { return sm_count(); }

template <typename K, typename... Args>
cudaError_t launch_pdl(K kernel, dim3 grid, dim3 block, size_t smem, cudaStream_t s, Args... args) {
    cudaLaunchConfig_t lc = {};
    lc.gridDim = grid;
    lc.blockDim = block;
    lc.dynamicSmemBytes = smem;
    lc.stream = s;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
    attr[0].val.programmaticStreamSerializationAllowed = 1;
    lc.attrs = attr;
    lc.numAttrs = 1;
    return cudaLaunchKernelEx(&lc, kernel, args...);
}

constexpr size_t kAdjSmem = sizeof(float4) * kAdjWarps * (32 * kStage + kGbufVerts * kGbufF4);

// Resident blocks per SM of the main kernel (read once per device and
// variant; sets its shared-memory attribute on the way).
template <bool SAVED>
cudaError_t adj_occupancy(int* occ_out) {
    static std::atomic<int> occ_cache[64];
    int dev = 0;
    cudaGetDevice(&dev);
    if (dev < 0 || dev >= 64) return cudaErrorInvalidDevice;
    int occ = occ_cache[dev].load(std::memory_order_relaxed);
    if (occ == 0) {
        cudaError_t e = cudaFuncSetAttribute(k_adjoint<SAVED>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                             (int)kAdjSmem);
        if (e != cudaSuccess) return e;
        int o = 0;
        e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&o, k_adjoint<SAVED>, 32 * kAdjWarps, kAdjSmem);
        if (e != cudaSuccess) return e;
        occ = o < 1 ? 1 : o;
        occ_cache[dev].store(occ, std::memory_order_relaxed);
    }
    *occ_out = occ;
    return cudaSuccess;
}

// The persistent main kernel: one grid of SMs x resident blocks.
template <bool SAVED>
cudaError_t launch_adj_main(int sms, int occ, cudaStream_t s, const wt_patch* patches, const HmDev& hm,
                            const float* gpos, const float* gnrm, uint32_t flags, char* w, const AdjLayout& L,
                            const float* sums) {
    return launch_pdl(k_adjoint<SAVED>, dim3(sms * occ), dim3(32 * kAdjWarps), kAdjSmem, s, patches, hm, gpos,
                      gnrm, flags, w, L, reinterpret_cast<const float4*>(sums));
}

}  // namespace

cudaError_t adjoint_scan_args(bool saved, const AdjLayout& L, AdjScanArgs* out) {
    const int sms = device_sms();
    if (sms <= 0) return cudaErrorInvalidDevice;
    int occ = 1;
    cudaError_t e = saved ? adj_occupancy<true>(&occ) : adj_occupancy<false>(&occ);
    if (e != cudaSuccess) return e;
    out->L = L;
    out->chunk_max = saved ? kAdjChunkSaved : kAdjChunkRecompute;
    out->min_tiles = kAdjChunkMinTilesPerWarp * (uint32_t)(sms * occ * kAdjWarps);
    return cudaSuccess;
}

uint64_t adjoint_records(const wt_patch& p) {
    if (p.cols < 2 || p.rows < 2) return 0;
    return (uint64_t)p.rows * dev::tiles_per_row(p.cols, 8) * p.wave_count;  // chunks of one tile
}

cudaError_t launch_adjoint(const wt_patch* patches, uint32_t n_patches, const wt_wave* waves, uint32_t n_waves,
                           uint32_t max_waves_per_patch, const HmDev& hm, const float* gpos, const float* gnrm,
                           uint32_t flags, wt_wave_grad* grad, void* ws, const AdjLayout& L, const float* sums,
                           cudaStream_t s) {
    char* w = static_cast<char*>(ws);
    const int sms = device_sms();
    int occ = 1;
    cudaError_t e = sums ? adj_occupancy<true>(&occ) : adj_occupancy<false>(&occ);
    if (e != cudaSuccess) return e;
    e = sums ? launch_adj_main<true>(sms, occ, s, patches, hm, gpos, gnrm, flags, w, L, sums)
             : launch_adj_main<false>(sms, occ, s, patches, hm, gpos, gnrm, flags, w, L, nullptr);
    if (e != cudaSuccess) return e;
    const dim3 cg((max_waves_per_patch * kAdjRecord + 31) / 32, n_patches < 65535u ? n_patches : 65535u);
    e = launch_pdl(k_adj_cols, cg, dim3(32 * kColLanes), 0, s, n_patches, static_cast<const char*>(ws), L);
    if (e != cudaSuccess) return e;
    const unsigned wb = (n_waves + 7) / 8 < (unsigned)sms * 16 ? (n_waves + 7) / 8 : (unsigned)sms * 16;
    if (wb == 0) return cudaSuccess;
    e = launch_pdl(k_adj_pairs, dim3((unsigned)sms), dim3(256), 0, s, patches, n_patches, waves,
                   static_cast<const char*>(ws), L);
    if (e != cudaSuccess) return e;
    return launch_pdl(k_adj_waves, dim3(wb), dim3(256), 0, s, patches, n_patches, n_waves,
                      static_cast<const char*>(ws), L, grad);
}

}  // namespace wt
