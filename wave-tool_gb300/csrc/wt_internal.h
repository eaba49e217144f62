// wt_internal.h — shared declarations of the host API (wt_api.cpp) and the
// kernels (*.cu).  Not part of the public ABI.
#pragma once
#include <cstddef>
#include <cstdint>

#include <cuda_runtime.h>

#include "../../include/wt.h"

namespace wt {

// ---- workspace layout ------------------------------------------------------
// [0, 256)                 WsHeader
// sorted   u32[n_patches]  patch indices, descending wave count (LPT order)
// tile_pre u32[n+1]        exclusive prefix of tiles over the sorted order
// pair_off u32[n+1]        exclusive prefix of wave_count (original order)
// tiles    u32[n]          tile count per patch (original order, 0 = invalid)
// aux      PatchAux[n]
// coef     PairCoef[total_wave_slots]
struct WsHeader {
    uint32_t status;       // wt_status of device-side validation (0 = ok)
    uint32_t bad_patch;    // smallest offending patch index (0xffffffff none)
    uint32_t tile_counter; // dynamic tile queue head
    uint32_t total_tiles;
    uint32_t n_patches;
    uint32_t tile_cols;    // vertices per tile row (32 * S)
    uint32_t total_chunks; // adjoint: tile chunks in its queue (0 = do not run)
    uint32_t adj_chunk;    // adjoint: tiles per chunk
    uint32_t pad[56];
};
static_assert(sizeof(WsHeader) == 256, "header size");

// Per-patch constants, computed once per launch by the prep kernel.
struct alignas(16) PatchAux {
    float e1x, e1z;     // BR - BL          (local frame, metres)
    float e2x, e2z;     // TL - BL
    float e3x, e3z;     // TR - TL - BR + BL
    float blx, blz;     // world BL (for world-space output)
    float inv_cm1;      // 1 / (cols - 1)
    float inv_rm1;      // 1 / (rows - 1)
    float hu0, hv0;     // heightmap texel coordinate of BL, reduced by the wrap period, minus 0.5
    float su, sv;       // texels per metre along x and along z (sv carries the -z flip)
    float y_offset;
    uint32_t pair_offset;
};
static_assert(sizeof(PatchAux) == 64, "aux size");

// Per-(patch, wave) constants.  The phase theta(col, row) of the wave on the
// patch's bilinear grid is, exactly,
//   theta = theta00 + col*a + row*b + col*row*g
// and is carried in turns (theta / 2pi) as 64-bit fixed point mod 1, so that
// integer wrap-around performs the mod-2pi reduction for free.
struct alignas(16) PairCoef {
    unsigned long long t00, ta, tb, tg;  // turns * 2^64
    float qadx, a, qadz, akdx;           // Q*A*Dx, A, Q*A*Dz, A*k*Dx
    float akdz, qakxx, qakxz, qakzz;     // A*k*Dz, Q*A*k*Dx^2, Q*A*k*Dx*Dz, Q*A*k*Dz^2
};
static_assert(sizeof(PairCoef) == 64, "coef size");

struct WsLayout {
    size_t sorted, tile_pre, pair_off, tiles, aux, coef, end;
};

inline size_t align_up(size_t x, size_t a) { return (x + a - 1) / a * a; }

inline WsLayout ws_layout(uint32_t n_patches, uint64_t total_wave_slots) {
    WsLayout L;
    size_t o = sizeof(WsHeader);
    L.sorted = o;   o = align_up(o + 4ull * n_patches, 16);
    L.tile_pre = o; o = align_up(o + 4ull * (n_patches + 1), 16);
    L.pair_off = o; o = align_up(o + 4ull * (n_patches + 1), 16);
    L.tiles = o;    o = align_up(o + 4ull * n_patches, 64);
    L.aux = o;      o = align_up(o + sizeof(PatchAux) * (size_t)n_patches, 64);
    L.coef = o;     o = align_up(o + sizeof(PairCoef) * (size_t)total_wave_slots, 256);
    L.end = o;
    return L;
}

// Adjoint workspace: the forward layout (prep stages are shared), then
// rank     u32[n]      sorted position of each patch
// partoff  u32[n+1]    exclusive prefix of records (chunks x waves) over the sorted order
// chunkpre u32[n+1]    exclusive prefix of tile chunks over the sorted order
// partial  float[11 x records]   per-(chunk, wave) FP32 partial sums
// colsum   float[11 x wave slots] per-(patch, wave) sums of the records
// pairg    double[8 x wave slots] per-(patch, wave) closed-form gradients
constexpr int kAdjRecord = 11;

struct AdjLayout {
    WsLayout f;
    size_t rank, part_off, chunk_pre, partials, colsum, pair_g64, end;
    uint64_t cap_records;
};

inline AdjLayout adj_layout(uint32_t n_patches, uint64_t total_wave_slots, uint64_t records) {
    AdjLayout A;
    A.f = ws_layout(n_patches, total_wave_slots);
    size_t o = A.f.end;
    A.rank = o;      o = align_up(o + 4ull * n_patches, 16);
    A.part_off = o;  o = align_up(o + 4ull * (n_patches + 1), 16);
    A.chunk_pre = o; o = align_up(o + 4ull * (n_patches + 1), 256);
    A.partials = o;  o = align_up(o + 4ull * kAdjRecord * records, 256);
    A.colsum = o;    o = align_up(o + 4ull * kAdjRecord * total_wave_slots, 256);
    A.pair_g64 = o;  o = align_up(o + 8ull * 8 * total_wave_slots, 256);
    A.end = o;
    A.cap_records = records;
    return A;
}

// Tuning of the forward launch.
struct FwdConfig {
    int s;              // vertices per lane per tile row (tile = 32*s columns)
    int chunk;          // waves staged per warp at a time (<= 32)
    int warps;          // warps per block
    int blocks_per_sm;  // persistent grid = SMs * blocks_per_sm (0 = occupancy max)
    int epi;            // 0: epilogue from registers, 1: through shared memory
};

// Outputs of the vertex stage (any may be NULL): clip float4, ndc0 float2,
// view / facing / nyaw in the call's vertex layout.
struct StageOut {
    float* clip;
    float* ndc0;
    float* view;
    float* facing;
    float* nyaw;
};

// Optional extra outputs of the forward (at most one of the two is set):
// sums: 8 floats per output vertex (its wave sums, for the adjoint);
// view: device wt_view, with `stage` the vertex-stage outputs written by the
// forward's own epilogue (float4 layouts, world positions).
struct FwdExtra {
    float* sums;
    const wt_view* view;
    StageOut stage;
};

struct HmDev {
    const float* texels;
    uint32_t width, height;
    float sample_scale, disp_scale;
    uint32_t wrap;
    int present;
};

// The adjoint's queue set-up (ranks, chunk and record prefixes), formed by the
// prep's scan kernel when the prep runs for an adjoint.
struct AdjScanArgs {
    AdjLayout L;
    uint32_t chunk_max;  // tiles per chunk when there are enough tiles
    uint32_t min_tiles;  // below this many tiles, chunks of one tile
};

// ---- launchers (wt_displace.cu) -------------------------------------------
// tile_cols: tile width (each row's last tile narrower, see tiles_per_row)
cudaError_t launch_prep(const wt_patch* patches, uint32_t n_patches, const wt_wave* waves,
                        uint32_t n_waves, const HmDev& hm, uint64_t out_capacity,
                        uint32_t tile_cols, void* ws, const WsLayout& L, cudaStream_t s,
                        const AdjScanArgs* adj = nullptr);
// pos may be NULL only with x.view set
cudaError_t launch_forward(const FwdConfig& cfg, const wt_patch* patches, uint32_t n_patches,
                           const HmDev& hm, float* pos, float* nrm, uint32_t flags, void* ws,
                           const WsLayout& L, const FwdExtra& x, cudaStream_t s);
cudaError_t launch_forward_naive(const wt_patch* patches, uint32_t n_patches, const wt_wave* waves,
                                 const HmDev& hm, float* pos, float* nrm, uint32_t flags,
                                 void* ws, const WsLayout& L, uint64_t total_vertices,
                                 cudaStream_t s);
bool forward_config_supported(const FwdConfig& cfg);

// ---- adjoint (wt_adjoint.cu) ----------------------------------------------
// Records (tile chunks x waves) of one patch, as the adjoint lays them out.
uint64_t adjoint_records(const wt_patch& p);
// The scan arguments of an adjoint over layout L (saved: from saved sums).
cudaError_t adjoint_scan_args(bool saved, const AdjLayout& L, AdjScanArgs* out);
// sums: NULL (phase 1 recomputes the forward sums) or the forward's saved sums;
// the prep ran with adjoint_scan_args
cudaError_t launch_adjoint(const wt_patch* patches, uint32_t n_patches, const wt_wave* waves, uint32_t n_waves,
                           uint32_t max_waves_per_patch, const HmDev& hm, const float* gpos, const float* gnrm,
                           uint32_t flags, wt_wave_grad* grad, void* ws, const AdjLayout& L, const float* sums,
                           cudaStream_t s);

// ---- host helpers (wt_api.cpp) ---------------------------------------------
void set_last_error(const char* msg);  // message returned by wt_last_error() on this thread
FwdConfig forward_config(uint32_t n_patches, uint32_t n_waves);  // tuning in effect for this shape
// SM count of the current device (cached per device; 0 if it cannot be read)
int sm_count();

// ---- misc kernels (wt_misc.cu) --------------------------------------------
cudaError_t launch_indices(uint32_t cols, uint32_t rows, uint32_t base, uint32_t* out, cudaStream_t s);
cudaError_t launch_unorm8(const uint8_t* px, uint32_t w, uint32_t h, uint32_t channels, uint64_t stride,
                          uint32_t flip, float* out, cudaStream_t s);
// rates: NULL or per-term phase rates (radians per second) at time t
cudaError_t launch_noise(const wt_noise_term* terms, uint32_t n_terms, const float* rates, double t, uint32_t w,
                         uint32_t h, float* out, void* ws, cudaStream_t s);
size_t noise_workspace_bytes(uint32_t n_terms, uint32_t w, uint32_t h);
cudaError_t measure_peaks(void* scratch, size_t bytes, double* fma, double* sin, cudaStream_t s);

}  // namespace wt
