// wt_displace.cu — forward Gerstner path on sm_103a.
//
// Replaces the per-vertex work of assets/shaders/water-grid.vert:114-194
// (grid bilerp :87-91, Gerstner sum :74-85, heightmap :93-111 sampled at the
// displaced point :141-144, bounce :147, normal :164-190) and the uniform
// upload of src/render-engine.cpp:1057-1110 (steepness already normalised by
// the caller, :1073).
//
// Three launches (two when the table has at most 1024 (patch, wave) pairs),
// all stream-ordered and graph-capturable:
//   k_prep_scan  (1 block)   validate patches and waves, prefix sums, LPT sort
//                            of patches by wave count, tile queue reset
//   k_prep_coef  (grid)      FP64 per-(patch, wave) phase constants in 64-bit
//                            fixed-point turns + FP32 sum coefficients;
//                            per-patch local frame; runs alongside the scan
//   k_forward    (persistent) one tile = one patch row segment of 32*S
//                            vertices per warp; lane l owns columns
//                            c0 + l + 32 j, j < S.  Per wave: one MUFU sincos
//                            per lane, an exact rotation to the second vertex,
//                            then the Chebyshev recurrence on the FMA pipe; 8
//                            FMAs, issued as 4 paired FP32 FMAs, accumulate
//                            displacement and the surface Jacobian.  Epilogue:
//                            heightmap bilerp + gradient, exact normal,
//                            streaming stores (and, by variant, the wave sums
//                            or the vertex stage).
#include <cuda_runtime.h>

#include <atomic>
#include <cstdint>

#include "wt_device.cuh"
#include "wt_internal.h"

namespace wt {
namespace {

using namespace wt::dev;

constexpr uint32_t kNoPatch = 0xffffffffu;
constexpr int kSortBins = 1024;         // wave counts >= 1023 share the last bin
constexpr uint32_t kWaveMaskWords = 512;  // waves validated into a shared bitmask up to 16384
constexpr uint32_t kRankSortMax = 64;


__device__ __forceinline__ void flag_error(WsHeader* h, uint32_t code, uint32_t patch) {
    atomicCAS(&h->status, 0u, code);
    atomicMin(&h->bad_patch, patch);
}

__device__ __forceinline__ bool finitef(float x) { return isfinite(x); }

__device__ bool wave_ok(const wt_wave& w) {
    bool lam_ok = (w.wavelength > 0.0f) && !isnan(w.wavelength);  // +inf allowed (k = 0)
    return lam_ok && finitef(w.amplitude) && finitef(w.dir_x) && finitef(w.dir_z) &&
           finitef(w.steepness_q) && finitef(w.speed) && finitef(w.phase);
}

__device__ __forceinline__ unsigned long long to_fixed_turns(double turns) {
    double f = turns - floor(turns);                 // [0, 1)
    double hi = floor(f * 4294967296.0);             // < 2^32
    double lo = floor((f * 4294967296.0 - hi) * 4294967296.0);
    return ((unsigned long long)hi << 32) | (unsigned long long)lo;
}

// positive remainder of x by m (FP64)
__device__ __forceinline__ double pmod(double x, double m) {
    double r = x - m * floor(x / m);
    return r >= m ? r - m : (r < 0.0 ? r + m : r);
}

// FP64 constants of wave w on patch Pt (the phase on the patch's bilinear grid
// as 64-bit fixed-point turns, and the FP32 coefficients of the eight sums).
__device__ PairCoef make_pair_coef(const wt_patch& Pt, const wt_wave w) {
    double lam = w.wavelength;
    double inv_lam = isinf(lam) ? 0.0 : 1.0 / lam;     // k / 2pi
    double k = kTwoPi * inv_lam;
    double Dx = w.dir_x, Dz = w.dir_z, A = w.amplitude, Q = w.steepness_q;
    double blx = Pt.bl[0], blz = Pt.bl[1];
    double e1x = (double)Pt.br[0] - blx, e1z = (double)Pt.br[1] - blz;
    double e2x = (double)Pt.tl[0] - blx, e2z = (double)Pt.tl[1] - blz;
    double e3x = (double)Pt.tr[0] - Pt.tl[0] - Pt.br[0] + blx;
    double e3z = (double)Pt.tr[1] - Pt.tl[1] - Pt.br[1] + blz;
    const double inv_cm1 = 1.0 / (double)(Pt.cols - 1), inv_rm1 = 1.0 / (double)(Pt.rows - 1);
    // theta / 2pi at (col, row) = t00 + col*ta + row*tb + col*row*tg
    double t00 = (Dx * blx + Dz * blz) * inv_lam + (double)w.speed * Pt.time_s * inv_lam +
                 (double)w.phase * (1.0 / kTwoPi);
    double ta = (Dx * e1x + Dz * e1z) * inv_lam * inv_cm1;
    double tb = (Dx * e2x + Dz * e2z) * inv_lam * inv_rm1;
    double tg = (Dx * e3x + Dz * e3z) * inv_lam * (inv_cm1 * inv_rm1);
    PairCoef c;
    c.t00 = to_fixed_turns(t00);
    c.ta = to_fixed_turns(ta);
    c.tb = to_fixed_turns(tb);
    c.tg = to_fixed_turns(tg);
    c.qadx = (float)(Q * A * Dx);
    c.a = (float)A;
    c.qadz = (float)(Q * A * Dz);
    c.akdx = (float)(A * k * Dx);
    c.akdz = (float)(A * k * Dz);
    c.qakxx = (float)(Q * A * k * Dx * Dx);
    c.qakxz = (float)(Q * A * k * Dx * Dz);
    c.qakzz = (float)(Q * A * k * Dz * Dz);
    return c;
}

// Per-patch constants: local frame, steps, texel origin reduced by the wrap
// period in FP64, bounce, first coefficient slot.
__device__ PatchAux make_patch_aux(const wt_patch& Pt, const HmDev& hm, uint32_t pair_offset) {
    double blx = Pt.bl[0], blz = Pt.bl[1];
    PatchAux a;
    a.e1x = (float)((double)Pt.br[0] - blx);
    a.e1z = (float)((double)Pt.br[1] - blz);
    a.e2x = (float)((double)Pt.tl[0] - blx);
    a.e2z = (float)((double)Pt.tl[1] - blz);
    a.e3x = (float)((double)Pt.tr[0] - Pt.tl[0] - Pt.br[0] + blx);
    a.e3z = (float)((double)Pt.tr[1] - Pt.tl[1] - Pt.br[1] + blz);
    a.blx = Pt.bl[0];
    a.blz = Pt.bl[1];
    a.inv_cm1 = Pt.cols > 1 ? 1.0f / (float)(Pt.cols - 1) : 0.0f;
    a.inv_rm1 = Pt.rows > 1 ? 1.0f / (float)(Pt.rows - 1) : 0.0f;
    if (hm.present) {
        double W = hm.width, H = hm.height;
        double pu = hm.wrap == WT_WRAP_MIRRORED_REPEAT ? 2.0 * W : W;
        double pv = hm.wrap == WT_WRAP_MIRRORED_REPEAT ? 2.0 * H : H;
        // texel coordinate of the world point X: sample_scale*W*X - 0.5;
        // the BL part is reduced by the wrap period in FP64
        a.hu0 = (float)(pmod((double)hm.sample_scale * W * blx, pu) - 0.5);
        a.hv0 = (float)(pmod(-(double)hm.sample_scale * H * blz, pv) - 0.5);
        a.su = (float)((double)hm.sample_scale * W);
        a.sv = (float)(-(double)hm.sample_scale * H);
    } else {
        a.hu0 = a.hv0 = a.su = a.sv = 0.0f;
    }
    a.y_offset = Pt.y_offset;
    a.pair_offset = pair_offset;
    return a;
}

// ---- stage 1: validation, prefix sums, LPT order ---------------------------
__device__ __forceinline__ bool patch_ok(const wt_patch& P, uint32_t n_waves, uint64_t out_capacity) {
    const uint64_t verts = (uint64_t)P.cols * P.rows;
    return P.cols >= 2 && P.rows >= 2 && P.cols <= (1u << 20) && P.rows <= (1u << 20) && verts < (1ull << 31) &&
           P.flags == 0 && (uint64_t)P.wave_offset + P.wave_count <= n_waves && P.out_offset <= out_capacity &&
           verts <= out_capacity - P.out_offset && finitef(P.bl[0]) && finitef(P.bl[1]) && finitef(P.br[0]) &&
           finitef(P.br[1]) && finitef(P.tl[0]) && finitef(P.tl[1]) && finitef(P.tr[0]) && finitef(P.tr[1]) &&
           isfinite(P.time_s) && finitef(P.y_offset);
}

// Tables of at most kSmallPrep patches whose constants are formed here too
// (k_prep_scan with fuse_coef): the whole prep through shared memory, with
// two dependent global loads (the patches, then each pair's wave) instead of
// the general path's chain of global-memory scans.  Writes what the general
// path writes: header, pair and tile prefixes, the order, tiles, the
// constants and, for the adjoint, its queue (adj_scan_body's arrays).
constexpr uint32_t kSmallPrep = 32;

__device__ void prep_small(const wt_patch* __restrict__ patches, uint32_t n, const wt_wave* __restrict__ waves,
                           uint32_t n_waves, uint64_t out_capacity, uint64_t coef_capacity, uint32_t tile_cols,
                           char* ws, const WsLayout& L, const HmDev& hm, int do_adj, const AdjLayout& AL,
                           uint32_t adj_chunk_max, uint32_t adj_min_tiles) {
    __shared__ wt_patch sp[kSmallPrep];
    __shared__ uint32_t s_sorted[kSmallPrep];      // patch at each sorted rank
    __shared__ uint32_t s_off[kSmallPrep + 1];     // pair prefix over the structurally valid patches
    __shared__ uint32_t s_rank_tiles[kSmallPrep];  // tiles of the patch at each sorted rank
    __shared__ uint32_t s_struct_bad, s_wave_bad;  // bit p: patch p fails that check
    WsHeader* hdr = reinterpret_cast<WsHeader*>(ws);
    uint32_t* sorted = reinterpret_cast<uint32_t*>(ws + L.sorted);
    uint32_t* tile_pre = reinterpret_cast<uint32_t*>(ws + L.tile_pre);
    uint32_t* pair_off = reinterpret_cast<uint32_t*>(ws + L.pair_off);
    uint32_t* tiles_g = reinterpret_cast<uint32_t*>(ws + L.tiles);
    PatchAux* aux = reinterpret_cast<PatchAux*>(ws + L.aux);
    PairCoef* coef = reinterpret_cast<PairCoef*>(ws + L.coef);
    const uint32_t tid = threadIdx.x, lane = tid & 31u;
    constexpr unsigned kAll = 0xffffffffu;

    if (tid < n) sp[tid] = patches[tid];
    if (tid == 0) s_wave_bad = 0;
    __syncthreads();
    uint32_t tiles_p = 0;  // warp 0: lane p's patch
    if (tid < 32) {
        bool ok = false;
        uint32_t wc = 0;
        if (tid < n) {
            const wt_patch& P = sp[tid];
            ok = patch_ok(P, n_waves, out_capacity);
            wc = ok ? P.wave_count : 0u;
            tiles_p = ok ? P.rows * tiles_per_row(P.cols, tile_cols / 32) : 0u;
        }
        uint32_t x = wc;  // inclusive prefix of the pair counts
        for (int o = 1; o < 32; o <<= 1) {
            const uint32_t y = __shfl_up_sync(kAll, x, o);
            if (lane >= (uint32_t)o) x += y;
        }
        if (tid < n) s_off[tid + 1] = x;
        if (tid == 0) s_off[0] = 0;
        const unsigned bad = __ballot_sync(kAll, tid < n && !ok);
        if (tid == 0) s_struct_bad = bad;
    }
    __syncthreads();
    const uint32_t total_pairs = s_off[n];
    const bool nomem = total_pairs > coef_capacity;
    // one (patch, wave) pair per thread (at most 1024 with fuse_coef)
    if (tid < total_pairs) {
        uint32_t p = 0;
        while (s_off[p + 1] <= tid) ++p;
        const wt_patch& Pt = sp[p];
        const wt_wave w = waves[Pt.wave_offset + (tid - s_off[p])];
        if (!wave_ok(w)) atomicOr(&s_wave_bad, 1u << p);
        if (!nomem) coef[tid] = make_pair_coef(Pt, w);
    }
    if (tid < n && !nomem) aux[tid] = make_patch_aux(sp[tid], hm, s_off[tid]);
    __syncthreads();
    if (tid >= 32) return;
    const unsigned bad = s_struct_bad | s_wave_bad;
    if (tid < n && ((s_wave_bad >> tid) & 1u)) tiles_p = 0;
    if (tid < n) {
        pair_off[tid] = s_off[tid];
        tiles_g[tid] = tiles_p;
    }
    bool adj_nomem = false;  // lane 0
    if (nomem) {
        // workspace too small for the wave slots: run nothing
        if (tid < n) tile_pre[tid] = 0;
        if (tid == 0) {
            tile_pre[n] = 0;
            pair_off[n] = 0;
            if (do_adj) hdr->total_chunks = 0;
        }
    } else {
        // descending wave count, ties by index (as the general path's rank sort)
        const uint32_t key = tid < n ? min(sp[tid].wave_count, (uint32_t)kSortBins - 1) : 0u;
        uint32_t rank = 0;
        for (uint32_t q = 0; q < n; ++q) {
            const uint32_t kq = __shfl_sync(kAll, key, q);
            rank += kq > key || (kq == key && q < tid);
        }
        if (tid < n) {
            sorted[rank] = tid;
            s_rank_tiles[rank] = tiles_p;
        }
        __syncwarp();
        const uint32_t tq = tid < n ? s_rank_tiles[tid] : 0u;
        uint32_t x = tq;
        for (int o = 1; o < 32; o <<= 1) {
            const uint32_t y = __shfl_up_sync(kAll, x, o);
            if (lane >= (uint32_t)o) x += y;
        }
        const uint32_t total_tiles = __shfl_sync(kAll, x, 31);
        if (tid < n) tile_pre[tid] = x - tq;
        if (tid == 0) {
            tile_pre[n] = total_tiles;
            pair_off[n] = total_pairs;
        }
        if (tid == 0) hdr->total_tiles = total_tiles;
        if (do_adj) {
            // the adjoint's queue: each patch's rank, its chunks of tiles and
            // the prefixes of chunks and of records (chunks x waves) over the
            // sorted order, summed in 32 bits as the general path does
            uint32_t* rank_g = reinterpret_cast<uint32_t*>(ws + AL.rank);
            uint32_t* part_off = reinterpret_cast<uint32_t*>(ws + AL.part_off);
            uint32_t* chunk_pre = reinterpret_cast<uint32_t*>(ws + AL.chunk_pre);
            if (tid < n) s_sorted[rank] = tid;
            __syncwarp();
            const uint32_t chunk = total_tiles >= adj_min_tiles ? adj_chunk_max : 1u;
            uint32_t chunks = 0, rec = 0;
            if (tid < n) {
                const uint32_t pq = s_sorted[tid];
                chunks = (tq + chunk - 1) / chunk;
                const uint64_t r = (uint64_t)chunks * (s_off[pq + 1] - s_off[pq]);
                rec = r > 0xffffffffull ? 0xffffffffu : (uint32_t)r;
                rank_g[pq] = tid;
            }
            uint32_t xr = rec, xc = chunks;
            for (int o = 1; o < 32; o <<= 1) {
                const uint32_t yr = __shfl_up_sync(kAll, xr, o), yc = __shfl_up_sync(kAll, xc, o);
                if (lane >= (uint32_t)o) {
                    xr += yr;
                    xc += yc;
                }
            }
            const uint32_t total_rec = __shfl_sync(kAll, xr, 31), total_chunks = __shfl_sync(kAll, xc, 31);
            if (tid < n) {
                part_off[tid] = xr - rec;
                chunk_pre[tid] = xc - chunks;
            }
            if (tid == 0) {
                part_off[n] = total_rec;
                chunk_pre[n] = total_chunks;
                hdr->adj_chunk = chunk;
                const bool over = (uint64_t)total_rec > AL.cap_records || total_rec == 0xffffffffu || total_tiles == 0;
                hdr->total_chunks = over ? 0u : total_chunks;
                adj_nomem = over && total_tiles != 0;
            }
        }
    }
    if (tid == 0) {
        hdr->status = bad ? (uint32_t)WT_ERR_INVALID_ARG : (nomem || adj_nomem ? (uint32_t)WT_ERR_NOMEM : 0u);
        hdr->bad_patch = bad ? (uint32_t)(__ffs(bad) - 1) : kNoPatch;
        hdr->tile_counter = 0;
        hdr->n_patches = n;
        hdr->tile_cols = tile_cols;
        if (nomem) hdr->total_tiles = 0;
    }
}

// fuse_coef: also form the per-(patch, wave) and per-patch constants here
// (small tables: the host passes it when n_patches * n_waves <= 1024, one
// pair per thread), so that no second prep kernel runs.
__global__ void __launch_bounds__(1024) k_prep_scan(const wt_patch* __restrict__ patches, uint32_t n,
                                                    const wt_wave* __restrict__ waves, uint32_t n_waves,
                                                    uint64_t out_capacity, uint64_t coef_capacity,
                                                    uint32_t tile_cols, char* ws, WsLayout L, HmDev hm,
                                                    int fuse_coef, int do_adj, AdjLayout AL,
                                                    uint32_t adj_chunk_max, uint32_t adj_min_tiles) {
#if __CUDA_ARCH__ >= 900
    // the coefficient kernel does not read what this one writes (it forms its
    // own offsets and waits for this grid before it completes): let it start
    // (with the constants formed here the next kernel is the forward, which
    // waits at its start anyway)
    if (!fuse_coef) cudaTriggerProgrammaticLaunchCompletion();
#endif
    if (n <= kSmallPrep && fuse_coef) {
        prep_small(patches, n, waves, n_waves, out_capacity, coef_capacity, tile_cols, ws, L, hm, do_adj, AL,
                   adj_chunk_max, adj_min_tiles);
        return;
    }
    WsHeader* hdr = reinterpret_cast<WsHeader*>(ws);
    uint32_t* sorted = reinterpret_cast<uint32_t*>(ws + L.sorted);
    uint32_t* tile_pre = reinterpret_cast<uint32_t*>(ws + L.tile_pre);
    uint32_t* pair_off = reinterpret_cast<uint32_t*>(ws + L.pair_off);
    uint32_t* tiles = reinterpret_cast<uint32_t*>(ws + L.tiles);
    __shared__ uint32_t bins[kSortBins];
    constexpr uint32_t kScanSmemOffsets = 4096;
    __shared__ uint32_t off_s[kScanSmemOffsets];
    __shared__ uint32_t good_wave[kWaveMaskWords];  // bit w: wave w passes wave_ok

    if (threadIdx.x == 0) {
        hdr->status = 0;
        hdr->bad_patch = kNoPatch;
        hdr->tile_counter = 0;
        hdr->n_patches = n;
        hdr->tile_cols = tile_cols;
    }
    // up to kRankSortMax patches are ordered by rank (their keys in bins[]),
    // more by a counting sort over the bins
    const bool rank_sort = n <= kRankSortMax;
    if (!rank_sort)
        for (int i = threadIdx.x; i < kSortBins; i += blockDim.x) bins[i] = 0;
    __syncthreads();

    // structural validation; pair_off <- wave counts of the patches that pass
    for (uint32_t p = threadIdx.x; p < n; p += blockDim.x) {
        const wt_patch P = patches[p];
        const bool ok = patch_ok(P, n_waves, out_capacity);
        if (!ok) flag_error(hdr, WT_ERR_INVALID_ARG, p);
        pair_off[p] = ok ? P.wave_count : 0u;
        tiles[p] = ok ? P.rows * tiles_per_row(P.cols, tile_cols / 32) : 0u;
        const uint32_t key = P.wave_count < kSortBins ? P.wave_count : kSortBins - 1;
        if (rank_sort) bins[p] = key;
        else atomicAdd(&bins[kSortBins - 1 - key], 1u);  // descending wave count
    }
    __syncthreads();
    const uint32_t total_pairs = block_exclusive_scan(pair_off, n);
    if (threadIdx.x == 0) pair_off[n] = total_pairs;
    __syncthreads();
    // wave validation; a patch with a bad wave runs no tiles.  More pairs
    // than threads and up to 16384 waves: each wave once, coalesced, into a
    // shared bitmask (a warp's 32 waves are one word), then each patch tests
    // its range of bits.  Otherwise one pair per thread, the owning patch
    // found by binary search.
    const bool off_in_smem = n + 1 <= kScanSmemOffsets;
    if (off_in_smem)
        for (uint32_t i = threadIdx.x; i <= n; i += blockDim.x) off_s[i] = pair_off[i];
    const uint32_t* off = off_in_smem ? off_s : pair_off;
    if (total_pairs > blockDim.x && n_waves <= 32u * kWaveMaskWords) {
        const uint32_t nw_round = (n_waves + 31u) & ~31u;
#pragma unroll 4
        for (uint32_t w = threadIdx.x; w < nw_round; w += blockDim.x) {
            const bool good = w < n_waves && wave_ok(waves[w]);
            const uint32_t word = __ballot_sync(0xffffffffu, good);
            if ((threadIdx.x & 31) == 0) good_wave[w >> 5] = word;
        }
        __syncthreads();
        for (uint32_t p = threadIdx.x; p < n; p += blockDim.x) {
            if (off[p + 1] == off[p]) continue;  // invalid patch (or no waves)
            const uint32_t w0 = patches[p].wave_offset, w1 = w0 + (off[p + 1] - off[p]);
            bool bad = false;
            for (uint32_t w = w0; w < w1 && !bad;) {
                const uint32_t bit = w & 31u, take = min(32u - bit, w1 - w);
                const uint32_t want = (take == 32u ? 0xffffffffu : ((1u << take) - 1u)) << bit;
                bad = (good_wave[w >> 5] & want) != want;
                w += take;
            }
            if (bad) {
                flag_error(hdr, WT_ERR_INVALID_ARG, p);
                tiles[p] = 0;
            }
        }
    } else {
        __syncthreads();
        for (uint32_t P = threadIdx.x; P < total_pairs; P += blockDim.x) {
            uint32_t lo = 0, hi = n + 1;
            while (lo < hi) {
                const uint32_t mid = (lo + hi) >> 1;
                if (off[mid] <= P) lo = mid + 1; else hi = mid;
            }
            const uint32_t p = lo - 1;
            if (!wave_ok(waves[patches[p].wave_offset + (P - off[p])])) {
                flag_error(hdr, WT_ERR_INVALID_ARG, p);
                tiles[p] = 0;
            }
        }
    }
    const bool nomem = total_pairs > coef_capacity;
    __syncthreads();
    if (nomem) {
        // workspace too small for the wave slots: run nothing.  pair_off[n]
        // bounds every coefficient write of the next kernel.
        if (threadIdx.x == 0) {
            atomicCAS(&hdr->status, 0u, (uint32_t)WT_ERR_NOMEM);
            hdr->total_tiles = 0;
            pair_off[n] = 0;
            if (do_adj) hdr->total_chunks = 0;
        }
        for (uint32_t p = threadIdx.x; p <= n; p += blockDim.x) tile_pre[p] = 0;
        return;
    }
    // sort by descending wave count, ties in any order: the order only
    // schedules tiles, results do not depend on it
    if (rank_sort) {
        for (uint32_t p = threadIdx.x; p < n; p += blockDim.x) {
            const uint32_t key = bins[p];
            uint32_t rank = 0;
            for (uint32_t q = 0; q < n; ++q) rank += bins[q] > key || (bins[q] == key && q < p);
            sorted[rank] = p;
        }
    } else {
        block_exclusive_scan(bins, kSortBins);
        __syncthreads();
        for (uint32_t p = threadIdx.x; p < n; p += blockDim.x) {
            const uint32_t wc = patches[p].wave_count;
            const uint32_t key = wc < kSortBins ? wc : kSortBins - 1;
            sorted[atomicAdd(&bins[kSortBins - 1 - key], 1u)] = p;
        }
    }
    __syncthreads();
    for (uint32_t q = threadIdx.x; q < n; q += blockDim.x) tile_pre[q] = tiles[sorted[q]];
    __syncthreads();
    const uint32_t total_tiles = block_exclusive_scan(tile_pre, n);
    if (threadIdx.x == 0) {
        tile_pre[n] = total_tiles;
        hdr->total_tiles = total_tiles;
    }
    if (fuse_coef) {
        PatchAux* aux = reinterpret_cast<PatchAux*>(ws + L.aux);
        PairCoef* coef = reinterpret_cast<PairCoef*>(ws + L.coef);
        for (uint32_t P = threadIdx.x; P < total_pairs; P += blockDim.x) {
            uint32_t lo = 0, hi = n + 1;
            while (lo < hi) {
                const uint32_t mid = (lo + hi) >> 1;
                if (off[mid] <= P) lo = mid + 1; else hi = mid;
            }
            const wt_patch& Pt = patches[lo - 1];
            coef[P] = make_pair_coef(Pt, waves[Pt.wave_offset + (P - off[lo - 1])]);
        }
        for (uint32_t p = threadIdx.x; p < n; p += blockDim.x) aux[p] = make_patch_aux(patches[p], hm, off[p]);
    }
    if (do_adj) {
        __syncthreads();  // sorted, tile_pre and the header's total_tiles are complete
        adj_scan_body(ws, AL, n, adj_chunk_max, adj_min_tiles);
    }
}

// ---- stage 2: FP64 constants per (patch, wave) and per patch ---------------
// Up to kSmemOffsets - 1 patches each block forms the wave-count prefix of
// the structurally valid patches itself, so this kernel runs alongside the
// scan kernel and waits for it only before it completes (the forward kernel
// waits for this one); with more patches it waits first and reads the scan's
// prefix.
__global__ void __launch_bounds__(256) k_prep_coef(const wt_patch* __restrict__ patches, uint32_t n,
                                                   const wt_wave* __restrict__ waves, uint32_t n_waves,
                                                   uint64_t out_capacity, uint64_t coef_capacity, HmDev hm,
                                                   char* ws, WsLayout L) {
    const uint32_t* pair_off_g = reinterpret_cast<const uint32_t*>(ws + L.pair_off);
    PatchAux* aux = reinterpret_cast<PatchAux*>(ws + L.aux);
    PairCoef* coef = reinterpret_cast<PairCoef*>(ws + L.coef);
    constexpr uint32_t kSmemOffsets = 4096;
    __shared__ uint32_t off_s[kSmemOffsets];
    const bool own = n + 1 <= kSmemOffsets;
    uint32_t total;
    if (own) {
        for (uint32_t p = threadIdx.x; p < n; p += blockDim.x) {
            const wt_patch P = patches[p];
            off_s[p] = patch_ok(P, n_waves, out_capacity) ? P.wave_count : 0u;
        }
        __syncthreads();
        total = block_exclusive_scan(off_s, n);
        if (threadIdx.x == 0) off_s[n] = total;
        __syncthreads();
        if (total > coef_capacity) total = 0;  // the scan kernel reports the shortfall
    } else {
#if __CUDA_ARCH__ >= 900
        cudaGridDependencySynchronize();
#endif
        total = pair_off_g[n];  // 0 when the workspace is short
    }
    const uint32_t* pair_off = own ? off_s : pair_off_g;
    const uint32_t stride = gridDim.x * blockDim.x;
    for (uint32_t P = blockIdx.x * blockDim.x + threadIdx.x; P < total; P += stride) {
        // owning patch: last p with pair_off[p] <= P
        uint32_t lo = 0, hi = n + 1;
        while (lo < hi) {
            uint32_t mid = (lo + hi) >> 1;
            if (pair_off[mid] <= P) lo = mid + 1; else hi = mid;
        }
        uint32_t p = lo - 1;
        const wt_patch& Pt = patches[p];
        coef[P] = make_pair_coef(Pt, waves[Pt.wave_offset + (P - pair_off[p])]);
    }
    for (uint32_t p = blockIdx.x * blockDim.x + threadIdx.x; p < n; p += stride)
        aux[p] = make_patch_aux(patches[p], hm, pair_off[p]);
#if __CUDA_ARCH__ >= 900
    // complete only after the scan kernel: whatever waits for this grid then
    // sees both (a no-op when already waited for above)
    if (own) cudaGridDependencySynchronize();
#endif
}

// ---- stage 3: the persistent forward kernel --------------------------------
// EPI = 0: epilogue unrolled over the lane's vertices straight from the
// accumulator registers; EPI = 1: the sums are parked in shared memory and a
// single rolled copy of the epilogue runs (smaller code, larger smem carve-out).
// MODE (FwdMode): kModeSave also stores each vertex's eight wave sums to `sums`,
// kModeStage the vertex-stage outputs of `view` (a compile-time switch: a
// run-time null test of the sums pointer in the epilogue cost 4 % of the
// kernel).
// A patch in the forward's shared-memory tile table (queue order).
struct QInfo {
    uint32_t cols, nwaves, pair_offset, p;
    uint64_t out0;
};
constexpr uint32_t kTabPatches = 1024;
// Per warp in the forward's shared memory (float4 units): the wave staging
// and, for the shared-memory epilogue, the parked sums.
__host__ __device__ constexpr int fwd_warp_f4(int epi, int smax) { return 32 * kStage + epi * smax * 2 * 32; }
__host__ __device__ constexpr size_t tab_bytes(uint32_t n) {
    return n <= kTabPatches ? sizeof(QInfo) * n + 4 * (n + 1) : 0;
}

template <int THREADS, int MINB, int SMAX, int EPI, int MODE>
__global__ void __launch_bounds__(THREADS, MINB)
k_forward(const wt_patch* __restrict__ patches, HmDev hm, float* __restrict__ pos,
          float* __restrict__ nrm, uint32_t flags, char* __restrict__ ws, WsLayout L, uint32_t chunk,
          float4* __restrict__ sums_arg, const wt_view* __restrict__ view, StageOut so, uint32_t tab_in_smem) {
#if __CUDA_ARCH__ >= 900
    cudaGridDependencySynchronize();
#endif
    float4* const sums = MODE == kModeSave ? sums_arg : nullptr;
    // per warp: wave staging (32 x kStage float4), then the parked sums of
    // the tile's vertices ([j][half][lane] float4, conflict-free); after the
    // warps' parts, the 36 floats of the view (kModeStage)
    extern __shared__ float4 fwd_smem[];
    float4* const wbase = fwd_smem + (threadIdx.x >> 5) * fwd_warp_f4(EPI, SMAX);
    float* const su = reinterpret_cast<float*>(fwd_smem + (THREADS / 32) * fwd_warp_f4(EPI, SMAX));
    if (MODE == kModeStage) {
        if (threadIdx.x < 36) su[threadIdx.x] = reinterpret_cast<const float*>(view)[threadIdx.x];
        __syncthreads();
    }
    WsHeader* hdr = reinterpret_cast<WsHeader*>(ws);
    const uint32_t* sorted = reinterpret_cast<const uint32_t*>(ws + L.sorted);
    const uint32_t* tile_pre = reinterpret_cast<const uint32_t*>(ws + L.tile_pre);
    const PatchAux* aux = reinterpret_cast<const PatchAux*>(ws + L.aux);
    const PairCoef* coef = reinterpret_cast<const PairCoef*>(ws + L.coef);
    const int lane = threadIdx.x & 31;
    float4* wst = wbase;
    float4* ebuf = wbase + 32 * kStage;
    const uint32_t n = hdr->n_patches;
    const uint32_t total = hdr->total_tiles;
    const bool pow2 = hm.present && (hm.width & (hm.width - 1)) == 0 && (hm.height & (hm.height - 1)) == 0;
    // the plain epilogue's mask-only texel wrap (the other modes keep one
    // general copy of the epilogue: two would spill their extra outputs)
    const bool fast = pow2 && hm.wrap == WT_WRAP_REPEAT;

    // The tile table: with at most kTabPatches patches each block copies, in
    // queue (sorted) order, the tile prefix and each patch's columns, wave
    // count, first coefficient slot and output offset into shared memory,
    // so a tile's look-up reads no global memory (1.0594 -> 1.0547 ms on 256
    // uneven patches at 8 vertices per lane, 1.0777 -> 1.0680 at 4).
    QInfo* const tab = reinterpret_cast<QInfo*>(su + (MODE == kModeStage ? 36 : 0));
    uint32_t* const tab_pre = reinterpret_cast<uint32_t*>(tab + (tab_in_smem ? n : 0));
    // (a table the prep refused, total 0, has no order to copy: skipped)
    if (tab_in_smem && total > 0) {
        for (uint32_t qq = threadIdx.x; qq < n; qq += THREADS) {
            const uint32_t pp = sorted[qq];
            tab[qq] = QInfo{patches[pp].cols, patches[pp].wave_count, aux[pp].pair_offset, pp,
                            patches[pp].out_offset};
        }
        for (uint32_t qq = threadIdx.x; qq <= n; qq += THREADS) tab_pre[qq] = tile_pre[qq];
        __syncthreads();
    }
    const bool ts = tab_in_smem && total > 0;
    const uint32_t* const tpre = ts ? tab_pre : tile_pre;

    // The queue index of the next tile is fetched while the current one runs;
    // the tile's patch is searched forward from the previous tile's (tiles
    // come out of the queue in increasing order), galloping when it is far.
    uint32_t t_a = 0;
    if (lane == 0) t_a = atomicAdd(&hdr->tile_counter, 1u);
    uint32_t t = __shfl_sync(0xffffffffu, t_a, 0);
    uint32_t q = 0;
    while (t < total) {
        if (lane == 0) t_a = atomicAdd(&hdr->tile_counter, 1u);
        if (tpre[q + 1] <= t) {
            uint32_t step = 1, lo = q + 1, hi = q + 2;
            while (hi <= n && tpre[hi] <= t) { lo = hi; step <<= 1; hi = lo + step; }
            hi = min(hi, n + 1);
            while (hi - lo > 1) {  // tile_pre[lo] <= t < tile_pre[hi]
                const uint32_t mid = (lo + hi) >> 1;
                if (tpre[mid] <= t) lo = mid; else hi = mid;
            }
            q = lo;
        }
        uint32_t p, cols, nwaves, pair_offset;
        uint64_t out0;
        // the rest of the patch's constants are loaded after the wave loop
        // (held across it they would take 15 registers), except for the
        // saving forward, which spills less with them loaded here
        constexpr bool kLateAux = MODE != kModeSave;
        PatchAux a;
        if (ts) {
            const QInfo e = tab[q];
            p = e.p;
            cols = e.cols;
            nwaves = e.nwaves;
            pair_offset = e.pair_offset;
            out0 = e.out0;
            if (!kLateAux) a = aux[p];
        } else {
            p = sorted[q];
            cols = patches[p].cols;
            nwaves = patches[p].wave_count;
            out0 = patches[p].out_offset;
            if (!kLateAux) a = aux[p];
            pair_offset = kLateAux ? aux[p].pair_offset : a.pair_offset;
        }
        const uint32_t lt = t - tpre[q];
        const uint32_t tpr = tiles_per_row(cols, SMAX);
        const uint32_t row = lt / tpr;
        const uint32_t c0 = (lt - row * tpr) * 32u * SMAX;
        const uint32_t S = min((uint32_t)SMAX, (cols - c0 + 31u) / 32u);  // the row's last tile is narrower

        float2 acc[SMAX][4];
#pragma unroll
        for (int j = 0; j < SMAX; ++j)
#pragma unroll
            for (int m = 0; m < 4; ++m) acc[j][m] = make_float2(0.0f, 0.0f);

        for (uint32_t w0 = 0; w0 < nwaves; w0 += chunk) {
            const uint32_t nw = min(chunk, nwaves - w0);
            __syncwarp();
            if ((uint32_t)lane < nw) {
                stage_wave(coef[pair_offset + w0 + lane], c0, row, wst + kStage * lane);
            }
            __syncwarp();
            wave_loop_dispatch<SMAX>(S, acc, wst, nw, lane);
        }
        if (kLateAux) a = aux[p];

        // grid position along the row: x(col) = col * du * (e1 + v e3) + v e2
        const float v = (float)row * a.inv_rm1;
        const float gx = (a.e1x + v * a.e3x) * a.inv_cm1, gz = (a.e1z + v * a.e3z) * a.inv_cm1;
        const float colf = (float)(c0 + lane);
        const float xb = fmaf(colf, gx, v * a.e2x), zb = fmaf(colf, gz, v * a.e2z);
        const uint64_t rowbase = out0 + (uint64_t)row * cols;
        if (EPI == 1) {
            // park the sums, then one rolled copy of the per-vertex epilogue
            // (each lane reads back only its own slots)
#pragma unroll
            for (int j = 0; j < SMAX; ++j) {
                if ((uint32_t)j < S) {
                    ebuf[(2 * j) * 32 + lane] = make_float4(acc[j][0].x, acc[j][0].y, acc[j][1].x, acc[j][1].y);
                    ebuf[(2 * j + 1) * 32 + lane] = make_float4(acc[j][2].x, acc[j][2].y, acc[j][3].x, acc[j][3].y);
                }
            }
#pragma unroll 1
            for (uint32_t j = 0; j < S; ++j) {
                const uint32_t col = c0 + lane + 32 * j;
                if (col < cols) {
                    const float4 s0 = ebuf[(2 * j) * 32 + lane], s1 = ebuf[(2 * j + 1) * 32 + lane];
                    const float xl = fmaf(32.0f * (float)j, gx, xb);
                    const float zl = fmaf(32.0f * (float)j, gz, zb);
                    const float2 pr[4] = {make_float2(s0.x, s0.y), make_float2(s0.z, s0.w), make_float2(s1.x, s1.y),
                                          make_float2(s1.z, s1.w)};
                    if (MODE == kModePlain && fast)
                        finish_vertex<MODE, true>(sums_of(pr), xl, zl, a, hm, pow2, rowbase + col, pos, nrm, flags,
                                                  sums, su, so);
                    else
                        finish_vertex<MODE>(sums_of(pr), xl, zl, a, hm, pow2, rowbase + col, pos, nrm, flags, sums,
                                            su, so);
                }
            }
        } else {
            // kB vertices at a time: their texel loads are all issued before
            // the first of them is used (half the lane's vertices: 1.079 ->
            // 1.059 ms on 256 uneven patches at 8 per lane, 4 and 1 measured
            // the same; the saving and staging epilogues, with more outputs
            // live, take one at a time: more would spill)
            constexpr int kB = MODE == kModePlain ? SMAX / 2 : 1;
#pragma unroll
            for (int jb = 0; jb < SMAX; jb += kB) {
                HmTexels T[kB];
#pragma unroll
                for (int u = 0; u < kB; ++u) {
                    const int j = jb + u;
                    const uint32_t col = c0 + lane + 32 * j;
                    T[u] = HmTexels{};
                    if ((uint32_t)j < S && col < cols && hm.present) {
                        const float xd = fmaf(32.0f * j, gx, xb) + acc[j][0].x;
                        const float zd = fmaf(32.0f * j, gz, zb) + acc[j][1].x;
                        if (MODE == kModePlain && fast) T[u] = hm_fetch<true>(hm, a, xd, zd, pow2);
                        else T[u] = hm_fetch<false>(hm, a, xd, zd, pow2);
                    }
                }
#pragma unroll
                for (int u = 0; u < kB; ++u) {
                    const int j = jb + u;
                    const uint32_t col = c0 + lane + 32 * j;
                    if ((uint32_t)j < S && col < cols) {
                        const float xl = fmaf(32.0f * j, gx, xb);
                        const float zl = fmaf(32.0f * j, gz, zb);
                        finish_vertex_t<MODE>(sums_of(acc[j]), xl, zl, a, hm, T[u], rowbase + col, pos, nrm, flags,
                                              sums, su, so);
                    }
                }
            }
        }
        t = __shfl_sync(0xffffffffu, t_a, 0);
    }
}

// ---- FP32-naive phase (precision studies only) -----------------------------
// The reference's arithmetic: theta = w*dot(D, xz) + phi*t in FP32 with world
// xz (water-grid.vert:78), accurate sinf/cosf so that only the phase
// representation differs from the default path.
__global__ void __launch_bounds__(256) k_forward_naive(const wt_patch* __restrict__ patches, uint32_t n,
                                                       const wt_wave* __restrict__ waves, HmDev hm,
                                                       float* __restrict__ pos, float* __restrict__ nrm,
                                                       uint32_t flags, const char* __restrict__ ws, WsLayout L) {
    const PatchAux* aux = reinterpret_cast<const PatchAux*>(ws + L.aux);
    const uint32_t* tile_pre = reinterpret_cast<const uint32_t*>(ws + L.tile_pre);
    const uint32_t* sorted = reinterpret_cast<const uint32_t*>(ws + L.sorted);
    const bool pow2 = hm.present && (hm.width & (hm.width - 1)) == 0 && (hm.height & (hm.height - 1)) == 0;
    for (uint32_t q = 0; q < n; ++q) {
        if (tile_pre[q + 1] == tile_pre[q]) continue;  // invalid patch
        const uint32_t p = sorted[q];
        const wt_patch P = patches[p];
        const PatchAux a = aux[p];
        const uint64_t nv = (uint64_t)P.cols * P.rows;
        const float t = (float)P.time_s;
        for (uint64_t v = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; v < nv;
             v += (uint64_t)gridDim.x * blockDim.x) {
            uint32_t row = (uint32_t)(v / P.cols), col = (uint32_t)(v - (uint64_t)row * P.cols);
            float u = (float)col * a.inv_cm1, vv = (float)row * a.inv_rm1, uv = u * vv;
            float xl = fmaf(u, a.e1x, fmaf(vv, a.e2x, uv * a.e3x));
            float zl = fmaf(u, a.e1z, fmaf(vv, a.e2z, uv * a.e3z));
            float xw = a.blx + xl, zw = a.blz + zl;
            VertexSums s{0, 0, 0, 0, 0, 0, 0, 0};
            for (uint32_t i = 0; i < P.wave_count; ++i) {
                const wt_wave w = waves[P.wave_offset + i];
                float k = isinf(w.wavelength) ? 0.0f : (float)(kTwoPi / (double)w.wavelength);
                float phi = w.speed * k;
                float th = k * (w.dir_x * xw + w.dir_z * zw) + phi * t + w.phase;
                float sn, c;
                sincosf(th, &sn, &c);
                float A = w.amplitude, Q = w.steepness_q;
                s.dx += Q * A * w.dir_x * c; s.dy += A * sn; s.dz += Q * A * w.dir_z * c;
                s.jx += A * k * w.dir_x * c; s.jz += A * k * w.dir_z * c;
                s.sxx += Q * A * k * w.dir_x * w.dir_x * sn;
                s.sxz += Q * A * k * w.dir_x * w.dir_z * sn;
                s.szz += Q * A * k * w.dir_z * w.dir_z * sn;
            }
            finish_vertex<kModePlain>(s, xl, zl, a, hm, pow2, P.out_offset + v, pos, nrm, flags, nullptr, nullptr,
                                  StageOut{});
        }
    }
}

template <int THREADS, int MINB, int SMAX, int EPI, int MODE>
cudaError_t launch_fwd_t(const FwdConfig& cfg, const wt_patch* patches, uint32_t n_patches, const HmDev& hm,
                         float* pos, float* nrm, uint32_t flags, void* ws, const WsLayout& L, const FwdExtra& x,
                         cudaStream_t s) {
    constexpr int kMaxDev = 64;
    static std::atomic<int> occ_cache[kMaxDev];  // resident blocks per SM, per device
    int dev = 0;
    cudaGetDevice(&dev);
    if (dev < 0 || dev >= kMaxDev) return cudaErrorInvalidDevice;
    const int sm = sm_count();
    if (sm <= 0) return cudaErrorInvalidDevice;
    constexpr size_t smem_base =
        sizeof(float4) * ((THREADS / 32) * fwd_warp_f4(EPI, SMAX) + (MODE == kModeStage ? 9 : 0));
    // the tile table of up to kTabPatches patches follows; occupancy is
    // taken at its largest size
    constexpr size_t smem_max = smem_base + tab_bytes(kTabPatches);
    const uint32_t tab_in_smem = n_patches <= kTabPatches ? 1u : 0u;
    const size_t smem = smem_base + (tab_in_smem ? tab_bytes(n_patches) : 0);
    int occ = occ_cache[dev].load(std::memory_order_relaxed);
    if (occ == 0) {
        int o = 0;
        cudaError_t e = cudaFuncSetAttribute(k_forward<THREADS, MINB, SMAX, EPI, MODE>,
                                             cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem_max);
        if (e != cudaSuccess) return e;
        e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&o, k_forward<THREADS, MINB, SMAX, EPI, MODE>, THREADS,
                                                          smem_max);
        if (e != cudaSuccess) return e;
        occ = o < 1 ? 1 : o;
        occ_cache[dev].store(occ, std::memory_order_relaxed);
    }
    const int bps = cfg.blocks_per_sm > 0 ? (cfg.blocks_per_sm < occ ? cfg.blocks_per_sm : occ) : occ;
    cudaLaunchConfig_t lc = {};
    lc.gridDim = dim3((unsigned)(sm * bps));
    lc.blockDim = dim3(THREADS);
    lc.dynamicSmemBytes = smem;
    lc.stream = s;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
    attr[0].val.programmaticStreamSerializationAllowed = 1;
    lc.attrs = attr;
    lc.numAttrs = 1;
    const uint32_t chunk = cfg.chunk >= 1 && cfg.chunk <= 32 ? (uint32_t)cfg.chunk : 32u;
    return cudaLaunchKernelEx(&lc, k_forward<THREADS, MINB, SMAX, EPI, MODE>, patches, hm, pos, nrm, flags,
                              static_cast<char*>(ws), L, chunk, reinterpret_cast<float4*>(x.sums), x.view, x.stage,
                              tab_in_smem);
}

}  // namespace

cudaError_t launch_prep(const wt_patch* patches, uint32_t n_patches, const wt_wave* waves, uint32_t n_waves,
                        const HmDev& hm, uint64_t out_capacity, uint32_t tile_cols, void* ws,
                        const WsLayout& L, cudaStream_t s, const AdjScanArgs* adj) {
    char* w = static_cast<char*>(ws);
    // coefficient capacity = what the caller's workspace holds past the fixed part
    // (the header records the real total; the scan refuses to overflow it)
    uint64_t coef_cap = (L.end - L.coef) / sizeof(PairCoef);
    // at most 1024 (patch, wave) pairs: the scan kernel forms the constants too
    const int fuse = (uint64_t)n_patches * n_waves <= 1024u;
    const AdjScanArgs none{};
    const AdjScanArgs& A = adj ? *adj : none;
    k_prep_scan<<<1, 1024, 0, s>>>(patches, n_patches, waves, n_waves, out_capacity, coef_cap, tile_cols, w, L,
                                   hm, fuse, adj ? 1 : 0, A.L, A.chunk_max, A.min_tiles);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return e;
    if (fuse) return cudaSuccess;
    const int sms = sm_count();
    if (sms <= 0) return cudaErrorInvalidDevice;
    cudaLaunchConfig_t lc = {};
    lc.gridDim = dim3((unsigned)sms);
    lc.blockDim = dim3(256);
    lc.stream = s;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
    attr[0].val.programmaticStreamSerializationAllowed = 1;
    lc.attrs = attr;
    lc.numAttrs = 1;
    return cudaLaunchKernelEx(&lc, k_prep_coef, patches, n_patches, waves, n_waves, out_capacity, coef_cap, hm, w,
                              L);
}

bool forward_config_supported(const FwdConfig& c) {
    if (c.epi != 0 && c.epi != 1) return false;
    if (c.s == 8) return c.warps == 8 || c.warps == 16 || (c.warps == 20 && c.epi == 0);
    if (c.s == 4) return c.warps == 8 && c.epi == 0;
    return false;
}

// The epilogue variants beyond the plain one exist with the register
// epilogue only: a tuning with the shared-memory epilogue runs them through
// the register one, same shape; 20 warps (the plain forward's 96-register
// shape) run as 16.
template <int MODE>
cudaError_t launch_forward_mode(const FwdConfig& cfg, const wt_patch* patches, uint32_t n_patches, const HmDev& hm,
                                float* pos, float* nrm, uint32_t flags, void* ws, const WsLayout& L,
                                const FwdExtra& x, cudaStream_t s) {
    if (cfg.s == 4 && cfg.warps == 8)
        return launch_fwd_t<256, 3, 4, 0, MODE>(cfg, patches, n_patches, hm, pos, nrm, flags, ws, L, x, s);
    if (cfg.s == 8 && cfg.warps == 8)
        return launch_fwd_t<256, 2, 8, 0, MODE>(cfg, patches, n_patches, hm, pos, nrm, flags, ws, L, x, s);
    if (cfg.s == 8 && (cfg.warps == 16 || cfg.warps == 20))
        return launch_fwd_t<512, 1, 8, 0, MODE>(cfg, patches, n_patches, hm, pos, nrm, flags, ws, L, x, s);
    return cudaErrorInvalidValue;
}

cudaError_t launch_forward(const FwdConfig& cfg, const wt_patch* patches, uint32_t n_patches, const HmDev& hm,
                           float* pos, float* nrm, uint32_t flags, void* ws, const WsLayout& L, const FwdExtra& x,
                           cudaStream_t s) {
    if (x.sums && x.view) return cudaErrorInvalidValue;
    if (x.sums) return launch_forward_mode<kModeSave>(cfg, patches, n_patches, hm, pos, nrm, flags, ws, L, x, s);
    if (x.view) return launch_forward_mode<kModeStage>(cfg, patches, n_patches, hm, pos, nrm, flags, ws, L, x, s);
    // warps per block; the minimum-blocks hint sets the register budget
    if (cfg.s == 4 && cfg.warps == 8 && cfg.epi == 0)
        return launch_fwd_t<256, 3, 4, 0, kModePlain>(cfg, patches, n_patches, hm, pos, nrm, flags, ws, L, x, s);  // 80 regs
    if (cfg.s == 8 && cfg.epi == 0) {
        if (cfg.warps == 8) return launch_fwd_t<256, 2, 8, 0, kModePlain>(cfg, patches, n_patches, hm, pos, nrm, flags, ws, L, x, s);
        if (cfg.warps == 16) return launch_fwd_t<512, 1, 8, 0, kModePlain>(cfg, patches, n_patches, hm, pos, nrm, flags, ws, L, x, s);
        // 20 warps at 96 registers (a few bytes spilled): more warps to hide
        // the wave loop's latencies (256 uneven patches: 1.041 against 1.054
        // ms for 16 warps; 18 and 24 warps were slower)
        if (cfg.warps == 20) return launch_fwd_t<640, 1, 8, 0, kModePlain>(cfg, patches, n_patches, hm, pos, nrm, flags, ws, L, x, s);
    }
    if (cfg.s == 8 && cfg.epi == 1) {
        if (cfg.warps == 8) return launch_fwd_t<256, 2, 8, 1, kModePlain>(cfg, patches, n_patches, hm, pos, nrm, flags, ws, L, x, s);
        if (cfg.warps == 16) return launch_fwd_t<512, 1, 8, 1, kModePlain>(cfg, patches, n_patches, hm, pos, nrm, flags, ws, L, x, s);
    }
    return cudaErrorInvalidValue;
}

cudaError_t launch_forward_naive(const wt_patch* patches, uint32_t n_patches, const wt_wave* waves,
                                 const HmDev& hm, float* pos, float* nrm, uint32_t flags, void* ws,
                                 const WsLayout& L, uint64_t, cudaStream_t s) {
    const int sms = sm_count();
    if (sms <= 0) return cudaErrorInvalidDevice;
    k_forward_naive<<<sms * 4, 256, 0, s>>>(patches, n_patches, waves, hm, pos, nrm, flags,
                                            static_cast<const char*>(ws), L);
    return cudaGetLastError();
}

}  // namespace wt
