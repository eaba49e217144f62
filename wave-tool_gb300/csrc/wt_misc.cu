// wt_misc.cu — index buffer, noise heightmap synthesis, peak-rate probes.
#include <cuda_runtime.h>
#include <cstdint>

#include "wt_internal.h"

namespace wt {
namespace {

// ---- projected-grid index buffer (src/program.cpp:686-717) ----------------
// One thread per output index: k = 6*cell + m, cell = row*(cols-1) + col,
// triangles (r,c) (r+1,c+1) (r+1,c) and (r,c) (r,c+1) (r+1,c+1).
// Coalesced 4-byte stores; the buffer is HBM-write-bound.
__global__ void __launch_bounds__(256) k_indices(uint32_t cols, uint32_t rows, uint32_t base, uint32_t* __restrict__ out,
                                                 uint64_t total) {
    const uint32_t cm1 = cols - 1;
    for (uint64_t k = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; k < total;
         k += (uint64_t)gridDim.x * blockDim.x) {
        uint64_t cell = k / 6;
        uint32_t m = (uint32_t)(k - cell * 6);
        uint32_t row = (uint32_t)(cell / cm1);
        uint32_t col = (uint32_t)(cell - (uint64_t)row * cm1);
        // m:      0     1       2     3     4     5
        // dr:     0     1       1     0     0     1
        // dc:     0     1       0     0     1     1
        uint32_t dr = (0x26u >> m) & 1u;  // bits 1,2,5
        uint32_t dc = (0x32u >> m) & 1u;  // bits 1,4,5
        __stcs(out + k, base + (row + dr) * cols + col + dc);
    }
}

// ---- 8-bit heightmap ingestion -------------------------------------------
// texel (i, j) = R of pixel (i, row j counted from the bottom when flipped)
// as UNORM8 -> float: c / 255, correctly rounded (GL's conversion of an
// RGBA8 texel's red channel, sampled by water-grid.vert:106).
__global__ void __launch_bounds__(256) k_unorm8(const uint8_t* __restrict__ px, uint32_t w, uint32_t h,
                                                uint32_t channels, uint64_t stride, uint32_t flip,
                                                float* __restrict__ out) {
    const uint64_t n = (uint64_t)w * h;
    for (uint64_t k = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; k < n; k += (uint64_t)gridDim.x * blockDim.x) {
        const uint32_t j = (uint32_t)(k / w);
        const uint32_t i = (uint32_t)(k - (uint64_t)j * w);
        const uint32_t src = flip ? h - 1 - j : j;
        out[k] = (float)px[(uint64_t)src * stride + (uint64_t)i * channels] / 255.0f;
    }
}

// ---- noise heightmap -------------------------------------------------------
constexpr size_t kNoiseHeader = 256;  // workspace: min / max, then the factor tables
__device__ __forceinline__ uint32_t ordered(float f) {
    uint32_t b = __float_as_uint(f);
    return (b & 0x80000000u) ? ~b : (b | 0x80000000u);
}
__device__ __forceinline__ float unordered(uint32_t k) {
    return __uint_as_float((k & 0x80000000u) ? (k & 0x7fffffffu) : ~k);
}

__global__ void k_noise_init(uint32_t* mm) {
    mm[0] = 0xffffffffu;  // min (ordered)
    mm[1] = 0u;           // max (ordered)
}

// h(i, j) = sum_m a_m sin(x_m(i) + y_m(j)),
//   x_m(i) = 2 pi (kx_m i mod W) / W,  y_m(j) = 2 pi (ky_m j mod H) / H + psi_m + rate_m t,
// is separable: sin(x + y) = sin x cos y + cos x sin y.  k_noise_tables forms,
// once per term, the column factors (sin x, cos x) for every column and the
// row factors a (cos y, sin y) for every row (integer products reduced
// exactly, the time-shifted row turn reduced in FP64, sines by FP32
// sincospi); k_noise_tiles then spends two FMAs per texel and term.
constexpr uint32_t kNoiseTile = 32;     // texels per block side (16 x 16 threads, 2 x 2 each)
constexpr uint32_t kNoiseChunk = 32;    // terms staged in shared memory at a time

__global__ void __launch_bounds__(256) k_noise_tables(const wt_noise_term* __restrict__ terms, uint32_t n_terms,
                                                      const float* __restrict__ rates, double t, uint32_t W,
                                                      uint32_t H, float2* __restrict__ col, float2* __restrict__ row) {
    const uint64_t per = (uint64_t)W + H, n = per * n_terms;
    for (uint64_t k = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; k < n; k += (uint64_t)gridDim.x * blockDim.x) {
        const uint32_t m = (uint32_t)(k / per);
        const uint32_t r = (uint32_t)(k - (uint64_t)m * per);
        const wt_noise_term tm = terms[m];
        float sn, cs;
        if (r < W) {
            long long ni = ((long long)tm.kx * r) % (long long)W;
            ni += ni < 0 ? W : 0;
            sincospif(2.0f * (float)((double)ni / W), &sn, &cs);
            col[(size_t)m * W + r] = make_float2(sn, cs);
        } else {
            const uint32_t j = r - W;
            long long nj = ((long long)tm.ky * j) % (long long)H;
            nj += nj < 0 ? H : 0;
            // the row's turn: exact fraction plus (psi + rate t) / 2 pi,
            // reduced mod 1 in FP64 (t may be large), then an FP32 sincospi
            double turns = (double)nj / H + ((double)tm.phase + (rates ? (double)rates[m] * t : 0.0)) *
                                                (0.5 / 3.14159265358979323846);
            turns -= floor(turns);
            sincospif(2.0f * (float)turns, &sn, &cs);
            row[(size_t)m * H + j] = make_float2(tm.amplitude * cs, tm.amplitude * sn);
        }
    }
}

__global__ void __launch_bounds__(256) k_noise_tiles(const float2* __restrict__ col, const float2* __restrict__ row,
                                                     uint32_t n_terms, uint32_t W, uint32_t H,
                                                     float* __restrict__ out, uint32_t* mm) {
    __shared__ float2 sc[kNoiseChunk][kNoiseTile], sr[kNoiseChunk][kNoiseTile];
    const uint32_t tx = threadIdx.x & 15, ty = threadIdx.x >> 4;
    const uint32_t i0 = blockIdx.x * kNoiseTile, j0 = blockIdx.y * kNoiseTile;
    float h[2][2] = {{0.0f, 0.0f}, {0.0f, 0.0f}};
    for (uint32_t m0 = 0; m0 < n_terms; m0 += kNoiseChunk) {
        const uint32_t nm = min(kNoiseChunk, n_terms - m0);
        __syncthreads();
        for (uint32_t e = threadIdx.x; e < kNoiseChunk * kNoiseTile; e += blockDim.x) {
            const uint32_t m = e / kNoiseTile, q = e - m * kNoiseTile;
            const bool tm = m < nm;
            sc[m][q] = tm && i0 + q < W ? col[(size_t)(m0 + m) * W + i0 + q] : make_float2(0.0f, 0.0f);
            sr[m][q] = tm && j0 + q < H ? row[(size_t)(m0 + m) * H + j0 + q] : make_float2(0.0f, 0.0f);
        }
        __syncthreads();
        for (uint32_t m = 0; m < nm; ++m) {
#pragma unroll
            for (int b = 0; b < 2; ++b) {
                const float2 y = sr[m][2 * ty + b];
#pragma unroll
                for (int a = 0; a < 2; ++a) {
                    const float2 x = sc[m][2 * tx + a];
                    h[b][a] = fmaf(x.x, y.x, fmaf(x.y, y.y, h[b][a]));
                }
            }
        }
    }
    // block min / max, then one atomic each
    float lo = INFINITY, hi = -INFINITY;
#pragma unroll
    for (int b = 0; b < 2; ++b)
#pragma unroll
        for (int a = 0; a < 2; ++a) {
            const uint32_t i = i0 + 2 * tx + a, j = j0 + 2 * ty + b;
            if (i < W && j < H) {
                lo = fminf(lo, h[b][a]);
                hi = fmaxf(hi, h[b][a]);
                out[(size_t)j * W + i] = h[b][a];
            }
        }
    for (int o = 16; o > 0; o >>= 1) {
        lo = fminf(lo, __shfl_xor_sync(0xffffffffu, lo, o));
        hi = fmaxf(hi, __shfl_xor_sync(0xffffffffu, hi, o));
    }
    if ((threadIdx.x & 31) == 0 && lo <= hi) {
        atomicMin(mm, ordered(lo));
        atomicMax(mm + 1, ordered(hi));
    }
}

__global__ void __launch_bounds__(256) k_noise_norm(float* __restrict__ out, size_t n, const uint32_t* mm) {
    const float lo = unordered(mm[0]), hi = unordered(mm[1]);
    const float span = hi - lo;
    // a correctly rounded division maps the extremes to exactly 0 and 1
    for (size_t v = blockIdx.x * (size_t)blockDim.x + threadIdx.x; v < n; v += (size_t)gridDim.x * blockDim.x)
        out[v] = span > 0.0f ? (out[v] - lo) / span : 0.0f;
}

// ---- peak probes -----------------------------------------------------------
// Eight independent dependent chains per thread: issue-bound FP32 FMA and
// MUFU sine, the two pipes the Gerstner sum can run on.
__global__ void __launch_bounds__(256) k_peak_fma(float* out, int iters, float a, float b) {
    float x[8];
#pragma unroll
    for (int j = 0; j < 8; ++j) x[j] = threadIdx.x * 1e-3f + j;
    for (int i = 0; i < iters; ++i) {
#pragma unroll
        for (int j = 0; j < 8; ++j) x[j] = fmaf(x[j], a, b);
    }
    float s = 0.0f;
#pragma unroll
    for (int j = 0; j < 8; ++j) s += x[j];
    out[blockIdx.x * blockDim.x + threadIdx.x] = s;
}

__global__ void __launch_bounds__(256) k_peak_sin(float* out, int iters) {
    float x[8];
#pragma unroll
    for (int j = 0; j < 8; ++j) x[j] = threadIdx.x * 1e-3f + j;
    for (int i = 0; i < iters; ++i) {
#pragma unroll
        for (int j = 0; j < 8; ++j) x[j] = __sinf(x[j]);
    }
    float s = 0.0f;
#pragma unroll
    for (int j = 0; j < 8; ++j) s += x[j];
    out[blockIdx.x * blockDim.x + threadIdx.x] = s;
}

int device_sms() { return sm_count(); }

}  // namespace

cudaError_t launch_indices(uint32_t cols, uint32_t rows, uint32_t base, uint32_t* out, cudaStream_t s) {
    uint64_t total = 6ull * (cols - 1) * (rows - 1);
    if (total == 0) return cudaSuccess;
    uint64_t want = (total + 255) / 256;
    unsigned blocks = (unsigned)(want < (uint64_t)device_sms() * 16 ? want : (uint64_t)device_sms() * 16);
    k_indices<<<blocks, 256, 0, s>>>(cols, rows, base, out, total);
    return cudaGetLastError();
}

cudaError_t launch_unorm8(const uint8_t* px, uint32_t w, uint32_t h, uint32_t channels, uint64_t stride,
                          uint32_t flip, float* out, cudaStream_t s) {
    const uint64_t n = (uint64_t)w * h;
    const uint64_t want = (n + 255) / 256;
    const unsigned blocks = (unsigned)(want < (uint64_t)device_sms() * 16 ? want : (uint64_t)device_sms() * 16);
    k_unorm8<<<blocks, 256, 0, s>>>(px, w, h, channels, stride, flip, out);
    return cudaGetLastError();
}

cudaError_t launch_noise(const wt_noise_term* terms, uint32_t n_terms, const float* rates, double t, uint32_t w,
                         uint32_t h, float* out, void* ws, cudaStream_t s) {
    uint32_t* mm = static_cast<uint32_t*>(ws);
    float2* col = reinterpret_cast<float2*>(static_cast<char*>(ws) + kNoiseHeader);
    float2* row = col + (size_t)n_terms * w;
    k_noise_init<<<1, 1, 0, s>>>(mm);
    const uint64_t entries = (uint64_t)n_terms * ((uint64_t)w + h);
    if (entries > 0) {
        const uint64_t tb = (entries + 255) / 256;
        k_noise_tables<<<(unsigned)(tb < 65536 ? tb : 65536), 256, 0, s>>>(terms, n_terms, rates, t, w, h, col, row);
    }
    dim3 grid((w + kNoiseTile - 1) / kNoiseTile, (h + kNoiseTile - 1) / kNoiseTile);
    k_noise_tiles<<<grid, 256, 0, s>>>(col, row, n_terms, w, h, out, mm);
    size_t n = (size_t)w * h;
    unsigned blocks = (unsigned)((n + 255) / 256 < 4096 ? (n + 255) / 256 : 4096);
    k_noise_norm<<<blocks, 256, 0, s>>>(out, n, mm);
    return cudaGetLastError();
}

size_t noise_workspace_bytes(uint32_t n_terms, uint32_t w, uint32_t h) {
    return kNoiseHeader + sizeof(float2) * (size_t)n_terms * ((size_t)w + h);
}

cudaError_t measure_peaks(void* scratch, size_t bytes, double* fma, double* sin_rate, cudaStream_t s) {
    const int sms = device_sms();
    const int blocks = sms * 8, threads = 256;
    if ((size_t)blocks * threads * sizeof(float) > bytes) return cudaErrorInvalidValue;
    float* out = static_cast<float*>(scratch);
    cudaEvent_t e0, e1;
    cudaError_t e = cudaEventCreate(&e0);
    if (e != cudaSuccess) return e;
    e = cudaEventCreate(&e1);
    if (e != cudaSuccess) { cudaEventDestroy(e0); return e; }
    const int it_fma = 1 << 15, it_sin = 1 << 12;
    float best_fma = 1e30f, best_sin = 1e30f;
    for (int rep = 0; rep < 4; ++rep) {
        float ms = 0.0f;
        cudaEventRecord(e0, s);
        k_peak_fma<<<blocks, threads, 0, s>>>(out, it_fma, 0.999f, 0.001f);
        cudaEventRecord(e1, s);
        cudaEventSynchronize(e1);
        cudaEventElapsedTime(&ms, e0, e1);
        if (rep > 0 && ms < best_fma) best_fma = ms;
        cudaEventRecord(e0, s);
        k_peak_sin<<<blocks, threads, 0, s>>>(out, it_sin);
        cudaEventRecord(e1, s);
        cudaEventSynchronize(e1);
        cudaEventElapsedTime(&ms, e0, e1);
        if (rep > 0 && ms < best_sin) best_sin = ms;
    }
    e = cudaGetLastError();
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    if (e != cudaSuccess) return e;
    const double lanes = (double)blocks * threads;
    *fma = lanes * 8.0 * it_fma / (best_fma * 1e-3);
    *sin_rate = lanes * 8.0 * it_sin / (best_sin * 1e-3);
    return cudaSuccess;
}

}  // namespace wt
