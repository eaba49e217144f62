// wt_noalloc.cu — wt_gerstner_displace without a caller-provided workspace,
// for callers that cannot allocate device memory (see include/wt.h).
//
// The scratch the prep and forward kernels need (header, LPT order, prefix
// sums, per-patch and per-(patch, wave) constants) is a file-scope device
// array.  Host code cannot use the array's name as a device pointer, so the
// first call on each device looks up its address with cudaGetSymbolAddress
// (with that device current) and every launch is given that address.
#include <cuda_runtime.h>

#include <cmath>
#include <cstdio>
#include <mutex>

#include "wt_internal.h"

namespace {

constexpr size_t kScratchBytes = 1152u * 1024u;  // >= ws_layout(WT_NOALLOC_MAX_PATCHES, WT_NOALLOC_MAX_WAVE_SLOTS)
constexpr int kMaxDevices = 64;

static __device__ __align__(256) unsigned char g_scratch[kScratchBytes];

std::mutex g_setup_mu;
void* g_scratch_addr[kMaxDevices] = {};

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

// Device address of g_scratch on the current device, looked up once per device.
wt_status scratch_address(void** out) {
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return cuda_fail(e, "cudaGetDevice");
    if (dev < 0 || dev >= kMaxDevices) return fail(WT_ERR_UNSUPPORTED, "device ordinal beyond 63");
    std::lock_guard<std::mutex> g(g_setup_mu);
    if (!g_scratch_addr[dev]) {
        void* p = nullptr;
        e = cudaGetSymbolAddress(&p, g_scratch);
        if (e != cudaSuccess) return cuda_fail(e, "cudaGetSymbolAddress of the no-alloc scratch");
        g_scratch_addr[dev] = p;
    }
    *out = g_scratch_addr[dev];
    return WT_OK;
}

bool aligned(const void* p, size_t a) { return (reinterpret_cast<uintptr_t>(p) % a) == 0; }

}  // namespace

extern "C" wt_status wt_gerstner_displace_noalloc(const wt_patch* patches, uint32_t n_patches,
                                                  uint64_t total_wave_slots, const wt_wave* waves,
                                                  uint32_t n_waves, const wt_heightmap* hm, float* pos_out,
                                                  float* nrm_out, uint64_t out_capacity, uint32_t flags,
                                                  wt_stream stream) {
    if (n_patches > WT_NOALLOC_MAX_PATCHES)
        return fail(WT_ERR_INVALID_ARG, "wt_gerstner_displace_noalloc: more than WT_NOALLOC_MAX_PATCHES (1024) patches");
    if (total_wave_slots > WT_NOALLOC_MAX_WAVE_SLOTS)
        return fail(WT_ERR_INVALID_ARG,
                    "wt_gerstner_displace_noalloc: total_wave_slots above WT_NOALLOC_MAX_WAVE_SLOTS (16384)");
    if (!patches || !aligned(patches, 8)) return fail(WT_ERR_INVALID_ARG, "patches NULL or not 8-byte aligned");
    if (n_waves > 0 && (!waves || !aligned(waves, 4))) return fail(WT_ERR_INVALID_ARG, "waves NULL or misaligned");
    const uint32_t known = WT_OUT_DISPLACEMENT | WT_LAYOUT_VEC3 | WT_PHASE_FP32_NAIVE;
    if (flags & ~known) return fail(WT_ERR_INVALID_ARG, "unknown flags");
    if (out_capacity == 0) return fail(WT_ERR_INVALID_ARG, "out_capacity is 0");
    const size_t oa = (flags & WT_LAYOUT_VEC3) ? 4 : 16;
    if (!pos_out || !aligned(pos_out, oa)) return fail(WT_ERR_INVALID_ARG, "pos_out NULL or misaligned");
    if (nrm_out && !aligned(nrm_out, oa)) return fail(WT_ERR_INVALID_ARG, "nrm_out misaligned");
    wt::HmDev h = {};
    if (hm) {
        if (!hm->texels || !aligned(hm->texels, 4)) return fail(WT_ERR_INVALID_ARG, "heightmap texels NULL or misaligned");
        if (hm->width < 1 || hm->height < 1 || hm->width > 32768 || hm->height > 32768)
            return fail(WT_ERR_INVALID_ARG, "heightmap size outside [1, 32768]");
        if (!std::isfinite(hm->sample_scale) || hm->sample_scale < 0.0f || !std::isfinite(hm->disp_scale))
            return fail(WT_ERR_INVALID_ARG, "heightmap scales must be finite (sample_scale >= 0)");
        if (hm->wrap != WT_WRAP_REPEAT && hm->wrap != WT_WRAP_MIRRORED_REPEAT)
            return fail(WT_ERR_INVALID_ARG, "heightmap: unknown wrap mode");
        if (hm->_pad != 0) return fail(WT_ERR_INVALID_ARG, "heightmap: _pad must be 0");
        h = {hm->texels, hm->width, hm->height, hm->sample_scale, hm->disp_scale, hm->wrap, 1};
    }
    if (n_patches == 0) return WT_OK;
    void* ws = nullptr;
    wt_status st = scratch_address(&ws);
    if (st != WT_OK) return st;
    // every byte past the fixed part holds per-(patch, wave) constants; the
    // first kernel refuses to run patches whose wave slots do not fit
    const wt::WsLayout L0 = wt::ws_layout(n_patches, 0);
    const wt::WsLayout L = wt::ws_layout(n_patches, (kScratchBytes - L0.coef) / sizeof(wt::PairCoef) - 4);
    if (L.end > kScratchBytes || (L.end - L.coef) / sizeof(wt::PairCoef) < WT_NOALLOC_MAX_WAVE_SLOTS)
        return fail(WT_ERR_UNSUPPORTED, "no-alloc scratch smaller than its stated limits");
    const wt::FwdConfig cfg = wt::forward_config(n_patches, n_waves);
    cudaStream_t s = (cudaStream_t)stream;
    cudaError_t e = wt::launch_prep(patches, n_patches, waves, n_waves, h, out_capacity, 32u * cfg.s, ws, L, s);
    if (e != cudaSuccess) return cuda_fail(e, "prep launch");
    if (flags & WT_PHASE_FP32_NAIVE)
        e = wt::launch_forward_naive(patches, n_patches, waves, h, pos_out, nrm_out, flags, ws, L, out_capacity, s);
    else
        e = wt::launch_forward(cfg, patches, n_patches, h, pos_out, nrm_out, flags, ws, L, wt::FwdExtra{}, s);
    if (e != cudaSuccess) return cuda_fail(e, "forward launch");
    return WT_OK;
}

extern "C" wt_status wt_noalloc_status(wt_stream stream, uint32_t* bad_patch) {
    void* ws = nullptr;
    const wt_status st = scratch_address(&ws);
    if (st != WT_OK) return st;
    uint32_t h[2] = {0, 0};  // the header's status word and first offending patch
    cudaError_t e = cudaMemcpyAsync(h, ws, sizeof(h), cudaMemcpyDeviceToHost, (cudaStream_t)stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize((cudaStream_t)stream);
    if (e != cudaSuccess) return cuda_fail(e, "reading the no-alloc status");
    if (bad_patch) *bad_patch = h[1];
    if (h[0] == WT_OK) return WT_OK;
    if (h[0] == WT_ERR_NOMEM) return fail(WT_ERR_NOMEM, "no-alloc scratch too small for the patches' wave slots");
    char buf[96];
    snprintf(buf, sizeof(buf), "device-side validation failed at patch %u", h[1]);
    return fail((wt_status)h[0], buf);
}
