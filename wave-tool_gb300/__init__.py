"""wave-tool GB300: the water-surface hot path of wave-tool as sm_103a CUDA
behind a C ABI (include/wt.h), with this thin Python host layer on top.

The reference computes this path in its GLSL vertex shader
(assets/shaders/water-grid.vert:74-194) fed by RenderEngine::render
(src/render-engine.cpp:1045-1115).  Here the same work is one persistent
CUDA launch over many patches, called through ctypes on the in-tree
``_build/libwt_gb300.so``.  PyTorch is used only for device memory and
streams.  There is no CPU fallback: without the CUDA library every call
raises.
"""
from __future__ import annotations

import ctypes as C
import math
from pathlib import Path

import numpy as np

from . import abi
from . import build as _build_recipe  # bound before build() below, which must not be shadowed by the submodule
from .abi import (CAMERA_DTYPE, NOISE_TERM_DTYPE, PATCH_DTYPE, VIEW_DTYPE, WAVE_DTYPE, WAVE_GRAD_DTYPE, WT_LAYOUT_FLOAT4,
                  WT_LAYOUT_VEC3, WT_OUT_DISPLACEMENT, WT_OUT_WORLD, WT_PHASE_FP32_NAIVE, WT_PHASE_FP64,
                  WT_WRAP_MIRRORED_REPEAT, WT_WRAP_REPEAT)

HERE = Path(__file__).resolve().parent
LIB_PATH = HERE / "_build" / "libwt_gb300.so"

# every symbol include/wt.h declares
EXPORTED = [
    "wt_version", "wt_last_error", "wt_displace_workspace_size", "wt_adjoint_workspace_size",
    "wt_workspace_status", "wt_gerstner_displace", "wt_gerstner_displace_noalloc", "wt_noalloc_status",
    "wt_gerstner_displace_unbatched",
    "wt_gerstner_adjoint", "wt_grid_indices", "wt_noise_synth", "wt_wave_from_reference",
    "wt_measure_peaks", "wt_set_tuning", "wt_get_tuning", "wt_autotune_displace", "wt_autotune_displace_stage",
    "wt_projected_grid", "wt_projected_grid_async", "wt_vertex_stage", "wt_heightmap_from_unorm8",
    "wt_water_raster", "wt_water_raster_workspace_size", "wt_water_shade",
    "wt_gerstner_displace_saving", "wt_gerstner_adjoint_saved", "wt_gerstner_displace_stage",
    "wt_noise_workspace_size", "wt_noise_synth_animated",
]


class WtError(RuntimeError):
    def __init__(self, status: int, message: str):
        super().__init__(f"{abi.STATUS_NAMES.get(status, status)}: {message}")
        self.status = status


class CHeightmap(C.Structure):
    _fields_ = [("texels", C.c_void_p), ("width", C.c_uint32), ("height", C.c_uint32),
                ("sample_scale", C.c_float), ("disp_scale", C.c_float), ("wrap", C.c_uint32),
                ("_pad", C.c_uint32)]


class CTuning(C.Structure):
    _fields_ = [("warps_per_block", C.c_uint32), ("blocks_per_sm", C.c_uint32), ("wave_chunk", C.c_uint32),
                ("max_vertices_per_lane", C.c_uint32), ("epilogue_in_shared", C.c_uint32)]


class CWaterShading(C.Structure):
    _fields_ = [("sun_position", C.c_float * 3), ("sun_shininess", C.c_float), ("sun_strength", C.c_float),
                ("water_clarity", C.c_float), ("soft_edges_threshold", C.c_float), ("tint_threshold", C.c_float),
                ("fog_colour", C.c_float * 4), ("fog_radius_near", C.c_float), ("fog_radius_far", C.c_float),
                ("z_near", C.c_float), ("z_far", C.c_float)]


class CWaterTextures(C.Structure):
    _fields_ = [("scene_depth", C.c_void_p), ("local_reflections", C.c_void_p), ("local_refractions", C.c_void_p),
                ("skybox", C.c_void_p), ("skybox_size", C.c_uint32), ("_pad", C.c_uint32)]


class CStageOutputs(C.Structure):
    _fields_ = [(n, C.c_void_p) for n in ("clip", "ndc0", "view", "facing", "nrm_yaw")]


# the reference's water shading defaults (render-engine.h:221-235, Z_NEAR / Z_FAR)
WATER_SHADING_DEFAULTS = dict(sun_position=(0.0, 1.0, 0.0), sun_shininess=50.0, sun_strength=1.0,
                              water_clarity=0.3, soft_edges_threshold=0.05, tint_threshold=0.1,
                              fog_colour=(1.0, 1.0, 1.0, 0.1), fog_radius_near=0.0, fog_radius_far=1.0,
                              z_near=0.1, z_far=100.0)


class CWave(C.Structure):
    _fields_ = [(n, C.c_float) for n in WAVE_DTYPE.names]


_lib = None


def build(force: bool = False) -> Path:
    return _build_recipe.build(force=force)


def lib():
    """The CUDA library; raises if it has not been built."""
    global _lib
    if _lib is None:
        if not LIB_PATH.exists():
            raise RuntimeError(f"CUDA library {LIB_PATH} is missing: run build() first "
                               "(there is no CPU fallback)")
        L = C.CDLL(str(LIB_PATH))
        vp, u32, u64, sz = C.c_void_p, C.c_uint32, C.c_uint64, C.c_size_t
        L.wt_version.restype = C.c_char_p
        L.wt_last_error.restype = C.c_char_p
        L.wt_displace_workspace_size.argtypes = [u32, u64, C.POINTER(sz)]
        L.wt_adjoint_workspace_size.argtypes = [vp, u32, C.POINTER(sz)]
        L.wt_workspace_status.argtypes = [vp, vp, C.POINTER(u32)]
        L.wt_noalloc_status.argtypes = [vp, C.POINTER(u32)]
        L.wt_gerstner_displace.argtypes = [vp, u32, vp, u32, C.POINTER(CHeightmap), vp, vp, u64, u32, vp, sz, vp]
        L.wt_gerstner_displace_noalloc.argtypes = [vp, u32, u64, vp, u32, C.POINTER(CHeightmap), vp, vp, u64, u32,
                                                   vp]
        L.wt_gerstner_displace_unbatched.argtypes = [vp, vp, u32, vp, u32, C.POINTER(CHeightmap), vp, vp, u64,
                                                     u32, vp, sz, vp]
        L.wt_gerstner_adjoint.argtypes = [vp, vp, u32, vp, u32, C.POINTER(CHeightmap), vp, vp, u64, u32, vp,
                                          vp, sz, vp]
        L.wt_gerstner_displace_saving.argtypes = [vp, u32, vp, u32, C.POINTER(CHeightmap), vp, vp, u64, u32, vp,
                                                  vp, sz, vp]
        L.wt_gerstner_adjoint_saved.argtypes = [vp, vp, u32, vp, u32, C.POINTER(CHeightmap), vp, vp, u64, u32, vp,
                                                vp, vp, sz, vp]
        L.wt_gerstner_displace_stage.argtypes = [vp, u32, vp, u32, C.POINTER(CHeightmap), vp, vp, vp, u64, u32,
                                                 C.POINTER(CStageOutputs), vp, sz, vp]
        L.wt_grid_indices.argtypes = [u32, u32, u32, vp, vp]
        L.wt_noise_synth.argtypes = [vp, u32, u32, u32, vp, vp, sz, vp]
        L.wt_noise_workspace_size.argtypes = [u32, u32, u32, C.POINTER(sz)]
        L.wt_noise_synth_animated.argtypes = [vp, u32, vp, C.c_double, u32, u32, vp, vp, sz, vp]
        L.wt_wave_from_reference.argtypes = [C.c_float] * 6 + [u32, C.POINTER(CWave)]
        L.wt_measure_peaks.argtypes = [vp, sz, C.POINTER(C.c_double), C.POINTER(C.c_double), vp]
        L.wt_set_tuning.argtypes = [C.POINTER(CTuning)]
        L.wt_get_tuning.argtypes = [C.POINTER(CTuning)]
        L.wt_autotune_displace.argtypes = [vp, u32, vp, u32, C.POINTER(CHeightmap), vp, vp, u64, u32, vp, sz, u32,
                                           C.POINTER(CTuning), vp]
        L.wt_autotune_displace_stage.argtypes = [vp, u32, vp, u32, C.POINTER(CHeightmap), vp, vp, vp, u64, u32,
                                                 C.POINTER(CStageOutputs), vp, sz, u32, C.POINTER(CTuning), vp]
        L.wt_projected_grid.argtypes = [vp, vp, vp, C.POINTER(u32)]
        L.wt_projected_grid_async.argtypes = [vp, vp, vp, vp]
        L.wt_vertex_stage.argtypes = [vp, vp, vp, u64, u32, vp, vp, vp, vp, vp, vp]
        L.wt_heightmap_from_unorm8.argtypes = [vp, u32, u32, u32, u64, u32, vp, vp]
        L.wt_water_raster.argtypes = [vp, u64, vp, u64, u32, u32, vp, vp, vp, sz, vp]
        L.wt_water_raster_workspace_size.argtypes = [u64, u64, C.POINTER(sz)]
        L.wt_water_shade.argtypes = [vp, vp, u64, vp, u64, vp, vp, vp, vp, u32, u32, C.POINTER(CWaterShading),
                                     C.POINTER(CWaterTextures), vp, vp, vp]
        for name in EXPORTED:
            if name not in ("wt_version", "wt_last_error"):
                getattr(L, name).restype = C.c_int
        _lib = L
    return _lib


def version() -> str:
    return lib().wt_version().decode()


def check(status: int) -> None:
    if status != abi.WT_OK:
        raise WtError(status, lib().wt_last_error().decode())


# ---- torch plumbing ----------------------------------------------------------

def _torch():
    import torch
    return torch


def stream_handle(stream=None) -> int:
    torch = _torch()
    s = stream if stream is not None else torch.cuda.current_stream()
    return s.cuda_stream


def to_device(arr: np.ndarray, device="cuda"):
    """Copy a (structured) numpy array to a device byte tensor."""
    torch = _torch()
    a = np.ascontiguousarray(arr)
    return torch.from_numpy(a.view(np.uint8).reshape(-1).copy()).to(device)


def empty_bytes(n: int, device="cuda"):
    torch = _torch()
    # 256-byte aligned by the caching allocator
    return torch.empty(max(int(n), 1), dtype=torch.uint8, device=device)


def _ptr(t) -> int | None:
    return None if t is None else t.data_ptr()


class DeviceHeightmap:
    """A heightmap layer with texels in device memory (texels[j, i], j = t row)."""

    def __init__(self, texels, sample_scale: float, disp_scale: float, wrap: int = WT_WRAP_REPEAT):
        assert texels.is_cuda and texels.dtype == _torch().float32 and texels.dim() == 2
        self.texels = texels.contiguous()
        self.sample_scale = float(sample_scale)
        self.disp_scale = float(disp_scale)
        self.wrap = int(wrap)

    def cstruct(self) -> CHeightmap:
        h, w = self.texels.shape
        return CHeightmap(self.texels.data_ptr(), w, h, self.sample_scale, self.disp_scale, self.wrap, 0)


def displace_workspace_bytes(n_patches: int, total_wave_slots: int) -> int:
    out = C.c_size_t()
    check(lib().wt_displace_workspace_size(n_patches, total_wave_slots, C.byref(out)))
    return out.value


def adjoint_workspace_bytes(host_patches: np.ndarray) -> int:
    out = C.c_size_t()
    hp = np.ascontiguousarray(host_patches)
    check(lib().wt_adjoint_workspace_size(hp.ctypes.data, len(hp), C.byref(out)))
    return out.value


def workspace_status(ws, stream=None) -> tuple[int, int]:
    bad = C.c_uint32()
    st = lib().wt_workspace_status(ws.data_ptr(), stream_handle(stream), C.byref(bad))
    return st, bad.value


class Surface:
    """Device-resident patch table, waves and heightmap for the C ABI.

    Mirrors the reference's per-frame inputs: `waves` are the GerstnerWave
    uniforms (render-engine.cpp:1067-1081), `patches` the projected-grid
    corners + gridLength + time (:1045-1108), `heightmap` the noise texture
    (program.cpp:719, water-grid.vert:93-111)."""

    def __init__(self, patches: np.ndarray, waves: np.ndarray, heightmap: DeviceHeightmap | None = None,
                 device="cuda"):
        assert patches.dtype == PATCH_DTYPE and waves.dtype == WAVE_DTYPE
        self.host_patches = np.ascontiguousarray(patches)
        self.host_waves = np.ascontiguousarray(waves)
        self.patches = to_device(self.host_patches, device)
        self.waves = to_device(self.host_waves, device)
        self.heightmap = heightmap
        self.n_patches = len(patches)
        self.n_waves = len(waves)
        self.n_vertices = int(max((int(p["out_offset"]) + int(p["cols"]) * int(p["rows"]) for p in patches),
                                  default=0))
        self.wave_slots = int(np.sum(patches["wave_count"].astype(np.uint64)))
        self.workspace = empty_bytes(displace_workspace_bytes(self.n_patches, self.wave_slots), device)

    def alloc_outputs(self, flags: int = 0, normals: bool = True):
        torch = _torch()
        w = 3 if flags & WT_LAYOUT_VEC3 else 4
        pos = torch.empty((self.n_vertices, w), dtype=torch.float32, device=self.patches.device)
        nrm = torch.empty_like(pos) if normals else None
        return pos, nrm

    def displace(self, pos=None, nrm=None, flags: int = 0, normals: bool = True, stream=None, unbatched=False,
                 sums=None):
        """Positions and normals; with `sums` (an (n_vertices, 8) float32
        tensor) also the per-vertex wave sums an adjoint can reuse."""
        if pos is None:
            pos, nrm = self.alloc_outputs(flags, normals)
        hm = self.heightmap.cstruct() if self.heightmap is not None else None
        hmp = C.byref(hm) if hm is not None else None
        cap = pos.shape[0]
        if sums is not None:
            assert sums.shape[0] >= cap and sums.shape[-1] == 8 and sums.is_contiguous()
            check(lib().wt_gerstner_displace_saving(
                self.patches.data_ptr(), self.n_patches, self.waves.data_ptr(), self.n_waves, hmp,
                pos.data_ptr(), _ptr(nrm), cap, flags, sums.data_ptr(), self.workspace.data_ptr(),
                self.workspace.numel(), stream_handle(stream)))
        elif unbatched:
            check(lib().wt_gerstner_displace_unbatched(
                self.host_patches.ctypes.data, self.patches.data_ptr(), self.n_patches, self.waves.data_ptr(),
                self.n_waves, hmp, pos.data_ptr(), _ptr(nrm), cap, flags, self.workspace.data_ptr(),
                self.workspace.numel(), stream_handle(stream)))
        else:
            check(lib().wt_gerstner_displace(
                self.patches.data_ptr(), self.n_patches, self.waves.data_ptr(), self.n_waves, hmp,
                pos.data_ptr(), _ptr(nrm), cap, flags, self.workspace.data_ptr(), self.workspace.numel(),
                stream_handle(stream)))
        return pos, nrm

    def displace_stage(self, view_dev, out=None, pos=None, nrm=None, flags: int = 0, stream=None,
                       stage=("clip", "ndc0", "view", "facing", "nrm_yaw")) -> dict:
        """wt_gerstner_displace_stage: the displacement with the vertex stage
        fused into its epilogue.  Returns the dict of (new or given) stage
        outputs (float4, ndc0 float2); pos / nrm are written only if given."""
        torch = _torch()
        n = self.n_vertices
        out = dict(out or {})
        for k in stage:
            if k not in out:
                out[k] = torch.empty((n, 2 if k == "ndc0" else 4), dtype=torch.float32, device=self.patches.device)
        so = CStageOutputs(*[_ptr(out.get(k)) for k in ("clip", "ndc0", "view", "facing", "nrm_yaw")])
        hm = self.heightmap.cstruct() if self.heightmap is not None else None
        hmp = C.byref(hm) if hm is not None else None
        check(lib().wt_gerstner_displace_stage(
            self.patches.data_ptr(), self.n_patches, self.waves.data_ptr(), self.n_waves, hmp, view_dev.data_ptr(),
            _ptr(pos), _ptr(nrm), n, flags, C.byref(so), self.workspace.data_ptr(), self.workspace.numel(),
            stream_handle(stream)))
        return out

    def status(self, stream=None):
        return workspace_status(self.workspace, stream)

    def adjoint(self, d_pos, d_nrm=None, flags: int = 0, grad=None, stream=None, sums=None):
        """dL/dwave (n_waves x 8 float32 tensor, the wt_wave_grad fields) for
        upstream gradients d_pos / d_nrm laid out like the outputs; with the
        `sums` a saving displace wrote, the forward is not recomputed."""
        torch = _torch()
        if getattr(self, "adj_workspace", None) is None:
            self.adj_workspace = empty_bytes(adjoint_workspace_bytes(self.host_patches), self.patches.device)
        if grad is None:
            grad = torch.empty((self.n_waves, 8), dtype=torch.float32, device=self.patches.device)
        hm = self.heightmap.cstruct() if self.heightmap is not None else None
        hmp = C.byref(hm) if hm is not None else None
        if sums is not None:
            check(lib().wt_gerstner_adjoint_saved(
                self.host_patches.ctypes.data, self.patches.data_ptr(), self.n_patches, self.waves.data_ptr(),
                self.n_waves, hmp, d_pos.data_ptr(), _ptr(d_nrm), d_pos.shape[0], flags, sums.data_ptr(),
                grad.data_ptr(), self.adj_workspace.data_ptr(), self.adj_workspace.numel(), stream_handle(stream)))
            return grad
        check(lib().wt_gerstner_adjoint(
            self.host_patches.ctypes.data, self.patches.data_ptr(), self.n_patches, self.waves.data_ptr(),
            self.n_waves, hmp, d_pos.data_ptr(), _ptr(d_nrm), d_pos.shape[0],
            flags, grad.data_ptr(), self.adj_workspace.data_ptr(), self.adj_workspace.numel(),
            stream_handle(stream)))
        return grad

    def set_waves(self, waves: np.ndarray) -> None:
        """Replace the wave parameters (same count) in place on the device."""
        assert waves.dtype == WAVE_DTYPE and len(waves) == self.n_waves
        self.host_waves = np.ascontiguousarray(waves)
        self.waves.copy_(to_device(self.host_waves, self.patches.device))

    def autotune(self, pos, nrm, flags: int = 0, reps: int = 3, stream=None) -> dict:
        """Times the candidate launch shapes on this surface and keeps the
        fastest (process-wide)."""
        hm = self.heightmap.cstruct() if self.heightmap is not None else None
        best = CTuning()
        check(lib().wt_autotune_displace(
            self.patches.data_ptr(), self.n_patches, self.waves.data_ptr(), self.n_waves,
            C.byref(hm) if hm is not None else None, pos.data_ptr(), _ptr(nrm), pos.shape[0], flags,
            self.workspace.data_ptr(), self.workspace.numel(), reps, C.byref(best), stream_handle(stream)))
        return {f: getattr(best, f) for f, _ in CTuning._fields_}

    def autotune_stage(self, view_dev, out, pos=None, nrm=None, flags: int = 0, reps: int = 3, stream=None) -> dict:
        """Times the candidate launch shapes of displace_stage on this surface
        (out: the stage outputs, as displace_stage returns them) and keeps the
        fastest for later displace_stage calls (process-wide)."""
        hm = self.heightmap.cstruct() if self.heightmap is not None else None
        so = CStageOutputs(*[_ptr(out.get(k)) for k in ("clip", "ndc0", "view", "facing", "nrm_yaw")])
        best = CTuning()
        check(lib().wt_autotune_displace_stage(
            self.patches.data_ptr(), self.n_patches, self.waves.data_ptr(), self.n_waves,
            C.byref(hm) if hm is not None else None, view_dev.data_ptr(), _ptr(pos), _ptr(nrm), self.n_vertices,
            flags, C.byref(so), self.workspace.data_ptr(), self.workspace.numel(), reps, C.byref(best),
            stream_handle(stream)))
        return {f: getattr(best, f) for f, _ in CTuning._fields_}


def grid_indices(cols: int, rows: int, base_vertex: int = 0, stream=None):
    torch = _torch()
    out = torch.empty(6 * (cols - 1) * (rows - 1), dtype=torch.int32, device="cuda")
    check(lib().wt_grid_indices(cols, rows, base_vertex, out.data_ptr(), stream_handle(stream)))
    return out


def noise_workspace_bytes(n_terms: int, width: int, height: int) -> int:
    out = C.c_size_t()
    check(lib().wt_noise_workspace_size(n_terms, width, height, C.byref(out)))
    return out.value


def noise_synth(terms: np.ndarray, width: int, height: int, stream=None, rates=None, time_s: float = 0.0,
                out=None, workspace=None):
    """The noise heightmap (h, w) on the device; with `rates` (radians per
    second per term, host array or device tensor) the layer at `time_s`."""
    torch = _torch()
    if isinstance(terms, np.ndarray):
        assert terms.dtype == NOISE_TERM_DTYPE
        t = to_device(terms)
    else:
        t = terms
    n = t.numel() // NOISE_TERM_DTYPE.itemsize if t.dtype == torch.uint8 else len(terms)
    if out is None:
        out = torch.empty((height, width), dtype=torch.float32, device="cuda")
    if workspace is None:
        workspace = empty_bytes(noise_workspace_bytes(n, width, height))
    r = None
    if rates is not None:
        r = rates if hasattr(rates, "data_ptr") else torch.as_tensor(np.asarray(rates, np.float32), device="cuda")
    check(lib().wt_noise_synth_animated(t.data_ptr(), n, _ptr(r), float(time_s), width, height, out.data_ptr(),
                                        workspace.data_ptr(), workspace.numel(), stream_handle(stream)))
    return out


def wave_from_reference(amplitude_A, frequency_w, phase_constant_phi, steepness_Q, dir_x, dir_z,
                        wave_count) -> np.ndarray:
    w = CWave()
    check(lib().wt_wave_from_reference(amplitude_A, frequency_w, phase_constant_phi, steepness_Q, dir_x, dir_z,
                                       wave_count, C.byref(w)))
    out = np.zeros(1, WAVE_DTYPE)
    for n in WAVE_DTYPE.names:
        out[n] = getattr(w, n)
    return out


def set_tuning(warps_per_block: int = 0, blocks_per_sm: int = 0, wave_chunk: int = 0,
               max_vertices_per_lane: int = 0, epilogue_in_shared: int = 1) -> None:
    check(lib().wt_set_tuning(C.byref(CTuning(warps_per_block, blocks_per_sm, wave_chunk, max_vertices_per_lane,
                                              epilogue_in_shared))))


def get_tuning() -> dict:
    t = CTuning()
    check(lib().wt_get_tuning(C.byref(t)))
    return {f: getattr(t, f) for f, _ in CTuning._fields_}


def measure_peaks(stream=None) -> tuple[float, float]:
    scratch = empty_bytes(4 << 20)
    f, s = C.c_double(), C.c_double()
    check(lib().wt_measure_peaks(scratch.data_ptr(), scratch.numel(), C.byref(f), C.byref(s),
                                 stream_handle(stream)))
    return f.value, s.value


# ---- frame set-up and the rest of the vertex stage ---------------------------

def camera(position=(0.0, 4.0, 70.0), yaw_deg=-90.0, pitch_deg=0.0, fov_deg=72.0, aspect=16.0 / 9.0,
           z_near=0.1, z_far=100.0, displaceable_amplitude=0.0) -> np.ndarray:
    """A wt_camera (defaults: the reference's start camera, render-engine.cpp:52)."""
    c = np.zeros(1, CAMERA_DTYPE)
    c["position"] = position
    for k, v in (("yaw_deg", yaw_deg), ("pitch_deg", pitch_deg), ("fov_deg", fov_deg), ("aspect", aspect),
                 ("z_near", z_near), ("z_far", z_far), ("displaceable_amplitude", displaceable_amplitude)):
        c[k] = v
    return c


def displaceable_amplitude(waves: np.ndarray, heightmap_disp_scale: float = 0.0, bounce_amplitude: float = 0.0):
    """DISPLACEABLE_AMPLITUDE of render-engine.cpp:803: total wave amplitude
    + heightmap displacement scale + vertical bounce amplitude."""
    return float(np.sum(np.abs(waves["amplitude"].astype(np.float64)))) + abs(heightmap_disp_scale) + \
        abs(bounce_amplitude)


def projected_grid(cam: np.ndarray, patch: np.ndarray | None = None):
    """Host FP64 projected grid: (patch with corners set, wt_view, status).
    `patch` (one PATCH_DTYPE record) keeps its other fields."""
    assert cam.dtype == CAMERA_DTYPE
    cam = np.ascontiguousarray(cam.reshape(1))
    p = np.zeros(1, PATCH_DTYPE) if patch is None else np.ascontiguousarray(patch.reshape(1)).copy()
    v = np.zeros(1, VIEW_DTYPE)
    st = C.c_uint32()
    check(lib().wt_projected_grid(cam.ctypes.data, p.ctypes.data, v.ctypes.data, C.byref(st)))
    return p, v, st.value


def projected_grid_async(cam_dev, patch_dev, view_dev, stream=None) -> None:
    """Device projected grid: camera (device bytes of a wt_camera) -> corners
    of the device patch and the device wt_view."""
    check(lib().wt_projected_grid_async(cam_dev.data_ptr(), patch_dev.data_ptr(), view_dev.data_ptr(),
                                        stream_handle(stream)))


def vertex_stage(view_dev, pos, nrm=None, flags: int = 0, clip=True, ndc0=True, view=True, facing=True,
                 nrm_yaw=True, out=None, stream=None) -> dict:
    """water-grid.vert's remaining outputs for world positions/normals of
    wt_gerstner_displace.  Returns the dict of (new or given) output tensors."""
    torch = _torch()
    n = pos.shape[0]
    w = 3 if flags & WT_LAYOUT_VEC3 else 4
    out = dict(out or {})
    want = {"clip": (clip, 4), "ndc0": (ndc0, 2), "view": (view, w), "facing": (facing, w), "nrm_yaw": (nrm_yaw, w)}
    for k, (on, width) in want.items():
        if on and k not in out:
            out[k] = torch.empty((n, width), dtype=torch.float32, device=pos.device)
    check(lib().wt_vertex_stage(view_dev.data_ptr(), pos.data_ptr(), _ptr(nrm), n, flags, _ptr(out.get("clip")),
                                _ptr(out.get("ndc0")), _ptr(out.get("view")), _ptr(out.get("facing")),
                                _ptr(out.get("nrm_yaw")), stream_handle(stream)))
    return out


# ---- water shading (the fragment stage) --------------------------------------

def water_shading(**kw) -> CWaterShading:
    """A wt_water_shading: the reference's defaults, overridden by kw."""
    vals = dict(WATER_SHADING_DEFAULTS, **kw)
    s = CWaterShading()
    for k, v in vals.items():
        f = getattr(s, k)
        if hasattr(f, "__len__"):
            f[:] = [float(x) for x in v]
        else:
            setattr(s, k, float(v))
    return s


def water_raster_workspace_bytes(n_vertices: int, n_triangles: int) -> int:
    out = C.c_size_t()
    check(lib().wt_water_raster_workspace_size(n_vertices, n_triangles, C.byref(out)))
    return out.value


def water_raster(clip, indices, width: int, height: int, scene_depth=None, fragments=None, workspace=None,
                 stream=None):
    """Visibility buffer (int64 tensor of height x width keys) of the
    triangles `indices` over float4 clip positions."""
    torch = _torch()
    if fragments is None:
        fragments = torch.empty((height, width), dtype=torch.int64, device=clip.device)
    if workspace is None:
        workspace = empty_bytes(water_raster_workspace_bytes(clip.shape[0], indices.numel() // 3), clip.device)
    check(lib().wt_water_raster(clip.data_ptr(), clip.shape[0], indices.data_ptr(), indices.numel() // 3, width,
                                height, _ptr(scene_depth), fragments.data_ptr(), workspace.data_ptr(),
                                workspace.numel(), stream_handle(stream)))
    return fragments


def water_shade(fragments, clip, indices, stage: dict, width: int, height: int, shading: CWaterShading, skybox,
                scene_depth=None, local_reflections=None, local_refractions=None, colour=None, composite=None,
                stream=None):
    """Shades the water pixels of a visibility buffer.  `stage` holds the
    vertex-stage outputs (facing, nrm_yaw, view, ndc0); skybox: (6, S, S, 4)
    uint8 device tensor; local textures (H, W, 4) uint8; scene depth (H, W)
    float32.  Returns the (H, W, 4) float32 colour tensor (colour=False: none,
    for a call that only blends into `composite`)."""
    torch = _torch()
    if colour is None:
        colour = torch.empty((height, width, 4), dtype=torch.float32, device=clip.device)
    elif colour is False:
        colour = None
    tex = CWaterTextures(_ptr(scene_depth), _ptr(local_reflections), _ptr(local_refractions), skybox.data_ptr(),
                         int(skybox.shape[1]), 0)
    check(lib().wt_water_shade(fragments.data_ptr(), clip.data_ptr(), clip.shape[0], indices.data_ptr(),
                               indices.numel() // 3, stage["facing"].data_ptr(),
                               stage["nrm_yaw"].data_ptr(), stage["view"].data_ptr(), stage["ndc0"].data_ptr(),
                               width, height, C.byref(shading), C.byref(tex), _ptr(colour), _ptr(composite),
                               stream_handle(stream)))
    return colour


def heightmap_from(workload_hm, texels=None) -> DeviceHeightmap | None:
    """Device heightmap of a workloads.Heightmap: synthesised on the GPU
    unless texels are given."""
    if workload_hm is None:
        return None
    if texels is None:
        texels = noise_synth(workload_hm.terms, workload_hm.width, workload_hm.height)
    return DeviceHeightmap(texels, workload_hm.sample_scale, workload_hm.disp_scale, workload_hm.wrap)


__all__ = [
    "abi", "build", "lib", "version", "check", "WtError", "Surface", "DeviceHeightmap", "grid_indices",
    "noise_synth", "wave_from_reference", "measure_peaks", "displace_workspace_bytes",
    "adjoint_workspace_bytes", "workspace_status", "heightmap_from", "PATCH_DTYPE", "WAVE_DTYPE",
    "NOISE_TERM_DTYPE", "WAVE_GRAD_DTYPE", "WT_OUT_WORLD", "WT_OUT_DISPLACEMENT", "WT_LAYOUT_FLOAT4",
    "WT_LAYOUT_VEC3", "WT_PHASE_FP64", "WT_PHASE_FP32_NAIVE", "WT_WRAP_REPEAT", "WT_WRAP_MIRRORED_REPEAT",
    "EXPORTED", "math", "CAMERA_DTYPE", "VIEW_DTYPE", "camera", "displaceable_amplitude", "projected_grid",
    "projected_grid_async", "vertex_stage", "water_shading", "water_raster",
    "water_raster_workspace_bytes", "water_shade",
    "WATER_SHADING_DEFAULTS",
]
