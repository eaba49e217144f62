"""numpy mirrors of the structs in include/wt.h (byte-identical layouts).

The reference keeps these as GL uniforms (assets/shaders/water-grid.vert:37-64)
filled from `struct GerstnerWave` (src/render-engine.h:130-167); here they are
plain arrays that are copied to device memory and handed to the C ABI.
"""
from __future__ import annotations

import numpy as np

WAVE_DTYPE = np.dtype(
    [
        ("amplitude", "<f4"),
        ("wavelength", "<f4"),
        ("dir_x", "<f4"),
        ("dir_z", "<f4"),
        ("steepness_q", "<f4"),
        ("speed", "<f4"),
        ("phase", "<f4"),
        ("_pad", "<f4"),
    ],
    align=True,
)

PATCH_DTYPE = np.dtype(
    [
        ("bl", "<f4", (2,)),
        ("br", "<f4", (2,)),
        ("tl", "<f4", (2,)),
        ("tr", "<f4", (2,)),
        ("cols", "<u4"),
        ("rows", "<u4"),
        ("wave_offset", "<u4"),
        ("wave_count", "<u4"),
        ("time_s", "<f8"),
        ("y_offset", "<f4"),
        ("flags", "<u4"),
        ("out_offset", "<u8"),
    ],
    align=True,
)

NOISE_TERM_DTYPE = np.dtype(
    [("kx", "<i4"), ("ky", "<i4"), ("amplitude", "<f4"), ("phase", "<f4")], align=True
)

WAVE_GRAD_DTYPE = np.dtype(
    [
        ("d_amplitude", "<f4"),
        ("d_wavelength", "<f4"),
        ("d_direction", "<f4"),
        ("d_steepness_q", "<f4"),
        ("d_phase", "<f4"),
        ("d_speed", "<f4"),
        ("d_dir_x", "<f4"),
        ("d_dir_z", "<f4"),
    ],
    align=True,
)

CAMERA_DTYPE = np.dtype(
    [
        ("position", "<f8", (3,)),
        ("yaw_deg", "<f8"),
        ("pitch_deg", "<f8"),
        ("fov_deg", "<f8"),
        ("aspect", "<f8"),
        ("z_near", "<f8"),
        ("z_far", "<f8"),
        ("displaceable_amplitude", "<f8"),
    ],
    align=True,
)

VIEW_DTYPE = np.dtype(
    [
        ("view_projection", "<f4", (16,)),
        ("view_only_yaw", "<f4", (16,)),
        ("camera_position", "<f4", (3,)),
        ("status", "<u4"),
    ],
    align=True,
)

assert WAVE_DTYPE.itemsize == 32
assert PATCH_DTYPE.itemsize == 72
assert NOISE_TERM_DTYPE.itemsize == 16
assert WAVE_GRAD_DTYPE.itemsize == 32
assert CAMERA_DTYPE.itemsize == 80
assert VIEW_DTYPE.itemsize == 144

# status codes (wt_status)
WT_OK = 0
WT_ERR_INVALID_ARG = 1
WT_ERR_CUDA = 2
WT_ERR_TIMEOUT = 3
WT_ERR_NOMEM = 4
WT_ERR_UNSUPPORTED = 5
STATUS_NAMES = {
    0: "WT_OK",
    1: "WT_ERR_INVALID_ARG",
    2: "WT_ERR_CUDA",
    3: "WT_ERR_TIMEOUT",
    4: "WT_ERR_NOMEM",
    5: "WT_ERR_UNSUPPORTED",
}

# flags
WT_WRAP_REPEAT = 0
WT_WRAP_MIRRORED_REPEAT = 1
WT_OUT_WORLD = 0
WT_OUT_DISPLACEMENT = 1
WT_LAYOUT_FLOAT4 = 0
WT_LAYOUT_VEC3 = 2
WT_PHASE_FP64 = 0
WT_PHASE_FP32_NAIVE = 4

# wt_view.status
WT_VIEW_EMPTY = 0
WT_VIEW_VISIBLE = 1
WT_VIEW_INVALID_CAMERA = 2


def patch_vertices(patches: np.ndarray) -> np.ndarray:
    return patches["cols"].astype(np.uint64) * patches["rows"].astype(np.uint64)


def terms_of(patches: np.ndarray) -> int:
    """Gerstner terms (vertices x waves) of a patch table."""
    return int(np.sum(patch_vertices(patches) * patches["wave_count"].astype(np.uint64)))
