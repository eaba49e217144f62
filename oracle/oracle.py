"""ctypes binding of the CPU oracle.  TEST INFRASTRUCTURE ONLY.

Loaded by tests/, by the smoke check and by the CPU-baseline leg of bench.py,
only as the checker / the timed CPU restatement.  The product under
wave-tool_gb300/ never imports this module.
"""
from __future__ import annotations

import ctypes as C
import os
from pathlib import Path

import numpy as np

from . import build as _build

_lib = None
_ref = None


class Heightmap(C.Structure):
    _fields_ = [("texels", C.c_void_p), ("width", C.c_uint32), ("height", C.c_uint32),
                ("sample_scale", C.c_float), ("disp_scale", C.c_float), ("wrap", C.c_uint32),
                ("_pad", C.c_uint32)]


class RefWave(C.Structure):
    _fields_ = [(n, C.c_float) for n in
                ("amplitude_A", "frequency_w", "phaseConstant_phi", "steepness_Q_i", "dir_x", "dir_z")]


class RefUniforms(C.Structure):
    _fields_ = [("bottom_left", C.c_float * 4), ("bottom_right", C.c_float * 4),
                ("top_left", C.c_float * 4), ("top_right", C.c_float * 4),
                ("camera_position", C.c_float * 3), ("grid_length", C.c_uint32),
                ("wave_count", C.c_uint32), ("waves", C.POINTER(RefWave)),
                ("phase_offset", C.POINTER(C.c_float)), ("hm", Heightmap),
                ("vertical_bounce", C.c_float), ("time_s", C.c_float),
                ("view_only_yaw", C.c_float * 16), ("view_projection", C.c_float * 16)]


class RefOutputs(C.Structure):
    _fields_ = [(n, C.POINTER(C.c_float)) for n in
                ("position", "clip", "ndc0", "view", "normal", "normal_yaw", "colour")]


class WaterShading(C.Structure):
    _fields_ = [("sun_position", C.c_float * 3), ("sun_shininess", C.c_float), ("sun_strength", C.c_float),
                ("water_clarity", C.c_float), ("soft_edges_threshold", C.c_float), ("tint_threshold", C.c_float),
                ("fog_colour", C.c_float * 4), ("fog_radius_near", C.c_float), ("fog_radius_far", C.c_float),
                ("z_near", C.c_float), ("z_far", C.c_float)]


class WaterTextures(C.Structure):
    _fields_ = [("scene_depth", C.c_void_p), ("local_reflections", C.c_void_p), ("local_refractions", C.c_void_p),
                ("skybox", C.c_void_p), ("skybox_size", C.c_uint32), ("_pad", C.c_uint32)]


class FragUniforms(C.Structure):
    _fields_ = [("s", WaterShading), ("tex", WaterTextures), ("width", C.c_uint32), ("height", C.c_uint32)]


FRAG_IN_DTYPE = np.dtype([("frag_coord", "<f4", (4,)), ("normal", "<f4", (3,)), ("normal_yaw", "<f4", (3,)),
                          ("view", "<f4", (3,)), ("ndc0", "<f4", (2,))])


def _ptr(a):
    return None if a is None else a.ctypes.data_as(C.c_void_p)


def _fptr(a):
    return None if a is None else a.ctypes.data_as(C.POINTER(C.c_float))


def lib():
    global _lib
    if _lib is None:
        path = _build.LIB
        if not path.exists():
            _build.build_oracle()
        _lib = C.CDLL(str(path))
        vp = C.c_void_p
        _lib.wto_displace_f64.argtypes = [vp, vp, vp, C.c_uint32, C.c_uint32, vp, vp, vp, vp]
        _lib.wto_adjoint_f64.argtypes = [vp, vp, vp, vp, vp, vp]
        _lib.wto_displace_f64_rows.argtypes = [vp, vp, vp, vp, C.c_uint32, vp, vp, vp, vp]
        _lib.wto_reference_vertex.argtypes = [C.POINTER(RefUniforms), C.c_uint32, C.c_uint32,
                                              C.POINTER(RefOutputs)]
        for f in (_lib.wto_cpu_reference, _lib.wto_cpu_analytic):
            f.argtypes = [vp, C.c_uint32, vp, vp, C.c_uint32, C.c_int, vp, vp]
            f.restype = C.c_uint64
        _lib.wto_grid_indices.argtypes = [C.c_uint32, C.c_uint32, C.c_uint32, vp]
        _lib.wto_noise_f64.argtypes = [vp, C.c_uint32, C.c_uint32, C.c_uint32, vp]
        _lib.wto_noise_f64_at.argtypes = [vp, C.c_uint32, vp, C.c_double, C.c_uint32, C.c_uint32, vp]
        _lib.wto_wave_to_reference.argtypes = [vp, C.POINTER(RefWave)]
        for f in (_lib.wto_projected_grid_f32, _lib.wto_projected_grid_f64):
            f.argtypes = [vp, vp, vp, vp, C.POINTER(C.c_uint32)]
            f.restype = C.c_int
        _lib.wto_vertex_stage_f64.argtypes = [vp, vp, vp, C.c_uint64, vp, vp, vp, vp, vp]
        _lib.wto_water_fragment.argtypes = [C.POINTER(FragUniforms), vp, C.c_uint64, vp]
        _lib.wto_water_raster.argtypes = [vp, C.c_uint64, vp, C.c_uint64, C.c_uint32, C.c_uint32, vp, vp]
        _lib.wto_water_shade.argtypes = [vp, vp, vp, vp, vp, vp, vp, C.POINTER(FragUniforms), vp, vp]
    return _lib


def ref_lib():
    """The reference shader compiled from its own source, or None when the
    reference checkout is not on this machine."""
    global _ref
    if _ref is None:
        path = _build.REF_LIB
        if not path.exists():
            if _build.build_ref() is None:
                return None
        _ref = C.CDLL(str(path))
        _ref.wtref_vertex.argtypes = [C.POINTER(RefUniforms), C.c_uint32, C.c_uint32,
                                      C.POINTER(RefOutputs)]
        _ref.wtref_vertex.restype = C.c_int
    return _ref


def make_hm(texels: np.ndarray | None, sample_scale=0.0, disp_scale=0.0, wrap=0) -> Heightmap:
    h = Heightmap()
    if texels is None:
        h.texels = None
        h.width = h.height = 1
    else:
        assert texels.dtype == np.float32 and texels.flags.c_contiguous
        h.texels = texels.ctypes.data
        h.height, h.width = texels.shape
    h.sample_scale, h.disp_scale, h.wrap = sample_scale, disp_scale, wrap
    return h


def displace_f64(patches, waves, texels=None, hm_params=None, rows=None):
    """FP64 truth over every patch.  Returns (pos, disp, nrm, edge) arrays with
    one row per output vertex (placed at each patch's out_offset)."""
    L = lib()
    n_out = int(max(int(p["out_offset"]) + int(p["cols"]) * int(p["rows"]) for p in patches))
    pos = np.zeros((n_out, 3)); disp = np.zeros((n_out, 3)); nrm = np.zeros((n_out, 3))
    edge = np.full(n_out, np.inf)
    hm = None
    if texels is not None:
        hm = make_hm(texels, hm_params.sample_scale, hm_params.disp_scale, hm_params.wrap)
    for p in patches:
        o = int(p["out_offset"]); nv = int(p["cols"]) * int(p["rows"])
        r1 = int(p["rows"]) if rows is None else min(int(p["rows"]), rows)
        pp = np.array(p).copy()
        L.wto_displace_f64(_ptr(pp), _ptr(waves), C.byref(hm) if hm else None, 0, r1,
                           _ptr(pos[o:o + nv]), _ptr(disp[o:o + nv]), _ptr(nrm[o:o + nv]),
                           _ptr(edge[o:o + nv]))
    return pos, disp, nrm, edge


def displace_f64_rows(patch, waves, rows, texels=None, hm_params=None, with_edge=False):
    """FP64 truth on selected rows of one patch: (disp, nrm[, edge]), row k at
    k*cols."""
    L = lib()
    rows = np.ascontiguousarray(rows, dtype=np.uint32)
    cols = int(patch["cols"])
    disp = np.zeros((len(rows) * cols, 3)); nrm = np.zeros((len(rows) * cols, 3))
    edge = np.full(len(rows) * cols, np.inf)
    hm = make_hm(texels, hm_params.sample_scale, hm_params.disp_scale, hm_params.wrap) if texels is not None else None
    pp = np.array(patch).copy()
    L.wto_displace_f64_rows(_ptr(pp), _ptr(waves), C.byref(hm) if hm else None, _ptr(rows), len(rows), None,
                            _ptr(disp), _ptr(nrm), _ptr(edge))
    return (disp, nrm, edge) if with_edge else (disp, nrm)


def sampled_rows(n_rows: int, per_patch: int = 8) -> np.ndarray:
    """The rows of a patch the sampled accuracy check visits: the first, the
    last and per_patch - 2 spread evenly between them."""
    return np.unique(np.round(np.linspace(0, n_rows - 1, min(per_patch, n_rows))).astype(np.uint32))


def accuracy_sampled_rows(patches, waves, disp32, nrm32, texels=None, hm_params=None, per_patch=8,
                          edge_texels=1e-3, threads=None):
    """The path's error metric on sampled rows of EVERY patch of a table,
    against the FP64 truth: displacement error max|d32 - d64| / max|d64| over
    all checked vertices (and the worst single patch), RMS of |d32 - d64| over
    max|d64|, and the largest normal angle (vertices whose heightmap sample
    lies within edge_texels of a texel-cell boundary excluded: the bilinear
    gradient jumps there).  disp32 / nrm32: (n_out, >=3) arrays of the GPU's
    displacement and normal, patch p's vertex (row, col) at out_offset + row *
    cols + col."""
    from concurrent.futures import ThreadPoolExecutor
    threads = threads or os.cpu_count() or 1

    def one(p):
        rows = sampled_rows(int(p["rows"]), per_patch)
        d64, n64, edge = displace_f64_rows(p, waves, rows, texels, hm_params, with_edge=True)
        cols = int(p["cols"])
        idx = (int(p["out_offset"]) + rows.astype(np.int64)[:, None] * cols + np.arange(cols)[None, :]).ravel()
        d = disp32[idx, :3].astype(np.float64)
        n = nrm32[idx, :3].astype(np.float64)
        err = np.abs(d - d64)
        ok = edge > edge_texels
        ang = np.degrees(np.arctan2(np.linalg.norm(np.cross(n[ok], n64[ok]), axis=1),
                                    np.sum(n[ok] * n64[ok], axis=1)))
        return (float(err.max()), float(np.abs(d64).max()), float(np.sum(err ** 2)), len(idx),
                float(ang.max()) if ang.size else 0.0, len(rows), len(idx))

    with ThreadPoolExecutor(max_workers=threads) as ex:
        res = list(ex.map(one, list(patches)))
    emax = max(r[0] for r in res)
    dmax = max(r[1] for r in res)
    return {"max_rel_err": emax / dmax,
            "rms_rel_err": float(np.sqrt(sum(r[2] for r in res) / sum(r[3] for r in res))) / dmax,
            "per_patch_max_rel_err": max(r[0] / r[1] for r in res if r[1] > 0),
            "max_normal_deg": max(r[4] for r in res),
            "patches_checked": len(res), "rows_checked": sum(r[5] for r in res),
            "vertices_checked": sum(r[6] for r in res)}


def adjoint_f64(patches, waves, gpos, gnrm=None, texels=None, hm_params=None):
    L = lib()
    grad = np.zeros((len(waves), 8))
    hm = None
    if texels is not None:
        hm = make_hm(texels, hm_params.sample_scale, hm_params.disp_scale, hm_params.wrap)
    gpos = np.ascontiguousarray(gpos, dtype=np.float32)
    gnrm = None if gnrm is None else np.ascontiguousarray(gnrm, dtype=np.float32)
    for p in patches:
        pp = np.array(p).copy()
        L.wto_adjoint_f64(_ptr(pp), _ptr(waves), C.byref(hm) if hm else None, _ptr(gpos),
                          _ptr(gnrm), _ptr(grad))
    return grad


def reference_uniforms(corners_xz, grid_length, ref_waves, time_s, texels=None, sample_scale=0.02,
                       disp_scale=1.0, wrap=1, bounce=0.0, camera=(0.0, 4.0, 70.0),
                       view_projection=None, view_yaw=None, phase_offset=None):
    """A wto_ref_uniforms; corners_xz = (BL, BR, TL, TR) world xz, ref_waves a
    list of (A, w, phi, Q_i, Dx, Dz).  Returns (uniforms, keepalive)."""
    U = RefUniforms()
    for name, (x, z) in zip(("bottom_left", "bottom_right", "top_left", "top_right"), corners_xz):
        getattr(U, name)[:] = [x, 0.0, z, 1.0]
    U.camera_position[:] = list(camera)
    U.grid_length = grid_length
    arr = (RefWave * max(1, len(ref_waves)))()
    for i, w in enumerate(ref_waves):
        arr[i] = RefWave(*[float(v) for v in w])
    U.wave_count = len(ref_waves)
    U.waves = arr
    ph = None
    if phase_offset is not None:
        ph = np.ascontiguousarray(phase_offset, dtype=np.float32)
        U.phase_offset = _fptr(ph)
    U.hm = make_hm(texels, sample_scale, disp_scale, wrap)
    U.vertical_bounce = bounce
    U.time_s = time_s
    eye = np.eye(4, dtype=np.float32).ravel(order="F")
    U.view_projection[:] = list(eye if view_projection is None else np.asarray(view_projection, np.float32).ravel(order="F"))
    U.view_only_yaw[:] = list(eye if view_yaw is None else np.asarray(view_yaw, np.float32).ravel(order="F"))
    return U, (arr, ph, texels)


def _outputs(n):
    o = {k: np.zeros((n, d), np.float32) for k, d in
         (("position", 4), ("clip", 4), ("ndc0", 2), ("view", 3), ("normal", 3), ("normal_yaw", 3), ("colour", 4))}
    R = RefOutputs(*[_fptr(o[k]) for k in ("position", "clip", "ndc0", "view", "normal", "normal_yaw", "colour")])
    return o, R


def reference_vertex(U, id0, id1):
    """The FP32 restatement (oracle/reference_mode.c)."""
    o, R = _outputs(id1 - id0)
    lib().wto_reference_vertex(C.byref(U), id0, id1, C.byref(R))
    return o


def reference_shader_vertex(U, id0, id1):
    """The reference's own shader source compiled as C++ (oracle/_ref)."""
    r = ref_lib()
    if r is None:
        return None
    o, R = _outputs(id1 - id0)
    R.position = None
    rc = r.wtref_vertex(C.byref(U), id0, id1, C.byref(R))
    if rc != 0:
        raise ValueError("uniforms not expressible by the reference shader")
    del o["position"]
    return o


def projected_grid(cam, fp64=True):
    """src/render-engine.cpp:797-1042 for one wt_camera record: (status,
    corners (4, 2) in the order BL, BR, TL, TR, view-projection (16,),
    yaw-only view (16,), both column-major, number of slab points)."""
    dt = np.float64 if fp64 else np.float32
    corners = np.zeros((4, 2), dt); vp = np.zeros(16, dt); vy = np.zeros(16, dt)
    n = C.c_uint32()
    c = np.ascontiguousarray(cam.reshape(1))
    f = lib().wto_projected_grid_f64 if fp64 else lib().wto_projected_grid_f32
    st = f(_ptr(c), _ptr(corners), _ptr(vp), _ptr(vy), C.byref(n))
    return st, corners, vp, vy, n.value


def vertex_stage_f64(view, pos4, nrm4):
    """water-grid.vert:150-158, 190-193 in FP64 on float4 positions/normals."""
    n = len(pos4)
    out = {"clip": np.zeros((n, 4)), "ndc0": np.zeros((n, 2)), "view": np.zeros((n, 3)),
           "facing": np.zeros((n, 3)), "nrm_yaw": np.zeros((n, 3))}
    v = np.ascontiguousarray(view.reshape(1))
    p = np.ascontiguousarray(pos4, dtype=np.float32)
    q = np.ascontiguousarray(nrm4, dtype=np.float32)
    lib().wto_vertex_stage_f64(_ptr(v), _ptr(p), _ptr(q), n, *[_ptr(out[k]) for k in
                                                                ("clip", "ndc0", "view", "facing", "nrm_yaw")])
    return out


def heightmap_from_unorm8(pixels, flip=True):
    """(h, w, channels) uint8 pixels -> (h, w) float32 texels as the reference
    uploads them: stbi_set_flip_vertically_on_load(true) + stbi_load forced to
    RGBA (src/render-engine.cpp:1310-1311; grey is copied to red), a GL_RGBA8
    texture (src/texture.cpp:66) whose red channel the shader samples
    (water-grid.vert:106), UNORM8 -> float as c / 255."""
    red = np.asarray(pixels, np.uint8)[..., 0]
    if flip:
        red = red[::-1]
    return np.ascontiguousarray(red.astype(np.float32) / np.float32(255.0))


_ref_frag = None


def ref_frag_lib():
    """The reference's water fragment shader compiled from its own source, or
    None when the reference checkout is not on this machine."""
    global _ref_frag
    if _ref_frag is None:
        path = _build.REF_FRAG_LIB
        if not path.exists():
            if _build.build_ref_frag() is None:
                return None
        _ref_frag = C.CDLL(str(path))
        _ref_frag.wtref_fragment.argtypes = [C.POINTER(FragUniforms), C.c_void_p, C.c_uint64, C.c_void_p]
        _ref_frag.wtref_fragment.restype = C.c_int
    return _ref_frag


def frag_uniforms(shading: dict, width, height, scene_depth=None, local_reflections=None, local_refractions=None,
                  skybox=None):
    """A wto_frag_uniforms over host arrays; returns (uniforms, keepalive).
    skybox: (6, S, S, 4) uint8; local textures (H, W, 4) uint8; depth (H, W) float32."""
    U = FragUniforms()
    for k, v in shading.items():
        f = getattr(U.s, k)
        if hasattr(f, "__len__"):
            f[:] = list(v)
        else:
            setattr(U.s, k, float(v))
    keep = []
    for name, arr, dt in (("scene_depth", scene_depth, np.float32), ("local_reflections", local_reflections, np.uint8),
                          ("local_refractions", local_refractions, np.uint8), ("skybox", skybox, np.uint8)):
        if arr is not None:
            a = np.ascontiguousarray(arr, dtype=dt)
            keep.append(a)
            setattr(U.tex, name, a.ctypes.data)
    U.tex.skybox_size = 0 if skybox is None else int(np.asarray(skybox).shape[1])
    U.width, U.height = width, height
    return U, keep


def water_fragment(U, frags):
    """The FP32 restatement of water-grid.frag (oracle/water.c)."""
    f = np.ascontiguousarray(frags, dtype=FRAG_IN_DTYPE)
    out = np.zeros((len(f), 4), np.float32)
    lib().wto_water_fragment(C.byref(U), _ptr(f), len(f), _ptr(out))
    return out


def reference_water_fragment(U, frags):
    """water-grid.frag itself compiled as C++ (oracle/_ref), or None."""
    r = ref_frag_lib()
    if r is None:
        return None
    f = np.ascontiguousarray(frags, dtype=FRAG_IN_DTYPE)
    out = np.zeros((len(f), 4), np.float32)
    if r.wtref_fragment(C.byref(U), _ptr(f), len(f), _ptr(out)) != 0:
        raise ValueError("fragment uniforms need a sky box")
    return out


def water_raster(clip4, idx, width, height, scene_depth=None):
    c = np.ascontiguousarray(clip4, dtype=np.float32)
    i = np.ascontiguousarray(idx, dtype=np.uint32)
    out = np.zeros(width * height, np.uint64)
    d = None if scene_depth is None else np.ascontiguousarray(scene_depth, dtype=np.float32)
    lib().wto_water_raster(_ptr(c), len(c), _ptr(i), len(i) // 3, width, height, _ptr(d), _ptr(out))
    return out


def water_shade(frags, clip4, idx, facing4, nyaw4, view4, ndc0, U, composite=None):
    arrs = [np.ascontiguousarray(a, dtype=np.float32) for a in (clip4, facing4, nyaw4, view4, ndc0)]
    fr = np.ascontiguousarray(frags, dtype=np.uint64)
    i = np.ascontiguousarray(idx, dtype=np.uint32)
    out = np.zeros((U.width * U.height, 4), np.float32)
    comp = None if composite is None else np.ascontiguousarray(composite, dtype=np.float32).copy()
    lib().wto_water_shade(_ptr(fr), _ptr(arrs[0]), _ptr(i), _ptr(arrs[1]), _ptr(arrs[2]), _ptr(arrs[3]),
                          _ptr(arrs[4]), C.byref(U), _ptr(out), _ptr(comp))
    return out, comp


def grid_indices(cols, rows, base=0):
    out = np.zeros(6 * (cols - 1) * (rows - 1), np.uint32)
    lib().wto_grid_indices(cols, rows, base, _ptr(out))
    return out


def noise_f64(terms, width, height, rates=None, time_s=0.0):
    out = np.zeros((height, width))
    t = np.ascontiguousarray(terms)
    r = None if rates is None else np.ascontiguousarray(rates, dtype=np.float32)
    lib().wto_noise_f64_at(_ptr(t), len(t), None if r is None else _ptr(r), float(time_s), width, height, _ptr(out))
    return out


def wave_to_reference(wave):
    r = RefWave()
    w = np.array(wave).copy()
    lib().wto_wave_to_reference(_ptr(w), C.byref(r))
    return (r.amplitude_A, r.frequency_w, r.phaseConstant_phi, r.steepness_Q_i, r.dir_x, r.dir_z)


_timed = None


def timed_lib():
    """The timed CPU baseline: reference_mode.c built for speed
    (build.TIMED_CFLAGS), separate from the bit-exact oracle build."""
    global _timed
    if _timed is None:
        path = _build.build_timed()
        _timed = C.CDLL(str(path))
        vp = C.c_void_p
        _timed.wto_cpu_reference_rows.argtypes = [vp, C.c_uint32, vp, vp, C.c_uint32, C.c_uint32, C.c_int, vp, vp,
                                                  C.c_int]
        _timed.wto_cpu_reference_rows.restype = C.c_uint64
    return _timed


def cpu_baseline_rows(patches, waves, texels=None, hm_params=None, row_stride=1, row_phase=0, threads=None,
                      analytic=False, out=None):
    """The timed CPU restatement over rows row_phase + k * row_stride of every
    patch; returns (vertices, terms).  out: optional (pos4, nrm4) float32
    arrays to write into (allocated when None)."""
    threads = threads or os.cpu_count() or 1
    if out is None:
        n_out = int(max(int(p["out_offset"]) + int(p["cols"]) * int(p["rows"]) for p in patches))
        out = (np.zeros((n_out, 4), np.float32), np.zeros((n_out, 4), np.float32))
    hm = make_hm(texels, hm_params.sample_scale, hm_params.disp_scale, hm_params.wrap) if texels is not None else None
    pp = np.ascontiguousarray(patches)
    nv = timed_lib().wto_cpu_reference_rows(_ptr(pp), len(pp), _ptr(waves), C.byref(hm) if hm else None,
                                            row_stride, row_phase, threads, _ptr(out[0]), _ptr(out[1]),
                                            1 if analytic else 0)
    terms = 0
    for p in patches:
        r = int(p["rows"])
        n_rows = (r - row_phase + row_stride - 1) // row_stride if r > row_phase else 0
        terms += n_rows * int(p["cols"]) * int(p["wave_count"])
    return int(nv), terms


def cpu_baseline(patches, waves, texels=None, hm_params=None, row_limit=1 << 30, threads=None,
                 analytic=False):
    """Runs the timed CPU restatement; returns (vertices, pos4, nrm4)."""
    threads = threads or os.cpu_count() or 1
    n_out = int(max(int(p["out_offset"]) + int(p["cols"]) * int(p["rows"]) for p in patches))
    pos = np.zeros((n_out, 4), np.float32)
    nrm = np.zeros((n_out, 4), np.float32)
    hm = make_hm(texels, hm_params.sample_scale, hm_params.disp_scale, hm_params.wrap) if texels is not None else None
    f = lib().wto_cpu_analytic if analytic else lib().wto_cpu_reference
    pp = np.ascontiguousarray(patches)
    nv = f(_ptr(pp), len(pp), _ptr(waves), C.byref(hm) if hm else None, row_limit, threads,
           _ptr(pos), _ptr(nrm))
    return int(nv), pos, nrm
