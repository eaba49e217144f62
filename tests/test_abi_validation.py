"""Host-side argument validation of the frame-stage entry points (no GPU
needed: every call here is rejected before any CUDA call)."""
from __future__ import annotations

import ctypes as C

import pytest

FAKE = 0x10000  # an aligned, never dereferenced address
ODD = 0x10004   # 4-byte aligned, not 8 / 16


@pytest.fixture(scope="module")
def L(wt):
    wt.build()
    return wt.lib()


def test_vertex_stage_rejects_bad_arguments(wt, L):
    E = wt.abi.WT_ERR_INVALID_ARG
    assert L.wt_vertex_stage(None, FAKE, FAKE, 10, 0, FAKE, None, None, None, None, None) == E  # no view
    assert L.wt_vertex_stage(FAKE, None, FAKE, 10, 0, FAKE, None, None, None, None, None) == E  # no positions
    assert L.wt_vertex_stage(FAKE, ODD, FAKE, 10, 0, FAKE, None, None, None, None, None) == E   # float4 misaligned
    assert L.wt_vertex_stage(FAKE, FAKE, None, 10, 0, None, None, None, FAKE, None, None) == E  # facing needs nrm
    assert L.wt_vertex_stage(FAKE, FAKE, FAKE, 10, 0, ODD, None, None, None, None, None) == E   # clip misaligned
    assert L.wt_vertex_stage(FAKE, FAKE, FAKE, 10, 8, FAKE, None, None, None, None, None) == E  # unknown flag
    assert b"wt_vertex_stage" in L.wt_last_error()


def test_water_raster_rejects_bad_arguments(wt, L):
    E, N = wt.abi.WT_ERR_INVALID_ARG, wt.abi.WT_ERR_NOMEM
    ok = (FAKE, 4, FAKE, 2, 64, 32, None, FAKE, FAKE, 16 * 4 + 16 + 16 * 2, None)

    def call(**kw):
        a = list(ok)
        names = ["clip", "nv", "idx", "nt", "w", "h", "depth", "frags", "ws", "wsb", "stream"]
        for k, v in kw.items():
            a[names.index(k)] = v
        return L.wt_water_raster(*a)

    assert call(w=0) == E and call(h=16385) == E
    assert call(frags=None) == E and call(frags=ODD) == E
    assert call(clip=ODD) == E and call(idx=None) == E
    assert call(ws=None) == E and call(wsb=16 * 4 + 16 + 16 * 2 - 1) == N
    sz = C.c_size_t()
    assert L.wt_water_raster_workspace_size(1000, 1800, C.byref(sz)) == 0 and sz.value == 16000 + 16 + 16 * 1800
    assert L.wt_water_raster_workspace_size(1000, 1 << 32, C.byref(sz)) == E


def test_water_shade_rejects_bad_arguments(wt, L):
    E = wt.abi.WT_ERR_INVALID_ARG
    sh = wt.water_shading()
    tex = wt.CWaterTextures(None, None, None, FAKE, 8, 0)

    def call(shading=sh, textures=tex, w=64, h=32, frags=FAKE, ndc0=FAKE, colour=FAKE):
        return L.wt_water_shade(frags, FAKE, 4, FAKE, 2, FAKE, FAKE, FAKE, ndc0, w, h,
                                C.byref(shading) if shading is not None else None,
                                C.byref(textures) if textures is not None else None, colour, None, None)

    assert call(w=0) == E
    assert call(frags=None) == E and call(ndc0=ODD + 2) == E
    assert call(shading=None) == E and call(textures=None) == E
    assert call(textures=wt.CWaterTextures(None, None, None, None, 8, 0)) == E   # a sky box is required
    assert call(shading=wt.water_shading(z_near=0.0)) == E
    assert call(shading=wt.water_shading(z_far=0.05)) == E
    assert call(shading=wt.water_shading(sun_strength=float("nan"))) == E
    assert call(colour=ODD) == E


def test_projected_grid_async_and_unorm8_reject_bad_arguments(wt, L):
    E = wt.abi.WT_ERR_INVALID_ARG
    assert L.wt_projected_grid_async(None, FAKE, FAKE, None) == E
    assert L.wt_projected_grid_async(FAKE, None, FAKE, None) == E
    assert L.wt_projected_grid_async(FAKE, FAKE, None, None) == E
    assert L.wt_heightmap_from_unorm8(FAKE, 16, 16, 5, 80, 1, FAKE, None) == E   # channels
    assert L.wt_heightmap_from_unorm8(FAKE, 16, 16, 4, 60, 1, FAKE, None) == E   # stride < width * channels
    assert L.wt_heightmap_from_unorm8(FAKE, 16, 16, 4, 64, 2, FAKE, None) == E   # flip flag
    assert L.wt_heightmap_from_unorm8(None, 16, 16, 4, 64, 1, FAKE, None) == E
    assert L.wt_heightmap_from_unorm8(FAKE, 0, 16, 4, 64, 1, FAKE, None) == E


def test_saving_and_stage_entry_points_reject_bad_arguments(wt, L):
    """wt_gerstner_displace_saving / _stage and wt_gerstner_adjoint_saved:
    their own arguments are checked before the shared ones and before any
    CUDA call."""
    E, U = wt.abi.WT_ERR_INVALID_ARG, wt.abi.WT_ERR_UNSUPPORTED
    # displace_saving(patches, n, waves, nw, hm, pos, nrm, cap, flags, sums, ws, bytes, stream)
    assert L.wt_gerstner_displace_saving(FAKE, 1, FAKE, 1, None, FAKE, FAKE, 10, 0, None, FAKE, 1 << 20, None) == E
    assert L.wt_gerstner_displace_saving(FAKE, 1, FAKE, 1, None, FAKE, FAKE, 10, 0, ODD, FAKE, 1 << 20, None) == E
    assert L.wt_gerstner_displace_saving(FAKE, 1, FAKE, 1, None, FAKE, FAKE, 10, wt.WT_PHASE_FP32_NAIVE, FAKE,
                                         FAKE, 1 << 20, None) == U
    L.wt_gerstner_displace_saving(FAKE, 1, FAKE, 1, None, FAKE, FAKE, 10, 0, None, FAKE, 1 << 20, None)
    assert b"sums" in L.wt_last_error()
    # adjoint_saved(host_patches, patches, n, waves, nw, hm, d_pos, d_nrm, cap, flags, sums, grad, ws, bytes, stream)
    assert L.wt_gerstner_adjoint_saved(FAKE, FAKE, 1, FAKE, 1, None, FAKE, FAKE, 10, 0, None, FAKE, FAKE,
                                       1 << 20, None) == E
    assert L.wt_gerstner_adjoint_saved(FAKE, FAKE, 1, FAKE, 1, None, FAKE, FAKE, 10, 0, ODD, FAKE, FAKE,
                                       1 << 20, None) == E
    # displace_stage(patches, n, waves, nw, hm, view, pos, nrm, cap, flags, outputs, ws, bytes, stream)
    so = wt.CStageOutputs(FAKE, FAKE, FAKE, FAKE, FAKE)
    stage = L.wt_gerstner_displace_stage
    assert stage(FAKE, 1, FAKE, 1, None, None, None, None, 10, 0, C.byref(so), FAKE, 1 << 20, None) == E  # no view
    assert stage(FAKE, 1, FAKE, 1, None, FAKE, None, None, 10, 0, None, FAKE, 1 << 20, None) == E  # no outputs
    assert stage(FAKE, 1, FAKE, 1, None, FAKE, None, None, 10, wt.WT_OUT_DISPLACEMENT, C.byref(so), FAKE,
                 1 << 20, None) == E
    for field in ("clip", "view", "facing", "nrm_yaw"):
        bad = wt.CStageOutputs(FAKE, FAKE, FAKE, FAKE, FAKE)
        setattr(bad, field, ODD)
        assert stage(FAKE, 1, FAKE, 1, None, FAKE, None, None, 10, 0, C.byref(bad), FAKE, 1 << 20, None) == E, field
    bad = wt.CStageOutputs(FAKE, FAKE + 4, FAKE, FAKE, FAKE)  # ndc0 needs 8-byte alignment
    assert stage(FAKE, 1, FAKE, 1, None, FAKE, None, None, 10, 0, C.byref(bad), FAKE, 1 << 20, None) == E


def test_stage_autotuner_rejects_bad_arguments(wt, L):
    """wt_autotune_displace_stage checks the stage arguments (view, outputs,
    flags, alignment) before timing anything."""
    E = wt.abi.WT_ERR_INVALID_ARG
    so = wt.CStageOutputs(FAKE, FAKE, FAKE, FAKE, FAKE)
    tune = L.wt_autotune_displace_stage
    best = wt.CTuning()
    # (patches, n, waves, nw, hm, view, pos, nrm, cap, flags, outputs, ws, bytes, reps, best, stream)
    assert tune(FAKE, 1, FAKE, 1, None, None, None, None, 10, 0, C.byref(so), FAKE, 1 << 20, 1, C.byref(best),
                None) == E
    assert tune(FAKE, 1, FAKE, 1, None, FAKE, None, None, 10, 0, None, FAKE, 1 << 20, 1, C.byref(best), None) == E
    assert tune(FAKE, 1, FAKE, 1, None, FAKE, None, None, 10, wt.WT_PHASE_FP32_NAIVE, C.byref(so), FAKE, 1 << 20, 1,
                C.byref(best), None) == E
    bad = wt.CStageOutputs(ODD, FAKE, FAKE, FAKE, FAKE)
    assert tune(FAKE, 1, FAKE, 1, None, FAKE, None, None, 10, 0, C.byref(bad), FAKE, 1 << 20, 1, C.byref(best),
                None) == E
    assert b"clip" in L.wt_last_error()
