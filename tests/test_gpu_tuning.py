"""Every launch shape the forward kernel supports (and the autotuner may
pick) against the FP64 oracle, through the C ABI: vertices per lane 4 / 8,
8 / 16 / 20 warps per block, register or shared-memory epilogue, wave chunks of
16 and 32.  Shapes with the same vertices per lane tile every patch the same way
and give identical bits."""
from __future__ import annotations

import numpy as np
import pytest

from helpers import angle_deg, rel_err

pytestmark = pytest.mark.gpu

SHAPES = [(8, 8, 0), (8, 16, 0), (8, 20, 0), (8, 8, 1), (8, 16, 1), (4, 8, 0)]  # (vpl, warps, epi)


@pytest.fixture
def default_tuning(wt):
    yield
    wt.check(wt.lib().wt_set_tuning(None))


def test_every_launch_shape(wt, oracle, gpu, default_tuning):
    import torch
    from wave_tool_gb300 import workloads
    w = workloads.small_random(17, n_patches=6, side_range=(2, 400))
    hm = wt.heightmap_from(w.heightmap)
    surf = wt.Surface(w.patches, w.waves, hm)
    tex = hm.texels.cpu().numpy()
    _, disp64, nrm64, edge = oracle.displace_f64(w.patches, w.waves, tex, w.heightmap)
    ok = edge > 1e-3
    first = {}
    for vpl, warps, epi in SHAPES:
        for chunk in (16, 32):
            wt.set_tuning(warps, 0, chunk, vpl, epi)
            assert wt.get_tuning()["epilogue_in_shared"] == epi
            pos, nrm = surf.displace(flags=wt.WT_OUT_DISPLACEMENT)
            torch.cuda.synchronize()
            assert surf.status()[0] == 0
            p, n = pos.cpu().numpy(), nrm.cpu().numpy()
            assert rel_err(p[:, :3].astype(np.float64), disp64) <= 1e-5, (vpl, warps, epi, chunk)
            assert angle_deg(n[ok, :3].astype(np.float64), nrm64[ok]).max() < 1e-2, (vpl, warps, epi, chunk)
            if vpl in first:
                assert np.array_equal(p, first[vpl][0]) and np.array_equal(n, first[vpl][1]), (vpl, warps, epi,
                                                                                                  chunk)
            else:
                first[vpl] = (p, n)


def test_unsupported_shape_is_rejected(wt, gpu, default_tuning):
    with pytest.raises(wt.WtError):
        wt.set_tuning(16, 0, 32, 4, 1)   # 4 vertices per lane only with 8 warps and the register epilogue
    with pytest.raises(wt.WtError):
        wt.set_tuning(8, 0, 32, 8, 3)
    with pytest.raises(wt.WtError):
        wt.set_tuning(20, 0, 32, 8, 1)   # 20 warps only with the register epilogue


def test_autotune_picks_a_supported_shape(wt, gpu, default_tuning):
    from wave_tool_gb300 import workloads
    w = workloads.config3(n_patches=16, seed=4)
    surf = wt.Surface(w.patches, w.waves, wt.heightmap_from(w.heightmap))
    pos, nrm = surf.alloc_outputs(0)
    best = surf.autotune(pos, nrm, reps=2)
    assert (best["max_vertices_per_lane"], best["warps_per_block"], best["epilogue_in_shared"]) in SHAPES
    assert best["wave_chunk"] in (16, 32)
