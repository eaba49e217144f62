"""wt_gerstner_displace_noalloc: the entry point for callers that cannot
allocate device memory (an engine or renderer plugin running inside a host
application's frame, where the host owns every device buffer and a cudaMalloc
could stall the device; a caller that only receives finished input and output
buffers).  Its scratch is a fixed array inside the library instead of a
caller-provided workspace.

Checked through the C ABI against wt_gerstner_displace (which takes a
workspace) on consecutive calls with different patch tables, so that scratch
contents left by one call cannot leak into the next.  Collected last; it also
passes alone in a fresh process (the first call on the device does the
set-up)."""
from __future__ import annotations

import numpy as np
import pytest

from helpers import angle_deg, rel_err

pytestmark = pytest.mark.gpu

DISP_TOL = 1e-5
ANGLE_TOL_DEG = 1e-2


def _noalloc(wt, surf, pos, nrm, flags, n_patches=None, slots=None):
    import torch
    hm = surf.heightmap.cstruct() if surf.heightmap is not None else None
    import ctypes as C
    st = wt.lib().wt_gerstner_displace_noalloc(
        surf.patches.data_ptr(), surf.n_patches if n_patches is None else n_patches,
        surf.wave_slots if slots is None else slots, surf.waves.data_ptr(), surf.n_waves,
        C.byref(hm) if hm is not None else None, pos.data_ptr(), nrm.data_ptr(), pos.shape[0], flags,
        wt.stream_handle())
    torch.cuda.synchronize()
    return st


def _status(wt):
    """wt_noalloc_status: (status, first offending patch)."""
    import ctypes as C
    bad = C.c_uint32(0)
    st = wt.lib().wt_noalloc_status(wt.stream_handle(), C.byref(bad))
    return st, bad.value


def _compare(ref_pos, ref_nrm, pos, nrm):
    """The same launches on the same inputs: the same bits (the tolerances
    of the other parity tests hold a fortiori)."""
    import torch
    a = pos.cpu().numpy().astype(np.float64)
    b = ref_pos.cpu().numpy().astype(np.float64)
    assert rel_err(a[:, :3], b[:, :3]) <= DISP_TOL
    assert angle_deg(nrm.cpu().numpy()[:, :3].astype(np.float64),
                     ref_nrm.cpu().numpy()[:, :3].astype(np.float64)).max() < ANGLE_TOL_DEG
    assert torch.equal(pos, ref_pos) and torch.equal(nrm, ref_nrm)


@pytest.mark.parametrize("flag_name", ["WT_OUT_DISPLACEMENT", "WT_LAYOUT_VEC3", "WT_PHASE_FP32_NAIVE"])
def test_noalloc_matches_workspace_entry_point_on_consecutive_calls(wt, gpu, flag_name):
    """Displacement in float4, world positions in the reference's packed
    vec3 layout, and the FP32-naive phase (its own forward kernel)."""
    import torch
    from wave_tool_gb300 import workloads
    flags = getattr(wt, flag_name)
    cases = [workloads.config3(n_patches=16, seed=2), workloads.small_random(5, n_patches=7, side_range=(2, 200))]
    surfs = [wt.Surface(w.patches, w.waves, wt.heightmap_from(w.heightmap)) for w in cases]
    refs = []
    for s in surfs:
        p, n = s.displace(flags=flags)
        refs.append((p.clone(), n.clone()))
    torch.cuda.synchronize()
    # A, B, then A again right after B: each call must see nothing of the last
    for k in (0, 1, 0):
        s = surfs[k]
        pos, nrm = s.alloc_outputs(flags)
        pos.fill_(float("nan"))
        nrm.fill_(float("nan"))
        assert _noalloc(wt, s, pos, nrm, flags) == 0, wt.lib().wt_last_error()
        assert _status(wt)[0] == 0
        _compare(*refs[k], pos, nrm)


def test_noalloc_rejects_sizes_beyond_its_limits(wt, gpu):
    from wave_tool_gb300 import workloads
    w = workloads.small_random(6, n_patches=2)
    s = wt.Surface(w.patches, w.waves)
    pos, nrm = s.alloc_outputs()
    assert _noalloc(wt, s, pos, nrm, 0, n_patches=1025) == wt.abi.WT_ERR_INVALID_ARG
    assert b"1024" in wt.lib().wt_last_error()
    assert _noalloc(wt, s, pos, nrm, 0, slots=16385) == wt.abi.WT_ERR_INVALID_ARG
    assert b"16384" in wt.lib().wt_last_error()


def test_noalloc_leaves_outputs_unwritten_when_the_wave_slots_overflow_its_scratch(wt, gpu):
    """The host checks the wave-slot count the caller states; when the
    patches' real count is larger than the scratch holds, the first kernel
    refuses the whole table: the call returns WT_OK and writes nothing (as
    documented in wt.h), and the next call with a fitting table runs."""
    import torch
    from wave_tool_gb300 import workloads
    from wave_tool_gb300.abi import PATCH_DTYPE
    base = workloads.small_random(8, n_patches=1, side_range=(2, 4), n_waves_range=(64, 64), heightmap=False)
    waves = base.waves
    n = 300   # 300 patches x 64 waves = 19200 slots > the scratch's 17k
    p0 = base.patches[0]
    pt = np.array([p0] * n, dtype=PATCH_DTYPE)
    verts = int(p0["cols"]) * int(p0["rows"])
    pt["out_offset"] = np.arange(n, dtype=np.uint64) * verts
    pt["wave_offset"] = 0
    pt["wave_count"] = 64
    s = wt.Surface(pt, waves)
    pos, nrm = s.alloc_outputs(0)
    pos.fill_(float("nan"))
    nrm.fill_(float("nan"))
    assert _noalloc(wt, s, pos, nrm, 0, slots=16384) == 0  # understated: passes the host check
    assert torch.isnan(pos).all() and torch.isnan(nrm).all()
    assert _status(wt)[0] == wt.abi.WT_ERR_NOMEM
    small = wt.Surface(pt[:8], waves)
    p2, n2 = small.alloc_outputs(0)
    assert _noalloc(wt, small, p2, n2, 0) == 0
    assert _status(wt)[0] == 0
    ref_p, ref_n = small.displace()
    torch.cuda.synchronize()
    assert torch.equal(p2, ref_p) and torch.equal(n2, ref_n)


def test_noalloc_status_names_the_patch_that_fails_device_side_validation(wt, gpu):
    """A patch whose wave range runs past the wave array passes the host's
    checks (the table is device memory) and fails the first kernel's: the
    call returns WT_OK, that patch's outputs stay unwritten, the others are
    written, and wt_noalloc_status reports WT_ERR_INVALID_ARG at that patch."""
    import torch
    from wave_tool_gb300 import workloads
    w = workloads.small_random(11, n_patches=3, side_range=(4, 40), heightmap=False)
    pt = w.patches.copy()
    pt[1]["wave_offset"] = len(w.waves)
    pt[1]["wave_count"] = 1
    s = wt.Surface(pt, w.waves)
    pos, nrm = s.alloc_outputs(0)
    pos.fill_(float("nan"))
    nrm.fill_(float("nan"))
    assert _noalloc(wt, s, pos, nrm, 0) == 0
    assert _status(wt) == (wt.abi.WT_ERR_INVALID_ARG, 1)
    assert b"patch 1" in wt.lib().wt_last_error()
    for p in range(3):
        o, n = int(pt[p]["out_offset"]), int(pt[p]["cols"]) * int(pt[p]["rows"])
        assert bool(torch.isnan(pos[o:o + n]).all()) == (p == 1)

