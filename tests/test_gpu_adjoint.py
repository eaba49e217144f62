"""GPU adjoint (wt_gerstner_adjoint, through the C ABI) against the FP64
reference gradient (oracle/gerstner_f64.c:wto_adjoint_f64, itself checked
against FP64 central differences in test_oracle.py).

Tolerance: for each gradient field, max over waves |g_gpu - g_64| <=
1e-4 * max over waves |g_64| (the path's 1e-4 relative bound on gradients, taken
relative to the field's scale so that near-zero entries do not divide by zero)."""
from __future__ import annotations

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

GRAD_TOL = 1e-4
FIELDS = ["d_amplitude", "d_wavelength", "d_direction", "d_steepness_q", "d_phase", "d_speed", "d_dir_x", "d_dir_z"]


def _upstream(n, seed, scale_pos=1.0, scale_nrm=1.0):
    import torch
    g = torch.Generator().manual_seed(seed)
    gp = (torch.randn((n, 4), generator=g) * scale_pos).float()
    gn = (torch.randn((n, 4), generator=g) * scale_nrm).float()
    return gp, gn


def _check(grad_gpu, grad64, tol=GRAD_TOL, used=None):
    g = grad_gpu.astype(np.float64)
    if used is not None:
        g, grad64 = g[used], grad64[used]
    for f, name in enumerate(FIELDS):
        scale = np.abs(grad64[:, f]).max()
        err = np.abs(g[:, f] - grad64[:, f]).max()
        assert err <= tol * max(scale, 1e-30), f"{name}: max err {err:.3e} vs scale {scale:.3e}"


EDGE_MARGIN = 2e-3  # texels


def run_adjoint(wt, w, gp, gn, flags=0, texels=None, saved=False, oracle=None):
    """saved: the forward's sums from wt_gerstner_displace_saving instead of
    the adjoint's own recompute.

    oracle (with a heightmap): the upstream gradients gp, gn (CPU tensors) are
    zeroed IN PLACE at the vertices whose FP64 sample point lies within
    EDGE_MARGIN texels of a texel-cell boundary.  The bilinear layer's slope
    and cross derivative jump there, so an FP32 sample point a rounding away
    from the FP64 one can fall in the neighbouring cell; those few vertices
    would measure the cell they landed in, not the gradient arithmetic."""
    import torch
    hm = wt.heightmap_from(w.heightmap, texels)
    surf = wt.Surface(w.patches, w.waves, hm)
    if oracle is not None and hm is not None:
        tex = hm.texels.cpu().numpy()
        edge = oracle.displace_f64(w.patches, w.waves, tex, w.heightmap)[3]
        near = torch.from_numpy(edge < EDGE_MARGIN)
        gp[near[:gp.shape[0]]] = 0
        if gn is not None:
            gn[near[:gn.shape[0]]] = 0
    sums = None
    if saved:
        sums = torch.empty((max(surf.n_vertices, 1), 8), dtype=torch.float32, device="cuda")
        surf.displace(flags=flags & wt.WT_LAYOUT_VEC3, sums=sums)
    grad = surf.adjoint(gp.cuda(), None if gn is None else gn.cuda(), flags=flags, sums=sums)
    torch.cuda.synchronize()
    st, bad = wt.workspace_status(surf.adj_workspace)
    assert st == 0, (st, bad)
    tex = None if hm is None else hm.texels.cpu().numpy()
    return grad.cpu().numpy(), tex


@pytest.mark.parametrize("seed", range(4))
def test_adjoint_no_heightmap(wt, oracle, gpu, seed):
    from wave_tool_gb300 import workloads
    w = workloads.small_random(seed, n_patches=3, side_range=(2, 120), n_waves_range=(1, 40), heightmap=False)
    gp, gn = _upstream(w.n_vertices, seed)
    g, _ = run_adjoint(wt, w, gp, gn)
    g64 = oracle.adjoint_f64(w.patches, w.waves, gp.numpy(), gn.numpy())
    _check(g, g64)


def test_adjoint_position_only_loss(wt, oracle, gpu):
    from wave_tool_gb300 import workloads
    w = workloads.small_random(11, n_patches=2, side_range=(40, 200), heightmap=False)
    gp, _ = _upstream(w.n_vertices, 5)
    g, _ = run_adjoint(wt, w, gp, None)
    g64 = oracle.adjoint_f64(w.patches, w.waves, gp.numpy(), None)
    _check(g, g64)


def test_adjoint_with_noise_heightmap(wt, oracle, gpu):
    """Config-3 patches with the 512^2 noise layer (heightmap gradient and its
    cross derivative in the normal's adjoint)."""
    from wave_tool_gb300 import workloads
    w = workloads.config3(n_patches=4, seed=7)
    gp, gn = _upstream(w.n_vertices, 3, 1.0, 1.0)
    g, tex = run_adjoint(wt, w, gp, gn, oracle=oracle)
    g64 = oracle.adjoint_f64(w.patches, w.waves, gp.numpy(), gn.numpy(), tex, w.heightmap)
    _check(g, g64)


def test_adjoint_deterministic_and_layouts(wt, gpu):
    import torch
    from wave_tool_gb300 import workloads
    w = workloads.config3(n_patches=6, seed=9)
    gp, gn = _upstream(w.n_vertices, 8)
    a, _ = run_adjoint(wt, w, gp, gn)
    b, _ = run_adjoint(wt, w, gp, gn)
    assert np.array_equal(a.view(np.uint32), b.view(np.uint32))
    c, _ = run_adjoint(wt, w, gp[:, :3].contiguous(), gn[:, :3].contiguous(), flags=wt.WT_LAYOUT_VEC3)
    assert np.array_equal(a.view(np.uint32), c.view(np.uint32))
    del torch


def test_adjoint_shared_waves_add_up(wt, oracle, gpu):
    """Three patches over one wave set: each wave's gradient is the sum of its
    per-patch gradients; a wave no patch uses gets zeros."""
    from wave_tool_gb300 import workloads
    w = workloads.small_random(21, n_patches=3, side_range=(20, 90), n_waves_range=(6, 6), heightmap=False)
    patches = w.patches.copy()
    patches["wave_offset"] = 0
    patches["wave_count"] = 5
    waves = w.waves[:6].copy()   # wave 5 is unused
    ws = workloads.Workload("shared", patches, waves)
    gp, gn = _upstream(ws.n_vertices, 2)
    g, _ = run_adjoint(wt, ws, gp, gn)
    g64 = oracle.adjoint_f64(patches, waves, gp.numpy(), gn.numpy())
    assert np.all(g[5] == 0)
    _check(g[:5], g64[:5])


def test_adjoint_validation(wt, gpu):
    from wave_tool_gb300 import workloads
    w = workloads.small_random(2, n_patches=2, heightmap=False)
    surf = wt.Surface(w.patches, w.waves)
    gp, gn = _upstream(w.n_vertices, 1)
    with pytest.raises(wt.WtError):
        surf.adjoint(gp.cuda(), gn.cuda(), flags=wt.WT_PHASE_FP32_NAIVE)
    bad = w.patches.copy()
    bad[1]["cols"] = 1
    s2 = wt.Surface(bad, w.waves)
    grad = s2.adjoint(gp.cuda(), gn.cuda())
    st, first = wt.workspace_status(s2.adj_workspace)
    assert st == wt.abi.WT_ERR_INVALID_ARG and first == 1
    assert np.isfinite(grad.cpu().numpy()).all()


@pytest.mark.parametrize("saved", [False, True])
@pytest.mark.parametrize("seed", range(3))
def test_adjoint_ragged_with_heightmap(wt, oracle, gpu, seed, saved):
    """Ragged patches up to 300 x 300, with and without the heightmap layer
    (both wrap modes): wt_gerstner_adjoint, and wt_gerstner_adjoint_saved (the
    forward's sums instead of a recompute), against the FP64 gradient."""
    from wave_tool_gb300 import workloads
    w = workloads.small_random(seed + 10, n_patches=3, side_range=(2, 300), n_waves_range=(1, 40),
                               heightmap=bool(seed % 2), wrap=seed % 2)
    gp, gn = _upstream(w.n_vertices, seed)
    g, tex = run_adjoint(wt, w, gp, gn, saved=saved, oracle=oracle)
    g64 = oracle.adjoint_f64(w.patches, w.waves, gp.numpy(), gn.numpy(), tex, w.heightmap)
    _check(g, g64)


def test_saving_forward_outputs_and_batched_saved_adjoint(wt, oracle, gpu):
    """The saving forward writes the same positions and normals as the plain
    one; on uneven batched patches the saved-sums adjoint agrees with the
    recomputing one to FP32 rounding of the sums."""
    import torch
    from wave_tool_gb300 import workloads
    w = workloads.config3(n_patches=10, seed=31)
    hm = wt.heightmap_from(w.heightmap)
    surf = wt.Surface(w.patches, w.waves, hm)
    p0, n0 = surf.displace(flags=0)
    sums = torch.empty((surf.n_vertices, 8), dtype=torch.float32, device="cuda")
    p1, n1 = surf.displace(flags=0, sums=sums)
    torch.cuda.synchronize()
    assert torch.equal(p0, p1) and torch.equal(n0, n1)
    assert torch.isfinite(sums).all()
    gp, gn = _upstream(surf.n_vertices, 5)
    gp, gn = gp.cuda(), gn.cuda()
    a = surf.adjoint(gp, gn).cpu().numpy().astype(np.float64)
    b = surf.adjoint(gp, gn, sums=sums).cpu().numpy().astype(np.float64)
    _check(b, a, tol=GRAD_TOL)  # FP32 rounding of the sums (see the chunked-records test)
    with pytest.raises(wt.WtError):
        surf.displace(flags=wt.WT_PHASE_FP32_NAIVE, sums=sums)


def test_chunked_records_match_single_tile_records(wt, gpu):
    """With at least 8 tiles per resident warp the recomputing adjoint takes
    tiles two at a time into one record (header field adj_chunk = 2); its
    gradients agree with the saved-sums adjoint (single-tile records) within
    the path's bound, and repeat bit for bit."""
    import torch
    from wave_tool_gb300 import workloads
    w = workloads.config3(n_patches=64, seed=41)
    surf = wt.Surface(w.patches, w.waves, wt.heightmap_from(w.heightmap))
    sums = torch.empty((surf.n_vertices, 8), dtype=torch.float32, device="cuda")
    surf.displace(flags=0, sums=sums)
    gp, gn = _upstream(surf.n_vertices, 9)
    gp, gn = gp.cuda(), gn.cuda()
    a = surf.adjoint(gp, gn).clone()
    torch.cuda.synchronize()
    hdr = surf.adj_workspace[:32].cpu().numpy().view(np.uint32)
    assert hdr[7] == 2, f"adj_chunk {hdr[7]}: the workload did not take the chunked path"
    b = surf.adjoint(gp, gn).clone()
    c = surf.adjoint(gp, gn, sums=sums)
    torch.cuda.synchronize()
    assert torch.equal(a, b)
    hdr = surf.adj_workspace[:32].cpu().numpy().view(np.uint32)
    assert hdr[7] == 1
    # the saved sums come from the forward's launch shape, the recompute from
    # 4-vertex half tiles (different recurrence lengths): the two differ by
    # FP32 rounding of the sums, within the path's 1e-4 gradient bound
    _check(a.cpu().numpy().astype(np.float64), c.cpu().numpy().astype(np.float64), tol=GRAD_TOL)
