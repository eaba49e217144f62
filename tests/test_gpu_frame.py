"""GPU parity of the per-frame set-up (wt_projected_grid_async) and of the
vertex-stage outputs (wt_vertex_stage), through the C ABI.

 - the device projected grid equals the host FP64 one to FP32 rounding of
   the corners (host and device libm may differ in the last FP64 bit);
 - the vertex stage is held to the FP64 oracle on the same FP32 inputs,
   within a few FP32 roundings of each output's magnitude, and reproduces the
   reference shader's own outputs (tests/golden) when fed the shader's own
   positions and normals;
 - camera -> corners -> displaced vertices -> vertex outputs, captured in one
   CUDA graph and replayed with new cameras, equals the same calls made
   eagerly."""
from __future__ import annotations

import numpy as np
import pytest

from helpers import angle_deg, golden_cases

pytestmark = pytest.mark.gpu

EPS32 = 2.0 ** -24


def dev_view(wt, view_np):
    return wt.to_device(view_np)


def frame_surface(wt, cam, side=257, n_waves=32):
    """config2's waves and noise heightmap on a side x side grid placed by
    the host projected grid of `cam`."""
    from wave_tool_gb300 import workloads
    w = workloads.config2()
    patch = w.patches.copy()
    patch["cols"] = patch["rows"] = side
    patch["wave_count"] = n_waves
    p, view, st = wt.projected_grid(cam, patch)
    assert st == 1
    return wt.Surface(p, w.waves[:n_waves], wt.heightmap_from(w.heightmap)), view


def check_stage_against_f64(out, ref, pos, nrm, view, vec3=False):
    M = view["view_projection"][0].astype(np.float64).reshape(4, 4).T
    p = pos[:, :3].astype(np.float64)
    ph = np.c_[p, np.ones(len(p))]
    S = np.abs(ph) @ np.abs(M).T                     # per-row magnitude bound
    assert np.all(np.abs(out["clip"] - ref["clip"]) <= 4 * EPS32 * S + 1e-30)
    p0 = ph.copy(); p0[:, 1] = 0.0
    c0 = p0 @ M.T
    S0 = np.abs(p0) @ np.abs(M).T
    w = np.abs(c0[:, 3])
    bound = 4 * EPS32 * (S0[:, :2] + np.abs(ref["ndc0"]) * S0[:, 3:4]) / w[:, None] + 2 * EPS32 * np.abs(ref["ndc0"])
    assert np.all(np.abs(out["ndc0"] - ref["ndc0"]) <= bound)
    k = 3
    assert np.all(np.abs(out["view"][:, :k] - ref["view"]) <= EPS32 * np.abs(ref["view"]))
    v = ref["view"]
    n = nrm[:, :3].astype(np.float64)
    d = np.abs(np.sum(n * v, axis=1)) / np.linalg.norm(v, axis=1)
    clear = d > 1e-5                                  # far from the flip's tie
    assert np.array_equal(out["facing"][clear, :k], ref["facing"][clear].astype(np.float32))
    ang = angle_deg(out["nrm_yaw"][clear, :k].astype(np.float64), ref["nrm_yaw"][clear])
    assert ang.max() < 1e-4
    assert np.abs(np.linalg.norm(out["nrm_yaw"][:, :k], axis=1) - 1).max() < 1e-6
    if not vec3:
        for key in ("view", "facing", "nrm_yaw"):
            assert np.all(out[key][:, 3] == 0)
    return clear.mean()


def test_async_projected_grid_matches_host(wt, gpu):
    import torch
    rng = np.random.default_rng(3)
    statuses = set()
    for i in range(40):
        cam = wt.camera(position=(rng.uniform(-200, 200), rng.uniform(-5, 60), rng.uniform(-200, 200)),
                        yaw_deg=rng.uniform(-360, 360), pitch_deg=rng.uniform(-89, 60), fov_deg=rng.uniform(30, 100),
                        aspect=rng.uniform(0.7, 2.2), z_far=rng.uniform(60, 400),
                        displaceable_amplitude=rng.uniform(0, 3))
        patch0 = np.zeros(1, wt.PATCH_DTYPE)
        patch0["cols"] = patch0["rows"] = 9
        ph, vh, st = wt.projected_grid(cam, patch0)
        cd, pd, vd = wt.to_device(cam), wt.to_device(patch0), wt.to_device(np.zeros(1, wt.VIEW_DTYPE))
        wt.projected_grid_async(cd, pd, vd)
        torch.cuda.synchronize()
        pg = pd.cpu().numpy().view(wt.PATCH_DTYPE)
        vg = vd.cpu().numpy().view(wt.VIEW_DTYPE)
        assert int(vg["status"][0]) == st
        statuses.add(st)
        np.testing.assert_allclose(vg["view_projection"][0], vh["view_projection"][0], rtol=0,
                                   atol=2 * EPS32 * np.abs(vh["view_projection"][0]).max())
        np.testing.assert_allclose(vg["view_only_yaw"][0], vh["view_only_yaw"][0], rtol=0,
                                   atol=2 * EPS32 * np.abs(vh["view_only_yaw"][0]).max())
        for k in ("bl", "br", "tl", "tr"):
            scale = max(np.abs(ph[k]).max(), 1.0)
            np.testing.assert_allclose(pg[k], ph[k], rtol=0, atol=4 * EPS32 * scale)
        for k in ("cols", "rows", "time_s", "out_offset"):
            assert pg[k][0] == ph[k][0]
    assert statuses == {0, 1}
    # an invalid camera is reported on the device, the patch left alone
    bad = wt.camera(fov_deg=200.0)
    patch0 = np.zeros(1, wt.PATCH_DTYPE)
    patch0["bl"] = (3.0, 4.0)
    cd, pd, vd = wt.to_device(bad), wt.to_device(patch0), wt.to_device(np.zeros(1, wt.VIEW_DTYPE))
    wt.projected_grid_async(cd, pd, vd)
    torch.cuda.synchronize()
    assert int(vd.cpu().numpy().view(wt.VIEW_DTYPE)["status"][0]) == wt.abi.WT_VIEW_INVALID_CAMERA
    assert pd.cpu().numpy().tobytes() == patch0.tobytes()


@pytest.mark.parametrize("pitch", [-35.0, -4.0, 10.0])
def test_vertex_stage_against_f64(wt, oracle, gpu, pitch):
    """Forward on a camera's projected grid, then every vertex-stage output in
    both layouts against the FP64 oracle on the same positions and normals."""
    import torch
    cam = wt.camera(position=(3.0, 6.0, 20.0), yaw_deg=-80.0, pitch_deg=pitch, aspect=1.6,
                    displaceable_amplitude=2.0)
    surf, view = frame_surface(wt, cam)
    vd = dev_view(wt, view)
    pos, nrm = surf.displace(flags=wt.WT_OUT_WORLD)
    out = wt.vertex_stage(vd, pos, nrm)
    torch.cuda.synchronize()
    P, N = pos.cpu().numpy(), nrm.cpu().numpy()
    ref = oracle.vertex_stage_f64(view, P, N)
    got = {k: v.cpu().numpy() for k, v in out.items()}
    assert check_stage_against_f64(got, ref, P, N, view) > 0.99
    # packed vec3 layout: the same values
    pos3, nrm3 = surf.displace(flags=wt.WT_OUT_WORLD | wt.WT_LAYOUT_VEC3)
    out3 = wt.vertex_stage(vd, pos3, nrm3, flags=wt.WT_LAYOUT_VEC3)
    torch.cuda.synchronize()
    for k in ("view", "facing", "nrm_yaw"):
        assert np.array_equal(out3[k].cpu().numpy(), got[k][:, :3]), k
    for k in ("clip", "ndc0"):
        assert np.array_equal(out3[k].cpu().numpy(), got[k]), k
    # only some outputs, and the facing normal written in place over nrm
    part = wt.vertex_stage(vd, pos, nrm, clip=False, ndc0=True, view=False, facing=False, nrm_yaw=False)
    assert set(part) == {"ndc0"}
    wt.vertex_stage(vd, pos, nrm, clip=False, ndc0=False, view=False, facing=False, nrm_yaw=False,
                    out={"facing": nrm})
    torch.cuda.synchronize()
    assert np.array_equal(part["ndc0"].cpu().numpy(), got["ndc0"])
    assert np.array_equal(nrm.cpu().numpy(), got["facing"])


@pytest.mark.parametrize("tuning", [None, dict(warps_per_block=8, max_vertices_per_lane=4, epilogue_in_shared=0),
                                    dict(warps_per_block=16, max_vertices_per_lane=8, epilogue_in_shared=1)])
def test_fused_vertex_stage_bit_identical(wt, gpu, tuning):
    """wt_gerstner_displace_stage (the vertex stage in the forward's epilogue)
    writes the same bits as wt_gerstner_displace followed by wt_vertex_stage,
    with and without the positions and normals, under each launch shape (the
    shared-memory epilogue shape runs its register twin)."""
    import torch
    cam = wt.camera(position=(3.0, 6.0, 20.0), yaw_deg=-80.0, pitch_deg=-20.0, aspect=1.6,
                    displaceable_amplitude=2.0)
    surf, view = frame_surface(wt, cam, side=301, n_waves=24)
    vd = dev_view(wt, view)
    old = wt.get_tuning()
    try:
        if tuning is not None:
            wt.set_tuning(**tuning)
        pos, nrm = surf.displace(flags=wt.WT_OUT_WORLD)
        ref = wt.vertex_stage(vd, pos, nrm)
        fpos, fnrm = torch.full_like(pos, 7.0), torch.full_like(nrm, 7.0)
        fused = surf.displace_stage(vd, pos=fpos, nrm=fnrm)
        bare = surf.displace_stage(vd)
        pos3, nrm3 = surf.alloc_outputs(wt.WT_LAYOUT_VEC3)
        only_n = torch.full_like(nrm3, 7.0)
        surf.displace_stage(vd, pos=None, nrm=only_n, flags=wt.WT_LAYOUT_VEC3, stage=("clip",))
        torch.cuda.synchronize()
    finally:
        wt.set_tuning(**old)
    assert surf.status()[0] == 0
    assert torch.equal(fpos, pos) and torch.equal(fnrm, nrm)
    for k in ("clip", "ndc0", "view", "facing", "nrm_yaw"):
        assert torch.equal(fused[k], ref[k]), k
        assert torch.equal(bare[k], ref[k]), k
    assert torch.equal(only_n, nrm[:, :3])


@pytest.mark.parametrize("seed", range(3))
def test_fused_vertex_stage_ragged_batches(wt, gpu, seed):
    """Ragged batches (uneven sides, 0..40 waves, skewed corners, both wrap
    modes): the fused vertex stage equals the two-call path bit for bit."""
    import torch
    from wave_tool_gb300 import workloads
    w = workloads.small_random(seed + 50, n_patches=4, side_range=(2, 200), n_waves_range=(0, 40),
                               heightmap=True, wrap=seed % 2)
    surf = wt.Surface(w.patches, w.waves, wt.heightmap_from(w.heightmap))
    cam = wt.camera(position=(10.0, 30.0, 60.0), yaw_deg=-100.0, pitch_deg=-35.0, aspect=1.5,
                    displaceable_amplitude=3.0)
    _, view, _ = wt.projected_grid(cam, w.patches[:1].copy())
    vd = dev_view(wt, view)
    pos, nrm = surf.displace(flags=wt.WT_OUT_WORLD)
    ref = wt.vertex_stage(vd, pos, nrm)
    fused = surf.displace_stage(vd)
    torch.cuda.synchronize()
    assert surf.status()[0] == 0
    covered = np.zeros(surf.n_vertices, bool)
    for p in w.patches:
        o = int(p["out_offset"])
        covered[o:o + int(p["cols"]) * int(p["rows"])] = True
    cov = torch.from_numpy(covered).cuda()
    for k in ("clip", "ndc0", "view", "facing", "nrm_yaw"):
        assert torch.equal(fused[k][cov], ref[k][cov]), k


def test_stage_autotuner_keeps_its_own_shape(wt, gpu):
    """wt_autotune_displace_stage picks one of the candidate shapes and later
    displace_stage calls in that bucket use it (the same bits as with the
    shape set explicitly), while plain displace calls keep theirs; validation
    as displace_stage's."""
    import torch
    cam = wt.camera(position=(3.0, 6.0, 20.0), yaw_deg=-80.0, pitch_deg=-20.0, aspect=1.6,
                    displaceable_amplitude=2.0)
    surf, view = frame_surface(wt, cam, side=257, n_waves=24)
    vd = dev_view(wt, view)
    old = wt.get_tuning()
    try:
        wt.set_tuning(warps_per_block=16, max_vertices_per_lane=8, wave_chunk=32, epilogue_in_shared=0)
        plain_before = surf.displace(flags=wt.WT_OUT_WORLD)[0].clone()
        out = surf.displace_stage(vd)
        best = surf.autotune_stage(vd, out, reps=1)
        assert (best["max_vertices_per_lane"], best["warps_per_block"]) in {(8, 8), (8, 16), (8, 20), (4, 8)}
        assert best["wave_chunk"] in (16, 32)
        tuned = {k: v.clone() for k, v in surf.displace_stage(vd).items()}
        plain_after = surf.displace(flags=wt.WT_OUT_WORLD)[0]
        wt.set_tuning(**best)
        explicit = surf.displace_stage(vd)
        torch.cuda.synchronize()
        with pytest.raises(wt.WtError):
            surf.autotune_stage(vd, out, flags=wt.WT_OUT_DISPLACEMENT, reps=1)
    finally:
        wt.set_tuning(**old)
    assert surf.status()[0] == 0
    assert torch.equal(plain_before, plain_after)
    for k in ("clip", "ndc0", "view", "facing", "nrm_yaw"):
        assert torch.equal(tuned[k], explicit[k]), k


def test_fused_vertex_stage_validation(wt, gpu):
    surf, view = frame_surface(wt, wt.camera(position=(0.0, 4.0, 30.0), displaceable_amplitude=1.0), side=33)
    vd = dev_view(wt, view)
    with pytest.raises(wt.WtError):
        surf.displace_stage(vd, flags=wt.WT_OUT_DISPLACEMENT)
    with pytest.raises(wt.WtError):
        surf.displace_stage(vd, flags=wt.WT_PHASE_FP32_NAIVE)


def test_vertex_stage_reproduces_reference_shader(wt, gpu):
    """Fed the reference shader's own positions and (flipped) normals, the
    kernel reproduces its clip position, NDC at height 0, view vector and
    yaw-only view-space normal (tests/golden: water-grid.vert compiled as
    C++) to a few FP32 roundings; normals given pointing away from the camera
    come back flipped."""
    import torch
    for c in golden_cases():
        view = np.zeros(1, wt.VIEW_DTYPE)
        view["view_projection"] = c["view_projection"].ravel(order="F")
        view["view_only_yaw"] = c["view_only_yaw"].ravel(order="F")
        view["camera_position"] = c["camera"]
        vd = dev_view(wt, view)
        P = np.ascontiguousarray(c["world"], dtype=np.float32)
        N = np.zeros_like(P)
        N[:, :3] = c["normal"]
        N[1::2, :3] *= -1.0  # every other normal turned away: the stage must flip it back
        out = wt.vertex_stage(vd, torch.from_numpy(P).cuda(), torch.from_numpy(N).cuda())
        torch.cuda.synchronize()
        got = {k: v.cpu().numpy() for k, v in out.items()}
        M = c["view_projection"].astype(np.float64)
        ph = P.astype(np.float64)
        S = np.abs(ph) @ np.abs(M).T
        assert np.all(np.abs(got["clip"] - c["clip"]) <= 8 * EPS32 * S), c["name"]
        p0 = ph.copy(); p0[:, 1] = 0.0
        S0 = np.abs(p0) @ np.abs(M).T
        w = np.abs(p0 @ M.T)[:, 3]
        bound = 8 * EPS32 * (S0[:, :2] + np.abs(c["ndc0"]) * S0[:, 3:4]) / w[:, None] + 4 * EPS32 * np.abs(c["ndc0"])
        assert np.all(np.abs(got["ndc0"] - c["ndc0"]) <= bound), c["name"]
        assert np.all(np.abs(got["view"][:, :3] - c["view"]) <= 2 * EPS32 * np.abs(c["view"])), c["name"]
        v = c["view"].astype(np.float64)
        n = c["normal"].astype(np.float64)
        clear = np.abs(np.sum(n * v, 1)) / np.linalg.norm(v, axis=1) > 1e-5
        assert np.array_equal(got["facing"][clear, :3], c["normal"][clear]), c["name"]
        ang = angle_deg(got["nrm_yaw"][clear, :3].astype(np.float64), c["normal_yaw"][clear].astype(np.float64))
        assert ang.max() < 1e-4, c["name"]


def test_camera_to_vertices_frame_graph(wt, gpu):
    """projected grid -> displacement -> vertex stage captured once as a CUDA
    graph; replayed with three new cameras it matches the eager calls."""
    import torch
    cams = [wt.camera(position=(0.0, 4.0, 70.0), aspect=16 / 9, displaceable_amplitude=1.5),
            wt.camera(position=(12.0, 9.0, -30.0), yaw_deg=20.0, pitch_deg=-25.0, aspect=1.3,
                      displaceable_amplitude=1.5),
            wt.camera(position=(-40.0, -2.0, 5.0), yaw_deg=200.0, pitch_deg=15.0, aspect=2.0,
                      displaceable_amplitude=1.5)]
    surf, view = frame_surface(wt, cams[0], side=129, n_waves=16)
    cam_dev = wt.to_device(cams[0])
    view_dev = wt.to_device(view)
    pos, nrm = surf.alloc_outputs(0)
    outs = {k: torch.empty((pos.shape[0], 4 if k != "ndc0" else 2), device="cuda")
            for k in ("clip", "ndc0", "view", "facing", "nrm_yaw")}

    def frame(stream=None):
        wt.projected_grid_async(cam_dev, surf.patches, view_dev, stream=stream)
        surf.displace(pos, nrm, flags=wt.WT_OUT_WORLD, stream=stream)
        wt.vertex_stage(view_dev, pos, nrm, out=outs, stream=stream)

    frame()  # eager warm-up (first-call set-up happens outside the capture)
    torch.cuda.synchronize()
    s = torch.cuda.Stream()
    s.wait_stream(torch.cuda.current_stream())
    g = torch.cuda.CUDAGraph()
    with torch.cuda.graph(g, stream=s):
        frame(stream=s)
    torch.cuda.synchronize()
    for cam in cams:
        cam_dev.copy_(wt.to_device(cam))
        g.replay()
        torch.cuda.synchronize()
        replayed = {k: v.clone() for k, v in outs.items()}
        rpos = pos.clone()
        assert surf.status()[0] == 0
        # eager reference: host projected grid, then the same kernels
        p_host, v_host, st = wt.projected_grid(cam, surf.host_patches)
        assert st == 1
        s2 = wt.Surface(p_host, surf.host_waves, surf.heightmap)
        epos, enrm = s2.displace(flags=wt.WT_OUT_WORLD)
        eout = wt.vertex_stage(wt.to_device(v_host), epos, enrm)
        torch.cuda.synchronize()
        scale = float(epos[:, :3].abs().max())
        assert float((rpos - epos).abs().max()) <= 8 * EPS32 * scale
        for k in ("view", "nrm_yaw"):
            assert float((replayed[k] - eout[k]).abs().max()) <= 1e-4 * max(1.0, float(eout[k].abs().max())), k


@pytest.mark.parametrize("fused", [False, True])
def test_camera_to_pixels_frame_graph(wt, gpu, fused):
    """The whole water pass (projected grid -> displacement -> vertex stage ->
    rasterisation -> shading) captured once; replayed with new cameras it gives
    the same pixels as the same calls made eagerly.  fused: the vertex stage
    in the displacement's epilogue (wt_gerstner_displace_stage)."""
    import torch
    VW, VH = 160, 100
    cams = [wt.camera(position=(0.0, 4.0, 70.0), pitch_deg=-15.0, aspect=VW / VH, displaceable_amplitude=1.5),
            wt.camera(position=(20.0, 6.0, 10.0), yaw_deg=-120.0, pitch_deg=-30.0, aspect=VW / VH,
                      displaceable_amplitude=1.5)]
    surf, view = frame_surface(wt, cams[0], side=97, n_waves=12)
    cam_dev, view_dev = wt.to_device(cams[0]), wt.to_device(view)
    pos, nrm = surf.alloc_outputs(0)
    n = pos.shape[0]
    outs = {k: torch.empty((n, 2 if k == "ndc0" else 4), device="cuda")
            for k in ("clip", "ndc0", "view", "facing", "nrm_yaw")}
    idx = wt.grid_indices(97, 97)
    frags = torch.empty((VH, VW), dtype=torch.int64, device="cuda")
    rws = wt.empty_bytes(wt.water_raster_workspace_bytes(n, idx.numel() // 3))
    colour = torch.empty((VH, VW, 4), dtype=torch.float32, device="cuda")
    gen = torch.Generator(device="cuda").manual_seed(5)
    sky = torch.randint(0, 256, (6, 8, 8, 4), dtype=torch.uint8, device="cuda", generator=gen)
    refl = torch.randint(0, 256, (VH, VW, 4), dtype=torch.uint8, device="cuda", generator=gen)
    shading = wt.water_shading(sun_position=(0.6, 0.8, 0.0))

    def frame(stream=None):
        wt.projected_grid_async(cam_dev, surf.patches, view_dev, stream=stream)
        if fused:
            surf.displace_stage(view_dev, out=outs, stream=stream)
        else:
            surf.displace(pos, nrm, flags=wt.WT_OUT_WORLD, stream=stream)
            wt.vertex_stage(view_dev, pos, nrm, out=outs, stream=stream)
        wt.water_raster(outs["clip"], idx, VW, VH, fragments=frags, workspace=rws, stream=stream)
        wt.water_shade(frags, outs["clip"], idx, outs, VW, VH, shading, sky, local_reflections=refl,
                       colour=colour, stream=stream)

    frame()
    torch.cuda.synchronize()
    s = torch.cuda.Stream()
    s.wait_stream(torch.cuda.current_stream())
    g = torch.cuda.CUDAGraph()
    with torch.cuda.graph(g, stream=s):
        frame(stream=s)
    torch.cuda.synchronize()
    for cam in cams:
        cam_dev.copy_(wt.to_device(cam))
        g.replay()
        torch.cuda.synchronize()
        replayed = (frags.clone(), colour.clone())
        frame()
        torch.cuda.synchronize()
        assert torch.equal(replayed[0], frags) and torch.equal(replayed[1], colour)
        assert float(((frags & 0xffffffff) != 0).float().mean()) > 0.05
