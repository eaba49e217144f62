"""GPU parity of the water fragment stage (wt_water_raster, wt_water_shade)
through the C ABI against the oracle's restatement (oracle/water.c, itself
pinned bit for bit to water-grid.frag compiled as C++).

 - the visibility buffer (coverage, depth, winning triangle) is bit-exact;
 - colours agree to 2e-5 (1 + |c|): both sides round every FP32 operation
   once in the same order; they differ only through the powers: the sun's
   powf (the CUDA and C library implementations differ in the last bits)
   and the Fresnel term's fifth power, which the kernel forms as products
   where the oracle calls powf."""
from __future__ import annotations

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

W, H = 320, 200


def frame(wt, cam, side=129, n_waves=16):
    """camera -> projected grid -> displacement -> vertex stage -> indices."""
    import torch
    from wave_tool_gb300 import workloads
    w = workloads.config2()
    patch = w.patches.copy()
    patch["cols"] = patch["rows"] = side
    patch["wave_count"] = n_waves
    p, view, st = wt.projected_grid(cam, patch)
    assert st == 1
    surf = wt.Surface(p, w.waves[:n_waves], wt.heightmap_from(w.heightmap))
    pos, nrm = surf.displace(flags=wt.WT_OUT_WORLD)
    stage = wt.vertex_stage(wt.to_device(view), pos, nrm)
    idx = wt.grid_indices(side, side)
    torch.cuda.synchronize()
    return stage, idx


def textures(rng, W, H, sky_size=16):
    import torch
    return dict(skybox=torch.from_numpy(rng.integers(0, 256, (6, sky_size, sky_size, 4), dtype=np.uint8)).cuda(),
                scene_depth=torch.from_numpy(rng.uniform(0.985, 1.0, (H, W)).astype(np.float32)).cuda(),
                local_reflections=torch.from_numpy(rng.integers(0, 256, (H, W, 4), dtype=np.uint8)).cuda(),
                local_refractions=torch.from_numpy(rng.integers(0, 256, (H, W, 4), dtype=np.uint8)).cuda())


def np_(t):
    return None if t is None else t.cpu().numpy()


CAMERAS = [
    dict(position=(0.0, 4.0, 70.0), pitch_deg=-12.0, aspect=W / H),
    dict(position=(10.0, 1.2, 20.0), yaw_deg=-70.0, pitch_deg=-40.0, aspect=W / H),     # close: near-plane clipping
    dict(position=(-5.0, -1.5, 30.0), yaw_deg=-100.0, pitch_deg=10.0, aspect=W / H),    # underwater, looking up
]


@pytest.mark.parametrize("cam_kw", CAMERAS)
def test_raster_bit_exact(wt, oracle, gpu, cam_kw):
    import torch
    cam = wt.camera(displaceable_amplitude=1.5, **cam_kw)
    stage, idx = frame(wt, cam)
    clip = stage["clip"]
    rng = np.random.default_rng(5)
    depth = torch.from_numpy(rng.uniform(0.99, 1.0, (H, W)).astype(np.float32)).cuda()
    for sd in (None, depth):
        k = wt.water_raster(clip, idx, W, H, scene_depth=sd)
        torch.cuda.synchronize()
        want = oracle.water_raster(np_(clip), np_(idx).view(np.uint32), W, H, np_(sd))
        got = k.cpu().numpy().view(np.uint64).ravel()
        assert np.array_equal(got, want)
        assert np.mean((want & 0xffffffff) != 0) > 0.05  # the water covers part of the screen
    c = np_(clip)
    print(f"vertices behind the near plane: {(c[:, 2] < -c[:, 3]).sum()} of {len(c)}")


def test_raster_clipping_and_degenerate_triangles(wt, oracle, gpu):
    """A triangle soup with vertices behind the eye, far outside the guard
    band, degenerate and non-finite ones, and out-of-range indices."""
    import torch
    rng = np.random.default_rng(9)
    n = 3000
    clip = np.empty((n, 4), np.float32)
    w = rng.uniform(-2.0, 6.0, n)
    clip[:, 3] = w
    clip[:, 0] = rng.normal(size=n) * np.abs(w) * rng.choice([0.5, 2.0, 300.0], n)
    clip[:, 1] = rng.normal(size=n) * np.abs(w) * rng.choice([0.5, 2.0, 300.0], n)
    clip[:, 2] = rng.uniform(-1.2, 1.2, n) * np.abs(w)
    clip[5] = (np.nan, 0.0, 0.0, 1.0)
    clip[6] = (0.0, 0.0, 0.0, 0.0)
    idx = rng.integers(0, n, (4000, 3)).astype(np.uint32)
    idx[10] = (1, 1, 2)          # degenerate
    idx[11] = (5, 6, 7)          # non-finite / w = 0
    idx[12] = (0, 1, n + 5)      # out of range: skipped
    ct, it = torch.from_numpy(clip).cuda(), torch.from_numpy(idx.view(np.int32).ravel()).cuda()
    k = wt.water_raster(ct, it, W, H)
    torch.cuda.synchronize()
    want = oracle.water_raster(clip, idx.ravel(), W, H)
    assert np.array_equal(k.cpu().numpy().view(np.uint64).ravel(), want)
    assert np.mean((want & 0xffffffff) != 0) > 0.5


def test_raster_large_triangles_take_the_second_pass(wt, oracle, gpu):
    """A full-viewport quad (two triangles of 64,000 box pixels), triangles
    with boxes around and above the per-thread limit of 128 pixels (about
    8 x 16 to 16 x 23) and one of exactly 128, over a field of one-pixel
    triangles: the queue, its spread over the warps and the per-thread path
    give the oracle's buffer bit for bit."""
    import torch
    rng = np.random.default_rng(31)
    verts, tris = [], []

    def add(pts):
        base = len(verts)
        verts.extend(pts)
        tris.append((base, base + 1, base + 2))
    add([(-1.0, -1.0, 0.5, 1.0), (1.0, -1.0, 0.5, 1.0), (1.0, 1.0, 0.5, 1.0)])
    add([(-1.0, -1.0, 0.4, 1.0), (1.0, 1.0, 0.4, 1.0), (-1.0, 1.0, 0.6, 1.0)])
    for k in range(40):                      # boxes of about 8 x 16 .. 16 x 23 pixels
        x0, y0 = rng.uniform(-0.9, 0.8), rng.uniform(-0.9, 0.8)
        dx, dy = (8 + k / 5) * 2 / W, (16 + k / 6) * 2 / H
        add([(x0, y0, 0.3, 1.0), (x0 + dx, y0, 0.35, 1.0), (x0, y0 + dy, 0.25, 1.0)])
    add([(0.0, 0.0, 0.2, 1.0), (16 * 2 / W, 0.0, 0.2, 1.0), (0.0, 8 * 2 / H, 0.2, 1.0)])  # 128-pixel box
    for k in range(3000):                    # one-pixel triangles
        x0, y0 = rng.uniform(-1, 1), rng.uniform(-1, 1)
        add([(x0, y0, 0.1, 1.0), (x0 + 2.2 / W, y0, 0.1, 1.0), (x0, y0 + 2.2 / H, 0.1, 1.0)])
    clip = np.asarray(verts, np.float32)
    idx = np.asarray(tris, np.uint32)
    ct, it = torch.from_numpy(clip).cuda(), torch.from_numpy(idx.view(np.int32).ravel()).cuda()
    got = wt.water_raster(ct, it, W, H)
    torch.cuda.synchronize()
    want = oracle.water_raster(clip, idx.ravel(), W, H)
    assert np.array_equal(got.cpu().numpy().view(np.uint64).ravel(), want)
    assert np.all((want & 0xffffffff) != 0)  # the quad covers every pixel


def test_raster_reuses_its_workspace(wt, oracle, gpu):
    """One workspace for consecutive frames of different meshes (A, B, A):
    the queue of large and clipped triangles starts empty every call."""
    import torch
    meshes = []
    for cam_kw, side in ((CAMERAS[1], 129), (CAMERAS[0], 65)):
        stage, idx = frame(wt, wt.camera(displaceable_amplitude=1.5, **cam_kw), side=side)
        meshes.append((stage["clip"], idx, oracle.water_raster(np_(stage["clip"]), np_(idx).view(np.uint32), W, H)))
    ws = wt.empty_bytes(max(wt.water_raster_workspace_bytes(c.shape[0], i.numel() // 3) for c, i, _ in meshes))
    for k in (0, 1, 0):
        clip, idx, want = meshes[k]
        got = wt.water_raster(clip, idx, W, H, workspace=ws)
        torch.cuda.synchronize()
        assert np.array_equal(got.cpu().numpy().view(np.uint64).ravel(), want)


@pytest.mark.parametrize("cam_kw", CAMERAS[:2])
def test_shade_against_oracle(wt, oracle, gpu, cam_kw):
    import torch
    cam = wt.camera(displaceable_amplitude=1.5, **cam_kw)
    stage, idx = frame(wt, cam)
    rng = np.random.default_rng(13)
    tx = textures(rng, W, H)
    a = 0.5
    sh = wt.water_shading(sun_position=(np.cos(a), np.sin(a), 0.0), fog_colour=(0.8, 0.85, 0.9, 0.3),
                          fog_radius_near=0.1, fog_radius_far=0.6)
    frags = wt.water_raster(stage["clip"], idx, W, H, scene_depth=tx["scene_depth"])
    comp0 = torch.from_numpy(rng.uniform(0, 1, (H, W, 4)).astype(np.float32)).cuda()
    comp = comp0.clone()
    col = wt.water_shade(frags, stage["clip"], idx, stage, W, H, sh, composite=comp, **tx)
    torch.cuda.synchronize()
    shd = {k: getattr(sh, k) for k, _ in sh._fields_}
    shd = {k: (tuple(v) if hasattr(v, "__len__") else v) for k, v in shd.items()}
    U, keep = oracle.frag_uniforms(shd, W, H, scene_depth=np_(tx["scene_depth"]),
                                   local_reflections=np_(tx["local_reflections"]),
                                   local_refractions=np_(tx["local_refractions"]), skybox=np_(tx["skybox"]))
    want, want_comp = oracle.water_shade(frags.cpu().numpy().view(np.uint64).ravel(), np_(stage["clip"]),
                                         np_(idx).view(np.uint32), np_(stage["facing"]), np_(stage["nrm_yaw"]),
                                         np_(stage["view"]), np_(stage["ndc0"]), U,
                                         composite=np_(comp0).reshape(-1, 4))
    got = col.cpu().numpy().reshape(-1, 4)
    water = (frags.cpu().numpy().view(np.uint64).ravel() & 0xffffffff) != 0
    assert water.mean() > 0.05
    tol = 2e-5 * (1.0 + np.abs(want))
    print(f"max colour difference against the oracle: {float(np.abs(got - want).max()):.2e}")
    assert np.all(np.abs(got - want) <= tol), float(np.abs(got - want).max())
    assert np.all(got[~water] == 0.0)
    gc = comp.cpu().numpy().reshape(-1, 4)
    assert np.all(np.abs(gc - want_comp) <= 2e-5 * (1.0 + np.abs(want_comp)))
    assert np.array_equal(gc[~water], np_(comp0).reshape(-1, 4)[~water])


def test_shade_without_optional_textures(wt, oracle, gpu):
    import torch
    cam = wt.camera(displaceable_amplitude=1.5, **CAMERAS[0])
    stage, idx = frame(wt, cam, side=65)
    rng = np.random.default_rng(2)
    sky = torch.from_numpy(rng.integers(0, 256, (6, 4, 4, 4), dtype=np.uint8)).cuda()
    sh = wt.water_shading()
    frags = wt.water_raster(stage["clip"], idx, W, H)
    col = wt.water_shade(frags, stage["clip"], idx, stage, W, H, sh, sky)
    torch.cuda.synchronize()
    shd = {k: getattr(sh, k) for k, _ in sh._fields_}
    shd = {k: (tuple(v) if hasattr(v, "__len__") else v) for k, v in shd.items()}
    U, keep = oracle.frag_uniforms(shd, W, H, skybox=np_(sky))
    want, _ = oracle.water_shade(frags.cpu().numpy().view(np.uint64).ravel(), np_(stage["clip"]),
                                 np_(idx).view(np.uint32), np_(stage["facing"]), np_(stage["nrm_yaw"]),
                                 np_(stage["view"]), np_(stage["ndc0"]), U)
    got = col.cpu().numpy().reshape(-1, 4)
    assert np.all(np.abs(got - want) <= 2e-5 * (1.0 + np.abs(want)))
    water = (frags.cpu().numpy().view(np.uint64).ravel() & 0xffffffff) != 0
    assert np.all(got[water, 3] == 1.0)  # nothing behind the water: hard edges
    with pytest.raises(wt.WtError):
        wt.water_shade(frags, stage["clip"], idx, stage, W, H, wt.water_shading(z_near=0.0), sky)
