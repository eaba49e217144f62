"""CPU tests of the projected grid (wt_projected_grid, a host-only FP64 entry
point of the C ABI) against the oracle's restatements of
src/render-engine.cpp:797-1042.

Tolerances: the library computes in FP64 and rounds the corners to FP32, so
it matches the FP64 oracle to 2^-22 of the largest corner coordinate.  The
FP32 restatement (the reference's precision) differs from FP64 by a median
~1e-4 and up to a few 1e-2 of the corner scale on random cameras (large
world coordinates, high cameras): that is the reference's own rounding
error, reported here, not a bound the library is held to."""
from __future__ import annotations

import numpy as np
import pytest


@pytest.fixture(scope="module")
def built(wt):
    wt.build()
    return wt.lib()


def random_cameras(wt, rng, n):
    for _ in range(n):
        height = rng.choice([rng.uniform(-5.0, 40.0), rng.uniform(-0.5, 0.5), rng.uniform(100.0, 300.0)])
        pitch = rng.choice([rng.uniform(-89.0, 89.0), rng.uniform(-0.2, 0.2), rng.choice([-95.0, 95.0])])
        yield wt.camera(position=(rng.uniform(-500, 500), height, rng.uniform(-500, 500)),
                        yaw_deg=rng.uniform(-720.0, 720.0), pitch_deg=pitch, fov_deg=rng.uniform(20.0, 110.0),
                        aspect=rng.uniform(0.5, 2.5), z_near=rng.uniform(0.05, 1.0), z_far=rng.uniform(50.0, 500.0),
                        displaceable_amplitude=rng.choice([0.0, rng.uniform(0.0, 3.0)]))


def corners_of(p):
    return np.stack([p["bl"][0], p["br"][0], p["tl"][0], p["tr"][0]]).astype(np.float64)


def test_matches_f64_oracle_and_reference_precision(wt, oracle, built):
    rng = np.random.default_rng(7)
    seen = {0: 0, 1: 0}
    err32 = []
    for cam in random_cameras(wt, rng, 600):
        p, v, st = wt.projected_grid(cam)
        s64, c64, vp64, vy64, _ = oracle.projected_grid(cam, fp64=True)
        assert st == s64, cam
        assert int(v["status"][0]) == st
        seen[st] += 1
        np.testing.assert_allclose(v["view_projection"][0], vp64, rtol=0, atol=2e-7 * np.abs(vp64).max())
        np.testing.assert_allclose(v["view_only_yaw"][0], vy64, rtol=0, atol=2e-7 * np.abs(vy64).max())
        np.testing.assert_array_equal(v["camera_position"][0], cam["position"][0].astype(np.float32))
        if st != 1:
            continue
        scale = np.abs(c64).max() + 1.0
        assert np.abs(corners_of(p) - c64).max() <= 2.0 ** -22 * scale, cam
        s32, c32, _, _, _ = oracle.projected_grid(cam, fp64=False)
        if s32 == 1:
            err32.append(float(np.abs(c32 - c64).max() / scale))
    assert seen[0] > 20 and seen[1] > 300, seen
    print(f"FP32 reference-mode corner error / corner scale: median {np.median(err32):.2e}, "
          f"max {np.max(err32):.2e} over {len(err32)} cameras")
    assert np.median(err32) < 1e-3 and np.max(err32) < 0.1


def test_reference_start_camera(wt, oracle, built):
    """The reference's start camera (render-engine.cpp:52: (0, 4, 70), yaw
    -90, fov 72, near 0.1, far 100) over its default waves' amplitude: the
    grid is mirror-symmetric about x = 0 and lies ahead of the camera (-z)."""
    amp = 0.06 + 0.1 + 1.0  # default wave amplitudes + heightmap scale (render-engine.cpp:46-49, render-engine.h)
    cam = wt.camera(aspect=1280.0 / 720.0, displaceable_amplitude=amp)
    p, v, st = wt.projected_grid(cam)
    assert st == wt.abi.WT_VIEW_VISIBLE
    c = corners_of(p)
    s64, c64, _, _, n = oracle.projected_grid(cam)
    assert s64 == 1 and n > 0
    bl, br, tl, tr = c
    tol = 1e-5 * np.abs(c).max()
    assert abs(bl[0] + br[0]) <= tol and abs(tl[0] + tr[0]) <= tol
    assert abs(bl[1] - br[1]) <= tol and abs(tl[1] - tr[1]) <= tol
    assert tl[1] < bl[1] < 70.0  # the far edge is further along -z


def _inside_quad(pts, quad, tol):
    s = []
    for i in range(4):
        a, b = quad[i], quad[(i + 1) % 4]
        s.append((b[0] - a[0]) * (pts[:, 1] - a[1]) - (b[1] - a[1]) * (pts[:, 0] - a[0]))
    s = np.stack(s)
    return np.all(s >= -tol, axis=0) | np.all(s <= tol, axis=0)


def test_grid_covers_the_visible_base_plane(wt, built):
    """Every point of y = 0 the camera sees (rays through its unpadded NDC
    square, within near..far) lies inside the projected grid's quad."""
    rng = np.random.default_rng(11)
    checked = 0
    for cam in random_cameras(wt, rng, 400):
        p, v, st = wt.projected_grid(cam)
        if st != 1:
            continue
        M = v["view_projection"][0].astype(np.float64).reshape(4, 4).T
        Mi = np.linalg.inv(M)
        nd = rng.uniform(-1.0, 1.0, (256, 2))
        a = np.c_[nd, -np.ones(256), np.ones(256)] @ Mi.T
        b = np.c_[nd, np.ones(256), np.ones(256)] @ Mi.T
        a = a[:, :3] / a[:, 3:]
        b = b[:, :3] / b[:, 3:]
        t = -a[:, 1] / (b[:, 1] - a[:, 1])
        ok = (t >= 0) & (t <= 1)
        if not ok.any():
            continue
        pts = (a + t[:, None] * (b - a))[ok][:, [0, 2]]
        c = corners_of(p)
        quad = np.array([c[0], c[1], c[3], c[2]])  # BL, BR, TR, TL around the quad
        assert _inside_quad(pts, quad, 1e-5 * np.abs(quad).max() ** 2).all(), cam
        checked += 1
    assert checked > 100


def test_empty_view_and_invalid_camera(wt, built):
    """A frustum entirely above the slab gives WT_VIEW_EMPTY and leaves the
    patch as it was; invalid cameras are rejected on the host."""
    cam = wt.camera(position=(0.0, 500.0, 0.0), pitch_deg=89.0, z_far=100.0, displaceable_amplitude=2.0)
    before = np.zeros(1, wt.PATCH_DTYPE)
    before["bl"] = (1.0, 2.0)
    p, v, st = wt.projected_grid(cam, before)
    assert st == wt.abi.WT_VIEW_EMPTY and int(v["status"][0]) == st
    assert p.tobytes() == before.tobytes()
    for k, bad in (("fov_deg", 0.0), ("fov_deg", 180.0), ("aspect", 0.0), ("z_near", 0.0), ("z_far", 0.05),
                   ("displaceable_amplitude", -1.0), ("yaw_deg", np.inf), ("pitch_deg", np.nan)):
        c = wt.camera()
        c[k] = bad
        with pytest.raises(wt.WtError) as e:
            wt.projected_grid(c)
        assert e.value.status == wt.abi.WT_ERR_INVALID_ARG


def test_underwater_and_horizon_cameras(wt, oracle, built):
    """Cameras below the surface and exactly level (the SAFE_EPSILON path,
    render-engine.cpp:924-930) agree with the FP64 oracle."""
    for pos_y in (-3.0, -0.01, 0.0, 0.5, 2.0):
        for pitch in (-30.0, -1e-4, 0.0, 1e-4, 30.0):
            cam = wt.camera(position=(5.0, pos_y, -7.0), yaw_deg=33.0, pitch_deg=pitch, aspect=1.5,
                            displaceable_amplitude=1.5)
            p, v, st = wt.projected_grid(cam)
            s64, c64, _, _, _ = oracle.projected_grid(cam)
            assert st == s64 == 1, (pos_y, pitch)
            assert np.abs(corners_of(p) - c64).max() <= 2.0 ** -22 * (np.abs(c64).max() + 1.0)
