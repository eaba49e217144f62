"""CPU tests of the water fragment-stage oracle (oracle/water.c): its FP32
restatement of water-grid.frag reproduces the reference shader source itself
(compiled as C++) bit for bit, on the committed golden fixtures and (where
the reference checkout is present) on fresh random fragments; its
rasteriser covers every pixel of a watertight mesh exactly once."""
from __future__ import annotations

from pathlib import Path

import numpy as np
import pytest

GOLDEN = Path(__file__).resolve().parent / "golden" / "reference_fragment_stage.npz"
SHADING_KEYS = ("sun_position", "sun_shininess", "sun_strength", "water_clarity", "soft_edges_threshold",
                "tint_threshold", "fog_colour", "fog_radius_near", "fog_radius_far", "z_near", "z_far")
SIZES = {"sun_position": 3, "fog_colour": 4}


def golden_frag_cases():
    z = np.load(GOLDEN)
    out = []
    for n in z["names"]:
        n = str(n)
        c = {k.split("/", 1)[1]: z[k] for k in z.files if k.startswith(n + "/")}
        vals, i, sh = c["shading"], 0, {}
        for k in SHADING_KEYS:
            m = SIZES.get(k, 1)
            sh[k] = tuple(float(x) for x in vals[i:i + m]) if m > 1 else float(vals[i])
            i += m
        c["shading_dict"] = sh
        c["name"] = n
        out.append(c)
    return out


def uniforms_of(O, c):
    W, H = (int(x) for x in c["viewport"])
    return O.frag_uniforms(c["shading_dict"], W, H, scene_depth=c.get("depth"), local_reflections=c.get("refl"),
                           local_refractions=c.get("refr"), skybox=c["sky"])


def bits(a):
    return np.asarray(a, np.float32).view(np.uint32)


def test_restatement_reproduces_golden_bit_exact(oracle):
    for c in golden_frag_cases():
        U, keep = uniforms_of(oracle, c)
        got = oracle.water_fragment(U, c["frags"])
        assert np.array_equal(bits(got), bits(c["colour"])), c["name"]


def test_restatement_matches_reference_shader_random(oracle):
    if oracle.ref_frag_lib() is None:
        pytest.skip("reference checkout not on this machine")
    import sys
    sys.path.insert(0, str(Path(__file__).resolve().parent / "golden"))
    from make_golden_frag import fragments
    rng = np.random.default_rng(77)
    for trial in range(6):
        W, H = int(rng.integers(3, 40)), int(rng.integers(3, 40))
        sh = dict(sun_position=tuple(rng.normal(size=3)), sun_shininess=float(rng.uniform(1, 100)),
                  sun_strength=float(rng.uniform(0, 1)), water_clarity=float(rng.uniform(0, 1)),
                  soft_edges_threshold=float(rng.choice([0.0, rng.uniform(0, 0.2)])),
                  tint_threshold=float(rng.choice([0.0, rng.uniform(0, 0.2)])),
                  fog_colour=tuple(rng.uniform(0, 1, 4)), fog_radius_near=float(rng.uniform(0, 0.4)),
                  fog_radius_far=float(rng.uniform(0.5, 1.0)), z_near=float(rng.uniform(0.05, 1)),
                  z_far=float(rng.uniform(50, 500)))
        S = int(rng.integers(1, 12))
        U, keep = oracle.frag_uniforms(
            sh, W, H, scene_depth=rng.uniform(0.5, 1, (H, W)).astype(np.float32) if trial % 2 else None,
            local_reflections=rng.integers(0, 256, (H, W, 4), dtype=np.uint8) if trial % 3 else None,
            local_refractions=rng.integers(0, 256, (H, W, 4), dtype=np.uint8) if trial % 3 != 1 else None,
            skybox=rng.integers(0, 256, (6, S, S, 4), dtype=np.uint8))
        f = fragments(rng, 2000, W, H)
        a, b = oracle.water_fragment(U, f), oracle.reference_water_fragment(U, f)
        assert np.array_equal(bits(a), bits(b)), trial


def _mask(oracle, clip, tri, W, H):
    k = oracle.water_raster(clip, tri, W, H)
    return (k & 0xffffffff) != 0


def test_raster_covers_a_watertight_mesh_exactly_once(oracle):
    """A jittered triangulated grid spanning more than the viewport: each
    triangle rasterised on its own, the coverage masks are disjoint and cover
    every pixel (shared edges through pixel centres included)."""
    rng = np.random.default_rng(3)
    W, H = 40, 28
    n = 9
    xs, ys = np.meshgrid(np.linspace(-1.3, 1.3, n), np.linspace(-1.3, 1.3, n))
    jit = rng.uniform(-0.08, 0.08, (2, n, n))
    jit[:, 4, :] = 0.0  # one row of vertices exactly on pixel centres / edges
    xs, ys = xs + jit[0], ys + jit[1]
    xs[:, 4] = 2.0 * (np.round((xs[:, 4] + 1) * W / 2 - 0.5) + 0.5) / W - 1.0
    w = rng.uniform(1.0, 3.0, (n, n))
    clip = np.stack([xs * w, ys * w, np.zeros_like(xs), w], axis=-1).reshape(-1, 4).astype(np.float32)
    idx = []
    for r in range(n - 1):
        for c in range(n - 1):
            a, b, d, e = r * n + c, r * n + c + 1, (r + 1) * n + c, (r + 1) * n + c + 1
            idx += [(a, e, d), (a, b, e)]
    count = np.zeros(W * H, np.int32)
    for t in idx:
        count += _mask(oracle, clip, np.array(t, np.uint32), W, H)
    assert count.min() == 1 and count.max() == 1
    whole = oracle.water_raster(clip, np.array(idx, np.uint32).ravel(), W, H)
    assert np.all((whole & 0xffffffff) != 0)


def test_raster_depth_test_and_ties(oracle):
    """GL_LESS against the scene depth; equal depths go to the lower index."""
    W, H = 8, 8
    quad = np.array([[-1, -1, 0, 1], [1, -1, 0, 1], [1, 1, 0, 1], [-1, 1, 0, 1]], np.float32)
    idx = np.array([0, 1, 2, 0, 2, 3, 0, 1, 2, 0, 2, 3], np.uint32)  # the same quad twice
    k = oracle.water_raster(quad, idx, W, H)
    tri = (k & 0xffffffff).astype(np.int64) - 1
    assert set(np.unique(tri)) == {0, 1}
    assert np.all((k >> 32).astype(np.uint32).view(np.float32) == np.float32(0.5))
    depth = np.full((H, W), 0.5, np.float32)
    depth[:, :4] = 0.75
    k = oracle.water_raster(quad, idx, W, H, scene_depth=depth)
    tri = ((k & 0xffffffff).astype(np.int64) - 1).reshape(H, W)
    assert np.all(tri[:, 4:] == -1) and np.all(tri[:, :4] >= 0)  # 0.5 < 0.5 fails, 0.5 < 0.75 passes
