"""Generates tests/golden/reference_fragment_stage.npz from the reference's own
water fragment shader (assets/shaders/water-grid.frag compiled as C++ over
oracle/glsl_frag_shim.hpp by oracle/build.py; needs the reference checkout on
this machine).

Each case stores the shader's uniforms (shading parameters, a seeded 8 x 8
sky box, seeded local reflection / refraction textures and scene depth at a
small viewport, or none of the optional textures) and a seeded set of
fragments (gl_FragCoord and varyings) with the colour main() writes for each.

    python tests/golden/make_golden_frag.py
"""
from __future__ import annotations

import sys
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parents[2]
sys.path.insert(0, str(ROOT))

from oracle import oracle as O  # noqa: E402

OUT = Path(__file__).resolve().parent / "reference_fragment_stage.npz"
SHADING_KEYS = ("sun_position", "sun_shininess", "sun_strength", "water_clarity", "soft_edges_threshold",
                "tint_threshold", "fog_colour", "fog_radius_near", "fog_radius_far", "z_near", "z_far")


def fragments(rng, n, W, H):
    f = np.zeros(n, O.FRAG_IN_DTYPE)
    f["frag_coord"][:, 0] = rng.integers(0, W, n) + 0.5
    f["frag_coord"][:, 1] = rng.integers(0, H, n) + 0.5
    f["frag_coord"][:, 2] = rng.uniform(0.8, 1.0, n)
    f["frag_coord"][:, 3] = 1.0
    nrm = rng.normal(size=(n, 3))
    nrm /= np.linalg.norm(nrm, axis=1, keepdims=True)
    nrm[:, 1] = np.abs(nrm[:, 1]) + 0.5
    nrm /= np.linalg.norm(nrm, axis=1, keepdims=True)
    f["normal"] = nrm * rng.uniform(0.97, 1.0, (n, 1))  # interpolated normals are a little short
    ny = rng.normal(size=(n, 3))
    f["normal_yaw"] = ny / np.linalg.norm(ny, axis=1, keepdims=True)
    v = rng.normal(size=(n, 3)) * rng.uniform(0.5, 140.0, (n, 1))
    v[:, 1] = np.abs(v[:, 1])
    f["view"] = v
    f["ndc0"] = rng.uniform(-1.3, 1.3, (n, 2))
    return f


def cases():
    rng = np.random.default_rng(1712)
    W, H = 32, 24
    sky = rng.integers(0, 256, (6, 8, 8, 4), dtype=np.uint8)
    out = []
    base = dict(sun_position=(0.0, 1.0, 0.0), sun_shininess=50.0, sun_strength=1.0, water_clarity=0.3,
                soft_edges_threshold=0.05, tint_threshold=0.1, fog_colour=(1.0, 1.0, 1.0, 0.1), fog_radius_near=0.0,
                fog_radius_far=1.0, z_near=0.1, z_far=100.0)
    # 1. the reference's defaults, noon sun, nothing else drawn
    out.append(dict(name="defaults_noon", shading=base, W=W, H=H, sky=sky))
    # 2. low sun, fog band, every texture present
    a = 0.4
    s2 = dict(base, sun_position=(np.cos(a), np.sin(a), 0.0), sun_shininess=20.0, sun_strength=0.8,
              water_clarity=0.6, fog_colour=(0.7, 0.8, 0.9, 0.5), fog_radius_near=0.2, fog_radius_far=0.7)
    out.append(dict(name="low_sun_fog_textures", shading=s2, W=W, H=H, sky=sky,
                    depth=rng.uniform(0.97, 1.0, (H, W)).astype(np.float32),
                    refl=rng.integers(0, 256, (H, W, 4), dtype=np.uint8),
                    refr=rng.integers(0, 256, (H, W, 4), dtype=np.uint8)))
    # 3. zero thresholds (the 0 == threshold branches), sun below the horizon
    s3 = dict(base, sun_position=(0.0, -0.3, 0.95), soft_edges_threshold=0.0, tint_threshold=0.0)
    out.append(dict(name="zero_thresholds_night", shading=s3, W=W, H=H, sky=sky,
                    depth=rng.uniform(0.9, 1.0, (H, W)).astype(np.float32)))
    for c in out:
        c["frags"] = fragments(rng, 600, W, H)
    return out


def main():
    if O.ref_frag_lib() is None:
        raise SystemExit("reference checkout not found: cannot build the reference fragment shader")
    arrays = {}
    names = []
    for c in cases():
        U, keep = O.frag_uniforms(c["shading"], c["W"], c["H"], scene_depth=c.get("depth"),
                                  local_reflections=c.get("refl"), local_refractions=c.get("refr"), skybox=c["sky"])
        col = O.reference_water_fragment(U, c["frags"])
        n = c["name"]
        names.append(n)
        arrays[f"{n}/shading"] = np.concatenate([np.ravel(np.asarray(c["shading"][k], np.float32))
                                                 for k in SHADING_KEYS])
        arrays[f"{n}/viewport"] = np.array([c["W"], c["H"]], np.uint32)
        arrays[f"{n}/sky"] = c["sky"]
        for k in ("depth", "refl", "refr"):
            if k in c:
                arrays[f"{n}/{k}"] = c[k]
        arrays[f"{n}/frags"] = c["frags"]
        arrays[f"{n}/colour"] = col
    arrays["names"] = np.array(names)
    np.savez_compressed(OUT, **arrays)
    print(f"wrote {OUT} ({OUT.stat().st_size} bytes), cases: {names}")


if __name__ == "__main__":
    main()
