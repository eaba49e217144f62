"""Helpers shared by the tests: golden-case loading, conversion of reference
uniforms to ABI structs, error metrics."""
from __future__ import annotations

import math
from pathlib import Path

import numpy as np

GOLDEN = Path(__file__).resolve().parent / "golden" / "reference_vertex_stage.npz"


def golden_cases():
    z = np.load(GOLDEN)
    out = []
    for n in z["names"]:
        n = str(n)
        c = {k.split("/", 1)[1]: z[k] for k in z.files if k.startswith(n + "/")}
        c["name"] = n
        out.append(c)
    return out


def golden_uniforms(O, c, identity=False):
    t, ss, ds, wrap, bounce = [float(x) for x in c["scalars"]]
    waves = [tuple(float(v) for v in w) for w in c["waves"]]
    corners = [tuple(float(v) for v in p) for p in c["corners"]]
    kw = dict(texels=np.ascontiguousarray(c["tex"]), sample_scale=ss, disp_scale=ds, wrap=int(wrap), bounce=bounce,
              camera=tuple(float(v) for v in c["camera"]))
    if not identity:
        kw["view_projection"] = c["view_projection"]
        kw["view_yaw"] = c["view_only_yaw"]
    return O.reference_uniforms(corners, int(c["L"]), waves, np.float32(t), **kw)


def golden_to_abi(c):
    """A golden (reference-uniform) case as one wt_patch + wt_waves + heightmap
    parameters: wavelength = 2 pi / w, speed = phi / w, phase 0."""
    from wave_tool_gb300.abi import PATCH_DTYPE, WAVE_DTYPE
    from wave_tool_gb300.workloads import Heightmap
    t, ss, ds, wrap, bounce = [float(x) for x in c["scalars"]]
    L = int(c["L"])
    waves = []
    for a, w, phi, q, dx, dz in c["waves"]:
        lam = 2.0 * math.pi / w if w > 0 else math.inf
        waves.append((a, lam, dx, dz, q, phi / w if w > 0 else 0.0, 0.0, 0.0))
    if not waves:
        waves = [(0.0, 1.0, 1.0, 0.0, 0.0, 0.0, 0.0, 0.0)]
        n = 0
    else:
        n = len(waves)
    bl, br, tl, tr = [tuple(float(v) for v in p) for p in c["corners"]]
    patches = np.array([(bl, br, tl, tr, L, L, 0, n, float(np.float32(t)), bounce, 0, 0)], dtype=PATCH_DTYPE)
    hm = Heightmap(c["tex"].shape[1], c["tex"].shape[0], ss, ds, int(wrap), None)
    return patches, np.array(waves, dtype=WAVE_DTYPE), hm


def rel_err(a, b):
    """max |a - b| / max |b| (the displacement metric of the benchmark)."""
    den = float(np.abs(b).max())
    return float(np.abs(a - b).max()) / (den if den > 0 else 1.0)


def angle_deg(n1, n2):
    """Angle between vectors, atan2(|a x b|, a.b): accurate near zero."""
    return np.degrees(np.arctan2(np.linalg.norm(np.cross(n1, n2), axis=-1), np.sum(n1 * n2, axis=-1)))
