"""Generates tests/golden/reference_vertex_stage.npz from the reference's own
vertex shader (assets/shaders/water-grid.vert compiled as C++ by
oracle/build_ref.py; needs the reference checkout on this machine).

Each case stores the shader's uniforms and every output of its main() for
all gl_VertexID of the grid: gl_Position with the identity view-projection
(= the displaced world position), and with a camera view-projection the
clip position, xyPositionNDCSpaceHeight0, viewVecRaw, normal (after the
camera flip), normalVecInViewSpaceOnlyYaw and heightmap_colour.

Heightmaps are seeded 8-bit grey textures (UNORM8 / 255, as the reference
uploads its PNG), not the reference's asset.

    python tests/golden/make_golden.py
"""
from __future__ import annotations

import math
import sys
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parents[2]
sys.path.insert(0, str(ROOT))

from oracle import oracle as O  # noqa: E402

OUT = Path(__file__).resolve().parent / "reference_vertex_stage.npz"


def perspective(fovy_deg, aspect, near, far):
    f = 1.0 / math.tan(math.radians(fovy_deg) / 2.0)
    m = np.zeros((4, 4))
    m[0, 0] = f / aspect
    m[1, 1] = f
    m[2, 2] = (far + near) / (near - far)
    m[2, 3] = 2.0 * far * near / (near - far)
    m[3, 2] = -1.0
    return m


def look_at(eye, center, up):
    eye, center, up = map(np.asarray, (eye, center, up))
    f = center - eye
    f = f / np.linalg.norm(f)
    s = np.cross(f, up)
    s = s / np.linalg.norm(s)
    u = np.cross(s, f)
    m = np.eye(4)
    m[0, :3], m[1, :3], m[2, :3] = s, u, -f
    m[0, 3], m[1, 3], m[2, 3] = -s @ eye, -u @ eye, f @ eye
    return m


def q_normalised(q_user, w, a, count):
    """render-engine.cpp:1073 in FP32."""
    wa = np.float32(w) * np.float32(a)
    if wa == 0:
        return np.float32(0.0)
    return np.float32(q_user) / (wa * np.float32(count))


def cases():
    rng = np.random.default_rng(591)
    out = []
    # 1. the reference's default waves (render-engine.cpp:46-49), all four
    #    counted by GerstnerWave::Count(), default sampler/scales/camera
    defaults = [(0.06, 1.0, 2.0, 1.0, (1.0, 0.0)), (0.1, 1.0, 0.2, 0.0, (math.sqrt(0.5), math.sqrt(0.5))),
                (0.0, 0.0, 0.0, 0.0, (0.0, 1.0)), (0.0, 0.0, 0.0, 0.0, (0.0, 1.0))]
    waves = [(a, w, p, q_normalised(q, w, a, 4), d[0], d[1]) for a, w, p, q, d in defaults]
    tex = (rng.integers(0, 256, (16, 16)) / 255.0).astype(np.float32)
    out.append(dict(name="defaults", corners=((-30, 30), (30, 30), (-30, -30), (30, -30)), L=17, waves=waves,
                    t=12.5, tex=tex, ss=0.02, ds=1.0, wrap=1, bounce=0.1 * math.sin(2 * math.pi * 0.3),
                    camera=(0.0, 4.0, 70.0)))
    # 2. four random waves, offset patch, repeat wrap, larger texture scale
    rw = []
    for _ in range(4):
        w = float(rng.uniform(0.3, 3.0)); a = float(rng.uniform(0.01, 0.2)); ang = float(rng.uniform(0, 2 * math.pi))
        rw.append((a, w, float(rng.uniform(0, 3)), q_normalised(float(rng.uniform(0, 1)), w, a, 4), math.cos(ang),
                   math.sin(ang)))
    tex2 = (rng.integers(0, 256, (32, 24)) / 255.0).astype(np.float32)
    out.append(dict(name="random4_offset", corners=((480, 540), (530, 545), (470, 495), (525, 490)), L=33,
                    waves=rw, t=250.0, tex=tex2, ss=0.11, ds=0.3, wrap=0, bounce=-0.02, camera=(500.0, 30.0, 600.0)))
    # 3. Q = 0: a pure sine in y
    out.append(dict(name="q0_sine", corners=((-5, 5), (5, 5), (-5, -5), (5, -5)), L=21,
                    waves=[(0.3, 2.0, 1.5, 0.0, 0.6, 0.8)], t=3.0, tex=tex, ss=0.05, ds=0.0, wrap=1, bounce=0.0,
                    camera=(0.0, 10.0, 20.0)))
    # 4. no waves: heightmap only
    out.append(dict(name="heightmap_only", corners=((-8, 8), (8, 8), (-8, -8), (8, -8)), L=25, waves=[], t=0.0,
                    tex=tex2, ss=0.07, ds=0.5, wrap=1, bounce=0.05, camera=(0.0, 5.0, 15.0)))
    # 5. late time (the UI's 3600 s maximum, program.cpp:433)
    out.append(dict(name="late_time", corners=((-30, 30), (30, 30), (-30, -30), (30, -30)), L=17, waves=waves,
                    t=3600.0, tex=tex, ss=0.02, ds=1.0, wrap=1, bounce=0.0, camera=(0.0, 4.0, 70.0)))
    return out


def run_case(c):
    L = c["L"]
    vp = (perspective(72.0, 1.0, 0.1, 1000.0) @ look_at(c["camera"], (c["camera"][0], 0.0, c["camera"][2] - 60.0),
                                                         (0, 1, 0))).astype(np.float32)
    yaw = look_at((0, 0, 0), (0.3, 0.0, -1.0), (0, 1, 0)).astype(np.float32)
    args = dict(texels=c["tex"], sample_scale=c["ss"], disp_scale=c["ds"], wrap=c["wrap"], bounce=c["bounce"],
                camera=c["camera"])
    U0, k0 = O.reference_uniforms(c["corners"], L, c["waves"], c["t"], **args)
    world = O.reference_shader_vertex(U0, 0, L * L)["clip"]
    U1, k1 = O.reference_uniforms(c["corners"], L, c["waves"], c["t"], view_projection=vp, view_yaw=yaw, **args)
    o = O.reference_shader_vertex(U1, 0, L * L)
    return world, vp, yaw, o


def main():
    if O.ref_lib() is None:
        raise SystemExit("reference checkout not found: cannot build the reference shader")
    arrays = {}
    names = []
    for c in cases():
        world, vp, yaw, o = run_case(c)
        n = c["name"]
        names.append(n)
        arrays[f"{n}/corners"] = np.array(c["corners"], np.float32)
        arrays[f"{n}/L"] = np.array(c["L"], np.uint32)
        arrays[f"{n}/waves"] = np.array(c["waves"], np.float32).reshape(-1, 6)
        arrays[f"{n}/scalars"] = np.array([c["t"], c["ss"], c["ds"], c["wrap"], c["bounce"]], np.float32)
        arrays[f"{n}/camera"] = np.array(c["camera"], np.float32)
        arrays[f"{n}/tex"] = c["tex"]
        arrays[f"{n}/view_projection"] = vp
        arrays[f"{n}/view_only_yaw"] = yaw
        arrays[f"{n}/world"] = world
        for k, v in o.items():
            arrays[f"{n}/{k}"] = v
    arrays["names"] = np.array(names)
    np.savez_compressed(OUT, **arrays)
    print(f"wrote {OUT} ({OUT.stat().st_size} bytes), cases: {names}")


if __name__ == "__main__":
    main()
