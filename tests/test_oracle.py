"""CPU tests of the oracle: pinned to the reference shader itself, to the
golden fixtures made from it, and to known answers."""
from __future__ import annotations

import math
import struct
import zlib
from pathlib import Path

import numpy as np
import pytest

from helpers import golden_cases, golden_uniforms, rel_err

from oracle.build import reference_dir  # noqa: E402

REF_ASSET = reference_dir() / "assets" / "textures" / "noise" / "waves" / "waves3" / "00.png"


def decode_grey_png(path: Path) -> np.ndarray:
    """8-bit greyscale PNG decoder (zlib + the five scanline filters)."""
    d = path.read_bytes()
    assert d[:8] == b"\x89PNG\r\n\x1a\n"
    pos, idat, w, h = 8, b"", 0, 0
    while pos < len(d):
        ln, = struct.unpack(">I", d[pos:pos + 4]); typ = d[pos + 4:pos + 8]; body = d[pos + 8:pos + 8 + ln]
        if typ == b"IHDR":
            w, h, depth, ctype = struct.unpack(">IIBB", body[:10])
            assert depth == 8 and ctype == 0
        elif typ == b"IDAT":
            idat += body
        pos += 12 + ln
    raw = zlib.decompress(idat)
    img = np.zeros((h, w), np.int32)
    prev = np.zeros(w, np.int32)
    for r in range(h):
        f = raw[r * (w + 1)]
        line = np.frombuffer(raw, np.uint8, w, r * (w + 1) + 1).astype(np.int32)
        out = np.zeros(w, np.int32)
        if f == 0:
            out = line
        elif f == 2:
            out = (line + prev) & 255
        else:
            for i in range(w):
                a = out[i - 1] if i else 0
                b = prev[i]
                c = prev[i - 1] if i else 0
                if f == 1:
                    x = a
                elif f == 3:
                    x = (a + b) // 2
                else:
                    p = a + b - c
                    pa, pb, pc = abs(p - a), abs(p - b), abs(p - c)
                    x = a if pa <= pb and pa <= pc else (b if pb <= pc else c)
                out[i] = (line[i] + x) & 255
        img[r] = out
        prev = out
    return img


def equal_bits(a, b):
    return np.array_equal(np.asarray(a, np.float32).view(np.uint32), np.asarray(b, np.float32).view(np.uint32))


def test_port_reproduces_golden_bit_exact(oracle):
    """The FP32 restatement reproduces every output of the reference shader
    (fixtures made from the shader source) bit for bit."""
    for c in golden_cases():
        U, keep = golden_uniforms(oracle, c, identity=True)
        L = int(c["L"])
        o = oracle.reference_vertex(U, 0, L * L)
        assert equal_bits(o["clip"], c["world"]), c["name"]
        assert equal_bits(o["position"], c["world"]), c["name"]
        U, keep = golden_uniforms(oracle, c)
        o = oracle.reference_vertex(U, 0, L * L)
        for k in ("clip", "ndc0", "view", "normal", "normal_yaw", "colour"):
            assert equal_bits(o[k], c[k]), (c["name"], k)


def test_port_matches_reference_shader_on_real_asset(oracle):
    """Against the reference shader compiled from its own source, with the
    reference's heightmap asset (flipped on load like stbi_set_flip_vertically_on_load,
    render-engine.cpp:1310), its default waves and sampler state."""
    if oracle.ref_lib() is None or not REF_ASSET.exists():
        pytest.skip("reference checkout not on this machine")
    img = decode_grey_png(REF_ASSET)
    tex = (img[::-1] / 255.0).astype(np.float32)
    tex = np.ascontiguousarray(tex)
    q0 = np.float32(1.0) / (np.float32(1.0) * np.float32(0.06) * np.float32(4))
    waves = [(0.06, 1.0, 2.0, float(q0), 1.0, 0.0), (0.1, 1.0, 0.2, 0.0, math.sqrt(0.5), math.sqrt(0.5)),
             (0.0, 0.0, 0.0, 0.0, 0.0, 1.0), (0.0, 0.0, 0.0, 0.0, 0.0, 1.0)]
    for L, t, corners in ((33, 7.25, ((-40, 60), (45, 55), (-35, -20), (40, -25))),
                          (65, 1234.5, ((-200, 200), (200, 200), (-200, -200), (200, -200)))):
        U, keep = oracle.reference_uniforms(corners, L, waves, t, texels=tex, sample_scale=0.02, disp_scale=1.0,
                                            wrap=1, bounce=0.07)
        a = oracle.reference_vertex(U, 0, L * L)
        b = oracle.reference_shader_vertex(U, 0, L * L)
        for k in b:
            assert equal_bits(a[k], b[k]), k


def test_port_matches_reference_shader_random(oracle):
    if oracle.ref_lib() is None:
        pytest.skip("reference checkout not on this machine")
    rng = np.random.default_rng(3)
    for trial in range(6):
        n = int(rng.integers(0, 5))
        waves = []
        for _ in range(n):
            ang = rng.uniform(0, 2 * math.pi)
            waves.append((rng.uniform(0, 0.5), rng.uniform(0, 2), rng.uniform(0, 5), rng.uniform(0, 1),
                          math.cos(ang), math.sin(ang)))
        tex = rng.random((int(rng.integers(2, 40)), int(rng.integers(2, 40)))).astype(np.float32)
        L = int(rng.integers(2, 30))
        c = rng.uniform(-1000, 1000, 2)
        corners = tuple((c[0] + rng.uniform(-50, 50), c[1] + rng.uniform(-50, 50)) for _ in range(4))
        U, keep = oracle.reference_uniforms(corners, L, waves, float(rng.uniform(0, 3600)), texels=tex,
                                            sample_scale=float(rng.uniform(0, 0.5)),
                                            disp_scale=float(rng.uniform(0, 2)), wrap=int(trial % 2),
                                            bounce=float(rng.uniform(-1, 1)))
        a = oracle.reference_vertex(U, 0, L * L)
        b = oracle.reference_shader_vertex(U, 0, L * L)
        for k in b:
            assert equal_bits(a[k], b[k]), (trial, k)


def _one_patch(L=41, half=20.0, cx=0.0, cz=0.0, t=5.0):
    from wave_tool_gb300.abi import PATCH_DTYPE
    return np.array([((cx - half, cz + half), (cx + half, cz + half), (cx - half, cz - half), (cx + half, cz - half),
                      L, L, 0, 0, t, 0.0, 0, 0)], dtype=PATCH_DTYPE)


def _waves(rows):
    from wave_tool_gb300.abi import WAVE_DTYPE
    return np.array([tuple(r) + (0.0,) * (8 - len(r)) for r in rows], dtype=WAVE_DTYPE)


def test_f64_agrees_with_reference_mode(oracle):
    """FP64 truth vs the FP32 shader restatement: same conventions (direction
    sign, -z texture flip, mirrored wrap, bounce), differing only by FP32
    rounding."""
    from wave_tool_gb300 import workloads
    w = workloads.config1()
    p = w.patches.copy()
    p["cols"] = p["rows"] = 65
    waves = w.waves.copy()
    waves["phase"] = 0.0
    p["wave_count"] = len(waves)
    tex = np.random.default_rng(1).random((32, 32)).astype(np.float32)
    hm = workloads.Heightmap(32, 32, 0.02, 0.2, 1, None)
    pos64, disp64, nrm64, _ = oracle.displace_f64(p, waves, tex, hm)
    ref_waves = [oracle.wave_to_reference(x) for x in waves]
    corners = [tuple(map(float, p[0][k])) for k in ("bl", "br", "tl", "tr")]
    U, keep = oracle.reference_uniforms(corners, 65, ref_waves, float(p[0]["time_s"]), texels=tex,
                                        sample_scale=0.02, disp_scale=0.2, wrap=1, bounce=0.0)
    o = oracle.reference_vertex(U, 0, 65 * 65)
    assert rel_err(o["position"][:, :3].astype(np.float64), pos64) < 1e-5
    grid = pos64 - disp64
    assert rel_err(o["position"][:, :3] - grid, disp64) < 2e-4


def test_known_answers_f64(oracle):
    p = _one_patch()
    # A = 0: the flat grid, normal +y
    p["wave_count"] = 1
    pos, disp, nrm, _ = oracle.displace_f64(p, _waves([(0.0, 7.0, 1.0, 0.0, 0.3, 1.0, 0.2)]))
    assert np.abs(disp).max() == 0.0
    assert np.allclose(nrm, [0, 1, 0], atol=0)
    # Q = 0: y = A sin(theta), xz untouched
    A, lam, ang, sp, ph = 0.4, 9.0, 0.7, 2.5, 0.3
    D = (math.cos(ang), math.sin(ang))
    wq = _waves([(A, lam, D[0], D[1], 0.0, sp, ph)])
    pos, disp, nrm, _ = oracle.displace_f64(p, wq)
    grid = pos - disp
    A, lam, D, sp, ph = (float(wq[0]["amplitude"]), float(wq[0]["wavelength"]),
                         (float(wq[0]["dir_x"]), float(wq[0]["dir_z"])), float(wq[0]["speed"]), float(wq[0]["phase"]))
    k = 2 * math.pi / lam
    th = k * (D[0] * grid[:, 0] + D[1] * grid[:, 2]) + sp * k * 5.0 + ph
    assert np.abs(disp[:, 1] - A * np.sin(th)).max() < 1e-12
    assert np.abs(disp[:, [0, 2]]).max() == 0.0
    # time periodicity: t + 2 pi / omega
    wv = _waves([(A, lam, D[0], D[1], 0.5 / (k * A), sp, ph)])
    p2 = p.copy()
    p2["time_s"] = 5.0 + 2 * math.pi / (sp * k)
    _, d1, _, _ = oracle.displace_f64(p, wv)
    _, d2, _, _ = oracle.displace_f64(p2, wv)
    assert np.abs(d1 - d2).max() < 1e-9


def test_analytic_normal_matches_central_differences(oracle):
    """The exact normal equals the central-difference normal of the FP64
    surface in the limit (the reference's :164-187 with du -> 0)."""
    from wave_tool_gb300.abi import PATCH_DTYPE
    rng = np.random.default_rng(5)
    rows = []
    for _ in range(5):
        ang = rng.uniform(0, 2 * math.pi)
        lam = rng.uniform(3, 30)
        A = lam / 90
        rows.append((A, lam, math.cos(ang), math.sin(ang), 0.5 / (2 * math.pi / lam * A * 5), rng.uniform(0, 3),
                     rng.uniform(0, 6)))
    wv = _waves(rows)
    # a 3x3 grid with tiny spacing around random centres: vertex 4 is the centre
    for _ in range(20):
        c = rng.uniform(-50, 50, 2)
        h = 1e-4
        p = np.array([((c[0] - h, c[1] + h), (c[0] + h, c[1] + h), (c[0] - h, c[1] - h), (c[0] + h, c[1] - h),
                       3, 3, 0, 5, 2.0, 0.0, 0, 0)], dtype=PATCH_DTYPE)
        pos, _, nrm, _ = oracle.displace_f64(p, wv)
        pu = pos[5] - pos[3]   # +u (x)
        pv = pos[7] - pos[1]   # +v (-z)
        n_fd = np.cross(pu, pv)
        n_fd /= np.linalg.norm(n_fd)
        assert np.degrees(np.arccos(min(1.0, float(n_fd @ nrm[4])))) < 1e-4


def test_index_buffer_oracle_is_the_reference_loop(oracle):
    """src/program.cpp:686-717, restated as nested loops over a gridIndices
    table, equals the oracle for the reference's L = 513 and small sizes."""
    for L in (2, 3, 17, 513):
        grid = [[r * L + c for c in range(L)] for r in range(L)]
        faces = []
        for r in range(L - 1):
            for c in range(L - 1):
                faces += [grid[r][c], grid[r + 1][c + 1], grid[r + 1][c], grid[r][c], grid[r][c + 1], grid[r + 1][c + 1]]
        assert np.array_equal(oracle.grid_indices(L, L), np.array(faces, np.uint32))
    assert list(oracle.grid_indices(3, 2, 10)) == [10, 14, 13, 10, 11, 14, 11, 15, 14, 11, 12, 15]


def test_noise_oracle_tiles_and_normalises(oracle):
    from wave_tool_gb300 import workloads
    terms = workloads.noise_terms(workloads.SplitMix64(9), n=16, kmax=8)
    h = oracle.noise_f64(terms, 40, 24)
    assert h.min() == 0.0 and h.max() == 1.0
    # tileable: the formula at i = W equals i = 0 (checked directly)
    def raw(i, j):
        return sum(float(t["amplitude"]) * math.sin(2 * math.pi * (int(t["kx"]) * i / 40 + int(t["ky"]) * j / 24)
                                                     + float(t["phase"])) for t in terms)
    for j in (0, 5, 23):
        assert abs(raw(40, j) - raw(0, j)) < 1e-9 and abs(raw(7, j + 24) - raw(7, j)) < 1e-9


def test_adjoint_oracle_matches_finite_differences(oracle):
    """The hand-derived FP64 adjoint equals central differences of the FP64
    forward for every parameter (heightmap included, samples kept off texel
    edges)."""
    from wave_tool_gb300.abi import PATCH_DTYPE
    from wave_tool_gb300 import workloads
    rng = np.random.default_rng(11)
    rows = []
    for _ in range(3):
        ang = rng.uniform(0, 2 * math.pi)
        lam = rng.uniform(4, 20)
        A = lam / 60
        rows.append((A, lam, math.cos(ang), math.sin(ang), 0.4 / (2 * math.pi / lam * A * 3), rng.uniform(0.5, 3),
                     rng.uniform(0, 6)))
    wv = _waves(rows)
    p = np.array([((-9.0, 9.0), (9.5, 8.0), (-8.0, -9.0), (9.0, -9.5), 9, 8, 0, 3, 3.5, 0.1, 0, 0)],
                 dtype=PATCH_DTYPE)
    tex = rng.random((8, 8)).astype(np.float32)
    hm = workloads.Heightmap(8, 8, 0.05, 0.3, 0, None)
    nv = 9 * 8
    gpos = rng.standard_normal((nv, 4)).astype(np.float32)
    gnrm = rng.standard_normal((nv, 4)).astype(np.float32)
    grad = oracle.adjoint_f64(p, wv, gpos, gnrm, tex, hm)

    def loss(waves):
        pos, _, nrm, edge = oracle.displace_f64(p, waves, tex, hm)
        return float(np.sum(gpos[:, :3] * pos) + np.sum(gnrm[:, :3] * nrm)), edge

    _, edge = loss(wv)
    assert edge.min() > 1e-3  # no sample sits on a texel edge at this seed
    fields = ["amplitude", "wavelength", None, "steepness_q", "phase", "speed", "dir_x", "dir_z"]
    for i in range(3):
        for f, name in enumerate(fields):
            h = 1e-4
            wp, wm = wv.copy(), wv.copy()
            if name is None:  # direction angle, step taken from the stored FP32 components
                a = math.atan2(float(wv[i]["dir_z"]), float(wv[i]["dir_x"]))
                for ww, s in ((wp, 1), (wm, -1)):
                    ww[i]["dir_x"], ww[i]["dir_z"] = math.cos(a + s * h), math.sin(a + s * h)
                ap = math.atan2(float(wp[i]["dir_z"]), float(wp[i]["dir_x"]))
                am = math.atan2(float(wm[i]["dir_z"]), float(wm[i]["dir_x"]))
                fd_h = (ap - am) / 2
            else:
                # float32 parameters: perturb in FP32 and use the realised step
                x = float(wv[i][name])
                hp = np.float32(x + h * max(1.0, abs(x)))
                hm_ = np.float32(x - h * max(1.0, abs(x)))
                wp[i][name], wm[i][name] = hp, hm_
                fd_h = (float(hp) - float(hm_)) / 2
            fd = (loss(wp)[0] - loss(wm)[0]) / (2 * fd_h)
            an = grad[i, f]
            assert abs(fd - an) <= 2e-3 * max(1.0, abs(an)), (i, name, fd, an)


def test_noise_animation_restatement(oracle):
    """The FP64 noise at time t with rates r equals the static noise with the
    phases advanced by r t; whole turns per second repeat every second."""
    import numpy as np
    from wave_tool_gb300 import workloads
    terms = workloads.noise_terms(workloads.SplitMix64(3), n=12, kmax=6)
    rates = np.linspace(-2.0, 2.0, 12).astype(np.float32)
    moved = terms.copy()
    moved["phase"] = (terms["phase"].astype(np.float64) + rates.astype(np.float64) * 0.75).astype(np.float32)
    a = oracle.noise_f64(terms, 20, 12, rates=rates, time_s=0.75)
    b = oracle.noise_f64(moved, 20, 12)
    assert np.abs(a - b).max() < 1e-6
    whole = (2.0 * np.pi * np.arange(1, 13)).astype(np.float32)
    c = oracle.noise_f64(terms, 20, 12, rates=whole, time_s=1.0)
    d = oracle.noise_f64(terms, 20, 12)
    assert np.abs(c - d).max() < 1e-5


def test_timed_cpu_baseline_matches_the_reference_mode_oracle(oracle):
    """The timed CPU baseline (reference_mode.c built for speed: -O3, fused
    multiply-adds) computes what the bit-exact restatement computes: world
    positions to 1e-5 of the coordinates' scale, FD normals to 0.5 degree
    (central differences over 0.2 m amplify the FP32 rounding of kilometre
    coordinates), on every third row of eight batched patches."""
    import numpy as np
    import types
    from helpers import angle_deg
    from wave_tool_gb300 import workloads
    w = workloads.config3(n_patches=8, seed=2)
    tex = oracle.noise_f64(w.heightmap.terms, w.heightmap.width, w.heightmap.height).astype(np.float32)
    hmp = types.SimpleNamespace(sample_scale=w.heightmap.sample_scale, disp_scale=w.heightmap.disp_scale,
                                wrap=w.heightmap.wrap)
    nv, terms = oracle.cpu_baseline_rows(w.patches, w.waves, tex, hmp, row_stride=3, row_phase=1, threads=2)
    n_out = w.n_vertices
    out = (np.zeros((n_out, 4), np.float32), np.zeros((n_out, 4), np.float32))
    oracle.cpu_baseline_rows(w.patches, w.waves, tex, hmp, row_stride=3, row_phase=1, threads=2, out=out)
    _, pos_ref, nrm_ref = oracle.cpu_baseline(w.patches, w.waves, tex, hmp, threads=2)
    rows = np.concatenate([int(p["out_offset"]) + (np.arange(1, int(p["rows"]), 3)[:, None] * int(p["cols"])
                                                   + np.arange(int(p["cols"]))[None, :]).ravel()
                           for p in w.patches])
    assert nv == len(rows)
    assert terms == sum(len(range(1, int(p["rows"]), 3)) * int(p["cols"]) * int(p["wave_count"]) for p in w.patches)
    scale = float(np.abs(pos_ref[rows, :3]).max())
    assert np.abs(out[0][rows, :3] - pos_ref[rows, :3]).max() <= 1e-5 * scale
    assert angle_deg(out[1][rows, :3].astype(np.float64), nrm_ref[rows, :3].astype(np.float64)).max() < 0.5
