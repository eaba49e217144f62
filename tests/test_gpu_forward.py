"""GPU parity of the forward path (through the C ABI) against the FP64 oracle.

Tolerances: displacement max|d32 - d64| / max|d64| <= 1e-5 (the path's
stated bound); normals within 0.01 degree except where the heightmap sample
sits within 1e-3 texel of a cell edge (the bilinear gradient jumps there, and
a 1e-5 m position difference may pick the other cell)."""
from __future__ import annotations

import math

import numpy as np
import pytest

from helpers import angle_deg, golden_cases, golden_to_abi, rel_err

pytestmark = pytest.mark.gpu

DISP_TOL = 1e-5
ANGLE_TOL_DEG = 1e-2


def run(wt, w, flags=0, texels=None, unbatched=False, normals=True):
    hm = wt.heightmap_from(w.heightmap, texels)
    surf = wt.Surface(w.patches, w.waves, hm)
    pos, nrm = surf.displace(flags=flags, normals=normals, unbatched=unbatched)
    import torch
    torch.cuda.synchronize()
    st, bad = surf.status()
    assert st == 0, (st, bad)
    tex = None if hm is None else hm.texels.cpu().numpy()
    return pos.cpu().numpy(), (None if nrm is None else nrm.cpu().numpy()), tex


def check_against_f64(oracle, w, pos, nrm, tex, flags=0, disp_tol=DISP_TOL):
    pos64, disp64, nrm64, edge = oracle.displace_f64(w.patches, w.waves, tex, w.heightmap)
    if flags & 1:
        err = rel_err(pos[:, :3].astype(np.float64), disp64)
        assert err <= disp_tol, f"displacement rel err {err:.3e}"
    else:
        # world positions carry the FP32 rounding of the world coordinate on
        # top of the displacement error
        err = rel_err(pos[:, :3].astype(np.float64) - (pos64 - disp64), disp64)
        ulp = np.spacing(np.abs(pos64).astype(np.float32)).astype(np.float64)
        assert np.all(np.abs(pos[:, :3] - pos64) <= 4 * ulp + disp_tol * np.abs(disp64).max())
    if nrm is not None:
        ok = edge > 1e-3
        ang = angle_deg(nrm[ok, :3].astype(np.float64), nrm64[ok])
        assert ang.max() < ANGLE_TOL_DEG, f"normal angle {ang.max():.3e} deg"
        assert np.abs(np.linalg.norm(nrm[:, :3], axis=1) - 1).max() < 1e-5
        assert np.all(nrm[:, 3] == 0)
    return err


def test_config1_displacement_and_normals(wt, oracle, gpu):
    from wave_tool_gb300 import workloads
    w = workloads.config1()
    for flags in (wt.WT_OUT_DISPLACEMENT, wt.WT_OUT_WORLD):
        pos, nrm, tex = run(wt, w, flags)
        check_against_f64(oracle, w, pos, nrm, tex, flags)
        assert np.all(pos[:, 3] == (0.0 if flags else 1.0))


@pytest.mark.parametrize("seed", range(8))
def test_ragged_random_patches(wt, oracle, gpu, seed):
    """Uneven, non-square, skewed (non-parallelogram) patches at world offsets
    up to 3 km and times up to 5000 s; 0..40 waves; REPEAT and MIRRORED_REPEAT
    heightmaps of odd sizes; sides from 2 (the minimum) upward."""
    from wave_tool_gb300 import workloads
    w = workloads.small_random(seed, n_patches=4, side_range=(2, 300), wrap=seed % 2)
    pos, nrm, tex = run(wt, w, wt.WT_OUT_DISPLACEMENT)
    check_against_f64(oracle, w, pos, nrm, tex, 1)


def test_no_heightmap_and_no_waves(wt, oracle, gpu):
    from wave_tool_gb300 import workloads
    w = workloads.small_random(3, n_patches=3, heightmap=False, n_waves_range=(0, 0))
    pos, nrm, tex = run(wt, w, wt.WT_OUT_DISPLACEMENT)
    y = w.patches["y_offset"]
    for p in w.patches:
        o, n = int(p["out_offset"]), int(p["cols"]) * int(p["rows"])
        assert np.all(pos[o:o + n, [0, 2]] == 0) and np.allclose(pos[o:o + n, 1], p["y_offset"])
        assert np.all(nrm[o:o + n, :3] == np.array([0, 1, 0], np.float32))
    del y


def test_vec3_layout_matches_float4(wt, gpu):
    from wave_tool_gb300 import workloads
    w = workloads.small_random(5, n_patches=3)
    p4, n4, _ = run(wt, w, 0)
    p3, n3, _ = run(wt, w, wt.WT_LAYOUT_VEC3)
    assert np.array_equal(p4[:, :3], p3) and np.array_equal(n4[:, :3], n3)


def test_batched_equals_unbatched_and_is_deterministic(wt, gpu):
    from wave_tool_gb300 import workloads
    w = workloads.config3(n_patches=12, seed=21)
    a, na, _ = run(wt, w, 0)
    b, nb, _ = run(wt, w, 0, unbatched=True)
    c, nc, _ = run(wt, w, 0)
    assert np.array_equal(a, b) and np.array_equal(na, nb)
    assert np.array_equal(a, c) and np.array_equal(na, nc)


def test_small_table_prep_matches_the_general_prep(wt, oracle, gpu):
    """Tables of at most 32 patches with at most 1024 (patch, wave) pairs take
    a shared-memory prep; 33 patches take the general one (two prep kernels).
    The same 32 patches give the same bits either way, and the FP64 oracle
    agrees; a structurally invalid and a bad-wave patch are reported alike."""
    from wave_tool_gb300 import workloads
    w = workloads.small_random(23, n_patches=33, side_range=(2, 60), n_waves_range=(0, 32))
    pt = w.patches.copy()
    waves = w.waves[:32].copy()
    rng = np.random.default_rng(23)
    for i in range(len(pt)):
        off = int(rng.integers(0, 32))
        pt[i]["wave_offset"] = off
        pt[i]["wave_count"] = int(rng.integers(0, 33 - off))
    small = workloads.Workload("small32", pt[:32].copy(), waves, w.heightmap)
    a, na, tex = run(wt, small)
    b, nb, _ = run(wt, workloads.Workload("general33", pt, waves, w.heightmap))
    n32 = int(pt[31]["out_offset"] + pt[31]["cols"] * pt[31]["rows"])
    assert np.array_equal(a, b[:n32]) and np.array_equal(na, nb[:n32])
    check_against_f64(oracle, small, a, na, tex)
    bad = pt[:32].copy()
    bad[5]["cols"] = 1
    bad_waves = waves.copy()
    k = next(i for i in range(32) if i != 5 and bad[i]["wave_count"] > 0)
    bad_waves[int(bad[k]["wave_offset"])]["wavelength"] = np.nan
    for table in (bad, np.concatenate([bad, pt[32:]])):
        surf = wt.Surface(table, bad_waves, wt.heightmap_from(w.heightmap))
        surf.displace()
        assert surf.status() == (wt.abi.WT_ERR_INVALID_ARG, min(5, k))


def test_config3_subset_against_f64(wt, oracle, gpu):
    """Sixteen config-3 patches (uneven sides 64..1024, 8..64 waves, noise
    layer), all checked against FP64."""
    from wave_tool_gb300 import workloads
    w = workloads.config3(n_patches=16, seed=2)
    pos, nrm, tex = run(wt, w, wt.WT_OUT_DISPLACEMENT)
    check_against_f64(oracle, w, pos, nrm, tex, 1)


def test_config2_sampled_rows_against_f64(wt, oracle, gpu):
    """The single 1024 x 1024 / 32-wave / 512^2-noise patch: every vertex
    through the GPU, rows 0..63 and the last row against FP64."""
    from wave_tool_gb300 import workloads
    w = workloads.config2()
    pos, nrm, tex = run(wt, w, wt.WT_OUT_DISPLACEMENT)
    cols = int(w.patches[0]["cols"])
    _, disp64, nrm64, edge = oracle.displace_f64(w.patches, w.waves, tex, w.heightmap, rows=64)
    n = 64 * cols
    assert rel_err(pos[:n, :3].astype(np.float64), disp64[:n]) <= DISP_TOL
    ok = edge[:n] > 1e-3
    assert angle_deg(nrm[:n][ok, :3].astype(np.float64), nrm64[:n][ok]).max() < ANGLE_TOL_DEG
    assert np.isfinite(pos).all() and np.isfinite(nrm).all()


@pytest.mark.parametrize("t", [1.0e2, 1.0e4, 1.0e6])
def test_large_time_fp64_phase_vs_fp32_naive(wt, oracle, gpu, t):
    """The per-wave phase reduced in FP64 keeps the 1e-5 bound at t = 1e6 s;
    the reference's FP32 phase (w*dot(D,xz) + phi*t, water-grid.vert:78) does
    not."""
    from wave_tool_gb300 import workloads
    w = workloads.config5(time_s=t, side=128, n=16)
    pos, nrm, tex = run(wt, w, wt.WT_OUT_DISPLACEMENT)
    err = check_against_f64(oracle, w, pos, nrm, tex, 1)
    naive, _, _ = run(wt, w, wt.WT_OUT_DISPLACEMENT | wt.WT_PHASE_FP32_NAIVE)
    _, disp64, _, _ = oracle.displace_f64(w.patches, w.waves)
    err_naive = rel_err(naive[:, :3].astype(np.float64), disp64)
    if t >= 1e4:
        assert err_naive > 100 * err
    assert err <= DISP_TOL


def test_golden_reference_cases(wt, oracle, gpu):
    """The reference shader's own outputs (tests/golden, made from
    water-grid.vert compiled as C++): the displaced world positions agree with
    the GPU within the reference's FP32 phase error, and the GPU agrees with
    FP64 within 1e-5."""
    import torch
    from wave_tool_gb300 import workloads
    for c in golden_cases():
        patches, waves, hm = golden_to_abi(c)
        tex = torch.from_numpy(np.ascontiguousarray(c["tex"])).cuda()
        w = workloads.Workload(c["name"], patches, waves, hm)
        pos, nrm, _ = run(wt, w, 0, texels=tex)
        texn = np.ascontiguousarray(c["tex"])
        pos64, disp64, _, _ = oracle.displace_f64(patches, waves, texn, hm)
        ref = c["world"][:, :3].astype(np.float64)
        dmax = max(np.abs(disp64).max(), 1e-3)
        # the reference's own FP32 error: phase magnitude * 2^-22 * sum(A (1 + Q k A))
        th = float(np.max(np.abs(c["waves"][:, 1]), initial=0)) * float(np.abs(c["corners"]).max()) * 1.5 + \
            float(np.max(np.abs(c["waves"][:, 2]), initial=0)) * float(c["scalars"][0])
        ref_tol = (th + 10.0) * 2.0 ** -20 * (np.abs(waves["amplitude"]).sum() + 1.0) + \
            4 * np.spacing(np.float32(np.abs(ref).max())) + 2e-3 * float(c["scalars"][2])
        assert np.abs(pos[:, :3] - ref).max() <= ref_tol + 1e-5 * dmax, c["name"]
        assert np.abs(pos[:, :3] - pos64).max() <= 1e-5 * dmax + 4 * np.spacing(np.float32(np.abs(pos64).max()))


def test_reference_default_waves_through_conversion(wt, oracle, gpu):
    """The reference's four default waves (render-engine.cpp:46-49) through
    wt_wave_from_reference (render-engine.cpp:1073) reproduce the shader's
    positions on a 513-vertex grid (GRID_LENGTH, render-engine.cpp:1055)."""
    from wave_tool_gb300.abi import PATCH_DTYPE
    from wave_tool_gb300 import workloads
    defaults = [(0.06, 1.0, 2.0, 1.0, 1.0, 0.0), (0.1, 1.0, 0.2, 0.0, math.sqrt(0.5), math.sqrt(0.5))]
    waves = np.concatenate([wt.wave_from_reference(*d, 4) for d in defaults])
    L = 513
    patches = np.array([((-50, 50), (50, 50), (-50, -50), (50, -50), L, L, 0, 2, float(np.float32(7.5)), 0.0, 0, 0)],
                       dtype=PATCH_DTYPE)
    w = workloads.Workload("ref_defaults", patches, waves)
    pos, nrm, _ = run(wt, w, 0)
    U, keep = oracle.reference_uniforms(((-50, 50), (50, 50), (-50, -50), (50, -50)), L,
                                        [(0.06, 1.0, 2.0, float(waves[0]["steepness_q"]), 1.0, 0.0),
                                         (0.1, 1.0, 0.2, 0.0, math.sqrt(0.5), math.sqrt(0.5))], 7.5,
                                        texels=None, disp_scale=0.0)
    ref = oracle.reference_vertex(U, 0, L * L)["position"][:, :3]
    assert np.abs(pos[:, :3] - ref).max() < 2e-5


@pytest.mark.parametrize("t", [1.0e2, 1.0e4, 1.0e6])
def test_precision_stress_2048sq_128waves(wt, oracle, gpu, t):
    """The precision configuration at full size (2048^2 vertices, 128 waves,
    t = 1e2 / 1e4 / 1e6 s): every vertex through the GPU in both phase modes,
    32 rows spread over the patch against FP64.  FP64-reduced phase stays
    within 1e-5; the FP32-naive phase of the reference (water-grid.vert:78)
    degrades with t.  Prints max / RMS displacement error and max normal angle."""
    import torch
    from wave_tool_gb300 import workloads
    w = workloads.config5(time_s=t)
    surf = wt.Surface(w.patches, w.waves)
    rows = np.linspace(0, 2047, 32).astype(int)
    cols = 2048
    res = {}
    for mode, flags in (("fp64_phase", wt.WT_OUT_DISPLACEMENT),
                        ("fp32_naive", wt.WT_OUT_DISPLACEMENT | wt.WT_PHASE_FP32_NAIVE)):
        pos, nrm = surf.displace(flags=flags)
        torch.cuda.synchronize()
        idx = (rows[:, None] * cols + np.arange(cols)[None, :]).ravel()
        res[mode] = (pos[torch.from_numpy(idx).cuda()].cpu().numpy(), nrm[torch.from_numpy(idx).cuda()].cpu().numpy())
        del pos, nrm
    disp64, nrm64 = oracle.displace_f64_rows(w.patches[0], w.waves, rows)
    out = {}
    for mode, (p, n) in res.items():
        e = np.abs(p[:, :3].astype(np.float64) - disp64)
        out[mode] = (e.max() / np.abs(disp64).max(), np.sqrt((e ** 2).mean()) / np.abs(disp64).max(),
                     angle_deg(n[:, :3].astype(np.float64), nrm64).max())
    print(f"t={t:g}: " + "; ".join(f"{m} max {a:.2e} rms {b:.2e} normal {c:.2e} deg" for m, (a, b, c) in out.items()))
    assert out["fp64_phase"][0] <= DISP_TOL
    if t >= 1e4:
        assert out["fp32_naive"][0] > 10 * out["fp64_phase"][0]


@pytest.fixture
def restore_tuning(wt):
    yield
    wt.check(wt.lib().wt_set_tuning(None))


@pytest.mark.parametrize("shape", ["autotuned", (8, 16, 0), (4, 8, 0)])
def test_benchmarked_table_every_patch_against_f64(wt, oracle, gpu, restore_tuning, shape):
    """The exact table the benchmark times (256 uneven patches, seed 2, the
    512^2 noise layer) through the GPU, and sampled rows of EVERY patch (the
    first, the last and six between) against FP64: the metric's <= 1e-5
    bound measured on the timed inputs, with the shape the autotuner picks
    and with 8 and 4 vertices per lane (the recurrence's length)."""
    import torch
    from wave_tool_gb300 import workloads
    w = workloads.config3(n_patches=256, seed=2)
    hm = wt.heightmap_from(w.heightmap)
    surf = wt.Surface(w.patches, w.waves, hm)
    pos, nrm = surf.alloc_outputs(wt.WT_OUT_DISPLACEMENT)
    if shape == "autotuned":
        surf.autotune(pos, nrm, flags=wt.WT_OUT_DISPLACEMENT, reps=2)
    else:
        vpl, warps, epi = shape
        wt.set_tuning(warps, 0, 32, vpl, epi)
    surf.displace(pos, nrm, flags=wt.WT_OUT_DISPLACEMENT)
    torch.cuda.synchronize()
    assert surf.status()[0] == 0
    acc = oracle.accuracy_sampled_rows(w.patches, w.waves, pos.cpu().numpy(), nrm.cpu().numpy(),
                                       hm.texels.cpu().numpy(), w.heightmap)
    assert acc["patches_checked"] == 256 and acc["rows_checked"] == 256 * 8
    assert acc["max_rel_err"] <= DISP_TOL, acc
    assert acc["per_patch_max_rel_err"] <= DISP_TOL, acc
    assert acc["max_normal_deg"] < ANGLE_TOL_DEG, acc
