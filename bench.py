"""Benchmark of the Gerstner water-surface path on GB300.

Metric: Gerstner terms/s = sum over patches of (vertices x waves) per second,
at <= 1e-5 relative displacement error vs FP64 (enforced by tests/, and
measured here on the timed table after the timed region: sampled rows of every
patch against the FP64 oracle, the `accuracy` field).  Workload: the batched
configuration — 256
independent patches, grid side log-uniform in [64, 1024], 8..64 waves each,
t U[0, 1e3] s, with the 512^2 noise heightmap layer — as one persistent
launch.  A step = the three launches of one wt_gerstner_displace call
(validate/sort, FP64 phase constants, persistent forward).

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]

Prints one JSON line (rank 0).  Under torchrun each rank runs its own
256-patch workload (seed 2 + rank; weak scaling, no collective on the data
path) and the step time is the max over ranks; with --split the ranks share
ONE 256-patch table, each running its LPT shard of the patches (strong
scaling), and the value is the table's terms over the max step time.
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import time
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))

import __graft_entry__  # noqa: E402

METRIC = "Gerstner terms/s (verts x waves) at <=1e-5 rel err vs FP64; batched persistent launch"
UNIT = "terms/s"
PROFILE_TRAFFIC = ROOT / "profiles" / "forward_traffic.json"
E2E_GROUPS = 16  # streams the end-to-end step is split over (0.945 / 0.957 / 0.964 of the D2H link with 4 / 8 / 16)


def parse_args():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=200)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", choices=["ours", "reference"], default="ours")
    ap.add_argument("--patches", type=int, default=256)
    ap.add_argument("--cpu-seconds", type=float, default=12.0, help="target CPU time of the baseline sample")
    ap.add_argument("--no-extras", action="store_true", help="skip the unbatched / single-patch side runs")
    ap.add_argument("--mode", choices=["forward", "adjoint", "frame", "displace"], default="forward",
                    help="'adjoint' times only wt_gerstner_adjoint on 64 uneven patches, 'frame' only the "
                         "camera-to-pixels water frame, 'displace' only wt_gerstner_displace on --workload "
                         "(for profiling)")
    ap.add_argument("--workload", choices=["config2", "config3", "config5"], default="config3",
                    help="with --mode displace: the 1024^2 patch, the batched table (--patches) or 2048^2 x 128 "
                         "waves")
    ap.add_argument("--no-heightmap", action="store_true",
                    help="the batched workload without its noise layer (for instruction-mix comparisons)")
    ap.add_argument("--saved-sums", action="store_true",
                    help="with --mode adjoint: time wt_gerstner_adjoint_saved on a saving forward's sums")
    ap.add_argument("--tuning", default="auto",
                    help="'auto' (autotune before timing) or WARPS,CHUNK[,VPL,EPI] to fix the launch shape")
    ap.add_argument("--split", action="store_true",
                    help="under torchrun: the ranks share one table, each its LPT shard of the patches")
    ap.add_argument("--e2e-groups", type=int, default=E2E_GROUPS,
                    help="stream groups of the end-to-end step (copy-back of one overlaps the next's kernel)")
    ap.add_argument("--no-accuracy", action="store_true", help="skip the FP64 check of the timed table")
    return ap.parse_args()


def dist_env():
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", str(rank)))
    return rank, world, local


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled during the timed region."""

    FIELDS = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.hw_slowdown,"
              "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
              "clocks_event_reasons.sw_power_cap")

    def __init__(self, index: int):
        self.index = index
        self.proc = None

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.index), f"--query-gpu={self.FIELDS}", "--format=csv,noheader,nounits",
                 "-lms", "100"], stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
        except OSError:
            self.proc = None
        time.sleep(0.3)
        return self

    def __exit__(self, *a):
        self.out = ""
        if self.proc is not None:
            self.proc.terminate()
            try:
                self.out, _ = self.proc.communicate(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()
                self.out, _ = self.proc.communicate()

    def summary(self):
        rows = []
        for line in (self.out or "").strip().splitlines():
            parts = [p.strip() for p in line.split(",")]
            if len(parts) != 7:
                continue
            try:
                rows.append((float(parts[0]), float(parts[1]), float(parts[2]), parts[3:]))
            except ValueError:
                continue
        if not rows:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unavailable"], "samples": 0}
        # samples under load: power well above idle
        pmax = max(r[2] for r in rows)
        load = [r for r in rows if r[2] >= 0.5 * pmax] or rows
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[i] for r in load for i, v in enumerate(r[3]) if v.lower().startswith("active")})
        return {"sm_mhz": statistics.median(r[0] for r in load), "sm_max_mhz": max(r[1] for r in rows),
                "reasons": reasons, "samples": len(load), "power_w_max": pmax}


def traffic_from_profile(tuning, vertices):
    """DRAM bytes of one forward launch of the tuned shape: the bytes per
    vertex an ncu capture of that kernel measured (profiles/forward_traffic.json,
    keyed by the kernel's launch shape) times this launch's vertices; None
    when no capture of the shape exists."""
    if not PROFILE_TRAFFIC.exists():
        return None
    try:
        rec = json.loads(PROFILE_TRAFFIC.read_text())
    except ValueError:
        return None
    key = (f"warps={tuning['warps_per_block']},vpl={tuning['max_vertices_per_lane']},"
           f"epi={tuning['epilogue_in_shared']}")
    r = rec.get("shapes", {}).get(key)
    return None if r is None else r["dram_bytes_per_vertex"] * vertices


class CpuWorkload:
    """The timed CPU restatement of the reference shader (the oracle's
    reference_mode.c built for speed, oracle/_build/libcpu_timed.so) over the
    benchmark's table: 5 surface evaluations per vertex, central-difference
    normals (with `analytic`, one evaluation per vertex and Jacobian normals),
    on the rows r = phase + k * stride of EVERY patch, so a sample is spread
    evenly over each patch and `stride` consecutive phases cover the table."""

    def __init__(self, w):
        from oracle import oracle as O
        import types
        self.O, self.w = O, w
        self.tex = self.hmp = None
        if w.heightmap is not None:
            self.tex = O.noise_f64(w.heightmap.terms, w.heightmap.width, w.heightmap.height).astype(np.float32)
            self.hmp = types.SimpleNamespace(sample_scale=w.heightmap.sample_scale,
                                             disp_scale=w.heightmap.disp_scale, wrap=w.heightmap.wrap)
        n = int(w.n_vertices)
        self.out = (np.zeros((n, 4), np.float32), np.zeros((n, 4), np.float32))
        from oracle import build as ob
        self.flags = " ".join(ob.TIMED_CFLAGS)

    def run(self, stride, phase, threads, analytic=False):
        t0 = time.perf_counter()
        _, terms = self.O.cpu_baseline_rows(self.w.patches, self.w.waves, self.tex, self.hmp, stride, phase, threads,
                                            analytic, out=self.out)
        return terms, time.perf_counter() - t0

    def stride_for(self, seconds, threads, analytic=False):
        """Row stride whose sample takes about `seconds` (probed on every
        64th row)."""
        terms, dt = self.run(64, 0, threads, analytic)
        full = dt * self.w.n_terms / max(terms, 1)
        return max(1, int(np.ceil(full / max(seconds, 1e-3))))


def every_nth(n: int) -> str:
    if n == 1:
        return "every row"
    suffix = "th" if 10 <= n % 100 <= 20 else {1: "st", 2: "nd", 3: "rd"}.get(n % 10, "th")
    return f"every {n}{suffix} row"


def cpu_sample(cw, target_s: float, threads: int, analytic: bool = False):
    """One bounded sample of about target_s: every stride-th row of every
    patch (phase stride // 2).  Returns (terms/s, seconds, stride, terms)."""
    stride = cw.stride_for(target_s, threads, analytic)
    terms, dt = cw.run(stride, stride // 2, threads, analytic)
    return terms / dt, dt, stride, terms


def run_reference(args):
    rank, world, _ = dist_env()
    if rank != 0:
        return
    sys.path.insert(0, str(ROOT))
    from oracle import build as ob
    ob.build_oracle()
    wt = __graft_entry__.load_package()
    from wave_tool_gb300 import workloads
    w = workloads.config3(n_patches=args.patches, seed=2)
    threads = os.cpu_count() or 1
    cw = CpuWorkload(w)
    per_step = max(0.5, args.cpu_seconds / max(1, args.steps))
    stride = cw.stride_for(per_step, threads)
    terms_t, secs, dts = 0, 0.0, []
    for i in range(args.warmup + args.steps):
        terms, dt = cw.run(stride, i % stride, threads)   # phases cycle: `stride` steps cover the table
        if i >= args.warmup:
            terms_t += terms
            secs += dt
            dts.append(dt)
    value = terms_t / secs
    covered = min(1.0, args.steps / stride)
    sample = (f"per step {every_nth(stride)} of each of the {args.patches} patches (rows phase + k*{stride}, phase "
              f"cycling 0..{stride - 1}, so {stride} steps cover the whole table; the {args.steps} timed steps "
              f"covered {covered:.0%} of its rows, {terms_t} terms in {secs:.1f} s)")
    line = {
        "impl": "reference", "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": args.gpus,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * statistics.median(dts),
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
        "config": workload_config(args, w, world, args.split and world > 1),
        "implementation": "FP32 restatement of water-grid.vert (5 evaluations/vertex, FD normals, FP32 phase), "
                          f"gcc {cw.flags}, POSIX threads on all host cores",
        "cpu_baseline": {"value": value, "unit": UNIT, "cores": threads, "kind": "port", "sample": sample,
                         "build": f"gcc {cw.flags}"},
        "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    del wt
    print(json.dumps(line), flush=True)


def _event_ms(fn, reps, stream, flush=None):
    """Mean device time of fn() over reps calls (CUDA events on `stream`,
    optional L2 flush before each call, outside the events)."""
    import torch
    evs = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(reps)]
    for a, b in evs:
        if flush is not None:
            flush.zero_()
        a.record(stream)
        fn()
        b.record(stream)
    torch.cuda.synchronize()
    return sum(a.elapsed_time(b) for a, b in evs) / reps


def build_frame(wt, workloads):
    """One rendered frame of the water grid as the reference's render loop
    does it (render-engine.cpp:797-1135, water-grid.vert, water-grid.frag), on
    a 1024^2 grid with the 32 waves and noise heightmap of the 1024^2 workload:
    camera -> projected-grid corners (FP64, one warp) -> displacement +
    normals -> clip / NDC-at-height-0 / view vector / facing normal /
    yaw-only normal -> rasterisation at 1920 x 1080 -> water shading.
    Returns the stage callables and sizes."""
    import torch
    w = workloads.config2()
    amp = wt.displaceable_amplitude(w.waves, w.heightmap.disp_scale)
    cam = wt.camera(position=(0.0, 4.0, 70.0), pitch_deg=-20.0, aspect=16 / 9, displaceable_amplitude=amp)
    patch, view, st = wt.projected_grid(cam, w.patches)
    surf = wt.Surface(patch, w.waves, wt.heightmap_from(w.heightmap))
    cam_dev, view_dev = wt.to_device(cam), wt.to_device(view)
    pos, nrm = surf.alloc_outputs(wt.WT_OUT_WORLD)
    tuning = surf.autotune(pos, nrm, flags=wt.WT_OUT_WORLD, reps=5)  # once, as a renderer would at start-up
    n = pos.shape[0]
    outs = {k: torch.empty((n, 2 if k == "ndc0" else 4), device="cuda")
            for k in ("clip", "ndc0", "view", "facing", "nrm_yaw")}
    # and the fused displacement + vertex stage the frame runs
    stage_tuning = surf.autotune_stage(view_dev, outs, reps=5)

    # the fragment stage at 1920 x 1080: seeded sky box and local reflection /
    # refraction targets, nothing drawn behind the water
    VW, VH = 1920, 1080
    gen = torch.Generator(device="cuda").manual_seed(3)
    sky = torch.randint(0, 256, (6, 256, 256, 4), dtype=torch.uint8, device="cuda", generator=gen)
    lrefl = torch.randint(0, 256, (VH, VW, 4), dtype=torch.uint8, device="cuda", generator=gen)
    lrefr = torch.randint(0, 256, (VH, VW, 4), dtype=torch.uint8, device="cuda", generator=gen)
    idx = wt.grid_indices(int(patch["cols"][0]), int(patch["rows"][0]))
    frags = torch.empty((VH, VW), dtype=torch.int64, device="cuda")
    rws = wt.empty_bytes(wt.water_raster_workspace_bytes(n, idx.numel() // 3))
    colour = torch.empty((VH, VW, 4), dtype=torch.float32, device="cuda")
    shading = wt.water_shading(sun_position=(0.6, 0.8, 0.0))

    def raster():
        wt.water_raster(outs["clip"], idx, VW, VH, fragments=frags, workspace=rws)

    def shade():
        wt.water_shade(frags, outs["clip"], idx, outs, VW, VH, shading, sky, local_reflections=lrefl,
                       local_refractions=lrefr, colour=colour)

    def frame(s=None, fused=True):
        wt.projected_grid_async(cam_dev, surf.patches, view_dev, stream=s)
        if fused:   # the vertex stage in the displacement's epilogue
            surf.displace_stage(view_dev, out=outs, stream=s)
        else:
            surf.displace(pos, nrm, flags=wt.WT_OUT_WORLD, stream=s)
            wt.vertex_stage(view_dev, pos, nrm, out=outs, stream=s)
        wt.water_raster(outs["clip"], idx, VW, VH, fragments=frags, workspace=rws, stream=s)
        wt.water_shade(frags, outs["clip"], idx, outs, VW, VH, shading, sky, local_reflections=lrefl,
                       local_refractions=lrefr, colour=colour, stream=s)

    return dict(frame=frame, raster=raster, shade=shade, n=n, waves=len(w.waves), VW=VW, VH=VH, frags=frags,
                tuning=tuning, stage_tuning=stage_tuning,
                projected_grid=lambda: wt.projected_grid_async(cam_dev, surf.patches, view_dev),
                displace=lambda: surf.displace(pos, nrm, flags=wt.WT_OUT_WORLD),
                vertex_stage=lambda: wt.vertex_stage(view_dev, pos, nrm, out=outs),
                displace_stage=lambda: surf.displace_stage(view_dev, out=outs))


def frame_pipeline(wt, workloads, stream, flush):
    """The frame of build_frame replayed as one CUDA graph (the vertex stage
    fused into the displacement, and as its own kernel), and each stage alone
    (the stand-alone vertex stage against HBM)."""
    import torch
    F = build_frame(wt, workloads)
    frame, raster, shade, n, VW, VH, frags = (F[k] for k in ("frame", "raster", "shade", "n", "VW", "VH", "frags"))
    graph_ms = {}
    for fused in (True, False):
        for _ in range(3):
            frame(fused=fused)
        torch.cuda.synchronize()
        side = torch.cuda.Stream()
        side.wait_stream(stream)
        g = torch.cuda.CUDAGraph()
        with torch.cuda.graph(g, stream=side):
            frame(side, fused=fused)
        for _ in range(3):
            g.replay()
        torch.cuda.synchronize()
        graph_ms[fused] = _event_ms(g.replay, 20, stream, flush)
        del g
    fms = graph_ms[True]
    frame()  # leave the fused frame's pixels in frags
    gms = _event_ms(F["projected_grid"], 20, stream, flush)
    dms = _event_ms(F["displace"], 20, stream, flush)
    vms = _event_ms(F["vertex_stage"], 20, stream, flush)
    fsms = _event_ms(F["displace_stage"], 20, stream, flush)
    rms = _event_ms(raster, 20, stream, flush)
    sms = _event_ms(shade, 20, stream, flush)
    # the noise layer animated per frame (64 terms over 512^2 texels): what a
    # frame adds when it resynthesises the heightmap at the frame time
    hw = workloads.config2().heightmap
    nterms = wt.to_device(hw.terms)
    nrates = torch.linspace(-2.0, 2.0, len(hw.terms), device="cuda")
    ntex = torch.empty((hw.height, hw.width), dtype=torch.float32, device="cuda")
    nws = wt.empty_bytes(wt.noise_workspace_bytes(len(hw.terms), hw.width, hw.height))
    nclock = [0.0]

    def noise_frame():
        nclock[0] += 1.0 / 60.0
        wt.noise_synth(nterms, hw.width, hw.height, rates=nrates, time_s=nclock[0], out=ntex, workspace=nws)
    for _ in range(3):
        noise_frame()
    nms = _event_ms(noise_frame, 20, stream, flush)
    covered = float(((frags & 0xffffffff) != 0).float().mean())
    stage_bytes = n * (2 * 16 + 16 + 8 + 3 * 16)  # reads pos + nrm, writes clip, ndc0, view, facing, nrm_yaw
    try:
        hbm_peak = float(json.loads((ROOT / "MEASURED_PEAKS.json").read_text())["hbm_gbs"])
        peak_src = "MEASURED_PEAKS.json hbm_gbs (copy, measured)"
    except (OSError, KeyError, ValueError):
        hbm_peak, peak_src = 6800.0, "fallback 6.8 TB/s"
    return {"vertices": n, "terms": n * F["waves"], "viewport": [VW, VH], "water_pixels_frac": covered,
            "displace_tuning": F["tuning"], "stage_tuning": F["stage_tuning"],
            "frame_graph_ms": fms, "frame_graph_unfused_ms": graph_ms[False], "raster_ms": rms, "shade_ms": sms,
            "noise_512sq_64terms_animated_ms": nms,
            "displace_with_fused_stage_ms": fsms,
            "frames_per_s": 1e3 / fms, "projected_grid_kernel_ms": gms, "displace_ms": dms,
            "vertex_stage_ms": vms, "vertex_stage_bytes": stage_bytes,
            "vertex_stage_gbs": stage_bytes / (vms * 1e-3) / 1e9,
            "vertex_stage_hbm_frac": stage_bytes / (vms * 1e-3) / 1e9 / hbm_peak, "hbm_peak_source": peak_src}


# FP32 FMA-pipe operations of algorithmic work per (vertex, wave) term in the
# adjoint: the forward's 10 (recurrence 2 + eight sums), then per wave and
# vertex the recurrence (2), the eight moments (8), the two projections of the
# phase adjoint (8), its combination (2) and its two sums (2); the saved-sums
# adjoint skips the forward's 10.
ADJ_FMA_PER_TERM = 32
ADJ_SAVED_FMA_PER_TERM = 22


def side_measurements(wt, workloads, surf, pos, nrm, flags, flush, stream, ms_step, fma_s=None):
    """Graph replay of the batched step, adjoint vs forward, the precision
    configuration's throughput and the Adam fit (each reported, not the
    headline)."""
    import torch
    from wave_tool_gb300 import fit
    out = {}
    # one CUDA graph holding the three launches of the batched call
    s = torch.cuda.Stream()
    s.wait_stream(stream)
    g = torch.cuda.CUDAGraph()
    with torch.cuda.graph(g, stream=s):
        surf.displace(pos, nrm, flags=flags, stream=s)
    for _ in range(3):
        g.replay()
    torch.cuda.synchronize()
    gms = _event_ms(g.replay, 20, torch.cuda.current_stream(), flush)
    out["graph_replay"] = {"ms_per_step": gms, "value": surf.n_terms_cache / (gms * 1e-3)}
    # adjoint vs forward on the adjoint-fit grid and on 64 uneven patches
    for name, w in (("adjoint_512sq_16waves", workloads.config4()[0]),
                    ("adjoint_batched_64_uneven_patches", workloads.config5_batched_adjoint())):
        sa = wt.Surface(w.patches, w.waves, wt.heightmap_from(w.heightmap))
        pa, na = sa.alloc_outputs(flags)
        sa.autotune(pa, na, flags=flags, reps=5)
        gen = torch.Generator(device="cuda").manual_seed(1)
        gp = torch.randn(pa.shape, device="cuda", generator=gen)
        gn = torch.randn(na.shape, device="cuda", generator=gen)
        for _ in range(3):
            sa.displace(pa, na, flags=flags)
            sa.adjoint(gp, gn)
        fms = _event_ms(lambda: sa.displace(pa, na, flags=flags), 10, stream, flush)
        ams = _event_ms(lambda: sa.adjoint(gp, gn), 10, stream, flush)
        # the saving forward (also writes 32 B of wave sums per vertex) and the
        # adjoint that reads them instead of recomputing the wave sum
        sums = torch.empty((sa.n_vertices, 8), dtype=torch.float32, device="cuda")
        for _ in range(3):
            sa.displace(pa, na, flags=flags, sums=sums)
            sa.adjoint(gp, gn, sums=sums)
        sfms = _event_ms(lambda: sa.displace(pa, na, flags=flags, sums=sums), 10, stream, flush)
        sams = _event_ms(lambda: sa.adjoint(gp, gn, sums=sums), 10, stream, flush)
        out[name] = {"terms": w.n_terms, "forward_ms": fms, "adjoint_ms": ams, "adjoint_over_forward": ams / fms,
                     "saving_forward_ms": sfms, "saved_adjoint_ms": sams,
                     "saved_adjoint_over_forward": sams / fms}
        if fma_s:
            # the adjoint against its own FMA roofline (whole call, prep and reductions included)
            out[name]["adjoint_fma_frac"] = w.n_terms * ADJ_FMA_PER_TERM / (ams * 1e-3) / fma_s
            out[name]["saved_adjoint_fma_frac"] = w.n_terms * ADJ_SAVED_FMA_PER_TERM / (sams * 1e-3) / fma_s
        del sums
    # precision configuration: 2048^2 vertices x 128 waves at three times
    prec = {}
    for t in (1.0e2, 1.0e4, 1.0e6):
        w5 = workloads.config5(time_s=t)
        s5 = wt.Surface(w5.patches, w5.waves)
        p5, n5 = s5.alloc_outputs(flags)
        if t == 1.0e2:
            prec["tuning"] = s5.autotune(p5, n5, flags=flags, reps=5)
        for _ in range(3):
            s5.displace(p5, n5, flags=flags)
        ms5 = _event_ms(lambda: s5.displace(p5, n5, flags=flags), 10, stream, flush)
        prec[f"t={t:g}"] = {"ms_per_step": ms5, "value": w5.n_terms / (ms5 * 1e-3)}
        del s5, p5, n5
    out["precision_2048sq_128waves"] = prec
    out["frame_1024sq_32waves_noise"] = frame_pipeline(wt, workloads, stream, flush)
    # the Adam fit: 500 steps of forward + adjoint on 512^2 x 16 waves (after
    # a 50-step warm-up fit: the first use of the optimiser's kernels is slow)
    target, start = workloads.config4()
    fit.fit_waves(target.patches, target.waves, start, steps=50, lr=1e-2)
    r = fit.fit_waves(target.patches, target.waves, start, steps=500, lr=1e-2)
    out["adam_fit_512sq_16waves_500steps"] = {"ms_per_step": r["ms_per_step"], "loss_first": r["loss_first"],
                                              "loss_last": r["loss_last"],
                                              "param_errors": fit.parameter_errors(r["fitted"], target.waves)}
    return out


def workload_config(args, w, world, split=False):
    """The `config` object of both arms' lines: the workload only."""
    return {"workload": w.name.split("_shard")[0], "patches": args.patches, "vertices": w.n_vertices,
            "terms_per_step": w.n_terms, "waves_per_patch": "8..64", "grid_side": "64..1024 log-uniform",
            "heightmap": "none" if args.no_heightmap else "512^2 noise",
            "parallelism": (f"split x{world} (one {args.patches}-patch table, LPT shards of its patches)"
                            if split else f"weak x{world} (each GPU its own {args.patches} patches)")}


def timed_table_accuracy(w, hm, pos, nrm):
    """The path's error metric measured on the outputs of the timed table:
    the first, the last and six spread rows of EVERY patch against the FP64
    oracle (the checker; run after the timed region)."""
    from oracle import build as ob, oracle as O
    ob.build_oracle()
    tex = hm.texels.cpu().numpy() if hm is not None else None
    t0 = time.perf_counter()
    acc = O.accuracy_sampled_rows(w.patches, w.waves, pos.cpu().numpy(), nrm.cpu().numpy(), tex, w.heightmap)
    acc["bound"] = 1e-5
    acc["within_bound"] = bool(acc["max_rel_err"] <= 1e-5)
    acc["check_s"] = time.perf_counter() - t0
    acc["note"] = ("outputs of the last timed step; displacement error max|d32 - d64| / max|d64| over the checked "
                   "vertices (per_patch_max_rel_err: the worst single patch), normal angle excluding samples within "
                   "1e-3 texel of a heightmap cell edge")
    return acc


def measure_link(dev):
    """Host link bandwidth: 1 GiB device <-> pinned host cudaMemcpyAsync, best
    of 5 each way (CUDA events)."""
    import torch
    n = 1 << 30
    d = torch.empty(n, dtype=torch.uint8, device=dev)
    h = torch.empty(n, dtype=torch.uint8, pin_memory=True)
    d.fill_(1)
    out = {}
    for name, fn in (("d2h_gbs", lambda: h.copy_(d, non_blocking=True)),
                     ("h2d_gbs", lambda: d.copy_(h, non_blocking=True))):
        fn()
        torch.cuda.synchronize()
        best = float("inf")
        for _ in range(5):
            a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            a.record()
            fn()
            b.record()
            torch.cuda.synchronize()
            best = min(best, a.elapsed_time(b))
        out[name] = n / (best * 1e-3) / 1e9
    del d, h
    return out


def run_ours(args):
    import torch
    rank, world, local = dist_env()
    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl", device_id=dev)
    wt = __graft_entry__.load_package()
    wt.lib()
    from wave_tool_gb300 import workloads

    split = args.split and world > 1
    if split:
        # one table for every rank; each rank runs its LPT shard of the patches
        from wave_tool_gb300 import sharding
        full = workloads.config3(n_patches=args.patches, seed=2)
        mine, _ = sharding.shard_patches(full.patches, world, rank)
        w = workloads.Workload(f"{full.name}_shard{rank}of{world}", mine, full.waves, full.heightmap)
        table_terms = full.n_terms
    else:
        w = workloads.config3(n_patches=args.patches, seed=2 + rank)
        table_terms = None
    if args.no_heightmap:
        w.heightmap = None
    hm = wt.heightmap_from(w.heightmap)
    surf = wt.Surface(w.patches, w.waves, hm)
    surf.n_terms_cache = w.n_terms
    flags = wt.WT_OUT_DISPLACEMENT
    pos, nrm = surf.alloc_outputs(flags)
    stream = torch.cuda.current_stream()
    flush = torch.empty(256 << 20, dtype=torch.uint8, device=dev)  # > 129 MB L2

    def step():
        surf.displace(pos, nrm, flags=flags)

    if args.tuning == "auto":
        tuning = surf.autotune(pos, nrm, flags=flags, reps=5)  # launch shape, before any timing
    else:
        vals = [int(x) for x in args.tuning.split(",")] + [8, 1]
        wt.set_tuning(vals[0], 0, vals[1], vals[2], vals[3])
        tuning = wt.get_tuning()
    for _ in range(args.warmup):
        step()
    torch.cuda.synchronize()
    st, bad = surf.status()
    if st != 0:
        raise RuntimeError(f"device validation failed: {st} at patch {bad}")

    fma_s, sin_s = wt.measure_peaks()

    def barrier():
        if world > 1:
            import torch.distributed as dist
            dist.barrier()
        torch.cuda.synchronize()

    ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(args.steps)]
    with ClockSampler(local) as clk:
        barrier()
        t_wall = time.perf_counter()
        for e0, e1 in ev:
            flush.zero_()  # evict L2 between steps (outside the timed events)
            e0.record(stream)
            step()
            e1.record(stream)
        barrier()
        t_wall = time.perf_counter() - t_wall
    ms = [e0.elapsed_time(e1) for e0, e1 in ev]
    ms_step = sum(ms) / len(ms)
    if world > 1:
        import torch.distributed as dist
        t = torch.tensor([ms_step], device=dev)
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        ms_step = float(t.item())
    terms = w.n_terms
    # weak scaling: every rank the same amount of work; split: the one table
    job_terms = table_terms if split else terms * world
    value = job_terms / (ms_step * 1e-3)

    # the metric's error bound on the table just timed (outside the timed
    # region; the FP64 oracle is the checker): sampled rows of every patch
    accuracy = None
    if rank == 0 and not args.no_accuracy:
        accuracy = timed_table_accuracy(w, hm, pos, nrm)
    link = measure_link(dev) if rank == 0 else None

    # end to end through the C ABI from pinned host buffers, outputs in the
    # layout the reference's vertex array consumes (world positions and normals
    # as tightly packed vec3, render-engine.cpp:1175-1191).  The patches are
    # split into E2E_GROUPS contiguous groups of about equal terms, each a
    # wt_gerstner_displace call on its own stream with its own workspace: the
    # copy back of one group overlaps the kernel of the next.
    e2e_flags = wt.WT_OUT_WORLD | wt.WT_LAYOUT_VEC3
    epos, enrm = surf.alloc_outputs(e2e_flags)
    hpos = torch.empty(epos.shape, dtype=epos.dtype, pin_memory=True)
    hnrm = torch.empty(enrm.shape, dtype=enrm.dtype, pin_memory=True)
    htex = hm.texels.cpu().pin_memory() if hm is not None else None
    hw = torch.from_numpy(np.ascontiguousarray(w.waves).view(np.uint8).reshape(-1)).pin_memory()
    n_groups = max(1, args.e2e_groups)
    cum = np.cumsum(w.patches["cols"].astype(np.int64) * w.patches["rows"] * w.patches["wave_count"])
    cuts = [0] + [int(np.searchsorted(cum, cum[-1] * (g + 1) / n_groups)) + 1 for g in range(n_groups - 1)] + \
        [len(w.patches)]
    groups = []
    for g in range(n_groups):
        sub = w.patches[cuts[g]:cuts[g + 1]]
        if len(sub) == 0 or cuts[g] >= cuts[g + 1]:
            continue
        o0 = int(sub["out_offset"][0])
        o1 = int(sub["out_offset"][-1]) + int(sub["cols"][-1]) * int(sub["rows"][-1])
        gs = wt.Surface(sub, w.waves, hm)
        hp_g = torch.from_numpy(np.ascontiguousarray(sub).view(np.uint8).reshape(-1)).pin_memory()
        groups.append((gs, hp_g, o0, o1, torch.cuda.Stream()))
    h2d = (htex.numel() * 4 if htex is not None else 0) + sum(g[1].numel() + hw.numel() for g in groups)
    d2h = hpos.numel() * 4 + hnrm.numel() * 4

    def e2e_step():
        if htex is not None:
            hm.texels.copy_(htex, non_blocking=True)
        main = torch.cuda.current_stream()
        for gs, hp_g, o0, o1, st in groups:
            st.wait_stream(main)
            with torch.cuda.stream(st):
                gs.patches.copy_(hp_g, non_blocking=True)
                gs.waves.copy_(hw, non_blocking=True)
                gs.displace(epos, enrm, flags=e2e_flags, stream=st)
                hpos[o0:o1].copy_(epos[o0:o1], non_blocking=True)
                hnrm[o0:o1].copy_(enrm[o0:o1], non_blocking=True)
        for g in groups:
            main.wait_stream(g[4])

    e2e_steps = max(3, min(args.steps, 10))
    for _ in range(2):
        e2e_step()
    barrier()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    for _ in range(e2e_steps):
        e2e_step()
    e1.record(stream)
    barrier()
    e2e_ms = e0.elapsed_time(e1) / e2e_steps
    if world > 1:
        import torch.distributed as dist
        t = torch.tensor([e2e_ms], device=dev)
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        e2e_ms = float(t.item())
    e2e_value = job_terms / (e2e_ms * 1e-3)

    extras = {}
    if not args.no_extras and rank == 0:
        extras.update(side_measurements(wt, workloads, surf, pos, nrm, flags, flush, stream, ms_step, fma_s))
        # 256 plain launches (one wt_gerstner_displace per patch)
        for _ in range(2):
            surf.displace(pos, nrm, flags=flags, unbatched=True)
        torch.cuda.synchronize()
        a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        n_plain = 3
        a.record(stream)
        for _ in range(n_plain):
            surf.displace(pos, nrm, flags=flags, unbatched=True)
        b.record(stream)
        torch.cuda.synchronize()
        plain_ms = a.elapsed_time(b) / n_plain
        extras["unbatched_256_launches"] = {"ms_per_step": plain_ms, "value": terms / (plain_ms * 1e-3),
                                            "batched_speedup": plain_ms / ms_step}
        # the single 1024^2 / 32-wave / noise patch
        w2 = workloads.config2()
        s2 = wt.Surface(w2.patches, w2.waves, wt.heightmap_from(w2.heightmap))
        p2, n2 = s2.alloc_outputs(flags)
        for _ in range(5):
            s2.displace(p2, n2, flags=flags)
        torch.cuda.synchronize()
        evs = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(20)]
        for x, y in evs:
            flush.zero_()
            x.record(stream)
            s2.displace(p2, n2, flags=flags)
            y.record(stream)
        torch.cuda.synchronize()
        ms2 = statistics.median(x.elapsed_time(y) for x, y in evs)
        extras["single_patch_1024sq_32waves_noise"] = {"ms_per_step": ms2, "value": w2.n_terms / (ms2 * 1e-3)}
        # the reference-sized case: one 128^2 patch, 4 waves (launch-latency bound:
        # reported, not held to a roofline); eager call and graph replay
        w1 = workloads.config1()
        s1 = wt.Surface(w1.patches, w1.waves)
        p1, n1 = s1.alloc_outputs(flags)
        for _ in range(5):
            s1.displace(p1, n1, flags=flags)
        ms1 = _event_ms(lambda: s1.displace(p1, n1, flags=flags), 20, stream, flush)
        gs1 = torch.cuda.Stream()
        gs1.wait_stream(stream)
        g1 = torch.cuda.CUDAGraph()
        with torch.cuda.graph(g1, stream=gs1):
            s1.displace(p1, n1, flags=flags, stream=gs1)
        g1.replay()
        torch.cuda.synchronize()
        gms1 = _event_ms(g1.replay, 20, stream, flush)
        extras["plain_128sq_4waves"] = {"ms_per_step": ms1, "graph_ms_per_step": gms1,
                                        "value": w1.n_terms / (ms1 * 1e-3),
                                        "hbm_gbs": 32.0 * w1.n_vertices / (ms1 * 1e-3) / 1e9}

    cpu = None
    if rank == 0:
        cw = CpuWorkload(w)
        ncpu = os.cpu_count() or 1
        r, dt, stride, cterms = cpu_sample(cw, args.cpu_seconds, ncpu)
        cpu = {"value": r, "unit": UNIT, "cores": ncpu, "kind": "port",
               "sample": f"{every_nth(stride)} of each of the {len(w.patches)} patches of the timed table "
                         f"({cterms} terms, {dt:.1f} s); FP32 restatement of water-grid.vert, 5 evaluations/vertex",
               "build": f"gcc {cw.flags}"}
        # beside it: the same restatement on one thread, and the analytic form
        # (one evaluation per vertex, Jacobian normals) on every core
        short = max(1.0, args.cpu_seconds / 4)
        r1, _, stride1, _ = cpu_sample(cw, short, 1)
        ra, _, stridea, _ = cpu_sample(cw, short, ncpu, analytic=True)
        cpu["single_thread_value"] = r1
        cpu["analytic_value"] = ra
        cpu["analytic_note"] = (f"one evaluation per vertex, Jacobian normals, {ncpu} threads, {every_nth(stridea)} "
                                f"per patch; single thread: {every_nth(stride1)} per patch")
        del cw

    if rank == 0:
        clocks = clk.summary()
        peak_fma_terms = fma_s / 10.0   # 10 FMA of algorithmic work per term
        peak_mufu_terms = sin_s / 2.0   # sin + cos per term on the MUFU pipe
        achieved = value / world
        verts = int(np.sum(w.patches["cols"].astype(np.int64) * w.patches["rows"]))
        line = {
            "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": ms_step, "higher_is_better": True,
            "scaling": "strong" if split else "weak",
            "vs_baseline": None, "dtype": "f32",
            "data": "synthetic (SplitMix64 seed 2, shared by the ranks)" if split else
                    "synthetic (SplitMix64 seed 2 + rank)",
            "config": workload_config(args, full if split else w, world, split),
            "tuning": tuning,
            "outputs": "float4 displacement + float4 normal (e2e: packed vec3 world position + normal, the "
                       "reference's vertex-array layout); phase FP64-reduced",
            "l2": "256 MiB buffer zeroed between timed steps (outside the per-step events)",
            "roofline": {"bound": "fma+mufu", "achieved": achieved / 1e9,
                         "peak": min(peak_fma_terms, peak_mufu_terms) / 1e9,
                         "unit": "Gterms/s", "frac": achieved / min(peak_fma_terms, peak_mufu_terms),
                         "traffic": traffic_from_profile(tuning, verts),
                         "peak_source": "term roofline min(P_FMA/10, P_MUFU/2) (10 FMA + 2 sin/cos of algorithmic "
                                        "work per term), P_FMA and P_MUFU measured in this run by wt_measure_peaks",
                         "fma_leg_peak": peak_fma_terms / 1e9, "fma_leg_frac": achieved / peak_fma_terms,
                         "mufu_leg_peak": peak_mufu_terms / 1e9,
                         "hbm_gbs": 32.0 * verts / (ms_step * 1e-3) / 1e9,
                         "note": "achieved = terms per step / step time (prep launches included); the kernel "
                                 "takes sin/cos from an FMA recurrence, not 2 MUFU per term, so its own binding "
                                 "pipe is FMA issue: fma_leg_frac is its fraction of that leg"},
            "cpu_baseline": cpu,
            "e2e": {"value": e2e_value, "unit": UNIT, "h2d_bytes_per_step": int(h2d), "d2h_bytes_per_step": int(d2h),
                    "ms_per_step": e2e_ms, "stream_groups": len(groups),
                    "link_d2h_gbs_measured": link["d2h_gbs"], "link_h2d_gbs_measured": link["h2d_gbs"],
                    "link_bound_ms": 1e3 * (d2h / (link["d2h_gbs"] * 1e9) + h2d / (link["h2d_gbs"] * 1e9)),
                    "copy_frac": d2h / (e2e_ms * 1e-3) / (link["d2h_gbs"] * 1e9),
                    "note": "copy_frac: the copy-back bytes over the whole end-to-end step time, as a fraction of "
                            "the host link's D2H bandwidth measured in this run (1 GiB device -> pinned host "
                            "cudaMemcpyAsync, best of 5); link_bound_ms: the step's copies alone at those rates"},
            "accuracy": accuracy,
            "gpu_launches": 3 * args.steps,
            "clocks": clocks,
            "wall_s_timed_region": t_wall,
            "extras": extras,
        }
        print(json.dumps(line), flush=True)
    if world > 1:
        import torch.distributed as dist
        dist.destroy_process_group()


def run_adjoint_only(args):
    """wt_gerstner_adjoint on the 64-patch batched-adjoint workload: warmup,
    then `steps` timed calls; prints one JSON line (not the headline)."""
    import torch
    wt = __graft_entry__.load_package()
    from wave_tool_gb300 import workloads
    w = workloads.config5_batched_adjoint()
    surf = wt.Surface(w.patches, w.waves, wt.heightmap_from(w.heightmap))
    pos, nrm = surf.alloc_outputs(0)
    gen = torch.Generator(device="cuda").manual_seed(1)
    gp = torch.randn(pos.shape, device="cuda", generator=gen)
    gn = torch.randn(nrm.shape, device="cuda", generator=gen)
    sums = None
    if args.saved_sums:
        sums = torch.empty((surf.n_vertices, 8), dtype=torch.float32, device="cuda")
        surf.displace(pos, nrm, flags=0, sums=sums)
    for _ in range(args.warmup):
        surf.adjoint(gp, gn, sums=sums)
    ms = _event_ms(lambda: surf.adjoint(gp, gn, sums=sums), args.steps, torch.cuda.current_stream())
    print(json.dumps({"mode": "adjoint", "saved_sums": sums is not None, "workload": w.name, "terms": w.n_terms,
                      "ms_per_step": ms,
                      "terms_per_s": w.n_terms / (ms * 1e-3)}), flush=True)


def run_displace_only(args):
    """wt_gerstner_displace alone on one workload (warmup, then `steps`
    timed calls, L2 flushed between them); prints one JSON line (not the
    headline)."""
    import torch
    wt = __graft_entry__.load_package()
    from wave_tool_gb300 import workloads
    w = {"config2": workloads.config2, "config3": lambda: workloads.config3(n_patches=args.patches, seed=2),
         "config5": lambda: workloads.config5(time_s=100.0)}[args.workload]()
    surf = wt.Surface(w.patches, w.waves, wt.heightmap_from(w.heightmap))
    pos, nrm = surf.alloc_outputs(wt.WT_OUT_DISPLACEMENT)
    if args.tuning == "auto":
        tuning = surf.autotune(pos, nrm, flags=wt.WT_OUT_DISPLACEMENT, reps=5)
    else:
        vals = [int(x) for x in args.tuning.split(",")] + [8, 1]
        wt.set_tuning(vals[0], 0, vals[1], vals[2], vals[3])
        tuning = wt.get_tuning()
    for _ in range(args.warmup):
        surf.displace(pos, nrm, flags=wt.WT_OUT_DISPLACEMENT)
    flush = torch.empty(256 << 20, dtype=torch.uint8, device="cuda")
    ms = _event_ms(lambda: surf.displace(pos, nrm, flags=wt.WT_OUT_DISPLACEMENT), args.steps,
                   torch.cuda.current_stream(), flush)
    print(json.dumps({"mode": "displace", "workload": w.name, "terms": w.n_terms, "ms_per_step": ms,
                      "terms_per_s": w.n_terms / (ms * 1e-3), "tuning": tuning}), flush=True)


def run_frame_only(args):
    """The water frame (camera -> pixels at 1920 x 1080 over a 1024^2 grid,
    eager launches): warmup, then `steps` timed frames; prints one JSON line
    (not the headline)."""
    import torch
    wt = __graft_entry__.load_package()
    from wave_tool_gb300 import workloads
    F = build_frame(wt, workloads)
    for _ in range(args.warmup):
        F["frame"]()
    ms = _event_ms(F["frame"], args.steps, torch.cuda.current_stream())
    print(json.dumps({"mode": "frame", "vertices": F["n"], "viewport": [F["VW"], F["VH"]], "ms_per_frame": ms,
                      "frames_per_s": 1e3 / ms}), flush=True)


def main():
    args = parse_args()
    if args.mode == "adjoint":
        run_adjoint_only(args)
        return
    if args.mode == "frame":
        run_frame_only(args)
        return
    if args.mode == "displace":
        run_displace_only(args)
        return
    if args.impl == "reference":
        run_reference(args)
    else:
        run_ours(args)


if __name__ == "__main__":
    main()
