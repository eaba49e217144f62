"""Seeded synthetic workloads (SplitMix64), one per benchmark configuration.

The reference has no datasets: its waves are four hand-set defaults
(src/render-engine.cpp:46-49) edited through ImGui sliders
(src/program.cpp:368-408).  These generators produce the five configurations
the path is measured on, with the distributions stated for each; the n-th
configuration uses seed n-1.  Wave speed is not given by the configurations,
so deep-water dispersion omega = sqrt(g k), g = 9.81 m/s^2, is used
(speed = omega / k = sqrt(g / k)), and Q_i = q / (k A N) is the reference's
steepness normalisation (src/render-engine.cpp:1073) with q = 0.5.
"""
from __future__ import annotations

import math
from dataclasses import dataclass, field

import numpy as np

from .abi import NOISE_TERM_DTYPE, PATCH_DTYPE, WAVE_DTYPE, WT_WRAP_REPEAT, patch_vertices

G = 9.81
MASK64 = (1 << 64) - 1


class SplitMix64:
    """SplitMix64 (Steele, Lea, Flood 2014): state += golden gamma, then two
    xor-shift-multiply rounds."""

    def __init__(self, seed: int):
        self.state = seed & MASK64

    def next_u64(self) -> int:
        self.state = (self.state + 0x9E3779B97F4A7C15) & MASK64
        z = self.state
        z = ((z ^ (z >> 30)) * 0xBF58476D1CE4E5B9) & MASK64
        z = ((z ^ (z >> 27)) * 0x94D049BB133111EB) & MASK64
        return z ^ (z >> 31)

    def uniform(self, lo: float = 0.0, hi: float = 1.0) -> float:
        return lo + (hi - lo) * ((self.next_u64() >> 11) * (1.0 / (1 << 53)))

    def log_uniform(self, lo: float, hi: float) -> float:
        return math.exp(self.uniform(math.log(lo), math.log(hi)))

    def integer(self, lo: int, hi: int) -> int:
        """Uniform integer in [lo, hi]."""
        return lo + int(self.uniform() * (hi - lo + 1)) if hi > lo else lo


@dataclass
class Heightmap:
    width: int
    height: int
    sample_scale: float
    disp_scale: float
    wrap: int
    terms: np.ndarray  # NOISE_TERM_DTYPE


@dataclass
class Workload:
    name: str
    patches: np.ndarray  # PATCH_DTYPE
    waves: np.ndarray  # WAVE_DTYPE
    heightmap: Heightmap | None = None
    notes: dict = field(default_factory=dict)

    @property
    def n_vertices(self) -> int:
        return int(np.sum(patch_vertices(self.patches)))

    @property
    def n_terms(self) -> int:
        return int(np.sum(patch_vertices(self.patches) * self.patches["wave_count"].astype(np.uint64)))


def make_wave(k_lambda: float, amplitude: float, angle: float, q_user: float, n: int,
              phase: float) -> tuple:
    k = 2.0 * math.pi / k_lambda
    q_i = q_user / (k * amplitude * n) if amplitude > 0 else 0.0
    return (amplitude, k_lambda, math.cos(angle), math.sin(angle), q_i, math.sqrt(G / k), phase, 0.0)


def waves_wide(rng: SplitMix64, n: int, q_user: float = 0.5, lam=(0.5, 60.0),
               spread_deg: float = 90.0) -> list:
    """lambda log-uniform in `lam`, A = lambda/100 * U[0.5, 1], direction within
    +-spread of the wind (+x), phase U[0, 2pi)."""
    out = []
    for _ in range(n):
        lmb = rng.log_uniform(*lam)
        amp = lmb / 100.0 * rng.uniform(0.5, 1.0)
        ang = math.radians(rng.uniform(-spread_deg, spread_deg))
        ph = rng.uniform(0.0, 2.0 * math.pi)
        out.append(make_wave(lmb, amp, ang, q_user, n, ph))
    return out


def square_patch(cx: float, cz: float, half: float, side: int, wave_offset: int, wave_count: int,
                 time_s: float, out_offset: int, y_offset: float = 0.0) -> tuple:
    """Corners BL(-h,+h) BR(+h,+h) TL(-h,-h) TR(+h,-h): u along +x, v along -z
    (the heightmap lookup flips z, water-grid.vert:103)."""
    return (
        (cx - half, cz + half), (cx + half, cz + half), (cx - half, cz - half), (cx + half, cz - half),
        side, side, wave_offset, wave_count, time_s, y_offset, 0, out_offset,
    )


def noise_terms(rng: SplitMix64, n: int = 64, kmax: int = 32) -> np.ndarray:
    """n integer wavenumbers with 0 < |k| <= kmax, amplitude U[0.5,1]/|k|,
    phase U[0, 2pi)."""
    terms = []
    while len(terms) < n:
        kx = rng.integer(-kmax, kmax)
        ky = rng.integer(-kmax, kmax)
        r2 = kx * kx + ky * ky
        if r2 == 0 or r2 > kmax * kmax:
            continue
        amp = rng.uniform(0.5, 1.0) / math.sqrt(r2)
        terms.append((kx, ky, amp, rng.uniform(0.0, 2.0 * math.pi)))
    return np.array(terms, dtype=NOISE_TERM_DTYPE)


def config1() -> Workload:
    """128 x 128 vertices over a 200 m x 200 m patch, 4 waves: lambda U[2,20] m,
    A = lambda/80, directions within +-45 deg of +x, t = 100 s.  Seed 0."""
    rng = SplitMix64(0)
    n = 4
    waves = []
    for _ in range(n):
        lmb = rng.uniform(2.0, 20.0)
        ang = math.radians(rng.uniform(-45.0, 45.0))
        ph = rng.uniform(0.0, 2.0 * math.pi)
        waves.append(make_wave(lmb, lmb / 80.0, ang, 0.5, n, ph))
    patches = np.array([square_patch(0.0, 0.0, 100.0, 128, 0, n, 100.0, 0)], dtype=PATCH_DTYPE)
    return Workload("config1_plain_128sq_4waves", patches, np.array(waves, dtype=WAVE_DTYPE))


def _noise(rng: SplitMix64) -> Heightmap:
    return Heightmap(512, 512, 0.02, 0.2, WT_WRAP_REPEAT, noise_terms(rng))


def config2() -> Workload:
    """1024 x 1024 vertices over 200 m x 200 m, 32 waves (lambda log-uniform
    [0.5, 60] m, A = lambda/100 * U[0.5,1], +-90 deg of wind), t = 100 s, plus a
    512 x 512 R32F noise heightmap of 64 integer-wavenumber sinusoids
    (|k| <= 32), REPEAT, sample scale 0.02, displacement scale 0.2 m.  Seed 1."""
    rng = SplitMix64(1)
    n = 32
    waves = waves_wide(rng, n)
    hm = _noise(rng)
    patches = np.array([square_patch(0.0, 0.0, 100.0, 1024, 0, n, 100.0, 0)], dtype=PATCH_DTYPE)
    return Workload("config2_single_1024sq_32waves_noise", patches, np.array(waves, dtype=WAVE_DTYPE), hm)


def config3(n_patches: int = 256, seed: int = 2, spacing: float = 0.2) -> Workload:
    """256 independent patches: side round(exp U[ln 64, ln 1024]), 8..64 waves
    each (config-2 distributions), t U[0, 1e3] s, vertex spacing 0.2 m, laid
    out disjoint on a 16 x 16 lattice of 256 m cells; config-2 noise layer."""
    rng = SplitMix64(seed)
    waves = []
    patches = []
    out = 0
    per_row = int(math.ceil(math.sqrt(n_patches)))
    for i in range(n_patches):
        side = int(round(math.exp(rng.uniform(math.log(64.0), math.log(1024.0)))))
        n = rng.integer(8, 64)
        t = rng.uniform(0.0, 1.0e3)
        ws = waves_wide(rng, n)
        cx = (i % per_row) * 256.0
        cz = (i // per_row) * 256.0
        half = 0.5 * (side - 1) * spacing
        patches.append(square_patch(cx, cz, half, side, len(waves), n, t, out))
        waves.extend(ws)
        out += side * side
    hm = _noise(rng)
    return Workload(f"config3_batched_{n_patches}_uneven_patches", np.array(patches, dtype=PATCH_DTYPE),
                    np.array(waves, dtype=WAVE_DTYPE), hm)


def config4(seed: int = 3) -> tuple[Workload, np.ndarray]:
    """Adjoint fit: 512 x 512 vertices over 100 m x 100 m, a hidden 16-wave set
    (lambda log-uniform [1, 30] m, A = lambda/100 * U[0.5,1], +-90 deg), t = 10 s.
    Returns the target workload and the perturbed starting waves: A, lambda, Q
    scaled by U[0.9, 1.1], direction rotated U[-10, 10] deg, phase + U[-0.5, 0.5].
    Other seeds give other draws of the same distributions."""
    rng = SplitMix64(seed)
    n = 16
    hidden = np.array(waves_wide(rng, n, lam=(1.0, 30.0)), dtype=WAVE_DTYPE)
    patches = np.array([square_patch(0.0, 0.0, 50.0, 512, 0, n, 10.0, 0)], dtype=PATCH_DTYPE)
    start = hidden.copy()
    for w in start:
        w["amplitude"] *= rng.uniform(0.9, 1.1)
        w["wavelength"] *= rng.uniform(0.9, 1.1)
        w["steepness_q"] *= rng.uniform(0.9, 1.1)
        a = math.atan2(float(w["dir_z"]), float(w["dir_x"])) + math.radians(rng.uniform(-10.0, 10.0))
        w["dir_x"], w["dir_z"] = math.cos(a), math.sin(a)
        w["phase"] += rng.uniform(-0.5, 0.5)
    return Workload("config4_adjoint_fit_512sq_16waves", patches, hidden), start


def config5(time_s: float = 1.0e2, side: int = 2048, n: int = 128) -> Workload:
    """Precision stress: 2048 x 2048 vertices (0.2 m spacing), 128 waves of the
    config-2 distributions, t in {1e2, 1e4, 1e6} s.  Seed 4."""
    rng = SplitMix64(4)
    waves = waves_wide(rng, n)
    half = 0.5 * (side - 1) * 0.2
    patches = np.array([square_patch(0.0, 0.0, half, side, 0, n, time_s, 0)], dtype=PATCH_DTYPE)
    return Workload(f"config5_precision_{side}sq_{n}waves_t{time_s:g}", patches,
                    np.array(waves, dtype=WAVE_DTYPE))


def config5_batched_adjoint() -> Workload:
    """64 config-3-style uneven patches for the batched adjoint.  Seed 4."""
    w = config3(n_patches=64, seed=4)
    w.name = "config5_batched_adjoint_64_uneven_patches"
    return w


def small_random(seed: int, n_patches: int = 3, side_range=(2, 70), n_waves_range=(0, 40),
                 heightmap: bool = True, wrap: int = WT_WRAP_REPEAT, spacing: float = 0.37,
                 skew: bool = True) -> Workload:
    """Small ragged cases for parity tests: uneven sides (non-square too),
    0..n waves, optional skewed (non-parallelogram) corners, large world
    offsets and times."""
    rng = SplitMix64(1000 + seed)
    waves, patches, out = [], [], 0
    for i in range(n_patches):
        cols = rng.integer(*side_range)
        rows = rng.integer(*side_range)
        n = rng.integer(*n_waves_range)
        ws = waves_wide(rng, max(n, 1))[:n]
        cx, cz = rng.uniform(-3000, 3000), rng.uniform(-3000, 3000)
        hx, hz = 0.5 * (cols - 1) * spacing, 0.5 * (rows - 1) * spacing
        jitter = (lambda: rng.uniform(-0.2, 0.2) * hx) if skew else (lambda: 0.0)
        bl = (cx - hx + jitter(), cz + hz + jitter())
        br = (cx + hx + jitter(), cz + hz + jitter())
        tl = (cx - hx + jitter(), cz - hz + jitter())
        tr = (cx + hx + jitter(), cz - hz + jitter())
        t = rng.uniform(0.0, 5.0e3)
        patches.append((bl, br, tl, tr, cols, rows, len(waves), n, t, rng.uniform(-0.1, 0.1), 0, out))
        waves.extend(ws)
        out += cols * rows
    hm = None
    if heightmap:
        hm = Heightmap(rng.integer(3, 40), rng.integer(3, 40), rng.uniform(0.01, 0.3),
                       rng.uniform(0.05, 0.5), wrap, noise_terms(rng, n=8, kmax=3))
    if not waves:
        waves = [make_wave(10.0, 0.1, 0.0, 0.5, 1, 0.0)]
    return Workload(f"small_random_{seed}", np.array(patches, dtype=PATCH_DTYPE),
                    np.array(waves, dtype=WAVE_DTYPE), hm)


CONFIGS = {"config1": config1, "config2": config2, "config3": config3, "config5": config5}
