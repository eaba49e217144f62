"""Build recipe of the CPU oracle (test infrastructure only).

``build_oracle()`` compiles the C restatement (gerstner_f64.c,
reference_mode.c, indices_noise.c, projgrid.c) into ``oracle/_build/liboracle.so``.
``build_ref()`` compiles the reference's own vertex shader
(``assets/shaders/water-grid.vert`` under the reference checkout) as C++ over
``glsl_shim.hpp`` into ``oracle/_ref/libwgvert_ref.so``; it needs the
reference checkout and is skipped without it.

Both use -ffp-contract=off so that FP32 results do not depend on whether the
host compiler fuses multiply-adds (x86_64 and aarch64 give the same bits).
"""
from __future__ import annotations

import os
import subprocess
from pathlib import Path

HERE = Path(__file__).resolve().parent
BUILD = HERE / "_build"
REF_OUT = HERE / "_ref"
SOURCES = ["gerstner_f64.c", "reference_mode.c", "indices_noise.c", "projgrid.c", "water.c"]
LIB = BUILD / "liboracle.so"
REF_LIB = REF_OUT / "libwgvert_ref.so"
REF_FRAG_LIB = REF_OUT / "libwgfrag_ref.so"
CFLAGS = ["-O2", "-fPIC", "-ffp-contract=off", "-fno-fast-math", "-std=c11", "-Wall"]
# The timed CPU baseline: the same FP32 restatement of the shader
# (reference_mode.c) built for speed, in a library of its own so that the
# bit-exact oracle build above is untouched: -O3, multiply-adds fused, no
# errno or trap handling in libm calls.  -ffast-math is not used: its
# reassociation and reciprocal rules break the shader's float arithmetic on
# vertex ids (mod(id, L) through floor(id / L) lands on the wrong column at
# row starts; tests/test_oracle.py checks the build against the bit-exact
# one).  No -march=native: host code must build on the x86_64 and the
# aarch64 machines alike (the default aarch64 target already has the NEON
# vector unit and fused multiply-add).
TIMED_LIB = BUILD / "libcpu_timed.so"
TIMED_CFLAGS = ["-O3", "-ffp-contract=fast", "-fno-math-errno", "-fno-trapping-math", "-fPIC", "-std=c11", "-Wall"]


def reference_dir() -> Path:
    """The reference checkout: $WT_REFERENCE_DIR, else a directory named
    ``reference`` beside this repository's root."""
    return Path(os.environ.get("WT_REFERENCE_DIR", HERE.parent.parent / "reference"))


def _stale(out: Path, deps) -> bool:
    if not out.exists():
        return True
    t = out.stat().st_mtime
    return any(Path(d).stat().st_mtime > t for d in deps)


def build_oracle(force: bool = False) -> Path:
    BUILD.mkdir(exist_ok=True)
    deps = [HERE / s for s in SOURCES] + [HERE / "wt_oracle.h", HERE / "projgrid_body.inc",
                                          HERE.parent / "include" / "wt.h"]
    if force or _stale(LIB, deps):
        cmd = ["gcc", *CFLAGS, "-shared", "-o", str(LIB), *[str(HERE / s) for s in SOURCES],
               "-lm", "-lpthread"]
        subprocess.run(cmd, check=True)
    return LIB


def build_timed(force: bool = False, cflags=None, out: Path | None = None) -> Path:
    """The timed CPU baseline library (reference_mode.c with TIMED_CFLAGS)."""
    BUILD.mkdir(exist_ok=True)
    out = out or TIMED_LIB
    deps = [HERE / "reference_mode.c", HERE / "wt_oracle.h", HERE.parent / "include" / "wt.h"]
    if force or cflags is not None or _stale(out, deps):
        cmd = ["gcc", *(cflags or TIMED_CFLAGS), "-shared", "-o", str(out), str(HERE / "reference_mode.c"),
               "-lm", "-lpthread"]
        subprocess.run(cmd, check=True)
    return out


def build_ref(force: bool = False) -> Path | None:
    """Compile the reference vertex shader where it lies; None if it is absent."""
    return _build_shader("water-grid.vert", "glsl_shim.hpp", "ref_driver.inc", REF_LIB, force)


def build_ref_frag(force: bool = False) -> Path | None:
    """Compile the reference water fragment shader where it lies; None if absent."""
    return _build_shader("water-grid.frag", "glsl_frag_shim.hpp", "ref_frag_driver.inc", REF_FRAG_LIB, force)


def _build_shader(name: str, shim: str, driver: str, out: Path, force: bool) -> Path | None:
    src = reference_dir() / "assets" / "shaders" / name
    if not src.exists():
        return None
    REF_OUT.mkdir(exist_ok=True)
    deps = [src, HERE / shim, HERE / driver, HERE / "wt_oracle.h", HERE.parent / "include" / "wt.h"]
    if not (force or _stale(out, deps)):
        return out
    text = src.read_text()
    first, _, body = text.partition("\n")
    if not first.startswith("#version"):
        raise RuntimeError(f"unexpected first line in {src}: {first!r}")
    # The GLSL '#version' line is the only line that is not C++; it is dropped
    # and the rest is compiled unchanged between the shim and the driver.
    tu = (f'#include "{shim}"\n'
          f'#line 2 "{src}"\n' + body +
          f'\n#include "{driver}"\n')
    cmd = ["g++", "-O2", "-fPIC", "-shared", "-ffp-contract=off", "-fno-fast-math",
           "-std=gnu++17", "-w", "-I", str(HERE), "-x", "c++", "-", "-o", str(out)]
    subprocess.run(cmd, input=tu.encode(), check=True)
    return out


if __name__ == "__main__":
    print(build_oracle(force=True))
    print(build_timed(force=True))
    print(build_ref(force=True))
    print(build_ref_frag(force=True))
