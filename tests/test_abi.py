"""CPU tests of the C ABI library: it loads, exports every symbol the header
declares, its struct layouts match the numpy mirrors, and its host-only
entry points (no GPU needed) behave."""
from __future__ import annotations

import ctypes as C
import re
import subprocess
from pathlib import Path

import numpy as np
import pytest

ROOT = Path(__file__).resolve().parent.parent
HEADER = ROOT / "include" / "wt.h"


@pytest.fixture(scope="module")
def built(wt):
    wt.build()
    return wt.lib()


def declared_functions():
    text = HEADER.read_text()
    return sorted(set(re.findall(r"^\s*(?:const char\*|wt_status)\s+(wt_\w+)\s*\(", text, re.M)))


def test_library_exports_every_declared_symbol(wt, built):
    names = declared_functions()
    assert len(names) >= 12
    for n in names:
        assert hasattr(built, n), n
    assert sorted(wt.EXPORTED) == names
    assert "sm_103a" in wt.version()


def test_struct_layouts_match_c(wt, tmp_path):
    """offsetof/sizeof of every wt.h struct, from the C compiler, equal the
    numpy dtypes the host layer uploads."""
    from wave_tool_gb300 import abi
    checks = {"wt_wave": abi.WAVE_DTYPE, "wt_patch": abi.PATCH_DTYPE, "wt_noise_term": abi.NOISE_TERM_DTYPE,
              "wt_wave_grad": abi.WAVE_GRAD_DTYPE, "wt_camera": abi.CAMERA_DTYPE, "wt_view": abi.VIEW_DTYPE}
    lines = ['#include <stdio.h>', '#include <stddef.h>', f'#include "{HEADER}"', "int main(void) {"]
    for s, dt in checks.items():
        lines.append(f'printf("{s} sizeof %zu\\n", sizeof({s}));')
        for f in dt.names:
            lines.append(f'printf("{s} {f} %zu\\n", offsetof({s}, {f}));')
    lines.append("return 0; }")
    src = tmp_path / "layout.c"
    src.write_text("\n".join(lines))
    exe = tmp_path / "layout"
    subprocess.run(["gcc", "-o", str(exe), str(src)], check=True)
    out = subprocess.run([str(exe)], capture_output=True, text=True, check=True).stdout.split("\n")
    for line in filter(None, out):
        s, f, v = line.split()
        dt = checks[s]
        if f == "sizeof":
            assert dt.itemsize == int(v), s
        else:
            assert dt.fields[f][1] == int(v), (s, f)


def test_ctypes_layouts_match_c(wt, tmp_path):
    """offsetof/sizeof of the structs the host layer passes by pointer through
    ctypes equal the ctypes mirrors."""
    checks = {"wt_heightmap": wt.CHeightmap, "wt_tuning": wt.CTuning, "wt_water_shading": wt.CWaterShading,
              "wt_water_textures": wt.CWaterTextures, "wt_stage_outputs": wt.CStageOutputs}
    lines = ['#include <stdio.h>', '#include <stddef.h>', f'#include "{HEADER}"', "int main(void) {"]
    for s, S in checks.items():
        lines.append(f'printf("{s} sizeof %zu\\n", sizeof({s}));')
        for f, _ in S._fields_:
            lines.append(f'printf("{s} {f} %zu\\n", offsetof({s}, {f}));')
    lines.append("return 0; }")
    src = tmp_path / "layout_ctypes.c"
    src.write_text("\n".join(lines))
    exe = tmp_path / "layout_ctypes"
    subprocess.run(["gcc", "-o", str(exe), str(src)], check=True)
    out = subprocess.run([str(exe)], capture_output=True, text=True, check=True).stdout.split("\n")
    for line in filter(None, out):
        s, f, v = line.split()
        S = checks[s]
        if f == "sizeof":
            assert C.sizeof(S) == int(v), s
        else:
            assert getattr(S, f).offset == int(v), (s, f)


def test_wave_from_reference_applies_q_normalisation(wt, built):
    """render-engine.cpp:1073: Q_i = Q / (w * A * count) in FP32, 0 if w*A = 0."""
    w = wt.wave_from_reference(0.06, 1.0, 2.0, 1.0, 1.0, 0.0, 4)[0]
    exp = np.float32(1.0) / (np.float32(1.0) * np.float32(0.06) * np.float32(4))
    assert np.float32(w["steepness_q"]) == exp
    assert abs(float(w["wavelength"]) - 2 * np.pi) < 1e-6 and abs(float(w["speed"]) - 2.0) < 1e-6
    z = wt.wave_from_reference(0.0, 0.0, 0.0, 0.5, 0.0, 1.0, 4)[0]
    assert z["steepness_q"] == 0.0 and np.isinf(z["wavelength"])
    with pytest.raises(wt.WtError) as e:
        wt.wave_from_reference(0.3, 0.0, 1.0, 0.5, 0.0, 1.0, 4)
    assert e.value.status == wt.abi.WT_ERR_UNSUPPORTED
    with pytest.raises(wt.WtError):
        wt.wave_from_reference(-1.0, 1.0, 1.0, 0.5, 0.0, 1.0, 4)


def test_host_validation_without_gpu(wt, built):
    """Arguments rejected before any CUDA call."""
    L = built
    assert L.wt_gerstner_displace(None, 1, None, 0, None, None, None, 1, 0, None, 0, None) == 1
    assert b"NULL" in L.wt_last_error()
    assert L.wt_grid_indices(1, 5, 0, None, None) == 1
    assert L.wt_grid_indices(70000, 70000, 0, 16, None) == 1  # indices exceed uint32
    assert L.wt_noise_synth(None, 0, 0, 4, None, None, 0, None) == 1
    sz = C.c_size_t()
    assert L.wt_displace_workspace_size(256, 9000, C.byref(sz)) == 0
    assert sz.value > 9000 * 64 and sz.value % 256 == 0
    assert L.wt_displace_workspace_size(1 << 25, 0, C.byref(sz)) == 1


def test_package_has_no_cpu_fallback(wt, monkeypatch, tmp_path):
    """Without the CUDA library every entry point raises."""
    monkeypatch.setattr(wt, "_lib", None)
    monkeypatch.setattr(wt, "LIB_PATH", tmp_path / "missing.so")
    with pytest.raises(RuntimeError, match="no CPU fallback"):
        wt.lib()
