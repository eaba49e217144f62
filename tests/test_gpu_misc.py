"""GPU parity of the index buffer and the noise heightmap; device-side and
host-side validation through the C ABI."""
from __future__ import annotations

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("cols,rows,base", [(513, 513, 0), (2, 2, 0), (3, 3, 7), (65, 17, 100), (1025, 3, 0),
                                            (2048, 2048, 0)])
def test_grid_indices_bit_exact(wt, oracle, gpu, cols, rows, base):
    """src/program.cpp:686-717 (L = 513 there) bit for bit."""
    got = wt.grid_indices(cols, rows, base).cpu().numpy().view(np.uint32)
    assert np.array_equal(got, oracle.grid_indices(cols, rows, base))


def test_grid_indices_large_grid_on_device(wt, gpu):
    """A 4097^2 grid (100 M indices) checked against the closed form on the
    device (too large for the CPU loop)."""
    import torch
    L = 4097
    idx = wt.grid_indices(L, L).view(-1, 6).to(torch.int64)
    r = torch.arange(L - 1, device="cuda").repeat_interleave(L - 1)
    c = torch.arange(L - 1, device="cuda").repeat(L - 1)
    base = r * L + c
    exp = torch.stack([base, base + L + 1, base + L, base, base + 1, base + L + 1], 1)
    assert torch.equal(idx, exp)


def test_noise_matches_f64(wt, oracle, gpu):
    from wave_tool_gb300 import workloads
    for (w, h, n, k, seed) in ((512, 512, 64, 32, 1), (37, 21, 9, 5, 2), (1, 1, 3, 2, 3)):
        terms = workloads.noise_terms(workloads.SplitMix64(seed), n=n, kmax=k)
        got = wt.noise_synth(terms, w, h).cpu().numpy()
        exp = oracle.noise_f64(terms, w, h)
        if w * h > 1:
            assert np.abs(got - exp).max() < 2e-5
            assert got.min() == 0.0 and got.max() == 1.0


@pytest.mark.parametrize("time_s", [0.0, 1.7, 3.0e4])
def test_animated_noise_matches_f64(wt, oracle, gpu, time_s):
    """wt_noise_synth_animated: each term's phase advanced by its rate x t
    (FP64 reduction on the device) against the FP64 restatement."""
    from wave_tool_gb300 import workloads
    for (w, h, n, k, seed) in ((512, 512, 64, 32, 4), (37, 21, 9, 5, 5)):
        terms = workloads.noise_terms(workloads.SplitMix64(seed), n=n, kmax=k)
        rng = np.random.default_rng(seed)
        rates = rng.uniform(-3.0, 3.0, n).astype(np.float32)
        got = wt.noise_synth(terms, w, h, rates=rates, time_s=time_s).cpu().numpy()
        exp = oracle.noise_f64(terms, w, h, rates=rates, time_s=time_s)
        assert np.abs(got - exp).max() < 2e-5
        assert got.min() == 0.0 and got.max() == 1.0


def test_animated_noise_period_and_workspace(wt, gpu):
    """Rates of whole turns per second: the layer at t = 1 s is the layer at
    t = 0; a workspace below wt_noise_workspace_size is refused."""
    import torch
    from wave_tool_gb300 import workloads
    terms = workloads.noise_terms(workloads.SplitMix64(8), n=16, kmax=8)
    rates = (2.0 * np.pi * np.arange(1, 17)).astype(np.float32)
    a = wt.noise_synth(terms, 64, 48, rates=rates, time_s=0.0)
    b = wt.noise_synth(terms, 64, 48, rates=rates, time_s=1.0)
    assert float((a - b).abs().max()) < 2e-5
    need = wt.noise_workspace_bytes(16, 64, 48)
    assert need == 256 + 8 * 16 * (64 + 48)
    with pytest.raises(wt.WtError):
        wt.noise_synth(terms, 64, 48, workspace=wt.empty_bytes(need - 16))
    del torch


def test_device_side_validation(wt, gpu):
    """Invalid patches are skipped and reported with the first bad index."""
    import torch
    from wave_tool_gb300 import workloads
    w = workloads.small_random(1, n_patches=4)
    good = wt.Surface(w.patches, w.waves)
    ref, _ = good.displace()
    bad = w.patches.copy()
    bad[2]["cols"] = 1                      # grid too small
    bad[3]["wave_offset"] = len(w.waves)    # waves out of range
    s = wt.Surface(bad, w.waves)
    pos, nrm = s.alloc_outputs()
    pos.fill_(-7.0)
    s.displace(pos, nrm)
    st, first = s.status()
    assert st == wt.abi.WT_ERR_INVALID_ARG and first == 2
    o0, n0 = int(bad[0]["out_offset"]), int(bad[0]["cols"] * bad[0]["rows"])
    assert torch.equal(pos[o0:o0 + n0], ref[o0:o0 + n0])   # valid patches still ran
    o2 = int(bad[2]["out_offset"])
    assert float(pos[o2, 0]) == -7.0                        # invalid ones were not written
    # NaN wave parameter
    k = int(np.argmax(w.patches["wave_count"] > 0))
    wv = w.waves.copy()
    wv[int(w.patches[k]["wave_offset"])]["wavelength"] = np.nan
    s2 = wt.Surface(w.patches, wv)
    s2.displace()
    st, first = s2.status()
    assert st == wt.abi.WT_ERR_INVALID_ARG and first == k
    # output capacity too small for the last patch
    s3 = wt.Surface(w.patches, w.waves)
    p3, n3 = s3.alloc_outputs()
    s3.displace(p3[:-1], n3[:-1])
    st, first = s3.status()
    assert st == wt.abi.WT_ERR_INVALID_ARG and first == 3


@pytest.mark.parametrize("bad_kind", ["nan_wavelength", "inf_amplitude", "zero_wavelength"])
def test_bad_waves_in_large_tables(wt, gpu, bad_kind):
    """More (patch, wave) pairs than the scan block has threads (the shared
    bitmask validation): a patch using a bad wave is skipped and reported
    (the smallest such index), patches sharing no bad wave still run, and
    two patches sharing the bad wave are both skipped."""
    import torch
    from wave_tool_gb300 import workloads
    w = workloads.config3(n_patches=40, seed=13)
    assert int(w.patches["wave_count"].sum()) > 1024
    good = wt.Surface(w.patches, w.waves)
    ref, _ = good.displace()
    patches = w.patches.copy()
    victim = 17
    wv = int(patches[victim]["wave_offset"]) + 3
    patches[29]["wave_offset"] = patches[victim]["wave_offset"]   # 29 shares 17's waves
    patches[29]["wave_count"] = min(int(patches[29]["wave_count"]), int(patches[victim]["wave_count"]))
    waves = w.waves.copy()
    field, value = {"nan_wavelength": ("wavelength", np.nan), "inf_amplitude": ("amplitude", np.inf),
                    "zero_wavelength": ("wavelength", 0.0)}[bad_kind]
    waves[wv][field] = value
    s = wt.Surface(patches, waves)
    pos, nrm = s.alloc_outputs()
    pos.fill_(-7.0)
    s.displace(pos, nrm)
    st, first = s.status()
    assert st == wt.abi.WT_ERR_INVALID_ARG and first == victim
    for p in (victim, 29):
        o = int(patches[p]["out_offset"])
        assert float(pos[o, 0]) == -7.0
    o0, n0 = int(patches[0]["out_offset"]), int(patches[0]["cols"] * patches[0]["rows"])
    assert torch.equal(pos[o0:o0 + n0], ref[o0:o0 + n0])


def test_workspace_too_small_for_wave_slots(wt, gpu):
    import ctypes as C
    from wave_tool_gb300 import workloads
    w = workloads.small_random(2, n_patches=3, n_waves_range=(10, 20))
    s = wt.Surface(w.patches, w.waves)
    small = wt.empty_bytes(wt.displace_workspace_bytes(3, 1))
    pos, nrm = s.alloc_outputs()
    wt.check(wt.lib().wt_gerstner_displace(s.patches.data_ptr(), 3, s.waves.data_ptr(), len(w.waves), None,
                                           pos.data_ptr(), nrm.data_ptr(), pos.shape[0], 0, small.data_ptr(),
                                           small.numel(), wt.stream_handle()))
    st, _ = wt.workspace_status(small)
    assert st == wt.abi.WT_ERR_NOMEM
    del C


def test_host_side_validation(wt, gpu):
    from wave_tool_gb300 import workloads
    w = workloads.small_random(4, n_patches=2)
    s = wt.Surface(w.patches, w.waves)
    pos, nrm = s.alloc_outputs()
    L = wt.lib()
    ws = s.workspace
    args = [s.patches.data_ptr(), 2, s.waves.data_ptr(), len(w.waves), None, pos.data_ptr(), nrm.data_ptr(),
            pos.shape[0], 0, ws.data_ptr(), ws.numel(), wt.stream_handle()]
    assert L.wt_gerstner_displace(*args) == 0
    for i, v, code in ((0, None, 1), (5, pos.data_ptr() + 4, 1), (8, 0x100, 1), (10, 64, 4), (9, ws.data_ptr() + 16, 1),
                       (7, 0, 1)):
        a = list(args)
        a[i] = v
        assert L.wt_gerstner_displace(*a) == code, (i, v)
        assert L.wt_last_error()


@pytest.mark.parametrize("channels", [1, 2, 3, 4])
def test_heightmap_from_unorm8_bit_exact(wt, oracle, gpu, channels):
    """Pixels -> texels (flip on load, red/grey channel, c / 255) bit for bit,
    with a padded row stride and without the flip."""
    import ctypes as C
    import torch
    rng = np.random.default_rng(channels)
    h, w = 37, 53
    stride = w * channels + 5
    buf = rng.integers(0, 256, (h, stride), dtype=np.uint8)
    buf.reshape(-1)[:256] = np.arange(256, dtype=np.uint8)  # every code appears somewhere
    px = buf[:, :w * channels].reshape(h, w, channels)
    dev = torch.from_numpy(buf.reshape(-1).copy()).cuda()
    for flip in (1, 0):
        out = torch.empty((h, w), dtype=torch.float32, device="cuda")
        wt.check(wt.lib().wt_heightmap_from_unorm8(dev.data_ptr(), w, h, channels, stride, flip, out.data_ptr(),
                                                   wt.stream_handle()))
        torch.cuda.synchronize()
        want = oracle.heightmap_from_unorm8(px, bool(flip))
        assert np.array_equal(out.cpu().numpy().view(np.uint32), want.view(np.uint32))
    with pytest.raises(wt.WtError):
        wt.check(wt.lib().wt_heightmap_from_unorm8(dev.data_ptr(), w, h, channels, w * channels - 1, 1,
                                                   out.data_ptr(), wt.stream_handle()))


def test_png_heightmap_end_to_end(wt, oracle, gpu, tmp_path):
    """A grey PNG on disk -> device heightmap (wave_tool_gb300.png) equals
    the oracle's texels, and displaces a grid like the same texels given
    directly."""
    import sys
    from pathlib import Path
    import torch
    sys.path.insert(0, str(Path(__file__).resolve().parent))
    from test_png import encode
    from wave_tool_gb300 import png, workloads
    rng = np.random.default_rng(21)
    img = rng.integers(0, 256, (64, 96, 1))
    f = tmp_path / "hm.png"
    f.write_bytes(encode(img, 8, 0, rng))
    hm = png.load_heightmap(f, sample_scale=0.05, disp_scale=0.5, wrap=wt.WT_WRAP_MIRRORED_REPEAT)
    torch.cuda.synchronize()
    want = oracle.heightmap_from_unorm8(img.astype(np.uint8))
    assert np.array_equal(hm.texels.cpu().numpy(), want)
    w = workloads.config1()
    a = wt.Surface(w.patches, w.waves, hm).displace()[0]
    b = wt.Surface(w.patches, w.waves, wt.DeviceHeightmap(torch.from_numpy(want).cuda(), 0.05, 0.5,
                                                          wt.WT_WRAP_MIRRORED_REPEAT)).displace()[0]
    torch.cuda.synchronize()
    assert torch.equal(a, b)
