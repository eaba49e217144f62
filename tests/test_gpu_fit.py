"""The torch binding (forward = wt_gerstner_displace, backward =
wt_gerstner_adjoint), the Adam fit of the adjoint-fit configuration, and the
CUDA-graph replay of a batched launch."""
from __future__ import annotations

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def test_autograd_binding_matches_f64_gradient(wt, oracle, gpu):
    import torch
    from wave_tool_gb300 import fit, workloads
    w = workloads.small_random(4, n_patches=2, side_range=(30, 120), n_waves_range=(3, 12), heightmap=False)
    surf = wt.Surface(w.patches, w.waves)
    fields = fit.waves_to_fields(w.waves).requires_grad_(True)
    pos, nrm = fit.GerstnerFunction.apply(fields, surf, wt.WT_OUT_DISPLACEMENT)
    gen = torch.Generator().manual_seed(0)
    gp = torch.randn(pos.shape, generator=gen).cuda()
    gn = torch.randn(nrm.shape, generator=gen).cuda()
    loss = (pos * gp).sum() + (nrm * gn).sum()
    loss.backward()
    g64 = oracle.adjoint_f64(w.patches, w.waves, gp.cpu().numpy(), gn.cpu().numpy())
    got = fields.grad.cpu().numpy().astype(np.float64)
    # wt_wave field order (A, lambda, dx, dz, Q, speed, phase) vs the oracle's wt_wave_grad order
    for dst, src in enumerate((0, 1, 6, 7, 3, 5, 4)):
        scale = np.abs(g64[:, src]).max()
        assert np.abs(got[:, dst] - g64[:, src]).max() <= 1e-4 * scale, dst
    assert np.all(got[:, 7] == 0)


def test_adam_fit_reduces_loss(wt, gpu):
    """A shortened run of the adjoint-fit configuration (512^2, 16 waves)."""
    from wave_tool_gb300 import fit, workloads
    target, start = workloads.config4()
    r = fit.fit_waves(target.patches, target.waves, start, steps=60, lr=1e-2)
    assert np.isfinite(r["loss_last"])
    assert r["loss_last"] < 0.2 * r["loss_first"], {k: r[k] for k in ("loss_first", "loss_last")}


@pytest.mark.parametrize("seed", [3, 10, 12])
def test_adam_fit_recovers_the_hidden_waves(wt, gpu, seed):
    """The full adjoint-fit configuration (seed 3) and two other draws of it:
    500 Adam steps from the perturbed start (A, lambda, Q +-10 %, direction
    +-10 degrees, phase +-0.5 rad) recover the 16 hidden waves (median errors;
    the plain loss falls from above 1 to about 1e-4)."""
    from wave_tool_gb300 import fit, workloads
    target, start = workloads.config4(seed)
    r = fit.fit_waves(target.patches, target.waves, start, steps=500, lr=1e-2)
    e = fit.parameter_errors(r["fitted"], target.waves)
    assert r["loss_last"] < 2e-3 and r["loss_first"] > 0.5, (r["loss_first"], r["loss_last"])
    assert e["amplitude_rel"] < 1e-2 and e["wavelength_rel"] < 1e-3 and e["steepness_rel"] < 5e-2, e
    assert e["direction_deg"] < 0.1 and e["phase_rad"] < 1e-2, e


def test_cuda_graph_replay_equals_eager(wt, gpu):
    """The three launches of one batched call, captured once and replayed,
    give the eager result bit for bit (and again after the inputs change)."""
    import torch
    from wave_tool_gb300 import workloads
    w = workloads.config3(n_patches=24, seed=5)
    surf = wt.Surface(w.patches, w.waves, wt.heightmap_from(w.heightmap))
    pos, nrm = surf.alloc_outputs()
    surf.displace(pos, nrm)  # first call does the per-device set-up
    torch.cuda.synchronize()
    ref_p, ref_n = pos.clone(), nrm.clone()
    s = torch.cuda.Stream()
    g = torch.cuda.CUDAGraph()
    with torch.cuda.graph(g, stream=s):
        surf.displace(pos, nrm, stream=s)
    pos.zero_()
    g.replay()
    torch.cuda.synchronize()
    assert torch.equal(pos, ref_p) and torch.equal(nrm, ref_n)
    # new times through the same graph (device patch table updated in place)
    p2 = w.patches.copy()
    p2["time_s"] += 1.5
    surf.patches.copy_(wt.to_device(p2))
    g.replay()
    torch.cuda.synchronize()
    s2 = wt.Surface(p2, w.waves, surf.heightmap)
    ep, en = s2.displace()
    torch.cuda.synchronize()
    assert torch.equal(pos, ep) and torch.equal(nrm, en)


def test_fit_resumes_from_a_checkpoint_bit_for_bit(wt, gpu, tmp_path):
    """A fit stopped after 25 of 50 steps and resumed from its checkpoint
    ends with the parameters and loss history of the same fit run straight
    through (every kernel and the optimiser are deterministic)."""
    from wave_tool_gb300 import fit, workloads
    target, start = workloads.config4()
    straight = fit.fit_waves(target.patches, target.waves, start, steps=50, lr=1e-2)
    ck = str(tmp_path / "fit.ckpt")
    first = fit.fit_waves(target.patches, target.waves, start, steps=50, lr=1e-2, checkpoint=ck,
                          checkpoint_every=10, stop_after=25)
    assert first["steps_done"] == 25 and first["resumed_from"] == 0
    resumed = fit.fit_waves(target.patches, target.waves, start, steps=50, lr=1e-2, checkpoint=ck,
                            checkpoint_every=10)
    assert resumed["resumed_from"] == 25 and resumed["steps_done"] == 50
    assert np.array_equal(resumed["fitted"].view(np.uint32), straight["fitted"].view(np.uint32))
    assert resumed["history"] == straight["history"]
    assert resumed["loss_last"] == straight["loss_last"]
