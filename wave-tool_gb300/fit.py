"""Fitting wave parameters to a target surface with the forward/adjoint pair.

`GerstnerFunction` is a torch.autograd.Function whose forward is
wt_gerstner_displace_saving (the outputs plus each vertex's wave sums, kept as
the saved activation) and whose backward is wt_gerstner_adjoint_saved (both
through the C ABI); torch only carries the tensors and the optimiser.  `fit_waves`
runs Adam on (log A, log lambda, direction angle, log Q, phase) against an
L2 height + normal loss — the adjoint-fit configuration (512 x 512 grid,
16 hidden waves, 10 % / 10 degree / 0.5 rad perturbed start, 500 steps).
No reference counterpart: the reference only animates hand-set waves.

The loss is first restricted to a growing window.  A wave whose wavelength
starts 10 % off has a phase error that grows as dk * r across the patch (tens
of radians over 100 m for a 2 m wave), so the whole-patch loss holds no descent
direction back to it and Adam shrinks its amplitude instead.  Inside a
Gaussian window a few metres wide around each patch centre the phase error is
under a radian; the window then widens geometrically, no faster than the
wavelengths converge, and the last steps use the plain loss.
"""
from __future__ import annotations

import math
import time

import numpy as np

from . import Surface, WAVE_DTYPE, WT_LAYOUT_VEC3, WT_OUT_DISPLACEMENT


def _torch():
    import torch
    return torch


# wt_wave_grad field -> wt_wave field: (A, lambda, dir_x, dir_z, Q, speed, phase)
_GRAD_TO_WAVE = (0, 1, 6, 7, 3, 5, 4)


def rank_sum(t, group=None):
    """Sum of a tensor over the ranks of `group` in rank order (bitwise the
    same on every rank); the tensor itself without a group.  Gloo groups
    exchange through host memory."""
    if group is None:
        return t
    import torch.distributed as dist
    from .sharding import allreduce_grads_fixed_order
    if dist.get_backend(group) == "gloo" and t.is_cuda:
        return allreduce_grads_fixed_order(t.cpu(), group).to(t.device)
    return allreduce_grads_fixed_order(t, group)


class GerstnerFunction:
    """apply(wave_fields, surface, flags, group=None) -> (pos, nrm);
    wave_fields is an [n_waves, 8] float32 CUDA tensor in wt_wave field
    order.  With a process group, each rank's surface holds its shard of the
    patches and the backward sums the wave gradients (wt_wave_grad) over the
    ranks in rank order, so every rank steps its optimiser with the same
    gradient."""

    _fn = None

    @classmethod
    def apply(cls, wave_fields, surface: Surface, flags: int = WT_OUT_DISPLACEMENT, group=None):
        if cls._fn is None:
            torch = _torch()

            class _F(torch.autograd.Function):
                @staticmethod
                def forward(ctx, w, surf, fl, grp):
                    surf.waves.copy_(w.detach().contiguous().view(torch.uint8).reshape(-1))
                    sums = torch.empty((surf.n_vertices, 8), dtype=torch.float32, device=w.device)
                    pos, nrm = surf.displace(flags=fl, sums=sums)
                    ctx.surf, ctx.flags, ctx.group = surf, fl, grp
                    ctx.save_for_backward(sums)
                    return pos, nrm

                @staticmethod
                def backward(ctx, gpos, gnrm):
                    surf = ctx.surf
                    gpos = gpos.contiguous() if gpos is not None else torch.zeros(
                        (surf.n_vertices, 4), device=surf.patches.device)
                    (sums,) = ctx.saved_tensors
                    g = surf.adjoint(gpos, None if gnrm is None else gnrm.contiguous(),
                                     flags=ctx.flags & WT_LAYOUT_VEC3, sums=sums)
                    g = rank_sum(g, ctx.group)
                    out = torch.zeros((surf.n_waves, 8), dtype=torch.float32, device=g.device)
                    for dst, src in enumerate(_GRAD_TO_WAVE):
                        out[:, dst] = g[:, src]
                    return out, None, None, None

            cls._fn = _F
        return cls._fn.apply(wave_fields, surface, flags, group)


def waves_to_fields(waves: np.ndarray, device="cuda"):
    torch = _torch()
    return torch.from_numpy(np.ascontiguousarray(waves).view(np.float32).reshape(-1, 8).copy()).to(device)


def window_r2(patches: np.ndarray, n_vertices: int) -> np.ndarray:
    """Squared distance (m^2) of each output vertex's grid point from its
    patch's centre, in output order (vertex out_offset + row * cols + col at
    the bilerp of the corners, water-grid.vert:87-91); 0 for vertices no patch
    writes."""
    r2 = np.zeros(n_vertices, np.float32)
    for p in patches:
        cols, rows = int(p["cols"]), int(p["rows"])
        u = np.arange(cols, dtype=np.float64) / max(cols - 1, 1)
        v = np.arange(rows, dtype=np.float64) / max(rows - 1, 1)
        bl, br, tl, tr = (p[k].astype(np.float64) for k in ("bl", "br", "tl", "tr"))
        bot = bl[None, :] + u[:, None] * (br - bl)[None, :]  # [cols, 2]
        top = tl[None, :] + u[:, None] * (tr - tl)[None, :]
        xz = bot[None, :, :] + v[:, None, None] * (top - bot)[None, :, :]  # [rows, cols, 2]
        c = 0.25 * (bl + br + tl + tr)
        o = int(p["out_offset"])
        r2[o:o + rows * cols] = ((xz - c) ** 2).sum(-1).reshape(-1)
    return r2


def fit_waves(patches: np.ndarray, target_waves: np.ndarray, start_waves: np.ndarray, steps: int = 500,
              lr: float = 1e-2, normal_weight: float = 1.0, log_every: int = 0, phase_lr: float | None = None,
              window_start: float | None = 2.5, window_steps: int | None = None, group=None,
              checkpoint: str | None = None, checkpoint_every: int = 100, stop_after: int | None = None):
    """Adam on (log A, log lambda, angle, log Q, phase) of start_waves to match
    the heights (y displacement) and normals of target_waves.  Speed is kept.

    The phase learns at phase_lr (default 10 * lr): its starting error
    includes dk * speed * t, several radians for the short waves.  With
    window_start (m) set, the per-vertex loss is weighted by
    exp(-r^2 / (2 sigma^2)) (normalised to mean 1), r the distance from the
    patch centre, sigma growing geometrically from window_start to 2.8 patch
    half-diagonals over window_steps steps (default 70 % of the steps); the
    remaining steps use the plain loss.  None: the plain loss throughout.

    With a torch.distributed process group (data parallel over patches; no
    reference counterpart), each rank fits on its LPT shard of the patches
    (sharding.shard_patches): the loss is the mean over every rank's vertices,
    its normalisers and the wave gradients are summed over the ranks in rank
    order, and the ranks step identical parameters.

    With `checkpoint` (a file path), the fit's state (step, parameters, Adam
    state, loss history) is written there every `checkpoint_every` steps and
    at the end (rank 0 writes; through a temporary file, so a crash leaves the
    previous checkpoint whole), and a fit started with an existing checkpoint
    resumes from it: the steps it had done are skipped and the rest follow
    the same schedule, so a resumed fit ends with the same parameters, bit for
    bit, as one run straight through.  No reference counterpart (the
    reference saves only screenshots, src/program.cpp:505-511).

    Returns a dict: loss_first / loss_last (the plain loss of the starting and
    the fitted waves), the training-loss history, timings and the fitted waves."""
    torch = _torch()
    dev = torch.device("cuda")
    all_patches = patches
    if group is not None:
        import torch.distributed as dist
        from .sharding import shard_patches
        patches, _ = shard_patches(patches, dist.get_world_size(group), dist.get_rank(group))
    tgt = Surface(patches, target_waves)
    pos_t, nrm_t = tgt.displace(flags=WT_OUT_DISPLACEMENT)
    y_t = pos_t[:, 1].clone()
    n_t = nrm_t[:, :3].clone()
    if group is None:
        n_all = float(y_t.numel())
        y_scale = float(y_t.var())
    else:
        # vertex count and (unbiased) variance of the target heights over
        # every rank's vertices
        yd = y_t.double()
        mom = rank_sum(torch.stack([torch.tensor(float(y_t.numel()), dtype=torch.float64, device=dev), yd.sum(),
                                    (yd * yd).sum()]), group)
        n_all = float(mom[0])
        y_scale = float((mom[2] - mom[1] * mom[1] / n_all) / max(n_all - 1.0, 1.0))
    surf = Surface(patches, start_waves)
    f0 = waves_to_fields(start_waves, dev)
    logA = torch.log(f0[:, 0].clamp_min(1e-12)).clone().requires_grad_(True)
    logL = torch.log(f0[:, 1]).clone().requires_grad_(True)
    ang = torch.atan2(f0[:, 3], f0[:, 2]).clone().requires_grad_(True)
    logQ = torch.log(f0[:, 4].clamp_min(1e-12)).clone().requires_grad_(True)
    ph = f0[:, 6].clone().requires_grad_(True)
    speed = f0[:, 5].clone()
    opt = torch.optim.Adam([{"params": [logA, logL, ang, logQ], "lr": lr},
                            {"params": [ph], "lr": 10.0 * lr if phase_lr is None else phase_lr}])
    if window_start is not None:
        r2 = torch.from_numpy(window_r2(patches, surf.n_vertices)).to(dev)
        half_diag = max(0.5 * math.hypot(float(p["tr"][0] - p["bl"][0]), float(p["tr"][1] - p["bl"][1]))
                        for p in all_patches)
        sigma_end = max(2.8 * half_diag, window_start)
        wsteps = max(1, int(round(0.7 * steps)) if window_steps is None else window_steps)

    def fields_now():
        return torch.stack([logA.exp(), logL.exp(), ang.cos(), ang.sin(), logQ.exp(), speed, ph,
                            torch.zeros_like(ph)], 1)

    def plain_loss():
        with torch.no_grad():
            pos, nrm = GerstnerFunction.apply(fields_now(), surf, WT_OUT_DISPLACEMENT)
            if group is None:
                ey = ((pos[:, 1] - y_t) ** 2).mean() / y_scale
                return float(ey + normal_weight * ((nrm[:, :3] - n_t) ** 2).sum(1).mean())
            e = ((pos[:, 1] - y_t) ** 2).double().sum() / y_scale + \
                normal_weight * ((nrm[:, :3] - n_t) ** 2).double().sum()
            return float(rank_sum(e.reshape(1), group)[0]) / n_all

    loss_first = plain_loss()
    hist = []
    it0 = 0
    params = [logA, logL, ang, logQ, ph]
    if checkpoint is not None:
        import os
        if os.path.exists(checkpoint):
            ck = torch.load(checkpoint, map_location=dev, weights_only=False)
            if ck["steps"] != steps or ck["n_waves"] != len(start_waves):
                raise ValueError(f"checkpoint {checkpoint} is of another fit ({ck['steps']} steps, "
                                 f"{ck['n_waves']} waves)")
            with torch.no_grad():
                for t_, v in zip(params, ck["params"]):
                    t_.copy_(v)
            opt.load_state_dict(ck["opt"])
            it0 = ck["step"]
            hist = list(ck["history"])
            loss_first = ck["loss_first"]

    def save(step):
        if checkpoint is None:
            return
        if group is not None:
            import torch.distributed as dist
            if dist.get_rank(group) != 0:
                return
        import os
        tmp = checkpoint + ".tmp"
        torch.save({"step": step, "steps": steps, "n_waves": len(start_waves),
                    "params": [t_.detach().clone() for t_ in params], "opt": opt.state_dict(),
                    "history": [(i, float(l)) for i, l in hist], "loss_first": loss_first}, tmp)
        os.replace(tmp, checkpoint)

    torch.cuda.synchronize()
    t0 = time.perf_counter()
    it_end = steps if stop_after is None else min(steps, it0 + stop_after)
    for it in range(it0, it_end):
        opt.zero_grad(set_to_none=True)
        pos, nrm = GerstnerFunction.apply(fields_now(), surf, WT_OUT_DISPLACEMENT, group)
        ey = (pos[:, 1] - y_t) ** 2 / y_scale
        en = ((nrm[:, :3] - n_t) ** 2).sum(1)
        if window_start is not None and it < wsteps:
            sigma = window_start * (sigma_end / window_start) ** (it / wsteps)
            wgt = torch.exp(r2 * (-0.5 / (sigma * sigma)))
            if group is None:
                wgt = wgt / wgt.mean()
                loss = (wgt * (ey + normal_weight * en)).mean()
            else:
                wsum = rank_sum(wgt.sum().detach().reshape(1), group)[0]
                loss = (wgt * (ey + normal_weight * en)).sum() / wsum
        elif group is None:
            loss = (ey + normal_weight * en).mean()
        else:
            # this rank's share of the mean over every rank's vertices; the
            # backward sums the shares' wave gradients
            loss = (ey + normal_weight * en).sum() / n_all
        loss.backward()
        opt.step()
        if log_every and it % log_every == 0:
            hist.append((it, float(loss)))
        elif not log_every:
            hist.append((it, loss.detach()))
        if checkpoint is not None and (it + 1) % checkpoint_every == 0:
            save(it + 1)
    if it_end == steps or it_end % checkpoint_every != 0:
        save(it_end)
    torch.cuda.synchronize()
    dt = time.perf_counter() - t0
    hist = [(i, float(l)) for i, l in hist]
    loss_last = plain_loss()
    fitted = np.zeros(len(start_waves), WAVE_DTYPE)
    with torch.no_grad():
        fields = fields_now().cpu().numpy()
    fitted.view(np.float32).reshape(-1, 8)[:] = fields
    return {"loss_first": loss_first, "loss_last": loss_last, "history": hist, "seconds": dt,
            "ms_per_step": 1e3 * dt / max(it_end - it0, 1), "fitted": fitted, "resumed_from": it0,
            "steps_done": it_end}


def parameter_errors(fitted: np.ndarray, target: np.ndarray) -> dict:
    """Relative errors of A, lambda, Q; angle error (deg); wrapped phase error (rad)."""
    ang_f = np.arctan2(fitted["dir_z"], fitted["dir_x"])
    ang_t = np.arctan2(target["dir_z"], target["dir_x"])
    dph = np.angle(np.exp(1j * (fitted["phase"].astype(np.float64) - target["phase"])))
    return {
        "amplitude_rel": float(np.median(np.abs(fitted["amplitude"] / target["amplitude"] - 1))),
        "wavelength_rel": float(np.median(np.abs(fitted["wavelength"] / target["wavelength"] - 1))),
        "steepness_rel": float(np.median(np.abs(fitted["steepness_q"] / target["steepness_q"] - 1))),
        "direction_deg": float(np.median(np.degrees(np.abs(np.angle(np.exp(1j * (ang_f - ang_t))))))),
        "phase_rad": float(np.median(np.abs(dph))),
    }


__all__ = ["GerstnerFunction", "fit_waves", "waves_to_fields", "parameter_errors", "window_r2", "rank_sum"]
