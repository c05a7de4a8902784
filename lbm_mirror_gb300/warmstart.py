"""Learned warm start of batched D2Q9 channels (no counterpart in
keldu/lbm_mirror, whose drivers always start from rest equilibrium,
examples/stdkr_2d_bgk/init.hpp:16-54).

Pipeline, all on one GPU:
  1. steady states: seeded channels of one size run in the batched runner
     (kel_batch_run_until) from rest until the relative L2 change of u over
     `check_every` steps is below `tol`, in shifted FP32 arithmetic (with f
     itself in FP32 the rounding noise of slow channels stalls above 1e-6);
  2. training: the conv U-Net (kel_unet_*, bf16 tensor-core convolutions,
     FP32 accumulate, Adam on FP32 master weights) maps the obstacle mask,
     u_max and tau planes to the normalised steady field
     (u_x / u_max, u_y / u_max, (rho - 1) / (u_max * rho_scale));
  3. warm start: inference on new geometries, then kel_batch_warm_start
     builds f_eq + f_neq (Chapman-Enskog) populations from the prediction and
     the same runner continues to the same residual.  Convergence is tested
     as in the plain run from rest: a warm-started channel stops by the same
     residual test.

Device memory is held in torch tensors (plumbing only); every kernel on the
path is this library's.
"""
from __future__ import annotations

import math
import time
from dataclasses import dataclass, field

import numpy as np

from . import capi as K
from .lattice import Batch, UNet
from .workloads import batch_channels, channel_program


def _torch():
    import torch
    if not torch.cuda.is_available():
        raise RuntimeError("the warm-start pipeline needs a CUDA device")
    return torch


def fixed_size_channels(n, seed, nx=256, ny=64):
    """n seeded channels of one size (nx x ny): obstacles, u_max and tau as
    the batched-channel workload draws them."""
    return batch_channels(n=n, seed=seed, nx_range=(nx, nx), ny_range=(ny, ny))


def channel_inputs(channels):
    """Host arrays of the network inputs: mask (n, ny, nx) uint8 (1 = wall or
    obstacle), u_max (n,) and tau (n,) float32."""
    ny, nx = channels[0]["ny"], channels[0]["nx"]
    mask = np.stack([(np.asarray(c["flags"]).reshape(ny, nx) == 1).astype(np.uint8) for c in channels])
    u_max = np.array([c["u_max"] for c in channels], dtype=np.float32)
    tau = np.array([c["tau"] for c in channels], dtype=np.float32)
    return mask, u_max, tau


@dataclass
class SteadyStates:
    """Steady fields of a set of channels: rho (n, ny, nx), u (n, ny, nx, 2),
    steps to convergence and the last residual per channel, wall seconds."""
    channels: list
    rho: np.ndarray
    u: np.ndarray
    steps: np.ndarray
    residual: np.ndarray
    seconds: float
    tol: float = 1e-6

    @property
    def converged(self):
        """Reached the residual with finite fields (False for diverged runs)."""
        finite = np.isfinite(self.rho).all(axis=(1, 2)) & np.isfinite(self.u).all(axis=(1, 2, 3))
        return (self.residual < self.tol) & finite


def solve(channels, tol=1e-6, check_every=1000, max_steps=600_000, tile=128, chunk=1024, arithmetic=K.KEL_ARITH_SHIFTED):
    """Run the channels from rest to the residual `tol` in batches of `chunk`
    channels; returns SteadyStates (fields downloaded to the host)."""
    n = len(channels)
    ny, nx = channels[0]["ny"], channels[0]["nx"]
    rho = np.empty((n, ny, nx), np.float32)
    u = np.empty((n, ny, nx, 2), np.float32)
    steps = np.empty(n, np.uint64)
    res = np.empty(n, np.float64)
    t0 = time.perf_counter()
    for a in range(0, n, chunk):
        part = channels[a:a + chunk]
        b = Batch(part, channel_program(0.8, arithmetic), tile=tile)
        s, r = b.run_until(tol=tol, check_every=check_every, max_steps=max_steps)
        steps[a:a + len(part)] = s
        res[a:a + len(part)] = r
        for k in range(len(part)):
            rr, uu = b.macros(k)
            rho[a + k] = rr.reshape(ny, nx)
            u[a + k] = uu.reshape(ny, nx, 2)
        b.close()
    return SteadyStates(channels, rho, u, steps, res, time.perf_counter() - t0, tol)


def steady_subset(states: SteadyStates):
    """The channels that reached the residual (unsteady or diverged ones are
    no steady states and are left out of training)."""
    k = np.flatnonzero(states.converged)
    return SteadyStates([states.channels[i] for i in k], states.rho[k], states.u[k], states.steps[k],
                        states.residual[k], states.seconds, states.tol)


@dataclass
class WarmStartNet:
    """The trained U-Net plus the density normalisation it was trained with:
    rho_norm "global": rho - 1 = target x u_max x rho_scale;
    rho_norm "lubrication": rho - 1 = target x rho_scale x the channel's
    lubrication pressure drop (lubrication_drho)."""
    net: UNet
    rho_scale: float
    history: list = field(default_factory=list)
    rho_norm: str = "global"

    @property
    def shape(self):
        return self.net.shape


class WarmStartEnsemble:
    """Networks trained on the same steady states with different seeds; the
    prediction is the mean of theirs (the members share the normalisation:
    rho_norm and rho_scale come from the training data).  Independent
    trainings err differently, so the mean is nearer the steady state than a
    typical member, and the slowest warm-started channel varies less."""

    def __init__(self, members):
        members = list(members)
        if not members:
            raise ValueError("empty ensemble")
        m0 = members[0]
        for m in members[1:]:
            if m.rho_norm != m0.rho_norm or m.rho_scale != m0.rho_scale or m.shape != m0.shape:
                raise ValueError("ensemble members differ in normalisation or shape")
        self.members = members
        self.rho_norm, self.rho_scale = m0.rho_norm, m0.rho_scale

    @property
    def shape(self):
        return self.members[0].shape


def train_ensemble(states: SteadyStates, seeds=(1, 2), **kw):
    """train() once per seed; a WarmStartEnsemble of the results."""
    return WarmStartEnsemble([train(states, seed=s, **kw) for s in seeds])


def _gap_h3(fluid):
    """Per (channel, column): sum over the column's vertical runs of fluid
    cells of the run length cubed.  fluid: (n, ny, nx) bool numpy array or
    torch tensor."""
    run = fluid[:, 0] * 0.0
    s3 = fluid[:, 0] * 0.0
    for y in range(fluid.shape[1]):
        f = fluid[:, y] * 1.0
        s3 = s3 + run ** 3 * (1.0 - f)
        run = (run + 1.0) * f
    return s3 + run ** 3


def lubrication_drho(mask, u_max, tau):
    """Pressure drop (as rho) from inlet to outlet that lubrication theory
    gives for each channel: each column's Poiseuille gradient is
    dp/dx = 12 nu Q / sum h^3 (gaps of height h, flux Q = 2/3 u_max (ny - 2)
    of the parabolic inlet), p = rho / 3, so
    drho = 36 nu Q sum_x 1 / sum h^3.  Works on numpy arrays or torch tensors
    (mask (n, ny, nx), 1 = solid; u_max and tau (n,))."""
    fluid = mask == 0
    ny = mask.shape[1]
    S0 = (1.0 / _gap_h3(fluid).clip(min=1.0)).sum(1)
    nu = (tau - 0.5) / 3.0
    Q = 2.0 / 3.0 * u_max * (ny - 2)
    return 36.0 * nu * Q * S0


def targets(states: SteadyStates, rho_scale=None, rho_target_rms=0.25, rho_norm="global"):
    """Normalised training targets (n, ny, nx, 3) float32 and the density
    scale.  rho_norm "global": (rho - 1) / u_max over non-wall cells is scaled
    to RMS rho_target_rms (unless rho_scale is given), which weights the
    density in the squared-error loss below the velocity (u / u_max is of
    order 1).  rho_norm "lubrication": (rho - 1) over each channel's
    lubrication pressure drop (about 1 at the inlet, 0 at the outlet), times
    1 / rho_scale, rho_scale set the same way."""
    mask, u_max, tau = channel_inputs(states.channels)
    um = u_max[:, None, None]
    if rho_norm == "lubrication":
        drho = (states.rho - 1.0) / lubrication_drho(mask, u_max, tau)[:, None, None]
    else:
        drho = (states.rho - 1.0) / um
    if rho_scale is None:
        fluid = mask == 0
        rho_scale = float(np.sqrt(np.mean(drho[fluid] ** 2)) / rho_target_rms) or 1.0
    t = np.empty(states.u.shape[:3] + (3,), np.float32)
    t[..., 0] = states.u[..., 0] / um
    t[..., 1] = states.u[..., 1] / um
    t[..., 2] = drho / rho_scale
    return t, rho_scale


def rho_denominator(model, d_mask, d_umax, d_tau):
    """Per-channel factor turning the network's density output into rho - 1
    (torch tensor on the inputs' device)."""
    torch = _torch()
    um = d_umax.to(torch.float32)
    if model.rho_norm == "lubrication":
        return (lubrication_drho(d_mask, um, d_tau.to(torch.float32)) * model.rho_scale).to(torch.float32)
    return um * model.rho_scale


def train(states: SteadyStates, epochs=30, batch=32, lr=2e-3, lr_min_frac=0.02, warmup=100, seed=1,
          widths=(32, 64, 128, 128), log_every=0, rho_target_rms=0.25, residual=False, weight_by_steps=False,
          rho_norm="global", rho_residual=False, flip=False):
    """Train the U-Net on the steady states with Adam (cosine schedule).
    rho_target_rms sets the weight of the density in the loss (see targets).
    With weight_by_steps the minibatches draw channels with probability
    proportional to the steps their run from rest took (the slow channels
    dominate the time to steady state), instead of a permutation per epoch.
    With `residual` the u_x output is the correction to the local Poiseuille
    estimate the input planes carry (2 x plane 9 = u_x / u_max of the column's
    gap, its flux share by h^3): kel_unet_set_residual(0, 9, 2).  rho_norm
    selects the density target (see targets); with rho_residual (lubrication
    norm) the density output is the correction to the lubrication pressure
    plane 10 (scaled to the target): kel_unet_set_residual(2, 10, 1 / rho_scale).
    With flip, a random half of every minibatch is the y-mirror image of its
    channels (mask and targets mirrored, u_y negated; the input planes are
    built from the mirrored mask): a channel and its mirror image (walls,
    parabolic inlet and all) have mirrored steady flows, so this doubles the
    distinct samples the network sees.
    Returns a WarmStartNet; its history holds (step, loss) pairs."""
    torch = _torch()
    ny, nx = states.rho.shape[1:]
    mask, u_max, tau = channel_inputs(states.channels)
    tgt, rho_scale = targets(states, rho_target_rms=rho_target_rms, rho_norm=rho_norm)
    dev = torch.device("cuda")
    d_mask = torch.from_numpy(mask).to(dev)
    d_umax = torch.from_numpy(u_max).to(dev)
    d_tau = torch.from_numpy(tau).to(dev)
    d_tgt = torch.from_numpy(tgt).to(dev)
    n = mask.shape[0]
    net = UNet(height=ny, width=nx, widths=widths, out_channels=3, max_batch=batch, seed=seed)
    if residual:
        net.set_residual(0, 9, 2.0)
    if rho_residual:
        if rho_norm != "lubrication":
            raise ValueError("rho_residual goes with rho_norm='lubrication'")
        net.set_residual(2, 10, 1.0 / rho_scale)
    model = WarmStartNet(net, rho_scale, rho_norm=rho_norm)
    steps_per_epoch = n // batch
    total = max(1, epochs * steps_per_epoch)
    gen = torch.Generator(device=dev)
    gen.manual_seed(seed)
    step = 0
    pw = None
    if weight_by_steps:
        w = np.asarray(states.steps, dtype=np.float64)
        pw = torch.from_numpy(w / w.sum()).to(dev)
    for _ in range(epochs):
        if pw is None:
            perm = torch.randperm(n, device=dev, generator=gen)
        else:
            perm = torch.multinomial(pw, n, replacement=True, generator=gen)
        for i in range(steps_per_epoch):
            idx = perm[i * batch:(i + 1) * batch]
            mb_mask = d_mask.index_select(0, idx).contiguous()
            mb_umax = d_umax.index_select(0, idx).contiguous()
            mb_tau = d_tau.index_select(0, idx).contiguous()
            mb_tgt = d_tgt.index_select(0, idx).contiguous()
            if flip:
                f = torch.rand(batch, device=dev, generator=gen) < 0.5
                mt = mb_tgt.flip(1)
                mt[..., 1] = -mt[..., 1]
                mb_mask = torch.where(f[:, None, None], mb_mask.flip(1), mb_mask).contiguous()
                mb_tgt = torch.where(f[:, None, None, None], mt, mb_tgt).contiguous()
            torch.cuda.synchronize()
            net.make_input(mb_mask.data_ptr(), mb_umax.data_ptr(), mb_tau.data_ptr(), batch)
            if step < warmup:
                rate = lr * (step + 1) / warmup
            else:
                q = (step - warmup) / max(1, total - warmup)
                rate = lr * (lr_min_frac + (1 - lr_min_frac) * 0.5 * (1 + math.cos(math.pi * q)))
            # forward + backward + Adam, a captured graph from the second step on;
            # the loss is read back only when it is logged
            net.train_step(mb_tgt.data_ptr(), batch, lr=rate)
            step += 1
            if not log_every or step % log_every == 0:
                model.history.append((step, net.last_loss()))
    net.synchronize()
    return model


def _predict_once(model, d_mask, d_umax, d_tau):
    if isinstance(model, WarmStartEnsemble):
        out = _predict_once(model.members[0], d_mask, d_umax, d_tau)
        for m in model.members[1:]:
            out += _predict_once(m, d_mask, d_umax, d_tau)
        return out * (1.0 / len(model.members))
    torch = _torch()
    n = d_mask.shape[0]
    ny, nx, oc = model.shape
    out = torch.empty((n, ny, nx, oc), dtype=torch.float32, device=d_mask.device)
    mb = model.net.max_batch
    torch.cuda.synchronize()
    for a in range(0, n, mb):
        k = min(mb, n - a)
        model.net.make_input(d_mask[a:].data_ptr(), d_umax[a:].data_ptr(), d_tau[a:].data_ptr(), k)
        model.net.forward(k, out[a:].data_ptr())
    model.net.synchronize()
    return out


def predict(model: WarmStartNet, d_mask, d_umax, d_tau, mirror=False):
    """Normalised prediction (n, ny, nx, 3) float32 on the device for device
    inputs (mask uint8 (n, ny, nx), u_max and tau float32 (n,)); for a
    WarmStartEnsemble the mean of its members' predictions.  With mirror,
    the mean of the prediction and the mirror image of the prediction for the
    y-mirrored channel (u_y negated): a channel and its mirror image, walls,
    parabolic inlet and all, have mirrored flows, so the average keeps the
    exact symmetry and halves the part of the error that breaks it."""
    out = _predict_once(model, d_mask, d_umax, d_tau)
    if not mirror:
        return out
    m = _predict_once(model, d_mask.flip(1).contiguous(), d_umax, d_tau).flip(1)
    m[..., 1] = -m[..., 1]
    return 0.5 * (out + m)


def warm_start(batch: Batch, model: WarmStartNet, d_mask, d_umax, d_tau, with_neq=True, rho_from_net=True,
               refine=0, keep_rho=False, mirror=False):
    """Inference for every channel of `batch` (all of the network's size,
    in channel order) and the populations built from it.  With
    rho_from_net False the density starts at 1 (only u is predicted).  With
    refine > 0, that many refinement passes (kel_batch_warm_refine) follow.
    mirror: see predict."""
    torch = _torch()
    pred = predict(model, d_mask, d_umax, d_tau, mirror)
    n = pred.shape[0]
    um = d_umax.to(torch.float32)
    rs = rho_denominator(model, d_mask, d_umax, d_tau) if rho_from_net else torch.zeros_like(um)
    scale = torch.stack([um, um, rs], dim=1).contiguous()
    offset = torch.zeros((n, 3), dtype=torch.float32, device=pred.device)
    offset[:, 2] = 1.0
    torch.cuda.synchronize()
    ny, nx, oc = model.shape
    batch.warm_start(0, n, pred.data_ptr(), ny * nx * oc, scale.data_ptr(), offset.data_ptr(), with_neq)
    if refine:
        batch.warm_refine(0, n, pred.data_ptr(), ny * nx * oc, scale.data_ptr(), offset.data_ptr(), refine, keep_rho)
    return pred


def model_init(model: WarmStartNet, with_neq=True, rho_from_net=True, refine=0, keep_rho=False, mirror=False):
    """Initialiser for time_to_steady: the network's prediction."""
    def init(batch, d_mask, d_umax, d_tau):
        return warm_start(batch, model, d_mask, d_umax, d_tau, with_neq, rho_from_net, refine, keep_rho, mirror)
    return init


def field_init(fields, with_neq=True, refine=0, keep_rho=False):
    """Initialiser for time_to_steady from given physical fields (n, ny, nx, 3)
    = (u_x, u_y, rho) per cell, e.g. a known steady state (diagnostics)."""
    def init(batch, d_mask, d_umax, d_tau):
        torch = _torch()
        n = fields.shape[0]
        d = torch.from_numpy(np.ascontiguousarray(fields, dtype=np.float32)).cuda()
        one = torch.ones((n, 3), dtype=torch.float32, device="cuda")
        zero = torch.zeros((n, 3), dtype=torch.float32, device="cuda")
        torch.cuda.synchronize()
        batch.warm_start(0, n, d.data_ptr(), d[0].numel(), one.data_ptr(), zero.data_ptr(), with_neq)
        if refine:
            batch.warm_refine(0, n, d.data_ptr(), d[0].numel(), one.data_ptr(), zero.data_ptr(), refine, keep_rho)
        batch.synchronize()
        return d
    return init


def _rel_l2(a, b):
    d = float(np.sqrt(np.sum((a - b) ** 2)))
    r = float(np.sqrt(np.sum(b ** 2)))
    return d / r if r > 0 else d


@dataclass
class SteadyRun:
    """One timed run: wall seconds, steps and last residual per channel, the
    final u (n, ny, nx, 2) and rho (n, ny, nx), the initialiser's output (or
    None) and how many channels fell back to a run from rest."""
    seconds: float
    steps: np.ndarray
    residual: np.ndarray
    u: np.ndarray
    rho: np.ndarray
    pred: np.ndarray | None
    fell_back: int = 0
    init_seconds: float = 0.0


def time_to_steady(channels, init=None, tol=1e-6, check_every=1000, max_steps=600_000, tile=128,
                   arithmetic=K.KEL_ARITH_SHIFTED):
    """One batched run of `channels` to the residual `tol`, from rest (init
    None) or from init(batch, d_mask, d_umax, d_tau) (model_init /
    field_init).  The timed region holds the initialiser (inference and
    population reconstruction) and every sweep; the batch set-up (flags and
    the rest state) is outside it for both.  Returns a SteadyRun."""
    torch = _torch()
    ny, nx = channels[0]["ny"], channels[0]["nx"]
    b = Batch(channels, channel_program(0.8, arithmetic), tile=tile)
    mask, u_max, tau = channel_inputs(channels)
    dev = torch.device("cuda")
    d_mask = torch.from_numpy(mask).to(dev)
    d_umax = torch.from_numpy(u_max).to(dev)
    d_tau = torch.from_numpy(tau).to(dev)
    b.synchronize()
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    pred = None
    if init is not None:
        pred = init(b, d_mask, d_umax, d_tau)
        b.synchronize()
    t_init = time.perf_counter() - t0
    steps, res = b.run_until(tol=tol, check_every=check_every, max_steps=max_steps)
    u = np.empty((len(channels), ny, nx, 2), np.float32)
    rho = np.empty((len(channels), ny, nx), np.float32)
    fell_back = np.zeros(len(channels), bool)
    if init is not None:
        # the plain run from rest is the fallback: a warm-started channel
        # that diverged (NaN / inf residual) or ended above the residual (it
        # stalled until max_steps) is run again from rest, in the timed
        # region, its steps added to those it spent
        bad = np.flatnonzero(~(res < tol))
        if len(bad):
            fb = Batch([channels[k] for k in bad], channel_program(0.8, arithmetic), tile=tile)
            s2, r2 = fb.run_until(tol=tol, check_every=check_every, max_steps=max_steps)
            for j, k in enumerate(bad):
                steps[k] += s2[j]
                res[k] = r2[j]
                r_, uu = fb.macros(j)
                u[k] = uu.reshape(ny, nx, 2)
                rho[k] = r_.reshape(ny, nx)
            fb.close()
            fell_back[bad] = True
    seconds = time.perf_counter() - t0
    for k in range(len(channels)):
        if fell_back[k]:
            continue
        r, uu = b.macros(k)
        u[k] = uu.reshape(ny, nx, 2)
        rho[k] = r.reshape(ny, nx)
    b.close()
    pred_np = pred.cpu().numpy() if pred is not None else None
    return SteadyRun(seconds, steps, res, u, rho, pred_np, int(fell_back.sum()), t_init)


def evaluate(model: WarmStartNet, channels, tol=1e-6, check_every=1000, max_steps=600_000, tile=128,
             with_neq=True, variants=False, mirror=False):
    """Plain (rest) vs warm-started runs of the same channels.  Channels whose
    run from rest does not reach `tol` within max_steps (unsteady flow: vortex
    shedding behind an obstacle; or diverged) have no time to steady state;
    they are counted and left out, and both arms are timed on the rest.
    Returns a dict with wall seconds, steps per channel, the final-field
    error of the warm run against the plain run and the prediction's own
    error.  With variants, also the mean steps from the plain run's own
    steady state (the floor any prediction can reach), from the network's
    u with rho = 1, and without the non-equilibrium part."""
    # untimed warm-up of both arms (first launches, device allocations)
    warm_ch = channels[:min(8, len(channels))]
    time_to_steady(warm_ch, None, tol, check_every, min(max_steps, 2 * check_every), tile)
    time_to_steady(warm_ch, model_init(model, with_neq, mirror=mirror), tol, check_every,
                   min(max_steps, 2 * check_every), tile)
    pr = time_to_steady(channels, None, tol, check_every, max_steps, tile)
    ok = np.flatnonzero(pr.residual < tol)
    excluded = len(channels) - len(ok)
    if excluded:
        channels = [channels[k] for k in ok]
        pr = time_to_steady(channels, None, tol, check_every, max_steps, tile)
    t_plain, s_plain, r_plain, u_plain, rho_plain = pr.seconds, pr.steps, pr.residual, pr.u, pr.rho
    wr = time_to_steady(channels, model_init(model, with_neq, mirror=mirror), tol, check_every, max_steps, tile)
    t_warm, s_warm, r_warm, u_warm, pred, fallbacks = wr.seconds, wr.steps, wr.residual, wr.u, wr.pred, wr.fell_back
    mask, u_max, _ = channel_inputs(channels)
    final_err = np.array([_rel_l2(u_warm[k], u_plain[k]) for k in range(len(channels))])
    pred_u = pred[..., :2] * u_max[:, None, None, None]
    pred_u[mask == 1] = 0.0
    pred_err = np.array([_rel_l2(pred_u[k], u_plain[k]) for k in range(len(channels))])
    if model.rho_norm == "lubrication":
        _, _, tau_h = channel_inputs(channels)
        den = lubrication_drho(mask, u_max, tau_h) * model.rho_scale
    else:
        den = u_max * model.rho_scale
    pred_rho = pred[..., 2] * den[:, None, None] + 1.0
    fl = mask == 0
    rho_err = np.array([_rel_l2(pred_rho[k][fl[k]] - 1, rho_plain[k][fl[k]] - 1) for k in range(len(channels))])
    nonfinite = dict(pred=int(sum(not np.isfinite(pred[k][fl[k]]).all() for k in range(len(channels)))),
                     u_warm=int(sum(not np.isfinite(u_warm[k]).all() for k in range(len(channels)))),
                     u_plain=int(sum(not np.isfinite(u_plain[k]).all() for k in range(len(channels)))))
    out = dict(
        channels=len(channels), excluded_unsteady=excluded, tol=tol, check_every=check_every,
        plain_seconds=t_plain, warm_seconds=t_warm, speedup=t_plain / t_warm,
        plain_steps_mean=float(np.mean(s_plain)), warm_steps_mean=float(np.mean(s_warm)),
        plain_steps_max=int(np.max(s_plain)), warm_steps_max=int(np.max(s_warm)),
        plain_unconverged=int(np.sum(~(r_plain < tol))), warm_unconverged=int(np.sum(~(r_warm < tol))),
        final_u_rel_l2_mean=float(np.nanmean(final_err)), final_u_rel_l2_max=float(np.nanmax(final_err)),
        prediction_u_rel_l2_mean=float(np.nanmean(pred_err)), prediction_u_rel_l2_max=float(np.nanmax(pred_err)),
        prediction_drho_rel_l2_mean=float(np.nanmean(rho_err)), nonfinite_channels=nonfinite,
        warm_fallbacks_to_rest=fallbacks, warm_init_seconds=wr.init_seconds,
        steps_plain=s_plain, steps_warm=s_warm,
    )
    if variants:
        exact = np.concatenate([u_plain, rho_plain[..., None]], axis=-1)
        s_ex = time_to_steady(channels, field_init(exact, with_neq), tol, check_every, max_steps, tile).steps
        s_r1 = time_to_steady(channels, model_init(model, with_neq, rho_from_net=False), tol, check_every,
                              max_steps, tile).steps
        s_nn = time_to_steady(channels, model_init(model, False), tol, check_every, max_steps, tile).steps
        # which predicted field limits: the exact u with the predicted rho,
        # and the predicted u with the exact rho
        phys = np.concatenate([pred_u, pred_rho[..., None]], axis=-1)
        u_ex = np.concatenate([u_plain, pred_rho[..., None]], axis=-1)
        rho_ex = np.concatenate([phys[..., :2], rho_plain[..., None]], axis=-1)
        s_uex = time_to_steady(channels, field_init(u_ex, with_neq), tol, check_every, max_steps, tile).steps
        s_rex = time_to_steady(channels, field_init(rho_ex, with_neq), tol, check_every, max_steps, tile).steps
        out.update(steady_init_steps_mean=float(np.mean(s_ex)), rho_one_steps_mean=float(np.mean(s_r1)),
                   no_neq_steps_mean=float(np.mean(s_nn)), exact_u_net_rho_steps_mean=float(np.mean(s_uex)),
                   net_u_exact_rho_steps_mean=float(np.mean(s_rex)))
    return out
