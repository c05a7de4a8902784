"""Benchmark of the lattice-Boltzmann sweep on GB300.

Default workload (the configuration the headline metric is quoted on): D3Q19
BGK lid-driven cavity, 256^3 cells, FP32 populations, tau = 0.55, lid
u = (0.1, 0, 0) by moving bounce-back, all other walls full-way bounce-back,
rest-equilibrium start.  One bench step = one time step = one fused
collide+boundary+stream sweep over all 16.8 M cells.  The populations
(1.27 GB) are far larger than L2 (129 MB), so no flush is needed between
steps.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl gb300|reference]
                    [--workload d3q19_cavity_256|d3q27_cavity_256|d2q9_poiseuille_256x64|...]
                    [--storage fp32|fp16s]

Prints one JSON line (rank 0).  For N > 1 (torchrun), every rank runs an
independent replica of the workload on its own GPU (the sweep has no exchange
step on one lattice); value = all ranks' cell updates / max time.
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import tempfile
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

WORKLOADS = {
    # name: (descriptor, dims, tau, kind)
    "d3q19_cavity_256": (19, (256, 256, 256), 0.55, "cavity"),
    "d3q27_cavity_256": (27, (256, 256, 256), 0.55, "cavity"),
    "d3q19_cavity_128": (19, (128, 128, 128), 0.55, "cavity"),
    "d3q19_cavity_192": (19, (192, 192, 192), 0.55, "cavity"),
    "d3q27_cavity_128": (27, (128, 128, 128), 0.55, "cavity"),
    "d3q27_cavity_192": (27, (192, 192, 192), 0.55, "cavity"),
    "d2q9_poiseuille_256x64": (9, (256, 64), 0.8, "poiseuille"),
    "d2q9_channel_4096x4096": (9, (4096, 4096), 0.8, "poiseuille"),
    "d2q9_batch_1024": (9, None, None, "batch"),
    "d2q9_batch_1024_converge": (9, None, None, "batch_converge"),
    "d2q9_warm_start_256x64": (9, (256, 64), None, "warm_start"),
    "unet_train_256x64": (9, (256, 64), None, "unet_train"),
    "d2q9_psm_particles_2048x512": (9, (2048, 512), 0.7, "particles"),
}


def max_over_ranks(x, dist, device="cuda"):
    """The slowest rank's time (barrier-bracketed timing reports the max)."""
    if not dist:
        return x
    import torch
    t = torch.tensor([float(x)], device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def whole_job_rate(units_per_rank, world, seconds):
    """Replicas: every rank processes units_per_rank; the whole job's rate is
    all ranks' units over the slowest rank's time."""
    return world * units_per_rank / seconds


def bytes_per_update(q, storage):
    s = 4 if storage == "fp32" else 2
    return 2 * q * s + 1  # read + write every population, read the flag byte


def load_peaks():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        d = json.load(open(p))
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


def make_case(name):
    from tests import cases
    q, dims, tau, kind = WORKLOADS[name]
    if kind == "cavity":
        return cases.cavity_3d(q, dims=dims, steps=0, tau=tau)
    return cases.poiseuille_2d(dims[0], dims[1], steps=0, tau=tau)


class ClockSampler:
    """nvidia-smi clocks / throttle reasons sampled while the GPU is busy.

    The GPU is named by its UUID (an ordinal would name another GPU under
    CUDA_VISIBLE_DEVICES remapping).  A timed region of a few milliseconds is
    shorter than the 200 ms sampling period, so the bench brackets it with
    back-to-back untimed sweeps: the samples cover a window of about a second
    of sustained load that contains the timed region."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device):
        self.gpu = self.gpu_id(device)
        self.proc = None
        self.file = None
        self.t0 = None

    @staticmethod
    def gpu_id(device):
        try:
            import torch
            u = getattr(torch.cuda.get_device_properties(device), "uuid", None)
            if u is not None:
                u = str(u)
                return u if u.startswith("GPU-") else "GPU-" + u
        except Exception:
            pass
        return str(device)

    def start(self):
        try:
            self.file = tempfile.NamedTemporaryFile("w+", suffix=".csv", delete=False)
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", self.gpu, f"--query-gpu={self.FIELDS}", "--format=csv,noheader,nounits",
                 "-lms", "200"], stdout=self.file, stderr=subprocess.DEVNULL)
            self.t0 = time.perf_counter()
        except Exception:
            self.proc = None

    def _rows(self):
        if self.file is None:
            return []
        self.file.flush()
        rows = []
        for line in open(self.file.name):
            parts = [x.strip() for x in line.split(",")]
            if len(parts) >= 9:
                rows.append(parts)
        return rows

    def keep_busy(self, work, seconds):
        """Run work() back to back (each call ends with a device sync) until
        `seconds` have passed and at least one sample has been written (at
        most 5 s more).  Returns the number of calls."""
        n, t0 = 0, time.perf_counter()
        while True:
            work()
            n += 1
            dt = time.perf_counter() - t0
            if dt >= seconds and (self.proc is None or self._rows() or dt >= seconds + 5.0):
                return n

    def stop(self):
        if self.proc is None:
            return None
        window = time.perf_counter() - self.t0
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        rows = self._rows()
        os.unlink(self.file.name)
        if not rows:
            return None
        sm = [float(r[1]) for r in rows if r[1].replace(".", "").isdigit()]
        mx = [float(r[2]) for r in rows if r[2].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[k] for r in rows for k in range(4) if r[5 + k].lower() == "active"})
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": reasons, "samples": len(rows), "window_s": round(window, 3), "gpu": self.gpu}


def cpu_baseline_sample(name, seconds=10.0):
    """The CPU oracle (plain-C restatement of the reference sweep, all host
    threads) on the same lattice, timed over a bounded sample of rows."""
    from oracle.oracle import OracleLattice
    case = make_case(name)
    q, dims = case["q"], case["dims"]
    lat = OracleLattice(q, dims)
    lat.set_flags(case["flags"])
    if case["profile"] is not None:
        lat.set_profile(case["profile"])
    nrows = int(np.prod(dims[1:]))
    nx = dims[0]
    chunk = max(1, min(nrows, 1_048_576 // nx))
    lat.run_rows(case["program"], 0, chunk)  # warm-up
    done = 0
    t0 = time.perf_counter()
    r = 0
    while True:
        r1 = min(nrows, r + chunk)
        lat.run_rows(case["program"], r, r1)
        done += (r1 - r) * nx
        r = 0 if r1 >= nrows else r1
        if time.perf_counter() - t0 >= seconds:
            break
    dt = time.perf_counter() - t0
    cores = int(os.environ.get("OMP_NUM_THREADS", os.cpu_count() or 1))
    return {"value": done / dt / 1e6, "unit": "MLUPS", "cores": cores, "kind": "port",
            "sample": f"{done} cell updates of {name} ({done / (nx * nrows):.2f} sweeps, "
                      f"row blocks of {chunk * nx} cells) in {dt:.1f} s"}


def run_reference(args, rank, world):
    if rank != 0:
        print(json.dumps({"impl": "reference", "rank": rank, "skipped": "rank 0 runs the CPU reference"}),
              file=sys.stderr)
        return
    from oracle.oracle import OracleLattice
    case = make_case(args.workload)
    q, dims = case["q"], case["dims"]
    lat = OracleLattice(q, dims)
    lat.set_flags(case["flags"])
    if case["profile"] is not None:
        lat.set_profile(case["profile"])
    nrows = int(np.prod(dims[1:]))
    nx = dims[0]
    chunk = max(1, min(nrows, 1_048_576 // nx))  # ~1 M cell updates per bench step
    r = 0
    for _ in range(args.warmup):
        r1 = min(nrows, r + chunk)
        lat.run_rows(case["program"], r, r1)
        r = 0 if r1 >= nrows else r1
    done = 0
    t0 = time.perf_counter()
    for _ in range(args.steps):
        r1 = min(nrows, r + chunk)
        lat.run_rows(case["program"], r, r1)
        done += (r1 - r) * nx
        r = 0 if r1 >= nrows else r1
    dt = time.perf_counter() - t0
    v = done / dt / 1e6
    cores = int(os.environ.get("OMP_NUM_THREADS", os.cpu_count() or 1))
    line = {
        "impl": "reference", "metric": "MLUPS", "value": v, "unit": "MLUPS", "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": dt / args.steps * 1e3,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
        "config": {"workload": args.workload, "cells": int(np.prod(dims)), "storage": "fp32 AoS two-lattice",
                   "sample_cells_per_step": chunk * nx},
        "cpu_baseline": {"value": v, "unit": "MLUPS", "cores": cores, "kind": "port",
                         "sample": f"{args.steps} steps of {chunk * nx} cell updates (row blocks of the "
                                   f"{'x'.join(map(str, dims))} lattice), oracle restatement of the reference's "
                                   f"two-lattice sweep, OpenMP"},
        "e2e": {"value": v, "unit": "MLUPS", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line))


def run_batch(args, rank, world):
    """1024 seeded uneven D2Q9 channels in one batched launch."""
    import torch
    from lbm_mirror_gb300 import Batch
    from tests import cases
    chans = cases.batch_channels()
    b = Batch(chans, cases.channel_program(0.8))
    tile, tune_ms = b.autotune(steps=6)
    cells, padded, _ = b.info()
    b.step(args.warmup)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    b.step(args.steps)
    dt = time.perf_counter() - t0
    value = world * cells * args.steps / dt / 1e6
    bpu = bytes_per_update(9, "fp32")
    peak, src = load_peaks()
    line = {"metric": "MLUPS", "value": value, "unit": "MLUPS", "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": dt / args.steps * 1e3, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f32", "data": "synthetic",
            "config": {"workload": "d2q9_batch_1024", "channels": len(chans), "cells": cells, "padded_cells": padded,
                       "tile": tile, "autotune_ms_per_step": tune_ms},
            "roofline": {"bound": "hbm", "achieved": bpu * cells / (dt / args.steps) / 1e9, "peak": peak,
                         "unit": "GB/s", "frac": bpu * cells / (dt / args.steps) / 1e9 / peak, "traffic": None,
                         "peak_source": src, "bytes_per_update": bpu},
            "gpu_launches": args.steps}
    if rank == 0:
        print(json.dumps(line))


def run_batch_converge(args, rank, world):
    """The 1024 seeded uneven channels run from rest until every channel's
    relative L2 change of u over 1000 steps is below --tol (one persistent
    CUDA-graph replay per 1000 steps; converged channels' tiles are dropped
    from the launch).  value = wall seconds to the last channel."""
    import torch
    from lbm_mirror_gb300 import Batch
    from lbm_mirror_gb300 import capi as K
    from lbm_mirror_gb300.workloads import batch_channels, channel_program
    chans = batch_channels()
    b = Batch(chans, channel_program(0.8, K.KEL_ARITH_SHIFTED))
    tile, _ = b.autotune(steps=6)
    cells, padded, _ = b.info()
    b.synchronize()
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    steps, res = b.run_until(tol=args.tol, check_every=1000, max_steps=args.max_steps)
    dt = time.perf_counter() - t0
    sizes = np.array([c["nx"] * c["ny"] for c in chans], dtype=np.float64)
    updates = float(np.sum(sizes * steps.astype(np.float64)))
    bpu = bytes_per_update(9, "fp32")
    peak, src = load_peaks()
    line = {"metric": "time_to_steady_state_s", "value": dt, "unit": "s", "n_gpus": world, "steps": int(steps.max()),
            "warmup": 0, "ms_per_step": None, "higher_is_better": False, "scaling": "weak", "vs_baseline": None,
            "dtype": "f32 (shifted: g = f - w)", "data": "synthetic",
            "config": {"workload": "d2q9_batch_1024_converge", "channels": len(chans), "cells": cells,
                       "padded_cells": padded, "tile": tile, "tol": args.tol, "check_every": 1000,
                       "max_steps": args.max_steps},
            "channel_steps": {"mean": float(steps.mean()), "median": float(np.median(steps)),
                              "max": int(steps.max()), "unconverged": int(np.sum(res >= args.tol))},
            "active_MLUPS": updates / dt / 1e6,
            "roofline": {"bound": "hbm", "achieved": bpu * updates / dt / 1e9, "peak": peak, "unit": "GB/s",
                         "frac": bpu * updates / dt / 1e9 / peak, "traffic": None, "peak_source": src,
                         "bytes_per_update": bpu, "kernel": "batched sweep, averaged over the whole run"},
            "gpu_launches": int(steps.max() // 1000 * 1002)}
    if rank == 0:
        print(json.dumps(line))


def unet_flops_per_sample(h, w, widths, in_ch=16, out_ch=3):
    """Multiply-adds x 2 of one U-Net forward pass (3x3 convolutions and the
    1x1 head) on an h x w grid."""
    w0, w1, w2, w3 = widths
    convs = [(0, in_ch, w0), (0, w0, w0), (1, w0, w1), (1, w1, w1), (2, w1, w2), (2, w2, w2), (3, w2, w3),
             (3, w3, w3), (2, w3 + w2, w2), (2, w2, w2), (1, w2 + w1, w1), (1, w1, w1), (0, w1 + w0, w0), (0, w0, w0)]
    f = sum(2 * 9 * ci * co * (h >> lv) * (w >> lv) for lv, ci, co in convs)
    return f + 2 * w0 * out_ch * h * w


def run_warm_start(args, rank, world):
    """Learned warm start on 256x64 channels: --train seeded steady states
    (batched runner to --tol), U-Net training on them, then --test held-out
    geometries run to --tol from rest and from the network's prediction.
    value = wall seconds of the warm-started runs (inference and population
    reconstruction included); plain_seconds = the same from rest."""
    import torch
    from lbm_mirror_gb300 import warmstart as WS
    nx, ny = WORKLOADS[args.workload][1]
    widths = (48, 96, 128, 128)
    train_ch = WS.fixed_size_channels(args.train, seed=5, nx=nx, ny=ny)
    test_ch = WS.fixed_size_channels(args.test, seed=6, nx=nx, ny=ny)
    states = WS.solve(train_ch, tol=args.tol, check_every=1000, max_steps=args.max_steps)
    gen_updates = float(np.sum(states.steps.astype(np.float64)) * nx * ny)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    kw = dict(epochs=args.epochs, batch=32, lr=2e-3, widths=widths, log_every=32, rho_target_rms=args.rho_rms,
              residual=args.residual, weight_by_steps=args.weight_by_steps, rho_norm=args.rho_norm,
              rho_residual=args.rho_residual, flip=args.flip)
    if args.ensemble > 1:
        # the mean prediction of networks trained with seeds 1 .. K
        model = WS.train_ensemble(WS.steady_subset(states), seeds=tuple(range(1, args.ensemble + 1)), **kw)
    else:
        model = WS.train(WS.steady_subset(states), **kw)
    torch.cuda.synchronize()
    t_train = time.perf_counter() - t0
    n_steps = args.epochs * (args.train // 32) * max(args.ensemble, 1)
    train_flops = 3 * unet_flops_per_sample(ny, nx, widths) * 32 * n_steps
    r = WS.evaluate(model, test_ch, tol=args.tol, check_every=1000, max_steps=args.max_steps, variants=True)
    r2 = WS.evaluate(model, test_ch, tol=args.tol, check_every=1000, max_steps=args.max_steps)  # a second pair
    # inference alone, timed with CUDA events on the network's own stream path
    mask, u_max, tau = WS.channel_inputs(test_ch)
    d_mask = torch.from_numpy(mask).cuda()
    d_umax = torch.from_numpy(u_max).cuda()
    d_tau = torch.from_numpy(tau).cuda()
    WS.predict(model, d_mask, d_umax, d_tau)
    torch.cuda.synchronize()
    t1 = time.perf_counter()
    WS.predict(model, d_mask, d_umax, d_tau)
    t_inf = time.perf_counter() - t1
    inf_flops = unet_flops_per_sample(ny, nx, widths) * args.test * max(args.ensemble, 1)
    bf16 = None
    pk = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(pk):
        bf16 = json.load(open(pk)).get("bf16_tflops")
    # the first member's training history stands for the ensemble's
    hist = model.members[0].history if args.ensemble > 1 else model.history
    if rank == 0:
        if args.save_dir:
            nets = [m.net for m in model.members] if args.ensemble > 1 else [model.net]
            for k, net in enumerate(nets):
                np.save(os.path.join(args.save_dir, "warm_start_unet_params_%d.npy" % k), net.params())
        line = {"metric": "time_to_steady_state_s", "value": r["warm_seconds"], "unit": "s", "n_gpus": world,
                "steps": r["warm_steps_max"], "warmup": 0, "ms_per_step": None, "higher_is_better": False,
                "scaling": "weak", "vs_baseline": None, "dtype": "f32 lattice, bf16 network", "data": "synthetic",
                "config": {"workload": "d2q9_warm_start_256x64", "train": args.train, "test": args.test,
                           "tol": args.tol, "check_every": 1000, "epochs": args.epochs,
                           "rho_target_rms": args.rho_rms, "residual_u": args.residual,
                           "weight_by_steps": args.weight_by_steps, "rho_norm": args.rho_norm,
                           "rho_residual": args.rho_residual, "flip_augment": args.flip,
                           "ensemble": args.ensemble,
                           "widths": list(widths),
                           "params": sum(m.net.n_params for m in model.members) if args.ensemble > 1
                           else model.net.n_params, "rho_scale": model.rho_scale},
                "plain_seconds": r["plain_seconds"], "speedup": r["speedup"],
                "repeat": {"plain_seconds": r2["plain_seconds"], "warm_seconds": r2["warm_seconds"],
                           "speedup": r2["speedup"]},
                "warm_init_seconds": r["warm_init_seconds"],
                "channel_steps": {k: r[k] for k in ("plain_steps_mean", "warm_steps_mean", "plain_steps_max",
                                                    "warm_steps_max", "plain_unconverged", "warm_unconverged")},
                "final_u_rel_l2": {"mean": r["final_u_rel_l2_mean"], "max": r["final_u_rel_l2_max"]},
                "prediction_u_rel_l2": {"mean": r["prediction_u_rel_l2_mean"], "max": r["prediction_u_rel_l2_max"]},
                "prediction_drho_rel_l2_mean": r["prediction_drho_rel_l2_mean"],
                "nonfinite_channels": r["nonfinite_channels"],
                "warm_fallbacks_to_rest": r["warm_fallbacks_to_rest"],
                "init_variants_steps_mean": {"steady_state_itself": r["steady_init_steps_mean"],
                                             "net_u_rho_one": r["rho_one_steps_mean"],
                                             "net_without_neq": r["no_neq_steps_mean"],
                                             "exact_u_net_rho": r["exact_u_net_rho_steps_mean"],
                                             "net_u_exact_rho": r["net_u_exact_rho_steps_mean"]},
                "training": {"seconds": t_train, "adam_steps": n_steps, "batch": 32,
                             "loss_first": hist[0][1] if hist else None,
                             "loss_last": hist[-1][1] if hist else None,
                             "tflops": train_flops / t_train / 1e12},
                "inference": {"seconds": t_inf, "samples": args.test, "tflops": inf_flops / t_inf / 1e12},
                "data_generation": {"seconds": states.seconds, "channels": args.train,
                                    "unconverged": int(np.sum(~states.converged)),
                                    "residual_max_converged": float(np.max(states.residual[states.converged]))
                                    if states.converged.any() else None,
                                    "active_MLUPS": gen_updates / states.seconds / 1e6},
                "roofline": {"bound": "tensor", "achieved": train_flops / t_train / 1e12,
                             "peak": bf16, "unit": "TFLOP/s",
                             "frac": (train_flops / t_train / 1e12 / bf16) if bf16 else None, "traffic": None,
                             "peak_source": "measured" if bf16 else None,
                             "kernel": "U-Net training step (whole step, host loop included)"},
                "gpu_launches": None}
        print(json.dumps(line))


def run_unet_train(args, rank, world):
    """Training steps of the warm-start U-Net (widths 32, 64, 128, 128; 256x64
    grids; batch 32) on the input planes of seeded channels and a synthetic
    target: make_input + one captured training step (forward, backward, Adam)
    per step; the loss is read back after the timed steps.
    value = model TFLOP/s of the whole step (3 x the forward FLOPs)."""
    import torch
    from lbm_mirror_gb300 import UNet
    from lbm_mirror_gb300 import warmstart as WS
    nx, ny = WORKLOADS[args.workload][1]
    n, widths = 32, (32, 64, 128, 128)
    chans = WS.fixed_size_channels(n, seed=77, nx=nx, ny=ny)
    mask, umax, tau = WS.channel_inputs(chans)
    dm, du, dt = (torch.from_numpy(a).cuda() for a in (mask, umax, tau))
    tgt = torch.randn((n, ny, nx, 3), device="cuda", generator=torch.Generator(device="cuda").manual_seed(5)) * 0.1
    net = UNet(height=ny, width=nx, widths=widths, max_batch=n, seed=1)

    def step():
        # forward + backward + Adam as one captured graph (kel_unet_train_step)
        net.make_input(dm.data_ptr(), du.data_ptr(), dt.data_ptr(), n)
        net.train_step(tgt.data_ptr(), n, lr=1e-3)

    torch.cuda.synchronize()
    for _ in range(args.warmup):
        step()
    net.synchronize()
    t0 = time.perf_counter()
    for _ in range(args.steps):
        step()
    loss = net.last_loss()  # synchronises
    dt_s = (time.perf_counter() - t0) / args.steps
    flops = 3 * unet_flops_per_sample(ny, nx, widths) * n
    pk = os.path.join(ROOT, "MEASURED_PEAKS.json")
    bf16 = json.load(open(pk)).get("bf16_tflops") if os.path.exists(pk) else None
    t0 = time.perf_counter()
    for _ in range(args.steps):
        net.forward(n)
    net.synchronize()
    fwd_s = (time.perf_counter() - t0) / args.steps
    line = {"metric": "unet_train_tflops", "value": flops / dt_s / 1e12, "unit": "TFLOP/s", "n_gpus": world,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": dt_s * 1e3, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "bf16 x bf16 -> fp32", "data": "synthetic",
            "config": {"workload": "unet_train_256x64", "batch": n, "widths": list(widths),
                       "params": net.n_params, "conv": "tcgen05"},
            "forward_ms": fwd_s * 1e3, "forward_tflops": unet_flops_per_sample(ny, nx, widths) * n / fwd_s / 1e12,
            "loss": loss,
            "roofline": {"bound": "tensor", "achieved": flops / dt_s / 1e12, "peak": bf16, "unit": "TFLOP/s",
                         "frac": flops / dt_s / 1e12 / bf16 if bf16 else None, "traffic": None,
                         "peak_source": "measured" if bf16 else None, "kernel": "whole training step"},
            "gpu_launches": None}
    if rank == 0:
        print(json.dumps(line))


def run_particles(args, rank, world):
    """Particle-laden channel: 2048x512 periodic channel, PSM + Guo gravity, 64 discs R = 8,
    4x4 sub-cell solid fraction, DEM k = 100, damping 0.1, FP64 bodies."""
    import torch
    from lbm_mirror_gb300 import Lattice, Particles
    from lbm_mirror_gb300 import capi as K
    from tests import cases
    q, dims, tau, _ = WORKLOADS[args.workload]
    flags, st = cases.particle_channel(*dims)
    g = 1e-6
    ops = {1: dict(bc=K.KEL_BC_BOUNCE_BACK), 2: dict(bc=K.KEL_BC_FLUID, collide=1)}
    prog = K.make_program(tau, K.KEL_COLL_PSM_GUO, ops, global_force=(0.0, -g, 0.0))
    prm = K.make_particle_params(K.KEL_POROSITY_SUBCELL, sub_steps=1, k_n=100.0, zeta_n=0.1,
                                 body_acceleration=(0.0, -g), wall_axes=0b10)
    stream = torch.cuda.Stream()
    lat = Lattice("D2Q9", dims, periodic_x=True, stream=stream.cuda_stream)
    lat.upload_flags(flags)
    ps = Particles(lat, st)
    tuned = lat.autotune(prog, steps=8)
    # warm-up long enough to capture the two-step graph the coupled step replays
    ps.step(prm, prog, max(args.warmup, 8), write_macros=False)
    lat.synchronize()
    ev = [torch.cuda.Event(enable_timing=True) for _ in range(4)]
    # the NVTX range "timed" marks the coupled steps for a profiler's filter
    torch.cuda.nvtx.range_push("timed")
    ev[0].record(stream)
    ps.step(prm, prog, args.steps, write_macros=False)
    ev[1].record(stream)
    torch.cuda.nvtx.range_pop()
    lat.step(prog, args.steps, write_macros=False)
    ev[2].record(stream)
    ev[2].synchronize()
    coupled_ms = ev[0].elapsed_time(ev[1]) / args.steps
    sweep_ms = ev[1].elapsed_time(ev[2]) / args.steps
    cells = dims[0] * dims[1]
    bpu = 2 * 9 * 4 + 1 + 4  # populations, flag, porosity
    peak, src = load_peaks()
    line = {"metric": "MLUPS", "value": world * cells / (coupled_ms / 1e3) / 1e6, "unit": "MLUPS", "n_gpus": world,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": coupled_ms, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32 lattice, f64 bodies", "data": "synthetic",
            "config": {"workload": args.workload, "cells": cells, "particles": int(st.shape[0]), "radius": 8.0,
                       "porosity": "4x4 sub-cell", "launch": list(tuned[:2])},
            "particle_phases_ms_per_step": coupled_ms - sweep_ms, "sweep_only_ms_per_step": sweep_ms,
            "roofline": {"bound": "hbm", "achieved": bpu * cells / (sweep_ms / 1e3) / 1e9, "peak": peak,
                         "unit": "GB/s", "frac": bpu * cells / (sweep_ms / 1e3) / 1e9 / peak, "traffic": None,
                         "peak_source": src, "bytes_per_update": bpu, "kernel": "PSM+Guo sweep"},
            "gpu_launches": args.steps * 3,
            "launches_per_step": "couple + gather (the bodies' boxes only, blocks per body), contact + integrate "
                                 "(one warp per body, beside the sweep), sweep; graph-replayed in pairs of steps"}
    if rank == 0:
        print(json.dumps(line))


# DRAM bytes (read + write) per cell update of the one-cell sweep, from ncu
# dram__bytes_read.sum + dram__bytes_write.sum on the 192^3 cavity (both
# parities averaged).  The 256^3 bench
# lattice is too large to capture under ncu's memory save/restore, so its
# per-launch traffic is this figure times the cells (traffic grows with the
# cells: every population is read and written once).
SWEEP1_TRAFFIC_PER_CELL = {(19, "fp32"): 144.6, (19, "fp16s"): 69.1, (27, "fp32"): 208.8}


def sweep_traffic(q, storage, cpt, cells):
    per = SWEEP1_TRAFFIC_PER_CELL.get((q, storage))
    return per * cells if (per is not None and cpt == 1) else None


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=1000)
    ap.add_argument("--warmup", type=int, default=20)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--workload", default="d3q19_cavity_256", choices=sorted(WORKLOADS))
    ap.add_argument("--storage", default="fp32", choices=["fp32", "fp16s"])
    ap.add_argument("--arith", default="fast", choices=["fast", "reference"],
                    help="collision arithmetic of the headline sweep (reference: the reference's own rounding, "
                         "bit-exact with it)")
    ap.add_argument("--cpt", type=int, default=0, help="cells per thread of the sweep (0: library default)")
    ap.add_argument("--block", type=int, default=256)
    ap.add_argument("--e2e-iters", type=int, default=3)
    ap.add_argument("--e2e-lbm-steps", type=int, default=100)
    ap.add_argument("--cpu-seconds", type=float, default=10.0)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--tol", type=float, default=1e-6, help="steady-state residual (converge / warm-start workloads)")
    ap.add_argument("--max-steps", type=int, default=2_000_000)
    ap.add_argument("--train", type=int, default=4096, help="warm start: training steady states")
    ap.add_argument("--test", type=int, default=512, help="warm start: held-out geometries")
    ap.add_argument("--epochs", type=int, default=60)
    ap.add_argument("--rho-rms", type=float, default=0.25,
                    help="warm start: RMS of the normalised density target (its weight in the loss)")
    ap.add_argument("--weight-by-steps", action="store_true",
                    help="warm start: draw training channels in proportion to their steps from rest")
    ap.add_argument("--residual", action="store_true",
                    help="warm start: predict the correction to the local Poiseuille estimate of u_x")
    ap.add_argument("--save-dir", default="", help="warm start: directory for the trained parameters")
    ap.add_argument("--rho-norm", default="lubrication", choices=["global", "lubrication"],
                    help="warm start: density target over u_max (global) or over the channel's lubrication "
                         "pressure drop")
    ap.add_argument("--no-flip", dest="flip", action="store_false",
                    help="warm start: no y-mirrored copies in the training minibatches")
    ap.add_argument("--rho-residual", action="store_true",
                    help="warm start: the density output corrects the lubrication pressure plane")
    ap.add_argument("--ensemble", type=int, default=1,
                    help="warm start: networks trained with seeds 1 .. K, predictions averaged")
    args = ap.parse_args()
    args.warmup = max(args.warmup, 3)

    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))

    if args.impl == "reference":
        if world > 1:
            os.environ.setdefault("MASTER_ADDR", "127.0.0.1")
        run_reference(args, rank, world)
        return

    import torch
    torch.cuda.set_device(local)
    if WORKLOADS[args.workload][3] == "batch":
        run_batch(args, rank, world)
        return
    if WORKLOADS[args.workload][3] == "particles":
        run_particles(args, rank, world)
        return
    if WORKLOADS[args.workload][3] == "batch_converge":
        run_batch_converge(args, rank, world)
        return
    if WORKLOADS[args.workload][3] == "warm_start":
        run_warm_start(args, rank, world)
        return
    if WORKLOADS[args.workload][3] == "unet_train":
        run_unet_train(args, rank, world)
        return
    dist = None
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl", device_id=torch.device("cuda", local))

    from lbm_mirror_gb300 import Lattice
    from lbm_mirror_gb300 import capi as K
    from tests.gpu_util import QNAME, with_arith

    case = make_case(args.workload)
    q, dims = case["q"], case["dims"]
    ncell = int(np.prod(dims))
    stream = torch.cuda.Stream()
    lat = Lattice(QNAME[q], dims, storage=args.storage, stream=stream.cuda_stream)
    lat.upload_flags(case["flags"])
    if case["profile"] is not None:
        lat.upload_inlet_profile(case["profile"])
    arith = {"fast": K.KEL_ARITH_FAST, "reference": K.KEL_ARITH_REFERENCE}
    prog = with_arith(case["program"], arith[args.arith])
    if args.cpt:
        lat.set_launch(args.cpt, args.block)
        tuned = None
    else:
        tuned = lat.autotune(prog, steps=8)  # the project's launch-shape autotuner
    cpt, block = lat.launch()

    # ---- device-resident throughput (value) and per-launch duration -------
    lat.step(prog, args.warmup, write_macros=False)
    lat.synchronize()
    clocks = ClockSampler(torch.cuda.current_device())
    ev0 = torch.cuda.Event(enable_timing=True)
    ev1 = torch.cuda.Event(enable_timing=True)

    def busy():  # untimed sweeps around the timed region (also warms kel_step's graph)
        lat.step(prog, 256, write_macros=False)
        lat.synchronize()

    clocks.start()
    soak = clocks.keep_busy(busy, 0.5)
    if dist:
        dist.barrier()
    torch.cuda.synchronize()
    ev0.record(stream)
    lat.step(prog, args.steps, write_macros=False)
    ev1.record(stream)
    ev1.synchronize()
    torch.cuda.synchronize()
    soak += clocks.keep_busy(busy, 0.5)
    clk = clocks.stop()
    if clk is not None:
        clk["note"] = (f"sampled over back-to-back sweeps containing the timed region "
                       f"({soak} x 256 untimed sweeps around it)")
    ms = max_over_ranks(ev0.elapsed_time(ev1), dist)
    per_launch_s = ms / 1e3 / args.steps
    value = whole_job_rate(ncell * args.steps, world, ms / 1e3) / 1e6

    bpu = bytes_per_update(q, args.storage)
    peak, peak_src = load_peaks()
    achieved = bpu * ncell / per_launch_s / 1e9

    # ---- the other collision arithmetic, same lattice, same step count -----
    # (the reference's rounding sequence exists for FP32 storage only)
    other_line = None
    if args.storage == "fp32":
        other = "reference" if args.arith == "fast" else "fast"
        oprog = with_arith(case["program"], arith[other])
        lat.step(oprog, args.warmup, write_macros=False)
        lat.synchronize()
        if dist:
            dist.barrier()
        torch.cuda.synchronize()
        ev0.record(stream)
        lat.step(oprog, args.steps, write_macros=False)
        ev1.record(stream)
        ev1.synchronize()
        oms = max_over_ranks(ev0.elapsed_time(ev1), dist)
        other_line = {"arithmetic": other, "value": whole_job_rate(ncell * args.steps, world, oms / 1e3) / 1e6,
                      "unit": "MLUPS", "ms_per_step": oms / args.steps,
                      "hbm_frac": bpu * ncell / (oms / 1e3 / args.steps) / 1e9 / peak}
        lat.step(prog, 2, write_macros=False)  # back on the headline program for the e2e leg

    # ---- end to end through the C ABI with pinned host buffers ------------
    Q, D = q, (2 if q == 9 else 3)
    h_flags = torch.from_numpy(np.ascontiguousarray(case["flags"], dtype=np.uint8)).pin_memory()
    from tests.cases import _weights
    init = np.broadcast_to(_weights(q).astype(np.float32), (ncell, Q))
    h_pop = torch.empty((ncell, Q), dtype=torch.float32).pin_memory()
    h_pop.numpy()[:] = init
    h_rho = torch.empty(ncell, dtype=torch.float32).pin_memory()
    h_u = torch.empty(ncell * D, dtype=torch.float32).pin_memory()
    lib = lat.lib
    import ctypes as C

    def e2e_once():
        rc = lib.kel_upload_flags(lat.handle, C.c_void_p(h_flags.data_ptr()))
        rc |= lib.kel_upload_populations(lat.handle, C.c_void_p(h_pop.data_ptr()), K.KEL_DTYPE_F32, K.KEL_LAYOUT_AOS)
        rc |= lib.kel_step(lat.handle, C.byref(prog), args.e2e_lbm_steps, K.KEL_STEP_WRITE_MACROS)
        rc |= lib.kel_download_macros(lat.handle, C.c_void_p(h_rho.data_ptr()), C.c_void_p(h_u.data_ptr()))
        if rc:
            raise RuntimeError(lib.kel_last_error_string().decode())

    e2e_once()  # warm-up (staging buffer allocation)
    if dist:
        dist.barrier()
    t0 = time.perf_counter()
    for _ in range(args.e2e_iters):
        e2e_once()
    e2e_s = max_over_ranks(time.perf_counter() - t0, dist)
    e2e_value = whole_job_rate(ncell * args.e2e_lbm_steps * args.e2e_iters, world, e2e_s) / 1e6
    mass = float(h_rho.numpy()[case["flags"] == 2].astype(np.float64).mean())
    # one more pass, each call timed alone (not part of the e2e value)
    phases = {}
    tp = time.perf_counter()
    lib.kel_upload_flags(lat.handle, C.c_void_p(h_flags.data_ptr()))
    phases["upload_flags"] = (time.perf_counter() - tp) * 1e3
    tp = time.perf_counter()
    lib.kel_upload_populations(lat.handle, C.c_void_p(h_pop.data_ptr()), K.KEL_DTYPE_F32, K.KEL_LAYOUT_AOS)
    phases["upload_populations"] = (time.perf_counter() - tp) * 1e3
    tp = time.perf_counter()
    lib.kel_step(lat.handle, C.byref(prog), args.e2e_lbm_steps, K.KEL_STEP_WRITE_MACROS)
    lib.kel_lattice_synchronize(lat.handle)
    phases["steps"] = (time.perf_counter() - tp) * 1e3
    tp = time.perf_counter()
    lib.kel_download_macros(lat.handle, C.c_void_p(h_rho.data_ptr()), C.c_void_p(h_u.data_ptr()))
    phases["download_macros"] = (time.perf_counter() - tp) * 1e3

    line = {
        "metric": "MLUPS", "value": value, "unit": "MLUPS", "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": ms / args.steps, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f32" if args.storage == "fp32" else "f16-shifted storage, f32 arithmetic",
        "data": "synthetic",
        "config": {"workload": args.workload, "descriptor": f"D{D}Q{Q}", "dims": list(dims), "cells": ncell,
                   "storage": args.storage, "tau": float(prog.tau), "collision": "BGK", "arithmetic": args.arith,
                   "scheme": "AA in-place, SoA", "cells_per_thread": cpt, "block": block,
                   "autotuned": tuned is not None, "l2": "populations 1.27 GB >> 129 MB L2, no flush needed"
                   if ncell * Q * 4 > 4e8 else "working set smaller than L2",
                   "parallelism": f"replicas x{world}"},
        "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s", "frac": achieved / peak,
                     "traffic": sweep_traffic(Q, args.storage, cpt, ncell), "peak_source": peak_src,
                     "bytes_per_update": bpu, "per_launch_ms": per_launch_s * 1e3},
        "e2e": {"value": e2e_value, "unit": "MLUPS", "h2d_bytes_per_step": int(ncell + ncell * Q * 4),
                "d2h_bytes_per_step": int(ncell * 4 * (1 + D)), "lbm_steps_per_step": args.e2e_lbm_steps,
                "iters": args.e2e_iters, "mean_rho_fluid": mass, "phases_ms": phases},
        "gpu_launches": args.steps,
        "clocks": clk,
        "other_arithmetic": other_line,
    }
    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        line["cpu_baseline"] = cpu_baseline_sample(args.workload, args.cpu_seconds)
    lat.close()
    if rank == 0:
        print(json.dumps(line))
    if dist:
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
