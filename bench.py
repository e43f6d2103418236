#!/usr/bin/env python
"""Benchmark of the IB3D per-time-step hot path on one GB300.

Workload (sphere256, Re 275): flow past a fixed sphere (icosphere D = 1, 2562
nodes, 5120 triangles) on a 256x192x192 non-uniform staggered grid (D/40
uniform core on [-0.8,0.8]^3, geometric stretching to the domain
[-5,15]x[-5,5]x[-5,5]), dt = 0.002, impulsive start u = 1, at Re 275 -- the
Reynolds number the shipped network was never trained on (its training runs used
200-350 without 275). Each step is the reference's full step (momentum predictor,
boundary conditions, ghost-point forcing, red-black SOR pressure solve with
relaxation 1.99 to an FP64 residual L-inf <= 1e-6, pressure/velocity correction,
drag/lift). Every arm runs W untimed warm-up steps from the impulsive start and
times steps W+1..W+K: the same physical steps in every arm.

value  = steps/s of the headline form: FP32 red-black sweeps inside an FP64
         defect-correction loop (passes of 512 sweeps, the last one cut to what
         the measured rate needs, the first six at relaxation 1), warm-started
         by the trained U-Net of ib3d-gpu_gb300/weights, stopped at the same FP64
         residual as the plain path. `fp32_previous_correction` is the same form
         warm-started from the previous step's correction (the network's
         fallback).
plain_fp64 / plain_fp64_fast = steps/s of the plain FP64 method (zero initial
         correction, FP64 sweeps): reference arithmetic (bit-identical to the
         oracle), and the fast form (contracted multiply-adds, omega/diag per
         cell). `drag_rel_vs_fp64` / `lift_rel_vs_fp64`: the headline's worst
         per-step error against the reference-arithmetic path.
e2e    = the headline form through the C ABI with host buffers: the state is
         uploaded from pinned host memory at the start of the timed region and
         every step downloads u,v,w,ut,vt,wt,p to pinned host memory, as the
         reference's per-step `update host` (main.f90:55) does.
cpu_baseline = the FP64 oracle (the reference's algorithm restated in C, OpenMP
         on all host cores) on a bounded sample (two capped steps) scaled to the
         plain path's sweep count on the same window. --impl reference times whole
         oracle steps of the same window instead.

Timing: W untimed warm-up steps, then K steps between CUDA events recorded on
the library's own stream, with a barrier and synchronize on both sides; every
step reads and writes seven FP64 fields of 77.7 MB, so the inputs of each timed
step are larger than the 129 MB L2.
"""
from __future__ import annotations

import argparse
import importlib.util
import json
import os
import pathlib
import statistics
import subprocess
import sys
import tempfile
import time

ROOT = pathlib.Path(__file__).resolve().parent
METRIC = "steps/s at 256×192×192 sphere: learned+FP32 vs plain FP64, residual ≤1e-6"
# the Reynolds number of the headline run: held out of every training set of the shipped networks
HEADLINE_RE = 275.0
# Algorithmic bytes per grid cell of one red+black sweep: FP32 inner sweep = e read 4 + e
# written 4 + r 4 + flag 1; FP64 sweep = pc read 8 + written 8 + b/dt 8 + flag 1.
BYTES_SOR32_SWEEP = 13.0
BYTES_SOR64_SWEEP = 25.0
# DRAM bytes (read + written) per grid cell and sweep of the FP32 sweep kernel
# (k_sor32p2) at 256x192x192, from one ncu capture of four launches inside the sweep
# loop (warm: caches as the previous launch left them; 9,702,144 B in all) and of two
# launches after a cache flush (cold; 60,701,696 B each on average). Other workloads
# scale them by their cell count.
DRAM_BYTES_PER_CELL_SWEEP32 = 2 * 9702144.0 / 4 / 9437184.0
DRAM_BYTES_PER_CELL_SWEEP32_COLD = 2 * 60701696.0 / 9437184.0


def package():
    if "ib3d_gpu_gb300" in sys.modules:
        return sys.modules["ib3d_gpu_gb300"]
    pkg = ROOT / "ib3d-gpu_gb300"
    spec = importlib.util.spec_from_file_location("ib3d_gpu_gb300", pkg / "__init__.py",
                                                  submodule_search_locations=[str(pkg)])
    mod = importlib.util.module_from_spec(spec)
    sys.modules["ib3d_gpu_gb300"] = mod
    spec.loader.exec_module(mod)
    return mod


def workload(pkg, name: str, re: float | None = None):
    cs = pkg.grids.case(name)
    cs.omega = 1.99     # the reference's relaxation factor (subPcorVcor.f90:158)
    cs.eps = 1e-6
    if re is not None:
        cs.re = float(re)
    return cs


# FP32 inner sweeps use their own relaxation factor (the FP64 defect correction fixes the final
# accuracy). On this grid, over steps 4-19 of the run, 1.9935-1.9937 needs the fewest sweeps with
# either warm start (1.99-1.999 scanned; 1.9932 and 1.994 need 3-10 % more); passes of 512
# sweeps with the last one cut to what the measured rate needs (IB3D_INNER_TAIL); the solve's first
# 6 sweeps at relaxation 1 (smooth_sweeps: 4, 6 and 10 need 6.2, 7.0 and 7.4 % fewer sweeps with the
# learned guess than none, 2-3 % with the previous correction), then 32 sweeps whose relaxation
# rises linearly to omega_inner (ramp_sweeps: 1.0 % fewer sweeps with the learned guess, 1.9 % with
# the previous correction; 4-12 less, 64-256 worse)
FAST = dict(precision=1, warm_start=1, criterion=1, inner_sweeps=512, inner_schedule=2, omega_inner=1.9937,
            smooth_sweeps=6, ramp_sweeps=32, sweep_kernel=0, max_sweeps=400000)
# the plain FP64 method: zero initial correction, FP64 sweeps, residual tested every 8 sweeps;
# reference arithmetic, and the fast form (IB3D_PREC_FP64_FAST)
PLAIN = dict(precision=0, warm_start=0, criterion=1, check_every=8, max_sweeps=400000)
PLAIN_FAST = dict(PLAIN, precision=2)
# U-Net weights trained on the GPU by this library's own kernels (bench.py --train-net);
# networks.json names the default and each file's coarsening
WEIGHTS_DIR = ROOT / "ib3d-gpu_gb300" / "weights"

def load_net(pkg, name: str = "", coarsen: int = 4):
    """The trained warm-start network (networks.json's default, or `name` there), or
    None when no weights are present. A `name` with a directory part is a weights file
    outside the package, run at coarsening `coarsen`."""
    import numpy as np
    if os.sep in name:
        path, f = pathlib.Path(name), coarsen
    else:
        manifest = WEIGHTS_DIR / "networks.json"
        if not manifest.exists():
            return None
        info = json.loads(manifest.read_text())
        name = name or info["default"]
        path, f = WEIGHTS_DIR / name, int(info["networks"].get(name, {}).get("coarsen", coarsen))
    if not path.exists():
        return None
    net = pkg.Net(seed=0)
    net.set_coarsening(f)
    w = np.fromfile(path, dtype="<f4")
    if w.size != net.nparams:
        raise SystemExit(f"{path}: {w.size} weights, the network has {net.nparams}")
    net.set_params(w)
    net.weights = name
    return net


def train_net(pkg, cs, out: str, seconds: float, coarsen: int = 2, reynolds=(200.0, 250.0, 300.0, 350.0),
              steps: int = 24, patches: int = 8, init: str = "", lr0: float = 1e-3, windows=None,
              eval_spinup: int = 0) -> dict:
    """Generates snapshots (perturbed runs at the given Reynolds numbers -- by default
    Re 200/250/300/350 --, `steps` steps each, `patches` random patches of 128^3 cells
    per step from step 3), trains with Adam for `seconds` (batch 8, lr 1e-3 then 2e-4
    for the last 30 %), writes the FP32 weights, and compares sweeps on a held-out Re
    275 run (adaptive pass lengths, so that the counts resolve differences below 256
    sweeps). With `init` the training starts from those weights (a networks.json name or
    a path), at learning rate lr0 (then lr0/5 for the last 30 %). With `windows` the
    patches come from those step windows of each run ((first, last), 1-based; runs go
    on to the last window's end, so later windows see the developed wake), and with
    `eval_spinup` the held-out run is also compared on a developed wake after that
    many steps."""
    import dataclasses
    import numpy as np
    learned = importlib.import_module("ib3d_gpu_gb300.learned")
    net = load_net(pkg, init, coarsen) if init else None
    if net is None:
        net = pkg.Net(seed=0)
    net.set_coarsening(coarsen)
    per_run = sum(b - a + 1 for a, b in windows) if windows else steps - 2
    net.reserve(128 // coarsen, len(reynolds) * per_run * patches)     # patches of 128^3 cells
    net.coarsen = coarsen
    if windows:
        gen = learned.generate_windows(net, cs, list(reynolds), windows, patches)
    else:
        gen = learned.generate(net, cs, list(reynolds), steps, patches)
    fit = lambda: float(np.mean([net.train(1, batch=8, lr=0.0, seed=10 ** 6 + q) for q in range(16)]))
    before = fit()
    t0, steps = time.perf_counter(), 0
    while time.perf_counter() - t0 < seconds:
        lr = lr0 if time.perf_counter() - t0 < 0.7 * seconds else lr0 / 5
        learned.train(net, 100, batch=8, lr=lr, chunk=100, seed=steps)
        steps += 100
    after = fit()
    pathlib.Path(out).parent.mkdir(parents=True, exist_ok=True)
    net.get_params().astype("<f4").tofile(out)
    t_train = time.perf_counter() - t0
    ev = learned.evaluate(net, dataclasses.replace(cs), 275.0, 12, inner_schedule=1)
    res = {"weights": str(out), "patches": gen["patches"], "generate_s": gen["seconds"], "adam_steps": steps,
           "train_s": t_train, "training_set_loss": [before, after],
           "eval_re275": {k: {"sweeps": v["sweeps"], "seconds": v["seconds"], "initial_err": v["initial_err"]}
                          for k, v in ev.items()}}
    if eval_spinup:
        fd, path = tempfile.mkstemp(suffix=".ib3drst")
        os.close(fd)
        try:
            dev = learned.evaluate_developed(net, dataclasses.replace(cs), 275.0, eval_spinup, 12, path,
                                             inner_schedule=1)
        finally:
            os.unlink(path)
        res["eval_re275_developed"] = {k: {"sweeps": v["sweeps"]} for k, v in dev.items()}
        res["eval_re275_developed"]["spinup"] = eval_spinup
    return res


def train_moving(pkg, cs, out: str, seconds: float, weights: str = "", coarsen: int = 4, steps: int = 200,
                 patches: int = 8) -> dict:
    """Fine-tunes a trained network on the moving sphere: captures `patches` patches of
    128^3 cells per step from steps 3..`steps` of a run whose initial u carries a seeded
    1 % perturbation (FP32 form, previous-correction warm start), then trains with Adam
    for `seconds` from the given weights (lr 2e-4, then 5e-5 for the last 30 %) and
    writes the FP32 weights."""
    import numpy as np
    learned = importlib.import_module("ib3d_gpu_gb300.learned")
    net = load_net(pkg, weights, coarsen)
    if net is None:
        raise SystemExit("train-moving: no network to start from")
    net.reserve(128 // net.coarsen, (steps - 2) * patches)
    t0 = time.perf_counter()
    gen = run_moving(pkg, cs, FAST, 0, steps, perturb=0.01, seed=1, capture=(net, patches))
    t_gen = time.perf_counter() - t0
    fit = lambda: float(np.mean([net.train(1, batch=8, lr=0.0, seed=10 ** 6 + q) for q in range(16)]))
    before = fit()
    t0, done = time.perf_counter(), 0
    while time.perf_counter() - t0 < seconds:
        lr = 2e-4 if time.perf_counter() - t0 < 0.7 * seconds else 5e-5
        learned.train(net, 100, batch=8, lr=lr, chunk=100, seed=done)
        done += 100
    after = fit()
    pathlib.Path(out).parent.mkdir(parents=True, exist_ok=True)
    net.get_params().astype("<f4").tofile(out)
    return {"weights": str(out), "patches": net.dataset_size(), "generate_s": t_gen,
            "generate_sweeps_per_step": gen["sweeps_per_step"], "adam_steps": done,
            "train_s": time.perf_counter() - t0, "training_set_loss": [before, after]}


# ------------------------------------------------------------------ clocks

class Clocks:
    """Samples nvidia-smi every 200 ms while the timed region runs."""
    Q = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,clocks_event_reasons.hw_slowdown,"
         "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
         "clocks_event_reasons.sw_power_cap")

    def __init__(self, device: int):
        self.device = device
        self.proc = None
        self.f = None

    def start(self):
        try:
            self.f = tempfile.NamedTemporaryFile("w+", suffix=".csv", delete=False)
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.device), f"--query-gpu={self.Q}",
                                          "--format=csv,noheader,nounits", "-lms", "200"], stdout=self.f,
                                         stderr=subprocess.DEVNULL)
        except (OSError, FileNotFoundError):
            self.proc = None

    def stop(self) -> dict:
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        time.sleep(0.25)
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        self.f.flush()
        rows = [ln.split(",") for ln in open(self.f.name).read().splitlines() if ln.strip()]
        os.unlink(self.f.name)
        sm, mx, pw, reasons = [], [], [], set()
        names = ("hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap")
        for r in rows:
            try:
                sm.append(float(r[0])); mx.append(float(r[1])); pw.append(float(r[2]))
            except (ValueError, IndexError):
                continue
            for q, n in enumerate(names):
                if len(r) > 4 + q and r[4 + q].strip().lower() == "active":
                    reasons.add(n)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "power_w_max": max(pw) if pw else None, "samples": len(sm), "reasons": sorted(reasons)}


# ------------------------------------------------------------ distributed

class Dist:
    def __init__(self):
        self.world = int(os.environ.get("WORLD_SIZE", "1"))
        self.rank = int(os.environ.get("RANK", "0"))
        self.local = int(os.environ.get("LOCAL_RANK", "0"))
        self.pg = None
        if self.world > 1:
            import torch.distributed as dist
            dist.init_process_group("gloo")
            self.pg = dist

    def barrier(self):
        if self.pg:
            self.pg.barrier()

    def max(self, x: float) -> float:
        if not self.pg:
            return x
        import torch
        t = torch.tensor([x], dtype=torch.float64)
        self.pg.all_reduce(t, op=self.pg.ReduceOp.MAX)
        return float(t.item())

    def close(self):
        if self.pg:
            self.pg.destroy_process_group()




# -------------------------------------------------------------- GPU arms

def run_arm(pkg, cs, mode: dict, warmup: int, steps: int, dist: Dist, timers: bool = True, clocks=None,
            net=None, restart: str | None = None):
    """W untimed warm-up steps, then K steps timed with CUDA events on the library's
    stream; returns the time, every timed step's solve statistics and drag/lift, the
    phase timers and the clocks. `restart` starts from a restart file (the first step
    after it runs stressCal1, as a fresh run does)."""
    import torch
    s = pkg.setup_case(cs, **mode)
    if net is not None:
        s.attach_net(net)
    if restart:
        s.read_restart(restart)
    first = True
    for _ in range(warmup):
        s.step(first)
        first = False
    s.synchronize()
    if timers:
        s.timers_enable(True)
    stream = torch.cuda.ExternalStream(s.stream())
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    dist.barrier()
    torch.cuda.synchronize()
    if clocks:
        clocks.start()
    torch.cuda.nvtx.range_push("ib3d_timed")
    e0.record(stream)
    stats, coefs = [], []
    for _ in range(steps):
        st, coef = s.step(first)
        first = False
        stats.append(st)
        coefs.append([float(c) for c in coef])
    e1.record(stream)
    torch.cuda.nvtx.range_pop()
    e1.synchronize()
    torch.cuda.synchronize()
    clk = clocks.stop() if clocks else None
    dist.barrier()
    t = e0.elapsed_time(e1) / 1e3
    tm = s.timers_read() if timers else None
    s.close()
    return {"seconds": t, "stats": stats, "coefs": coefs, "coef": coefs[-1], "timers": tm, "clocks": clk}


def coef_errors(coefs, ref_coefs) -> dict:
    """Worst per-step drag and lift error of one arm against another on the same steps:
    drag relative to the reference drag, lift relative to the reference lift (floored at
    1e-3 of the drag, since the lift of a sphere passes through zero)."""
    cd_err = cl_err = 0.0
    for c, r in zip(coefs, ref_coefs):
        cd, cd_ref = c[0] + c[1], r[0] + r[1]
        cl, cl_ref = c[2] + c[3], r[2] + r[3]
        cd_err = max(cd_err, abs(cd - cd_ref) / abs(cd_ref))
        cl_err = max(cl_err, abs(cl - cl_ref) / max(abs(cl_ref), 1e-3 * abs(cd_ref)))
    return {"drag_rel": cd_err, "lift_rel": cl_err, "steps_compared": min(len(coefs), len(ref_coefs))}


def run_e2e(pkg, cs, mode: dict, warmup: int, steps: int, dist: Dist, net=None, restart: str | None = None,
            overlap: bool = True):
    """The headline form through the C ABI with pinned host buffers in the timed region:
    the inputs uploaded once, then every step followed by the download of its seven
    fields, and the clock stops when the last download has landed. overlap: the
    download is ib3d_download_fields_async (a device snapshot, then host copies that
    run during the next step; a final ib3d_download_wait), else the blocking
    ib3d_download_fields."""
    import torch
    s = pkg.setup_case(cs, **mode)
    if net is not None:
        s.attach_net(net)
    if restart:
        s.read_restart(restart)
    first = True
    for _ in range(warmup):
        s.step(first)
        first = False
    shape, n3 = s.shape, s.shape[0] * s.shape[1] * s.shape[2]

    def pinned():
        return torch.empty(n3, dtype=torch.float64, pin_memory=True).numpy().reshape(shape, order="F")

    host_in = {f: pinned() for f in ("u", "v", "w", "p")}
    host_out = {f: pinned() for f in ("u", "v", "w", "ut", "vt", "wt", "p")}
    for f in host_in:
        host_in[f][...] = s.get_field(f)
    # the first download creates the transfer streams and, for the overlapped form, the
    # device snapshot (one allocation per context): done once, outside the timed region
    if overlap:
        s.download_fields_async(host_out)
    else:
        s.download_fields(host_out)
    s.download_wait()
    stream = torch.cuda.ExternalStream(s.stream())
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    dist.barrier()
    torch.cuda.synchronize()
    e0.record(stream)
    s.upload_fields(host_in["u"], host_in["v"], host_in["w"], host_in["p"])
    for _ in range(steps):
        s.step(first)
        first = False
        if overlap:
            s.download_fields_async(host_out)
        else:
            s.download_fields(host_out)
    s.download_wait()
    e1.record(stream)
    e1.synchronize()
    torch.cuda.synchronize()
    dist.barrier()
    t = e0.elapsed_time(e1) / 1e3
    s.close()
    return {"seconds": t, "h2d": 4 * n3 * 8 / steps, "d2h": 7 * n3 * 8 + 4 * 8}


def spin_up(pkg, cs, nsteps: int, path: str) -> dict:
    """Runs the headline form (previous-correction warm start) for `nsteps` steps from
    the impulsive start and writes a restart file: a developed wake to time from."""
    t0 = time.perf_counter()
    s = pkg.setup_case(cs, **FAST)
    sweeps = []
    for n in range(nsteps):
        st, _ = s.step(n == 0)
        sweeps.append(st["sweeps"])
    s.write_restart(path, totime=nsteps * cs.dt, ita=nsteps, ita1=nsteps)
    s.close()
    return {"steps": nsteps, "seconds": time.perf_counter() - t0, "t_end": nsteps * cs.dt,
            "fp32_sweeps_last_10": sum(sweeps[-10:]) / max(1, len(sweeps[-10:]))}


# ---------------------------------------------------------- CPU baseline

def _oracle():
    if str(ROOT) not in sys.path:
        sys.path.insert(0, str(ROOT))
    from oracle import oracle
    return oracle


def cpu_sample(pkg, cs, sweeps_per_step: float, threads: int) -> dict:
    """Times the FP64 oracle (the reference's algorithm, its sweep loop in the row
    form) on two capped steps of the workload and scales to steps/s: t_step = t_fixed
    + n * t_sweep, where t_sweep and t_fixed come from steps capped at 8 and 40 sweeps,
    and n is the number of sweeps the plain FP64 path took on the timed window (the
    reference-arithmetic GPU path is bit-identical to the oracle, so its sweep counts
    are the oracle's)."""
    oracle = _oracle()
    oracle.set_threads(threads)
    s1, s2 = 8, 40
    o = oracle.setup_case(cs, criterion=1, check_every=8, max_sweeps=1)
    o.set_sweep_rows(True)
    o.step(True, allow_noconv=True)          # first step: drag-probe search and thread start-up, untimed
    o.set_solver(cs.omega, cs.eps, 1, s1, 8)
    t0 = time.perf_counter()
    o.step(False, allow_noconv=True)
    t1 = time.perf_counter() - t0
    o.set_solver(cs.omega, cs.eps, 1, s2, 8)
    t0 = time.perf_counter()
    o.step(False, allow_noconv=True)
    t2 = time.perf_counter() - t0
    o.close()
    t_sweep = max((t2 - t1) / (s2 - s1), 1e-9)
    t_fixed = max(t1 - s1 * t_sweep, 0.0)
    t_step = t_fixed + sweeps_per_step * t_sweep
    return {"value": 1.0 / t_step, "unit": "steps/s", "cores": threads, "kind": "port",
            "sample": (f"FP64 oracle (C restatement of the reference, OpenMP {threads} threads) on the "
                       f"{cs.name} Re {cs.re:g} workload: after one untimed step, 2 steps capped at {s1} and {s2} SOR "
                       f"sweeps gave t_sweep={t_sweep * 1e3:.2f} ms and t_fixed={t_fixed:.3f} s per step, scaled to "
                       f"{sweeps_per_step:.0f} sweeps per step (the plain FP64 path's count on the timed steps)"),
            "t_sweep_s": t_sweep, "t_fixed_s": t_fixed, "sample_seconds": t1 + t2}


def reference_arm(pkg, cs, warmup: int, steps: int, threads: int, budget_s: float) -> dict:
    """The reference's algorithm on the host cores, whole steps: the FP64 oracle (OpenMP
    on `threads` threads, the sweep loop in its bit-identical row form) runs the W
    warm-up steps from the impulsive start untimed, then times steps W+1..W+K one by
    one, each a complete step to the FP64 residual tolerance. A step that would end
    past `budget_s` seconds of timed work is not started (the line then reports the
    steps it timed). Cross-check: a least-squares fit t_step = t_fixed + n t_sweep
    over the timed steps."""
    oracle = _oracle()
    oracle.set_threads(threads)
    t_setup = time.perf_counter()
    o = oracle.setup_case(cs, criterion=1, check_every=8, max_sweeps=400000)
    o.set_sweep_rows(True)
    t_setup = time.perf_counter() - t_setup
    first = True
    tw = time.perf_counter()
    warm_sweeps = []
    for _ in range(warmup):
        st, _ = o.step(first)
        first = False
        warm_sweeps.append(st["sweeps"])
    tw = time.perf_counter() - tw
    times, sweeps, coefs = [], [], []
    t0 = time.perf_counter()
    for _ in range(steps):
        if times and (time.perf_counter() - t0) + max(times) > budget_s:
            break
        ta = time.perf_counter()
        st, coef = o.step(first)
        first = False
        times.append(time.perf_counter() - ta)
        sweeps.append(st["sweeps"])
        coefs.append([float(c) for c in coef])
    elapsed = time.perf_counter() - t0
    o.close()
    fit = None
    if len(times) >= 2 and max(sweeps) > min(sweeps):
        n = len(times)
        mx, my = sum(sweeps) / n, sum(times) / n
        sxx = sum((x - mx) ** 2 for x in sweeps)
        t_sweep = sum((x - mx) * (y - my) for x, y in zip(sweeps, times)) / sxx
        fit = {"t_sweep_ms": 1e3 * t_sweep, "t_fixed_s": my - t_sweep * mx}
    return {"value": len(times) / elapsed, "seconds": elapsed, "steps_timed": len(times),
            "seconds_per_step": times, "sweeps_per_step": sweeps, "coefs": coefs, "warmup_seconds": tw,
            "warmup_sweeps": warm_sweeps, "setup_seconds": t_setup, "fit": fit, "threads": threads}


# ------------------------------------------------------------------ main

def run_poisson(pkg, n: int) -> dict:
    """Standalone pressure-Poisson solve (tanh-clustered n^3 cube, Neumann on all
    faces, divergence of a seeded filtered random field, omega 1.85 to a residual of
    1e-8) in FP64 and in FP32-sweep/FP64-defect-correction form: sweeps/s and the
    sweep kernels' algorithmic GB/s."""
    P = pkg.grids.poisson_problem(n, seed=0)
    out = {"workload": f"standalone Poisson {n}^3, tanh-clustered, all-Neumann, omega 1.85, residual 1e-8",
           "cells": n ** 3}
    arms = {"fp64": dict(precision=0, criterion=1, check_every=8),
            "fp64_fast": dict(precision=2, criterion=1, check_every=8),
            "fp32dc": dict(precision=1, criterion=1, inner_sweeps=256, omega_inner=1.85, sweep_kernel=0)}
    for name, kw in arms.items():
        p = pkg.default_params(re=100.0, deltat=1.0, omega=1.85, eps=1e-8, max_sweeps=1_000_000)
        for k, v in kw.items():
            setattr(p, k, v)
        s = pkg.Solver(P["x"], P["y"], P["z"], p)
        s.set_poisson_coefficients(*P["acoef"])
        s.set_field("b", P["b"])
        s.timers_enable(True)
        st = s.redblack_sor()
        tm = s.timers_read()
        sweeps = st["sweeps"]
        if name != "fp32dc":
            t_sweep = tm["sor64_ms"] / max(tm["sweeps64"], 1) * 1e-3
            gbs = BYTES_SOR64_SWEEP * n ** 3 / t_sweep / 1e9
        else:
            t_sweep = tm["sor32_ms"] / max(tm["sweeps32"], 1) * 1e-3
            gbs = BYTES_SOR32_SWEEP * n ** 3 / t_sweep / 1e9
        out[name] = {"sweeps": sweeps, "seconds": st["solve_seconds"], "sweeps_per_s": sweeps / st["solve_seconds"],
                     "final_residual": st["final_err"], "ms_per_sweep": t_sweep * 1e3, "sweep_gbs_algorithmic": gbs}
        s.close()
    return out


def sweep_bench(pkg, cases=("sphere256", "sphere384"), kernels=(0, 2), steps: int = 3) -> dict:
    """FP32 sweep kernels alone: `steps` steps of the FP32 form (previous-correction warm
    start) on each workload with each sweep kernel; microseconds per red+black sweep
    from the library's CUDA-event phase timers, and the algorithmic rate at 13 B per
    cell and sweep against the measured HBM peak."""
    peaks = json.loads((ROOT / "MEASURED_PEAKS.json").read_text()) if (ROOT / "MEASURED_PEAKS.json").exists() else {}
    hbm = float(peaks.get("hbm_gbs", 6800.0))
    out = {"peak_gbs": hbm}
    for name in cases:
        cs = workload(pkg, name)
        for kern in kernels:
            s = pkg.setup_case(cs, **dict(FAST, sweep_kernel=kern))
            s.step(True)
            s.timers_enable(True)
            for _ in range(steps):
                s.step(False)
            tm = s.timers_read()
            s.close()
            us = 1e3 * tm["sor32_ms"] / max(tm["sweeps32"], 1)
            gbs = BYTES_SOR32_SWEEP * cs.cells / (us * 1e-6) / 1e9
            out[f"{name}/kernel{kern}"] = {"us_per_sweep": us, "sweeps": tm["sweeps32"], "launches": tm["launches32"],
                                           "gbs_algorithmic": gbs, "frac": gbs / hbm}
    return out


# the U-Net's convolutions (input channels K, output channels N, level 1-3) in layer order
UNET_CONVS = [(16, 16, 1), (16, 16, 1), (16, 32, 2), (32, 32, 2), (32, 64, 3), (64, 64, 3), (96, 32, 2),
              (32, 32, 2), (48, 16, 1), (16, 16, 1)]


def unet_train_flops(batch: int, s: int) -> float:
    """FLOPs of one Adam step's convolutions as the kernels compute them (the first
    layer's 4 input channels padded to 16): forward 2*27*K*N per voxel of its level,
    the weight gradient the same, the input gradient the same for every layer but the
    first."""
    total = 0.0
    for q, (k, n, lvl) in enumerate(UNET_CONVS):
        vox = batch * (s >> (lvl - 1)) ** 3
        f = 2.0 * 27 * k * n * vox
        total += f * (2 if q == 0 else 3)
    return total


def train_bench(pkg, seconds: float = 15.0, batch: int = 8) -> dict:
    """Adam steps of the warm-start U-Net on patches captured from the 256x192x192
    sphere (4x4x4 coarsening, 32^3-voxel patches of 128^3 cells), timed with the weight
    gradients on the tensor cores and on the CUDA cores: steps/s and TFLOP/s of the
    convolutions against the measured BF16 peak."""
    peaks = json.loads((ROOT / "MEASURED_PEAKS.json").read_text()) if (ROOT / "MEASURED_PEAKS.json").exists() else {}
    peak = float(peaks.get("bf16_tflops", 1900.0))
    cs = workload(pkg, "sphere256")
    net = pkg.Net(seed=0)
    net.set_coarsening(4)
    S = 32
    net.reserve(S, 96)
    s = pkg.setup_case(cs, **FAST)
    s.enable_history()
    for n in range(8):
        s.step(n == 0)
        if n >= 2:
            net.capture(s, 16, seed=n)
    s.close()
    flops = unet_train_flops(batch, S)
    out = {"workload": f"U-Net training: batch {batch} patches of {S}^3 voxels (4x4x4 coarsening of 128^3 cells), "
                       f"{net.dataset_size()} patches captured from the sphere256 run",
           "gflop_per_step": flops / 1e9, "peak_tflops": peak,
           "peak_source": "MEASURED_PEAKS.json bf16_tflops (of measured)" if "bf16_tflops" in peaks else "fallback"}
    for name, tc in (("tensor_core_wgrad", True), ("cuda_core_wgrad", False)):
        net.set_wgrad_tensor_cores(tc)
        net.train(5, batch=batch, lr=1e-4, seed=1)
        n, t0 = 0, time.perf_counter()
        while time.perf_counter() - t0 < seconds:
            net.train(20, batch=batch, lr=1e-4, seed=100 + n)
            n += 20
        dt = time.perf_counter() - t0
        out[name] = {"adam_steps_per_s": n / dt, "tflops": n * flops / dt / 1e12,
                     "frac_of_peak": n * flops / dt / 1e12 / peak}
    net.set_wgrad_tensor_cores(True)
    net.close()
    return out


def compare_fp64(pkg, cs, steps: int, net=None) -> dict:
    """The mixed-precision form (the bench's FP32 arm, learned warm start when a
    network is given) against the plain FP64 path over the same `steps` steps, both to
    the same FP64 residual: drag and lift of every step, and u, v, w, p after the last
    step (largest difference relative to the field's largest magnitude)."""
    import numpy as np
    fast = dict(FAST, warm_start=pkg.WARM_LEARNED) if net is not None else dict(FAST)
    a = pkg.setup_case(cs, **PLAIN)
    b = pkg.setup_case(cs, **fast)
    if net is not None:
        b.attach_net(net)
    rows = []
    for q in range(1, steps + 1):
        sa, ca = a.step(q == 1)
        sb, cb = b.step(q == 1)
        cd, cd_ref = cb[0] + cb[1], ca[0] + ca[1]
        cl, cl_ref = cb[2] + cb[3], ca[2] + ca[3]
        rows.append({"step": q, "sweeps_fp64": sa["sweeps"], "sweeps_fp32": sb["sweeps"],
                     "drag_rel": abs(cd - cd_ref) / abs(cd_ref),
                     "lift_abs": abs(cl - cl_ref), "lift_rel_to_drag": abs(cl - cl_ref) / abs(cd_ref)})
    fields = {}
    for f in ("u", "v", "w", "p"):
        x, y = a.get_field(f), b.get_field(f)
        fields[f] = float(np.max(np.abs(x - y)) / np.max(np.abs(x)))
    a.close()
    b.close()
    return {"workload": f"{cs.name} {cs.shape[0]}x{cs.shape[1]}x{cs.shape[2]}, Re {cs.re:g}, {steps} steps, "
                        f"residual <= {cs.eps:g}",
            "mode": "learned warm start" if net is not None else "previous-correction warm start",
            "worst_drag_rel": max(r["drag_rel"] for r in rows),
            "worst_lift_rel_to_drag": max(r["lift_rel_to_drag"] for r in rows),
            "fields_max_rel_after_last_step": fields, "steps": rows}


def run_moving(pkg, cs, mode: dict, warmup: int, steps: int, amp: float = 0.2, freq: float = 0.2, net=None,
               perturb: float = 0.0, seed: int = 0, capture=None, selective: bool = True) -> dict:
    """The body oscillates as y(t) = amp sin(2 pi freq t): before every step the nodes
    move (ib3d_move_body, surface velocity y'(t)), then selectiveRetagging re-tags the
    neighbourhoods of the IB cells (selective=False: the search re-tags a whole box
    around the new position), then the step runs. Timed with CUDA events on the library
    stream around the timed steps (move, search and step together). With `net` the
    solve starts from the network's guess; `perturb` adds a seeded relative
    perturbation to the initial u; `capture` = (network, patches) captures training
    patches of every step from step 3."""
    import math
    import numpy as np
    import torch
    if net is not None:
        mode = dict(mode, warm_start=pkg.WARM_LEARNED)
    s = pkg.setup_case(cs, **mode)
    if net is not None:
        s.attach_net(net)
    if capture is not None:
        s.enable_history()
    if perturb:
        u = s.get_field("u")
        s.set_field("u", u + perturb * np.random.default_rng(seed).standard_normal(u.shape))
    w = 2.0 * math.pi * freq
    y = 0.0
    stream = torch.cuda.ExternalStream(s.stream())
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    sweeps, coef, t_search = [], None, 0.0
    for n in range(1, warmup + steps + 1):
        if n == warmup + 1:
            s.synchronize()
            e0.record(stream)
        t = n * cs.dt
        yn = amp * math.sin(w * t)
        s.move_body(0.0, yn - y, 0.0, 0.0, amp * w * math.cos(w * t), 0.0)
        y = yn
        t0 = time.perf_counter()
        if selective:
            s.selective_retag()
        else:
            s.search(pkg.grids.body_box(cs, (0.0, y, 0.0)))
        if n > warmup:
            t_search += time.perf_counter() - t0
        st, coef = s.step(n == 1)
        if n > warmup:
            sweeps.append(st["sweeps"])
        if capture is not None and n >= 3:
            capture[0].capture(s, capture[1], seed=1000 * seed + n)
    e1.record(stream)
    e1.synchronize()
    sec = e0.elapsed_time(e1) / 1e3
    s.close()
    return {"value": steps / sec, "unit": "steps/s", "ms_per_step": 1e3 * sec / steps,
            "sweeps_per_step": sum(sweeps) / len(sweeps), "search_ms_per_step": 1e3 * t_search / steps,
            "search": "selectiveRetagging" if selective else "tagging of the whole box",
            "drag_lift": list(map(float, coef)), "y_end": y}




def developed_run(pkg, cs, spinup: int, warmup: int, steps: int, dist: Dist, net, arms: set) -> dict:
    """Every arm timed from the same developed wake: the headline form (previous-
    correction warm start) spins the impulsive start up for `spinup` steps untimed and
    writes a restart file; each arm loads it, runs W warm-up steps and times K."""
    fd, path = tempfile.mkstemp(suffix=".ib3drst")
    os.close(fd)
    try:
        out = {"workload": f"{cs.name} {cs.shape[0]}x{cs.shape[1]}x{cs.shape[2]}, Re {cs.re:g}, developed wake: "
                           f"steps {spinup + warmup + 1}..{spinup + warmup + steps} (t = "
                           f"{(spinup + warmup + 1) * cs.dt:g}..{(spinup + warmup + steps) * cs.dt:g})",
               "spin_up": spin_up(pkg, cs, spinup, path)}
        res = {}
        if net is not None:
            res["learned"] = run_arm(pkg, cs, dict(FAST, warm_start=pkg.WARM_LEARNED), warmup, steps, dist, net=net,
                                     restart=path)
        res["previous_correction"] = run_arm(pkg, cs, FAST, warmup, steps, dist, restart=path)
        if "plain_fast" in arms:
            res["plain_fp64_fast"] = run_arm(pkg, cs, PLAIN_FAST, warmup, steps, dist, restart=path)
        if "plain" in arms:
            res["plain_fp64"] = run_arm(pkg, cs, PLAIN, warmup, steps, dist, restart=path)
        ref = res.get("plain_fp64") or res.get("plain_fp64_fast")
        for name, r in res.items():
            out[name] = {"value": steps / r["seconds"], "unit": "steps/s",
                         "sweeps_per_step": sum(s["sweeps"] for s in r["stats"]) / steps,
                         "worst_final_residual": max(s["final_err"] for s in r["stats"])}
            if ref is not None and r is not ref:
                out[name]["vs_plain"] = coef_errors(r["coefs"], ref["coefs"])
        if "learned" in res:
            out["learned_sweeps_saved"] = 1.0 - out["learned"]["sweeps_per_step"] / \
                out["previous_correction"]["sweeps_per_step"]
        plains = [out[k]["value"] for k in ("plain_fp64", "plain_fp64_fast") if k in out]
        head = out.get("learned", out["previous_correction"])["value"]
        if plains:
            out["speedup_vs_fastest_plain"] = head / max(plains)
        return out
    finally:
        os.unlink(path)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", choices=("ours", "reference"), default="ours")
    ap.add_argument("--case", default="sphere256")
    ap.add_argument("--re", type=float, default=HEADLINE_RE,
                    help="Reynolds number of the step benchmark (default 275, held out of the network's training)")
    ap.add_argument("--no-cpu", action="store_true", help="skip the CPU baseline")
    ap.add_argument("--ref-budget", type=float, default=1200.0,
                    help="--impl reference: seconds of timed CPU steps after which no further step is started")
    ap.add_argument("--developed", type=int, default=0,
                    help="instead of the step benchmark: spin the flow up for this many steps, then time every "
                         "arm from that developed wake")
    ap.add_argument("--sweep-bench", action="store_true",
                    help="instead of the step benchmark: microseconds per FP32 sweep of each sweep kernel on the "
                         "256x192x192 and 384x256x256 workloads")
    ap.add_argument("--train-bench", action="store_true",
                    help="instead of the step benchmark: Adam steps/s and TFLOP/s of the warm-start network's training")
    ap.add_argument("--sweep-cases", default="sphere256,sphere384", help="workloads of --sweep-bench")
    ap.add_argument("--sweep-kernels", default="0,2", help="sweep kernels of --sweep-bench")
    ap.add_argument("--sweep-steps", type=int, default=3, help="timed steps of --sweep-bench per workload and kernel")
    ap.add_argument("--poisson", type=int, default=0,
                    help="instead of the step benchmark: the standalone all-Neumann Poisson cube of this edge "
                         "(omega 1.85, residual 1e-8), FP64 and FP32-sweep forms")
    ap.add_argument("--train-net", default="",
                    help="instead of the benchmark: generate snapshots, train the warm-start U-Net and write "
                         "its weights to this file")
    ap.add_argument("--train-seconds", type=float, default=300.0)
    ap.add_argument("--coarsen", type=int, default=4, help="coarsening of the network trained by --train-net")
    ap.add_argument("--train-moving", default="",
                    help="instead of the benchmark: fine-tune the network given by --weights (default: "
                         "networks.json's) on the first --train-steps steps of a perturbed run of the moving "
                         "sphere (--case, default sphere384) and write its weights to this file")
    ap.add_argument("--train-re", default="200,250,300,350", help="Reynolds numbers of --train-net's runs")
    ap.add_argument("--train-steps", type=int, default=24, help="steps of each --train-net run")
    ap.add_argument("--train-patches", type=int, default=8, help="patches captured per step by --train-net")
    ap.add_argument("--train-init", default="", help="weights --train-net starts from (default: random)")
    ap.add_argument("--train-windows", default="",
                    help="--train-net: comma-separated step windows first-last whose steps are captured "
                         "(default: steps 3..--train-steps)")
    ap.add_argument("--eval-spinup", type=int, default=0,
                    help="--train-net: also compare the warm starts on held-out Re 275 after this many steps")
    ap.add_argument("--train-lr", type=float, default=1e-3, help="--train-net's learning rate (then a fifth)")
    ap.add_argument("--weights", default="", help="weights file in ib3d-gpu_gb300/weights (default: networks.json's)")
    ap.add_argument("--moving", action="store_true",
                    help="instead of the step benchmark: the transversely oscillating sphere "
                         "(y = 0.2 sin(2 pi 0.2 t), search every step) on --case (default sphere384), "
                         "FP32 form and plain FP64")
    ap.add_argument("--plain-steps", type=int, default=2, help="timed steps of --moving's plain FP64 arm")
    ap.add_argument("--compare-fp64", type=int, default=0,
                    help="instead of the benchmark: this many steps of the FP32 form (learned warm start) "
                         "against the plain FP64 path: drag/lift and field differences")
    ap.add_argument("--set", default="",
                    help="comma-separated key=value overrides of the FP32-sweep arm's solver parameters")
    ap.add_argument("--arms", default="learned,fast,plain_fast,plain,e2e,cpu",
                    help="comma-separated subset of learned,fast,plain_fast,plain,e2e,cpu")
    args = ap.parse_args()
    warmup = max(args.warmup, 3)
    dist = Dist()
    pkg = package()
    for kv in filter(None, args.set.split(",")):
        k, v = kv.split("=")
        FAST[k.strip()] = float(v) if "." in v or "e" in v else int(v)
    arms = set(args.arms.split(","))
    if args.train_net:
        if dist.rank == 0:
            windows = [tuple(int(x) for x in w.split("-")) for w in args.train_windows.split(",")] \
                if args.train_windows else None
            print(json.dumps(train_net(pkg, workload(pkg, args.case), args.train_net, args.train_seconds,
                                       args.coarsen, [float(r) for r in args.train_re.split(",")],
                                       args.train_steps, args.train_patches, args.train_init,
                                       args.train_lr, windows, args.eval_spinup)), flush=True)
        dist.close()
        return
    if args.train_moving:
        if dist.rank == 0:
            mcs = workload(pkg, args.case if args.case != "sphere256" else "sphere384")
            print(json.dumps(train_moving(pkg, mcs, args.train_moving, args.train_seconds, args.weights, args.coarsen,
                                          args.train_steps, args.train_patches)), flush=True)
        dist.close()
        return
    if args.moving:
        if dist.rank == 0:
            mcs = workload(pkg, args.case if args.case != "sphere256" else "sphere384")
            out = {"workload": f"{mcs.name} {mcs.shape[0]}x{mcs.shape[1]}x{mcs.shape[2]}, Re {mcs.re:g}, moving sphere "
                               "y = 0.2 sin(2 pi 0.2 t), search every step, residual <= 1e-6",
                   "fp32": run_moving(pkg, mcs, FAST, warmup, args.steps),
                   "fp32_full_search": run_moving(pkg, mcs, FAST, warmup, args.steps, selective=False)}
            mnet = load_net(pkg, args.weights, args.coarsen)
            if mnet is not None:
                out["fp32_learned"] = run_moving(pkg, mcs, FAST, warmup, args.steps, net=mnet)
                out["fp32_learned"]["weights"] = mnet.weights
            out["plain_fp64_fast"] = run_moving(pkg, mcs, PLAIN_FAST, warmup, max(1, args.plain_steps))
            out["speedup_vs_plain_fast"] = out["fp32"]["value"] / out["plain_fp64_fast"]["value"]
            if mnet is not None:
                out["speedup_learned_vs_plain_fast"] = out["fp32_learned"]["value"] / out["plain_fp64_fast"]["value"]
            print(json.dumps(out), flush=True)
        dist.close()
        return
    if args.train_bench:
        if dist.rank == 0:
            print(json.dumps(train_bench(pkg, args.train_seconds if args.train_seconds != 300.0 else 15.0)),
                  flush=True)
        dist.close()
        return
    if args.sweep_bench:
        if dist.rank == 0:
            print(json.dumps(sweep_bench(pkg, tuple(args.sweep_cases.split(",")),
                                         tuple(int(k) for k in args.sweep_kernels.split(",")), args.sweep_steps)),
                  flush=True)
        dist.close()
        return
    if args.poisson:
        if dist.rank == 0:
            print(json.dumps(run_poisson(pkg, args.poisson)), flush=True)
        dist.close()
        return
    if args.compare_fp64:
        if dist.rank == 0:
            print(json.dumps(compare_fp64(pkg, workload(pkg, args.case, args.re), args.compare_fp64,
                                          load_net(pkg, args.weights, args.coarsen))), flush=True)
        dist.close()
        return
    cs = workload(pkg, args.case, args.re)
    threads = os.cpu_count() or 1
    window = f"steps {warmup + 1}..{warmup + args.steps} from the impulsive start u = 1 (t = " \
             f"{(warmup + 1) * cs.dt:g}..{(warmup + args.steps) * cs.dt:g})"
    config = {"workload": f"{cs.name}: {cs.shape[0]}x{cs.shape[1]}x{cs.shape[2]} non-uniform grid, sphere D=1, "
                          f"Re {cs.re:g} (held out of the network's training), dt {cs.dt:g}, red-black SOR omega "
                          f"{cs.omega:g} to FP64 residual L-inf <= {cs.eps:g}; timed window: {window}",
              "window": window,
              "l2": "inputs larger than L2: each step reads/writes 7 FP64 fields of 77.7 MB",
              "parallelism": "replicas" if dist.world > 1 else "single GPU"}

    if args.impl == "reference":
        if dist.rank != 0:
            dist.close()
            return
        ref = reference_arm(pkg, cs, warmup, args.steps, threads, args.ref_budget)
        n = ref["steps_timed"]
        sample = (f"FP64 oracle (C restatement of the reference, sweep loop in its bit-identical row form, OpenMP "
                  f"{threads} threads): {warmup} untimed warm-up steps from the impulsive start, then {n} whole "
                  f"steps timed ({window if n == args.steps else f'steps {warmup + 1}..{warmup + n}'}), each to "
                  f"the FP64 residual tolerance ({sum(ref['sweeps_per_step']) / max(n, 1):.0f} sweeps per step)")
        line = {"impl": "reference", "metric": METRIC, "value": ref["value"], "unit": "steps/s", "n_gpus": args.gpus,
                "steps": n, "warmup": warmup, "ms_per_step": 1e3 * ref["seconds"] / max(n, 1),
                "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
                "data": "synthetic: icosphere body, stretched grid, impulsive start",
                "config": dict(config, mode="reference algorithm in FP64 on the host cores"),
                "cpu_baseline": {"value": ref["value"], "unit": "steps/s", "cores": threads, "kind": "port",
                                 "sample": sample},
                "e2e": {"value": ref["value"], "unit": "steps/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
                "reference_detail": {k: ref[k] for k in ("seconds", "seconds_per_step", "sweeps_per_step",
                                                         "warmup_seconds", "warmup_sweeps", "setup_seconds", "fit")},
                "drag_lift": ref["coefs"][-1] if ref["coefs"] else None}
        if n < args.steps:
            line["note"] = f"the timed-work budget of {args.ref_budget:g} s stopped the arm after {n} of {args.steps} steps"
        print(json.dumps(line), flush=True)
        dist.close()
        return

    import torch
    torch.cuda.set_device(dist.local)
    net = load_net(pkg, args.weights, args.coarsen) if "learned" in arms else None

    if args.developed:
        if dist.rank == 0:
            print(json.dumps(developed_run(pkg, cs, args.developed, warmup, args.steps, dist, net, arms)), flush=True)
        if net is not None:
            net.close()
        dist.close()
        return

    # Headline: FP32 sweeps in FP64 defect correction with the learned warm start (the
    # trained network in the package); without weights, the previous-correction warm start.
    head_mode = dict(FAST, warm_start=pkg.WARM_LEARNED) if net is not None else FAST
    clocks = Clocks(dist.local)
    head = run_arm(pkg, cs, head_mode, warmup, args.steps, dist, timers=True, clocks=clocks, net=net)
    t = dist.max(head["seconds"])
    value = dist.world * args.steps / t
    tm = head["timers"]
    ncell = cs.cells
    sweeps = sum(st["sweeps"] for st in head["stats"])
    launches32 = max(tm["launches32"], 1)
    t_launch32 = tm["sor32_ms"] * 1e-3 / launches32
    sweeps_per_launch = tm["sweeps32"] / launches32
    bytes_launch = BYTES_SOR32_SWEEP * ncell * sweeps_per_launch
    achieved = bytes_launch / t_launch32 / 1e9
    peaks = json.loads((ROOT / "MEASURED_PEAKS.json").read_text()) if (ROOT / "MEASURED_PEAKS.json").exists() else {}
    hbm = float(peaks.get("hbm_gbs", 6800.0))
    peak_src = "MEASURED_PEAKS.json hbm_gbs (of measured)" if "hbm_gbs" in peaks else "fallback 6800 GB/s (of fallback)"
    phase_total = sum(tm[f"{p}_ms"] for p in pkg.Timers.PHASES)

    def summary(r, steps):
        tt = dist.max(r["seconds"])
        return {"value": dist.world * steps / tt, "unit": "steps/s", "ms_per_step": 1e3 * tt / steps,
                "sweeps_per_step": sum(st["sweeps"] for st in r["stats"]) / steps,
                "worst_final_residual": max(st["final_err"] for st in r["stats"]), "drag_lift": r["coef"]}

    # the same form end to end through the C ABI, right after the device-timed arm (the
    # long FP64 arms below would otherwise run between the two)
    if "e2e" in arms:
        e2e = run_e2e(pkg, cs, head_mode, warmup, args.steps, dist, net=net)
        e2e_value = dist.world * args.steps / dist.max(e2e["seconds"])
        blocking = run_e2e(pkg, cs, head_mode, warmup, args.steps, dist, net=net, overlap=False)
        e2e["blocking_value"] = dist.world * args.steps / dist.max(blocking["seconds"])
    else:
        e2e, e2e_value = {"h2d": None, "d2h": None, "blocking_value": None}, None

    prev_line = None
    if net is not None and "fast" in arms:
        prv = run_arm(pkg, cs, FAST, warmup, args.steps, dist, timers=True)
        prev_line = summary(prv, args.steps)
        prev_line["learned_sweeps_saved"] = 1.0 - (sweeps / args.steps) / prev_line["sweeps_per_step"]
    plain_runs = {}
    for name, mode in (("plain_fp64_fast", PLAIN_FAST), ("plain_fp64", PLAIN)):
        if (name == "plain_fp64" and "plain" in arms) or (name == "plain_fp64_fast" and "plain_fast" in arms):
            r = run_arm(pkg, cs, mode, warmup, args.steps, dist, timers=True)
            line_p = summary(r, args.steps)
            ptm = r["timers"]
            t_sweep = ptm["sor64_ms"] * 1e-3 / max(ptm["sweeps64"], 1)
            line_p["ms_per_sweep"] = 1e3 * t_sweep
            line_p["sweep_gbs_algorithmic"] = BYTES_SOR64_SWEEP * ncell / t_sweep / 1e9
            line_p["sweep_hbm_frac"] = line_p["sweep_gbs_algorithmic"] / hbm
            line_p["sweep_bound"] = "FP64 ALU (GB300 FP64 ~0.5 TFMA/s measured)"
            plain_runs[name] = (r, line_p)
    ref_run = plain_runs.get("plain_fp64", plain_runs.get("plain_fp64_fast", (None, None)))[0]
    plain_lines = {k: v[1] for k, v in plain_runs.items()}
    if "plain_fp64_fast" in plain_runs and "plain_fp64" in plain_runs:
        plain_lines["plain_fp64_fast"]["vs_plain_fp64"] = coef_errors(plain_runs["plain_fp64_fast"][0]["coefs"],
                                                                      plain_runs["plain_fp64"][0]["coefs"])
    plain_values = [v["value"] for v in plain_lines.values()]

    errs = coef_errors(head["coefs"], ref_run["coefs"]) if ref_run is not None else None
    line = {
        "metric": METRIC, "value": value, "unit": "steps/s", "n_gpus": dist.world, "steps": args.steps,
        "warmup": warmup, "ms_per_step": 1e3 * t / args.steps, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f32/f64",
        "data": "synthetic: icosphere body (2562 nodes, 5120 triangles), stretched grid, impulsive start u=1",
        "config": dict(config, mode=(f"FP32 red-black sweeps inside FP64 defect correction, inner relaxation "
                                     f"{FAST['omega_inner']:g}, "
                                     + (f"learned warm start (BF16 U-Net on the {net.coarsen}x{net.coarsen}x"
                                        f"{net.coarsen}-coarsened domain, weights ib3d-gpu_gb300/weights/"
                                        f"{net.weights})" if net is not None
                                        else "warm start from the previous step's correction")),
                       inner_sweeps=FAST["inner_sweeps"],
                       inner_schedule=("passes of inner_sweeps FP32 sweeps between FP64 residual checks; the "
                                       "last pass cut to the sweeps the measured rate needs")
                       if FAST.get("inner_schedule") == 2 else "fixed passes"),
        "worst_final_residual": max(st["final_err"] for st in head["stats"]),
        "drag_rel_vs_fp64": errs["drag_rel"] if errs else None,
        "lift_rel_vs_fp64": errs["lift_rel"] if errs else None,
        "fp64_reference_arm": ("plain_fp64" if "plain_fp64" in plain_runs else "plain_fp64_fast") if errs else None,
        **plain_lines,
        "speedup_vs_plain_fp64": value / plain_lines["plain_fp64"]["value"] if "plain_fp64" in plain_lines else None,
        "speedup_vs_fastest_plain": value / max(plain_values) if plain_values else None,
        "fp32_previous_correction": prev_line,
        "net_ms_per_step": tm["net_ms"] / args.steps,
        "sweeps_per_step": sweeps / args.steps,
        "sweeps_per_s": tm["sweeps32"] / (tm["sor32_ms"] * 1e-3) if tm["sor32_ms"] else None,
        "cells_per_s": value * ncell,
        "phase_ms_per_step": {p: tm[f"{p}_ms"] / args.steps for p in pkg.Timers.PHASES},
        "drag_lift": head["coef"],
        "roofline": {"kernel": "k_sor32p2 (FP32 red-black sweep, colour-packed, two rows per thread; one launch per colour pass)",
                     "bound": "hbm", "achieved": achieved, "peak": hbm, "unit": "GB/s", "frac": achieved / hbm,
                     "traffic": DRAM_BYTES_PER_CELL_SWEEP32 * ncell * sweeps_per_launch,
                     "traffic_cold": DRAM_BYTES_PER_CELL_SWEEP32_COLD * ncell * sweeps_per_launch,
                     "bytes_per_launch": bytes_launch, "bytes_per_cell_sweep": BYTES_SOR32_SWEEP,
                     "sweeps_per_launch": sweeps_per_launch, "cells": ncell, "ms_per_launch": t_launch32 * 1e3,
                     "us_per_sweep": 1e6 * tm["sor32_ms"] * 1e-3 / max(tm["sweeps32"], 1),
                     "share_of_step": tm["sor32_ms"] / phase_total if phase_total else None,
                     "peak_source": peak_src},
        "e2e": {"value": e2e_value, "unit": "steps/s", "h2d_bytes_per_step": e2e["h2d"],
                "d2h_bytes_per_step": e2e["d2h"],
                "download": "ib3d_download_fields_async every step (device snapshot of the seven fields, host "
                            "copies overlapped with the next step), ib3d_download_wait before the clock stops",
                "blocking_download_value": e2e["blocking_value"]},
        "gpu_launches": tm["launches"],
        "clocks": head["clocks"],
    }
    if dist.rank == 0 and dist.world == 1 and not args.no_cpu and "cpu" in arms:
        if plain_lines:
            n_plain = next(iter(plain_lines.values()))["sweeps_per_step"]
            if "plain_fp64" in plain_lines:
                n_plain = plain_lines["plain_fp64"]["sweeps_per_step"]
            cpu = cpu_sample(pkg, cs, n_plain, threads)
            line["cpu_baseline"] = {k: cpu[k] for k in ("value", "unit", "cores", "kind", "sample")}
    if net is not None:
        net.close()
    if dist.rank == 0:
        print(json.dumps(line), flush=True)
    dist.close()


if __name__ == "__main__":
    main()
