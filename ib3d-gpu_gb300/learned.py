"""Training and evaluation of the learned warm start (the ib3d_net entry points).

The network is trained on snapshots the solver generates: runs of a sphere case at
several Reynolds numbers, each started from u = 1 with a seeded 1 % random
perturbation of the initial streamwise velocity, solved with the previous
correction as warm start while ib3d_net_capture stores random patches of S^3
voxels (each voxel the average of 2x2x2 cells) of every step: the inputs and the
solved change of the correction. Training is Adam on random
batches of those patches. Evaluation runs a held-out Reynolds number twice, once
warm-started from the previous correction and once from the network, and compares
the SOR sweeps and the drag/lift at the same FP64 residual tolerance.
"""
from __future__ import annotations

import dataclasses
import time

import numpy as np

from . import Net, Solver, setup_case, WARM_PREV, WARM_LEARNED, PREC_FP32DC, CRIT_RESIDUAL


def solver_options(**kw) -> dict:
    """FP32 sweeps in FP64 defect correction, residual stopping test."""
    opts = dict(precision=PREC_FP32DC, criterion=CRIT_RESIDUAL, inner_sweeps=256, omega_inner=1.994,
                sweep_kernel=0, max_sweeps=400000)
    opts.update(kw)
    return opts


def perturbed_run(cs, re: float, seed: int, amplitude: float = 0.01, **opts) -> Solver:
    """Solver for case cs at Reynolds number re, u = 1 + amplitude * N(0,1) at t = 0."""
    c = dataclasses.replace(cs, re=re)
    s = setup_case(c, **opts)
    if amplitude:
        u = s.get_field("u")
        rng = np.random.default_rng(seed)
        u = u + amplitude * rng.standard_normal(u.shape)
        s.set_field("u", u)
    return s


def generate(net: Net, cs, reynolds, steps: int, patches_per_step: int, first_capture: int = 3,
             seed: int = 0, **opts) -> dict:
    """Runs cs at each Reynolds number for `steps` steps and captures patches of every
    step from `first_capture` on. Returns counts and timings."""
    t0 = time.perf_counter()
    sweeps = []
    for re in reynolds:
        s = perturbed_run(cs, re, seed=int(re) + seed, **solver_options(warm_start=WARM_PREV, **opts))
        s.enable_history()
        for q in range(1, steps + 1):
            st, _ = s.step(q == 1)
            sweeps.append(st["sweeps"])
            if q >= first_capture:
                net.capture(s, patches_per_step, seed=1000 * int(re) + q + seed)
        s.close()
    return {"patches": net.dataset_size(), "seconds": time.perf_counter() - t0, "sweeps": sweeps}


def generate_windows(net: Net, cs, reynolds, windows, patches_per_step: int, seed: int = 0, **opts) -> dict:
    """Runs cs at each Reynolds number from the impulsive start to the end of the last
    window and captures patches of every step inside the windows ((first, last) step
    numbers, 1-based): the transient after the start and the developed wake later on."""
    t0 = time.perf_counter()
    last = max(b for _, b in windows)
    sweeps = []
    for re in reynolds:
        s = perturbed_run(cs, re, seed=int(re) + seed, **solver_options(warm_start=WARM_PREV, **opts))
        s.enable_history()
        for q in range(1, last + 1):
            st, _ = s.step(q == 1)
            if any(a <= q <= b for a, b in windows):
                sweeps.append(st["sweeps"])
                net.capture(s, patches_per_step, seed=1000 * int(re) + q + seed)
        s.close()
    return {"patches": net.dataset_size(), "seconds": time.perf_counter() - t0, "sweeps": sweeps}


def evaluate_developed(net: Net, cs, re: float, spinup: int, steps: int, path: str, seed: int = 7,
                       **opts) -> dict:
    """Held-out run at re spun up for `spinup` steps (previous-correction warm start)
    and saved to the restart file `path`; then both warm starts continue from it for
    `steps` steps. The first two steps after the restart have no history for the
    network (both arms then start from zero and from the previous correction), so the
    comparison is over the steps after them."""
    s = perturbed_run(cs, re, seed=seed, **solver_options(warm_start=WARM_PREV, **opts))
    for q in range(1, spinup + 1):
        s.step(q == 1)
    s.write_restart(path, totime=spinup * cs.dt, ita=spinup, ita1=spinup)
    s.close()
    out = {}
    for name, mode in (("prev", WARM_PREV), ("learned", WARM_LEARNED)):
        s = setup_case(dataclasses.replace(cs, re=re), **solver_options(warm_start=mode, **opts))
        if mode == WARM_LEARNED:
            s.attach_net(net)
        s.read_restart(path)
        sw, coefs = [], []
        for q in range(1, steps + 1):
            st, coef = s.step(q == 1)
            sw.append(st["sweeps"])
            coefs.append(list(coef))
        s.close()
        out[name] = {"sweeps": sw, "coef": coefs}
    return out


def train(net: Net, steps: int, batch: int = 8, lr: float = 1e-3, chunk: int = 100, seed: int = 0) -> dict:
    """Adam steps in chunks (the loss of each chunk's last step is recorded)."""
    t0 = time.perf_counter()
    losses = []
    done = 0
    while done < steps:
        n = min(chunk, steps - done)
        losses.append(net.train(n, batch=batch, lr=lr, seed=seed + done))
        done += n
    return {"losses": losses, "seconds": time.perf_counter() - t0, "steps": steps}


def evaluate(net: Net, cs, re: float, steps: int, seed: int = 7, **opts) -> dict:
    """Held-out run at re, previous-correction warm start against the network's.
    Both stop at the same FP64 residual; returns sweeps per step and drag/lift."""
    out = {}
    for name, mode in (("prev", WARM_PREV), ("learned", WARM_LEARNED)):
        s = perturbed_run(cs, re, seed=seed, **solver_options(warm_start=mode, **opts))
        if mode == WARM_LEARNED:
            s.attach_net(net)
        sw, coefs, secs, r0 = [], [], [], []
        for q in range(1, steps + 1):
            t = time.perf_counter()
            st, coef = s.step(q == 1)
            secs.append(time.perf_counter() - t)
            sw.append(st["sweeps"])
            r0.append(st["initial_err"])
            coefs.append(list(coef))
        s.close()
        out[name] = {"sweeps": sw, "coef": coefs, "seconds": secs, "initial_err": r0}
    return out
