"""Writes the golden fixtures of tests/golden/ with the CPU oracle.

    python tests/golden/make_golden.py [name ...]      (default: every fixture)

Each fixture stores its inputs and the oracle's outputs (see fixtures.py):

  tiny_fp64         40x32x32 sphere, Re 100: search counts, flags, IB list, 3 FP64 steps
  tiny_outlet_ab2   the same case with the convective outlet and the AB2 predictor, 4 steps
  tiny_moving       the body oscillating transversely, y = 0.15 sin(2 pi 5 t): search and
                    step every step, 6 steps
  poisson24         all-Neumann tanh-clustered 24^3 cube, REDBLACKSOR alone, omega 1.85,
                    residual 1e-8
  sphere96_fp64     96x64x64 sphere, Re 100, dt 0.005, omega 1.8, eps 1e-6: 200 FP64 steps
                    (sweeps and drag/lift of every step; fields after steps 1 and 200)
  sphere96_convective  the same with the convective (Orlanski) outlet

Each sphere96 record takes about half an hour on 8 cores; the others a few seconds.
"""
from __future__ import annotations

import math
import pathlib
import sys
import time

import numpy as np

HERE = pathlib.Path(__file__).resolve().parent
ROOT = HERE.parent.parent
for p in (str(ROOT), str(HERE)):
    if p not in sys.path:
        sys.path.insert(0, p)

import fixtures  # noqa: E402


def _grids():
    import __graft_entry__
    return __graft_entry__._package().grids


def _oracle():
    from oracle import oracle
    return oracle


def _inputs(cs) -> dict:
    nodes, tris = _grids().icosphere(cs.subdivisions, cs.radius)
    return {"x": cs.x, "y": cs.y, "z": cs.z, "nodes": nodes, "tris": tris.astype(np.int64),
            "box": np.array(cs.box, dtype=np.int64), "flow": np.array([cs.re, cs.dt, cs.omega, cs.eps])}


def _counts(c: dict) -> np.ndarray:
    return np.array([c["fluid"], c["solid"], c["ib"], c["red"], c["black"]], dtype=np.int64)


def _steps(o, n: int, out: dict, record_after=()) -> None:
    sweeps, coef = [], []
    for step in range(1, n + 1):
        st, c = o.step(step == 1)
        sweeps.append(st["sweeps"])
        coef.append(np.asarray(c, dtype=np.float64))
        if step in record_after:
            out.update(fixtures.field_record(o.get_field, f"step{step}"))
    out["sweeps"] = np.array(sweeps, dtype=np.int64)
    out["coef"] = np.array(coef)


def make_tiny_fp64() -> dict:
    fx = _inputs(_grids().case("tiny"))
    o = fixtures.build_oracle(_oracle(), fx)
    srch = o.get_search()
    fx["counts"] = _counts(o.counts)
    fx["cell"] = np.asarray(srch["cell"]).astype(np.int8)
    fx["ib"] = np.asarray(srch["ib"], dtype=np.int64)
    fx["nelp"] = np.asarray(srch["nelp"], dtype=np.int64)
    fx["normdis"] = fixtures.summary(np.asarray(srch["normdis"]))
    _steps(o, 3, fx, record_after=(3,))
    o.close()
    return fx


def make_tiny_outlet_ab2() -> dict:
    fx = _inputs(_grids().case("tiny"))
    o = fixtures.build_oracle(_oracle(), fx, outlet=1, momentum=1)
    _steps(o, 4, fx, record_after=(4,))
    o.close()
    return fx


def make_tiny_moving() -> dict:
    cs = _grids().case("tiny")
    fx = _inputs(cs)
    amp, freq, n = 0.15, 5.0, 6
    w = 2.0 * math.pi * freq
    dy = [amp * math.sin(w * s * cs.dt) - amp * math.sin(w * (s - 1) * cs.dt) for s in range(1, n + 1)]
    vs = [amp * w * math.cos(w * s * cs.dt) for s in range(1, n + 1)]
    fx["dy"], fx["vs"] = np.array(dy), np.array(vs)
    o = fixtures.build_oracle(_oracle(), fx)
    counts, sweeps, coef = [], [], []
    for s in range(1, n + 1):
        o.move_body(0.0, dy[s - 1], 0.0, 0.0, vs[s - 1], 0.0)
        counts.append(_counts(o.search(cs.box)))
        st, c = o.step(s == 1)
        sweeps.append(st["sweeps"])
        coef.append(np.asarray(c, dtype=np.float64))
    fx["counts"], fx["sweeps"], fx["coef"] = np.array(counts), np.array(sweeps, dtype=np.int64), np.array(coef)
    fx.update(fixtures.field_record(o.get_field, f"step{n}"))
    o.close()
    return fx


def make_poisson24() -> dict:
    P = _grids().poisson_problem(24, seed=0)
    ax, ay, az = P["acoef"]
    fx = {"x": P["x"], "y": P["y"], "z": P["z"], "acx": ax, "acy": ay, "acz": az, "b": P["b"],
          "solver": np.array([1.85, 1e-8])}
    o = _oracle().Oracle(P["x"], P["y"], P["z"], 100.0, 1.0, omega=1.85, eps=1e-8, criterion=1,
                         max_sweeps=200000, check_every=1)
    o.no_body()
    o.set_acoef(ax, ay, az)
    o.set_field("b", P["b"])
    r = o.redblack_sor()
    fx["sweeps"] = np.array([r["sweeps"]], dtype=np.int64)
    pc = o.get_field("pc")
    fx["pc"] = fixtures.summary(pc)
    fx["pc_sha"] = np.array(fixtures.digest(pc))
    o.close()
    return fx


def make_sphere96_fp64() -> dict:
    cs = _grids().case("sphere96")
    fx = _inputs(cs)
    o = fixtures.build_oracle(_oracle(), fx)
    fx["counts"] = _counts(o.counts)
    fx["cell"] = np.asarray(o.get_search()["cell"]).astype(np.int8)
    _steps(o, cs.steps, fx, record_after=(1, cs.steps))
    o.close()
    return fx


def make_sphere96_convective() -> dict:
    cs = _grids().case("sphere96")
    fx = _inputs(cs)
    o = fixtures.build_oracle(_oracle(), fx, outlet=1)
    fx["counts"] = _counts(o.counts)
    _steps(o, cs.steps, fx, record_after=(1, cs.steps))
    o.close()
    return fx


MAKERS = {"tiny_fp64": make_tiny_fp64, "tiny_outlet_ab2": make_tiny_outlet_ab2, "tiny_moving": make_tiny_moving,
          "poisson24": make_poisson24, "sphere96_fp64": make_sphere96_fp64,
          "sphere96_convective": make_sphere96_convective}


def main(names) -> None:
    import os
    _oracle().set_threads(os.cpu_count() or 1)
    for name in names or MAKERS:
        t = time.time()
        fx = MAKERS[name]()
        np.savez_compressed(fixtures.path(name), **fx)
        print(f"{name}: {fixtures.path(name).stat().st_size} bytes, {time.time() - t:.1f} s", flush=True)


if __name__ == "__main__":
    main(sys.argv[1:])
