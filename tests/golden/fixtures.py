"""Golden fixtures of the FP64 path, made by the CPU oracle (make_golden.py).

The reference ships no tests, fixtures or golden outputs and cannot be run here,
so these files pin the oracle and the CUDA path against a fixed record instead:
each fixture stores its inputs (grid node coordinates, the surface mesh, the
search box and the solver settings, so that no machine regenerates them with its
own libm) and the oracle's outputs -- search counts and flags, SOR sweep counts
and drag/lift per step, and summaries of the fields after chosen steps.

A field summary is exact and order-independent: the correctly rounded sum and sum
of squares (math.fsum), the largest magnitude, 64 values at seeded positions and
the SHA-256 of the array's bytes.
"""
from __future__ import annotations

import hashlib
import math
import pathlib

import numpy as np

HERE = pathlib.Path(__file__).resolve().parent
FIELDS = ("u", "v", "w", "p")
NSAMPLE = 64


def path(name: str) -> pathlib.Path:
    return HERE / f"{name}.npz"


def load(name: str) -> dict:
    with np.load(path(name), allow_pickle=False) as z:
        return {k: z[k] for k in z.files}


def summary(a: np.ndarray) -> np.ndarray:
    """[sum, sum of squares, max |a|, 64 sampled values] (float64), see module doc."""
    flat = np.ascontiguousarray(a, dtype=np.float64).ravel()
    idx = np.random.default_rng(0).choice(flat.size, size=min(NSAMPLE, flat.size), replace=False)
    head = [math.fsum(flat.tolist()), math.fsum((flat * flat).tolist()), float(np.max(np.abs(flat)))]
    return np.concatenate([np.array(head), flat[np.sort(idx)]])


def digest(a: np.ndarray) -> str:
    return hashlib.sha256(np.ascontiguousarray(a, dtype="<f8").tobytes()).hexdigest()


def field_record(get_field, prefix: str) -> dict:
    """Summaries (and digests) of u, v, w, p under keys '<prefix>_<field>' and '<prefix>_<field>_sha'."""
    out = {}
    for f in FIELDS:
        a = get_field(f)
        out[f"{prefix}_{f}"] = summary(a)
        out[f"{prefix}_{f}_sha"] = np.array(digest(a))
    return out


def compare_fields(get_field, fx: dict, prefix: str, rtol: float) -> dict:
    """Checks u, v, w, p against the fixture's summaries: every entry within rtol of
    the field's largest magnitude. Returns {field: bit-identical (digest equal)}."""
    exact = {}
    for f in FIELDS:
        a = get_field(f)
        got, ref = summary(a), fx[f"{prefix}_{f}"]
        scale = max(ref[2], 1e-300)
        # sums scale with the cell count: compare them relative to their own size
        assert abs(got[0] - ref[0]) <= rtol * max(abs(ref[0]), scale * a.size ** 0.5), (prefix, f, "sum", got[0], ref[0])
        assert abs(got[1] - ref[1]) <= rtol * ref[1] + 1e-300, (prefix, f, "sumsq", got[1], ref[1])
        err = np.max(np.abs(got[2:] - ref[2:]))
        assert err <= rtol * scale, (prefix, f, "values", err, scale)
        exact[f] = digest(a) == str(fx[f"{prefix}_{f}_sha"])
    return exact


def build_oracle(oracle_mod, fx: dict, **kw):
    """Oracle from a fixture's stored inputs: grid, mesh, search and initial conditions."""
    re, dt, omega, eps = (float(v) for v in fx["flow"])
    o = oracle_mod.Oracle(fx["x"], fx["y"], fx["z"], re, dt, omega=omega, eps=eps, **kw)
    o.set_mesh(fx["nodes"], fx["tris"])
    o.search(tuple(int(b) for b in fx["box"]))
    o.initial_conditions()
    return o


def build_solver(ib3d, fx: dict, **kw):
    """CUDA solver from a fixture's stored inputs, same sequence as build_oracle."""
    re, dt, omega, eps = (float(v) for v in fx["flow"])
    p = ib3d.default_params(re=re, deltat=dt, omega=omega, eps=eps)
    for k, v in kw.items():
        setattr(p, k, v)
    s = ib3d.Solver(fx["x"], fx["y"], fx["z"], p)
    s.set_mesh(fx["nodes"], fx["tris"])
    s.search(tuple(int(b) for b in fx["box"]))
    s.initial_conditions()
    return s
