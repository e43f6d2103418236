"""The oracle against its committed golden fixtures (tests/golden/), on the CPU.

The fixtures were written by tests/golden/make_golden.py with this oracle; these
tests keep the oracle (and the generators of the workloads' inputs) from drifting:
rebuilt from the stored inputs, the oracle must give the same search counts and
flags, the same sweep counts, drag/lift within 1e-12 and the same field summaries
within 1e-12 of each field's magnitude (in practice bit for bit; the tolerance only
absorbs a different libm on another host)."""
from __future__ import annotations

import sys

import numpy as np
import pytest

from conftest import ROOT

sys.path.insert(0, str(ROOT / "tests" / "golden"))
import fixtures  # noqa: E402

RTOL = 1e-12


def _coef_close(got, ref, rtol):
    got, ref = np.asarray(got), np.asarray(ref)
    return np.all(np.abs(got - ref) <= rtol * np.maximum(np.abs(ref), 1e-300) + 1e-300)


def test_fixture_inputs_match_the_generators(grids):
    """The stored grids and mesh are what grids.case / grids.icosphere make here."""
    fx = fixtures.load("sphere96_fp64")
    cs = grids.case("sphere96")
    for a in "xyz":
        assert np.allclose(getattr(cs, a), fx[a], rtol=0, atol=1e-13), a
    assert tuple(fx["box"]) == tuple(cs.box)
    nodes, tris = grids.icosphere(cs.subdivisions, cs.radius)
    assert np.array_equal(tris, fx["tris"]) and np.allclose(nodes, fx["nodes"], rtol=0, atol=1e-15)


@pytest.mark.parametrize("name,kw,nsteps", [("tiny_fp64", {}, 3), ("tiny_outlet_ab2", dict(outlet=1, momentum=1), 4)])
def test_oracle_reproduces_steps(oracle_mod, name, kw, nsteps):
    fx = fixtures.load(name)
    o = fixtures.build_oracle(oracle_mod, fx, **kw)
    if "cell" in fx:
        c = o.counts
        assert [c["fluid"], c["solid"], c["ib"], c["red"], c["black"]] == fx["counts"].tolist()
        srch = o.get_search()
        assert np.array_equal(np.asarray(srch["cell"]).astype(np.int8), fx["cell"])
        assert np.array_equal(srch["ib"], fx["ib"]) and np.array_equal(srch["nelp"], fx["nelp"])
    for step in range(1, nsteps + 1):
        st, coef = o.step(step == 1)
        assert st["sweeps"] == fx["sweeps"][step - 1], step
        assert _coef_close(coef, fx["coef"][step - 1], RTOL), (step, coef, fx["coef"][step - 1])
    fixtures.compare_fields(o.get_field, fx, f"step{nsteps}", RTOL)
    o.close()


def test_oracle_reproduces_moving_body(oracle_mod):
    fx = fixtures.load("tiny_moving")
    o = fixtures.build_oracle(oracle_mod, fx)
    box = tuple(int(b) for b in fx["box"])
    for s in range(len(fx["dy"])):
        o.move_body(0.0, float(fx["dy"][s]), 0.0, 0.0, float(fx["vs"][s]), 0.0)
        c = o.search(box)
        assert [c["fluid"], c["solid"], c["ib"], c["red"], c["black"]] == fx["counts"][s].tolist(), s
        st, coef = o.step(s == 0)
        assert st["sweeps"] == fx["sweeps"][s]
        assert _coef_close(coef, fx["coef"][s], RTOL), s
    fixtures.compare_fields(o.get_field, fx, f"step{len(fx['dy'])}", RTOL)
    o.close()


def test_oracle_reproduces_poisson_cube(oracle_mod):
    fx = fixtures.load("poisson24")
    omega, eps = (float(v) for v in fx["solver"])
    o = oracle_mod.Oracle(fx["x"], fx["y"], fx["z"], 100.0, 1.0, omega=omega, eps=eps, criterion=1,
                          max_sweeps=200000, check_every=1)
    o.no_body()
    o.set_acoef(fx["acx"], fx["acy"], fx["acz"])
    o.set_field("b", fx["b"])
    r = o.redblack_sor()
    assert r["sweeps"] == fx["sweeps"][0]
    pc = o.get_field("pc")
    got = fixtures.summary(pc)
    assert np.max(np.abs(got[2:] - fx["pc"][2:])) <= RTOL * fx["pc"][2]
    o.close()


@pytest.mark.parametrize("name,kw", [("sphere96_fp64", {}), ("sphere96_convective", dict(outlet=1))])
def test_oracle_reproduces_first_step_of_the_96_case(oracle_mod, name, kw):
    """Step 1 of the 96x64x64 sphere (the 200-step records are checked on the GPU)."""
    fx = fixtures.load(name)
    o = fixtures.build_oracle(oracle_mod, fx, **kw)
    c = o.counts
    assert [c["fluid"], c["solid"], c["ib"], c["red"], c["black"]] == fx["counts"].tolist()
    if "cell" in fx:
        assert np.array_equal(np.asarray(o.get_search()["cell"]).astype(np.int8), fx["cell"])
    st, coef = o.step(True)
    assert st["sweeps"] == fx["sweeps"][0]
    assert _coef_close(coef, fx["coef"][0], RTOL)
    fixtures.compare_fields(o.get_field, fx, "step1", RTOL)
    o.close()
