"""The CUDA path against the committed golden fixtures (tests/golden/), which the
CPU oracle wrote from the same stored inputs.

The small records must be met bit for bit: search counts and flags, IB list,
sweep counts, drag/lift and the fields' digests. The 200-step records of the
96x64x64 sphere (Re 100, dt 0.005, omega 1.8, eps 1e-6; zero-gradient and
convective outlet) are checked against the parity bar of the plain FP64 path:
velocity and pressure within 1e-8 of each field's magnitude and drag/lift within
1e-6 relative after 200 steps, at every step's sweep count; whether the fields
are also bit-identical is printed."""
from __future__ import annotations

import sys

import numpy as np
import pytest

from conftest import ROOT

sys.path.insert(0, str(ROOT / "tests" / "golden"))
import fixtures  # noqa: E402

pytestmark = pytest.mark.gpu


def _counts(c):
    return [c["fluid"], c["solid"], c["ib"], c["red"], c["black"]]


@pytest.mark.parametrize("name,kw,nsteps", [("tiny_fp64", {}, 3),
                                            ("tiny_outlet_ab2", dict(outlet=1, momentum=1), 4)])
def test_steps_meet_the_record_bit_for_bit(ib3d, name, kw, nsteps):
    fx = fixtures.load(name)
    s = fixtures.build_solver(ib3d, fx, **kw)
    if "cell" in fx:
        assert _counts(s.counts) == fx["counts"].tolist()
        srch = s.get_search()
        assert np.array_equal(np.asarray(srch["cell"]).astype(np.int8), fx["cell"])
        assert np.array_equal(srch["ib"], fx["ib"]) and np.array_equal(srch["nelp"], fx["nelp"])
    for step in range(1, nsteps + 1):
        st, coef = s.step(step == 1)
        assert st["sweeps"] == fx["sweeps"][step - 1], step
        assert np.array_equal(np.asarray(coef), fx["coef"][step - 1]), (step, coef, fx["coef"][step - 1])
    exact = fixtures.compare_fields(s.get_field, fx, f"step{nsteps}", 0.0)
    assert all(exact.values()), exact
    s.close()


def test_moving_body_meets_the_record_bit_for_bit(ib3d):
    fx = fixtures.load("tiny_moving")
    s = fixtures.build_solver(ib3d, fx)
    box = tuple(int(b) for b in fx["box"])
    for q in range(len(fx["dy"])):
        s.move_body(0.0, float(fx["dy"][q]), 0.0, 0.0, float(fx["vs"][q]), 0.0)
        assert _counts(s.search(box)) == fx["counts"][q].tolist(), q
        st, coef = s.step(q == 0)
        assert st["sweeps"] == fx["sweeps"][q], q
        assert np.array_equal(np.asarray(coef), fx["coef"][q]), q
    exact = fixtures.compare_fields(s.get_field, fx, f"step{len(fx['dy'])}", 0.0)
    assert all(exact.values()), exact
    s.close()


def test_poisson_cube_meets_the_record_bit_for_bit(ib3d):
    fx = fixtures.load("poisson24")
    omega, eps = (float(v) for v in fx["solver"])
    p = ib3d.default_params(re=100.0, deltat=1.0, omega=omega, eps=eps, max_sweeps=200000)
    p.criterion, p.check_every = 1, 1
    s = ib3d.Solver(fx["x"], fx["y"], fx["z"], p)
    s.set_poisson_coefficients(fx["acx"], fx["acy"], fx["acz"])
    s.set_field("b", fx["b"])
    r = s.redblack_sor()
    assert r["sweeps"] == fx["sweeps"][0]
    assert fixtures.digest(s.get_field("pc")) == str(fx["pc_sha"])
    s.close()


@pytest.mark.parametrize("name,kw", [("sphere96_fp64", {}), ("sphere96_convective", dict(outlet=1)),
                                     ("sphere96_fp64", dict(precision=2))],
                         ids=["fp64", "fp64-convective", "fp64-fast"])
def test_200_steps_of_the_96_case_meet_the_fp64_parity_bar(ib3d, name, kw):
    """The 96x64x64 sphere at Re 100 for 200 steps, with the reference's active
    zero-gradient outlet and with the convective (Orlanski) outlet, and the fast
    plain FP64 form (contracted multiply-adds, omega/diag per cell) against the same
    record at the same bar."""
    fx = fixtures.load(name)
    s = fixtures.build_solver(ib3d, fx, **kw)
    assert _counts(s.counts) == fx["counts"].tolist()
    if "cell" in fx:
        assert np.array_equal(np.asarray(s.get_search()["cell"]).astype(np.int8), fx["cell"])
    nsteps = len(fx["sweeps"])
    same_sweeps = worst = 0
    for step in range(1, nsteps + 1):
        st, coef = s.step(step == 1)
        same_sweeps += int(st["sweeps"] == fx["sweeps"][step - 1])
        ref = fx["coef"][step - 1]
        cd, cd_ref = coef[0] + coef[1], ref[0] + ref[1]
        cl, cl_ref = coef[2] + coef[3], ref[2] + ref[3]
        worst = max(worst, abs(cd - cd_ref) / abs(cd_ref))
        assert abs(cd - cd_ref) <= 1e-6 * abs(cd_ref), (step, cd, cd_ref)
        assert abs(cl - cl_ref) <= 1e-6 * max(abs(cl_ref), 1e-3 * abs(cd_ref)), (step, cl, cl_ref)
        if step == 1:
            fixtures.compare_fields(s.get_field, fx, "step1", 1e-8)
    exact = fixtures.compare_fields(s.get_field, fx, f"step{nsteps}", 1e-8)
    print(f"{nsteps} steps: sweep counts equal at {same_sweeps}/{nsteps} steps, worst drag error {worst:.2e}, "
          f"fields bit-identical: {exact}")
    s.close()
