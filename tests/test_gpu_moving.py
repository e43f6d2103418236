"""Prescribed body motion (ib3d_move_body): the body oscillates transversely as
y(t) = A sin(2 pi f t); every step shifts the surface nodes, runs the search again
(tagging, cell lists, normal distances, ghost-point schedule) and steps with the
body velocity in the velocity forcing and its acceleration in the pressure
forcing's dpdn. The CUDA path must match the FP64 oracle bit for bit: flags, index
lists, normal distances, every field, sweep counts and drag/lift, at every step."""
from __future__ import annotations

import math

import numpy as np
import pytest

from test_gpu_parity import FIELDS, _pair, _same

pytestmark = pytest.mark.gpu


def motion(t: float, amp: float, freq: float):
    w = 2.0 * math.pi * freq
    return amp * math.sin(w * t), amp * w * math.cos(w * t)


@pytest.mark.parametrize("name", ["tiny", "small"])
def test_oscillating_body_bit_exact(ib3d, oracle_mod, grids, name):
    cs = grids.case(name)
    s, o = _pair(ib3d, oracle_mod, cs)
    amp, freq = 0.15, 5.0     # over 8 steps the body crosses more than one core cell
    flags0 = s.get_search()["cell"]
    changed = 0
    for step in range(1, 9):
        y0, _ = motion((step - 1) * cs.dt, amp, freq)
        y1, v1 = motion(step * cs.dt, amp, freq)
        s.move_body(0.0, y1 - y0, 0.0, 0.0, v1, 0.0)
        o.move_body(0.0, y1 - y0, 0.0, 0.0, v1, 0.0)
        assert s.search(cs.box) == o.search(cs.box), step
        gs, os_ = s.get_search(), o.get_search()
        _same(gs["cell"], os_["cell"], f"step {step} cell flags")
        _same(gs["ib"], os_["ib"], f"step {step} IB list")
        _same(gs["nelp"], os_["nelp"], f"step {step} nelp")
        _same(gs["normdis"], os_["normdis"], f"step {step} normal distances")
        changed = max(changed, int(np.count_nonzero(gs["cell"] != flags0)))
        gst, gcoef = s.step(step == 1)
        ost, ocoef = o.step(step == 1)
        assert gst["sweeps"] == ost["sweeps"], step
        assert np.array_equal(gcoef, ocoef), (step, gcoef, ocoef)
    for f in FIELDS:
        _same(s.get_field(f), o.get_field(f), f"after 8 moving steps {f}")
    assert changed > 0, "the motion never changed a flag"
    s.close()


@pytest.mark.parametrize("name", ["tiny", "small"])
def test_selective_retagging_bit_exact_and_equal_to_the_full_search(ib3d, oracle_mod, grids, name):
    """selectiveRetagging (subSearch.f90:327-512) every step of the oscillating body:
    the CUDA path re-tags only the 6^3 neighbourhoods of the IB cells and must match
    the oracle's restatement of the same routine bit for bit (counts, flags, IB list,
    nearest elements, normal distances, sweeps, drag/lift, fields), and a third
    context re-tagging its whole box after the same moves must reach the same flags
    and lists (the body moves less than a core cell per step)."""
    cs = grids.case(name)
    s, o = _pair(ib3d, oracle_mod, cs)
    full = ib3d.setup_case(cs)
    amp, freq = 0.15, 5.0
    flags0 = s.get_search()["cell"]
    changed = 0
    for step in range(1, 9):
        y0, _ = motion((step - 1) * cs.dt, amp, freq)
        y1, v1 = motion(step * cs.dt, amp, freq)
        for x in (s, o, full):
            x.move_body(0.0, y1 - y0, 0.0, 0.0, v1, 0.0)
        cg = s.selective_retag()
        assert cg == o.selective_retag(), step
        assert cg == full.search(grids.body_box(cs, (0.0, y1, 0.0))), step
        gs, os_, gf = s.get_search(), o.get_search(), full.get_search()
        for key in ("cell", "ib", "nelp", "normdis"):
            _same(gs[key], os_[key], f"step {step} {key} vs oracle")
            _same(gs[key], gf[key], f"step {step} {key} vs full search")
        changed = max(changed, int(np.count_nonzero(gs["cell"] != flags0)))
        gst, gcoef = s.step(step == 1)
        ost, ocoef = o.step(step == 1)
        assert gst["sweeps"] == ost["sweeps"], step
        assert np.array_equal(gcoef, ocoef), (step, gcoef, ocoef)
    for f in FIELDS:
        _same(s.get_field(f), o.get_field(f), f"after 8 moving steps {f}")
    assert changed > 0, "the motion never changed a flag"
    for x in (s, full):
        x.close()


def test_selective_retag_needs_an_ib_list_of_the_same_mesh(ib3d, grids):
    cs = grids.case("tiny")
    s = ib3d.Solver(cs.x, cs.y, cs.z)
    nodes, tris = grids.icosphere(cs.subdivisions, cs.radius)
    s.set_mesh(nodes, tris)
    with pytest.raises(ib3d.IB3DError):
        s.selective_retag()
    s.search(cs.box)
    s.move_body(0.0, 0.01, 0.0)
    s.selective_retag()
    s.set_mesh(nodes, tris)
    with pytest.raises(ib3d.IB3DError):
        s.selective_retag()
    s.close()


def test_step_requires_search_after_move(ib3d, grids):
    cs = grids.case("tiny")
    s = ib3d.setup_case(cs)
    s.move_body(0.0, 0.01, 0.0, 0.0, 1.0, 0.0)
    with pytest.raises(ib3d.IB3DError):
        s.step(True)
    s.search(cs.box)
    s.step(True)
    s.close()


def test_force_driven_motion_bit_exact(ib3d, oracle_mod, grids):
    """shiftSurfaceNodesMovingbody: the body velocity integrates the given force
    (density 1, unit-diameter sphere); the GPU and the oracle move, re-tag and step
    identically."""
    cs = grids.case("tiny")
    s, o = _pair(ib3d, oracle_mod, cs)
    for step in range(1, 5):
        force = (0.0, 40.0 * (-1) ** step, 5.0)
        vg = s.move_body_free(*force)
        vo = o.move_body_free(*force)
        assert np.array_equal(vg, vo)
        assert s.search(cs.box) == o.search(cs.box)
        gst, gcoef = s.step(step == 1)
        ost, ocoef = o.step(step == 1)
        assert gst["sweeps"] == ost["sweeps"] and np.array_equal(gcoef, ocoef), step
    for f in FIELDS:
        _same(s.get_field(f), o.get_field(f), f"after force-driven steps {f}")
    s.close()


def test_mesh_file_gives_the_same_search(ib3d, grids, tmp_path):
    cs = grids.case("tiny")
    nodes, tris = grids.icosphere(cs.subdivisions, cs.radius)
    a = ib3d.setup_case(cs)
    for fmt, writer in ((ib3d.MESH_GMSH, grids.write_gmsh), (ib3d.MESH_GAMBIT, grids.write_gambit)):
        path = tmp_path / f"body{fmt}"
        writer(path, nodes, tris)
        b = ib3d.Solver(cs.x, cs.y, cs.z, ib3d.default_params(re=cs.re, deltat=cs.dt))
        b.set_mesh_file(path, fmt)
        assert b.search(cs.box) == a.counts
        assert np.array_equal(b.get_search()["cell"], a.get_search()["cell"])
        b.close()
    a.close()
