"""Parity of the CUDA hot path (through the C ABI) with the FP64 oracle.

The FP64 path must be bit-identical to the oracle: search flags, index lists and
normal distances; every per-step routine; whole steps including the SOR sweep
count and the drag/lift coefficients. The mixed-precision path is checked
against the FP64 path at the same FP64 residual tolerance (drag within 1e-4
relative).
"""
from __future__ import annotations

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

FIELDS = ("u", "v", "w", "ut", "vt", "wt", "p")


def _pair(ib3d, oracle_mod, cs, **kw):
    o = oracle_mod.setup_case(cs, **{k: v for k, v in kw.items() if k in ("criterion", "eps", "max_sweeps",
                                                                           "check_every", "omega", "outlet",
                                                                           "momentum")})
    s = ib3d.setup_case(cs, **kw)
    return s, o


def _same(a, b, what):
    assert a.shape == b.shape, what
    bad = np.argwhere(~(a == b))
    assert bad.size == 0, f"{what}: {len(bad)} mismatches, first at {bad[0]} ({a[tuple(bad[0])]} vs {b[tuple(bad[0])]})"


@pytest.mark.parametrize("name", ["tiny", "small"])
def test_search_bit_exact(ib3d, oracle_mod, grids, name):
    cs = grids.case(name)
    s, o = _pair(ib3d, oracle_mod, cs)
    assert s.counts == o.counts
    gs, os_ = s.get_search(), o.get_search()
    _same(gs["cell"], os_["cell"], "cell flags")
    _same(gs["ib"], os_["ib"], "interceptedIndexPtr")
    _same(gs["nelp"], os_["nelp"], "nelp")
    _same(gs["normdis"], os_["normdis"], "normal distances")
    s.close()


def test_initial_conditions_and_momentum_bit_exact(ib3d, oracle_mod, grids):
    cs = grids.case("small")
    s, o = _pair(ib3d, oracle_mod, cs)
    for f in FIELDS:
        _same(s.get_field(f), o.get_field(f), f"initial {f}")
    s.ns_momentum(); o.ns_momentum()
    for f in ("ut", "vt", "wt"):
        _same(s.get_field(f), o.get_field(f), f"momentum {f}")
    s.velocity_bc(); o.velocity_bc()
    s.solid_cell_bc(); o.solid_cell_bc()
    for f in ("ut", "vt", "wt", "p"):
        _same(s.get_field(f), o.get_field(f), f"bc {f}")
    s.velocity_forcing(); o.velocity_forcing()
    for f in ("ut", "vt", "wt"):
        _same(s.get_field(f), o.get_field(f), f"velocity forcing {f}")
    s.close()


def test_momentum_on_random_fields_bit_exact(ib3d, oracle_mod, grids):
    """Random velocity and pressure fields exercise every branch of the predictor
    (third- and first-order upwinding, both signs of the advecting velocity)."""
    cs = grids.case("tiny")
    s, o = _pair(ib3d, oracle_mod, cs)
    rng = np.random.default_rng(7)
    for f in ("u", "v", "w", "p"):
        a = np.asfortranarray(rng.standard_normal(s.shape))
        s.set_field(f, a); o.set_field(f, a)
    s.ns_momentum(); o.ns_momentum()
    for f in ("ut", "vt", "wt"):
        _same(s.get_field(f), o.get_field(f), f"momentum {f}")
    s.close()


def test_fast_momentum_matches_reference_arithmetic(ib3d, grids):
    """The mixed-precision path's momentum kernel (1-D reciprocal tables, contracted
    multiply-adds) agrees with the bit-parity kernel to rounding: relative 1e-12."""
    cs = grids.case("small")
    s = ib3d.setup_case(cs)
    rng = np.random.default_rng(3)
    for f in ("u", "v", "w", "p"):
        s.set_field(f, np.asfortranarray(rng.standard_normal(s.shape)))
    s.ns_momentum()
    ref = {f: s.get_field(f) for f in ("ut", "vt", "wt")}
    s.set_params(precision=ib3d.PREC_FP32DC)
    for f in ("ut", "vt", "wt"):
        s.set_field(f, np.zeros(s.shape))
    s.ns_momentum()
    cell = s.get_search()["cell"]
    fluid = cell == 0
    for f in ("ut", "vt", "wt"):
        got = s.get_field(f)
        err = np.abs(got - ref[f])[fluid].max() / np.abs(ref[f][fluid]).max()
        assert err < 1e-12, (f, err)
    s.close()


def test_forcing_serial_semantics_on_random_fields(ib3d, oracle_mod, grids):
    """Random ut/vt/wt/p make every read-after-write between ghost points visible:
    the level-scheduled forcing must reproduce the serial loop exactly."""
    cs = grids.case("small")
    s, o = _pair(ib3d, oracle_mod, cs)
    rng = np.random.default_rng(11)
    for f in ("ut", "vt", "wt", "p"):
        a = np.asfortranarray(rng.standard_normal(s.shape))
        s.set_field(f, a); o.set_field(f, a)
    s.velocity_forcing(); o.velocity_forcing()
    s.pressure_forcing(); o.pressure_forcing()
    for f in ("ut", "vt", "wt", "p"):
        _same(s.get_field(f), o.get_field(f), f"forcing {f}")
    s.close()


@pytest.mark.parametrize("criterion", [0, 1])
def test_poisson_solver_bit_exact(ib3d, oracle_mod, grids, criterion):
    cs = grids.case("tiny")
    kw = dict(criterion=criterion, check_every=3) if criterion else {}
    s, o = _pair(ib3d, oracle_mod, cs, **kw)
    for x in (s, o):
        x.ns_momentum(); x.velocity_bc(); x.solid_cell_bc(); x.velocity_forcing(); x.velocity_bc()
    gs = s.poisson_solver()
    os_ = o.poisson_solver()
    assert gs["sweeps"] == os_["sweeps"]
    assert gs["divmax"] == os_["divmax"] and gs["derr_std_st"] == os_["derr_std_st"]
    assert gs["final_err"] == os_["final_err"]
    for f in ("pc", "b", "p", "u", "v", "w", "ut", "vt", "wt"):
        _same(s.get_field(f), o.get_field(f), f"poisson {f}")
    s.close()


def test_steps_bit_exact(ib3d, oracle_mod, grids):
    """Whole time steps (main.f90:42-66): fields, sweep counts and drag/lift."""
    cs = grids.case("small")
    s, o = _pair(ib3d, oracle_mod, cs)
    for step in range(1, 4):
        gst, gcoef = s.step(step == 1)
        ost, ocoef = o.step(step == 1)
        assert gst["sweeps"] == ost["sweeps"], step
        assert np.array_equal(gcoef, ocoef), (step, gcoef, ocoef)
    for f in FIELDS:
        _same(s.get_field(f), o.get_field(f), f"after 3 steps {f}")
    s.close()


def test_noconv_is_reported_with_valid_fields(ib3d, grids):
    cs = grids.case("tiny")
    s = ib3d.setup_case(cs, max_sweeps=5)
    st, _ = s.step(True, allow_noconv=True)
    assert st["rc"] == ib3d.ERR_NOCONV and st["sweeps"] == 5
    assert np.all(np.isfinite(s.get_field("p")))
    s.close()


def test_bad_mesh_index_is_rejected(ib3d, grids):
    cs = grids.case("tiny")
    s = ib3d.Solver(cs.x, cs.y, cs.z, ib3d.default_params(re=cs.re, deltat=cs.dt))
    nodes, tris = grids.icosphere(1, 0.5)
    tris = tris.copy()
    tris[3, 1] = len(nodes) + 5
    with pytest.raises(ib3d.IB3DError) as e:
        s.set_mesh(nodes, tris)
    assert e.value.code == ib3d.ERR_MESH
    s.close()


def test_probe_outside_grid_is_reported(ib3d, grids):
    """A body whose surface lies in the first cell, with its normal pointing out of
    the domain, sends ghost-point probes off the grid: the search reports
    IB3D_ERR_PROBE instead of reading out of bounds."""
    cs = grids.case("tiny")
    s = ib3d.Solver(cs.x, cs.y, cs.z, ib3d.default_params(re=cs.re, deltat=cs.dt))
    x0 = cs.x[0]
    assert cs.x[1] - x0 > 0.3
    nodes, tris = grids.icosphere(3, 0.5, centre=(x0 + 0.65, 0.0, 0.0))
    s.set_mesh(nodes, tris)
    with pytest.raises(ib3d.IB3DError) as e:
        s.search((2, 12, 2, s.ny + 1, 2, s.nz + 1))
    assert e.value.code == ib3d.ERR_PROBE
    s.close()


def test_mixed_precision_matches_fp64_drag(ib3d, grids):
    """FP32 sweeps inside FP64 defect correction, stopped at the same FP64
    residual tolerance as the FP64 path: drag/lift within 1e-4 relative."""
    cs = grids.case("small")
    common = dict(criterion=ib3d.CRIT_RESIDUAL, eps=1e-6, check_every=1)
    s64 = ib3d.setup_case(cs, precision=ib3d.PREC_FP64, **common)
    s32 = ib3d.setup_case(cs, precision=ib3d.PREC_FP32DC, inner_sweeps=40, **common)
    for step in range(1, 6):
        st64, c64 = s64.step(step == 1)
        st32, c32 = s32.step(step == 1)
        assert st32["final_err"] < 1e-6 and st64["final_err"] < 1e-6
    cd64, cd32 = c64[0] + c64[1], c32[0] + c32[1]
    assert abs(cd32 - cd64) <= 1e-4 * abs(cd64), (cd64, cd32)
    assert np.max(np.abs(s32.get_field("u") - s64.get_field("u"))) < 1e-4
    s64.close(); s32.close()


@pytest.mark.parametrize("name,kernel,inner", [("tiny", 0, 7), ("small", 0, 7), ("small", 0, 40), ("tiny", 2, 7),
                                               ("small", 2, 7), ("small", 3, 7), ("small", 3, 40), ("tiny", 4, 7),
                                               ("small", 4, 7)])
def test_packed_fp32_sweep_matches_padded_layout(ib3d, grids, name, kernel, inner):
    """The FP32 sweep on colour-packed arrays (two colour passes with two rows per
    thread, kernel 0; with one row per thread and the loads free of branches, kernel 3,
    or behind branches, kernel 4; or one fused z-wavefront launch per sweep, kernel 2)
    performs the same red-then-black update with the same FP32 operation order as the
    sweep on the padded field layout, so whole mixed-precision steps agree bit for bit.
    Passes of 40 sweeps run 32 of them as one replay of the captured sweep graph."""
    cs = grids.case(name)
    common = dict(precision=ib3d.PREC_FP32DC, criterion=ib3d.CRIT_RESIDUAL, eps=1e-6, inner_sweeps=7)
    a = ib3d.setup_case(cs, sweep_kernel=kernel, **dict(common, inner_sweeps=inner))
    b = ib3d.setup_case(cs, sweep_kernel=1, **dict(common, inner_sweeps=inner))
    for step in range(1, 4):
        sa, ca = a.step(step == 1)
        sb, cb = b.step(step == 1)
        assert sa["sweeps"] == sb["sweeps"] and sa["outer"] == sb["outer"], step
        assert np.array_equal(ca, cb), (step, ca, cb)
    for f in ("u", "v", "w", "p", "pc"):
        _same(a.get_field(f), b.get_field(f), f)
    a.close(); b.close()


def test_warm_start_previous_correction(ib3d, grids):
    cs = grids.case("small")
    common = dict(criterion=ib3d.CRIT_RESIDUAL, eps=1e-6)
    s0 = ib3d.setup_case(cs, **common)
    s1 = ib3d.setup_case(cs, warm_start=ib3d.WARM_PREV, **common)
    n0 = n1 = 0
    for step in range(1, 6):
        st0, c0 = s0.step(step == 1)
        st1, c1 = s1.step(step == 1)
        n0 += st0["sweeps"]; n1 += st1["sweeps"]
    assert abs((c1[0] + c1[1]) - (c0[0] + c0[1])) <= 1e-4 * abs(c0[0] + c0[1])
    s0.close(); s1.close()


def test_download_matches_get_field(ib3d, grids):
    cs = grids.case("tiny")
    s = ib3d.setup_case(cs)
    s.step(True)
    d = s.download_fields()
    for f in FIELDS:
        _same(d[f], s.get_field(f), f)
    s.close()


def test_async_download_holds_the_fields_of_its_step(ib3d, grids):
    """ib3d_download_fields_async snapshots the fields on the device, so the host
    buffers receive the fields of the step it was called after even while the next
    steps run and change them; two calls in a row keep their order."""
    import torch
    cs = grids.case("small")
    s = ib3d.setup_case(cs, precision=ib3d.PREC_FP32DC, criterion=ib3d.CRIT_RESIDUAL, eps=1e-6)
    names = ("u", "v", "w", "ut", "vt", "wt", "p")
    n3 = s.shape[0] * s.shape[1] * s.shape[2]

    def pinned():
        return torch.empty(n3, dtype=torch.float64, pin_memory=True).numpy().reshape(s.shape, order="F")

    a, b = {f: pinned() for f in names}, {f: pinned() for f in names}
    s.step(True)
    ref1 = s.download_fields()
    s.download_fields_async(a)
    s.step(False)
    ref2 = s.download_fields()
    s.download_fields_async(b)
    s.step(False)
    s.step(False)
    s.download_wait()
    for f in names:
        _same(a[f], ref1[f], f)
        _same(b[f], ref2[f], f)
    assert not np.array_equal(ref1["u"], ref2["u"])
    s.close()


@pytest.mark.parametrize("outlet,momentum", [(1, 0), (0, 1), (1, 1)])
def test_convective_outlet_and_ab2_steps_bit_exact(ib3d, oracle_mod, grids, outlet, momentum):
    """The reference's optional branches: Orlanski outlet with calculateUc after each
    step (subBoundaryConditions.f90:153-155, subCalculateuc.f90:2-38) and the
    Adams-Bashforth predictor nsMomentumAB after the first step
    (subNavierStokes.f90:1128-1628), whole steps bit for bit."""
    cs = grids.case("small")
    s, o = _pair(ib3d, oracle_mod, cs, outlet=outlet, momentum=momentum)
    for step in range(1, 5):
        gst, gcoef = s.step(step == 1)
        ost, ocoef = o.step(step == 1)
        assert gst["sweeps"] == ost["sweeps"], step
        assert np.array_equal(gcoef, ocoef), (step, gcoef, ocoef)
    for f in FIELDS:
        _same(s.get_field(f), o.get_field(f), f"outlet {outlet} momentum {momentum}: {f}")
    if outlet:
        assert s.calculate_uc() == o.calculate_uc()
    s.close()


def test_ab2_differs_from_euler_after_the_first_step(ib3d, grids):
    cs = grids.case("tiny")
    e = ib3d.setup_case(cs)
    a = ib3d.setup_case(cs, momentum=ib3d.MOMENTUM_AB2)
    for step in (1, 2):
        e.step(step == 1)
        a.step(step == 1)
        if step == 1:
            assert np.array_equal(e.get_field("u"), a.get_field("u"))
    assert not np.array_equal(e.get_field("u"), a.get_field("u"))
    e.close()
    a.close()
