"""The headline form against the plain FP64 path at the benchmarked configuration.

Workload: the bench's 256x192x192 sphere (D/40 core, dt 0.002, relaxation 1.99,
FP64 residual L-inf <= 1e-6) at Re 275, the Reynolds number the shipped network
never saw in training, from the impulsive start u = 1. The plain FP64 path
(reference arithmetic, bit-identical to the oracle, zero initial correction) and
the headline form (FP32 red-black sweeps inside FP64 defect correction, the bench's
pass schedule, Gauss-Seidel smoothing and relaxation ramp, learned warm start with
the default network) run the same 8 steps. At every step both solves must end below
the residual tolerance, and the drag and lift of the headline form must lie within
1e-4 relative of the plain path's (the required bar for the mixed-precision and
learned forms). After the last step u, v, w and p must agree within 1e-7 of each
field's largest magnitude (measured: ~1e-9 after 20 steps).

Reference: stressCal1/2 (subStressCal1.f90:2-460, subStressCal2.f90:2-381) for the
coefficients, REDBLACKSOR (subPcorVcor.f90:148-212) for the solve.
"""
from __future__ import annotations

import importlib.util

import numpy as np
import pytest

from conftest import ROOT

pytestmark = pytest.mark.gpu

STEPS = 8
FIELD_RTOL = 1e-7
COEF_RTOL = 1e-4


def _bench():
    spec = importlib.util.spec_from_file_location("ib3d_bench", ROOT / "bench.py")
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    return mod


def test_headline_form_matches_plain_fp64_at_the_bench_configuration(ib3d):
    bench = _bench()
    cs = bench.workload(ib3d, "sphere256", bench.HEADLINE_RE)
    net = bench.load_net(ib3d)
    assert net is not None, "the package's default network is missing"
    plain = ib3d.setup_case(cs, **bench.PLAIN)
    head = ib3d.setup_case(cs, **dict(bench.FAST, warm_start=ib3d.WARM_LEARNED))
    head.attach_net(net)
    head.timers_enable(True)
    worst_cd = worst_cl = 0.0
    for step in range(1, STEPS + 1):
        sa, ca = plain.step(step == 1)
        sb, cb = head.step(step == 1)
        assert sa["final_err"] < cs.eps, (step, sa)
        assert sb["final_err"] < cs.eps, (step, sb)
        cd_ref, cd = ca[0] + ca[1], cb[0] + cb[1]
        cl_ref, cl = ca[2] + ca[3], cb[2] + cb[3]
        worst_cd = max(worst_cd, abs(cd - cd_ref) / abs(cd_ref))
        worst_cl = max(worst_cl, abs(cl - cl_ref) / max(abs(cl_ref), 1e-3 * abs(cd_ref)))
        assert abs(cd - cd_ref) <= COEF_RTOL * abs(cd_ref), (step, cd, cd_ref)
        assert abs(cl - cl_ref) <= COEF_RTOL * max(abs(cl_ref), 1e-3 * abs(cd_ref)), (step, cl, cl_ref)
    assert head.timers_read()["net_ms"] > 0.0   # the network ran
    errs = {}
    for f in ("u", "v", "w", "p"):
        a, b = plain.get_field(f), head.get_field(f)
        errs[f] = float(np.max(np.abs(a - b)) / np.max(np.abs(a)))
        assert errs[f] <= FIELD_RTOL, (f, errs[f])
    print(f"{STEPS} steps at Re {cs.re:g}: worst drag error {worst_cd:.2e}, worst lift error {worst_cl:.2e}, "
          f"fields {errs}")
    for x in (plain, head, net):
        x.close()


def test_fast_plain_fp64_matches_the_reference_arithmetic_at_the_bench_configuration(ib3d):
    """The fast plain FP64 form (contracted multiply-adds, omega/diag per cell) over
    4 steps of the same workload: drag within 1e-6 and fields within 1e-8 of the
    bit-identical path (the required bar for the plain path)."""
    bench = _bench()
    cs = bench.workload(ib3d, "sphere256", bench.HEADLINE_RE)
    a = ib3d.setup_case(cs, **bench.PLAIN)
    b = ib3d.setup_case(cs, **bench.PLAIN_FAST)
    for step in range(1, 5):
        sa, ca = a.step(step == 1)
        sb, cb = b.step(step == 1)
        assert sb["final_err"] < cs.eps
        cd_ref, cd = ca[0] + ca[1], cb[0] + cb[1]
        assert abs(cd - cd_ref) <= 1e-6 * abs(cd_ref), (step, cd, cd_ref, sa["sweeps"], sb["sweeps"])
    for f in ("u", "v", "w", "p"):
        x, y = a.get_field(f), b.get_field(f)
        assert np.max(np.abs(x - y)) <= 1e-8 * np.max(np.abs(x)), f
    a.close()
    b.close()
