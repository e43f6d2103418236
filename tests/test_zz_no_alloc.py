"""The allocation-free pressure solve (ib3d_pressure_solve_noalloc).

It exists for host codes that cannot call cudaMalloc themselves or through the
library -- device memory owned by another runtime, or no allocation allowed in
the time loop -- so it keeps its scratch in a static device array. Here the
caller's arrays are torch tensors (the caller may allocate; the entry point
does not). Two calls in a row are compared with the context-based
ib3d_poisson_solver in the same mixed-precision mode: the second call checks
that the scratch left by the first one is cleared. This file is named so that
pytest collects it last.
"""
from __future__ import annotations

import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def test_noalloc_solve_matches_poisson_solver_on_two_calls(ib3d, grids, oracle_mod):
    import torch

    cs = grids.case("tiny")
    inner = 16
    s = ib3d.setup_case(cs, precision=ib3d.PREC_FP32DC, criterion=ib3d.CRIT_RESIDUAL, eps=1e-7,
                        inner_sweeps=inner, sweep_kernel=1)
    n3 = int(np.prod(s.shape))
    assert n3 <= 1 << 21
    # the Poisson coefficients (coefficientMatrix) from the oracle, as device arrays
    o = oracle_mod.Oracle(cs.x, cs.y, cs.z, cs.re, cs.dt)
    coefs = [torch.from_numpy(np.ascontiguousarray(o.acoef(a).ravel(order="F"))).cuda() for a in range(3)]
    cell = torch.from_numpy(s.get_search()["cell"].ravel(order="F").astype(np.uint8)).cuda()
    L = ib3d.lib()
    for call in range(2):
        # advance the context to a fresh right-hand side and solve it there
        s.ns_momentum(); s.velocity_bc(); s.solid_cell_bc(); s.velocity_forcing(); s.velocity_bc()
        ref = s.poisson_solver()
        b = torch.from_numpy(s.get_field("b").ravel(order="F")).cuda()
        pc = torch.zeros(n3, dtype=torch.float64, device="cuda")
        sweeps = np.zeros(1, np.int64)
        resid = np.zeros(1, np.float64)
        rc = L.ib3d_pressure_solve_noalloc(s.nx, s.ny, s.nz, coefs[0].data_ptr(), coefs[1].data_ptr(),
                                           coefs[2].data_ptr(), cell.data_ptr(), b.data_ptr(), cs.dt,
                                           pc.data_ptr(), cs.omega, 1e-7, 1_000_000, inner, None,
                                           sweeps.ctypes.data_as(C.POINTER(C.c_int64)),
                                           resid.ctypes.data_as(C.POINTER(C.c_double)))
        torch.cuda.synchronize()
        assert rc == ib3d.OK, rc
        got = pc.cpu().numpy().reshape(s.shape, order="F")
        want = s.get_field("pc")
        assert int(sweeps[0]) == ref["sweeps"], (call, sweeps[0], ref["sweeps"])
        assert resid[0] < 1e-7
        scale = max(1.0, float(np.abs(want).max()))
        assert np.abs(got - want).max() <= 1e-6 * scale, (call, np.abs(got - want).max())
        s.pressure_forcing()
        s.stress(call == 0)
    s.close()


def test_noalloc_rejects_grids_beyond_its_scratch(ib3d):
    L = ib3d.lib()
    dummy = C.c_void_p(1)
    rc = L.ib3d_pressure_solve_noalloc(200, 200, 200, dummy, dummy, dummy, dummy, dummy, 0.001, dummy, 1.9, 1e-6,
                                       10, 4, None, None, None)
    assert rc == ib3d.ERR_TOO_LARGE
