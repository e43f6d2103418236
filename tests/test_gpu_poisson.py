"""The standalone pressure-Poisson problem: a tanh-clustered cube with Neumann
conditions on all six faces (coefficients replaced with
ib3d_set_poisson_coefficients), the right-hand side the divergence of a seeded,
box-filtered random face-velocity field, solved by REDBLACKSOR alone
(ib3d_redblack_sor) with omega 1.85 to a residual of 1e-8. The FP64 path must match
the oracle bit for bit; the FP32-sweep form must reach the same FP64 residual."""
from __future__ import annotations

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def residual(P, pc, dt=1.0):
    """max |b/dt - A pc| over the cube's interior, in numpy."""
    ax, ay, az = P["acoef"]
    b = P["b"]
    n = ax.shape[0]
    s = np.s_[1:n + 1, 1:n + 1, 1:n + 1]
    c = pc[s]
    Ap = (ax[:, 0][:, None, None] * pc[0:n, 1:n + 1, 1:n + 1] + ax[:, 2][:, None, None] * pc[2:n + 2, 1:n + 1, 1:n + 1]
          + ay[:, 0][None, :, None] * pc[1:n + 1, 0:n, 1:n + 1] + ay[:, 2][None, :, None] * pc[1:n + 1, 2:n + 2, 1:n + 1]
          + az[:, 0][None, None, :] * pc[1:n + 1, 1:n + 1, 0:n] + az[:, 2][None, None, :] * pc[1:n + 1, 1:n + 1, 2:n + 2]
          + (ax[:, 1][:, None, None] + ay[:, 1][None, :, None] + az[:, 1][None, None, :]) * c)
    return float(np.max(np.abs(b[s] / dt - Ap)))


def _gpu(ib3d, P, **kw):
    p = ib3d.default_params(re=100.0, deltat=1.0, omega=1.85, eps=1e-8, max_sweeps=200000)
    for k, v in kw.items():
        setattr(p, k, v)
    s = ib3d.Solver(P["x"], P["y"], P["z"], p)
    s.set_poisson_coefficients(*P["acoef"])
    s.set_field("b", P["b"])
    return s


@pytest.mark.parametrize("criterion", [0, 1])
def test_neumann_cube_fp64_bit_exact(ib3d, oracle_mod, grids, criterion):
    P = grids.poisson_problem(48, seed=0)
    eps = 1e-8 if criterion == 1 else 1e-9
    s = _gpu(ib3d, P, criterion=criterion, eps=eps, check_every=1)
    o = oracle_mod.Oracle(P["x"], P["y"], P["z"], 100.0, 1.0, omega=1.85, eps=eps, criterion=criterion,
                          max_sweeps=200000, check_every=1)
    o.no_body()
    o.set_acoef(*P["acoef"])
    o.set_field("b", P["b"])
    g = s.redblack_sor()
    r = o.redblack_sor()
    assert g["sweeps"] == r["sweeps"]
    pg, po = s.get_field("pc"), o.get_field("pc")
    bad = np.argwhere(pg != po)
    assert bad.size == 0, f"{len(bad)} pc mismatches, first {bad[0]}"
    if criterion == 1:
        assert residual(P, pg) < 1e-8
    s.close()


def test_neumann_cube_fp32_sweeps_reach_fp64_residual(ib3d, grids):
    P = grids.poisson_problem(64, seed=1)
    s64 = _gpu(ib3d, P, criterion=1, check_every=8)
    s32 = _gpu(ib3d, P, criterion=1, precision=ib3d.PREC_FP32DC, inner_sweeps=64)
    a = s64.redblack_sor()
    b = s32.redblack_sor()
    p64, p32 = s64.get_field("pc"), s32.get_field("pc")
    assert residual(P, p64) < 1e-8 and residual(P, p32) < 1e-8
    # all-Neumann: the solution is defined up to a constant
    n = 64
    s = np.s_[1:n + 1, 1:n + 1, 1:n + 1]
    d64, d32 = p64[s] - p64[s].mean(), p32[s] - p32[s].mean()
    assert np.max(np.abs(d64 - d32)) <= 1e-6 * np.max(np.abs(d64))
    print(f"FP64 sweeps {a['sweeps']}, FP32-sweep form {b['sweeps']} ({b['outer']} outer)")
    s64.close()
    s32.close()


@pytest.mark.parametrize("shape", [(300, 20, 18), (258, 17, 9), (64, 33, 31)])
def test_packed_sweep_on_ragged_rows_matches_padded_layout(ib3d, grids, shape):
    """The colour-packed FP32 sweeps (two colour passes with two rows per thread, or
    with one row per thread with and without branches around the loads, each pass of
    64 sweeps as two replays of the captured 32-sweep graph; and the fused z-wavefront
    sweep) against the one-array sweep on rows whose float4 groups fill no whole
    warp or spill into a second one (nx = 300: 38 groups; 258: 33; 64: 8), odd ny
    and nz, and row and plane counts that are no multiple of a block's rows or
    planes: all perform the same FP32 operations, so the sweep counts and the
    corrections agree bit for bit, and all meet the FP64 residual."""
    nx, ny, nz = shape
    x, y, z = grids.tanh_axis(nx), grids.tanh_axis(ny), grids.tanh_axis(nz)
    b = grids.divergence_rhs(x, y, z, grids.random_face_velocities(shape, 3))
    acoef = (grids.neumann_coefficients(x), grids.neumann_coefficients(y), grids.neumann_coefficients(z))
    out = []
    kernels = (1, 0, 2, 3, 4)   # sweep_kernel
    for kernel in kernels:
        p = ib3d.default_params(re=100.0, deltat=1.0, omega=1.85, eps=1e-8, max_sweeps=200000)
        p.precision, p.criterion, p.inner_sweeps, p.sweep_kernel = ib3d.PREC_FP32DC, 1, 64, kernel
        s = ib3d.Solver(x, y, z, p)
        s.set_poisson_coefficients(*acoef)
        s.set_field("b", b)
        st = s.redblack_sor()
        assert st["final_err"] < 1e-8
        out.append((st["sweeps"], s.get_field("pc")))
        s.close()
    for q in range(1, len(kernels)):
        assert out[q][0] == out[0][0], (kernels[q], out[q][0], out[0][0])
        bad = np.argwhere(out[q][1] != out[0][1])
        assert bad.size == 0, f"kernel {kernels[q]}: {len(bad)} pc mismatches, first {bad[0]}"
