"""CPU tests of the inputs and of the FP64 oracle: known-answer and analytic
checks that pin the oracle, since the reference ships no tests or fixtures and
cannot be run (no Fortran compiler)."""
from __future__ import annotations

import numpy as np
import pytest


def test_stretched_axis_fills_domain(grids):
    nodes, rl, rr = grids.stretched_axis(-5.0, 15.0, 256, -0.8, 0.8, 1.0 / 40)
    assert nodes.size == 257 and nodes[0] == -5.0 and nodes[-1] == 15.0
    d = np.diff(nodes)
    assert np.all(d > 0)
    core = d[(nodes[:-1] >= -0.8 - 1e-12) & (nodes[1:] <= 0.8 + 1e-12)]
    assert core.size == 64 and np.allclose(core, 1.0 / 40, rtol=0, atol=1e-14)
    assert rl > 1.0 and rr > 1.0
    # geometric growth away from the core on the high side
    hi = d[nodes[:-1] >= 0.8 - 1e-12]
    assert np.allclose(hi[1:-1] / hi[:-2], rr, rtol=1e-9)


def test_stretch_ratio_solves_side():
    from importlib import import_module
    g = import_module("ib3d_gpu_gb300.grids")
    r = g.solve_ratio(44, 0.025, 4.2)
    assert abs(0.025 * sum(r ** m for m in range(1, 45)) - 4.2) < 1e-9


def test_icosphere_counts_orientation_and_closure(grids):
    nodes, tris = grids.icosphere(4, 0.5)
    assert nodes.shape == (2562, 3) and tris.shape == (5120, 3)
    assert tris.min() == 1 and tris.max() == 2562
    assert np.allclose(np.linalg.norm(nodes, axis=1), 0.5, atol=1e-15)
    p = nodes[tris - 1]
    n = np.cross(p[:, 1] - p[:, 0], p[:, 2] - p[:, 0])
    c = p.mean(axis=1)
    assert np.all(np.einsum("ij,ij->i", n, c) > 0), "triangles must wind outward"
    edges = {}
    for a, b, cc in tris:
        for e in ((a, b), (b, cc), (cc, a)):
            edges[tuple(sorted(e))] = edges.get(tuple(sorted(e)), 0) + 1
    assert set(edges.values()) == {2}, "closed surface: every edge shared by two triangles"


def test_gmsh_round_trip(grids, tmp_path):
    nodes, tris = grids.icosphere(2, 0.5)
    f = tmp_path / "sphere.msh"
    grids.write_gmsh(f, nodes, tris)
    n2, t2 = grids.read_gmsh(f)
    assert np.array_equal(t2, tris) and np.array_equal(n2, nodes)


def _uniform_oracle(oracle_mod, n=12, h=0.5):
    x = np.arange(n + 1) * h
    return oracle_mod.Oracle(x, x.copy(), x.copy(), re=100.0, deltat=0.01)


def test_convection_coefficients_uniform_grid(oracle_mod):
    """On a uniform grid the third-order upwind stencil of non_uni_coeff reduces to
    u*(-u2+8u1-8um1+um2)/(12h) + |u|*(u2-4u1+6u0-4um1+um2)/(4h): the integer tables
    below, exact in FP64 (subNavierStokes.f90:36-116)."""
    o = _uniform_oracle(oracle_mod)
    ca = [o.conv_coef(0, m)[5] for m in range(6)]
    ck = [o.conv_coef(0, 6 + m)[5] for m in range(6)]
    assert ca == [8640.0, -69120.0, 0.0, 69120.0, -8640.0, -103680.0]
    assert ck == [2.0, -8.0, 12.0, -8.0, 2.0, 4.0]
    for fam in range(6):
        assert [o.conv_coef(fam, m)[4] for m in range(6)] == ca


def test_poisson_coefficients_exact_for_quadratics(oracle_mod, grids):
    """The 3-point operator of coefficientMatrix (subCoefficientMatrix.f90:8-33) is
    exact for quadratics on any spacing: A applied to x^2 gives 2 on interior rows."""
    nodes, _, _ = grids.stretched_axis(-2.0, 3.0, 20, -0.5, 0.5, 0.125)
    o = oracle_mod.Oracle(nodes, nodes.copy(), nodes.copy(), re=100.0, deltat=0.01)
    A = o.acoef(0)
    xp = o.grid1d(15, o.nx + 3)
    f = xp ** 2
    for i in range(3, o.nx + 1):   # interior rows without folded boundary terms
        val = A[i - 2, 0] * f[i - 1] + A[i - 2, 1] * f[i] + A[i - 2, 2] * f[i + 1]
        assert abs(val - 2.0) < 1e-9
    # boundary folding: inlet Neumann, outlet Dirichlet (x); Neumann both ends (y)
    Ay = o.acoef(1)
    assert A[0, 0] == 0.0 and A[-1, 2] == 0.0 and Ay[0, 0] == 0.0 and Ay[-1, 2] == 0.0


def test_uniform_flow_is_steady_under_momentum(oracle_mod, grids):
    """u = 1, v = w = p = 0 is a steady solution: the convection stencils sum to zero
    and diffusion vanishes, so ut = 1 away from the boundary layer of ghost cells."""
    cs = grids.case("tiny")
    o = oracle_mod.Oracle(cs.x, cs.y, cs.z, cs.re, cs.dt)
    nodes, tris = grids.icosphere(1, 0.1, centre=(4.0, 2.0, 2.0))
    o.set_mesh(nodes, tris)
    o.search((2, 3, 2, 3, 2, 3))   # a box without the body: every cell is fluid
    assert o.counts["solid"] == 0 and o.counts["ib"] == 0
    o.initial_conditions()
    o.ns_momentum()
    ut = o.get_field("ut")
    inner = ut[4:-4, 4:-4, 4:-4]
    assert np.max(np.abs(inner - 1.0)) < 1e-12


def test_search_of_centred_sphere_is_symmetric(oracle_mod, grids):
    """A sphere centred in a grid symmetric in y and z gives flags symmetric under
    y -> -y and z -> -z up to the mesh's own asymmetry (the icosphere is not
    mirror-symmetric), and solid cells lie inside the sphere, fluid cells outside."""
    cs = grids.case("tiny")
    o = oracle_mod.setup_case(cs)
    s = o.get_search()
    cell = s["cell"]
    xp, yp, zp = (o.grid1d(q, n + 3)[1:n + 3] for q, n in ((15, o.nx), (16, o.ny), (17, o.nz)))
    X, Y, Z = np.meshgrid(xp, yp, zp, indexing="ij")
    r = np.sqrt(X ** 2 + Y ** 2 + Z ** 2)
    assert np.all(r[cell == 1] < cs.radius)
    assert np.all(r[cell == 2] < cs.radius + 0.2)
    flagged = cell[1:-1, 1:-1, 1:-1]
    mirrored = flagged[:, ::-1, :]
    assert np.mean(flagged == mirrored) > 0.999
    c = o.counts
    assert c["fluid"] + c["solid"] + c["ib"] == o.nx * o.ny * o.nz
    assert c["red"] + c["black"] == c["fluid"]
    ib = s["ib"]
    # lexicographic order (k outer, j, i inner), as cellCount builds it
    key = ib[:, 2] * 10 ** 8 + ib[:, 1] * 10 ** 4 + ib[:, 0]
    assert np.all(np.diff(key) > 0)


def test_sor_solution_meets_residual_tolerance(oracle_mod, grids):
    """After the residual-criterion solve, the numpy residual b/dt - A pc is below
    eps on fluid cells and pc is zero off the fluid cells (Dirichlet at the body)."""
    cs = grids.case("tiny")
    o = oracle_mod.setup_case(cs, criterion=1, eps=1e-9, check_every=1)
    o.ns_momentum(); o.velocity_bc(); o.solid_cell_bc(); o.velocity_forcing(); o.velocity_bc()
    st = o.poisson_solver()
    assert st["final_err"] < 1e-9
    pc, b = o.get_field("pc"), o.get_field("b")
    cell = o.get_search()["cell"]
    A = [o.acoef(a) for a in range(3)]
    nx, ny, nz = o.nx, o.ny, o.nz
    sl = (slice(1, nx + 1), slice(1, ny + 1), slice(1, nz + 1))
    ax = lambda c: A[0][:, c][:, None, None]
    ay = lambda c: A[1][:, c][None, :, None]
    az = lambda c: A[2][:, c][None, None, :]
    r = (b[sl] / cs.dt - ax(0) * pc[0:nx, 1:ny + 1, 1:nz + 1] - ax(2) * pc[2:nx + 2, 1:ny + 1, 1:nz + 1]
         - ay(0) * pc[1:nx + 1, 0:ny, 1:nz + 1] - ay(2) * pc[1:nx + 1, 2:ny + 2, 1:nz + 1]
         - az(0) * pc[1:nx + 1, 1:ny + 1, 0:nz] - az(2) * pc[1:nx + 1, 1:ny + 1, 2:nz + 2]
         - (ax(1) + ay(1) + az(1)) * pc[sl])
    fluid = cell[sl] == 0
    assert np.max(np.abs(r[fluid])) < 1e-9 * 1.0001
    assert np.all(pc[sl][~fluid] == 0.0)


def test_sor_noconv_cap(oracle_mod, grids):
    cs = grids.case("tiny")
    o = oracle_mod.setup_case(cs, max_sweeps=7)
    o.ns_momentum(); o.velocity_bc(); o.solid_cell_bc(); o.velocity_forcing(); o.velocity_bc()
    st = o.poisson_solver(allow_noconv=True)
    assert st["rc"] == 1 and st["sweeps"] == 7


def test_moved_body_shifts_flags_and_zero_motion_changes_nothing(oracle_mod, grids):
    """or_move_body: a shift of exactly one core cell in y moves the core flags by one
    index in j (up to corners that sit on the surface within rounding); a zero shift
    at zero velocity leaves the search and a whole step unchanged (surface velocity
    0 and dpdn 0 as for the fixed body)."""
    cs = grids.case("tiny")
    h = 1.0 / 8                       # the tiny case's uniform core spacing
    a = oracle_mod.setup_case(cs)
    b = oracle_mod.setup_case(cs)
    b.move_body(0.0, h, 0.0, 0.0, 0.0, 0.0)
    b.search(cs.box)
    ca, cb = a.get_search()["cell"], b.get_search()["cell"]
    assert a.counts["solid"] == b.counts["solid"] or abs(a.counts["solid"] - b.counts["solid"]) <= 2
    i0, i1, j0, j1, k0, k1 = (int(v) for v in cs.box)
    core_a = ca[i0:i1, j0:j1 - 1, k0:k1]
    core_b = cb[i0:i1, j0 + 1:j1, k0:k1]
    assert np.mean(core_a == core_b) > 0.999
    c = oracle_mod.setup_case(cs)
    c.move_body(0.0, 0.0, 0.0, 0.0, 0.0, 0.0)
    c.search(cs.box)
    d = oracle_mod.setup_case(cs)
    assert np.array_equal(c.get_search()["cell"], d.get_search()["cell"])
    for step in (1, 2):
        sc, kc = c.step(step == 1)
        sd, kd = d.step(step == 1)
        assert sc["sweeps"] == sd["sweeps"] and np.array_equal(kc, kd)
    for f in ("u", "v", "w", "p"):
        assert np.array_equal(c.get_field(f), d.get_field(f)), f


def test_neumann_coefficients_and_standalone_sor(oracle_mod, grids):
    """grids.neumann_coefficients reproduces coefficientMatrix's interior rows and its
    Neumann folding, and REDBLACKSOR on the all-Neumann cube with the weighted-mean-free
    divergence reaches a residual of 1e-8 (independent numpy residual)."""
    P = grids.poisson_problem(20, seed=3)
    o = oracle_mod.Oracle(P["x"], P["y"], P["z"], 100.0, 1.0, omega=1.85, eps=1e-8, criterion=1,
                          max_sweeps=100000, check_every=1)
    ay = o.acoef(1)                        # y: Neumann at both ends in the reference as well
    assert np.array_equal(ay, P["acoef"][1])
    ax = o.acoef(0)                        # x: the outlet row differs (Dirichlet there)
    assert np.array_equal(ax[:-1], P["acoef"][0][:-1])
    o.no_body()
    o.set_acoef(*P["acoef"])
    o.set_field("b", P["b"])
    st = o.redblack_sor()
    assert st["final_err"] < 1e-8
    import importlib
    res = importlib.import_module("test_gpu_poisson").residual
    assert res(P, o.get_field("pc")) < 1e-8


def test_calculate_uc_and_ab2_known_answers(oracle_mod, grids):
    """calculateUc of uniform flow u = 1 is 1 (the mean over the fluid cells of plane
    nx-4); nsMomentumAB with resi = resid of the same fields equals the Euler update
    (0.5*(3r - r) = r), and with resi = 0 it is the Euler update with 1.5 r."""
    cs = grids.case("tiny")
    o = oracle_mod.setup_case(cs)
    o.set_field("ut", o.get_field("u"))
    assert o.calculate_uc() == 1.0
    p = oracle_mod.setup_case(cs)
    p.ns_momentum()
    ut_euler = p.get_field("ut")
    p.ns_momentum_ab()                       # resi now holds this state's resid
    assert np.allclose(p.get_field("ut"), ut_euler, rtol=0, atol=1e-13)


def test_force_driven_motion_known_answers(oracle_mod, grids):
    """or_move_body_free (shiftSurfaceNodesMovingbody's force integration): a body of
    volume pi/6 (D = 1, unit density) at rest under a force F reaches v = F/vol * dt
    after one step and has moved v * dt; with no force it keeps its velocity; the
    surface centroids move by exactly the displacements."""
    import math
    cs = grids.case("tiny")
    o = oracle_mod.setup_case(cs)
    vol = math.pi / 6.0
    c0 = o.surface()[:3].copy()          # element centroids before the move
    f = (0.0, 2.0, -1.0)
    v1 = o.move_body_free(*f)
    assert np.allclose(v1, [fq / vol * cs.dt for fq in f], rtol=1e-15, atol=0.0)
    c1 = o.surface()[:3].copy()
    assert np.allclose(c1 - c0, (v1 * cs.dt)[:, None], rtol=0.0, atol=1e-15)
    v2 = o.move_body_free(0.0, 0.0, 0.0)
    assert np.array_equal(v2, v1)
    c2 = o.surface()[:3].copy()
    assert np.allclose(c2 - c1, (v2 * cs.dt)[:, None], rtol=0.0, atol=1e-15)
    o.close()


def _cell_centres(nodes):
    c = 0.5 * (nodes[:-1] + nodes[1:])
    return np.concatenate([[2 * nodes[0] - c[0]], c, [2 * nodes[-1] - c[-1]]])


def test_drag_known_answers(oracle_mod, grids):
    """stressCal1 on fields with exact answers. A uniform stream with p = 0 exerts no
    force. A linear pressure p = x (fluid at rest) pushes the sphere with
    -grad(p) * volume = (-pi/6, 0, 0), i.e. Cd_p = 2 F_x / (pi/4) = -4/3, and p = y
    gives the same lift; the surface pressure is extrapolated from probe points, so
    the coefficient converges to -4/3 at first order in the core spacing h:
    (Cd + 4/3) / h is the same on h = 1/8 and 1/16, and the Richardson value
    2 Cd(1/16) - Cd(1/8) is -4/3 within 0.5 %."""
    cds = {}
    for name, h in (("tiny", 1.0 / 8), ("sphere96", 1.0 / 16)):
        cs = grids.case(name)
        o = oracle_mod.setup_case(cs)
        assert np.array_equal(o.stress(True), np.zeros(4))          # u = 1, p = 0
        shape = o.get_field("p").shape
        for f in ("u", "v", "w"):
            o.set_field(f, np.zeros(shape))
        o.set_field("p", np.broadcast_to(_cell_centres(cs.x)[:, None, None], shape).copy())
        cx = o.stress(True)
        o.set_field("p", np.broadcast_to(_cell_centres(cs.y)[None, :, None], shape).copy())
        cy = o.stress(True)
        o.close()
        assert cx[0] == 0.0 and cx[2] == 0.0 and abs(cx[3]) < 1e-12      # no viscous part, no lift
        assert abs(cy[3] - cx[1]) < 1e-12 and abs(cy[1]) < 1e-12          # p = y: the same, as lift
        cds[h] = cx[1]
    e8, e16 = (cds[1 / 8] + 4 / 3) * 8, (cds[1 / 16] + 4 / 3) * 16
    assert abs(e8 - e16) < 0.02 * abs(e16), (cds, e8, e16)
    assert abs((2 * cds[1 / 16] - cds[1 / 8]) + 4 / 3) < 0.005 * 4 / 3, cds


def test_linear_fields_known_answers(oracle_mod, grids):
    """On the stretched grid of the tiny case, without a body: the divergence
    (computeDiv) of the face velocity ut = x is exactly 1 in every interior cell, and
    the shear flow u = y (v = w = p = 0) is steady under the momentum predictor --
    convection vanishes with v = 0 and the non-uniform second difference of a linear
    profile is zero -- away from the ghost layers."""
    cs = grids.case("tiny")
    o = oracle_mod.Oracle(cs.x, cs.y, cs.z, cs.re, cs.dt, max_sweeps=1)
    o.no_body()
    shape = o.get_field("u").shape
    zero = np.zeros(shape)
    xf = np.asarray(cs.x)[np.minimum(np.arange(shape[0]), len(cs.x) - 1)]   # ut(i) sits on face x(i)
    faces = np.broadcast_to(xf[:, None, None], shape).copy()
    for f, val in (("u", faces), ("v", zero), ("w", zero), ("ut", faces), ("vt", zero), ("wt", zero)):
        o.set_field(f, val)
    o.poisson_solver(allow_noconv=True)
    assert np.array_equal(o.get_field("b")[2:-2, 2:-2, 2:-2], np.ones((shape[0] - 4, shape[1] - 4, shape[2] - 4)))
    shear = np.broadcast_to(_cell_centres(cs.y)[None, :, None], shape).copy()
    for f, val in (("u", shear), ("v", zero), ("w", zero), ("p", zero)):
        o.set_field(f, val)
    o.ns_momentum()
    ut = o.get_field("ut")
    inner = np.s_[4:-4, 4:-4, 4:-4]
    assert np.max(np.abs(ut[inner] - shear[inner])) < 1e-12 * np.max(np.abs(shear))
    o.close()


def test_poisson_boundary_rows_on_a_uniform_grid(oracle_mod):
    """coefficientMatrix's boundary folding (subCoefficientMatrix.f90:36-53) on a
    uniform grid of spacing h: interior rows (1, -2, 1)/h^2; the inlet and the y, z
    faces are Neumann (A2 += A1: (0, -1, 1)/h^2 at the first row, (1, -1, 0)/h^2 at
    the last y and z rows); the outlet is Dirichlet (A2 -= A3: (1, -3, 0)/h^2)."""
    h = 0.5
    o = _uniform_oracle(oracle_mod, n=12, h=h)
    r = 1.0 / (h * h)
    ax, ay, az = o.acoef(0), o.acoef(1), o.acoef(2)
    for A in (ax, ay, az):
        assert np.allclose(A[1:-1], [r, -2 * r, r], rtol=1e-15, atol=0.0)
        assert np.allclose(A[0], [0.0, -r, r], rtol=1e-15, atol=0.0)
    assert np.allclose(ax[-1], [r, -3 * r, 0.0], rtol=1e-15, atol=0.0)
    for A in (ay, az):
        assert np.allclose(A[-1], [r, -r, 0.0], rtol=1e-15, atol=0.0)


def test_normal_distances_follow_the_sphere(oracle_mod, grids):
    """computeNormDistance (subSearch.f90:599-678): for every IB cell of the 64x48x48
    case, the signed distance of the pressure node to the plane of its nearest
    element is the distance to the sphere r - 0.5 up to the faceting of the
    icosphere (< 1e-3), and those of the six face-centred velocity nodes (u at x -/+
    h/2, then v, w) are within 5e-3 (the plane of the cell's element, seen from a
    node half a cell away)."""
    cs = grids.case("small")
    o = oracle_mod.setup_case(cs)
    sr = o.get_search()
    ib, nd = sr["ib"], sr["normdis"]
    xc, yc, zc = (_cell_centres(np.asarray(a)) for a in (cs.x, cs.y, cs.z))
    a, b, c = ib[:, 0] - 1, ib[:, 1] - 1, ib[:, 2] - 1
    X, Y, Z = xc[a], yc[b], zc[c]
    x, y, z = (np.asarray(v) for v in (cs.x, cs.y, cs.z))
    nodes = [(X, Y, Z), (x[a - 1], Y, Z), (x[a], Y, Z), (X, y[b - 1], Z), (X, y[b], Z), (X, Y, z[c - 1]), (X, Y, z[c])]
    for q, (px, py, pz) in enumerate(nodes):
        err = np.abs(nd[:, q] - (np.sqrt(px * px + py * py + pz * pz) - 0.5)).max()
        assert err < (1e-3 if q == 0 else 5e-3), (q, err)
    o.close()


def test_tagging_follows_the_sphere(oracle_mod, grids):
    """tagging (subSearch.f90:134-321) against the exact sphere on the 64x48x48 case:
    every cell whose eight corners lie inside r < 0.5 - 2e-3 is solid, every cell
    whose corners all lie outside r > 0.5 + 2e-3 is fluid, and the IB cells are all
    among the cells the surface cuts (the 2e-3 band covers the icosphere's
    faceting)."""
    cs = grids.case("small")
    o = oracle_mod.setup_case(cs)
    cell = o.get_search()["cell"]
    o.close()
    x, y, z = (np.asarray(v) for v in (cs.x, cs.y, cs.z))
    nx, ny, nz = len(x) - 1, len(y) - 1, len(z) - 1
    rmin = np.full((nx, ny, nz), np.inf)
    rmax = np.zeros((nx, ny, nz))
    for dx in (0, 1):
        for dy in (0, 1):
            for dz in (0, 1):
                X = x[dx:nx + dx][:, None, None]
                Y = y[dy:ny + dy][None, :, None]
                Z = z[dz:nz + dz][None, None, :]
                r = np.sqrt(X * X + Y * Y + Z * Z)
                rmin, rmax = np.minimum(rmin, r), np.maximum(rmax, r)
    flags = cell[1:nx + 1, 1:ny + 1, 1:nz + 1]
    inside, outside = rmax < 0.5 - 2e-3, rmin > 0.5 + 2e-3
    assert inside.any() and np.all(flags[inside] == 1)
    assert np.all(flags[outside] == 0)
    cut = ~inside & ~outside
    assert np.all(np.isin(flags[cut], (0, 2))) and np.all(cut[flags == 2])


def _cube(lo: float, hi: float):
    """Axis-aligned cube [lo, hi]^3 as 12 outward counter-clockwise triangles (1-based)."""
    v = np.array([[lo, lo, lo], [hi, lo, lo], [hi, hi, lo], [lo, hi, lo],
                  [lo, lo, hi], [hi, lo, hi], [hi, hi, hi], [lo, hi, hi]])
    quads = [(0, 3, 2, 1), (4, 5, 6, 7), (0, 1, 5, 4), (2, 3, 7, 6), (1, 2, 6, 5), (0, 4, 7, 3)]
    tris = [t for a, b, c, d in quads for t in ((a, b, c), (a, c, d))]
    return v, np.array(tris, dtype=np.int64) + 1


def test_ghost_point_forcing_reproduces_affine_fields(oracle_mod):
    """velocityForcing1's quadratic ghost values (subForcing.f90:107-652) are exact for
    a field that is affine along the wall normal and meets the no-slip condition:
    a cube [1.02, 1.98]^3 at rest on a uniform grid (h = 0.1), ut = x - 1.98 (zero
    on the +x face), vt = wt = 0. Every ghost u value near the middle of the +x face,
    set to 10 beforehand, becomes x - 1.98 within 1e-12, and vt, wt stay 0 there."""
    h, n, lo, hi = 0.1, 30, 1.02, 1.98
    x = np.arange(n + 1) * h
    o = oracle_mod.Oracle(x, x.copy(), x.copy(), re=100.0, deltat=0.01)
    v, tris = _cube(lo, hi)
    o.set_mesh(v, tris)
    o.search((2, n + 1, 2, n + 1, 2, n + 1))
    shape = o.get_field("u").shape
    xf = x[np.minimum(np.arange(shape[0]), n)]                 # ut(i) sits on face x(i)
    yc = (np.arange(shape[1]) - 0.5) * h                       # cell centres in y and z
    exact = np.broadcast_to((xf - hi)[:, None, None], shape).copy()
    band = ((xf[:, None, None] > hi - 0.15) & (xf[:, None, None] < hi)
            & (np.abs(yc[None, :, None] - 1.5) < 0.3) & (np.abs(yc[None, None, :] - 1.5) < 0.3))
    ut0 = np.where(band, 10.0, exact)
    zero = np.zeros(shape)
    for f, val in (("u", ut0), ("ut", ut0), ("v", zero), ("vt", zero), ("w", zero), ("wt", zero)):
        o.set_field(f, val)
    o.velocity_forcing()
    ut, vt, wt = o.get_field("ut"), o.get_field("vt"), o.get_field("wt")
    ghost = band & (ut != 10.0)
    assert ghost.sum() > 20, ghost.sum()
    assert np.max(np.abs(ut[ghost] - exact[ghost])) < 1e-12
    assert np.max(np.abs(vt[ghost])) < 1e-12 and np.max(np.abs(wt[ghost])) < 1e-12
    o.close()


def test_ghost_point_pressure_forcing_reproduces_fields_with_zero_normal_gradient(oracle_mod):
    """pressureForcing1 (subForcing.f90:2-103, dp/dn = 0 for a body at rest) is exact
    for a pressure that does not vary along the wall normal: near the middle of the
    +x face of the cube, p = y, and every ghost pressure there, set to 10
    beforehand, becomes its cell's y within 1e-12."""
    h, n, lo, hi = 0.1, 30, 1.02, 1.98
    x = np.arange(n + 1) * h
    o = oracle_mod.Oracle(x, x.copy(), x.copy(), re=100.0, deltat=0.01)
    v, tris = _cube(lo, hi)
    o.set_mesh(v, tris)
    o.search((2, n + 1, 2, n + 1, 2, n + 1))
    shape = o.get_field("p").shape
    c = (np.arange(shape[0]) - 0.5) * h                        # cell centres (padded index)
    exact = np.broadcast_to(c[None, :, None], shape).copy()    # p = y
    band = ((c[:, None, None] > hi - 0.15) & (c[:, None, None] < hi)
            & (np.abs(c[None, :, None] - 1.5) < 0.3) & (np.abs(c[None, None, :] - 1.5) < 0.3))
    o.set_field("p", np.where(band, 10.0, exact))
    o.pressure_forcing()
    p = o.get_field("p")
    ghost = band & (p != 10.0)
    assert ghost.sum() > 10, ghost.sum()
    assert np.max(np.abs(p[ghost] - exact[ghost])) < 1e-12
    o.close()


def test_projection_makes_the_velocity_divergence_free(oracle_mod, grids):
    """poissonSolver's projection (computeDiv, REDBLACKSOR, correctVelocity) on a
    uniform grid without a body: from seeded face velocities with divergence ~10,
    the corrected velocity's discrete divergence inside the first layer of cells is
    dt times the SOR residual (1e-11 here), i.e. zero to 1e-12. (On the stretched
    grids the reference's Laplacian uses the pressure-node spacing and computeDiv the
    cell width, so the two agree only on uniform spacing.)"""
    n = 24
    x = np.arange(n + 1) * (1.0 / n)
    o = oracle_mod.Oracle(x, x.copy(), x.copy(), re=100.0, deltat=0.01, omega=1.8, eps=1e-11, criterion=1,
                          max_sweeps=200000, check_every=1)
    o.no_body()
    ut, vt, wt = grids.random_face_velocities((n, n, n), 5)
    for f, val in (("ut", ut), ("vt", vt), ("wt", wt), ("u", ut), ("v", vt), ("w", wt)):
        o.set_field(f, val)
    o.poisson_solver()
    u, v, w = o.get_field("u"), o.get_field("v"), o.get_field("w")
    h = 1.0 / n
    s = np.s_[2:n, 2:n, 2:n]
    div = ((u[2:n, 2:n, 2:n] - u[1:n - 1, 2:n, 2:n]) + (v[2:n, 2:n, 2:n] - v[2:n, 1:n - 1, 2:n])
           + (w[2:n, 2:n, 2:n] - w[2:n, 2:n, 1:n - 1])) / h
    assert np.abs(o.get_field("b")[s]).max() > 1.0
    assert np.abs(div).max() < 1e-12, np.abs(div).max()
    o.close()


def test_third_order_upwind_is_exact_for_cubics_on_a_stretched_grid(oracle_mod, grids):
    """non_uni_coeff's own-axis family (subNavierStokes.f90:36-116) on a stretched
    axis: the five-point convection stencil, divided by its sixth coefficient and
    the spacing, is the first derivative of any cubic exactly at every node it is
    used for -- third order on non-uniform spacing -- and its dissipation stencil
    annihilates cubics where the spacing is uniform."""
    nodes, _, _ = grids.stretched_axis(-2.0, 3.0, 20, -0.5, 0.5, 0.125)
    o = oracle_mod.Oracle(nodes, nodes.copy(), nodes.copy(), re=100.0, deltat=0.01)
    c = [o.conv_coef(0, m) for m in range(12)]
    f = lambda x: 0.3 * x ** 3 - x ** 2 + 2.0 * x + 1.0
    df = lambda x: 0.9 * x ** 2 - 2.0 * x + 2.0
    for i in range(4, o.nx):
        xs = [nodes[i + 1], nodes[i], nodes[i - 1], nodes[i - 2], nodes[i - 3]]   # u(i+2) .. u(i-2)
        sa = sum(c[m][i] * f(xs[m]) for m in range(5))
        expect = c[5][i] * (nodes[i] - nodes[i - 1]) * df(nodes[i - 1])
        assert abs(sa - expect) <= 1e-11 * abs(expect), (i, sa, expect)
        h = np.diff(nodes[i - 3:i + 2])
        if np.all(h == h[0]):
            sk = sum(c[6 + m][i] * f(xs[m]) for m in range(5))
            assert abs(sk) <= 1e-13 * max(abs(c[6 + m][i] * f(xs[m])) for m in range(5)), (i, sk)
    # the transverse families (a velocity carried across the other axes, at cell
    # centres): exact for cubics with the centre-to-centre spacing as normaliser
    centres = 0.5 * (nodes[:-1] + nodes[1:])
    for fam in (3, 4, 5):
        c = [o.conv_coef(fam, m) for m in range(6)]
        for i in range(4, o.nx - 1):
            xs = [centres[i], centres[i - 1], centres[i - 2], centres[i - 3], centres[i - 4]]
            sa = sum(c[m][i] * f(xs[m]) for m in range(5))
            expect = c[5][i] * (centres[i - 1] - centres[i - 2]) * df(centres[i - 2])
            assert abs(sa - expect) <= 1e-11 * abs(expect), (fam, i, sa, expect)
    o.close()


def test_diffusion_is_exact_for_a_quadratic_profile(oracle_mod, grids):
    """nsMomentum's viscous term (subNavierStokes.f90:879-887) on the stretched grid of
    the tiny case: for u = y^2 with v = w = p = 0 the convection vanishes and the
    non-uniform three-point second difference is exact, so ut = u + dt * 2 / Re away
    from the ghost layers."""
    cs = grids.case("tiny")
    o = oracle_mod.Oracle(cs.x, cs.y, cs.z, cs.re, cs.dt)
    o.no_body()
    shape = o.get_field("u").shape
    u = np.broadcast_to((_cell_centres(np.asarray(cs.y)) ** 2)[None, :, None], shape).copy()
    zero = np.zeros(shape)
    for f, val in (("u", u), ("v", zero), ("w", zero), ("p", zero)):
        o.set_field(f, val)
    o.ns_momentum()
    rate = (o.get_field("ut") - u)[4:-4, 4:-4, 4:-4] / cs.dt * cs.re
    assert np.max(np.abs(rate - 2.0)) < 1e-9
    o.close()


@pytest.mark.parametrize("criterion", [0, 1])
def test_row_form_sweeps_are_bit_identical_to_the_list_form(oracle_mod, grids, criterion):
    """The timed CPU baseline runs the sweep loop over the field's rows with a fluid
    mask; it must give the list form's sweep counts, drag and fields bit for bit."""
    cs = grids.case("tiny")
    a = oracle_mod.setup_case(cs, criterion=criterion, check_every=4)
    b = oracle_mod.setup_case(cs, criterion=criterion, check_every=4)
    b.set_sweep_rows(True)
    for q in range(3):
        sa, ca = a.step(q == 0)
        sb, cb = b.step(q == 0)
        assert sa["sweeps"] == sb["sweeps"]
        assert np.array_equal(ca, cb)
    for f in ("u", "v", "w", "p", "pc"):
        assert np.array_equal(a.get_field(f), b.get_field(f)), f
    a.close()
    b.close()


def test_result_text_round_trip_and_records_split_across_lines(oracle_mod, grids, tmp_path):
    """writeResult/lastConditions: the formatted restart reads back exactly, also when
    a list-directed record continues on the next line or uses commas."""
    cs = grids.case("tiny")
    a = oracle_mod.setup_case(cs)
    a.step(True)
    path = tmp_path / "result"
    a.write_result_text(path, 0.25, 7, 3)
    b = oracle_mod.setup_case(cs)
    assert b.read_result_text(path) == (0.25, 7, 3)
    for f in ("u", "v", "w", "p"):
        assert np.array_equal(a.get_field(f), b.get_field(f)), f
    for f, g in (("ut", "u"), ("vt", "v"), ("wt", "w")):
        assert np.array_equal(b.get_field(f), b.get_field(g)), f
    # the same records with each one broken after its fourth value, and commas
    lines = path.read_text().splitlines()
    split = []
    for ln in lines:
        v = ln.split()
        split.append(", ".join(v[:4]))
        split.append("  " + " ,".join(v[4:]) + "   ignored-rest")
    path2 = tmp_path / "result_split"
    path2.write_text("\n".join(split) + "\n")
    c = oracle_mod.setup_case(cs)
    assert c.read_result_text(path2) == (0.25, 7, 3)
    for f in ("u", "v", "w", "p"):
        assert np.array_equal(a.get_field(f), c.get_field(f)), f
    short = tmp_path / "result_short"
    short.write_text("\n".join(lines[:-1]) + "\n")
    with pytest.raises(oracle_mod.OracleError):
        c.read_result_text(short)
    for x in (a, b, c):
        x.close()


def test_selective_retagging_matches_the_full_search_after_small_moves(oracle_mod, grids):
    """selectiveRetagging re-tags only the 6^3 neighbourhoods of the IB cells. For a
    body that moves less than a cell per step, every cell whose flag changes lies in
    such a neighbourhood, so the flags, IB list, nearest elements and normal
    distances equal those of a full search of the box."""
    cs = grids.case("tiny")
    a = oracle_mod.setup_case(cs)
    b = oracle_mod.setup_case(cs)
    h = float(np.min(np.diff(cs.x)))
    y = 0.0
    for q in range(6):
        dy = 0.3 * h * (1 if q % 3 else -1)
        y += dy
        a.move_body(0.0, dy, 0.0)
        b.move_body(0.0, dy, 0.0)
        ca = a.search(grids.body_box(cs, (0.0, y, 0.0)))
        cb = b.selective_retag()
        assert ca == cb, q
        ga, gb = a.get_search(), b.get_search()
        for key in ("cell", "ib", "nelp", "normdis"):
            assert np.array_equal(ga[key], gb[key]), (q, key)
    a.close()
    b.close()


def test_max_of_quotients_is_the_quotient_of_the_max():
    """derrStdSt (subPcorVcor.f90:45-58) is max over cells of |ut-u|/dt. The library
    reduces max |ut-u| and divides once; rounded IEEE division by a positive number
    is monotone, so the two agree bit for bit. Checked here on values spanning the
    normal and subnormal range, ties, zeros, overflow and extreme time steps."""
    rng = np.random.default_rng(7)
    for dt in (0.002, 0.75e-3, 1e-300, 3.0, 7.0e200, 0.1):
        for scale in (1e-310, 1e-12, 1.0, 1e150):
            x = np.abs(rng.standard_normal(50_000)) * scale
            x[:5] = 0.0
            x[5:9] = x.max()   # ties at the maximum
            with np.errstate(over="ignore"):   # some pairs overflow to inf, on both sides
                per_cell = np.max(x / dt)
                once = x.max() / dt
            assert per_cell.tobytes() == np.float64(once).tobytes(), (dt, scale)
