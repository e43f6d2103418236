"""Host-side inputs of the solver: stretched grids, the icosphere body, the
Gmsh-2 surface-mesh format the reference reads, and the named workloads.

The reference reads its grid from gridx/y/z.dat (one node coordinate per line,
nx+1 lines; subReadInput.f90:55-99) and its body from geometries/sphere.msh
(Gmsh 2 ASCII; subReadInput.f90:137-176). That mesh file is not part of the
reference, so the body here is the synthetic icosphere the workloads specify.
"""
from __future__ import annotations

import dataclasses
import math

import numpy as np


# ----------------------------------------------------------------- grids

def solve_ratio(ncells: int, h: float, length: float) -> float:
    """Geometric ratio r with h * sum_{m=1..ncells} r**m == length (bisection)."""
    if ncells <= 0:
        if length > 1e-12:
            raise ValueError("no cells left for a side of non-zero length")
        return 1.0
    target = length / h

    def f(r: float) -> float:
        if abs(r - 1.0) < 1e-15:
            return ncells - target
        return r * (r ** ncells - 1.0) / (r - 1.0) - target

    lo, hi = 1e-6, 1.0
    while f(hi) < 0:
        hi *= 2.0
        if hi > 1e6:
            raise ValueError("cannot stretch: side too long for the cells given")
    for _ in range(200):
        mid = 0.5 * (lo + hi)
        if f(mid) < 0:
            lo = mid
        else:
            hi = mid
    return 0.5 * (lo + hi)


def stretched_axis(lo: float, hi: float, n: int, core_lo: float, core_hi: float, h: float):
    """Node coordinates (n+1 values) of one grid axis.

    Uniform spacing h on [core_lo, core_hi]; the remaining cells are shared by
    the two outer sides in proportion to their length, and each side grows
    geometrically from the core (cell m of a side has size h*r**m) with the
    ratio r that fills the side exactly. Returns (nodes, ratio_low, ratio_high).
    """
    ncore = int(round((core_hi - core_lo) / h))
    if abs(ncore * h - (core_hi - core_lo)) > 1e-9 * max(1.0, abs(core_hi - core_lo)):
        raise ValueError("core interval is not a whole number of cells")
    rest = n - ncore
    if rest < 0:
        raise ValueError("fewer cells than the uniform core needs")
    ll, lr = core_lo - lo, hi - core_hi
    nl = int(round(rest * ll / (ll + lr))) if (ll + lr) > 0 else 0
    nr = rest - nl
    rl, rr = solve_ratio(nl, h, ll), solve_ratio(nr, h, lr)
    core = [core_lo + m * h for m in range(ncore + 1)]
    right, x = [], core_hi
    for m in range(1, nr + 1):
        x = x + h * rr ** m
        right.append(x)
    if nr:
        right[-1] = hi
    left, x = [], core_lo
    for m in range(1, nl + 1):
        x = x - h * rl ** m
        left.append(x)
    if nl:
        left[-1] = lo
    nodes = np.array(left[::-1] + core + right, dtype=np.float64)
    assert nodes.size == n + 1 and np.all(np.diff(nodes) > 0)
    return nodes, rl, rr


def tanh_axis(n: int, length: float = 1.0, beta: float = 3.0) -> np.ndarray:
    """Node coordinates of a tanh-clustered axis on [0, length] whose spacing is
    proportional to 1 + 0.5*tanh(beta*|2*xi - 1|) (finest at the centre)."""
    xi = (np.arange(n) + 0.5) / n
    w = 1.0 + 0.5 * np.tanh(beta * np.abs(2.0 * xi - 1.0))
    w = w / w.sum() * length
    return np.concatenate([[0.0], np.cumsum(w)])


def neumann_coefficients(nodes: np.ndarray) -> np.ndarray:
    """(n,3) Poisson coefficients of one axis, as coefficientMatrix builds them
    (subCoefficientMatrix.f90:8-33: pressure-node spacings r1, r2 and
    2/(r1 rs), -2/(r1 r2), 2/(r2 rs)), with Neumann rows folded in at both ends
    (A2 += A1 at the first row, A2 += A3 at the last). nodes: the n+1 cell faces."""
    n = len(nodes) - 1
    x1 = np.zeros(n + 4)
    x1[2:n + 3] = nodes
    d = np.zeros(n + 3)
    d[2:n + 2] = x1[3:n + 3] - x1[2:n + 2]
    d[1], d[n + 2] = d[2], d[n + 1]
    x1[1] = x1[2] - d[1]
    x1[n + 3] = x1[n + 2] + d[n + 2]
    xp = np.zeros(n + 3)
    xp[1:n + 3] = 0.5 * (x1[1:n + 3] + x1[2:n + 4])
    a = np.zeros((n, 3))
    i = np.arange(2, n + 2)
    r1, r2 = xp[i] - xp[i - 1], xp[i + 1] - xp[i]
    rs = r1 + r2
    a[:, 0], a[:, 1], a[:, 2] = 2.0 / (r1 * rs), -2.0 / (r1 * r2), 2.0 / (r2 * rs)
    a[0, 1] += a[0, 0]
    a[0, 0] = 0.0
    a[n - 1, 1] += a[n - 1, 2]
    a[n - 1, 2] = 0.0
    return a


def random_face_velocities(n: tuple, seed: int = 0, passes: int = 3):
    """Seeded face velocities (ut, vt, wt) in the padded (nx+2, ny+2, nz+2) layout:
    i.i.d. N(0,1), `passes` passes of a separable [1,1,1]/3 box filter (periodic
    wrap), mean removed, and zero normal velocity on the six boundary faces so that
    the divergence is compatible with Neumann conditions."""
    shape = (n[0] + 2, n[1] + 2, n[2] + 2)
    rng = np.random.default_rng(seed)
    out = []
    for comp in range(3):
        a = rng.standard_normal(shape)
        for _ in range(passes):
            for ax in range(3):
                a = (np.roll(a, 1, ax) + a + np.roll(a, -1, ax)) / 3.0
        a -= a.mean()
        idx = [slice(None)] * 3
        for face in (0, n[comp]):        # u(1,:,:) and u(nx+1,:,:) (1-based) are the boundary faces
            idx[comp] = face
            a[tuple(idx)] = 0.0
        out.append(np.asfortranarray(a))
    return tuple(out)


def _pressure_nodes(nodes: np.ndarray) -> np.ndarray:
    """xp(1..n+2) of one axis (1-based, entry 0 unused), with the ghost cells the
    reference adds (subReadInput.f90:61-68, 119-123)."""
    n = len(nodes) - 1
    x1 = np.zeros(n + 4)
    x1[2:n + 3] = nodes
    x1[1] = x1[2] - (x1[3] - x1[2])
    x1[n + 3] = x1[n + 2] + (x1[n + 2] - x1[n + 1])
    xp = np.zeros(n + 3)
    xp[1:n + 3] = 0.5 * (x1[1:n + 3] + x1[2:n + 4])
    return xp


def divergence_rhs(x: np.ndarray, y: np.ndarray, z: np.ndarray, faces) -> np.ndarray:
    """b = div(ut, vt, wt) at every interior cell (computeDiv, subPcorVcor.f90:91-99),
    made solvable for all-Neumann coefficients: A is not symmetric, and its left null
    vector is w = wx (x) wy (x) wz with w(i) = (xp(i+1) - xp(i-1))/2 per axis (the row
    scaling that makes A symmetric), so the w-weighted mean of b is removed."""
    ut, vt, wt = faces
    n = (len(x) - 1, len(y) - 1, len(z) - 1)
    d = [np.diff(a) for a in (x, y, z)]
    b = np.zeros((n[0] + 2, n[1] + 2, n[2] + 2), order="F")
    s = np.s_[1:n[0] + 1, 1:n[1] + 1, 1:n[2] + 1]
    b[s] = ((ut[1:n[0] + 1, 1:n[1] + 1, 1:n[2] + 1] - ut[0:n[0], 1:n[1] + 1, 1:n[2] + 1]) / d[0][:, None, None]
            + (vt[1:n[0] + 1, 1:n[1] + 1, 1:n[2] + 1] - vt[1:n[0] + 1, 0:n[1], 1:n[2] + 1]) / d[1][None, :, None]
            + (wt[1:n[0] + 1, 1:n[1] + 1, 1:n[2] + 1] - wt[1:n[0] + 1, 1:n[1] + 1, 0:n[2]]) / d[2][None, None, :])
    w = []
    for a in (x, y, z):
        xp = _pressure_nodes(a)
        m = len(a) - 1
        w.append(0.5 * (xp[3:m + 3] - xp[1:m + 1]))
    W = w[0][:, None, None] * w[1][None, :, None] * w[2][None, None, :]
    b[s] -= (W * b[s]).sum() / W.sum()
    return b


def poisson_problem(n: int = 256, seed: int = 0):
    """Standalone pressure-Poisson problem on an n^3 tanh-clustered unit cube:
    (x, y, z) faces, all-Neumann (acx, acy, acz), the seeded face velocities and the
    solvable right-hand side b made from their divergence."""
    x = tanh_axis(n)
    a = neumann_coefficients(x)
    faces = random_face_velocities((n, n, n), seed)
    return {"x": x, "y": x.copy(), "z": x.copy(), "acoef": (a, a.copy(), a.copy()), "faces": faces,
            "b": divergence_rhs(x, x, x, faces)}


# ------------------------------------------------------------------ body

_ICO_FACES = [(0, 11, 5), (0, 5, 1), (0, 1, 7), (0, 7, 10), (0, 10, 11), (1, 5, 9), (5, 11, 4), (11, 10, 2),
              (10, 7, 6), (7, 1, 8), (3, 9, 4), (3, 4, 2), (3, 2, 6), (3, 6, 8), (3, 8, 9), (4, 9, 5),
              (2, 4, 11), (6, 2, 10), (8, 6, 7), (9, 8, 1)]


def icosphere(subdivisions: int = 4, radius: float = 0.5, centre=(0.0, 0.0, 0.0)):
    """Icosahedron refined `subdivisions` times (edge midpoints pushed to the sphere).

    Returns nodes (N,3) float64 and triangles (M,3) int64 with 1-based node ids,
    wound counter-clockwise seen from outside, so (p2-p1)x(p3-p1) points outward
    (the reference's normal convention with inor = +1, subSearch.f90:112-124).
    4 subdivisions give 2562 nodes and 5120 triangles.
    """
    t = (1.0 + math.sqrt(5.0)) / 2.0
    verts = [(-1, t, 0), (1, t, 0), (-1, -t, 0), (1, -t, 0), (0, -1, t), (0, 1, t), (0, -1, -t), (0, 1, -t),
             (t, 0, -1), (t, 0, 1), (-t, 0, -1), (-t, 0, 1)]
    pts = [np.array(v, dtype=np.float64) / math.sqrt(1.0 + t * t) for v in verts]
    faces = list(_ICO_FACES)
    for _ in range(subdivisions):
        cache: dict[tuple[int, int], int] = {}

        def mid(a: int, b: int) -> int:
            key = (a, b) if a < b else (b, a)
            if key not in cache:
                m = pts[a] + pts[b]
                pts.append(m / np.linalg.norm(m))
                cache[key] = len(pts) - 1
            return cache[key]

        nf = []
        for a, b, c in faces:
            ab, bc, ca = mid(a, b), mid(b, c), mid(c, a)
            nf += [(a, ab, ca), (b, bc, ab), (c, ca, bc), (ab, bc, ca)]
        faces = nf
    nodes = np.array(pts) * radius + np.asarray(centre, dtype=np.float64)
    tris = np.array(faces, dtype=np.int64) + 1
    return nodes, tris


def write_gmsh(path, nodes: np.ndarray, tris: np.ndarray) -> None:
    """Writes a Gmsh 2.2 ASCII surface mesh in the layout readSurfaceMeshGmsh reads
    (4 header lines, node count, 'id x y z', 2 lines, element count,
    'id type ntags tag tag n1 n2 n3'; subReadInput.f90:144-167)."""
    with open(path, "w") as f:
        f.write("$MeshFormat\n2.2 0 8\n$EndMeshFormat\n$Nodes\n")
        f.write(f"{len(nodes)}\n")
        for q, (x, y, z) in enumerate(nodes, 1):
            f.write(f"{q} {x:.17g} {y:.17g} {z:.17g}\n")
        f.write("$EndNodes\n$Elements\n")
        f.write(f"{len(tris)}\n")
        for q, (a, b, c) in enumerate(tris, 1):
            f.write(f"{q} 2 2 0 1 {a} {b} {c}\n")
        f.write("$EndElements\n")


def write_gambit(path, nodes: np.ndarray, tris: np.ndarray) -> None:
    """Writes a Gambit neutral (.neu) surface mesh in the layout readSurfaceMeshGambit
    reads (6 header lines, 'NUMNP NELEM NGRPS NBSETS NDFCD NDFVL', 2 lines, 'id x y z',
    2 lines, 'id type nnodes n1 n2 n3'; subReadInput.f90:187-206)."""
    with open(path, "w") as f:
        f.write("        CONTROL INFO 2.4.6\n** GAMBIT NEUTRAL FILE\nsurface\nPROGRAM:                Gambit     VERSION:  2.4.6\n")
        f.write("generated\n     NUMNP     NELEM     NGRPS    NBSETS     NDFCD     NDFVL\n")
        f.write(f"{len(nodes):10d}{len(tris):10d}{1:10d}{0:10d}{3:10d}{3:10d}\n")
        f.write("ENDOFSECTION\n   NODAL COORDINATES 2.4.6\n")
        for q, (x, y, z) in enumerate(nodes, 1):
            f.write(f"{q:10d} {x:.17g} {y:.17g} {z:.17g}\n")
        f.write("ENDOFSECTION\n      ELEMENTS/CELLS 2.4.6\n")
        for q, (a, b, c) in enumerate(tris, 1):
            f.write(f"{q:8d} 3  3 {a:8d}{b:8d}{c:8d}\n")
        f.write("ENDOFSECTION\n")


def read_gmsh(path, sur_geo_points: int = 0):
    """Reads a Gmsh 2 ASCII surface mesh as readSurfaceMeshGmsh does
    (subReadInput.f90:143-167): the first `sur_geo_points` element lines are
    skipped and the last three integers of each remaining line are the nodes."""
    with open(path) as f:
        lines = [ln for ln in f.read().splitlines()]
    pos = 4
    nn = int(lines[pos].split()[0]); pos += 1
    nodes = np.array([[float(v) for v in lines[pos + q].split()[1:4]] for q in range(nn)])
    pos += nn + 2
    ne = int(lines[pos].split()[0]); pos += 1
    pos += sur_geo_points
    ne -= sur_geo_points
    tris = np.array([[int(v) for v in lines[pos + q].split()[5:8]] for q in range(ne)], dtype=np.int64)
    return nodes, tris


# -------------------------------------------------------------- workloads

@dataclasses.dataclass
class Case:
    """One named workload: grid, body, flow and pressure-solver settings."""
    name: str
    x: np.ndarray
    y: np.ndarray
    z: np.ndarray
    re: float
    dt: float
    steps: int
    omega: float
    eps: float
    box: tuple
    radius: float = 0.5
    subdivisions: int = 4
    stretch: dict = dataclasses.field(default_factory=dict)

    @property
    def shape(self):
        return (len(self.x) - 1, len(self.y) - 1, len(self.z) - 1)

    @property
    def cells(self) -> int:
        nx, ny, nz = self.shape
        return nx * ny * nz


def search_box(nodes: np.ndarray, lo: float, hi: float) -> tuple[int, int]:
    """1-based cell range (cell i spans nodes[i-2]..nodes[i-1], interior i = 2..n+1)
    of the cells that intersect [lo, hi]."""
    i0 = int(np.searchsorted(nodes, lo, side="right")) - 1 + 2
    i1 = int(np.searchsorted(nodes, hi, side="left")) - 1 + 2
    n = len(nodes) - 1
    return max(i0, 2), min(i1, n + 1)


def sphere_case(name: str, n: tuple[int, int, int], h: float, core: float, re: float, dt: float, steps: int,
                omega: float, eps: float, domain=((-5.0, 15.0), (-5.0, 5.0), (-5.0, 5.0)), radius: float = 0.5,
                subdivisions: int = 4, margin_cells: int = 4) -> Case:
    axes, stretch = [], {}
    for a, (lo, hi) in enumerate(domain):
        nodes, rl, rr = stretched_axis(lo, hi, n[a], -core, core, h)
        axes.append(nodes)
        stretch["xyz"[a]] = (rl, rr)
    m = radius + margin_cells * h
    box = []
    for a in range(3):
        box += list(search_box(axes[a], -m, m))
    return Case(name, axes[0], axes[1], axes[2], re, dt, steps, omega, eps, tuple(box), radius, subdivisions,
                stretch)


def body_box(cs: Case, centre=(0.0, 0.0, 0.0), margin_cells: int = 4) -> tuple:
    """Search box of a body of cs's radius centred at `centre` (the cells within
    radius + margin_cells core cells of it), for re-tagging a moving body."""
    h = float(np.min(np.diff(cs.x)))
    m = cs.radius + margin_cells * h
    box = []
    for a, ax in enumerate((cs.x, cs.y, cs.z)):
        box += list(search_box(ax, centre[a] - m, centre[a] + m))
    return tuple(box)


def case(name: str) -> Case:
    """The named workloads.

    sphere96   - 96x64x64, Re 100, D/16 core on [-0.75,0.75]^3, dt 0.005, omega 1.8, eps 1e-6
    sphere256  - 256x192x192, Re 300, D/40 core on [-0.8,0.8]^3, dt 0.002, eps 1e-6
    sphere384  - 384x256x256, Re 200, D/48 core on [-1,1]^3, dt 0.002, eps 1e-6
    tiny       - 40x32x32 test case (D/8 core), Re 100
    small      - 64x48x48 test case (D/12 core), Re 100
    """
    if name == "sphere96":
        return sphere_case(name, (96, 64, 64), 1.0 / 16, 0.75, 100.0, 0.005, 200, 1.8, 1e-6)
    if name == "sphere256":
        return sphere_case(name, (256, 192, 192), 1.0 / 40, 0.8, 300.0, 0.002, 2000, 1.8, 1e-6)
    if name == "sphere384":
        return sphere_case(name, (384, 256, 256), 1.0 / 48, 1.0, 200.0, 0.002, 1000, 1.8, 1e-6)
    if name == "tiny":
        return sphere_case(name, (40, 32, 32), 1.0 / 8, 0.75, 100.0, 0.005, 20, 1.8, 1e-7,
                           domain=((-3.0, 6.0), (-3.0, 3.0), (-3.0, 3.0)), subdivisions=3)
    if name == "small":
        return sphere_case(name, (64, 48, 48), 1.0 / 12, 0.75, 100.0, 0.005, 20, 1.8, 1e-7,
                           domain=((-3.0, 9.0), (-3.5, 3.5), (-3.5, 3.5)), subdivisions=4)
    raise KeyError(name)
