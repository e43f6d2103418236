"""ctypes wrapper of the CPU oracle (liboracle.so, built by oracle/build.py).

Test infrastructure only: what the CUDA library is tested against, and the timed
CPU baseline of bench.py. Parity status: unpinned by the reference itself (no
Fortran compiler, no reference tests or fixtures); pinned by analytic
known-answer tests and by the committed fixtures in tests/golden/.

The methods mirror ib3d_gpu_gb300.Solver so that a parity test runs the same
call sequence on both.
"""
from __future__ import annotations

import ctypes as C
import pathlib

import numpy as np

HERE = pathlib.Path(__file__).resolve().parent
LIB_PATH = HERE / "liboracle.so"
_D = C.POINTER(C.c_double)
_I64 = C.POINTER(C.c_int64)
_VP = C.c_void_p
FIELDS = {"u": 0, "v": 1, "w": 2, "ut": 3, "vt": 4, "wt": 5, "p": 6, "pc": 7, "b": 8}
_lib = None


def lib() -> C.CDLL:
    global _lib
    if _lib is not None:
        return _lib
    if not LIB_PATH.exists():
        from . import build as _b  # type: ignore
        _b.build()
    L = C.CDLL(str(LIB_PATH))
    sig = {
        "or_create": (_VP, [C.c_int64, C.c_int64, C.c_int64, _D, _D, _D, C.c_double, C.c_double]),
        "or_destroy": (None, [_VP]),
        "or_set_solver": (None, [_VP, C.c_double, C.c_double, C.c_int, C.c_int64, C.c_int]),
        "or_set_mesh": (C.c_int, [_VP, C.c_int64, _D, _D, _D, C.c_int64, _I64, _I64, _I64, C.c_double, C.c_double,
                                  C.c_double, C.c_int64]),
        "or_search": (C.c_int, [_VP, _I64]),
        "or_selective_retag": (C.c_int, [_VP]),
        "or_move_body": (C.c_int, [_VP] + [C.c_double] * 6),
        "or_initial_conditions": (None, [_VP]),
        "or_coefficient_matrix": (None, [_VP]),
        "or_set_coefficients": (None, [_VP, _D, _D, _D]),
        "or_no_body": (None, [_VP]),
        "or_move_body_free": (C.c_int, [_VP, C.c_double, C.c_double, C.c_double, _D]),
        "or_redblack_sor": (C.c_int, [_VP, _I64, _D]),
        "or_non_uni_coeff": (None, [_VP]),
        "or_ns_momentum": (None, [_VP]),
        "or_ns_momentum_ab": (None, [_VP]),
        "or_set_momentum": (None, [_VP, C.c_int]),
        "or_set_outlet": (None, [_VP, C.c_int]),
        "or_calculate_uc": (None, [_VP]),
        "or_uc": (C.c_double, [_VP]),
        "or_velocity_bc": (None, [_VP]),
        "or_solid_cell_bc": (None, [_VP]),
        "or_velocity_forcing": (C.c_int, [_VP]),
        "or_pressure_forcing": (C.c_int, [_VP]),
        "or_poisson_solver": (C.c_int, [_VP, _I64, _D, _D, _D]),
        "or_stress": (C.c_int, [_VP, C.c_int, _D]),
        "or_step": (C.c_int, [_VP, C.c_int, _I64, _D]),
        "or_field": (_D, [_VP, C.c_int]),
        "or_cell": (_I64, [_VP]),
        "or_counts": (None, [_VP, _I64]),
        "or_list": (_I64, [_VP, C.c_int]),
        "or_surface": (_D, [_VP, C.c_int]),
        "or_normdis": (_D, [_VP, C.c_int]),
        "or_nelp": (_I64, [_VP]),
        "or_acoef": (_D, [_VP, C.c_int]),
        "or_conv_coef": (_D, [_VP, C.c_int, C.c_int]),
        "or_grid1d": (_D, [_VP, C.c_int]),
        "or_set_threads": (None, [C.c_int]),
        "or_set_sweep_rows": (None, [_VP, C.c_int]),
        "or_write_result_text": (C.c_int, [_VP, C.c_char_p, C.c_double, C.c_int64, C.c_int64]),
        "or_read_result_text": (C.c_int, [_VP, C.c_char_p, _D, _I64, _I64]),
    }
    for name, (res, args) in sig.items():
        fn = getattr(L, name)
        fn.restype = res
        fn.argtypes = args
    _lib = L
    return L


def set_threads(n: int) -> None:
    lib().or_set_threads(int(n))


class OracleError(RuntimeError):
    def __init__(self, code, what):
        super().__init__(f"oracle {what} returned {code}")
        self.code = code


class Oracle:
    """Serial FP64 restatement of the reference's hot path on one grid."""

    def __init__(self, x, y, z, re: float, deltat: float, omega: float = 1.99, eps: float = 1e-5,
                 criterion: int = 0, max_sweeps: int = 1_000_000, check_every: int = 1, outlet: int = 0,
                 momentum: int = 0):
        self.L = lib()
        self.x = np.ascontiguousarray(x, dtype=np.float64)
        self.y = np.ascontiguousarray(y, dtype=np.float64)
        self.z = np.ascontiguousarray(z, dtype=np.float64)
        self.nx, self.ny, self.nz = len(x) - 1, len(y) - 1, len(z) - 1
        self.shape = (self.nx + 2, self.ny + 2, self.nz + 2)
        self._h = self.L.or_create(self.nx, self.ny, self.nz, self.x.ctypes.data_as(_D), self.y.ctypes.data_as(_D),
                                   self.z.ctypes.data_as(_D), float(re), float(deltat))
        self.set_solver(omega, eps, criterion, max_sweeps, check_every)
        self.L.or_set_outlet(self._h, int(outlet))
        self.L.or_set_momentum(self._h, int(momentum))
        self.L.or_coefficient_matrix(self._h)
        self.L.or_non_uni_coeff(self._h)
        self.nelems = 0

    def close(self):
        if self._h:
            self.L.or_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def set_sweep_rows(self, on: bool = True):
        """Row form of the sweep loop (bit-identical; the timed CPU baseline uses it)."""
        self.L.or_set_sweep_rows(self._h, 1 if on else 0)

    def write_result_text(self, path, totime: float = 0.0, ita: int = 0, ita1: int = 0):
        """writeResult: the reference's formatted `result` restart file."""
        self._chk(self.L.or_write_result_text(self._h, str(path).encode(), float(totime), int(ita), int(ita1)),
                  "or_write_result_text")

    def read_result_text(self, path) -> tuple:
        """lastConditions: loads u, v, w, p (ut = u ...) from `result`; returns (totime, ita, ita1)."""
        t = np.zeros(1)
        it = np.zeros(2, np.int64)
        self._chk(self.L.or_read_result_text(self._h, str(path).encode(), t.ctypes.data_as(_D),
                                             it[0:1].ctypes.data_as(_I64), it[1:2].ctypes.data_as(_I64)),
                  "or_read_result_text")
        return float(t[0]), int(it[0]), int(it[1])

    def set_solver(self, omega, eps, criterion=0, max_sweeps=1_000_000, check_every=1):
        self.L.or_set_solver(self._h, float(omega), float(eps), int(criterion), int(max_sweeps), int(check_every))

    def _chk(self, rc, what):
        if rc:
            raise OracleError(rc, what)
        return rc

    def set_mesh(self, nodes, tris, shift=(0.0, 0.0, 0.0), inor=1):
        nodes = np.asarray(nodes, dtype=np.float64)
        tris = np.asarray(tris, dtype=np.int64)
        xn, yn, zn = (np.ascontiguousarray(nodes[:, q]) for q in range(3))
        e1, e2, e3 = (np.ascontiguousarray(tris[:, q]) for q in range(3))
        self._chk(self.L.or_set_mesh(self._h, len(nodes), xn.ctypes.data_as(_D), yn.ctypes.data_as(_D),
                                     zn.ctypes.data_as(_D), len(tris), e1.ctypes.data_as(_I64),
                                     e2.ctypes.data_as(_I64), e3.ctypes.data_as(_I64), float(shift[0]),
                                     float(shift[1]), float(shift[2]), int(inor)), "or_set_mesh")
        self.nelems = len(tris)

    def move_body_free(self, fx, fy, fz) -> np.ndarray:
        v = np.zeros(3)
        self._chk(self.L.or_move_body_free(self._h, fx, fy, fz, v.ctypes.data_as(_D)), "or_move_body_free")
        return v

    def no_body(self):
        """Every interior cell fluid (no surface mesh, no search)."""
        self.L.or_no_body(self._h)
        self.counts = {"fluid": self.nx * self.ny * self.nz, "solid": 0, "ib": 0}

    def move_body(self, dx, dy, dz, us=0.0, vs=0.0, ws=0.0):
        self._chk(self.L.or_move_body(self._h, dx, dy, dz, us, vs, ws), "or_move_body")

    def search(self, box) -> dict:
        b = np.asarray(box, dtype=np.int64)
        self._chk(self.L.or_search(self._h, b.ctypes.data_as(_I64)), "or_search")
        c = np.zeros(5, dtype=np.int64)
        self.L.or_counts(self._h, c.ctypes.data_as(_I64))
        self.counts = dict(zip(("fluid", "solid", "ib", "red", "black"), (int(v) for v in c)))
        return self.counts

    def selective_retag(self) -> dict:
        """selectiveRetagging: re-tag the 6^3 neighbourhoods of the current IB cells."""
        self._chk(self.L.or_selective_retag(self._h), "or_selective_retag")
        c = np.zeros(5, dtype=np.int64)
        self.L.or_counts(self._h, c.ctypes.data_as(_I64))
        self.counts = dict(zip(("fluid", "solid", "ib", "red", "black"), (int(v) for v in c)))
        return self.counts

    def get_search(self) -> dict:
        nib = self.counts["ib"]
        n3 = int(np.prod(self.shape))
        cell = np.ctypeslib.as_array(self.L.or_cell(self._h), shape=(n3,)).reshape(self.shape, order="F").copy()
        ib = np.ctypeslib.as_array(self.L.or_list(self._h, 2), shape=(3 * nib,)).reshape((nib, 3), order="F").copy() \
            if nib else np.zeros((0, 3), np.int64)
        nelp = np.ctypeslib.as_array(self.L.or_nelp(self._h), shape=(nib,)).copy() if nib else np.zeros(0, np.int64)
        nd = np.stack([np.ctypeslib.as_array(self.L.or_normdis(self._h, q), shape=(nib,)).copy() for q in range(7)],
                      axis=1) if nib else np.zeros((0, 7))
        return {"cell": cell, "ib": ib, "nelp": nelp, "normdis": nd}

    def list(self, which: int) -> np.ndarray:
        key = ("fluid", "solid", "ib", "red", "black")[which]
        n = self.counts[key]
        if n == 0:
            return np.zeros((0, 3), np.int64)
        return np.ctypeslib.as_array(self.L.or_list(self._h, which), shape=(3 * n,)).reshape((n, 3), order="F").copy()

    def surface(self) -> np.ndarray:
        return np.stack([np.ctypeslib.as_array(self.L.or_surface(self._h, q), shape=(self.nelems,)).copy()
                         for q in range(9)])

    def acoef(self, axis: int) -> np.ndarray:
        n = (self.nx, self.ny, self.nz)[axis]
        return np.ctypeslib.as_array(self.L.or_acoef(self._h, axis), shape=(3 * n,)).reshape((n, 3), order="F").copy()

    def set_acoef(self, acx, acy, acz):
        """Replaces Acx/Acy/Acz ((n,3) arrays) for other boundary conditions."""
        a = [np.asfortranarray(v, dtype=np.float64) for v in (acx, acy, acz)]
        self.L.or_set_coefficients(self._h, *(v.ctypes.data_as(_D) for v in a))

    def conv_coef(self, fam: int, m: int) -> np.ndarray:
        n = (self.nx, self.ny, self.nz)[fam % 3]
        return np.ctypeslib.as_array(self.L.or_conv_coef(self._h, fam, m), shape=(n + 3,)).copy()

    def grid1d(self, which: int, length: int) -> np.ndarray:
        return np.ctypeslib.as_array(self.L.or_grid1d(self._h, which), shape=(length,)).copy()

    def initial_conditions(self):
        self.L.or_initial_conditions(self._h)

    def get_field(self, name: str) -> np.ndarray:
        n3 = int(np.prod(self.shape))
        p = self.L.or_field(self._h, FIELDS[name])
        return np.ctypeslib.as_array(p, shape=(n3,)).reshape(self.shape, order="F").copy()

    def set_field(self, name: str, arr):
        n3 = int(np.prod(self.shape))
        p = self.L.or_field(self._h, FIELDS[name])
        dst = np.ctypeslib.as_array(p, shape=(n3,))
        dst[:] = np.asarray(arr, dtype=np.float64).reshape(-1, order="F")

    def ns_momentum(self):
        self.L.or_ns_momentum(self._h)

    def velocity_bc(self):
        self.L.or_velocity_bc(self._h)

    def solid_cell_bc(self):
        self.L.or_solid_cell_bc(self._h)

    def velocity_forcing(self):
        self._chk(self.L.or_velocity_forcing(self._h), "or_velocity_forcing")

    def pressure_forcing(self):
        self._chk(self.L.or_pressure_forcing(self._h), "or_pressure_forcing")

    def poisson_solver(self, allow_noconv: bool = False) -> dict:
        ns = np.zeros(1, np.int64)
        vals = np.zeros(3)
        rc = self.L.or_poisson_solver(self._h, ns.ctypes.data_as(_I64), vals[0:].ctypes.data_as(_D),
                                      vals[1:].ctypes.data_as(_D), vals[2:].ctypes.data_as(_D))
        if rc and not allow_noconv:
            raise OracleError(rc, "or_poisson_solver")
        return {"sweeps": int(ns[0]), "divmax": vals[0], "derr_std_st": vals[1], "final_err": vals[2], "rc": rc}

    def ns_momentum_ab(self):
        self.L.or_ns_momentum_ab(self._h)

    def calculate_uc(self) -> float:
        self.L.or_calculate_uc(self._h)
        return float(self.L.or_uc(self._h))

    @property
    def uc(self) -> float:
        return float(self.L.or_uc(self._h))

    def redblack_sor(self, allow_noconv: bool = False) -> dict:
        ns = np.zeros(1, np.int64)
        err = np.zeros(1)
        rc = self.L.or_redblack_sor(self._h, ns.ctypes.data_as(_I64), err.ctypes.data_as(_D))
        if rc and not (allow_noconv and rc == 1):
            raise OracleError(rc, "or_redblack_sor")
        return {"sweeps": int(ns[0]), "final_err": float(err[0]), "rc": rc}

    def stress(self, first: bool) -> np.ndarray:
        coef = np.zeros(4)
        self._chk(self.L.or_stress(self._h, 1 if first else 0, coef.ctypes.data_as(_D)), "or_stress")
        return coef

    def step(self, first: bool, allow_noconv: bool = False):
        ns = np.zeros(1, np.int64)
        coef = np.zeros(4)
        rc = self.L.or_step(self._h, 1 if first else 0, ns.ctypes.data_as(_I64), coef.ctypes.data_as(_D))
        if rc and not (allow_noconv and rc == 1):
            raise OracleError(rc, "or_step")
        return {"sweeps": int(ns[0]), "rc": rc}, coef


def setup_case(cs, **kw) -> Oracle:
    """Oracle for a grids.Case (same inputs as ib3d_gpu_gb300.setup_case)."""
    import importlib
    grids = importlib.import_module("ib3d_gpu_gb300.grids")
    args = dict(omega=cs.omega, eps=cs.eps)
    args.update(kw)
    o = Oracle(cs.x, cs.y, cs.z, cs.re, cs.dt, **args)
    nodes, tris = grids.icosphere(cs.subdivisions, cs.radius)
    o.set_mesh(nodes, tris)
    o.search(cs.box)
    o.initial_conditions()
    return o
